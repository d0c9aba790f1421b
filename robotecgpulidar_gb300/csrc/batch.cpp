#include "batch.hpp"

#include <algorithm>
#include <cstring>
#include <limits>
#include <set>

#include "scene.hpp"
#include "wave_split.hpp"

using rgl::format;
using rgl::InvalidPipeline;

namespace {
constexpr int kBranches = 4;     // forked streams at creation; grown to the largest wave
constexpr int kMaxBranches = 32;

bool sameSchedule(const rgl::BatchSchedule& a, const rgl::BatchSchedule& b)
{
	return a.block == b.block && a.packing == b.packing && a.order == b.order && a.chunk == b.chunk && a.regs == b.regs;
}

// Gives every kernel node of a captured frame except the traversal launches the greatest priority:
// a wave's later nodes, ready when its traversal completes, then take the SM slots that free up
// before the blocks of the next traversal launch waiting for them.
cudaError_t prioritizeNodeKernels(cudaGraph_t graph, int priority)
{
	size_t n = 0;
	cudaError_t e = cudaGraphGetNodes(graph, nullptr, &n);
	std::vector<cudaGraphNode_t> nodes(n);
	if (e == cudaSuccess && n > 0) {
		e = cudaGraphGetNodes(graph, nodes.data(), &n);
	}
	for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
		cudaGraphNodeType type;
		e = cudaGraphNodeGetType(nodes[i], &type);
		if (e != cudaSuccess || type != cudaGraphNodeTypeKernel) {
			continue;
		}
		cudaKernelNodeParams params = {};
		e = cudaGraphKernelNodeGetParams(nodes[i], &params);
		if (e != cudaSuccess || rgl::isTraceBatchKernel(params.func)) {
			continue;
		}
		cudaLaunchAttributeValue v = {};
		v.priority = priority;
		e = cudaGraphKernelNodeSetAttribute(nodes[i], cudaLaunchAttributePriority, &v);
	}
	return e;
}
} // namespace

BatchRun::BatchRun(std::vector<Node::Ptr> a) : anchors(std::move(a)), dKeys(false), dOrder(false), dSortScratch(false), dError(false)
{
	int least = 0;
	RGL_CHECK_CUDA(cudaDeviceGetStreamPriorityRange(&least, &priorityHigh));
	RGL_CHECK_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
	for (int b = 0; b < kBranches; ++b) {
		addBranch();
	}
	RGL_CHECK_CUDA(cudaEventCreateWithFlags(&forkEv, cudaEventDisableTiming));
	RGL_CHECK_CUDA(cudaStreamCreateWithPriority(&postStream, cudaStreamNonBlocking, priorityHigh));
	RGL_CHECK_CUDA(cudaEventCreateWithFlags(&postJoin, cudaEventDisableTiming));
	RGL_CHECK_CUDA(cudaEventCreate(&frameStart));
	RGL_CHECK_CUDA(cudaEventCreate(&frameStop));
	RGL_CHECK_CUDA(cudaEventCreate(&traceStart));
	RGL_CHECK_CUDA(cudaEventCreate(&traceStop));
	// Allocated here: the first use may be inside a stream capture, where allocation is not allowed.
	RGL_CHECK_CUDA(cudaMemsetAsync(dError.ensure(sizeof(int32_t)), 0, sizeof(int32_t), stream));
}

BatchRun::~BatchRun()
{
	if (running) {
		cudaEventSynchronize(frameStop);
	}
	for (auto& m : members) {
		for (cudaEvent_t e : waveDone) {
			m.ctx->forgetBatchEvent(e);
		}
	}
	releaseExec();
	for (size_t b = 0; b < branches.size(); ++b) {
		cudaEventDestroy(joinEv[b]);
		cudaStreamDestroy(branches[b]);
	}
	cudaEventDestroy(forkEv);
	cudaEventDestroy(frameStart);
	cudaEventDestroy(frameStop);
	cudaEventDestroy(traceStart);
	cudaEventDestroy(traceStop);
	cudaEventDestroy(postJoin);
	for (cudaEvent_t e : waveTraced) {
		cudaEventDestroy(e);
	}
	for (cudaEvent_t e : waveDone) {
		cudaEventDestroy(e);
	}
	cudaStreamDestroy(postStream);
	cudaStreamDestroy(stream);
}

void BatchRun::releaseExec()
{
	if (exec) {
		cudaGraphExecDestroy(exec);
		exec = nullptr;
	}
}

void BatchRun::synchronize()
{
	if (!running) {
		return;
	}
	running = false;
	RGL_CHECK_CUDA(cudaEventSynchronize(frameStop));
	RGL_CHECK_CUDA(cudaGetLastError());
	cudaEventElapsedTime(&lastFrameMs, frameStart, frameStop);
	cudaEventElapsedTime(&lastTraceMs, traceStart, traceStop);
	rgl::refreshErrorSlots(); // once for the whole frame
	for (auto& m : members) {
		m.ctx->synchronize(false);
	}
}

void BatchRun::resolveMembers()
{
	members.clear();
	std::set<GraphRunCtx*> seen;
	for (auto& a : anchors) {
		if (!a->ctx) {
			GraphRunCtx::createAndAttach(a);
		}
		if (seen.insert(a->ctx.get()).second) {
			members.push_back(Member{a->ctx, nullptr, {}, {}});
		}
	}
	if ((int) members.size() > rgl::kMaxBatchJobs) {
		throw rgl::InvalidAPIArgument(format("a batch holds at most %d sensor graphs, got %zu", rgl::kMaxBatchJobs, members.size()));
	}
}

void BatchRun::buildJobs()
{
	const size_t n = members.size();
	jobs.assign(n, rgl::BatchJob{});
	beamBase.assign(n + 1, 0);
	shape.clear();
	maxSamples = 1;
	shading = false;
	beams = 0;
	rays = 0;
	for (size_t j = 0; j < n; ++j) {
		rgl::BatchJob& b = jobs[j];
		members[j].trace->fillJob(b);
		const rgl::TraceParams& p = b.p;
		shading = shading || rgl::needsShadingKernel(p);
		maxSamples = std::max(maxSamples, (int) p.nSamples);
		beamBase[j] = beams;
		beams += p.nRays;
		rays += (int64_t) p.nRays * p.nSamples;
		shape.push_back(p.nRays);
		shape.push_back(p.nSamples);
	}
	beamBase[n] = beams;
	if (beams > (int64_t) std::numeric_limits<int32_t>::max() / 2) {
		throw rgl::InvalidAPIArgument(format("a batch casts at most %d beams per frame, got %lld", std::numeric_limits<int32_t>::max() / 2,
		                                     (long long) beams));
	}
	splitWaves();
	shape.push_back(waveCount());
}

// Cuts the members, in batch order, into waves of about equal traced rays (wave_split.hpp).
void BatchRun::splitWaves()
{
	std::vector<int64_t> memberRays(members.size());
	for (size_t j = 0; j < members.size(); ++j) {
		memberRays[j] = (int64_t) jobs[j].p.nRays * jobs[j].p.nSamples;
	}
	const int W = wavesWanted > 0 ? wavesWanted : (int) std::min<int64_t>(kAutoWaves, std::max<int64_t>(1, rays / kRaysPerWave));
	waveFirst = rgl::splitIntoWaves(memberRays, W);
}

// A forked stream at the greatest priority, so that the graphs' node kernels on it start before
// pending traversal blocks.
void BatchRun::addBranch()
{
	cudaStream_t st = nullptr;
	cudaEvent_t ev = nullptr;
	RGL_CHECK_CUDA(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, priorityHigh));
	branches.push_back(st);
	RGL_CHECK_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
	joinEv.push_back(ev);
}

// One counter block and one completion event per wave, and a forked stream per graph of the largest
// wave (up to kMaxBranches), so a wave's later nodes all start together; made outside any capture.
void BatchRun::ensureWaveResources()
{
	int widest = 0;
	for (int w = 0; w < waveCount(); ++w) {
		widest = std::max(widest, waveFirst[w + 1] - waveFirst[w]);
	}
	while ((int) branches.size() < std::min(widest, kMaxBranches)) {
		addBranch();
	}
	while ((int) waveTraced.size() < waveCount()) {
		cudaEvent_t e = nullptr, d = nullptr;
		RGL_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
		waveTraced.push_back(e);
		RGL_CHECK_CUDA(cudaEventCreateWithFlags(&d, cudaEventDisableTiming));
		waveDone.push_back(d);
	}
	const size_t bytes = rgl::kTraceCounterBytes * waveCount();
	if (bytes > counterBytesZeroed) {
		RGL_CHECK_CUDA(cudaStreamSynchronize(stream)); // the old counter blocks may still be in use
		RGL_CHECK_CUDA(cudaMemsetAsync(dCounter.ensure(bytes), 0, dCounter.capacity(), stream));
		counterBytesZeroed = dCounter.capacity();
	}
}

void BatchRun::uploadJobs(const rgl::BatchSchedule& s, cudaStream_t st)
{
	const size_t n = members.size();
	std::vector<int32_t> base(n + 1, 0);
	int64_t tasks = 0;
	for (size_t j = 0; j < n; ++j) {
		rgl::BatchJob& b = jobs[j];
		b.order = (s.order != rgl::kOrderNatural && orderHeld == s.order) ? dOrder.as<uint32_t>() + beamBase[j] : nullptr;
		base[j] = (int32_t) tasks;
		const int per = rgl::batchBeamsPerTask(s.packing, b.p.nSamples);
		tasks += (b.p.nRays + per - 1) / per;
	}
	base[n] = (int32_t) tasks;
	for (int w = 0; w < waveCount(); ++w) {
		const int lo = waveFirst[w], hi = waveFirst[w + 1];
		for (int j = lo; j <= hi; ++j) {
			base.push_back(base[j] - base[lo]);
		}
	}
	const size_t nBase = base.size();
	std::vector<uint8_t> bytes(sizeof(rgl::BatchJob) * n + sizeof(int32_t) * nBase);
	std::memcpy(bytes.data(), jobs.data(), sizeof(rgl::BatchJob) * n);
	std::memcpy(bytes.data() + sizeof(rgl::BatchJob) * n, base.data(), sizeof(int32_t) * nBase);
	if (bytes == uploaded) {
		return;
	}
	// Pageable sources: the copies are staged before the calls return, and the previous frame,
	// the only reader of these buffers, has completed.
	RGL_CHECK_CUDA(cudaMemcpyAsync(dJobs.ensure(sizeof(rgl::BatchJob) * std::max<size_t>(n, 1)), jobs.data(), sizeof(rgl::BatchJob) * n,
	                               cudaMemcpyHostToDevice, st));
	RGL_CHECK_CUDA(cudaMemcpyAsync(dTaskBase.ensure(sizeof(int32_t) * nBase), base.data(), sizeof(int32_t) * nBase,
	                               cudaMemcpyHostToDevice, st));
	RGL_CHECK_CUDA(cudaStreamSynchronize(st));
	uploaded = std::move(bytes);
}

void BatchRun::enqueueMembers(bool preTrace, size_t lo, size_t hi, cudaStream_t s)
{
	const int nb = (int) std::min<size_t>(branches.size(), hi - lo);
	if (nb <= 1) {
		for (size_t j = lo; j < hi; ++j) {
			for (auto& node : preTrace ? members[j].pre : members[j].post) {
				node->enqueueImpl(s);
			}
		}
		return;
	}
	RGL_CHECK_CUDA(cudaEventRecord(forkEv, s));
	for (int b = 0; b < nb; ++b) {
		RGL_CHECK_CUDA(cudaStreamWaitEvent(branches[b], forkEv, 0));
	}
	for (size_t j = lo; j < hi; ++j) {
		for (auto& node : preTrace ? members[j].pre : members[j].post) {
			node->enqueueImpl(branches[(j - lo) % nb]);
		}
	}
	for (int b = 0; b < nb; ++b) {
		RGL_CHECK_CUDA(cudaEventRecord(joinEv[b], branches[b]));
		RGL_CHECK_CUDA(cudaStreamWaitEvent(s, joinEv[b], 0));
	}
}

// One traversal launch over wave `wave`'s sensors, with its own counter block. Every wave after the
// first overlaps the tail of the launch before it on the stream.
void BatchRun::enqueueTrace(const rgl::BatchSchedule& s, int wave, cudaStream_t st)
{
	const int n = (int) members.size(), lo = waveFirst[wave], hi = waveFirst[wave + 1];
	rgl::launchTraceBatch(dJobs.as<rgl::BatchJob>() + lo, dTaskBase.as<int32_t>() + (n + 1) + lo + wave, hi - lo, maxSamples, shading, s,
	                      dCounter.as<uint32_t>() + wave * (rgl::kTraceCounterBytes / sizeof(uint32_t)), st, wave > 0);
}

// The frame's device work. On `s`: refit, every graph's nodes before the traversal, the traversal
// launches one after another; on the side stream: wave w's later nodes after its launch completes
// (an ordinary edge from that launch alone; the next launch's edge to it is programmatic), then
// wave w's completion event (an event node of the capture). The side stream rejoins `s` at the end.
void BatchRun::enqueueFrame(cudaStream_t s)
{
	for (Scene* sc : scenes) {
		sc->enqueueRefit(s);
	}
	enqueueMembers(true, 0, members.size(), s);
	recordEvent(traceStart, s);
	for (int w = 0; w < waveCount(); ++w) {
		enqueueTrace(schedule, w, s);
		RGL_CHECK_CUDA(cudaEventRecord(waveTraced[w], s));
		RGL_CHECK_CUDA(cudaStreamWaitEvent(postStream, waveTraced[w], 0));
		enqueueMembers(false, waveFirst[w], waveFirst[w + 1], postStream);
		recordEvent(waveDone[w], postStream);
	}
	recordEvent(traceStop, s);
	RGL_CHECK_CUDA(cudaEventRecord(postJoin, postStream));
	RGL_CHECK_CUDA(cudaStreamWaitEvent(s, postJoin, 0));
}

// Sorts every sensor's beams by `order` (job index in the key's top bits keeps each sensor's beams
// together) into dOrder; the world rays must be current, so the nodes before the traversal run first.
void BatchRun::computeOrder(int order, cudaStream_t st)
{
	if (order == rgl::kOrderNatural || beams == 0) {
		orderHeld = order;
		return;
	}
	enqueueMembers(true, 0, members.size(), st);
	auto* keys = static_cast<uint32_t*>(dKeys.ensure(sizeof(uint32_t) * beams));
	auto* vals = static_cast<uint32_t*>(dOrder.ensure(sizeof(uint32_t) * beams));
	for (size_t j = 0; j < members.size(); ++j) {
		const Scene* sc = members[j].trace->scene;
		rgl::launchBeamKeys(jobs[j].p.rays, jobs[j].hasRayTransform ? &jobs[j].rayTransform : nullptr, jobs[j].p.nRays, (uint32_t) j,
		                    order, sc->worldLower(), sc->worldUpper(), keys + beamBase[j], vals + beamBase[j], st);
	}
	int jobBits = 0;
	while ((size_t{1} << jobBits) < members.size()) {
		++jobBits;
	}
	const int keyBits = 22 + jobBits;
	rgl::sortPairs(keys, vals, (int) beams, keyBits, dSortScratch.ensure(rgl::sortPairsScratchBytes((int) beams, keyBits)),
	               dError.as<int32_t>(), st);
	RGL_CHECK_CUDA(cudaStreamSynchronize(st));
	int32_t e = 0;
	RGL_CHECK_CUDA(cudaMemcpy(&e, dError.get(), sizeof(e), cudaMemcpyDeviceToHost));
	if (e != 0) {
		RGL_CHECK_CUDA(cudaMemsetAsync(dError.get(), 0, sizeof(int32_t), st));
		throw std::runtime_error("batched beam ordering: radix sort look-back did not complete on the device");
	}
	orderHeld = order;
}

// Times the frame's traversal launches (one per wave, each overlapping the previous one's tail)
// under schedule s.
float BatchRun::timeTrace(const rgl::BatchSchedule& s, int reps)
{
	uploadJobs(s, stream);
	ensureWaveResources();
	for (int w = 0; w < waveCount(); ++w) {
		rgl::prepareTraceBatch(waveFirst[w + 1] - waveFirst[w], maxSamples, shading, s);
	}
	auto traceAll = [&]() {
		for (int w = 0; w < waveCount(); ++w) {
			enqueueTrace(s, w, stream);
		}
	};
	traceAll(); // warm-up
	float best = std::numeric_limits<float>::infinity();
	for (int r = 0; r < reps; ++r) {
		RGL_CHECK_CUDA(cudaEventRecord(traceStart, stream));
		traceAll();
		RGL_CHECK_CUDA(cudaEventRecord(traceStop, stream));
		RGL_CHECK_CUDA(cudaEventSynchronize(traceStop));
		float ms = 0.0f;
		RGL_CHECK_CUDA(cudaEventElapsedTime(&ms, traceStart, traceStop));
		best = std::min(best, ms);
	}
	return best;
}

// Staged search: packing x beam order first (128 threads, 128 registers: the setting at which both
// packings run without spills), then the register budget (64, 80, 96, 128), the block size (64, 128,
// 256) and the chunk (1, 2, 4), each stage keeping the best so far. Every candidate runs the real
// traversal of this frame's rays over the current scene; its outputs are overwritten by the frame.
void BatchRun::tune()
{
	lastTuning.clear();
	enqueueMembers(true, 0, members.size(), stream);
	auto measure = [&](const rgl::BatchSchedule& s) {
		const float probe = timeTrace(s, 1);
		const int reps = std::max(2, std::min(10, (int) (20.0f / std::max(probe, 1e-3f))));
		const float ms = std::min(probe, timeTrace(s, reps));
		lastTuning.push_back(Candidate{s, ms});
		return ms;
	};
	rgl::BatchSchedule best = rgl::BatchSchedule{256, rgl::kPackLaneGroup, rgl::kOrderNatural, 1, 80};
	float bestMs = std::numeric_limits<float>::infinity();
	for (int order : {rgl::kOrderNatural, rgl::kOrderOctahedral, rgl::kOrderMorton, rgl::kOrderElevation}) {
		computeOrder(order, stream);
		for (int packing : {rgl::kPackLaneGroup, rgl::kPackSerial}) {
			rgl::BatchSchedule s{128, packing, order, 1, 128};
			const float ms = measure(s);
			if (ms < bestMs) {
				bestMs = ms;
				best = s;
			}
		}
	}
	if (orderHeld != best.order) {
		computeOrder(best.order, stream);
	}
	auto tryVariant = [&](rgl::BatchSchedule s) {
		const float ms = measure(s);
		if (ms < bestMs) {
			bestMs = ms;
			best = s;
		}
	};
	const rgl::BatchSchedule afterOrder = best;
	for (int regs : {64, 80, 96, 128}) {
		if (regs != afterOrder.regs) {
			tryVariant(rgl::BatchSchedule{afterOrder.block, afterOrder.packing, afterOrder.order, afterOrder.chunk, regs});
		}
	}
	const rgl::BatchSchedule afterRegs = best;
	for (int block : {64, 128, 256}) {
		if (block != afterRegs.block) {
			tryVariant(rgl::BatchSchedule{block, afterRegs.packing, afterRegs.order, afterRegs.chunk, afterRegs.regs});
		}
	}
	const rgl::BatchSchedule afterBlock = best;
	for (int chunk : {1, 2, 4}) {
		if (chunk != afterBlock.chunk) {
			tryVariant(rgl::BatchSchedule{afterBlock.block, afterBlock.packing, afterBlock.order, chunk, afterBlock.regs});
		}
	}
	schedule = best;
	++tunings;
}

void BatchRun::run()
{
	synchronize();
	resolveMembers();
	if (members.empty()) {
		throw rgl::InvalidAPIArgument("a batch needs at least one graph");
	}
	// Graphs outside the batch may still read the scene this frame refits.
	GraphRunCtx::synchronizeAll();

	uint64_t version = 0;
	std::vector<GraphRunCtx*> ctxs;
	scenes.clear();
	for (auto& m : members) {
		version = std::max(version, m.ctx->validateForBatch());
		const auto& ord = m.ctx->executionOrder();
		int at = -1;
		for (size_t i = 0; i < ord.size(); ++i) {
			if (auto rt = std::dynamic_pointer_cast<RaytraceNode>(ord[i])) {
				if (at >= 0) {
					throw InvalidPipeline("a batched graph must hold exactly one RaytraceNode, found more");
				}
				at = (int) i;
				m.trace = rt;
			}
		}
		if (at < 0) {
			throw InvalidPipeline("a batched graph must hold exactly one RaytraceNode, found none");
		}
		m.pre.assign(ord.begin(), ord.begin() + at);
		m.post.assign(ord.begin() + at + 1, ord.end());
		if (std::find(scenes.begin(), scenes.end(), m.trace->scene) == scenes.end()) {
			scenes.push_back(m.trace->scene);
		}
		ctxs.push_back(m.ctx.get());
	}

	std::vector<uint64_t> sceneVersions;
	for (Scene* sc : scenes) {
		sc->prepareBatched(stream);
		sceneVersions.push_back(sc->structureVersion());
	}
	try {
		for (auto& m : members) {
			m.ctx->prepareForBatch(stream);
		}
		buildJobs();
		if (shape != tunedShape || (schedule.order != rgl::kOrderNatural && orderHeld != schedule.order)) {
			if (autotune) {
				tune();
			} else {
				computeOrder(schedule.order, stream);
			}
			tunedShape = shape;
		}
		uploadJobs(schedule, stream);
		// Launch configuration (occupancy, shared-memory limit) is resolved outside any capture.
		for (int w = 0; w < waveCount(); ++w) {
			rgl::prepareTraceBatch(waveFirst[w + 1] - waveFirst[w], maxSamples, shading, schedule);
		}
		ensureWaveResources();

		RGL_CHECK_CUDA(cudaEventRecord(frameStart, stream));
		if (!cudaGraphsEnabled()) {
			releaseExec();
			enqueueFrame(stream);
		} else {
			const bool stale = exec == nullptr || version > execVersion || execEpoch != rgl::allocationEpoch() ||
			                   execScenes != sceneVersions || execSceneList != scenes || !sameSchedule(schedule, execSchedule) ||
			                   ctxs != execCtxs || execWaveFirst != waveFirst;
			if (stale) {
				releaseExec();
				const uint64_t launches0 = rgl::launchCount();
				// The graphs' parameter blocks are copied by one gather node ahead of the frame instead of
				// one copy node each (a frame of many sensors would otherwise hold hundreds).
				std::vector<rgl::ParamCopy> paramCopies;
				RGL_CHECK_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
				rgl::deferredParamCopies = &paramCopies;
				try {
					enqueueFrame(stream);
				}
				catch (...) {
					rgl::deferredParamCopies = nullptr;
					cudaGraph_t partial = nullptr;
					cudaStreamEndCapture(stream, &partial);
					if (partial) {
						cudaGraphDestroy(partial);
					}
					throw;
				}
				rgl::deferredParamCopies = nullptr;
				cudaGraph_t graph = nullptr;
				RGL_CHECK_CUDA(cudaStreamEndCapture(stream, &graph));
				cudaError_t inst = cudaSuccess;
				if (!paramCopies.empty()) {
					const size_t bytes = sizeof(rgl::ParamCopy) * paramCopies.size();
					inst = cudaMemcpy(dParamTable.ensure(bytes), paramCopies.data(), bytes, cudaMemcpyHostToDevice);
					if (inst == cudaSuccess) {
						inst = rgl::addParamGatherNode(graph, dParamTable.as<rgl::ParamCopy>(), (int) paramCopies.size());
					}
				}
				if (inst == cudaSuccess) {
					inst = prioritizeNodeKernels(graph, priorityHigh);
				}
				if (inst == cudaSuccess) {
					inst = cudaGraphInstantiateWithFlags(&exec, graph, cudaGraphInstantiateFlagUseNodePriority);
				}
				cudaGraphDestroy(graph);
				RGL_CHECK_CUDA(inst);
				execKernels = rgl::launchCount() - launches0;
				execEpoch = rgl::allocationEpoch();
				execVersion = version;
				execScenes = sceneVersions;
				execSceneList = scenes;
				execSchedule = schedule;
				execCtxs = ctxs;
				execWaveFirst = waveFirst;
				++captures;
			} else {
				++replays;
				rgl::countLaunch(execKernels);
			}
			RGL_CHECK_CUDA(cudaGraphLaunch(exec, stream));
		}
		RGL_CHECK_CUDA(cudaEventRecord(frameStop, stream));
	}
	catch (...) {
		for (Scene* sc : scenes) {
			sc->markPosesDirty(); // the refit of this frame may not have been enqueued
		}
		throw;
	}
	for (Scene* sc : scenes) {
		sc->recordReady(stream);
	}
	for (int w = 0; w < waveCount(); ++w) {
		for (int j = waveFirst[w]; j < waveFirst[w + 1]; ++j) {
			members[j].ctx->markBatchedRun(waveDone[w]);
		}
	}
	running = true;
}
