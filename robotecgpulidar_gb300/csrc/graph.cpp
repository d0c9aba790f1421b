#include "graph.hpp"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>

#include "scene.hpp"

using rgl::format;
using rgl::InvalidPipeline;
using rgl::Mat34;

namespace {
std::atomic<uint64_t> gParamVersion{0};
bool gTiming = false;
bool gCudaGraphs = [] {
	const char* v = std::getenv("RGL_GB300_CUDA_GRAPH");
	return v == nullptr || std::string(v) != "0";
}();
} // namespace
uint64_t Node::nextParamVersion() { return gParamVersion.fetch_add(1, std::memory_order_relaxed) + 1; }

namespace {
// Schedule of single-graph traversals (a batch of one job). The default is the fastest measured on
// the 1M-triangle single-sensor scan: lane-group packing, 256-thread blocks, beams in scan-row order
// (elevation, then azimuth), one task per fetch, 128 registers per thread. With a warm L2 the
// traversal of that scan takes 0.254 ms in row order, 0.262 ms in octahedral direction order and
// 0.278 ms in the given order (column-major: one azimuth's 128 channels after another).
rgl::BatchSchedule gTraceSchedule{256, rgl::kPackLaneGroup, rgl::kOrderElevation, 1, 128};
} // namespace
rgl::BatchSchedule traceSchedule() { return gTraceSchedule; }
void setTraceSchedule(const rgl::BatchSchedule& s) { gTraceSchedule = s; }
bool timingEnabled() { return gTiming; }
void setTimingEnabled(bool on) { gTiming = on; }
bool cudaGraphsEnabled() { return gCudaGraphs; }

namespace {
std::atomic<uint64_t> gGraphEdits{1};
} // namespace
void noteGraphEdit() { gGraphEdits.fetch_add(1, std::memory_order_relaxed); }
uint64_t graphEditEpoch() { return gGraphEdits.load(std::memory_order_relaxed); }
void setCudaGraphsEnabled(bool on) { gCudaGraphs = on; }

void recordEvent(cudaEvent_t ev, cudaStream_t s)
{
	cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
	RGL_CHECK_CUDA(cudaStreamIsCapturing(s, &st));
	if (st == cudaStreamCaptureStatusActive) {
		RGL_CHECK_CUDA(cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal));
	} else {
		RGL_CHECK_CUDA(cudaEventRecord(ev, s));
	}
}

// ================================================================ Node links
// (reference src/graph/Node.cpp:23-215)

template<class T>
std::shared_ptr<T> Node::exactlyOneInput(const char* ifaceName)
{
	std::vector<std::shared_ptr<T>> typed;
	for (auto& in : inputs) {
		if (auto t = std::dynamic_pointer_cast<T>(in)) {
			typed.push_back(t);
		}
	}
	if (typed.size() != 1) {
		std::string names;
		for (size_t i = 0; i < inputs.size(); ++i) {
			names += (i ? ", " : "") + std::string(inputs[i]->name());
		}
		throw InvalidPipeline(format("looked for %s, but found [%s]", ifaceName, names.c_str()));
	}
	return typed[0];
}

void Node::addChild(const Ptr& child)
{
	if (child == nullptr) {
		throw InvalidPipeline(format("attempted to set an empty child for %s", name()));
	}
	if (std::find(outputs.begin(), outputs.end(), child) != outputs.end()) {
		throw InvalidPipeline(format("attempted to add child %s to parent %s twice", child->name(), name()));
	}
	if (ctx) {
		ctx->detachAndDestroy();
	}
	if (child->ctx) {
		child->ctx->detachAndDestroy();
	}
	outputs.push_back(child);
	child->inputs.push_back(shared_from_this());
	std::stable_sort(outputs.begin(), outputs.end(), [](const Ptr& a, const Ptr& b) { return a->priority > b->priority; });
	int32_t maxChild = outputs.front()->priority;
	if (maxChild > priority) {
		setPriority(maxChild);
	}
	dirty = true;
	child->dirty = true;
}

void Node::removeChild(const Ptr& child)
{
	if (child == nullptr) {
		throw InvalidPipeline(format("attempted to remove an empty child for %s", name()));
	}
	auto it = std::find(outputs.begin(), outputs.end(), child);
	if (it == outputs.end()) {
		throw InvalidPipeline(format("attempted to remove child %s from %s,but it was not found", child->name(), name()));
	}
	auto self = shared_from_this();
	auto jt = std::find(child->inputs.begin(), child->inputs.end(), self);
	if (jt == child->inputs.end()) {
		throw InvalidPipeline(format("attempted to remove parent %s from %s,but it was not found", name(), child->name()));
	}
	if (ctx) {
		ctx->detachAndDestroy();
	}
	outputs.erase(it);
	child->inputs.erase(jt);
	dirty = true;
	child->dirty = true;
}

void Node::setPriority(int32_t p)
{
	if (p == priority) {
		return;
	}
	if (!outputs.empty() && outputs.front()->priority > p) {
		throw InvalidPipeline(format("cannot set priority of node %s to %d, because it's children %s has higher priority %d", name(),
		                             (int) p, outputs.front()->name(), (int) outputs.front()->priority));
	}
	priority = p;
	for (auto& in : inputs) {
		std::stable_sort(in->outputs.begin(), in->outputs.end(), [](const Ptr& a, const Ptr& b) { return a->priority > b->priority; });
		if (in->priority < p) {
			in->setPriority(p);
		}
	}
	if (ctx) {
		ctx->invalidateOrder();
	}
}

std::set<Node::Ptr> Node::connectedComponent()
{
	if (ctx) {
		return ctx->nodes;
	}
	std::set<Ptr> visited;
	std::function<void(const Ptr&)> rec = [&](const Ptr& cur) {
		visited.insert(cur);
		for (auto& o : cur->outputs) {
			if (!visited.count(o)) {
				rec(o);
			}
		}
		for (auto& i : cur->inputs) {
			if (!visited.count(i)) {
				rec(i);
			}
		}
	};
	rec(shared_from_this());
	return visited;
}

std::set<Node::Ptr> Node::disconnectConnectedNodes()
{
	auto nodes = connectedComponent();
	for (auto& n : nodes) {
		n->inputs.clear();
		n->outputs.clear();
		n->ctx.reset();
		n->dirty = true;
	}
	return nodes;
}

// ================================================================ rays nodes

void RaysNodeSingleInput::validateImpl() { input = exactlyOneInput<RaysNode>("IRaysNode"); }

void FromMat3x4fRaysNode::setParameters(const rgl_mat3x4f* r, size_t n)
{
	const void* before = rays.get();
	RGL_CHECK_CUDA(cudaMemcpy(rays.ensure(sizeof(rgl_mat3x4f) * n), r, sizeof(rgl_mat3x4f) * n, cudaMemcpyHostToDevice));
	sameCount = (n == count) && (rays.get() == before);
	count = n;
}

void FromMat3x4fRaysNode::validateImpl()
{
	if (!inputs.empty()) {
		throw InvalidPipeline(format("inputs for node %s are not allowed", name()));
	}
}

void TransformRaysNode::prepareImpl(cudaStream_t)
{
	if (folded) {
		return; // the consuming raytrace applies the transform
	}
	out.ensure(sizeof(Mat34) * std::max<size_t>(1, rayCount()));
	staged.host() = transform;
	(void) staged.device();
}

void TransformRaysNode::enqueueImpl(cudaStream_t s)
{
	if (folded) {
		return;
	}
	rgl::launchTransformRays(input->raysDev(), out.as<Mat34>(), (int) rayCount(), staged.enqueue(s), s);
}

void SetRangeRaysNode::setParameters(const rgl_vec2f* r, size_t n)
{
	for (size_t i = 0; i < n; ++i) {
		float mn = r[i].value[0], mx = r[i].value[1];
		if (std::isnan(mn) || std::isnan(mx)) {
			throw rgl::InvalidAPIArgument("range must be a number");
		}
		if (mn > mx) {
			throw rgl::InvalidAPIArgument("minimum range must be lower or equal to maximum range");
		}
		if (mn < 0.0f) {
			throw rgl::InvalidAPIArgument("minimum range must not be negative");
		}
	}
	RGL_CHECK_CUDA(cudaMemcpy(ranges.ensure(sizeof(rgl_vec2f) * n), r, sizeof(rgl_vec2f) * n, cudaMemcpyHostToDevice));
	count = n;
}

void SetRangeRaysNode::validateImpl()
{
	RaysNodeSingleInput::validateImpl();
	if (!(count == 1 || count == input->rayCount())) {
		throw InvalidPipeline(format("ranges doesn't match number of rays. RangesCount(%zu) should be one or equal to RayCount(%zu)",
		                             count, input->rayCount()));
	}
}

void RaytraceNode::setRayMask(const int8_t* mask, size_t n)
{
	RGL_CHECK_CUDA(cudaMemcpy(rayMask.ensure(n), mask, n, cudaMemcpyHostToDevice));
	rayMaskCount = n;
}

void SetRingIdsRaysNode::setParameters(const int32_t* r, size_t n)
{
	RGL_CHECK_CUDA(cudaMemcpy(ids.ensure(sizeof(int32_t) * n), r, sizeof(int32_t) * n, cudaMemcpyHostToDevice));
	count = n;
}

void SetRingIdsRaysNode::validateImpl()
{
	RaysNodeSingleInput::validateImpl();
	if (input->rayCount() % count != 0) {
		throw InvalidPipeline(format("ring ids doesn't match number of rays. RayCount(%zu) mod RingIdsCount(%zu) should be zero",
		                             input->rayCount(), count));
	}
}

void SetTimeOffsetsRaysNode::setParameters(const float* o, size_t n)
{
	RGL_CHECK_CUDA(cudaMemcpy(offsets.ensure(sizeof(float) * n), o, sizeof(float) * n, cudaMemcpyHostToDevice));
	count = n;
}

void SetTimeOffsetsRaysNode::validateImpl()
{
	RaysNodeSingleInput::validateImpl();
	if (input->rayCount() != count) {
		throw InvalidPipeline(format("time offsets don't match number of rays. RayCount(%zu) and TimeOffsetsCount(%zu) should be equal",
		                             input->rayCount(), count));
	}
}

void GaussianNoiseAngularRaysNode::setParameters(float m, float sd, rgl_axis_t a)
{
	mean = m;
	stDev = sd;
	axis = a;
}

// Noise parameters of one run, staged before the run (the frame advances by one per run, also across
// replays of a captured run). Reference frame algebra: src/gpu/gaussianNoiseKernels.cu:20-66.
static void stageNoise(rgl::StagedParam<rgl::NoiseParams>& staged, uint64_t seed, uint64_t& frame, uint32_t kind, float mean, float sd,
                       float rise, int axis, const Mat34& lookAt)
{
	rgl::NoiseParams& np = staged.host();
	np = rgl::NoiseParams{};
	np.seedLo = (uint32_t) seed;
	np.seedHi = (uint32_t) (seed >> 32);
	np.frameLo = (uint32_t) frame;
	np.frameHi = (uint32_t) (frame >> 32);
	np.kind = kind;
	np.mean = mean;
	np.stDev = sd;
	np.stDevRise = rise;
	np.axis = axis;
	np.lookAt = lookAt;
	np.lookAtInv = rgl::inverse(lookAt);
	(void) staged.device();
	++frame;
}

void GaussianNoiseAngularRaysNode::prepareImpl(cudaStream_t)
{
	out.ensure(sizeof(Mat34) * std::max<size_t>(1, rayCount()));
	stageNoise(staged, seed, frame, 1, mean, stDev, 0.0f, axis, rgl::inverse(input->cumulativeRayTransform()));
}

void GaussianNoiseAngularRaysNode::enqueueImpl(cudaStream_t s)
{
	rgl::launchNoiseAngularRay(input->raysDev(), out.as<Mat34>(), (int) rayCount(), staged.enqueue(s), s);
}

// ================================================================ points nodes

size_t PointsNode::pointCountHost()
{
	if (const int32_t* hc = hostCount()) {
		return (size_t) *hc;
	}
	const int32_t* dc = deviceCount();
	if (dc == nullptr) {
		return capacity();
	}
	int32_t c = 0;
	RGL_CHECK_CUDA(cudaMemcpy(&c, dc, sizeof(c), cudaMemcpyDeviceToHost));
	return (size_t) c;
}

void PointsNodeSingleInput::validateImpl()
{
	input = exactlyOneInput<PointsNode>("IPointsNode");
	for (auto f : requiredFields()) {
		if (!input->hasField(f) && !rgl::isDummy(f)) {
			throw InvalidPipeline(format("%s requires %s to be present", name(), rgl::fieldName(f)));
		}
	}
}

// ---- RaytraceNode

static bool raytraceSupports(rgl_field_t f)
{
	switch (f) {
		case RGL_FIELD_XYZ_VEC3_F32:
		case RGL_FIELD_DISTANCE_F32:
		case RGL_FIELD_IS_HIT_I32:
		case RGL_FIELD_ENTITY_ID_I32:
		case RGL_FIELD_RETURN_TYPE_U8:
		case RGL_FIELD_INTENSITY_F32:
		case RGL_FIELD_INTENSITY_U8:
		case RGL_FIELD_RAY_IDX_U32:
		case RGL_FIELD_NORMAL_VEC3_F32:
		case RGL_FIELD_INCIDENT_ANGLE_F32:
		case RGL_FIELD_LASER_RETRO_F32:
		case RGL_FIELD_AZIMUTH_F32:
		case RGL_FIELD_ELEVATION_F32:
		case RGL_FIELD_RING_ID_U16:
		case RGL_FIELD_TIME_STAMP_F64:
		case RGL_FIELD_TIME_STAMP_U32:
		case RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32:
		case RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32:
		case RGL_FIELD_RADIAL_SPEED_F32: return true;
		default: return false;
	}
}

std::set<rgl_field_t> RaytraceNode::findFieldsToCompute()
{
	// XYZ plus every field required by point nodes reachable downstream (reference RaytraceNode.cpp:165-191).
	std::set<rgl_field_t> out{RGL_FIELD_XYZ_VEC3_F32};
	std::set<Node*> seen;
	std::function<void(Node*)> dfs = [&](Node* cur) {
		for (auto& o : cur->outputs) {
			auto pn = std::dynamic_pointer_cast<PointsNode>(o);
			if (!pn || seen.count(o.get())) {
				continue;
			}
			seen.insert(o.get());
			for (auto f : pn->requiredFields()) {
				if (!rgl::isDummy(f)) {
					out.insert(f);
				}
			}
			dfs(o.get());
		}
	};
	dfs(this);
	return out;
}

int RaytraceNode::sampleCount() const
{
	bool div = (hDivergence / 2.0f) > 0.0f && (vDivergence / 2.0f) > 0.0f;
	return div ? 1 + sampleLayers * sampleVertices : 1;
}

void RaytraceNode::validateImpl()
{
	// Fields the raytrace does not produce (IS_GROUND_I32 of a ground filter downstream, radar fields)
	// are left to the nodes that produce them; a node that needs one from the raytrace itself fails its
	// own validation ("requires ... to be present").
	fields = findFieldsToCompute();
	for (auto it = fields.begin(); it != fields.end();) {
		it = raytraceSupports(*it) ? std::next(it) : fields.erase(it);
	}
	rays = exactlyOneInput<RaysNode>("IRaysNode");
	if (scene == nullptr) {
		scene = &Scene::defaultScene();
	}
	// Fold the sensor transform into the traversal prologue when this node is its only consumer
	// (through nodes that pass rays through unchanged): one kernel and one pass over the rays less.
	if (foldedTransform) {
		foldedTransform->folded = false;
		foldedTransform.reset();
	}
	{
		Node* cur = this;
		std::shared_ptr<RaysNode> up = rays;
		while (up && up->outputs.size() == 1 && up->outputs[0].get() == cur && up->passesRaysThrough()) {
			cur = up.get();
			up = up->inputs.size() == 1 ? std::dynamic_pointer_cast<RaysNode>(up->inputs[0]) : nullptr;
		}
		auto tf = std::dynamic_pointer_cast<TransformRaysNode>(up);
		if (tf && tf->outputs.size() == 1 && tf->outputs[0].get() == cur) {
			tf->folded = true;
			foldedTransform = tf;
		}
	}
	// Reference src/graph/RaytraceNode.cpp:37-45.
	if (fields.count(RGL_FIELD_RING_ID_U16) && rays->ringIdsDev() == nullptr) {
		throw InvalidPipeline("requested for field RING_ID_U16, but RaytraceNode cannot get ring ids");
	}
	if (fields.count(RGL_FIELD_TIME_STAMP_F64) && !scene->timeSet) {
		throw InvalidPipeline("requested for field TIME_STAMP_F64, but RaytraceNode cannot get time from scene");
	}
	if (rayMaskCount != 0 && rayMaskCount != rays->rayCount()) {
		throw InvalidPipeline("Mask size does not match the number of rays");
	}
	if (distortion && rays->timeOffsetsDev() == nullptr) {
		throw InvalidPipeline("requested for raytrace with velocity distortion, but RaytraceNode cannot get time offsets");
	}
	if (sampleCount() > rgl::kMaxBeamSamples) {
		throw rgl::InvalidAPIArgument(format("beam sample pattern of %d rays exceeds %d", sampleCount(), rgl::kMaxBeamSamples));
	}
	// Sub-ray table (reference optixPrograms.cu:75-86,230-248), evaluated on the host in float with the
	// reference's operation order so every consumer sees identical sub-ray poses.
	int ns = sampleCount();
	if (ns != uploadedSamples || hDivergence != uploadedH || vDivergence != uploadedV) {
		std::vector<Mat34> table(ns, Mat34::identity());
		if (ns > 1) {
			const float hHalf = hDivergence / 2.0f, vHalf = vDivergence / 2.0f;
			const float step = 2.0f * static_cast<float>(M_PI) / (float) sampleVertices;
			int k = 1;
			for (int l = 0; l < sampleLayers; ++l) {
				for (int v = 0; v < sampleVertices; ++v) {
					volatile float frac = 1.0f - (float) l / (float) sampleLayers;
					volatile float a = (float) v * step;
					float hAngle = (hHalf * frac) * cosf(a);
					float vAngle = (vHalf * frac) * sinf(a);
					table[k++] = rgl::beamSampleRotation(hAngle, vAngle);
				}
			}
		}
		RGL_CHECK_CUDA(cudaMemcpy(sampleTable.ensure(sizeof(Mat34) * ns), table.data(), sizeof(Mat34) * ns, cudaMemcpyHostToDevice));
		uploadedSamples = ns;
		uploadedH = hDivergence;
		uploadedV = vDivergence;
	}
	if (defaultRange.get() == nullptr) {
		const float r[2] = {0.0f, FLT_MAX};
		RGL_CHECK_CUDA(cudaMemcpy(defaultRange.ensure(sizeof(r)), r, sizeof(r), cudaMemcpyHostToDevice));
	}
	(void) errorFlag.device();
	if (scene == nullptr) {
		scene = &Scene::defaultScene();
	}
}

const void* RaytraceNode::fieldDev(rgl_field_t f)
{
	auto it = outputs.find(f);
	if (it == outputs.end() || !fields.count(f)) {
		throw InvalidPipeline(format("RaytraceNode does not provide field %s", rgl::fieldName(f)));
	}
	return it->second.get();
}

void RaytraceNode::prepareImpl(cudaStream_t s)
{
	const size_t cap = std::max<size_t>(1, (size_t) returnCount() * rays->rayCount());
	for (auto f : fields) {
		outputs[f].ensure(rgl::fieldSize(f) * cap);
	}
	for (auto it = outputs.begin(); it != outputs.end();) {
		it = fields.count(it->first) ? std::next(it) : outputs.erase(it);
	}
	if (timingEnabled() && !evStart) {
		RGL_CHECK_CUDA(cudaEventCreate(&evStart));
		RGL_CHECK_CUDA(cudaEventCreate(&evStop));
	}
	scene->prepare(s);
	stageJob(s);
}

rgl::TraceParams RaytraceNode::traceParams()
{
	const size_t n = rays->rayCount();
	rgl::TraceParams p{};
	p.rays = rays->raysDev();
	p.ranges = rays->rangesDev() ? rays->rangesDev() : defaultRange.as<float>();
	p.nRanges = rays->rangesDev() ? (int32_t) rays->rangesCount() : 1;
	p.nRays = (int32_t) n;
	p.nSamples = sampleCount();
	p.returnMode = mode;
	p.returnCount = returnCount();
	p.nearNonHitDistance = nearDistance;
	p.farNonHitDistance = farDistance;
	p.defaultIntensity = defaultIntensity;
	bool strongestSelected = false;
	for (int r = 0; r < p.returnCount; ++r) {
		uint32_t t = (((uint32_t) mode) >> (8 * r)) & 0xffu;
		strongestSelected = strongestSelected || t == RGL_RETURN_TYPE_STRONGEST || t == RGL_RETURN_TYPE_SECOND_STRONGEST;
	}
	p.needIntensity = (fields.count(RGL_FIELD_INTENSITY_F32) || fields.count(RGL_FIELD_INTENSITY_U8) || strongestSelected) ? 1 : 0;
	p.errorFlag = errorFlag.device();
	p.scene = scene->view();
	auto ptr = [&](rgl_field_t f) -> void* { return fields.count(f) ? outputs[f].get() : nullptr; };
	p.out.xyz = static_cast<float*>(ptr(RGL_FIELD_XYZ_VEC3_F32));
	p.out.distance = static_cast<float*>(ptr(RGL_FIELD_DISTANCE_F32));
	p.out.isHit = static_cast<int32_t*>(ptr(RGL_FIELD_IS_HIT_I32));
	p.out.entityId = static_cast<int32_t*>(ptr(RGL_FIELD_ENTITY_ID_I32));
	p.out.returnType = static_cast<uint8_t*>(ptr(RGL_FIELD_RETURN_TYPE_U8));
	p.out.intensityF32 = static_cast<float*>(ptr(RGL_FIELD_INTENSITY_F32));
	p.out.rayIdx = static_cast<uint32_t*>(ptr(RGL_FIELD_RAY_IDX_U32));
	p.out.intensityU8 = static_cast<uint8_t*>(ptr(RGL_FIELD_INTENSITY_U8));
	p.out.normal = static_cast<float*>(ptr(RGL_FIELD_NORMAL_VEC3_F32));
	p.out.incidentAngle = static_cast<float*>(ptr(RGL_FIELD_INCIDENT_ANGLE_F32));
	p.out.laserRetro = static_cast<float*>(ptr(RGL_FIELD_LASER_RETRO_F32));
	p.out.ringId = static_cast<uint16_t*>(ptr(RGL_FIELD_RING_ID_U16));
	p.out.azimuth = static_cast<float*>(ptr(RGL_FIELD_AZIMUTH_F32));
	p.out.elevation = static_cast<float*>(ptr(RGL_FIELD_ELEVATION_F32));
	p.out.timeStampF64 = static_cast<double*>(ptr(RGL_FIELD_TIME_STAMP_F64));
	p.out.timeStampU32 = static_cast<uint32_t*>(ptr(RGL_FIELD_TIME_STAMP_U32));
	p.out.absVelocity = static_cast<float*>(ptr(RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32));
	p.out.relVelocity = static_cast<float*>(ptr(RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32));
	p.out.radialSpeed = static_cast<float*>(ptr(RGL_FIELD_RADIAL_SPEED_F32));
	p.ringIds = rays->ringIdsDev();
	p.nRingIds = (int32_t) rays->ringIdsCount();
	p.sensorToWorld = rays->cumulativeRayTransform();
	p.worldToSensor = rgl::inverse(p.sensorToWorld);
	Mat34 rot = p.sensorToWorld;
	rot.m[0][3] = rot.m[1][3] = rot.m[2][3] = 0.0f;
	p.worldToSensorRotation = rgl::inverse(rot);
	p.distortion = distortion ? 1 : 0;
	p.timeOffsetsMs = rays->timeOffsetsDev();
	p.sceneDeltaTime = scene->deltaTimeSeconds();
	p.sensorLinearVelocity = sensorLinearVelocity;
	p.sensorAngularVelocity = sensorAngularVelocity;
	p.rayMask = rayMaskCount ? rayMask.as<int8_t>() : nullptr;
	return p;
}

// The traversal is the persistent kernel of batched frames with this node as its only job: the job
// record and the task count are staged every run (new ray contents need no re-capture).
void RaytraceNode::fillJob(rgl::BatchJob& b)
{
	b = rgl::BatchJob{};
	b.p = traceParams();
	b.samples = sampleTable.as<Mat34>();
	b.order = nullptr;
	b.groupSize = std::min(b.p.nSamples, 32);
	if (foldedTransform) {
		b.p.rays = foldedTransform->sourceRaysDev();
		b.hasRayTransform = 1;
		b.rayTransform = foldedTransform->matrix();
	}
}

void RaytraceNode::ensureOrder(const rgl::BatchJob& b, cudaStream_t s)
{
	const int n = b.p.nRays;
	if (orderValid && orderCount == n && orderKind == schedule.order && orderRays == b.p.rays) {
		return;
	}
	orderValid = false;
	orderCount = n;
	orderKind = schedule.order;
	orderRays = b.p.rays;
	constexpr int kKeyBits = 22; // one job: no job bits above the 22-bit direction or position key
	const float lo[3] = {scene->worldLower()[0], scene->worldLower()[1], scene->worldLower()[2]};
	const float hi[3] = {scene->worldUpper()[0], scene->worldUpper()[1], scene->worldUpper()[2]};
	auto* keys = static_cast<uint32_t*>(orderKeys.ensure(sizeof(uint32_t) * n));
	auto* vals = static_cast<uint32_t*>(orderVals.ensure(sizeof(uint32_t) * n));
	auto* err = static_cast<int32_t*>(orderError.ensure(sizeof(int32_t)));
	RGL_CHECK_CUDA(cudaMemsetAsync(err, 0, sizeof(int32_t), s));
	rgl::launchBeamKeys(b.p.rays, b.hasRayTransform ? &b.rayTransform : nullptr, n, 0, schedule.order, lo, hi, keys, vals, s);
	rgl::sortPairs(keys, vals, n, kKeyBits, orderScratch.ensure(rgl::sortPairsScratchBytes(n, kKeyBits)), err, s);
	int32_t failed = 0;
	RGL_CHECK_CUDA(cudaMemcpyAsync(&failed, err, sizeof(failed), cudaMemcpyDeviceToHost, s));
	RGL_CHECK_CUDA(cudaStreamSynchronize(s));
	// A sort whose look-back gave up leaves no permutation: cast in the given order instead.
	orderValid = failed == 0;
	if (!orderValid) {
		rgl::logMessage(rgl::LogLevel::Warn, "RaytraceNode: beam ordering sort did not complete; casting beams in the given order");
	}
}

void RaytraceNode::stageJob(cudaStream_t s)
{
	rgl::BatchJob& b = job.host().job;
	schedule = traceSchedule();
	fillJob(b);
	if (schedule.order != rgl::kOrderNatural && b.p.nRays > 0) {
		ensureOrder(b, s);
		b.order = orderValid ? orderVals.as<uint32_t>() : nullptr;
	}
	const rgl::TraceParams& p = b.p;
	(void) job.device();
	const int per = rgl::batchBeamsPerTask(schedule.packing, p.nSamples);
	rgl::TaskRange& tr = job.host().tasks;
	tr.base[0] = 0;
	tr.base[1] = (p.nRays + per - 1) / per;
	shading = rgl::needsShadingKernel(p);
	if (counter.get() == nullptr) {
		RGL_CHECK_CUDA(cudaMemset(counter.ensure(rgl::kTraceCounterBytes), 0, rgl::kTraceCounterBytes));
	}
	rgl::prepareTraceBatch(1, p.nSamples, shading, schedule);
}

void RaytraceNode::enqueueImpl(cudaStream_t s)
{
	const StagedTrace* staged = job.enqueue(s);
	const rgl::BatchJob* dJob = &staged->job;
	const rgl::TaskRange* dTasks = &staged->tasks;
	if (timingEnabled() && evStart) {
		recordEvent(evStart, s);
	}
	rgl::launchTraceBatch(dJob, dTasks->base, 1, job.host().job.p.nSamples, shading, schedule, counter.as<uint32_t>(), s);
	RGL_CHECK_CUDA(cudaGetLastError());
	if (timingEnabled() && evStart) {
		recordEvent(evStop, s);
	}
}

void RaytraceNode::checkErrors()
{
	if (errorFlag.raised()) {
		errorFlag.clear();
		throw std::runtime_error("RaytraceNode: traversal stack overflow on the device (scene BVH too deep)");
	}
	if (scene) {
		scene->checkDeviceErrors();
	}
}

// ---- YieldPointsNode

void YieldPointsNode::setParameters(const std::vector<rgl_field_t>& f)
{
	if (std::find(f.begin(), f.end(), RGL_FIELD_DYNAMIC_FORMAT) != f.end()) {
		throw rgl::InvalidAPIArgument("cannot yield field 'RGL_FIELD_DYNAMIC_FORMAT'");
	}
	for (auto x : f) {
		(void) rgl::fieldSize(x);
	}
	fields = f;
}

bool YieldPointsNode::hasField(rgl_field_t f) const { return std::find(fields.begin(), fields.end(), f) != fields.end(); }

// ---- FormatPointsNode

void FormatPointsNode::setParameters(const std::vector<rgl_field_t>& f)
{
	if (std::find(f.begin(), f.end(), RGL_FIELD_DYNAMIC_FORMAT) != f.end()) {
		throw rgl::InvalidAPIArgument("cannot format field 'RGL_FIELD_DYNAMIC_FORMAT'");
	}
	for (auto x : f) {
		(void) rgl::fieldSize(x);
	}
	fields = f;
}

bool FormatPointsNode::hasField(rgl_field_t f) const
{
	return f == RGL_FIELD_DYNAMIC_FORMAT || std::find(fields.begin(), fields.end(), f) != fields.end();
}

size_t FormatPointsNode::fieldPointSize(rgl_field_t f) const
{
	return f == RGL_FIELD_DYNAMIC_FORMAT ? rgl::pointSize(fields) : rgl::fieldSize(f);
}

const void* FormatPointsNode::fieldDev(rgl_field_t f)
{
	if (f == RGL_FIELD_DYNAMIC_FORMAT) {
		return out.get();
	}
	return input->fieldDev(f);
}

void FormatPointsNode::prepareImpl(cudaStream_t) { out.ensure(std::max<size_t>(1, rgl::pointSize(fields) * input->capacity())); }

void FormatPointsNode::enqueueImpl(cudaStream_t s)
{
	const size_t ps = rgl::pointSize(fields);
	const size_t cap = input->capacity();
	if (fields.size() > (size_t) rgl::kMaxFieldCopies) {
		throw rgl::InvalidAPIArgument(format("format of %zu fields exceeds %d", fields.size(), rgl::kMaxFieldCopies));
	}
	rgl::FieldCopies fc{};
	int off = 0;
	for (auto f : fields) {
		rgl::FieldCopy c{};
		c.src = rgl::isDummy(f) ? nullptr : input->fieldDev(f);
		c.size = (int32_t) rgl::fieldSize(f);
		c.offset = off;
		off += c.size;
		fc.f[fc.count++] = c;
	}
	rgl::launchFormat(fc, (int) ps, (int) cap, input->deviceCount(), out.as<uint8_t>(), s);
}

// ---- CompactByFieldPointsNode

void CompactByFieldPointsNode::validateImpl()
{
	PointsNodeSingleInput::validateImpl();
	// Fields needed downstream are compacted eagerly in the run's single compaction kernel.
	eager.clear();
	std::set<Node*> seen;
	std::function<void(Node*)> dfs = [&](Node* cur) {
		for (auto& o : cur->outputs) {
			auto pn = std::dynamic_pointer_cast<PointsNode>(o);
			if (!pn || seen.count(o.get())) {
				continue;
			}
			seen.insert(o.get());
			for (auto f : pn->requiredFields()) {
				if (!rgl::isDummy(f) && input->hasField(f)) {
					eager.insert(f);
				}
			}
			dfs(o.get());
		}
	};
	dfs(this);
	// Transform and noise nodes that feed only this compaction (one consumer each, up the chain) run
	// inside its pass, on the kept points only; nodes are validated in execution order, so each one
	// has already reset its own flag this run.
	chain.clear();
	chainSource = input;
	while (auto pw = std::dynamic_pointer_cast<PointwisePointsNode>(chainSource)) {
		if (pw->outputs.size() != 1 || chain.size() == (size_t) rgl::kMaxPointOps) {
			break;
		}
		chain.insert(chain.begin(), pw);
		chainSource = pw->source();
	}
	for (auto& pw : chain) {
		pw->absorbed = true;
	}
	if (count.get() == nullptr) {
		count.ensure(sizeof(int32_t));
		RGL_CHECK_CUDA(cudaMemset(count.get(), 0, sizeof(int32_t)));
	}
	(void) errorFlag.device();
}

void CompactByFieldPointsNode::sizeBuffers(const std::vector<rgl_field_t>& which)
{
	const size_t cap = input->capacity();
	for (auto f : which) {
		outputs[f].ensure(std::max<size_t>(1, rgl::fieldSize(f) * cap));
	}
	// The compaction kernel leaves its scratch zeroed; a new allocation is zeroed once here.
	const void* old = scratch.get();
	const size_t bytes = rgl::compactScratchBytes((int) cap);
	if (scratch.ensure(bytes) != old) {
		RGL_CHECK_CUDA(cudaMemset(scratch.get(), 0, scratch.capacity()));
	}
}

// Per-run host state lives here, not in enqueueImpl: a replayed capture does not call enqueueImpl.
void CompactByFieldPointsNode::prepareImpl(cudaStream_t s)
{
	sizeBuffers(std::vector<rgl_field_t>(eager.begin(), eager.end()));
	if (hCountDev == nullptr) {
		void* d = nullptr;
		RGL_CHECK_CUDA(cudaHostGetDevicePointer(&d, hCount.ensure(sizeof(int32_t)), 0));
		hCountDev = static_cast<int32_t*>(d);
	}
	lastStream = s;
	lazyDone.clear();
}

void CompactByFieldPointsNode::compact(const std::vector<rgl_field_t>& which, cudaStream_t s, int32_t* hostCount)
{
	const size_t cap = input->capacity();
	rgl::FieldCopies fc{};
	rgl::PointOps ops{};
	ops.xyzField = -1;
	ops.distField = -1;
	const bool absorbs = !chain.empty();
	for (auto f : which) {
		if (fc.count == rgl::kMaxFieldCopies) {
			throw rgl::InvalidAPIArgument(format("compaction of more than %d fields", rgl::kMaxFieldCopies));
		}
		rgl::FieldCopy c{};
		c.size = (int32_t) rgl::fieldSize(f);
		if (absorbs && (f == RGL_FIELD_XYZ_VEC3_F32 || f == RGL_FIELD_DISTANCE_F32)) {
			(f == RGL_FIELD_XYZ_VEC3_F32 ? ops.xyzField : ops.distField) = fc.count;
			c.src = nullptr; // computed from the chain's source
		} else {
			c.src = input->fieldDev(f);
		}
		c.dst = outputs[f].get();
		fc.f[fc.count++] = c;
	}
	if (absorbs && (ops.xyzField >= 0 || ops.distField >= 0)) {
		for (auto& pw : chain) {
			pw->appendPointOp(ops, s);
		}
		ops.srcXyz = static_cast<const float*>(chainSource->fieldDev(RGL_FIELD_XYZ_VEC3_F32));
		ops.srcDist = chainSource->hasField(RGL_FIELD_DISTANCE_F32) ? static_cast<const float*>(chainSource->fieldDev(RGL_FIELD_DISTANCE_F32))
		                                                            : nullptr;
	}
	rgl::launchCompact(static_cast<const int32_t*>(input->fieldDev(field)), (int) cap, input->deviceCount(), fc,
	                   ops.count > 0 || ops.xyzField >= 0 || ops.distField >= 0 ? &ops : nullptr, count.as<int32_t>(), scratch.get(),
	                   errorFlag.device(), s, hostCount);
}

void CompactByFieldPointsNode::enqueueImpl(cudaStream_t s)
{
	// The count reaches the host with the run, stored by the kernel into the mapped pinned word:
	// reading results needs no blocking copy, and the run has no copy node waiting on the copy engine.
	compact(std::vector<rgl_field_t>(eager.begin(), eager.end()), s, hCountDev);
}

const void* CompactByFieldPointsNode::fieldDev(rgl_field_t f)
{
	if (eager.count(f) || lazyDone.count(f)) {
		return outputs[f].get();
	}
	if (!input->hasField(f)) {
		throw InvalidPipeline(format("CompactByFieldPointsNode: input does not provide field %s", rgl::fieldName(f)));
	}
	// A field nobody downstream declared: compact it now on the graph's stream and wait for it.
	sizeBuffers({f});
	compact({f}, lastStream);
	RGL_CHECK_CUDA(cudaStreamSynchronize(lastStream));
	lazyDone.insert(f);
	return outputs[f].get();
}

void CompactByFieldPointsNode::checkErrors()
{
	if (errorFlag.raised()) {
		errorFlag.clear();
		throw std::runtime_error("CompactByFieldPointsNode: decoupled look-back did not complete on the device");
	}
}

// ---- Pointwise nodes (transform, point noise)

void PointwisePointsNode::computeOnDemand()
{
	if (computedOnDemand) {
		return;
	}
	if (lastStream == nullptr) {
		throw InvalidPipeline(format("Cannot get results from %s; it hasn't been run yet", name()));
	}
	allocateOutputs();
	launchOwn(lastStream);
	RGL_CHECK_CUDA(cudaStreamSynchronize(lastStream));
	computedOnDemand = true;
}

// ---- TransformPointsNode

void TransformPointsNode::allocateOutputs() { out.ensure(std::max<size_t>(1, 12 * input->capacity())); }

void TransformPointsNode::prepareImpl(cudaStream_t s)
{
	beginRun(s);
	if (!absorbed) {
		allocateOutputs();
	}
	staged.host() = transform;
	(void) staged.device();
}

void TransformPointsNode::launchOwn(cudaStream_t s)
{
	const size_t cap = input->capacity();
	rgl::launchTransformPoints(static_cast<const float*>(input->fieldDev(RGL_FIELD_XYZ_VEC3_F32)), out.as<float>(), (int) cap,
	                           input->deviceCount(), staged.enqueue(s), s);
}

void TransformPointsNode::enqueueImpl(cudaStream_t s)
{
	if (!absorbed) {
		launchOwn(s);
	}
}

void TransformPointsNode::appendPointOp(rgl::PointOps& ops, cudaStream_t s)
{
	ops.op[ops.count++] = rgl::PointOp{rgl::kOpTransform, 0, staged.enqueue(s)};
}

const void* TransformPointsNode::fieldDev(rgl_field_t f)
{
	if (f != RGL_FIELD_XYZ_VEC3_F32) {
		return input->fieldDev(f);
	}
	if (absorbed) {
		computeOnDemand();
	}
	return out.get();
}

// ---- Gaussian noise on points

void GaussianNoiseAngularHitpointNode::setParameters(float m, float sd, rgl_axis_t a)
{
	mean = m;
	stDev = sd;
	axis = a;
}

void GaussianNoiseAngularHitpointNode::allocateOutputs()
{
	const size_t cap = input->capacity();
	outXyz.ensure(std::max<size_t>(1, 12 * cap));
	if (withDistance) {
		outDist.ensure(std::max<size_t>(1, 4 * cap));
	}
}

void GaussianNoiseAngularHitpointNode::prepareImpl(cudaStream_t s)
{
	beginRun(s);
	withDistance = input->hasField(RGL_FIELD_DISTANCE_F32);
	if (!absorbed) {
		allocateOutputs();
	}
	stageNoise(staged, seed, frame, 2, mean, stDev, 0.0f, axis, input->lookAtOriginTransform());
}

void GaussianNoiseAngularHitpointNode::launchOwn(cudaStream_t s)
{
	const size_t cap = input->capacity();
	rgl::launchNoiseAngularHitpoint(static_cast<const float*>(input->fieldDev(RGL_FIELD_XYZ_VEC3_F32)), outXyz.as<float>(),
	                                withDistance ? outDist.as<float>() : nullptr, (int) cap, input->deviceCount(), staged.enqueue(s), s);
}

void GaussianNoiseAngularHitpointNode::enqueueImpl(cudaStream_t s)
{
	if (!absorbed) {
		launchOwn(s);
	}
}

void GaussianNoiseAngularHitpointNode::appendPointOp(rgl::PointOps& ops, cudaStream_t s)
{
	ops.op[ops.count++] = rgl::PointOp{rgl::kOpNoiseAngularHitpoint, withDistance ? 1 : 0, staged.enqueue(s)};
}

const void* GaussianNoiseAngularHitpointNode::fieldDev(rgl_field_t f)
{
	const bool own = f == RGL_FIELD_XYZ_VEC3_F32 || (f == RGL_FIELD_DISTANCE_F32 && withDistance);
	if (!own) {
		return input->fieldDev(f);
	}
	if (absorbed) {
		computeOnDemand();
	}
	return f == RGL_FIELD_XYZ_VEC3_F32 ? outXyz.get() : outDist.get();
}

void GaussianNoiseDistanceNode::setParameters(float m, float b, float r)
{
	mean = m;
	base = b;
	rise = r;
}

void GaussianNoiseDistanceNode::allocateOutputs()
{
	const size_t cap = input->capacity();
	outXyz.ensure(std::max<size_t>(1, 12 * cap));
	outDist.ensure(std::max<size_t>(1, 4 * cap));
}

void GaussianNoiseDistanceNode::prepareImpl(cudaStream_t s)
{
	beginRun(s);
	if (!absorbed) {
		allocateOutputs();
	}
	stageNoise(staged, seed, frame, 3, mean, base, rise, 0, input->lookAtOriginTransform());
}

void GaussianNoiseDistanceNode::launchOwn(cudaStream_t s)
{
	const size_t cap = input->capacity();
	rgl::launchNoiseDistance(static_cast<const float*>(input->fieldDev(RGL_FIELD_XYZ_VEC3_F32)),
	                         static_cast<const float*>(input->fieldDev(RGL_FIELD_DISTANCE_F32)), outXyz.as<float>(),
	                         outDist.as<float>(), (int) cap, input->deviceCount(), staged.enqueue(s), s);
}

void GaussianNoiseDistanceNode::enqueueImpl(cudaStream_t s)
{
	if (!absorbed) {
		launchOwn(s);
	}
}

void GaussianNoiseDistanceNode::appendPointOp(rgl::PointOps& ops, cudaStream_t s)
{
	ops.op[ops.count++] = rgl::PointOp{rgl::kOpNoiseDistance, 1, staged.enqueue(s)};
}

const void* GaussianNoiseDistanceNode::fieldDev(rgl_field_t f)
{
	if (f != RGL_FIELD_XYZ_VEC3_F32 && f != RGL_FIELD_DISTANCE_F32) {
		return input->fieldDev(f);
	}
	if (absorbed) {
		computeOnDemand();
	}
	return f == RGL_FIELD_XYZ_VEC3_F32 ? outXyz.get() : outDist.get();
}

// ---- FromArrayPointsNode (reference src/graph/FromArrayPointsNode.cpp:18-46)

void FromArrayPointsNode::setParameters(const void* points, size_t n, const std::vector<rgl_field_t>& fields)
{
	if (std::find(fields.begin(), fields.end(), RGL_FIELD_DYNAMIC_FORMAT) != fields.end()) {
		throw rgl::InvalidAPIArgument("cannot create point cloud from field 'RGL_FIELD_DYNAMIC_FORMAT'");
	}
	if (fields.size() > (size_t) rgl::kMaxFieldCopies) {
		throw rgl::InvalidAPIArgument(format("more than %d fields", rgl::kMaxFieldCopies));
	}
	const size_t ps = rgl::pointSize(fields);
	data.clear();
	count = n;
	rgl::DeviceBuffer staging;
	RGL_CHECK_CUDA(cudaMemcpy(staging.ensure(ps * n), points, ps * n, cudaMemcpyHostToDevice));
	rgl::FieldCopies fc{};
	int off = 0;
	for (auto f : fields) {
		rgl::FieldCopy c{};
		c.size = (int32_t) rgl::fieldSize(f);
		c.offset = off;
		off += c.size;
		if (!rgl::isDummy(f) && !data.count(f)) {
			c.dst = data[f].ensure(std::max<size_t>(1, c.size * n));
		}
		fc.f[fc.count++] = c;
	}
	rgl::launchAosToSoa(staging.as<uint8_t>(), (int) ps, (int) n, fc, nullptr);
	RGL_CHECK_CUDA(cudaDeviceSynchronize());
}

void FromArrayPointsNode::validateImpl()
{
	if (!inputs.empty()) {
		throw InvalidPipeline(format("inputs for node %s are not allowed", name()));
	}
}

const void* FromArrayPointsNode::fieldDev(rgl_field_t f)
{
	auto it = data.find(f);
	if (it == data.end()) {
		throw InvalidPipeline(format("FromArrayPointsNode does not provide field %s", rgl::fieldName(f)));
	}
	return it->second.get();
}

// ---- FilterGroundPointsNode

void FilterGroundPointsNode::prepareImpl(cudaStream_t)
{
	flags.ensure(std::max<size_t>(1, sizeof(int32_t) * input->capacity()));
}

void FilterGroundPointsNode::enqueueImpl(cudaStream_t s)
{
	rgl::launchGroundFlags(static_cast<const float*>(input->fieldDev(RGL_FIELD_NORMAL_VEC3_F32)), (int) input->capacity(),
	                       input->deviceCount(), up, angle, flags.as<int32_t>(), s);
}

const void* FilterGroundPointsNode::fieldDev(rgl_field_t f)
{
	return f == RGL_FIELD_IS_GROUND_I32 ? flags.get() : input->fieldDev(f);
}

// ---- SpatialMergePointsNode

static std::vector<rgl_field_t> mergeFields(const std::vector<rgl_field_t>& f, const char* what)
{
	if (std::find(f.begin(), f.end(), RGL_FIELD_DYNAMIC_FORMAT) != f.end()) {
		throw rgl::InvalidAPIArgument(format("cannot perform %s merge on field 'RGL_FIELD_DYNAMIC_FORMAT'", what));
	}
	std::vector<rgl_field_t> out;
	for (auto x : f) {
		(void) rgl::fieldSize(x);
		if (!rgl::isDummy(x) && std::find(out.begin(), out.end(), x) == out.end()) {
			out.push_back(x);
		}
	}
	if (out.size() > (size_t) rgl::kMaxFieldCopies) {
		throw rgl::InvalidAPIArgument(format("merge of more than %d fields", rgl::kMaxFieldCopies));
	}
	return out;
}

void SpatialMergePointsNode::setParameters(const std::vector<rgl_field_t>& f)
{
	fields = mergeFields(f, "spatial");
	outputs.clear();
	for (auto x : fields) {
		outputs[x];
	}
}

void SpatialMergePointsNode::validateImpl()
{
	pointInputs.clear();
	for (auto& in : inputs) {
		if (auto p = std::dynamic_pointer_cast<PointsNode>(in)) {
			pointInputs.push_back(p);
		}
	}
	if (pointInputs.size() < 2) {
		// One input would make the node a no-op (reference SpatialMergePointsNode.cpp:39-43).
		throw InvalidPipeline(format("%s requires >= 2 input nodes, found %zu", name(), pointInputs.size()));
	}
	onDevice = false;
	for (auto& in : pointInputs) {
		for (auto f : fields) {
			if (!in->hasField(f)) {
				throw InvalidPipeline(format("%s input does not have required field '%s'", name(), rgl::fieldName(f)));
			}
		}
		onDevice = onDevice || in->deviceCount() != nullptr;
	}
	count.ensure(sizeof(int32_t));
	hCount.ensure(sizeof(int32_t));
}

bool SpatialMergePointsNode::isDense() const
{
	for (auto& in : pointInputs) {
		if (!in->isDense()) {
			return false;
		}
	}
	return true;
}

size_t SpatialMergePointsNode::capacity() const
{
	size_t c = 0;
	for (auto& in : pointInputs) {
		c += in->capacity();
	}
	return c;
}

void SpatialMergePointsNode::prepareImpl(cudaStream_t s)
{
	const size_t cap = capacity();
	if (cap > (size_t) INT32_MAX) {
		throw rgl::InvalidAPIArgument(format("%s: %zu points exceed the 32-bit point count", name(), cap));
	}
	std::vector<rgl::MergeInput> ins;
	std::vector<const void*> src;
	std::vector<rgl::FieldCopy> fl;
	maxCount = 0;
	for (auto& in : pointInputs) {
		ins.push_back({in->deviceCount(), (int32_t) in->capacity(), 0});
		maxCount = std::max(maxCount, (int) in->capacity());
		for (auto f : fields) {
			src.push_back(in->fieldDev(f));
		}
	}
	for (auto f : fields) {
		rgl::FieldCopy c{};
		c.size = (int32_t) rgl::fieldSize(f);
		c.dst = outputs[f].ensure(std::max<size_t>(1, rgl::fieldSize(f) * cap));
		fl.push_back(c);
	}
	const size_t bytes = rgl::mergeTableBytes((int) ins.size(), (int) fl.size());
	rgl::fillMergeTable(hTable.ensure(bytes), ins, src, fl);
	// The previous run has completed (runs synchronise first), so the pinned table is free to reuse.
	RGL_CHECK_CUDA(cudaMemcpyAsync(table.ensure(bytes), hTable.get(), bytes, cudaMemcpyHostToDevice, s));
}

void SpatialMergePointsNode::enqueueImpl(cudaStream_t s)
{
	rgl::launchMergePoints(table.get(), (int) pointInputs.size(), (int) fields.size(), maxCount, nullptr, count.as<int32_t>(), s);
	if (onDevice) {
		RGL_CHECK_CUDA(cudaMemcpyAsync(hCount.get(), count.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
	}
}

const void* SpatialMergePointsNode::fieldDev(rgl_field_t f)
{
	auto it = outputs.find(f);
	if (it == outputs.end()) {
		throw InvalidPipeline(format("%s does not provide field %s", name(), rgl::fieldName(f)));
	}
	return it->second.get();
}

// ---- TemporalMergePointsNode

void TemporalMergePointsNode::setParameters(const std::vector<rgl_field_t>& f)
{
	fields = mergeFields(f, "temporal");
	outputs.clear();
	for (auto x : fields) {
		outputs[x] = std::make_unique<rgl::DeviceBuffer>();
	}
	bound = 0;
	allocated = 0;
	reset = true;
}

void TemporalMergePointsNode::validateImpl()
{
	PointsNodeSingleInput::validateImpl();
	count.ensure(sizeof(int32_t));
	hCount.ensure(sizeof(int32_t));
}

void TemporalMergePointsNode::prepareImpl(cudaStream_t s)
{
	if (reset) {
		RGL_CHECK_CUDA(cudaMemsetAsync(count.get(), 0, sizeof(int32_t), s));
		reset = false;
	}
	const size_t kept = bound;
	bound += input->capacity();
	if (bound > (size_t) INT32_MAX) {
		throw rgl::InvalidAPIArgument(format("%s: %zu accumulated points exceed the 32-bit point count", name(), bound));
	}
	if (bound > allocated) {
		const size_t want = std::max(bound, 2 * allocated);
		for (auto f : fields) {
			auto grown = std::make_unique<rgl::DeviceBuffer>();
			grown->ensure(std::max<size_t>(1, rgl::fieldSize(f) * want));
			if (kept > 0) {
				RGL_CHECK_CUDA(cudaMemcpyAsync(grown->get(), outputs[f]->get(), rgl::fieldSize(f) * kept, cudaMemcpyDeviceToDevice, s));
			}
			// The old storage may be freed only after the copy has read it.
			RGL_CHECK_CUDA(cudaStreamSynchronize(s));
			outputs[f] = std::move(grown);
		}
		allocated = want;
	}
	std::vector<const void*> src;
	std::vector<rgl::FieldCopy> fl;
	for (auto f : fields) {
		src.push_back(input->fieldDev(f));
		rgl::FieldCopy c{};
		c.size = (int32_t) rgl::fieldSize(f);
		c.dst = outputs[f]->get();
		fl.push_back(c);
	}
	const std::vector<rgl::MergeInput> ins{{input->deviceCount(), (int32_t) input->capacity(), 0}};
	const size_t bytes = rgl::mergeTableBytes(1, (int) fl.size());
	rgl::fillMergeTable(hTable.ensure(bytes), ins, src, fl);
	RGL_CHECK_CUDA(cudaMemcpyAsync(table.ensure(bytes), hTable.get(), bytes, cudaMemcpyHostToDevice, s));
}

void TemporalMergePointsNode::enqueueImpl(cudaStream_t s)
{
	const int32_t inCap = (int32_t) input->capacity();
	rgl::launchMergePoints(table.get(), 1, (int) fields.size(), inCap, count.as<int32_t>(), nullptr, s);
	rgl::launchAddCount(count.as<int32_t>(), input->deviceCount(), inCap, s);
	RGL_CHECK_CUDA(cudaMemcpyAsync(hCount.get(), count.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
}

const void* TemporalMergePointsNode::fieldDev(rgl_field_t f)
{
	auto it = outputs.find(f);
	if (it == outputs.end()) {
		throw InvalidPipeline(format("%s does not provide field %s", name(), rgl::fieldName(f)));
	}
	return it->second->get();
}

// ================================================================ GraphRunCtx
// (reference src/graph/GraphRunCtx.cpp:23-211)

std::vector<std::shared_ptr<GraphRunCtx>>& GraphRunCtx::instances()
{
	static std::vector<std::shared_ptr<GraphRunCtx>> v;
	return v;
}

GraphRunCtx::GraphRunCtx()
{
	RGL_CHECK_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
	RGL_CHECK_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
	RGL_CHECK_CUDA(cudaEventCreate(&runStart));
	RGL_CHECK_CUDA(cudaEventCreate(&runStop));
}

GraphRunCtx::~GraphRunCtx()
{
	releaseGraph();
	cudaEventDestroy(done);
	cudaEventDestroy(runStart);
	cudaEventDestroy(runStop);
	cudaStreamDestroy(stream_);
}

std::shared_ptr<GraphRunCtx> GraphRunCtx::createAndAttach(const Node::Ptr& node)
{
	auto ctx = std::shared_ptr<GraphRunCtx>(new GraphRunCtx());
	ctx->nodes = node->connectedComponent();
	for (auto& n : ctx->nodes) {
		if (n->ctx) {
			throw std::logic_error(format("attempted to replace existing graphRunCtx in node %s when creating for %s", n->name(),
			                              node->name()));
		}
		n->ctx = ctx;
		n->dirty = true;
	}
	instances().push_back(ctx);
	return ctx;
}

std::vector<Node::Ptr> GraphRunCtx::findExecutionOrder(std::set<Node::Ptr> nodes)
{
	std::vector<Node::Ptr> reverseOrder;
	std::function<void(const Node::Ptr&)> dfs = [&](const Node::Ptr& cur) {
		nodes.erase(cur);
		for (auto it = cur->outputs.rbegin(); it != cur->outputs.rend(); ++it) {
			if (nodes.count(*it)) {
				dfs(*it);
			}
		}
		reverseOrder.push_back(cur);
	};
	std::vector<Node::Ptr> entries;
	for (auto& n : nodes) {
		if (n->inputs.empty()) {
			entries.push_back(n);
		}
	}
	std::stable_sort(entries.begin(), entries.end(), [](const Node::Ptr& a, const Node::Ptr& b) { return a->priority < b->priority; });
	for (auto& e : entries) {
		if (nodes.count(e)) {
			dfs(e);
		}
	}
	if (!nodes.empty()) {
		throw std::logic_error("bug: detected unreachable nodes");
	}
	return {reverseOrder.rbegin(), reverseOrder.rend()};
}

void GraphRunCtx::releaseGraph()
{
	if (exec) {
		cudaGraphExecDestroy(exec);
		exec = nullptr;
	}
}

// One run: validation and the prepare phase on the host, then the nodes' device work. The device
// work is captured into a CUDA graph once and replayed by later runs while no node's kernel
// parameters changed (parameter versions) and no device buffer moved (allocation epoch); otherwise it is
// captured again. With CUDA graphs disabled (RGL_GB300_CUDA_GRAPH=0) the work is enqueued directly.
void GraphRunCtx::run()
{
	synchronize();
	if (order.empty()) {
		order = findExecutionOrder(nodes);
		releaseGraph();
	}
	uint64_t version = 0;
	for (auto& n : order) {
		n->validateImpl();
		n->dirty = false;
		version = std::max(version, n->paramVersion);
	}
	running = true;
	batchedLast = false;
	for (auto& n : order) {
		n->prepareImpl(stream_);
	}
	// Run timing covers the device work of the run: in a captured run the two events are the first
	// and last nodes of the CUDA graph, so the host's launch call is not inside the interval.
	const bool timed = timingEnabled();
	if (!cudaGraphsEnabled()) {
		releaseGraph();
		if (timed) {
			recordEvent(runStart, stream_);
		}
		for (auto& n : order) {
			n->enqueueImpl(stream_);
		}
		if (timed) {
			recordEvent(runStop, stream_);
		}
	} else {
		if (version > execVersion || exec == nullptr || execEpoch != rgl::allocationEpoch() || execTimed != timed) {
			releaseGraph();
			const uint64_t launches0 = rgl::launchCount();
			RGL_CHECK_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
			try {
				if (timed) {
					recordEvent(runStart, stream_);
				}
				for (auto& n : order) {
					n->enqueueImpl(stream_);
				}
				if (timed) {
					recordEvent(runStop, stream_);
				}
			}
			catch (...) {
				cudaGraph_t partial = nullptr;
				cudaStreamEndCapture(stream_, &partial);
				if (partial) {
					cudaGraphDestroy(partial);
				}
				throw;
			}
			cudaGraph_t graph = nullptr;
			RGL_CHECK_CUDA(cudaStreamEndCapture(stream_, &graph));
			const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
			cudaGraphDestroy(graph);
			RGL_CHECK_CUDA(inst);
			execKernels = rgl::launchCount() - launches0;
			execEpoch = rgl::allocationEpoch();
			execVersion = version;
			execTimed = timed;
			++captures;
		} else {
			++replays;
			rgl::countLaunch(execKernels);
		}
		RGL_CHECK_CUDA(cudaGraphLaunch(exec, stream_));
	}
	RGL_CHECK_CUDA(cudaEventRecord(done, stream_));
}

// As run() but without the nodes' validation when no API call that may change a graph came since
// this graph's last successful validation (a frame after frame of re-posed entities).
uint64_t GraphRunCtx::validateForBatch()
{
	synchronize();
	if (order.empty()) {
		order = findExecutionOrder(nodes);
		releaseGraph();
		validated = false;
	}
	const uint64_t epoch = graphEditEpoch();
	const bool fresh = validated && validatedEpoch == epoch;
	validated = false;
	uint64_t version = 0;
	for (auto& n : order) {
		if (!fresh) {
			n->validateImpl();
		}
		n->dirty = false;
		version = std::max(version, n->paramVersion);
	}
	validated = true;
	validatedEpoch = epoch;
	return version;
}

void GraphRunCtx::prepareForBatch(cudaStream_t s)
{
	running = true; // a failure from here on leaves the graph to be synchronised like a run
	for (auto& n : order) {
		n->prepareImpl(s);
	}
}

void GraphRunCtx::markBatchedRun(cudaEvent_t frameDone)
{
	batchDone = frameDone;
	running = true;
	batchedLast = true;
}

void GraphRunCtx::forgetBatchEvent(cudaEvent_t frameDone)
{
	if (batchDone == frameDone && frameDone != nullptr) {
		cudaEventSynchronize(batchDone);
		batchDone = nullptr;
		if (batchedLast) {
			running = false;
		}
	}
}

void GraphRunCtx::synchronize(bool refreshErrors)
{
	if (!running) {
		return;
	}
	running = false;
	RGL_CHECK_CUDA(cudaEventSynchronize(batchedLast && batchDone ? batchDone : done));
	RGL_CHECK_CUDA(cudaGetLastError());
	if (refreshErrors) {
		rgl::refreshErrorSlots();
	}
	if (timingEnabled() && !batchedLast) {
		cudaEventElapsedTime(&lastRunMs, runStart, runStop);
		for (auto& n : order) {
			if (auto rt = std::dynamic_pointer_cast<RaytraceNode>(n); rt && rt->evStart) {
				cudaEventElapsedTime(&lastTraceMs, rt->evStart, rt->evStop);
			}
		}
	}
	for (auto& n : order) {
		n->checkErrors();
	}
}

void GraphRunCtx::detachAndDestroy()
{
	auto self = shared_from_this();
	synchronize();
	for (auto& n : nodes) {
		n->ctx.reset();
		n->dirty = true;
	}
	auto& v = instances();
	v.erase(std::remove(v.begin(), v.end(), self), v.end());
}

void GraphRunCtx::synchronizeAll()
{
	for (auto& c : instances()) {
		c->synchronize();
	}
}
