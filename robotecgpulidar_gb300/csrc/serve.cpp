#include "serve.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "scene.hpp"

using rgl::format;

namespace {

// Grows buf to hold `bytes`, at least doubling its capacity: a run of growing batches reallocates
// (and so waits for the device) only a few times.
void* grow(rgl::DeviceBuffer& buf, size_t bytes) { return buf.ensure(bytes <= buf.capacity() ? bytes : std::max(bytes, 2 * buf.capacity())); }

// Layout of a batch's upload (16-byte aligned parts): jobs[n] | task bases[n+1] | segments[n] | tile bases[n+1].
struct TableLayout
{
	size_t offTask, offSeg, offTile, bytes;
};
TableLayout tableLayout(int n)
{
	auto align = [](size_t x) { return (x + 15) & ~size_t{15}; };
	TableLayout t;
	t.offTask = align(sizeof(rgl::BatchJob) * n);
	t.offSeg = t.offTask + align(sizeof(int32_t) * (n + 1));
	t.offTile = t.offSeg + align(sizeof(rgl::SegCompactJob) * n);
	t.bytes = t.offTile + align(sizeof(int32_t) * (n + 1));
	return t;
}

} // namespace

Server::Server(int64_t hbmBudgetBytes, int32_t maxInFlightBatches) : budget(hbmBudgetBytes), maxInFlight(std::max(1, maxInFlightBatches))
{
	RGL_CHECK_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
	// Result arena: a quarter of the budget, between 64 MB and 32 GB, rounded down to a power of two
	// of the minimum block. Requests wait for arena space when clients hold results, so the arena
	// bounds how far a burst of requests runs ahead of the client's reads.
	const size_t want = (size_t) std::min<int64_t>(std::max<int64_t>(budget / 4, 64ll << 20), 32ll << 30);
	int order = 0;
	while ((Arena::kMinBlock << (order + 1)) <= want) {
		++order;
	}
	arena.maxOrder = order;
	arena.freeByOrder.assign(order + 1, {});
	arena.freeByOrder[order].insert(0);
	void* h = nullptr;
	RGL_CHECK_CUDA(cudaHostAlloc(&h, Arena::kMinBlock << order, cudaHostAllocPortable));
	arena.host = static_cast<uint8_t*>(h);
	// The copy engine writes every page of the arena once now (the path the result copies take), so
	// the first batches that land in a page do not pay the first access to it.
	{
		const size_t total = Arena::kMinBlock << order, piece = std::min<size_t>(total, 64u << 20);
		rgl::DeviceBuffer zeros{false};
		RGL_CHECK_CUDA(cudaMemsetAsync(zeros.ensure(piece), 0, piece, stream));
		for (size_t off = 0; off < total; off += piece) {
			RGL_CHECK_CUDA(cudaMemcpyAsync(arena.host + off, zeros.get(), std::min(piece, total - off), cudaMemcpyDeviceToHost, stream));
		}
		RGL_CHECK_CUDA(cudaStreamSynchronize(stream));
	}
	for (int i = 0; i < maxInFlight; ++i) {
		auto s = std::make_unique<Slot>();
		RGL_CHECK_CUDA(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming));
		RGL_CHECK_CUDA(cudaEventCreateWithFlags(&s->counted, cudaEventDisableTiming));
		RGL_CHECK_CUDA(cudaEventCreate(&s->t0));
		RGL_CHECK_CUDA(cudaEventCreate(&s->t1));
		RGL_CHECK_CUDA(cudaEventCreate(&s->tCounted));
		RGL_CHECK_CUDA(cudaEventCreate(&s->tCopy));
		RGL_CHECK_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
		RGL_CHECK_CUDA(cudaMemset(s->counter.ensure(rgl::kTraceCounterBytes), 0, rgl::kTraceCounterBytes));
		slots.push_back(std::move(s));
	}
	// Per-batch buffers sized up front for the largest batch (two returns per beam, kMaxBatchJobs
	// requests), within this slot's share of the budget: a batch never allocates or frees, which would
	// wait for the other slots' work on the device.
	const int64_t points = std::min<int64_t>(2 * maxBatchBeams, budget / (kRawBytesPerPoint * maxInFlight));
	const TableLayout most = tableLayout(rgl::kMaxBatchJobs);
	for (auto& sl : slots) {
		if (points > 0) {
			reserveRaw(*sl, points, points / rgl::kSegTile + 4096);
		}
		sl->hTables.ensure(most.bytes);
		sl->tables.ensure(most.bytes);
		void* hr = sl->hResults.ensure(sizeof(int32_t) * 2 * rgl::kMaxBatchJobs);
		void* hrDev = nullptr;
		RGL_CHECK_CUDA(cudaHostGetDevicePointer(&hrDev, hr, 0));
		sl->hResultsDev = static_cast<int32_t*>(hrDev);
		sl->results.ensure(sizeof(int32_t) * 2 * rgl::kMaxBatchJobs);
	}
	worker = std::thread([this] { loop(); });
}

Server::~Server()
{
	{
		std::lock_guard<std::mutex> g(m);
		stop = true;
	}
	cvWork.notify_all();
	if (worker.joinable()) {
		worker.join();
	}
	cudaStreamSynchronize(stream);
	for (auto& s : slots) {
		cudaStreamSynchronize(s->stream);
	}
	cudaFreeHost(arena.host);
	for (auto& s : slots) {
		cudaEventDestroy(s->done);
		cudaEventDestroy(s->counted);
		cudaEventDestroy(s->t0);
		cudaEventDestroy(s->t1);
		cudaEventDestroy(s->tCounted);
		cudaEventDestroy(s->tCopy);
		cudaStreamDestroy(s->stream);
	}
	cudaStreamDestroy(stream);
}

int Server::Arena::orderFor(size_t bytes)
{
	int o = 0;
	while ((kMinBlock << o) < bytes) {
		++o;
	}
	return o;
}

bool Server::Arena::take(size_t bytes, size_t& offset, int& order)
{
	order = orderFor(bytes);
	int o = order;
	while (o <= maxOrder && freeByOrder[o].empty()) {
		++o;
	}
	if (o > maxOrder) {
		return false;
	}
	offset = *freeByOrder[o].begin();
	freeByOrder[o].erase(freeByOrder[o].begin());
	while (o > order) { // split, keeping the lower half
		--o;
		freeByOrder[o].insert(offset + (kMinBlock << o));
	}
	return true;
}

void Server::Arena::give(size_t offset, int order)
{
	while (order < maxOrder) {
		const size_t buddy = offset ^ (kMinBlock << order);
		auto it = freeByOrder[order].find(buddy);
		if (it == freeByOrder[order].end()) {
			break;
		}
		freeByOrder[order].erase(it);
		offset = std::min(offset, buddy);
		++order;
	}
	freeByOrder[order].insert(offset);
}

namespace {
uint32_t spread2(uint32_t v)
{
	v &= 0xffffu;
	v = (v | (v << 8)) & 0x00ff00ffu;
	v = (v | (v << 4)) & 0x0f0f0f0fu;
	v = (v | (v << 2)) & 0x33333333u;
	v = (v | (v << 1)) & 0x55555555u;
	return v;
}

// 22-bit key of a sensor-local ray direction: the direction folded onto the octahedron, 11 bits per
// coordinate, interleaved. Neighbouring keys are neighbouring directions.
uint32_t octahedralKey(const rgl::Mat34& m)
{
	float x = m.m[0][2], y = m.m[1][2], z = m.m[2][2];
	const float l1 = std::fabs(x) + std::fabs(y) + std::fabs(z);
	float u = l1 > 0.0f ? x / l1 : 0.0f, v = l1 > 0.0f ? y / l1 : 0.0f;
	if (z < 0.0f) {
		const float fu = (1.0f - std::fabs(v)) * (u >= 0.0f ? 1.0f : -1.0f);
		const float fv = (1.0f - std::fabs(u)) * (v >= 0.0f ? 1.0f : -1.0f);
		u = fu;
		v = fv;
	}
	auto q = [](float c) { return (uint32_t) std::min(2047.0f, std::max(0.0f, (c * 0.5f + 0.5f) * 2048.0f)); };
	return (spread2(q(u)) << 1) | spread2(q(v));
}

// 22-bit key of a sensor-local ray direction in scan-row order: the sine of its elevation above the
// local xy plane in the high 11 bits, a pseudo-angle of its azimuth (monotonic in atan2(y, x), in
// (-2, 2]) in the low 11 bits. Beams of one row travel similar distances, so a warp's lanes finish
// together more often than in direction patches.
uint32_t rowKey(const rgl::Mat34& m)
{
	const float x = m.m[0][2], y = m.m[1][2], z = m.m[2][2];
	const float len = std::sqrt(x * x + y * y + z * z);
	const float l1 = std::fabs(x) + std::fabs(y);
	const float pa = l1 > 0.0f ? 1.0f - x / l1 : 0.0f;
	const float az = y < 0.0f ? -pa : pa;
	auto q = [](float c) { return (uint32_t) std::min(2047.0f, std::max(0.0f, c * 2048.0f)); };
	return (q(len > 0.0f ? z / len * 0.5f + 0.5f : 0.5f) << 11) | q(az * 0.25f + 0.5f);
}

std::vector<uint32_t> sortedBy(const rgl::Mat34* mats, int32_t count, uint32_t (*key)(const rgl::Mat34&))
{
	std::vector<uint32_t> k(count), order(count);
	for (int32_t i = 0; i < count; ++i) {
		k[i] = key(mats[i]);
		order[i] = (uint32_t) i;
	}
	std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return k[a] < k[b]; });
	return order;
}
} // namespace

Server::BatchTimes Server::batchTimes(bool reset)
{
	std::lock_guard<std::mutex> g(m);
	const BatchTimes out = bt;
	if (reset) {
		bt = BatchTimes{};
	}
	return out;
}

int32_t Server::addPattern(const void* rays, int32_t count)
{
	auto p = std::make_unique<Pattern>();
	RGL_CHECK_CUDA(cudaMemcpy(p->rays.ensure(sizeof(rgl::Mat34) * (size_t) count), rays, sizeof(rgl::Mat34) * (size_t) count,
	                          cudaMemcpyHostToDevice));
	// Visiting orders: a warp casts 32 beams (or 6 beams of 5 sub-rays); sorted by direction they form
	// a compact patch of the pattern, sorted by rows a stretch of one elevation, instead of, e.g., one
	// column of channels. Results stay in beam order.
	const auto* mats = static_cast<const rgl::Mat34*>(rays);
	const std::vector<uint32_t> byDirection = sortedBy(mats, count, octahedralKey), byRow = sortedBy(mats, count, rowKey);
	RGL_CHECK_CUDA(cudaMemcpy(p->order.ensure(sizeof(uint32_t) * (size_t) count), byDirection.data(), sizeof(uint32_t) * (size_t) count,
	                          cudaMemcpyHostToDevice));
	RGL_CHECK_CUDA(cudaMemcpy(p->rowOrder.ensure(sizeof(uint32_t) * (size_t) count), byRow.data(), sizeof(uint32_t) * (size_t) count,
	                          cudaMemcpyHostToDevice));
	p->count = count;
	std::lock_guard<std::mutex> g(m);
	patterns.push_back(std::move(p));
	return (int32_t) patterns.size() - 1;
}

int64_t Server::submit(std::shared_ptr<Scene> scene, int32_t pattern, const rgl::Mat34& pose, int32_t returnMode, float minRange,
                       float maxRange)
{
	std::unique_lock<std::mutex> lk(m);
	if (pattern < 0 || pattern >= (int32_t) patterns.size()) {
		throw rgl::InvalidAPIArgument(format("pattern %d was not added to this server", (int) pattern));
	}
	auto r = std::make_unique<Request>();
	r->id = nextId++;
	r->scene = std::move(scene);
	r->pattern = pattern;
	r->pose = pose;
	r->returnMode = returnMode;
	r->returnCount = (int32_t) (((uint32_t) returnMode) >> 24);
	r->minRange = minRange;
	r->maxRange = maxRange;
	r->beams = patterns[pattern]->count;
	r->points = r->beams * r->returnCount;
	r->reservedBytes = r->points * (kRawBytesPerPoint + kOutBytesPerPoint);
	if (r->reservedBytes > budget) {
		throw rgl::InvalidAPIArgument(
		    format("request needs %lld bytes, more than the server's HBM budget of %lld", (long long) r->reservedBytes, (long long) budget));
	}
	if ((size_t) (r->points * kOutBytesPerPoint) > (Arena::kMinBlock << arena.maxOrder)) {
		throw rgl::InvalidAPIArgument(format("request results need %lld bytes, more than the server's result arena of %lld",
		                                     (long long) (r->points * kOutBytesPerPoint), (long long) (Arena::kMinBlock << arena.maxOrder)));
	}
	r->submitted = Clock::now();
	const int64_t id = r->id;
	pending.push_back(r.get());
	requests.emplace(id, std::move(r));
	++st.submitted;
	++wakeups;
	lk.unlock();
	cvWork.notify_one();
	return id;
}

Server::Request& Server::get(int64_t id)
{
	auto it = requests.find(id);
	if (it == requests.end()) {
		throw rgl::InvalidAPIObject(format("RGL API Error: Object does not exist: Request %lld", (long long) id));
	}
	return *it->second;
}

bool Server::wait(int64_t id, double timeoutMs)
{
	std::unique_lock<std::mutex> lk(m);
	Request& r = get(id);
	auto ready = [&] { return r.state == State::Done || r.state == State::Failed; };
	if (timeoutMs < 0) {
		cvDone.wait(lk, ready);
		return true;
	}
	return cvDone.wait_for(lk, std::chrono::duration<double, std::milli>(timeoutMs), ready);
}

int32_t Server::waitCompleted(int64_t* ids, int32_t capacity, double timeoutMs)
{
	{
		std::unique_lock<std::mutex> lk(m);
		cvDone.wait_for(lk, std::chrono::duration<double, std::milli>(std::max(0.0, timeoutMs)), [&] { return !completedIds.empty(); });
	}
	return takeCompleted(ids, capacity);
}

int32_t Server::takeCompleted(int64_t* ids, int32_t capacity)
{
	std::lock_guard<std::mutex> g(m);
	int32_t n = 0;
	while (n < capacity && !completedIds.empty()) {
		const int64_t id = completedIds.front();
		completedIds.pop_front();
		if (requests.count(id)) { // released requests are not reported
			ids[n++] = id;
		}
	}
	return n;
}

void Server::resultSize(int64_t id, rgl_field_t field, int32_t& count, int32_t& size)
{
	std::lock_guard<std::mutex> g(m);
	Request& r = get(id);
	if (r.state == State::Failed) {
		// Recoverable: one failed request leaves the server and the library usable.
		throw rgl::InvalidPipeline(format("served request %lld failed: %s", (long long) id, r.error.c_str()));
	}
	if (r.state != State::Done) {
		throw rgl::InvalidPipeline(format("request %lld has not completed", (long long) id));
	}
	if (field != RGL_FIELD_XYZ_VEC3_F32 && field != RGL_FIELD_DISTANCE_F32 && field != RGL_FIELD_ENTITY_ID_I32) {
		throw rgl::InvalidAPIArgument(format("served requests provide XYZ_VEC3_F32, DISTANCE_F32 and ENTITY_ID_I32, not %s",
		                                     rgl::fieldName(field)));
	}
	count = r.count;
	size = (int32_t) rgl::fieldSize(field);
}

const void* Server::resultHost(int64_t id, rgl_field_t field, int32_t& count)
{
	int32_t size = 0;
	resultSize(id, field, count, size);
	std::lock_guard<std::mutex> g(m);
	Request& r = get(id);
	const float* base = r.hostOut;
	if (field == RGL_FIELD_XYZ_VEC3_F32) {
		return base;
	}
	return field == RGL_FIELD_DISTANCE_F32 ? base + 3 * (size_t) r.count : base + 4 * (size_t) r.count;
}

void Server::resultData(int64_t id, rgl_field_t field, void* dst)
{
	int32_t count = 0;
	const void* src = resultHost(id, field, count);
	if (count > 0) {
		std::memcpy(dst, src, (size_t) count * rgl::fieldSize(field));
	}
}

void Server::timing(int64_t id, double& queuedS, double& totalS)
{
	std::lock_guard<std::mutex> g(m);
	Request& r = get(id);
	if (r.state != State::Done && r.state != State::Failed) {
		throw rgl::InvalidPipeline(format("request %lld has not completed", (long long) id));
	}
	queuedS = std::chrono::duration<double>(r.admitted - r.submitted).count();
	totalS = std::chrono::duration<double>(r.completed - r.submitted).count();
}

void Server::release(int64_t id)
{
	std::unique_lock<std::mutex> lk(m);
	Request& r = get(id);
	if (r.state == State::Pending || r.state == State::InFlight) {
		lk.unlock();
		wait(id, -1.0);
		lk.lock();
	}
	Request& q = get(id);
	if (q.outOrder >= 0) {
		arena.give(q.outOffset, q.outOrder); // the GPU finished writing it
	}
	reserved -= q.points * kOutBytesPerPoint;
	requests.erase(id);
	++wakeups;
	lk.unlock();
	cvWork.notify_one();
}

void Server::drain()
{
	std::unique_lock<std::mutex> lk(m);
	cvDone.wait(lk, [&] { return pending.empty() && inFlight.empty(); });
}

Server::Stats Server::stats()
{
	std::lock_guard<std::mutex> g(m);
	Stats s = st;
	s.reserved = reserved;
	s.inFlight = (int64_t) inFlight.size();
	s.pending = (int64_t) pending.size();
	return s;
}

void Server::reserveRaw(Slot& slot, int64_t points, int64_t tiles)
{
	points = std::max<int64_t>(points, 1);
	tiles = std::max<int64_t>(tiles, 1);
	grow(slot.rawFlags, sizeof(int32_t) * (size_t) points);
	grow(slot.rawXyz, sizeof(float) * 3 * (size_t) points);
	grow(slot.rawDist, sizeof(float) * (size_t) points);
	grow(slot.rawEnt, sizeof(int32_t) * (size_t) points);
	grow(slot.staged, sizeof(float) * 5 * (size_t) points);
	grow(slot.tileCounts, sizeof(uint32_t) * (size_t) tiles);
	grow(slot.tileOffsets, sizeof(uint32_t) * (size_t) tiles);
}

void Server::configure(const rgl::BatchSchedule& s, int64_t maxBeams)
{
	std::lock_guard<std::mutex> g(m);
	schedule = s;
	maxBatchBeams = maxBeams;
}

// Builds and enqueues one batch from slot.reqs (already admitted, outputs allocated). Its traversal
// starts on the device once the batch launched before it (on slot `after`) has traced and compacted:
// batches trace one after another at the full speed of the GPU, while each batch's result copies
// (copy engine) overlap the next batch's traversal. Two traversals sharing the GPU would both finish
// late and then leave it idle during their copies.
void Server::launch(Slot& slot, const rgl::BatchSchedule& sched, Slot* after)
{
	const int n = (int) slot.reqs.size();
	int64_t points = 0;
	for (auto* r : slot.reqs) {
		points += r->points;
	}
	int64_t maxTiles = 0;
	for (auto* r : slot.reqs) {
		maxTiles += (r->points + rgl::kSegTile - 1) / rgl::kSegTile;
	}
	reserveRaw(slot, points, maxTiles);
	auto* flags = slot.rawFlags.as<int32_t>();
	auto* xyz = slot.rawXyz.as<float>();
	auto* dist = slot.rawDist.as<float>();
	auto* ent = slot.rawEnt.as<int32_t>();
	auto* staged = slot.staged.as<float>();
	slot.pointBase.assign((size_t) n, 0);

	const TableLayout lay = tableLayout(n);
	const size_t offTask = lay.offTask, offSeg = lay.offSeg, offTile = lay.offTile, tableBytes = lay.bytes;
	auto* hBase = static_cast<uint8_t*>(slot.hTables.ensure(tableBytes));
	auto* dBase = static_cast<uint8_t*>(grow(slot.tables, tableBytes));
	auto* jobs = reinterpret_cast<rgl::BatchJob*>(hBase);
	auto* taskBase = reinterpret_cast<int32_t*>(hBase + offTask);
	auto* segs = reinterpret_cast<rgl::SegCompactJob*>(hBase + offSeg);
	auto* tileBase = reinterpret_cast<int32_t*>(hBase + offTile);
	// Results: counts[n], then one traversal error flag per request.
	auto* dResults = static_cast<int32_t*>(grow(slot.results, sizeof(int32_t) * 2 * n));
	int64_t pointBase = 0, tasks = 0, tiles = 0;
	for (int j = 0; j < n; ++j) {
		Request& r = *slot.reqs[j];
		rgl::BatchJob b{};
		b.p.rays = patterns[r.pattern]->rays.as<rgl::Mat34>();
		b.p.ranges = nullptr;
		b.p.nRanges = 1;
		b.p.nRays = (int32_t) r.beams;
		b.p.nSamples = 1;
		b.p.returnMode = r.returnMode;
		b.p.returnCount = r.returnCount;
		b.p.nearNonHitDistance = INFINITY;
		b.p.farNonHitDistance = INFINITY;
		b.p.defaultIntensity = 0.0f;
		b.p.needIntensity = 0;
		b.p.errorFlag = dResults + n + j;
		b.p.scene = r.scene->view();
		b.p.out.xyz = xyz + 3 * pointBase;
		b.p.out.distance = dist + pointBase;
		b.p.out.isHit = flags + pointBase;
		b.p.out.entityId = ent + pointBase;
		b.samples = nullptr; // one sample per beam: never read
		b.order = sched.order == rgl::kOrderNatural     ? nullptr
		          : sched.order == rgl::kOrderElevation ? patterns[r.pattern]->rowOrder.as<uint32_t>()
		                                                : patterns[r.pattern]->order.as<uint32_t>();
		b.groupSize = 1;
		b.hasRayTransform = 1;
		b.rayTransform = r.pose;
		b.inlineRange[0] = r.minRange;
		b.inlineRange[1] = r.maxRange;
		jobs[j] = b;
		taskBase[j] = (int32_t) tasks;
		tasks += (r.beams + 31) / 32;

		rgl::SegCompactJob sg{};
		sg.flags = flags + pointBase;
		sg.xyz = xyz + 3 * pointBase;
		sg.dist = dist + pointBase;
		sg.ent = ent + pointBase;
		sg.outXyz = staged + 5 * pointBase; // the request's block: room for 5 words per point
		sg.outDist = nullptr;
		sg.outEnt = nullptr;
		sg.nPoints = (int32_t) r.points;
		sg.packed = 1;
		segs[j] = sg;
		slot.pointBase[(size_t) j] = pointBase;
		tileBase[j] = (int32_t) tiles;
		tiles += (r.points + rgl::kSegTile - 1) / rgl::kSegTile;
		pointBase += r.points;
	}
	taskBase[n] = (int32_t) tasks;
	tileBase[n] = (int32_t) tiles;

	auto* dTileCounts = slot.tileCounts.get();
	auto* dTileOffsets = slot.tileOffsets.get();
	RGL_CHECK_CUDA(cudaMemcpyAsync(dBase, hBase, tableBytes, cudaMemcpyHostToDevice, slot.stream));
	RGL_CHECK_CUDA(cudaMemsetAsync(dResults + n, 0, sizeof(int32_t) * n, slot.stream));
	if (after != nullptr && after != &slot) {
		RGL_CHECK_CUDA(cudaStreamWaitEvent(slot.stream, after->counted, 0));
	}
	RGL_CHECK_CUDA(cudaEventRecord(slot.t0, slot.stream));
	rgl::launchTraceBatch(reinterpret_cast<const rgl::BatchJob*>(dBase), reinterpret_cast<const int32_t*>(dBase + offTask), n, 1, false,
	                      sched, slot.counter.as<uint32_t>(), slot.stream);
	rgl::launchSegCompact(reinterpret_cast<const rgl::SegCompactJob*>(dBase + offSeg), reinterpret_cast<const int32_t*>(dBase + offTile), n,
	                      (int) tiles, static_cast<uint32_t*>(dTileCounts), static_cast<uint32_t*>(dTileOffsets), dResults, slot.stream);
	// Counts and error flags reach pinned host memory by a kernel's stores: a copy would queue behind
	// the other slot's result copies on the copy engine, and this batch's successor waits for it.
	rgl::launchPublishWords(dResults, slot.hResultsDev, 2 * n, slot.stream);
	RGL_CHECK_CUDA(cudaEventRecord(slot.counted, slot.stream));
	RGL_CHECK_CUDA(cudaEventRecord(slot.tCounted, slot.stream));
	slot.phase = Phase::Tracing;
	RGL_CHECK_CUDA(cudaLaunchHostFunc(slot.stream, &Server::batchDone, this));
}

// Once a batch's kept counts are in host memory: one copy per request of exactly its kept points'
// block (xyz, distances, entity ids back to back) from the slot's staging buffer into the request's
// block of the result arena, on the slot's stream (copy engine), then the batch's completion.
void Server::copyOut(Slot& slot)
{
	const auto* hCounts = static_cast<const volatile int32_t*>(slot.hResults.get());
	const size_t n = slot.reqs.size();
	const auto* staged = slot.staged.as<float>();
	RGL_CHECK_CUDA(cudaEventRecord(slot.tCopy, slot.stream));
	for (size_t j = 0; j < n; ++j) {
		const Request& r = *slot.reqs[j];
		const int64_t kept = hCounts[j];
		if (hCounts[n + j] != 0 || kept <= 0 || kept > r.points) {
			continue; // failed (retire reports it) or nothing kept
		}
		RGL_CHECK_CUDA(cudaMemcpyAsync(r.hostOut, staged + 5 * slot.pointBase[j], sizeof(float) * 5 * (size_t) kept, cudaMemcpyDeviceToHost,
		                               slot.stream));
	}
	RGL_CHECK_CUDA(cudaEventRecord(slot.t1, slot.stream));
	RGL_CHECK_CUDA(cudaEventRecord(slot.done, slot.stream));
	slot.phase = Phase::Copying;
	RGL_CHECK_CUDA(cudaLaunchHostFunc(slot.stream, &Server::batchDone, this));
}

// Runs on a CUDA host thread once a batch's stream work is done: wakes the scheduler, which then
// finds the batch's event complete. Makes no CUDA call.
void CUDART_CB Server::batchDone(void* self)
{
	auto* s = static_cast<Server*>(self);
	{
		// The scheduler never makes a CUDA call that waits for this stream while holding m.
		std::lock_guard<std::mutex> g(s->m);
		++s->wakeups;
	}
	s->cvWork.notify_all();
}

void Server::retire(Slot& slot)
{
	const auto* hCounts = static_cast<const int32_t*>(slot.hResults.get());
	const size_t n = slot.reqs.size();
	const auto now = Clock::now();
	float ms = 0.0f, phase[3] = {0.0f, 0.0f, 0.0f};
	cudaEventElapsedTime(&ms, slot.t0, slot.t1);
	const bool timed = cudaEventElapsedTime(&phase[0], slot.t0, slot.tCounted) == cudaSuccess &&
	                   cudaEventElapsedTime(&phase[1], slot.tCounted, slot.tCopy) == cudaSuccess &&
	                   cudaEventElapsedTime(&phase[2], slot.tCopy, slot.t1) == cudaSuccess;
	std::lock_guard<std::mutex> g(m);
	st.deviceSeconds += ms * 1e-3;
	if (timed) {
		for (int k = 0; k < 3; ++k) {
			bt.maxMs[k] = std::max(bt.maxMs[k], phase[k]);
			bt.over5ms[k] += phase[k] > 5.0f ? 1 : 0;
		}
		++bt.batches;
	}
	for (size_t j = 0; j < n; ++j) {
		Request& r = *slot.reqs[j];
		const bool failed = hCounts[n + j] != 0;
		r.count = hCounts[j];
		r.state = failed ? State::Failed : State::Done;
		if (failed) {
			r.error = hCounts[n + j] == 2 ? "the result copies could not be enqueued" : "traversal stack overflow on the device";
			++st.failed;
		}
		r.completed = now;
		reserved -= r.points * kRawBytesPerPoint;
		completedIds.push_back(r.id);
		++st.completed;
	}
	slot.reqs.clear();
	slot.busy = false;
	inFlight.pop_front();
	cvDone.notify_all();
}

// Scheduler thread: retire finished batches, admit and launch the next batch whenever a slot is free,
// otherwise wait for work or for the oldest batch.
void Server::loop()
{
	const int dev = [] {
		int d = 0;
		cudaGetDevice(&d);
		return d;
	}();
	cudaSetDevice(dev);
	std::unique_lock<std::mutex> lk(m);
	for (;;) {
		const uint64_t seen = wakeups;
		// Batches whose counts arrived get their result copies; finished batches retire in order.
		const std::vector<Slot*> running(inFlight.begin(), inFlight.end());
		for (Slot* s : running) {
			if (s->phase == Phase::Tracing && cudaEventQuery(s->counted) == cudaSuccess) {
				lk.unlock();
				try {
					copyOut(*s);
				}
				catch (std::exception& e) {
					// The copies could not be enqueued: the batch's requests fail when it retires.
					auto* hCounts = static_cast<int32_t*>(s->hResults.get());
					for (size_t j = 0; j < s->reqs.size(); ++j) {
						hCounts[s->reqs.size() + j] = 2;
					}
					cudaEventRecord(s->done, s->stream);
					s->phase = Phase::Copying;
				}
				lk.lock();
			}
		}
		while (!inFlight.empty() && inFlight.front()->phase == Phase::Copying && cudaEventQuery(inFlight.front()->done) == cudaSuccess) {
			Slot* s = inFlight.front();
			lk.unlock();
			retire(*s);
			lk.lock();
		}
		if (stop && pending.empty() && inFlight.empty()) {
			break;
		}
		Slot* freeSlot = nullptr;
		for (auto& s : slots) {
			if (!s->busy) {
				freeSlot = s.get();
				break;
			}
		}
		if (freeSlot != nullptr && !pending.empty()) {
			// Admission: first come first served, within the HBM budget and the batch limits.
			std::vector<Request*> batch;
			int64_t beams = 0;
			while (!pending.empty() && (int) batch.size() < rgl::kMaxBatchJobs) {
				Request* r = pending.front();
				if (reserved + r->reservedBytes > budget || (!batch.empty() && beams + r->beams > maxBatchBeams)) {
					break;
				}
				if (!arena.take((size_t) std::max<int64_t>(r->points * kOutBytesPerPoint, 1), r->outOffset, r->outOrder)) {
					break; // the result arena is full until clients release results
				}
				r->hostOut = reinterpret_cast<float*>(arena.host + r->outOffset);
				pending.pop_front();
				reserved += r->reservedBytes;
				st.peakReserved = std::max(st.peakReserved, reserved);
				beams += r->beams;
				r->state = State::InFlight;
				r->admitted = Clock::now();
				batch.push_back(r);
			}
			if (!batch.empty()) {
				// Jobs of one scene next to each other: warps take tasks in job order, so the device
				// works on few scenes at a time (L2 locality). Results do not depend on the order.
				std::stable_sort(batch.begin(), batch.end(), [](const Request* a, const Request* b) { return a->scene.get() < b->scene.get(); });
				freeSlot->busy = true;
				freeSlot->reqs = batch;
				inFlight.push_back(freeSlot);
				Slot* after = lastLaunched;
				lastLaunched = freeSlot;
				++st.batches;
				st.jobsInBatches += (int64_t) batch.size();
				const rgl::BatchSchedule sched = schedule;
				lk.unlock();
				bool ok = true;
				std::string why;
				try {
					std::vector<Scene*> prepared;
					for (auto* r : batch) {
						if (std::find(prepared.begin(), prepared.end(), r->scene.get()) == prepared.end()) {
							r->scene->prepare(freeSlot->stream);
							prepared.push_back(r->scene.get());
						}

					}
					launch(*freeSlot, sched, after);
				}
				catch (std::exception& e) {
					ok = false;
					why = e.what();
				}
				catch (...) {
					ok = false;
					why = "unknown exception";
				}
				lk.lock();
				if (!ok) {
					// The batch never reached the device: fail its requests.
					const auto now = Clock::now();
					for (auto* r : batch) {
						r->state = State::Failed;
						r->error = "batch launch failed: " + why;
						++st.failed;
						r->completed = now;
						reserved -= r->points * kRawBytesPerPoint;
						completedIds.push_back(r->id);
					}
					freeSlot->reqs.clear();
					freeSlot->busy = false;
					inFlight.erase(std::find(inFlight.begin(), inFlight.end(), freeSlot));
					cvDone.notify_all();
				}
				continue;
			}
		}
		if (inFlight.empty()) {
			cvDone.notify_all(); // drain() waiters
		}
		// Sleep until a submission, a release or a finished batch (its host function) changes the
		// picture; the timeout is only a safety net.
		cvWork.wait_for(lk, std::chrono::milliseconds(5), [&] { return wakeups != seen || stop; });
	}
}
