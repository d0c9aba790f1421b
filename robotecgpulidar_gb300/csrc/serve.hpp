// Serving loop behind rgl_gb300_server_t (extension; the reference has no serving layer: a client
// runs one rgl_graph_run per scan, src/api/apiCore.cpp:530-544).
//
// Virtual robots register their lidar ray patterns once (resident on the device) and then submit
// scan requests: (scene, pattern, sensor pose, return mode, range). A scheduler thread admits
// requests first-come-first-served while the bytes of admitted requests stay under an HBM budget
// and fewer than `maxInFlight` batches are on the GPU, coalesces every admitted request into one
// batch, and launches it: one persistent traversal over all requests (trace_batch.cu; each job
// names its scene and applies its pose in-kernel with the arithmetic of a rays-transform node) and
// one segmented compaction by is-hit (segcompact.cu). Requests that arrive while batches run are
// admitted as slots and memory free up and go into the next batch, so the device always has the
// next batch queued behind the running one (continuous batching).
//
// Each request's result is XYZ, distance and entity id of its hit points, in point order, equal to
// what the graph rays_from_mat3x4f(pattern) -> rays_transform(pose) -> rays_set_range ->
// raytrace(scene, mode) -> compact_by_field(IS_HIT) -> yield writes. The compaction writes every
// request's result into the batch slot's device staging buffers and the kept counts to pinned host
// memory; once the counts arrive, the scheduler enqueues copy-engine copies of exactly the kept bytes
// into each request's block of the pinned host result arena (the copies run while the other slot's
// batch traverses, and take no SM time). A completed request's result is in host memory; release()
// returns its block to the arena.
//
// While a server runs, the scenes it traces must not be modified (drain() first).
#pragma once

#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.hpp"
#include "kernels.hpp"

struct Scene;

struct Server
{
	using Clock = std::chrono::steady_clock;

	Server(int64_t hbmBudgetBytes, int32_t maxInFlightBatches);
	~Server();

	int32_t addPattern(const void* rays, int32_t count);
	int64_t submit(std::shared_ptr<Scene> scene, int32_t pattern, const rgl::Mat34& pose, int32_t returnMode, float minRange,
	               float maxRange);
	// True when the request completed (or failed) within timeoutMs; timeoutMs < 0 waits forever.
	bool wait(int64_t id, double timeoutMs);
	int32_t takeCompleted(int64_t* ids, int32_t capacity);
	// As takeCompleted, but waits up to timeoutMs for at least one completed request.
	int32_t waitCompleted(int64_t* ids, int32_t capacity, double timeoutMs);
	void resultSize(int64_t id, rgl_field_t field, int32_t& count, int32_t& size);
	void resultData(int64_t id, rgl_field_t field, void* dst);
	// Host address of a completed request's field (valid until release) and its element count.
	const void* resultHost(int64_t id, rgl_field_t field, int32_t& count);
	// Seconds from submission to admission into a batch, and to completion.
	void timing(int64_t id, double& queuedS, double& totalS);
	void release(int64_t id);
	void drain();

	// Schedule and batch size limit of batches launched from now on.
	void configure(const rgl::BatchSchedule& s, int64_t maxBeams);

	struct Stats
	{
		int64_t submitted = 0, completed = 0, failed = 0, batches = 0, jobsInBatches = 0, peakReserved = 0, reserved = 0, inFlight = 0,
		        pending = 0;
		double deviceSeconds = 0.0; // summed device time of the batches (they may overlap)
	};
	Stats stats();

	// Phases of the batches retired since the last reset, on the device's clock: traversal and
	// compaction (launch to counts published), the host's reaction (counts published to the first
	// result copy enqueued: the scheduler's wake-up), the result copies. Per phase the longest and the
	// number above 5 ms.
	struct BatchTimes
	{
		float maxMs[3] = {0.0f, 0.0f, 0.0f};
		int64_t over5ms[3] = {0, 0, 0};
		int64_t batches = 0;
	};
	BatchTimes batchTimes(bool reset);

private:
	enum class State
	{
		Pending,
		InFlight,
		Done,
		Failed
	};
	struct Request
	{
		int64_t id;
		std::shared_ptr<Scene> scene;
		int32_t pattern;
		rgl::Mat34 pose;
		int32_t returnMode, returnCount;
		float minRange, maxRange;
		int64_t beams, points;
		int64_t reservedBytes;
		// Result block in the pinned arena (room for `points` points), filled by one copy: xyz of the
		// kept points, then their distances, then their entity ids, back to back.
		float* hostOut = nullptr;
		size_t outOffset = 0;
		int outOrder = -1;
		int32_t count = 0;
		State state = State::Pending;
		std::string error; // why a failed request failed
		Clock::time_point submitted, admitted, completed;
	};
	struct Pattern
	{
		rgl::DeviceBuffer rays{false};
		rgl::DeviceBuffer order{false};    // beams sorted by octahedral direction: warps get compact patches
		rgl::DeviceBuffer rowOrder{false}; // beams sorted by elevation, then azimuth: warps get stretches of a row
		int32_t count = 0;
	};
	// One in-flight batch slot: device and pinned buffers reused by every batch launched from it.
	// The job table, task bases, compaction segments and tile bases travel in one upload; the
	// per-request counts and the traversal's error flag come back in one download. A batch is
	// Tracing until its counts arrive (event `counted`), then Copying until its result copies are
	// done (event `done`).
	enum class Phase
	{
		Tracing,
		Copying
	};
	struct Slot
	{
		std::vector<Request*> reqs;
		std::vector<int64_t> pointBase; // first point of each request in the slot's buffers
		cudaStream_t stream = nullptr;  // slots run on their own streams: one batch's tail overlaps the next
		cudaEvent_t counted = nullptr, done = nullptr;
		cudaEvent_t t0 = nullptr, t1 = nullptr; // device time of the batch
		cudaEvent_t tCounted = nullptr, tCopy = nullptr; // counts published; first result copy enqueued
		rgl::DeviceBuffer tables{false}, tileCounts{false}, tileOffsets{false}, results{false}, counter{false};
		rgl::DeviceBuffer rawFlags{false}, rawXyz{false}, rawDist{false}, rawEnt{false};
		rgl::DeviceBuffer staged{false}; // compacted results: per request one block, xyz | distance | entity id
		rgl::PinnedBuffer hTables, hResults;
		int32_t* hResultsDev = nullptr; // device address of hResults (written by a kernel, not a copy)
		Phase phase = Phase::Tracing;
		bool busy = false;
	};

	// Device bytes of a point while its batch is on the GPU: flags, xyz, distance and entity id as
	// traced, then xyz, distance and entity id compacted.
	static constexpr int64_t kRawBytesPerPoint = 4 + 12 + 4 + 4 + 12 + 4 + 4;
	// Grows a slot's raw point and compaction-tile buffers (never shrinks them).
	void reserveRaw(Slot& slot, int64_t points, int64_t tiles);
	static constexpr int64_t kOutBytesPerPoint = 12 + 4 + 4;

	// Result arena: one pinned, device-mapped host allocation made with the server, handed out by a
	// buddy allocator (blocks of 64 KB << order, coalesced on release). Guarded by m.
	struct Arena
	{
		uint8_t* host = nullptr;
		int maxOrder = 0;
		std::vector<std::set<size_t>> freeByOrder; // block offsets
		static constexpr size_t kMinBlock = 64 << 10;
		static int orderFor(size_t bytes);
		bool take(size_t bytes, size_t& offset, int& order);
		void give(size_t offset, int order);
	};
	Arena arena;

	void loop();
	void launch(Slot& slot, const rgl::BatchSchedule& sched, Slot* after);
	void copyOut(Slot& slot);
	void retire(Slot& slot);
	Request& get(int64_t id);
	static void CUDART_CB batchDone(void* self);

	int64_t budget;
	int maxInFlight;
	rgl::BatchSchedule schedule{256, rgl::kPackLaneGroup, rgl::kOrderElevation, 1, 128}; // guarded by m
	int64_t maxBatchBeams = 4 << 20;                                                       // guarded by m
	cudaStream_t stream = nullptr;
	std::vector<std::unique_ptr<Pattern>> patterns;
	std::vector<std::unique_ptr<Slot>> slots;
	std::deque<Slot*> inFlight;
	Slot* lastLaunched = nullptr; // slot of the most recent batch (guarded by m)

	std::mutex m;
	std::condition_variable cvWork, cvDone;
	std::deque<Request*> pending;
	std::unordered_map<int64_t, std::unique_ptr<Request>> requests;
	std::deque<int64_t> completedIds;

	int64_t nextId = 1;
	int64_t reserved = 0;
	Stats st;
	BatchTimes bt; // guarded by m
	bool stop = false;
	uint64_t wakeups = 0; // bumped (under m) by submissions, releases and finished batches
	std::thread worker;
};
