// Batched multi-sensor frames behind rgl_gb300_batch_t (extension; the reference runs every sensor's
// graph on its own with rgl_graph_run, src/api/apiCore.cpp:530-544).
//
// A batch is a list of ordinary RGL graphs, one per sensor, each with exactly one raytrace node (the
// sensors may trace different scenes). One frame = one rgl_gb300_batch_run:
//  * host: every graph is validated and prepared as for rgl_graph_run; the scene builds what cannot
//    be captured (new BLAS, TLAS topology) and otherwise refreshes its pinned instance records;
//  * device, captured once into one CUDA graph and replayed: upload of the instance records and TLAS
//    refit, every graph's nodes before its raytrace node, then the sensors in W waves (contiguous
//    runs of the batch's graphs with about equal ray counts): one persistent traversal launch per
//    wave (trace_batch.cu), each launched with programmatic stream serialization after the previous
//    one, so its blocks fill the SMs that the previous launch's tail leaves idle. A side stream runs
//    each wave's later nodes (compaction, formatting) once its traversal completes and then records
//    the wave's completion event, which the wave's graphs wait on. Per-sensor node work is spread over a few forked
//    streams, so it becomes parallel branches of the graph.
// Results are read per graph with rgl_graph_get_result_size/_data, as after rgl_graph_run, and equal
// what a run of that graph alone writes. A graph's results are ready when its wave's later nodes
// end, so reads of the first waves' results overlap the later waves' traversal.
//
// The traversal schedule (block size, packing, beam order, chunk, register budget) is picked by an
// autotuner the first time a batch runs with a new shape (per-sensor ray and sample counts): it times
// the traversal alone for a staged set of candidates and keeps the fastest.
#pragma once

#include <memory>
#include <vector>

#include "graph.hpp"

struct Scene;

struct BatchRun
{
	explicit BatchRun(std::vector<Node::Ptr> anchors);
	~BatchRun();
	void run();
	void synchronize();

	// Schedule: fixed by the client, or tuned (autotune) per batch shape.
	bool autotune = true;
	rgl::BatchSchedule schedule{256, rgl::kPackLaneGroup, rgl::kOrderNatural, 1, 80};
	// Waves per frame: 0 picks one wave per kRaysPerWave traced rays (at most kAutoWaves).
	int wavesWanted = 0;
	static constexpr int kAutoWaves = 16;
	static constexpr int64_t kRaysPerWave = int64_t{2} << 20;
	int waveCount() const { return (int) waveFirst.size() - 1; }

	// Statistics of the last frame and of the batch's lifetime.
	float lastFrameMs = 0.0f, lastTraceMs = 0.0f;
	uint64_t captures = 0, replays = 0, tunings = 0;
	int64_t beams = 0, rays = 0; // beams and traced sample rays of the last frame

	struct Candidate
	{
		rgl::BatchSchedule s;
		float ms;
	};
	std::vector<Candidate> lastTuning;

private:
	struct Member
	{
		std::shared_ptr<GraphRunCtx> ctx;
		std::shared_ptr<RaytraceNode> trace;
		std::vector<Node::Ptr> pre, post;
	};
	void resolveMembers();
	void buildJobs();
	void uploadJobs(const rgl::BatchSchedule& s, cudaStream_t st);
	void computeOrder(int order, cudaStream_t st);
	float timeTrace(const rgl::BatchSchedule& s, int reps);
	void tune();
	void splitWaves();
	void ensureWaveResources();
	void addBranch();
	void enqueueFrame(cudaStream_t s);
	void enqueueMembers(bool preTrace, size_t lo, size_t hi, cudaStream_t s);
	void enqueueTrace(const rgl::BatchSchedule& s, int wave, cudaStream_t st);
	void releaseExec();

	std::vector<Node::Ptr> anchors;
	std::vector<Member> members;
	std::vector<Scene*> scenes; // distinct scenes of the batch's raytrace nodes
	cudaStream_t stream = nullptr;
	std::vector<cudaStream_t> branches;
	cudaEvent_t forkEv = nullptr;
	std::vector<cudaEvent_t> joinEv;
	cudaStream_t postStream = nullptr; // later nodes of each wave
	int priorityHigh = 0;             // the device's greatest stream priority: every kernel but the traversal's
	cudaEvent_t frameStart = nullptr, frameStop = nullptr, traceStart = nullptr, traceStop = nullptr, postJoin = nullptr;
	std::vector<cudaEvent_t> waveTraced; // per wave: its traversal launch completed (capture edges)
	std::vector<cudaEvent_t> waveDone;   // per wave: its graphs' nodes completed (what their reads wait for)
	bool running = false;

	// Job table: host copy, device copy, task prefix sums for the current schedule (dTaskBase: the
	// whole batch's n + 1 sums at 0, then wave w's, rebased to 0, at n + 1 + waveFirst[w] + w).
	std::vector<rgl::BatchJob> jobs;
	std::vector<int64_t> beamBase;
	std::vector<int> waveFirst; // first member of each wave, then members.size()
	int maxSamples = 1;
	bool shading = false;
	std::vector<int64_t> shape;      // per sensor: rays, samples; the tuned shape in tunedShape
	std::vector<int64_t> tunedShape; // shape the schedule and the beam order were made for
	int orderHeld = rgl::kOrderNatural;
	rgl::DeviceBuffer dJobs, dTaskBase, dCounter, dKeys, dOrder, dSortScratch, dError; // dCounter: one block per wave
	size_t counterBytesZeroed = 0;
	std::vector<uint8_t> uploaded; // bytes of the job table and task bases last uploaded
	rgl::DeviceBuffer dParamTable{false}; // the captured frame's parameter copies (read by its gather node)

	// Captured frame.
	cudaGraphExec_t exec = nullptr;
	std::vector<int> execWaveFirst;
	uint64_t execEpoch = 0, execVersion = 0;
	std::vector<uint64_t> execScenes;
	std::vector<Scene*> execSceneList;
	rgl::BatchSchedule execSchedule{};
	std::vector<GraphRunCtx*> execCtxs;
	uint64_t execKernels = 0;
};
