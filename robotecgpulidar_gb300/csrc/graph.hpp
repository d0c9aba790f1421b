// Graph runtime behind rgl_node_t (reference src/graph/Node.hpp:57-214, Interfaces.hpp:24-145,
// GraphRunCtx.cpp:23-211, NodesCore.hpp).
//
// Nodes keep RGL's semantics: create-or-modify parameters, DAG links with priorities, a per-graph
// CUDA stream, validation on the client thread at rgl_graph_run, results readable from any node of
// the graph after the run. Differences in mechanism (not in results):
//  * runs are enqueued by the calling thread (no per-run host thread);
//  * compaction keeps its point count on the device; downstream kernels read it from there and the
//    host reads it only when a result size is requested;
//  * formatted output stays on the device until rgl_graph_get_result_data copies it.
#pragma once

#include <map>
#include <memory>
#include <optional>
#include <set>
#include <string>
#include <vector>

#include "common.hpp"
#include "kernels.hpp"

struct GraphRunCtx;
struct Scene;

struct Node : std::enable_shared_from_this<Node>
{
	using Ptr = std::shared_ptr<Node>;
	virtual ~Node() = default;
	virtual const char* name() const = 0;

	void addChild(const Ptr& child);
	void removeChild(const Ptr& child);
	void setPriority(int32_t p);
	std::set<Ptr> connectedComponent();
	std::set<Ptr> disconnectConnectedNodes();

	virtual void validateImpl() = 0;
	// Host-side work of a run that must not be captured into a CUDA graph: sizing buffers, scene
	// builds and refits, per-run parameters. Runs before every run, in execution order.
	virtual void prepareImpl(cudaStream_t) {}
	// Enqueues the node's device work; must not allocate (it may be captured into a CUDA graph).
	virtual void enqueueImpl(cudaStream_t s) = 0;
	// Called after the graph's stream completed; throws if a kernel of this node raised its error flag.
	virtual void checkErrors() {}
	// Host-side parameters changed: the node must re-upload or re-plan at the next run.
	void markDirty() { dirty = true; }

	template<class T>
	std::shared_ptr<T> exactlyOneInput(const char* ifaceName);

	// True when the last parameter update changed only device-buffer contents (same sizes), so a
	// captured run stays valid.
	virtual bool lastUpdateContentOnly() const { return false; }

	// A parameter baked into this node's launches changed: captured runs that contain the node are
	// stale. Versions come from one process-wide counter, so a capture that remembers the largest
	// version of its nodes detects every later change, whoever else captured the node meanwhile.
	void markParamsChanged() { paramVersion = nextParamVersion(); }
	static uint64_t nextParamVersion();

	std::vector<Ptr> inputs, outputs;
	int32_t priority = 0;
	bool dirty = true;
	uint64_t paramVersion = nextParamVersion();
	std::shared_ptr<GraphRunCtx> ctx;
};

// ---------------------------------------------------------------- rays

struct RaysNode : virtual Node
{
	virtual size_t rayCount() const = 0;
	virtual const rgl::Mat34* raysDev() const = 0;
	virtual const float* rangesDev() const { return nullptr; } // 2 floats per entry
	virtual size_t rangesCount() const { return 0; }
	virtual rgl::Mat34 cumulativeRayTransform() const { return rgl::Mat34::identity(); }
	virtual const int32_t* ringIdsDev() const { return nullptr; } // null: no ring ids upstream
	virtual size_t ringIdsCount() const { return 0; }
	virtual const float* timeOffsetsDev() const { return nullptr; }
	virtual size_t timeOffsetsCount() const { return 0; }
	// True for nodes that pass their input's ray poses through unchanged (ranges, ring ids, offsets).
	virtual bool passesRaysThrough() const { return false; }
};

struct RaysNodeSingleInput : RaysNode
{
	void validateImpl() override;
	size_t rayCount() const override { return input->rayCount(); }
	const rgl::Mat34* raysDev() const override { return input->raysDev(); }
	const float* rangesDev() const override { return input->rangesDev(); }
	size_t rangesCount() const override { return input->rangesCount(); }
	rgl::Mat34 cumulativeRayTransform() const override { return input->cumulativeRayTransform(); }
	const int32_t* ringIdsDev() const override { return input->ringIdsDev(); }
	size_t ringIdsCount() const override { return input->ringIdsCount(); }
	const float* timeOffsetsDev() const override { return input->timeOffsetsDev(); }
	size_t timeOffsetsCount() const override { return input->timeOffsetsCount(); }

protected:
	std::shared_ptr<RaysNode> input;
};

struct FromMat3x4fRaysNode : RaysNode
{
	const char* name() const override { return "FromMat3x4fRaysNode"; }
	void setParameters(const rgl_mat3x4f* rays, size_t count);
	void validateImpl() override;
	void enqueueImpl(cudaStream_t) override {}
	size_t rayCount() const override { return count; }
	const rgl::Mat34* raysDev() const override { return rays.as<rgl::Mat34>(); }
	bool lastUpdateContentOnly() const override { return sameCount; }

private:
	rgl::DeviceBuffer rays;
	size_t count = 0;
	bool sameCount = false;
};

struct TransformRaysNode : RaysNodeSingleInput
{
	const char* name() const override { return "TransformRaysNode"; }
	void setParameters(const rgl::Mat34& tf) { transform = tf; }
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	const rgl::Mat34* raysDev() const override { return out.as<rgl::Mat34>(); }
	rgl::Mat34 cumulativeRayTransform() const override { return rgl::mul(transform, input->cumulativeRayTransform()); }
	bool lastUpdateContentOnly() const override { return true; } // the transform is staged every run

	// Folded into the traversal of its only consumer: the raytrace reads this node's input rays and
	// applies `transform` in its prologue with the same arithmetic, and this node launches nothing.
	bool folded = false;
	const rgl::Mat34* sourceRaysDev() const { return input->raysDev(); }
	const rgl::Mat34& matrix() const { return transform; }

private:
	rgl::Mat34 transform = rgl::Mat34::identity();
	rgl::StagedParam<rgl::Mat34> staged;
	rgl::DeviceBuffer out;
};

struct SetRangeRaysNode : RaysNodeSingleInput
{
	const char* name() const override { return "SetRangeRaysNode"; }
	bool passesRaysThrough() const override { return true; }
	void setParameters(const rgl_vec2f* ranges, size_t count);
	void validateImpl() override;
	void enqueueImpl(cudaStream_t) override {}
	const float* rangesDev() const override { return ranges.as<float>(); }
	size_t rangesCount() const override { return count; }

private:
	rgl::DeviceBuffer ranges;
	size_t count = 0;
};

// Ring ids of the rays (reference src/graph/SetRaysRingIdsRaysNode.cpp:17-33): beam b gets
// ids[b % count]; the ray count must be a multiple of the id count.
struct SetRingIdsRaysNode : RaysNodeSingleInput
{
	const char* name() const override { return "SetRingIdsRaysNode"; }
	bool passesRaysThrough() const override { return true; }
	void setParameters(const int32_t* ids, size_t n);
	void validateImpl() override;
	void enqueueImpl(cudaStream_t) override {}
	const int32_t* ringIdsDev() const override { return ids.as<int32_t>(); }
	size_t ringIdsCount() const override { return count; }

private:
	rgl::DeviceBuffer ids;
	size_t count = 0;
};

// Per-ray time offsets in milliseconds (reference src/graph/SetTimeOffsetsRaysNode.cpp:17-33), one per
// ray. They feed velocity distortion, which this build does not apply.
struct SetTimeOffsetsRaysNode : RaysNodeSingleInput
{
	const char* name() const override { return "SetTimeOffsetsRaysNode"; }
	bool passesRaysThrough() const override { return true; }
	void setParameters(const float* offsets, size_t n);
	void validateImpl() override;
	void enqueueImpl(cudaStream_t) override {}
	const float* timeOffsetsDev() const override { return offsets.as<float>(); }
	size_t timeOffsetsCount() const override { return count; }

private:
	rgl::DeviceBuffer offsets;
	size_t count = 0;
};

struct GaussianNoiseAngularRaysNode : RaysNodeSingleInput
{
	const char* name() const override { return "GaussianNoiseAngularRaysNode"; }
	void setParameters(float mean, float stDev, rgl_axis_t axis);
	void setSeed(uint64_t s, uint64_t f)
	{
		seed = s;
		frame = f;
	}
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	const rgl::Mat34* raysDev() const override { return out.as<rgl::Mat34>(); }
	bool lastUpdateContentOnly() const override { return true; } // parameters are staged every run

private:
	float mean = 0, stDev = 0;
	rgl_axis_t axis = RGL_AXIS_X;
	uint64_t seed = 0, frame = 0;
	rgl::DeviceBuffer out;
	rgl::StagedParam<rgl::NoiseParams> staged;
};

// ---------------------------------------------------------------- points

struct PointsNode : virtual Node
{
	virtual std::vector<rgl_field_t> requiredFields() const { return {}; }
	virtual bool isDense() const = 0;
	virtual bool hasField(rgl_field_t f) const = 0;
	// Upper bound of the point count, exact unless deviceCount() is set.
	virtual size_t capacity() const = 0;
	// Device int32 holding the exact count when it is only known on the device (after compaction).
	virtual const int32_t* deviceCount() const { return nullptr; }
	// Pinned host copy of deviceCount(), written by the run itself; valid once the run completed.
	virtual const int32_t* hostCount() const { return nullptr; }
	virtual int32_t returnMode() const { return RGL_RETURN_UNKNOWN; }
	virtual rgl::Mat34 lookAtOriginTransform() const { return rgl::Mat34::identity(); }
	// Device pointer with capacity() elements of `field`; valid after this node's enqueue.
	virtual const void* fieldDev(rgl_field_t field) = 0;
	virtual size_t fieldPointSize(rgl_field_t field) const { return rgl::fieldSize(field); }
	// Exact point count; reads the device count (graph must be synchronised).
	size_t pointCountHost();
};

struct PointsNodeSingleInput : PointsNode
{
	void validateImpl() override;
	bool isDense() const override { return input->isDense(); }
	bool hasField(rgl_field_t f) const override { return input->hasField(f); }
	size_t capacity() const override { return input->capacity(); }
	const int32_t* deviceCount() const override { return input->deviceCount(); }
	const int32_t* hostCount() const override { return input->hostCount(); }
	int32_t returnMode() const override { return input->returnMode(); }
	rgl::Mat34 lookAtOriginTransform() const override { return input->lookAtOriginTransform(); }
	const void* fieldDev(rgl_field_t f) override { return input->fieldDev(f); }

protected:
	std::shared_ptr<PointsNode> input;
};

// A node that maps XYZ (and distance) point by point: transform and point noise. When its only
// consumer leads, through such nodes, to a compaction, the compaction applies it to the points it keeps
// in its own pass (kCompact's point operations) and this node launches nothing; its fields are then
// computed only if asked for directly after the run.
struct PointwisePointsNode : PointsNodeSingleInput
{
	void validateImpl() override
	{
		PointsNodeSingleInput::validateImpl();
		absorbed = false;
	}
	// Stages this node's parameters on `s` and appends its operation.
	virtual void appendPointOp(rgl::PointOps& ops, cudaStream_t s) = 0;
	std::shared_ptr<PointsNode> source() const { return input; }
	bool absorbed = false;

protected:
	// Per-run bookkeeping of an absorbed node (call from prepareImpl).
	void beginRun(cudaStream_t s)
	{
		lastStream = s;
		computedOnDemand = false;
	}
	// Runs the node's own kernel on the run's stream and waits, once per run (absorbed nodes only).
	void computeOnDemand();
	virtual void allocateOutputs() = 0;
	virtual void launchOwn(cudaStream_t s) = 0;

private:
	cudaStream_t lastStream = nullptr;
	bool computedOnDemand = false;
};

struct RaytraceNode : PointsNode
{
	const char* name() const override { return "RaytraceNode"; }
	void validateImpl() override;
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	bool isDense() const override { return false; }
	bool hasField(rgl_field_t f) const override { return fields.count(f) != 0; }
	size_t capacity() const override { return rays ? (size_t) returnCount() * rays->rayCount() : 0; }
	int32_t returnMode() const override { return mode; }
	rgl::Mat34 lookAtOriginTransform() const override { return rgl::inverse(rays->cumulativeRayTransform()); }
	const void* fieldDev(rgl_field_t f) override;

	int returnCount() const { return (int) (((uint32_t) mode) >> 24); }
	void setReturnMode(int32_t m) { mode = m; }
	void setBeamDivergence(float h, float v)
	{
		hDivergence = h;
		vDivergence = v;
	}
	void setBeamSamples(int layers, int vertices)
	{
		sampleLayers = layers;
		sampleVertices = vertices;
	}
	void setNonHits(float nearD, float farD)
	{
		nearDistance = nearD;
		farDistance = farD;
	}
	void setDefaultIntensity(float i) { defaultIntensity = i; }
	void setVelocity(rgl::Vec3 linear, rgl::Vec3 angular)
	{
		sensorLinearVelocity = linear;
		sensorAngularVelocity = angular;
	}
	void setDistortion(bool on) { distortion = on; }
	// Rays whose mask entry is 0 are not cast: their beams return the far non-hit (reference
	// optixPrograms.cu:55-58).
	void setRayMask(const int8_t* mask, size_t count);
	int sampleCount() const;
	void checkErrors() override;
	std::shared_ptr<Scene> sceneRef; // keeps a scene made by rgl_gb300_scene_create alive
	// Launch parameters of the traversal for the current buffers (valid after prepareImpl).
	rgl::TraceParams traceParams();
	// The node's job of a traversal launch (parameters, sub-ray table, lane-group width, a folded
	// sensor transform); order and task bases are the launcher's.
	void fillJob(rgl::BatchJob& b);
	void stageJob(cudaStream_t s);
	const rgl::Mat34* sampleTableDev() const { return sampleTable.as<rgl::Mat34>(); }
	Scene* scene = nullptr;

	// Timing (extension): device time of the traversal kernel of the last run.
	cudaEvent_t evStart = nullptr, evStop = nullptr;

private:
	std::set<rgl_field_t> findFieldsToCompute();
	std::shared_ptr<RaysNode> rays;
	std::shared_ptr<TransformRaysNode> foldedTransform; // see TransformRaysNode::folded
	std::set<rgl_field_t> fields;
	std::map<rgl_field_t, rgl::DeviceBuffer> outputs;
	rgl::DeviceBuffer defaultRange;
	rgl::DeviceBuffer sampleTable;
	int uploadedSamples = -1;
	float uploadedH = -1, uploadedV = -1;
	int32_t mode = RGL_RETURN_FIRST;
	float hDivergence = 0, vDivergence = 0;
	int sampleLayers = 3, sampleVertices = 19; // reference pattern: 1 + 3 * 19 = 58 samples
	float nearDistance = INFINITY, farDistance = INFINITY;
	float defaultIntensity = 0.0f;
	rgl::Vec3 sensorLinearVelocity{0.0f, 0.0f, 0.0f}, sensorAngularVelocity{0.0f, 0.0f, 0.0f};
	bool distortion = false;
	rgl::DeviceBuffer rayMask;
	size_t rayMaskCount = 0;
	rgl::ErrorSlot errorFlag;
	// The node's traversal as a one-job persistent launch.
	// The job and its task bases, uploaded by one copy per run.
	struct StagedTrace
	{
		rgl::BatchJob job;
		rgl::TaskRange tasks;
	};
	rgl::StagedParam<StagedTrace> job;
	rgl::DeviceBuffer counter;
	rgl::BatchSchedule schedule{};
	bool shading = false;
	// Beam visiting order of the launch (schedule.order other than as given): the sorted beam indices,
	// made when the ray count, the ray buffer or the order kind changes. Later ray contents of the same
	// count keep it: any permutation gives the same results, only the speed depends on it. The job
	// carries the pointer, staged every run, so the buffers may move without a new capture.
	void ensureOrder(const rgl::BatchJob& b, cudaStream_t s);
	rgl::DeviceBuffer orderKeys{false}, orderVals{false}, orderScratch{false}, orderError{false};
	int32_t orderCount = -1, orderKind = rgl::kOrderNatural;
	const void* orderRays = nullptr;
	bool orderValid = false;
};

struct YieldPointsNode : PointsNodeSingleInput
{
	const char* name() const override { return "YieldPointsNode"; }
	void setParameters(const std::vector<rgl_field_t>& f);
	std::vector<rgl_field_t> requiredFields() const override { return fields; }
	bool hasField(rgl_field_t f) const override;
	void enqueueImpl(cudaStream_t) override {}

private:
	std::vector<rgl_field_t> fields;
};

struct FormatPointsNode : PointsNodeSingleInput
{
	const char* name() const override { return "FormatPointsNode"; }
	void setParameters(const std::vector<rgl_field_t>& f);
	std::vector<rgl_field_t> requiredFields() const override { return fields; }
	bool hasField(rgl_field_t f) const override;
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	const void* fieldDev(rgl_field_t f) override;
	size_t fieldPointSize(rgl_field_t f) const override;

private:
	std::vector<rgl_field_t> fields;
	rgl::DeviceBuffer out;
};

struct CompactByFieldPointsNode : PointsNodeSingleInput
{
	const char* name() const override { return "CompactByFieldPointsNode"; }
	void setParameters(rgl_field_t f) { field = f; }
	std::vector<rgl_field_t> requiredFields() const override { return {field}; }
	void validateImpl() override;
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	bool isDense() const override { return true; }
	const int32_t* deviceCount() const override { return count.as<int32_t>(); }
	const int32_t* hostCount() const override { return static_cast<const int32_t*>(hCount.get()); }
	const void* fieldDev(rgl_field_t f) override;
	void checkErrors() override;
	// Number of transform / noise nodes this compaction applies in its own pass (for tests).
	size_t absorbedCount() const { return chain.size(); }

private:
	rgl_field_t field = RGL_FIELD_IS_HIT_I32;
	std::set<rgl_field_t> eager;               // fields compacted during the run
	std::map<rgl_field_t, rgl::DeviceBuffer> outputs;
	std::set<rgl_field_t> lazyDone;            // fields compacted on demand after the run
	std::vector<std::shared_ptr<PointwisePointsNode>> chain; // absorbed nodes, source side first
	std::shared_ptr<PointsNode> chainSource;   // input of chain.front()
	rgl::DeviceBuffer count;
	rgl::PinnedBuffer hCount;
	int32_t* hCountDev = nullptr; // device address of hCount (the kernel stores the count there)
	rgl::DeviceBuffer scratch;
	rgl::ErrorSlot errorFlag;
	cudaStream_t lastStream = nullptr;
	void sizeBuffers(const std::vector<rgl_field_t>& which);
	void compact(const std::vector<rgl_field_t>& which, cudaStream_t s, int32_t* hostCount = nullptr);
};

struct TransformPointsNode : PointwisePointsNode
{
	const char* name() const override { return "TransformPointsNode"; }
	void setParameters(const rgl::Mat34& tf) { transform = tf; }
	std::vector<rgl_field_t> requiredFields() const override { return {RGL_FIELD_XYZ_VEC3_F32}; }
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	rgl::Mat34 lookAtOriginTransform() const override
	{
		return rgl::mul(rgl::inverse(transform), input->lookAtOriginTransform());
	}
	const void* fieldDev(rgl_field_t f) override;
	bool lastUpdateContentOnly() const override { return true; } // the transform is staged every run
	void appendPointOp(rgl::PointOps& ops, cudaStream_t s) override;

protected:
	void allocateOutputs() override;
	void launchOwn(cudaStream_t s) override;

private:
	rgl::Mat34 transform = rgl::Mat34::identity();
	rgl::StagedParam<rgl::Mat34> staged;
	rgl::DeviceBuffer out;
};

struct GaussianNoiseAngularHitpointNode : PointwisePointsNode
{
	const char* name() const override { return "GaussianNoiseAngularHitpointNode"; }
	void setParameters(float mean, float stDev, rgl_axis_t axis);
	void setSeed(uint64_t s, uint64_t f)
	{
		seed = s;
		frame = f;
	}
	std::vector<rgl_field_t> requiredFields() const override { return {RGL_FIELD_XYZ_VEC3_F32}; }
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	const void* fieldDev(rgl_field_t f) override;
	bool lastUpdateContentOnly() const override { return true; } // parameters are staged every run
	void appendPointOp(rgl::PointOps& ops, cudaStream_t s) override;

protected:
	void allocateOutputs() override;
	void launchOwn(cudaStream_t s) override;

private:
	float mean = 0, stDev = 0;
	rgl_axis_t axis = RGL_AXIS_X;
	uint64_t seed = 0, frame = 0;
	bool withDistance = false;
	rgl::DeviceBuffer outXyz, outDist;
	rgl::StagedParam<rgl::NoiseParams> staged;
};

struct GaussianNoiseDistanceNode : PointwisePointsNode
{
	const char* name() const override { return "GaussianNoiseDistanceNode"; }
	void setParameters(float mean, float base, float rise);
	void setSeed(uint64_t s, uint64_t f)
	{
		seed = s;
		frame = f;
	}
	std::vector<rgl_field_t> requiredFields() const override { return {RGL_FIELD_XYZ_VEC3_F32, RGL_FIELD_DISTANCE_F32}; }
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	const void* fieldDev(rgl_field_t f) override;
	bool lastUpdateContentOnly() const override { return true; } // parameters are staged every run
	void appendPointOp(rgl::PointOps& ops, cudaStream_t s) override;

protected:
	void allocateOutputs() override;
	void launchOwn(cudaStream_t s) override;

private:
	float mean = 0, base = 0, rise = 0;
	uint64_t seed = 0, frame = 0;
	rgl::DeviceBuffer outXyz, outDist;
	rgl::StagedParam<rgl::NoiseParams> staged;
};

struct FromArrayPointsNode : PointsNode
{
	const char* name() const override { return "FromArrayPointsNode"; }
	void setParameters(const void* points, size_t count, const std::vector<rgl_field_t>& fields);
	void validateImpl() override;
	void enqueueImpl(cudaStream_t) override {}
	bool isDense() const override { return true; }
	bool hasField(rgl_field_t f) const override { return data.count(f) != 0; }
	size_t capacity() const override { return count; }
	const void* fieldDev(rgl_field_t f) override;

private:
	size_t count = 0;
	std::map<rgl_field_t, rgl::DeviceBuffer> data;
};

// Ground classification by normals (reference src/graph/FilterGroundPointsNode.cpp:17-50): adds
// IS_GROUND_I32, 1 where the normal is more than the threshold away from the sensor's up vector (the
// reference's flag marks the points to keep when compacting by it).
struct FilterGroundPointsNode : PointsNodeSingleInput
{
	const char* name() const override { return "FilterGroundPointsNode"; }
	void setParameters(rgl::Vec3 upVector, float threshold)
	{
		up = upVector;
		angle = threshold;
	}
	std::vector<rgl_field_t> requiredFields() const override { return {RGL_FIELD_XYZ_VEC3_F32, RGL_FIELD_NORMAL_VEC3_F32}; }
	bool hasField(rgl_field_t f) const override { return f == RGL_FIELD_IS_GROUND_I32 || input->hasField(f); }
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	const void* fieldDev(rgl_field_t f) override;
	bool lastUpdateContentOnly() const override { return false; }

private:
	rgl::Vec3 up{0.0f, 0.0f, 1.0f};
	float angle = 0.0f;
	rgl::DeviceBuffer flags;
};

// Concatenation of >= 2 unorganised point clouds, inputs in the order they were linked (reference
// src/graph/SpatialMergePointsNode.cpp:18-82). One kernel copies every field of every input; when an
// input's count lives on the device (after compaction) the offsets and the merged count are found on
// the device too, so the merge needs no host synchronisation.
struct SpatialMergePointsNode : PointsNode
{
	const char* name() const override { return "SpatialMergePointsNode"; }
	void setParameters(const std::vector<rgl_field_t>& f);
	std::vector<rgl_field_t> requiredFields() const override { return fields; }
	void validateImpl() override;
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	bool isDense() const override;
	bool hasField(rgl_field_t f) const override { return outputs.count(f) != 0; }
	size_t capacity() const override;
	const int32_t* deviceCount() const override { return onDevice ? count.as<int32_t>() : nullptr; }
	const int32_t* hostCount() const override { return onDevice ? static_cast<const int32_t*>(hCount.get()) : nullptr; }
	const void* fieldDev(rgl_field_t f) override;

private:
	std::vector<rgl_field_t> fields;
	std::map<rgl_field_t, rgl::DeviceBuffer> outputs;
	std::vector<std::shared_ptr<PointsNode>> pointInputs;
	bool onDevice = false;
	rgl::DeviceBuffer count, table;
	rgl::PinnedBuffer hCount, hTable;
	int maxCount = 0;
};

// Accumulates the input's points over runs until its fields are set again (reference
// src/graph/TemporalMergePointsNode.cpp:18-48, which appends into host arrays). Here the accumulated
// cloud stays on the device: each run appends at the device-resident count; storage grows
// geometrically in the prepare phase.
struct TemporalMergePointsNode : PointsNodeSingleInput
{
	const char* name() const override { return "TemporalMergePointsNode"; }
	void setParameters(const std::vector<rgl_field_t>& f);
	std::vector<rgl_field_t> requiredFields() const override { return fields; }
	bool hasField(rgl_field_t f) const override { return outputs.count(f) != 0; }
	void validateImpl() override;
	void prepareImpl(cudaStream_t s) override;
	void enqueueImpl(cudaStream_t s) override;
	size_t capacity() const override { return bound; }
	const int32_t* deviceCount() const override { return count.as<int32_t>(); }
	const int32_t* hostCount() const override { return static_cast<const int32_t*>(hCount.get()); }
	const void* fieldDev(rgl_field_t f) override;

private:
	std::vector<rgl_field_t> fields;
	std::map<rgl_field_t, std::unique_ptr<rgl::DeviceBuffer>> outputs;
	size_t bound = 0;     // upper bound of the accumulated count, including the current run
	size_t allocated = 0; // points each output buffer holds
	bool reset = true;
	rgl::DeviceBuffer count, table;
	rgl::PinnedBuffer hCount, hTable;
};

// ---------------------------------------------------------------- run context

struct GraphRunCtx : std::enable_shared_from_this<GraphRunCtx>
{
	static std::shared_ptr<GraphRunCtx> createAndAttach(const Node::Ptr& node);
	static void synchronizeAll();
	static std::vector<std::shared_ptr<GraphRunCtx>>& instances();

	~GraphRunCtx();
	void run();
	// Waits for the last run and checks the nodes' device error flags (re-reading them from the
	// device unless the caller has just done so for this run).
	void synchronize(bool refreshErrors = true);
	void detachAndDestroy();
	cudaStream_t stream() const { return stream_; }
	void invalidateOrder() { order.clear(); }

	// Batched frames (batch.cpp) drive the graph themselves: they validate and prepare it, enqueue
	// its nodes inside the frame, and mark the graph as running until `frameDone` (recorded by the
	// frame once the graph's nodes are done, owned by the batch) completes, so results are read
	// through the usual calls. forgetBatchEvent drops an event the batch is about to destroy.
	uint64_t validateForBatch(); // waits for the previous run; returns the largest parameter version
	void prepareForBatch(cudaStream_t s);
	void markBatchedRun(cudaEvent_t frameDone);
	void forgetBatchEvent(cudaEvent_t frameDone);
	const std::vector<Node::Ptr>& executionOrder() const { return order; }

	std::set<Node::Ptr> nodes;
	float lastRunMs = 0.0f, lastTraceMs = 0.0f;
	uint64_t captures = 0, replays = 0;

private:
	GraphRunCtx();
	static std::vector<Node::Ptr> findExecutionOrder(std::set<Node::Ptr> nodes);
	void releaseGraph();
	std::vector<Node::Ptr> order;
	cudaStream_t stream_ = nullptr;
	cudaEvent_t done = nullptr, runStart = nullptr, runStop = nullptr;
	cudaEvent_t batchDone = nullptr; // completion of the graph's part of the last batched frame
	uint64_t validatedEpoch = 0;     // graphEditEpoch() of the last successful batch validation
	bool validated = false;
	bool running = false;
	bool batchedLast = false; // the last run was part of a batched frame (no per-graph timing)
	// Captured run: replayed while no node changed and no buffer moved.
	cudaGraphExec_t exec = nullptr;
	uint64_t execEpoch = 0;
	uint64_t execVersion = 0;
	bool execTimed = false; // the capture holds the run-timing events
	uint64_t execKernels = 0;
};

bool timingEnabled();
void setTimingEnabled(bool on);
// Traversal schedule of single-graph runs (rgl_gb300_configure_trace_schedule).
rgl::BatchSchedule traceSchedule();
void setTraceSchedule(const rgl::BatchSchedule& s);
bool cudaGraphsEnabled();
void setCudaGraphsEnabled(bool on);
// Records `ev` on `s`; inside a stream capture the record becomes a node of the captured graph.
void recordEvent(cudaEvent_t ev, cudaStream_t s);
// Counter of API calls that may have changed a graph (nodes, parameters, links, scene time): a
// graph validated at the current value needs no validation again.
void noteGraphEdit();
uint64_t graphEditEpoch();
