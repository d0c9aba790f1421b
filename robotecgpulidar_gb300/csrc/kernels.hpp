// Host-side launchers of the CUDA kernels (defined in the .cu files of this directory).
#pragma once

#include <vector>

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "device_types.hpp"

namespace rgl {

struct ParamCopy; // common.hpp

// Counts kernel launches issued by this library (reported by rgl_gb300_get_kernel_launch_count).
void countLaunch(uint64_t n = 1);
uint64_t launchCount();

// ---- sort.cu
size_t sortPairsScratchBytes(int n, int keyBits);
void sortPairs(uint32_t* keys, uint32_t* values, int n, int keyBits, void* scratch, int32_t* errorFlag, cudaStream_t stream);

// ---- bvh.cu
struct BlasBuild
{
	WideNode* nodes = nullptr; // device
	TriRecord* tris = nullptr; // device
	uint32_t nodeCapacity = 0;
	uint32_t nodeCount = 0;      // wide nodes in use
	int32_t triCount = 0;
	float bounds[6] = {0, 0, 0, 0, 0, 0}; // object-space box lo.xyz, hi.xyz (host copy)
};
// Builds a BLAS on the device from device vertices/indices and synchronises `stream` at the end:
// triangle boxes, the binary topology (binned SAH, sah.cu, when `sah`; else Morton codes, onesweep
// sort and LBVH), then the wide collapse. Mesh BLASes use the SAH topology; animated entities, whose
// BLAS is rebuilt at every animation, the LBVH.
void buildBlas(const float* dVertices, int nVertices, const int32_t* dIndices, int nTris, BlasBuild& out, cudaStream_t stream,
               bool sah);
// ---- sah.cu: binary binned-SAH topology of n primitive boxes (device lo/hi), the host builder's tree
// (sah_build.hpp buildBinnedSahTree) computed on the device; output in the collapse's input format.
void buildSahTopologyDevice(const float4* lo, const float4* hi, int n, BinNode* bin, int32_t* rangeFirst, int32_t* rangeLast,
                            uint32_t* sortedIds, cudaStream_t stream);
// The same topology for 1..kSahSmallMax boxes, built by one block with no host interaction (so it can
// be captured in a CUDA graph); `scratch` holds sahSmallScratchBytes(n) bytes.
constexpr int kSahSmallMax = 2048;
size_t sahSmallScratchBytes(int n);
void enqueueSahTopologySmall(const float4* lo, const float4* hi, int n, void* scratch, BinNode* bin, int32_t* rangeFirst,
                             int32_t* rangeLast, uint32_t* sortedIds, cudaStream_t stream);
// Builds the BLAS of a mesh on the host from host vertices/indices (binned SAH topology, the same wide
// collapse) and uploads it; storage of `out` is reused when large enough.
void buildBlasHost(const float* hVertices, int nVertices, const int32_t* hIndices, int nTris, BlasBuild& out);
void freeBlas(BlasBuild& b);

struct TlasBuild
{
	WideNode* nodes = nullptr;       // wide nodes over the instances (at most nInstances)
	TriRecord* leaves = nullptr;     // one record per instance; primId = instance index
	float* boxes = nullptr;          // float box (6 floats) of every wide node, kept for the refit
	int32_t* levelStarts = nullptr;  // first node index of each depth, nLevels + 1 entries (device)
	int32_t* nLevels = nullptr;      // number of depths (device word, read by the refit)
	int32_t levelCapacity = 0;       // entries allocated for levelStarts
	int32_t capacity = 0;
	int32_t nInstances = 0;
	uint32_t nodeCount = 0;          // node count of the last host-synchronous build (statistics)
	// Scratch of the graph-capturable rebuild (instances up to kSahSmallMax), sized with `capacity`.
	float4* lo = nullptr;
	float4* hi = nullptr;
	void* sahScratch = nullptr;
	BinNode* bin = nullptr;
	int32_t* rangeFirst = nullptr;
	int32_t* rangeLast = nullptr;
	uint32_t* sortedIds = nullptr;
};
// Builds the TLAS over `nInstances` instance records (host copy hInstances, device copy dInstances,
// current on `stream`). Up to kSahSmallMax instances it enqueues the graph-capturable rebuild
// (rebuildTlas); beyond, the multi-block device build, which synchronises `stream`.
void buildTlas(const InstanceRec* hInstances, const InstanceRec* dInstances, int nInstances, TlasBuild& t, cudaStream_t stream);
// After instance poses changed (same instance set): a full rebuild of the topology over the new
// world boxes when it can be enqueued without host interaction (up to kSahSmallMax instances: the
// instance boxes, one-block binned SAH, one-block wide collapse), otherwise a refit that keeps the
// topology. A refit only is cheaper but degrades as entities move across the scene: after a few
// frames of random re-poses the old topology's boxes cover most of the scene.
void updateTlas(const InstanceRec* dInstances, TlasBuild& t, cudaStream_t stream);
// Refits the TLAS after instance boxes changed (same instance set): one single-block launch.
void refitTlas(const InstanceRec* dInstances, TlasBuild& t, cudaStream_t stream);
void freeTlas(TlasBuild& t);

// ---- animate.cu: mesh animation of entities
// Four bone influences of a vertex (layout of rgl_bone_weights_t).
struct BoneWeights
{
	float weight[4];
	int32_t bone[4];
};
// Skinned vertices out[i] = sum_k weight_k * (pose[b_k] * restposes[b_k]) * rest[i]; boneMatrices is
// scratch for nBones matrices. A non-zero weight on a bone outside [0, nBones) raises *errorFlag.
void launchSkin(int nVertices, const float* restVertices, const BoneWeights* weights, const Mat34* pose, const Mat34* restposes,
                int nBones, Mat34* boneMatrices, float* out, int32_t* errorFlag, cudaStream_t s);
// newToDisplacement holds the new vertices and receives new - old; oldToNew receives the new ones.
void launchUpdateVertices(int nVertices, float* newToDisplacement, float* oldToNew, cudaStream_t s);

// ---- trace_batch.cu: the traversal, one persistent launch over one or many sensors
constexpr int kMaxBatchJobs = 1024;
enum BatchPacking : int32_t
{
	kPackLaneGroup = 0, // a beam's samples on adjacent lanes, in-order shuffle reduction
	kPackSerial = 1,    // one lane per beam, samples traced one after another
};
enum BeamOrder : int32_t
{
	kOrderNatural = 0,    // beams in the order the client gave them
	kOrderOctahedral = 1, // sorted by an octahedral encoding of the world direction
	kOrderMorton = 2,     // sorted by the Morton code of a point a fixed distance along the ray
	kOrderElevation = 3,  // sorted by the elevation of the world direction, then its azimuth (scan rows)
};
struct BatchSchedule
{
	int32_t block;   // threads per block: 64, 128 or 256
	int32_t packing; // BatchPacking
	int32_t order;   // BeamOrder
	int32_t chunk;   // tasks taken per atomic fetch
	int32_t regs;    // register budget per thread: 64, 80, 96 or 128
};
// Task prefix sums of a one-job launch.
struct TaskRange
{
	int32_t base[2];
};
// Whether a raytrace needs the SHADING variant of the traversal kernel: intensity, normals, incident
// angles, velocities or velocity distortion (the plain variant carries none of that code).
inline bool needsShadingKernel(const TraceParams& p)
{
	return p.needIntensity != 0 || p.out.normal != nullptr || p.out.incidentAngle != nullptr || p.out.absVelocity != nullptr ||
	       p.out.relVelocity != nullptr || p.out.radialSpeed != nullptr || p.distortion != 0;
}
// Beams covered by one task (one warp's worth of work) of a sensor with `nSamples` samples.
int batchBeamsPerTask(int packing, int nSamples);
// Resolves and caches the launch configuration (occupancy, shared-memory opt-in) of a schedule;
// call it outside stream capture before the first captured launch of that schedule.
void prepareTraceBatch(int nJobs, int maxSamples, bool shading, const BatchSchedule& s);
// Adds to `graph` one kernel node that makes the n parameter copies listed in dTable (device memory,
// kept while the graph lives) and makes it the predecessor of every node that had none.
cudaError_t addParamGatherNode(cudaGraph_t graph, const ParamCopy* dTable, int n);
// Whether `fn` (a kernel node's function) is one of the persistent traversal kernels.
bool isTraceBatchKernel(const void* fn);
// The traversal's counter block: task ticket and finished blocks, zeroed once when allocated; every
// launch leaves it zero again.
constexpr size_t kTraceCounterBytes = 2 * sizeof(uint32_t);
// Persistent launch over `nJobs` sensors; dTaskBase holds nJobs + 1 prefix sums of tasks per sensor;
// dCounter is a kTraceCounterBytes counter block (launches that share one must be stream-ordered).
// With `overlapPrevious` the launch uses programmatic stream serialization: when the kernel before it
// on the stream is a traversal launch (which triggers once all its tasks are handed out), its blocks
// start as that launch's blocks exit. Only for launches that read nothing the previous one writes and
// use their own counter block.
void launchTraceBatch(const BatchJob* dJobs, const int32_t* dTaskBase, int nJobs, int maxSamples, bool shading,
                      const BatchSchedule& s, uint32_t* dCounter, cudaStream_t stream, bool overlapPrevious = false);
// ---- segcompact.cu: compaction of many requests' points in three launches
constexpr int kSegTile = 1024; // points per tile
struct SegCompactJob
{
	const int32_t* flags; // nPoints is-hit flags
	const float* xyz;     // nPoints x 3
	const float* dist;
	const int32_t* ent;
	float* outXyz; // kept points, in order
	float* outDist;
	int32_t* outEnt;
	int32_t nPoints;
	int32_t packed; // 1: the segment's output is one block, xyz | distance | entity id of its kept points
	                // back to back from outXyz (distance at outXyz + 3 * kept, entity id at + 4 * kept);
	                // outDist and outEnt are not read
};
// dTileBase: nSeg + 1 prefix sums of ceil(nPoints / kSegTile) per segment; dCounts receives the
// kept count of every segment.
// Copies n words from device memory into pinned host memory through the device's mapping (a kernel,
// not the copy engine, so it never waits behind other streams' copies).
void launchPublishWords(const int32_t* src, int32_t* dstMappedHost, int n, cudaStream_t stream);
void launchSegCompact(const SegCompactJob* dSegs, const int32_t* dTileBase, int nSeg, int totalTiles, uint32_t* dTileCounts,
                      uint32_t* dTileOffsets, int32_t* dCounts, cudaStream_t s);

// Sort keys of one sensor's beams (job index in the top bits) and their local indices.
void launchBeamKeys(const Mat34* rays, const Mat34* transform, int n, uint32_t jobIndex, int order, const float* worldLo, const float* worldHi,
                    uint32_t* keys, uint32_t* values, cudaStream_t stream);

// ---- points.cu
// Transforms and noise parameters are device pointers to values the host stages before each run.
void launchTransformRays(const Mat34* in, Mat34* out, int n, const Mat34* dTf, cudaStream_t s);
void launchTransformPoints(const float* inXyz, float* outXyz, int cap, const int32_t* dCount, const Mat34* dTf, cudaStream_t s);

struct NoiseParams
{
	uint32_t seedLo, seedHi;
	uint32_t frameLo, frameHi;
	uint32_t kind;
	float mean, stDev, stDevRise;
	int32_t axis;
	int32_t pad[3];
	Mat34 lookAt, lookAtInv;
};
void launchNoiseAngularRay(const Mat34* in, Mat34* out, int n, const NoiseParams* dNp, cudaStream_t s);
void launchNoiseAngularHitpoint(const float* inXyz, float* outXyz, float* outDist, int cap, const int32_t* dCount,
                                const NoiseParams* dNp, cudaStream_t s);
void launchNoiseDistance(const float* inXyz, const float* inDist, float* outXyz, float* outDist, int cap, const int32_t* dCount,
                         const NoiseParams* dNp, cudaStream_t s);

// One field of a compaction or format: device source/destination and element size in bytes.
struct FieldCopy
{
	const void* src;
	void* dst;
	int32_t size;   // bytes per element
	int32_t offset; // byte offset inside a formatted point (format only)
};
constexpr int kMaxFieldCopies = 32;
struct FieldCopies
{
	FieldCopy f[kMaxFieldCopies];
	int32_t count;
};

// Concatenation of point clouds (spatial and temporal merge). Input i contributes its first count_i
// points (count_i = *count when count is set, else staticCount).
struct MergeInput
{
	const int32_t* count;
	int32_t staticCount;
	int32_t pad;
};
// Device table of a merge: MergeInput[nInputs] | const void* src[nInputs * nFields] | FieldCopy[nFields]
// (dst and size used), each part 16-byte aligned.
size_t mergeTableBytes(int nInputs, int nFields);
void fillMergeTable(void* table, const std::vector<MergeInput>& inputs, const std::vector<const void*>& src,
                    const std::vector<FieldCopy>& fields);
// Writes input i's points at base + sum_{j<i} count_j of every field's dst (base = *dBase when dBase is
// set, else 0) and, when dOutCount is set, base + sum of all counts to *dOutCount. maxCount bounds every
// count_i.
void launchMergePoints(const void* dTable, int nInputs, int nFields, int maxCount, const int32_t* dBase, int32_t* dOutCount,
                       cudaStream_t s);
// *dAcc += (dAdd ? *dAdd : addStatic), one thread.
void launchAddCount(int32_t* dAcc, const int32_t* dAdd, int32_t addStatic, cudaStream_t s);

// IS_GROUND_I32 of the ground filter (reference nodeKernels.cu:322-332): out[i] = angle between the
// normal and the sensor's up vector (unsigned) > threshold, i.e. 1 for points that are not ground.
void launchGroundFlags(const float* normals, int cap, const int32_t* dCount, Vec3 up, float threshold, int32_t* out, cudaStream_t s);

// Point operations a compaction applies to the XYZ (and distance) of the points it keeps: the chain of
// transform and noise nodes between the compaction and its source, absorbed into its one pass. Each
// operation uses the point's index before compaction, as its own kernel would.
enum PointOpKind : int32_t
{
	kOpTransform = 0,           // params: Mat34 (TransformPointsNode)
	kOpNoiseAngularHitpoint = 1, // params: NoiseParams; withDistance: the distance is recomputed
	kOpNoiseDistance = 2,        // params: NoiseParams
};
constexpr int kMaxPointOps = 4;
struct PointOp
{
	int32_t kind;
	int32_t withDistance;
	const void* params; // device copy, staged by the absorbed node
};
struct PointOps
{
	PointOp op[kMaxPointOps];
	int32_t count;
	int32_t xyzField;     // index of XYZ among the compaction's fields (written from the chain), or -1
	int32_t distField;    // index of DISTANCE, or -1
	int32_t pad;
	const float* srcXyz;  // the chain source's XYZ
	const float* srcDist; // the chain source's distance, or null
};

size_t compactScratchBytes(int cap);
// Stable compaction of `cap` points (first *dInCount valid when dInCount != null) by int32 flags.
// Writes the kept count to *dOutCount. `scratch` (compactScratchBytes) is zero before the first launch
// and each launch leaves it zero. With `ops`, the fields at ops->xyzField / ops->distField are
// computed from the chain's source instead of copied.
// hostCount (optional): pinned host memory mapped for the device that also receives the kept count,
// written by the kernel (no copy node after it).
void launchCompact(const int32_t* flags, int cap, const int32_t* dInCount, const FieldCopies& fields, const PointOps* ops,
                   int32_t* dOutCount, void* scratch, int32_t* dError, cudaStream_t s, int32_t* hostCount = nullptr);
// AoS packing: point i, field k -> out + i*pointSize + offset_k; padding fields (src == null) are zeroed.
void launchFormat(const FieldCopies& fields, int pointSize, int cap, const int32_t* dCount, uint8_t* out, cudaStream_t s);
// AoS -> SoA split for points given as an array (rgl_node_points_from_array).
void launchAosToSoa(const uint8_t* in, int pointSize, int n, const FieldCopies& fields, cudaStream_t s);

} // namespace rgl

// ---- noalloc.cu: compaction whose scratch is a fixed device array (no allocation by the call)
namespace rgl {
constexpr int kNoAllocMaxPoints = 1 << 24;
// Stable compaction of `count` elements of `elementSize` bytes from src to dst (device pointers) by
// int32 flags; waits for completion on `stream` and returns the kept count.
int32_t compactNoAlloc(const int32_t* flags, const void* src, int32_t count, int32_t elementSize, void* dst, cudaStream_t stream);
} // namespace rgl
