// Data layouts in HBM shared by the BVH builder, the traversal kernel and the host scene code.
//
// Acceleration structure (replaces the OptiX GAS/IAS of reference src/scene/Scene.cpp:131-190 and
// src/scene/GASBuilder.hpp:31-100):
//  * BLAS, one per mesh, in object space: an 8-wide BVH with conservatively quantised child boxes
//    (node layout after Ylitie, Karras, Laine, "Efficient Incoherent Ray Traversal on GPUs Through
//    Compressed Wide BVHs", HPG 2017) plus the mesh's triangles re-ordered leaf by leaf.
//  * TLAS, one per scene: a binary BVH with float boxes over entity (instance) world boxes; its leaves
//    reference instance records that carry the world->object transform and the entity id.
#pragma once

#include <cstdint>
#include <vector_functions.h>
#include <vector_types.h>
#include "rgl_math.hpp"

namespace rgl {

// Maximum triangles referenced by one leaf child of a wide node (3-bit count, 5-bit offset in meta).
constexpr int kLeafMaxTris = 2;
constexpr int kWideArity = 8;

// 80-byte wide node = five 16-byte words, loaded with five 128-bit loads.
//  w0: origin p (3 x f32) | e.x e.y e.z (biased exponent bytes) imask (byte)
//  w1: childBase | triBase | meta[0..3] | meta[4..7]
//  w2: qlo.x[0..7] qlo.y[0..7]
//  w3: qlo.z[0..7] qhi.x[0..7]
//  w4: qhi.y[0..7] qhi.z[0..7]
// A child slot i is
//  * internal when bit i of imask is set: its wide node is childBase + popc(imask & ((1<<i)-1));
//  * a leaf when meta[i] != 0: triangles triBase + (meta[i] & 31) .. + (meta[i] >> 5) - 1;
//  * empty otherwise (its quantised box is empty: qlo = 255 > qhi = 0).
// Child box of slot i on axis a = [p_a + qlo_a[i] * 2^e_a, p_a + qhi_a[i] * 2^e_a], where each sum is
// one float addition whose result the builder verified to enclose the exact child box.
struct alignas(16) WideNode
{
	float px, py, pz;
	uint8_t ex, ey, ez, imask;
	uint32_t childBase;
	uint32_t triBase;
	uint8_t meta[8];
	uint8_t qlox[8], qloy[8], qloz[8];
	uint8_t qhix[8], qhiy[8], qhiz[8];
};
static_assert(sizeof(WideNode) == 80, "wide node is 80 bytes");

// Triangle in leaf order: three 16-byte words (v0.xyz, original triangle index), (v1.xyz, -), (v2.xyz, -).
struct alignas(16) TriRecord
{
	float v0x, v0y, v0z;
	int32_t primId;
	float v1x, v1y, v1z;
	int32_t pad1;
	float v2x, v2y, v2z;
	int32_t pad2;
};
static_assert(sizeof(TriRecord) == 48, "triangle record is 48 bytes");

// Binary BVH node with float bounds (LBVH stage of the BLAS build, and the TLAS).
// Children: value >= 0 internal node index; value < 0 leaf ~primitive (leaf index = ~value).
struct alignas(16) BinNode
{
	float lox, loy, loz;
	int32_t left;
	float hix, hiy, hiz;
	int32_t right;
};
static_assert(sizeof(BinNode) == 32, "binary node is 32 bytes");

// Per-entity record referenced by TLAS leaves.
struct alignas(16) InstanceRec
{
	Mat34 worldToObject;       // 48 B
	Mat34 objectToWorld;       // 48 B
	const WideNode* nodes;     // BLAS of the entity's mesh
	const TriRecord* tris;
	int32_t entityId;
	int32_t hasPrev;           // prevObjectToWorld holds the pose of the scene's previous time step
	float lox, loy, loz, hix, hiy, hiz; // world-space box (TLAS leaf bounds)
	float laserRetro;          // rgl_entity_set_laser_retro
	int32_t flags;             // kInstanceIdentity: objectToWorld is the identity
	Mat34 prevObjectToWorld;   // 48 B, for hit-point velocities
	const float* vertexDisplacement; // animated entity: per-vertex motion since the previous time step, or null
	const int32_t* indices;          // the mesh's triangle vertex indices (with vertexDisplacement, texCoords)
	uint64_t intensityTexture;       // cudaTextureObject_t of 8-bit texels, 0 without one
	const float* texCoords;          // uv per vertex when intensityTexture is set
};

constexpr int32_t kInstanceIdentity = 1;

// A world point in the instance's object frame, as worldToObject applied to the offset from the
// instance origin: the subtraction is exact (or nearly) for points near the instance, so the result
// keeps the precision of the offset instead of losing the instance origin's magnitude (an instance
// 400 m from the world origin would otherwise shift ray origins by ~3e-5 m).
RGL_HD Vec3 worldToInstance(const InstanceRec& ir, Vec3 pW) { return ir.worldToObject.vector(pW - ir.objectToWorld.translation()); }

// Device view of a scene, read by the traversal kernel through one pointer so a captured CUDA graph
// stays valid when the acceleration structure is rebuilt.
struct SceneView
{
	const WideNode* tlas;         // wide nodes over the instances (root = 0), the BLAS node format
	const TriRecord* tlasLeaves;  // leaf records of the TLAS: primId = instance index
	const InstanceRec* instances;
	int32_t nInstances;
	int32_t pad;
};

// Sub-ray table and per-launch parameters of a raytrace (reference RaytraceRequestContext,
// src/gpu/RaytraceRequestContext.hpp:21-78, reduced to what the path uses).
constexpr int kMaxBeamSamples = 64;

enum FieldMask : uint32_t
{
	kOutXyz = 1u << 0,
	kOutDistance = 1u << 1,
	kOutIsHit = 1u << 2,
	kOutEntityId = 1u << 3,
	kOutReturnType = 1u << 4,
	kOutIntensityF32 = 1u << 5,
	kOutRayIdx = 1u << 6,
	kOutIntensityU8 = 1u << 7,
	kOutNormal = 1u << 8,
	kOutIncidentAngle = 1u << 9,
	kOutLaserRetro = 1u << 10,
	kOutRayPose = 1u << 11,
};

struct TraceOutputs
{
	float* xyz;        // 3 floats per point
	float* distance;
	int32_t* isHit;
	int32_t* entityId;
	uint8_t* returnType;
	float* intensityF32;
	uint32_t* rayIdx;
	uint8_t* intensityU8;
	float* normal;     // 3 floats per point
	float* incidentAngle;
	float* laserRetro;
	uint16_t* ringId;
	float* azimuth;
	float* elevation;
	double* timeStampF64;
	uint32_t* timeStampU32;
	float* absVelocity;  // 3 floats per point
	float* relVelocity;  // 3 floats per point
	float* radialSpeed;
};

struct TraceParams
{
	const Mat34* rays;          // nRays ray poses (world)
	const float* ranges;        // 2 floats per entry
	int32_t nRanges;            // 1 or nRays
	int32_t nRays;
	int32_t nSamples;           // 1 + layers * vertices, or 1 without divergence
	int32_t returnMode;
	int32_t returnCount;
	float nearNonHitDistance;
	float farNonHitDistance;
	float defaultIntensity;
	int32_t needIntensity;      // intensity requested or a strongest-type return is selected
	int32_t* errorFlag;         // set when a traversal stack overflows
	const SceneView* scene;
	TraceOutputs out;
	const int32_t* ringIds;     // rays-set-ring-ids values (beam b gets ringIds[b % nRingIds]), or null
	int32_t nRingIds;
	int32_t distortion;         // velocity distortion: rays shifted by their time offset (needs timeOffsetsMs)
	Mat34 worldToSensor;        // inverse of the rays' cumulative transform (azimuth, elevation, distortion)
	Mat34 sensorToWorld;        // the rays' cumulative transform
	Mat34 worldToSensorRotation; // inverse of the rotation part of sensorToWorld
	const float* timeOffsetsMs; // per ray, or null
	float sceneDeltaTime;       // seconds between the scene's last two time steps, 0 when unknown
	Vec3 sensorLinearVelocity;  // rgl_node_raytrace_configure_velocity, sensor frame
	Vec3 sensorAngularVelocity; // roll, pitch, yaw rates in rad/s
	const int8_t* rayMask;      // per ray, 0: not cast (far non-hit), or null
};

// One sensor (or served request) of a batched traversal launch (trace_batch.cu): its raytrace
// parameters including its scene, its sub-ray rotations, an optional beam visiting order, the
// lane-group width of lane-group packing, and optionally a sensor pose applied to sensor-local rays
// and an inline range.
struct BatchJob
{
	TraceParams p;         // p.ranges == null: inlineRange applies to every ray
	const Mat34* samples;  // p.nSamples rotations (entry 0 is the primary ray and is not read)
	const uint32_t* order; // permutation of [0, p.nRays), or null for the natural order
	int32_t groupSize;     // min(p.nSamples, 32)
	int32_t hasRayTransform; // world ray = mul(rayTransform, ray), as a rays-transform node computes it
	Mat34 rayTransform;
	float inlineRange[2];
};

} // namespace rgl
