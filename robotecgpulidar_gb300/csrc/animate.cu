// Mesh animation of entities (reference src/gpu/sceneKernels.cu:17-63, src/scene/animator/*):
// skinning of a mesh's rest vertices by its bones, and the update of an entity's animated vertices
// that also keeps, per vertex, the displacement since the previous animation (for hit velocities).
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace rgl {

namespace {

constexpr int kBlock = 256;

// animation matrix of bone b = pose_b * restpose_b (restpose: inverse bind pose).
__global__ void kBoneMatrices(int bones, const Mat34* __restrict__ pose, const Mat34* __restrict__ restposes, Mat34* __restrict__ out)
{
	const int b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b < bones) {
		out[b] = mul(pose[b], restposes[b]);
	}
}

// Linear blend skinning with four bones per vertex; the weights are taken as given.
__global__ void kSkin(int n, const float* __restrict__ rest, const BoneWeights* __restrict__ weights, const Mat34* __restrict__ bones,
                      int nBones, float* __restrict__ out, int32_t* __restrict__ errorFlag)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) {
		return;
	}
	const Vec3 v = v3(rest[3 * i], rest[3 * i + 1], rest[3 * i + 2]);
	const BoneWeights w = weights[i];
	Vec3 acc = v3(0.0f, 0.0f, 0.0f);
	for (int k = 0; k < 4; ++k) {
		const int b = w.bone[k];
		if (b < 0 || b >= nBones) {
			if (w.weight[k] != 0.0f) {
				*(volatile int32_t*) errorFlag = 1; // a weighted bone outside the pose: reported, not read
			}
			continue;
		}
		acc = acc + bones[b].point(v) * w.weight[k];
	}
	out[3 * i] = acc.x;
	out[3 * i + 1] = acc.y;
	out[3 * i + 2] = acc.z;
}

// newToDisplacement: new vertices in, new - old out; oldToNew: old vertices in, new vertices out.
__global__ void kUpdateVertices(int n3, float* __restrict__ newToDisplacement, float* __restrict__ oldToNew)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n3) {
		const float fresh = newToDisplacement[i];
		newToDisplacement[i] = fsub(fresh, oldToNew[i]);
		oldToNew[i] = fresh;
	}
}

inline int blocks(long n) { return (int) ((n + kBlock - 1) / kBlock); }

} // namespace

void launchSkin(int nVertices, const float* restVertices, const BoneWeights* weights, const Mat34* pose, const Mat34* restposes,
                int nBones, Mat34* boneMatrices, float* out, int32_t* errorFlag, cudaStream_t s)
{
	kBoneMatrices<<<blocks(nBones), kBlock, 0, s>>>(nBones, pose, restposes, boneMatrices);
	countLaunch();
	kSkin<<<blocks(nVertices), kBlock, 0, s>>>(nVertices, restVertices, weights, boneMatrices, nBones, out, errorFlag);
	countLaunch();
}

void launchUpdateVertices(int nVertices, float* newToDisplacement, float* oldToNew, cudaStream_t s)
{
	kUpdateVertices<<<blocks(3L * nVertices), kBlock, 0, s>>>(3 * nVertices, newToDisplacement, oldToNew);
	countLaunch();
}

} // namespace rgl
