#include "scene.hpp"

#include <rgl/api/extensions/gb300.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <set>

using rgl::Mat34;

Mesh::Mesh(const rgl_vec3f* vertices, int32_t vc, const rgl_vec3i* indices, int32_t ic) : vertexCount(vc), triangleCount(ic)
{
	// Indices are validated here (the reference leaves out-of-range indices to device asserts).
	for (int32_t t = 0; t < ic; ++t) {
		for (int k = 0; k < 3; ++k) {
			int32_t v = indices[t].value[k];
			if (v < 0 || v >= vc) {
				throw rgl::InvalidAPIArgument(
				    rgl::format("triangle %d references vertex %d outside [0, %d)", (int) t, (int) v, (int) vc));
			}
		}
	}
	RGL_CHECK_CUDA(cudaMemcpy(dVertices.ensure(sizeof(rgl_vec3f) * vc), vertices, sizeof(rgl_vec3f) * vc, cudaMemcpyHostToDevice));
	RGL_CHECK_CUDA(cudaMemcpy(dIndices.ensure(sizeof(rgl_vec3i) * ic), indices, sizeof(rgl_vec3i) * ic, cudaMemcpyHostToDevice));
	hVertices.assign(&vertices[0].value[0], &vertices[0].value[0] + 3 * (size_t) vc);
	hIndices.assign(&indices[0].value[0], &indices[0].value[0] + 3 * (size_t) ic);
}

Mesh::~Mesh()
{
	if (blasBuilt) {
		rgl::freeBlas(blas);
	}
}

void Mesh::setBoneWeights(const rgl_bone_weights_t* w, int32_t count)
{
	if (count != vertexCount) {
		throw rgl::InvalidAPIArgument(rgl::format("Cannot set bone weights because vertex count do not match with bone weights count: "
		                                          "vertexCount=%d, boneWeightsCount=%d",
		                                          (int) vertexCount, (int) count));
	}
	RGL_CHECK_CUDA(cudaMemcpy(dBoneWeights.ensure(sizeof(rgl_bone_weights_t) * (size_t) count), w,
	                          sizeof(rgl_bone_weights_t) * (size_t) count, cudaMemcpyHostToDevice));
	boneWeightCount = count;
}

void Mesh::setRestposes(const rgl_mat3x4f* r, int32_t count)
{
	RGL_CHECK_CUDA(cudaMemcpy(dRestposes.ensure(sizeof(rgl_mat3x4f) * (size_t) count), r, sizeof(rgl_mat3x4f) * (size_t) count,
	                          cudaMemcpyHostToDevice));
	restposeCount = count;
}

void Mesh::setTexCoords(const rgl_vec2f* uvs, int32_t count)
{
	if (count != vertexCount) {
		throw rgl::InvalidAPIArgument(rgl::format("Cannot set texture coordinates because vertex count do not match with texture "
		                                          "coordinates count: vertexCount=%d, textureCoords=%d",
		                                          (int) vertexCount, (int) count));
	}
	RGL_CHECK_CUDA(cudaMemcpy(dTexCoords.ensure(sizeof(rgl_vec2f) * (size_t) count), uvs, sizeof(rgl_vec2f) * (size_t) count,
	                          cudaMemcpyHostToDevice));
	hasTexCoords = true;
}

Texture::Texture(const void* texels, int32_t w, int32_t h) : width(w), height(h)
{
	const cudaChannelFormatDesc channel = cudaCreateChannelDesc<unsigned char>();
	RGL_CHECK_CUDA(cudaMallocArray(&array, &channel, (size_t) w, (size_t) h));
	const size_t pitch = (size_t) w;
	cudaError_t e = cudaMemcpy2DToArray(array, 0, 0, texels, pitch, pitch, (size_t) h, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		cudaFreeArray(array);
		RGL_CHECK_CUDA(e);
	}
	cudaResourceDesc res{};
	res.resType = cudaResourceTypeArray;
	res.res.array.array = array;
	cudaTextureDesc tex{};
	tex.addressMode[0] = cudaAddressModeWrap;
	tex.addressMode[1] = cudaAddressModeWrap;
	tex.filterMode = cudaFilterModePoint;
	tex.readMode = cudaReadModeElementType;
	tex.normalizedCoords = 1;
	tex.maxAnisotropy = 1;
	tex.maxMipmapLevelClamp = 99;
	tex.minMipmapLevelClamp = 0;
	tex.mipmapFilterMode = cudaFilterModePoint;
	tex.borderColor[0] = 1.0f;
	e = cudaCreateTextureObject(&object, &res, &tex, nullptr);
	if (e != cudaSuccess) {
		cudaFreeArray(array);
		RGL_CHECK_CUDA(e);
	}
}

Texture::~Texture()
{
	if (object) {
		cudaDestroyTextureObject(object);
	}
	if (array) {
		cudaFreeArray(array);
	}
}

namespace {
std::atomic<int32_t> gBlasBuilder{RGL_GB300_BLAS_DEVICE_SAH};
std::atomic<int64_t> gBlasBuilds{0};
std::atomic<int64_t> gBlasBuildNs{0};
} // namespace

void setBlasBuilder(int32_t builder) { gBlasBuilder = builder; }
void blasBuildStats(int64_t& builds, double& ms)
{
	builds = gBlasBuilds.load();
	ms = (double) gBlasBuildNs.load() * 1e-6;
}

// The mesh's BLAS, built by the configured builder (rgl_gb300_configure_blas_builder) on first use:
// by default on the device (binned SAH topology, sah.cu, then the wide collapse); the host build of
// the same tree and the device LBVH stay selectable.
void Mesh::ensureBlas(cudaStream_t s)
{
	if (blasBuilt) {
		return;
	}
	const auto t0 = std::chrono::steady_clock::now();
	switch (gBlasBuilder.load()) {
		case RGL_GB300_BLAS_HOST_SAH:
			rgl::buildBlasHost(hVertices.data(), vertexCount, hIndices.data(), triangleCount, blas);
			break;
		case RGL_GB300_BLAS_DEVICE_LBVH:
			rgl::buildBlas(dVertices.as<float>(), vertexCount, dIndices.as<int32_t>(), triangleCount, blas, s, false);
			break;
		default:
			rgl::buildBlas(dVertices.as<float>(), vertexCount, dIndices.as<int32_t>(), triangleCount, blas, s, true);
			break;
	}
	gBlasBuildNs += std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
	++gBlasBuilds;
	blasBuilt = true;
}

Entity::Entity(std::shared_ptr<Mesh> m, Scene* s) : mesh(std::move(m)), scene(s) {}

Entity::~Entity()
{
	if (animBlas.nodes != nullptr) {
		rgl::freeBlas(animBlas);
	}
}

// First animation: the animated vertices start as the mesh's, the displacement as zero.
void Entity::startAnimation()
{
	if (animated) {
		return;
	}
	const size_t bytes = sizeof(float) * 3 * (size_t) mesh->vertexCount;
	RGL_CHECK_CUDA(cudaMemcpy(dAnimVertices.ensure(bytes), mesh->dVertices.get(), bytes, cudaMemcpyDeviceToDevice));
	RGL_CHECK_CUDA(cudaMemset(dAnimDisplacement.ensure(bytes), 0, bytes));
	animated = true;
}

// dAnimDisplacement holds the new vertices: turn it into new - old, store new, rebuild the entity's
// BLAS and record the animation time.
void Entity::finishAnimation(cudaStream_t s)
{
	rgl::launchUpdateVertices(mesh->vertexCount, dAnimDisplacement.as<float>(), dAnimVertices.as<float>(), s);
	rgl::buildBlas(dAnimVertices.as<float>(), mesh->vertexCount, mesh->dIndices.as<int32_t>(), mesh->triangleCount, animBlas, s, false);
	RGL_CHECK_CUDA(cudaStreamSynchronize(s));
	formerAnimTimed = animTimed;
	formerAnimTimeNs = animTimeNs;
	animTimed = scene->timeSet;
	animTimeNs = scene->timeNs;
	scene->markPosesDirty(); // the instance record points at the rebuilt BLAS
}

void Entity::applyExternalAnimation(const rgl_vec3f* vertices, int32_t count)
{
	if (skinned) {
		throw rgl::InvalidAPIArgument("entity is animated by its skeleton; external animation cannot be applied");
	}
	if (count != mesh->vertexCount) {
		throw rgl::InvalidAPIArgument(rgl::format(
		    "Invalid argument: cannot apply external animation because vertex counts do not match: old=%d, new=%d", (int) mesh->vertexCount,
		    (int) count));
	}
	startAnimation();
	RGL_CHECK_CUDA(cudaMemcpy(dAnimDisplacement.get(), vertices, sizeof(float) * 3 * (size_t) count, cudaMemcpyHostToDevice));
	finishAnimation(nullptr);
}

void Entity::setPoseAndAnimate(const rgl_mat3x4f* pose, int32_t bones)
{
	if (animated && !skinned) {
		throw rgl::InvalidAPIArgument("entity is animated externally; skeleton animation cannot be applied");
	}
	if (mesh->boneWeightCount == 0) {
		throw rgl::InvalidAPIArgument("Cannot create SkeletonAnimator because mesh has no bone weights defined.");
	}
	if (mesh->restposeCount == 0) {
		throw rgl::InvalidAPIArgument("Cannot create SkeletonAnimator because mesh has no restposes defined.");
	}
	if (bones != mesh->restposeCount) {
		throw rgl::InvalidAPIArgument(rgl::format(
		    "Cannot perform skeleton animation because bones count do not match restposes count: bones=%d, restposes=%d", (int) bones,
		    (int) mesh->restposeCount));
	}
	startAnimation();
	skinned = true;
	RGL_CHECK_CUDA(cudaMemcpy(dPose.ensure(sizeof(rgl_mat3x4f) * (size_t) bones), pose, sizeof(rgl_mat3x4f) * (size_t) bones,
	                          cudaMemcpyHostToDevice));
	rgl::launchSkin(mesh->vertexCount, mesh->dVertices.as<float>(), mesh->dBoneWeights.as<rgl::BoneWeights>(), dPose.as<Mat34>(),
	                mesh->dRestposes.as<Mat34>(), bones, static_cast<Mat34*>(dBoneMatrices.ensure(sizeof(Mat34) * (size_t) bones)),
	                dAnimDisplacement.as<float>(), skinError.device(), nullptr);
	finishAnimation(nullptr);
	rgl::refreshErrorSlots();
	if (skinError.raised()) {
		skinError.clear();
		throw rgl::InvalidAPIArgument("bone weights reference a bone outside the pose");
	}
}

const float* Entity::vertexDisplacementSincePrevFrame() const
{
	if (!animated || !formerAnimTimed || !scene->prevTimeSet || formerAnimTimeNs != scene->prevTimeNs) {
		return nullptr;
	}
	return dAnimDisplacement.as<float>();
}

void Entity::setTransform(const Mat34& tf)
{
	formerTransform = transform;
	formerTimed = transformTimed;
	formerTimeNs = transformTimeNs;
	transform = tf;
	transformTimed = scene->timeSet;
	transformTimeNs = scene->timeNs;
	scene->markPosesDirty();
}

bool Entity::previousTransform(Mat34& out) const
{
	// Set only once: assume the same pose one step earlier (zero velocity), as for static objects.
	if (transformTimed && !formerTimed) {
		out = transform;
		return true;
	}
	if (formerTimed && scene->prevTimeSet && formerTimeNs == scene->prevTimeNs) {
		out = formerTransform;
		return true;
	}
	return false;
}

void Scene::setTime(uint64_t ns)
{
	prevTimeNs = timeNs;
	prevTimeSet = timeSet;
	timeNs = ns;
	timeSet = true;
	markPosesDirty(); // previous poses in the instance records depend on the time step
}

float Scene::deltaTimeSeconds() const
{
	if (!timeSet || !prevTimeSet) {
		return 0.0f;
	}
	return (float) ((double) ((int64_t) (timeNs - prevTimeNs)) * 1e-9);
}

void Entity::setId(int32_t newId)
{
	// The reference limits ids to the OptiX instance-id range (src/scene/Entity.cpp:43-52).
	constexpr int32_t maxId = 1 << 28;
	if (newId >= maxId) {
		throw std::invalid_argument(rgl::format("Entity ID (%d) must be less than %d", (int) newId, (int) maxId));
	}
	id = newId;
	scene->markPosesDirty();
}

void Entity::setIntensityTexture(std::shared_ptr<Texture> t)
{
	intensityTexture = std::move(t);
	scene->markPosesDirty(); // the texture travels in the instance record
}

void Entity::setLaserRetro(float retro)
{
	laserRetro = retro;
	scene->markPosesDirty(); // the value travels in the instance record
}

Scene& Scene::defaultScene()
{
	static Scene scene;
	return scene;
}

Scene::Scene() = default;

Scene::~Scene()
{
	// The default scene lives until process exit; the CUDA context may already be gone then.
}

void Scene::addEntity(const std::shared_ptr<Entity>& e)
{
	entities.push_back(e);
	topologyDirty = true;
}

void Scene::removeEntity(Entity* e)
{
	entities.erase(std::remove_if(entities.begin(), entities.end(), [&](const std::shared_ptr<Entity>& p) { return p.get() == e; }),
	               entities.end());
	topologyDirty = true;
}

void Scene::clear()
{
	entities.clear();
	topologyDirty = true;
	posesDirty = true;
	timeSet = false;
	timeNs = 0;
	prevTimeSet = false;
	prevTimeNs = 0;
}

void Scene::releaseDevice()
{
	rgl::freeTlas(tlas);
	dInstances.release();
	dView.release();
	if (ready) {
		cudaEventDestroy(ready);
		ready = nullptr;
	}
	readyRecorded = false;
	topologyDirty = true;
	posesDirty = true;
}

void Scene::stats(int64_t& nodeBytes, int64_t& triangleBytes) const
{
	std::set<const Mesh*> seen;
	nodeBytes = 0;
	triangleBytes = 0;
	for (auto& e : entities) {
		const Mesh* m = e->mesh.get();
		if (!m->blasBuilt || !seen.insert(m).second) {
			continue;
		}
		nodeBytes += (int64_t) m->blas.nodeCount * (int64_t) sizeof(rgl::WideNode);
		triangleBytes += (int64_t) m->blas.triCount * (int64_t) sizeof(rgl::TriRecord);
	}
}

void Scene::checkDeviceErrors()
{
	if (dError.raised()) {
		dError.clear();
		throw std::runtime_error("acceleration structure build failed on the device (radix sort look-back timed out)");
	}
}

// Instance records (world boxes padded outward) in pinned host memory, and the world bounds.
rgl::InstanceRec* Scene::fillInstanceRecords()
{
	static const Mat34 identityPose = Mat34::identity();
	const int n = (int) entities.size();
	worldLo[0] = worldLo[1] = worldLo[2] = INFINITY;
	worldHi[0] = worldHi[1] = worldHi[2] = -INFINITY;
	auto* rec = static_cast<rgl::InstanceRec*>(hInstances.ensure(sizeof(rgl::InstanceRec) * std::max(1, n)));
	for (int i = 0; i < n; ++i) {
		const Entity& e = *entities[i];
		rgl::InstanceRec r{};
		r.objectToWorld = e.transform;
		r.worldToObject = rgl::inverse(e.transform);
		r.flags = std::memcmp(&e.transform, &identityPose, sizeof(Mat34)) == 0 ? rgl::kInstanceIdentity : 0;
		const rgl::BlasBuild& bl = e.activeBlas();
		r.nodes = bl.nodes;
		r.tris = bl.tris;
		r.vertexDisplacement = e.vertexDisplacementSincePrevFrame();
		r.indices = e.mesh->dIndices.as<int32_t>();
		const bool textured = e.intensityTexture && e.mesh->hasTexCoords;
		r.intensityTexture = textured ? (uint64_t) e.intensityTexture->object : 0;
		r.texCoords = textured ? e.mesh->dTexCoords.as<float>() : nullptr;
		r.entityId = e.id;
		r.laserRetro = e.laserRetro;
		r.hasPrev = e.previousTransform(r.prevObjectToWorld) ? 1 : 0;
		const float* b = bl.bounds;
		float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
		for (int c = 0; c < 8; ++c) {
			rgl::Vec3 p = e.transform.point(rgl::v3((c & 1) ? b[3] : b[0], (c & 2) ? b[4] : b[1], (c & 4) ? b[5] : b[2]));
			float q[3] = {p.x, p.y, p.z};
			for (int a = 0; a < 3; ++a) {
				lo[a] = std::min(lo[a], q[a]);
				hi[a] = std::max(hi[a], q[a]);
			}
		}
		// Outward padding covers the rounding of the corner transform.
		float mag = 1.0f;
		for (int a = 0; a < 3; ++a) {
			mag = std::max({mag, std::fabs(lo[a]), std::fabs(hi[a])});
		}
		float pad = 4e-6f * mag;
		r.lox = lo[0] - pad;
		r.loy = lo[1] - pad;
		r.loz = lo[2] - pad;
		r.hix = hi[0] + pad;
		r.hiy = hi[1] + pad;
		r.hiz = hi[2] + pad;
		rec[i] = r;
		for (int a = 0; a < 3; ++a) {
			worldLo[a] = std::min(worldLo[a], (&r.lox)[a]);
			worldHi[a] = std::max(worldHi[a], (&r.hix)[a]);
		}
	}
	return rec;
}

void Scene::prepare(cudaStream_t s)
{
	if (ready == nullptr) {
		RGL_CHECK_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
	}
	(void) dError.device();
	if (!topologyDirty && !posesDirty && readyRecorded) {
		RGL_CHECK_CUDA(cudaStreamWaitEvent(s, ready, 0));
		return;
	}
	const int n = (int) entities.size();
	if (n >= (1 << 24)) {
		// The traversal packs the hit's instance index into 24 bits.
		throw rgl::InvalidAPIArgument(rgl::format("a scene holds at most %d entities, got %d", (1 << 24) - 1, n));
	}
	for (auto& e : entities) {
		e->mesh->ensureBlas(s);
	}
	auto* rec = fillInstanceRecords();
	auto* dInst = static_cast<rgl::InstanceRec*>(dInstances.ensure(sizeof(rgl::InstanceRec) * std::max(1, n)));
	if (n > 0) {
		RGL_CHECK_CUDA(cudaMemcpyAsync(dInst, rec, sizeof(rgl::InstanceRec) * n, cudaMemcpyHostToDevice, s));
	}
	if (topologyDirty || tlas.nInstances != n) {
		rgl::buildTlas(rec, dInst, n, tlas, s);
		++tlasBuilds;
	} else {
		rgl::updateTlas(dInst, tlas, s);
		++tlasRefits;
	}
	auto* v = static_cast<rgl::SceneView*>(hView.ensure(sizeof(rgl::SceneView)));
	v->tlas = tlas.nodes;
	v->tlasLeaves = tlas.leaves;
	v->instances = dInst;
	v->nInstances = n;
	v->pad = 0;
	RGL_CHECK_CUDA(cudaMemcpyAsync(dView.ensure(sizeof(rgl::SceneView)), v, sizeof(rgl::SceneView), cudaMemcpyHostToDevice, s));
	RGL_CHECK_CUDA(cudaEventRecord(ready, s));
	readyRecorded = true;
	topologyDirty = false;
	posesDirty = false;
}

void Scene::prepareBatched(cudaStream_t s)
{
	if (topologyDirty || !readyRecorded || tlas.nInstances != (int) entities.size()) {
		prepare(s);
		return;
	}
	if (posesDirty) {
		fillInstanceRecords();
		posesDirty = false;
	}
}

void Scene::enqueueRefit(cudaStream_t s)
{
	const int n = (int) entities.size();
	if (n == 0) {
		return;
	}
	RGL_CHECK_CUDA(cudaMemcpyAsync(dInstances.get(), hInstances.get(), sizeof(rgl::InstanceRec) * n, cudaMemcpyHostToDevice, s));
	rgl::updateTlas(dInstances.as<rgl::InstanceRec>(), tlas, s);
}

void Scene::recordReady(cudaStream_t s)
{
	RGL_CHECK_CUDA(cudaEventRecord(ready, s));
	readyRecorded = true;
}
