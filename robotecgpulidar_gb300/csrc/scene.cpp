#include "scene.hpp"

#include <algorithm>
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
}

Mesh::~Mesh()
{
	if (blasBuilt) {
		rgl::freeBlas(blas);
	}
}

void Mesh::ensureBlas(cudaStream_t s)
{
	if (blasBuilt) {
		return;
	}
	rgl::buildBlas(dVertices.as<float>(), vertexCount, dIndices.as<int32_t>(), triangleCount, blas, s);
	blasBuilt = true;
}

Entity::Entity(std::shared_ptr<Mesh> m, Scene* s) : mesh(std::move(m)), scene(s) {}

void Entity::setTransform(const Mat34& tf)
{
	transform = tf;
	scene->markPosesDirty();
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
	const int n = (int) entities.size();
	worldLo[0] = worldLo[1] = worldLo[2] = INFINITY;
	worldHi[0] = worldHi[1] = worldHi[2] = -INFINITY;
	auto* rec = static_cast<rgl::InstanceRec*>(hInstances.ensure(sizeof(rgl::InstanceRec) * std::max(1, n)));
	for (int i = 0; i < n; ++i) {
		const Entity& e = *entities[i];
		rgl::InstanceRec r{};
		r.objectToWorld = e.transform;
		r.worldToObject = rgl::inverse(e.transform);
		r.nodes = e.mesh->blas.nodes;
		r.tris = e.mesh->blas.tris;
		r.entityId = e.id;
		r.laserRetro = e.laserRetro;
		const float* b = e.mesh->blas.bounds;
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
	for (auto& e : entities) {
		e->mesh->ensureBlas(s);
	}
	auto* rec = fillInstanceRecords();
	auto* dInst = static_cast<rgl::InstanceRec*>(dInstances.ensure(sizeof(rgl::InstanceRec) * std::max(1, n)));
	if (n > 0) {
		RGL_CHECK_CUDA(cudaMemcpyAsync(dInst, rec, sizeof(rgl::InstanceRec) * n, cudaMemcpyHostToDevice, s));
	}
	if (topologyDirty || tlas.nInstances != n) {
		rgl::buildTlas(rec, n, tlas, s);
		++tlasBuilds;
	} else {
		rgl::refitTlas(dInst, tlas, s);
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
	rgl::refitTlas(dInstances.as<rgl::InstanceRec>(), tlas, s);
}

void Scene::recordReady(cudaStream_t s)
{
	RGL_CHECK_CUDA(cudaEventRecord(ready, s));
	readyRecorded = true;
}
