// Scene objects behind rgl_mesh_t / rgl_entity_t (reference src/scene/Mesh.cpp, Entity.cpp, Scene.cpp).
//
// A Mesh owns its device vertices/indices and, once a raytrace needs it, its BLAS (shared by every
// entity of the mesh). A Scene owns the per-entity instance records and the TLAS. Pose and id changes
// only mark the scene; the next raytrace refits the TLAS (same entity set) or rebuilds it (entities
// added or removed) on its own stream, without blocking the host.
#pragma once

#include <memory>
#include <vector>

#include "common.hpp"
#include "kernels.hpp"

struct Scene;

// Builder of mesh BLASes built from now on (RGL_GB300_BLAS_*), and the count and wall time of builds.
void setBlasBuilder(int32_t builder);
void blasBuildStats(int64_t& builds, double& ms);

struct Mesh
{
	Mesh(const rgl_vec3f* vertices, int32_t vertexCount, const rgl_vec3i* indices, int32_t indexCount);
	~Mesh();
	void ensureBlas(cudaStream_t s);

	// Skinning data (reference src/scene/Mesh.cpp:44-66): one rgl_bone_weights_t per vertex, one
	// restpose (inverse bind pose) per bone.
	void setBoneWeights(const rgl_bone_weights_t* w, int32_t count);
	void setRestposes(const rgl_mat3x4f* r, int32_t count);

	int32_t vertexCount = 0;
	int32_t triangleCount = 0;
	rgl::DeviceBuffer dVertices{false};
	rgl::DeviceBuffer dIndices{false};
	std::vector<float> hVertices;   // host copies for the host BLAS build (RGL_GB300_BLAS_HOST_SAH)
	std::vector<int32_t> hIndices;
	rgl::BlasBuild blas;
	bool blasBuilt = false;
	rgl::DeviceBuffer dBoneWeights{false}, dRestposes{false};
	int32_t boneWeightCount = 0, restposeCount = 0;
	// Texture coordinates, one per vertex (reference Mesh.cpp:24-37).
	void setTexCoords(const rgl_vec2f* uvs, int32_t count);
	rgl::DeviceBuffer dTexCoords{false};
	bool hasTexCoords = false;
};

struct Entity
{
	Entity(std::shared_ptr<Mesh> m, Scene* s);
	void setTransform(const rgl::Mat34& tf);
	void setId(int32_t id);
	void setLaserRetro(float retro);
	~Entity();
	// Mesh animation of this entity (reference src/scene/Entity.cpp:83-118, animator/*): new object-space
	// vertices (given, or skinned from the mesh's bones); the entity then has its own BLAS over them.
	void applyExternalAnimation(const rgl_vec3f* vertices, int32_t count);
	void setPoseAndAnimate(const rgl_mat3x4f* pose, int32_t bones);
	// Per-vertex displacement since the previous scene time step, or null (reference Entity.cpp:112-118).
	const float* vertexDisplacementSincePrevFrame() const;
	const rgl::BlasBuild& activeBlas() const { return animated ? animBlas : mesh->blas; }

	// Pose of the scene's previous time step, if known (reference src/scene/Entity.cpp:62-81).
	bool previousTransform(rgl::Mat34& out) const;

	std::shared_ptr<Mesh> mesh;
	Scene* scene;
	rgl::Mat34 transform = rgl::Mat34::identity();
	bool transformTimed = false;       // the transform was set while the scene had a time
	uint64_t transformTimeNs = 0;
	rgl::Mat34 formerTransform = rgl::Mat34::identity();
	bool formerTimed = false;
	uint64_t formerTimeNs = 0;
	// Animation state: animated vertices, their displacement since the previous animation, bone
	// matrices (skinning), the entity's BLAS over the animated vertices, animation times.
	bool animated = false;
	bool skinned = false;
	rgl::DeviceBuffer dAnimVertices{false}, dAnimDisplacement{false}, dBoneMatrices{false}, dPose{false};
	rgl::BlasBuild animBlas;
	bool animTimed = false, formerAnimTimed = false;
	uint64_t animTimeNs = 0, formerAnimTimeNs = 0;
	rgl::ErrorSlot skinError;
	int32_t id = RGL_DEFAULT_ENTITY_ID;
	float laserRetro = 0.0f;
	std::shared_ptr<Texture> intensityTexture;
	void setIntensityTexture(std::shared_ptr<Texture> t);

private:
	void startAnimation();
	void finishAnimation(cudaStream_t s);
};

// Intensity texture (reference src/scene/Texture.cpp:22-67): 8-bit texels in a CUDA array behind a
// texture object with the reference's sampling (point filter, wrap addressing, normalised coordinates,
// element reads).
struct Texture
{
	Texture(const void* texels, int32_t width, int32_t height);
	~Texture();
	cudaArray_t array = nullptr;
	cudaTextureObject_t object = 0;
	int32_t width = 0, height = 0;
};

struct Scene
{
	static Scene& defaultScene();
	Scene();
	~Scene();

	void addEntity(const std::shared_ptr<Entity>& e);
	void removeEntity(Entity* e);
	void clear();
	// Frees the TLAS and instance buffers (a scene made by rgl_gb300_scene_create being destroyed).
	void releaseDevice();
	void markPosesDirty() { posesDirty = true; }

	// Builds/refits what changed on stream `s`; afterwards `s` may read view().
	void prepare(cudaStream_t s);
	// Batched frames refit inside their captured graph: prepareBatched() does what cannot be
	// captured (new BLAS, TLAS topology: through prepare()) and otherwise only refreshes the pinned
	// instance records after pose changes; enqueueRefit() uploads the records and refits the TLAS on
	// `s` and may be captured. structureVersion() changes whenever the buffers enqueueRefit() uses
	// may have moved.
	void prepareBatched(cudaStream_t s);
	void enqueueRefit(cudaStream_t s);
	void recordReady(cudaStream_t s);
	uint64_t structureVersion() const { return tlasBuilds; }
	// World bounds of the instance boxes at the last prepare.
	const float* worldLower() const { return worldLo; }
	const float* worldUpper() const { return worldHi; }
	const rgl::SceneView* view() const { return dView.as<rgl::SceneView>(); }
	size_t entityCount() const { return entities.size(); }
	// Bytes of built BLAS wide nodes and triangle records over the distinct meshes in the scene.
	void stats(int64_t& nodeBytes, int64_t& triangleBytes) const;
	int32_t* errorFlag() { return dError.device(); }
	void checkDeviceErrors();

	uint64_t timeNs = 0;
	bool timeSet = false;
	uint64_t prevTimeNs = 0;
	bool prevTimeSet = false;
	// rgl_scene_set_time: the current time becomes the previous one (reference src/scene/Scene.hpp:60-67).
	void setTime(uint64_t ns);
	// Seconds between the last two time steps, 0 when there is no previous one.
	float deltaTimeSeconds() const;

	// Statistics for the extension API.
	uint64_t tlasBuilds = 0, tlasRefits = 0;

private:
	rgl::InstanceRec* fillInstanceRecords();
	std::vector<std::shared_ptr<Entity>> entities;
	float worldLo[3] = {0, 0, 0}, worldHi[3] = {0, 0, 0};
	bool topologyDirty = true;
	bool posesDirty = true;
	rgl::DeviceBuffer dInstances{false};
	rgl::PinnedBuffer hInstances;
	rgl::DeviceBuffer dView; // fixed size: its address never changes once allocated
	rgl::PinnedBuffer hView;
	rgl::ErrorSlot dError;
	rgl::TlasBuild tlas;
	cudaEvent_t ready = nullptr;
	bool readyRecorded = false;
};
