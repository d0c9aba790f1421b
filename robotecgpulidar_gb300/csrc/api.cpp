// C API of libRobotecGPULidar.so (declarations: include/rgl/api/core.h and
// include/rgl/api/extensions/gb300.h).
//
// Error handling follows reference src/api/apiCommon.hpp:55-139 and apiCommon.cpp:18-91: every call
// runs inside safeCall(), which maps exceptions to status codes, stores the last error string and
// latches RGL_INVALID_STATE after an unrecoverable error. Argument checks produce the reference's
// message "RGL API Error: Invalid argument, condition unsatisfied: <expression>"; unknown handles
// produce "RGL API Error: Object does not exist: <Type> <pointer>".
#include <cmath>
#include <cstring>
#include <functional>
#include <optional>
#include <random>
#include <set>
#include <unordered_map>

#include <rgl/api/core.h>
#include <rgl/api/extensions/gb300.h>
#include <rgl/api/extensions/tape.h>

#include "batch.hpp"
#include "tape.hpp"
#include "serve.hpp"
#include "graph.hpp"
#include "scene.hpp"

namespace T = rgl::tape;

using namespace rgl;

namespace {

rgl_status_t lastStatus = RGL_SUCCESS;
std::optional<std::string> lastMessage;

const char* lastErrorString()
{
	if (lastMessage) {
		return lastMessage->c_str();
	}
	switch (lastStatus) {
		case RGL_SUCCESS: return "operation successful";
		case RGL_INVALID_ARGUMENT: return "invalid argument";
		case RGL_INTERNAL_EXCEPTION: return "unhandled internal exception";
		case RGL_INVALID_STATE: return "invalid state - unrecoverable error occurred";
		case RGL_NOT_IMPLEMENTED: return "operation not (yet) implemented";
		case RGL_LOGGING_ERROR: return "logging error";
		case RGL_INVALID_FILE_PATH: return "invalid file path";
		case RGL_TAPE_ERROR: return "tape error";
		case RGL_UDP_ERROR: return "UDP error";
		case RGL_ROS2_ERROR: return "ROS2 error";
		default: return "???";
	}
}

bool recoverable(rgl_status_t s)
{
	static const std::set<rgl_status_t> ok = {RGL_INVALID_ARGUMENT,  RGL_INVALID_API_OBJECT, RGL_INVALID_PIPELINE,
	                                          RGL_INVALID_FILE_PATH, RGL_NOT_IMPLEMENTED,    RGL_TAPE_ERROR,
	                                          RGL_UDP_ERROR,         RGL_ROS2_ERROR};
	return s == RGL_SUCCESS || ok.count(s) != 0;
}

rgl_status_t updateState(rgl_status_t s, std::optional<std::string> msg = std::nullopt)
{
	lastMessage = std::move(msg);
	lastStatus = s;
	if (s != RGL_SUCCESS) {
		if (recoverable(s)) {
			logMessage(LogLevel::Error, format("Recoverable error (code=%d): %s", (int) s, lastErrorString()));
		} else {
			logMessage(LogLevel::Critical, format("Unrecoverable error (code=%d): %s", (int) s, lastErrorString()));
		}
	}
	return s;
}

// Calls that cannot change what a graph's validation finds (runs, result reads, poses, statistics)
// use safeCallKeepingValidation; every other call counts as a possible graph edit (noteGraphEdit), so
// a batched frame re-validates its graphs only after some other call.
template<class Fn>
rgl_status_t safeCallKeepingValidation(Fn&& fn)
{
	static bool initTried = false;
	if (!initTried) {
		initTried = true;
		try {
			ensureCudaInitialized();
		}
		catch (std::exception& e) {
			return updateState(RGL_INITIALIZATION_ERROR, std::string(e.what()));
		}
	}
	if (!recoverable(lastStatus)) {
		return updateState(RGL_INVALID_STATE);
	}
	try {
		fn();
	}
	catch (InvalidAPIObject& e) {
		return updateState(RGL_INVALID_API_OBJECT, std::string(e.what()));
	}
	catch (rgl::tape::RecordError& e) {
		return updateState(RGL_TAPE_ERROR, std::string(e.what()));
	}
	catch (rgl::tape::InvalidFilePath& e) {
		return updateState(RGL_INVALID_FILE_PATH, std::string(e.what()));
	}
	catch (InvalidPipeline& e) {
		return updateState(RGL_INVALID_PIPELINE, std::string(e.what()));
	}
	catch (NotImplemented& e) {
		return updateState(RGL_NOT_IMPLEMENTED, std::string(e.what()));
	}
	catch (std::invalid_argument& e) {
		return updateState(RGL_INVALID_ARGUMENT, std::string(e.what()));
	}
	catch (std::exception& e) {
		return updateState(RGL_INTERNAL_EXCEPTION, std::string(e.what()));
	}
	catch (...) {
		return updateState(RGL_INTERNAL_EXCEPTION, std::string("exceptional exception"));
	}
	return updateState(RGL_SUCCESS);
}

template<class Fn>
rgl_status_t safeCall(Fn&& fn)
{
	noteGraphEdit();
	return safeCallKeepingValidation(std::forward<Fn>(fn));
}

#define CHECK_ARG(expr)                                                                                                        \
	do {                                                                                                                       \
		if (!(expr)) {                                                                                                         \
			throw std::invalid_argument("RGL API Error: Invalid argument, condition unsatisfied: " #expr);                    \
		}                                                                                                                      \
	} while (0)

// Handle registry (reference src/APIObject.hpp:35-110): raw handle -> owning shared_ptr.
template<class T>
struct Registry
{
	static std::unordered_map<T*, std::shared_ptr<T>>& map()
	{
		static std::unordered_map<T*, std::shared_ptr<T>> m;
		return m;
	}
	static T* add(const std::shared_ptr<T>& p)
	{
		map()[p.get()] = p;
		return p.get();
	}
	static std::shared_ptr<T> get(T* raw, const char* typeName)
	{
		auto it = map().find(raw);
		if (it == map().end()) {
			throw InvalidAPIObject(format("RGL API Error: Object does not exist: %s %p", typeName, (void*) raw));
		}
		return it->second;
	}
	static void release(T* raw, const char* typeName)
	{
		get(raw, typeName);
		map().erase(raw);
	}
	static bool contains(T* raw) { return map().count(raw) != 0; }
};

using Nodes = Registry<Node>;
using Meshes = Registry<Mesh>;
using Entities = Registry<Entity>;
using Textures = Registry<Texture>;
using Batches = Registry<BatchRun>;
using Servers = Registry<Server>;
using Scenes = Registry<Scene>; // scenes made by rgl_gb300_scene_create (NULL is the default scene)

// The scene behind a handle: NULL is the default scene, as in the reference; other handles come from
// rgl_gb300_scene_create. The returned pointer keeps a created scene alive for nodes that trace it.
std::shared_ptr<Scene> sceneOf(rgl_scene_t scene)
{
	if (scene == nullptr) {
		return std::shared_ptr<Scene>(&Scene::defaultScene(), [](Scene*) {});
	}
	return Scenes::get(scene, "Scene");
}

std::shared_ptr<Node> getNode(rgl_node_t n) { return Nodes::get(n, "Node"); }

template<class T>
std::shared_ptr<T> getNodeAs(rgl_node_t n, const char* typeName)
{
	auto node = getNode(n);
	auto t = std::dynamic_pointer_cast<T>(node);
	if (!t) {
		throw InvalidAPIObject(format("RGL API Error: Node type mismatch: expected %s, got %s", typeName, node->name()));
	}
	return t;
}

// Create-or-modify idiom (reference apiCommon.hpp:108-139).
template<class T, class Setter>
void createOrUpdateNode(rgl_node_t* handle, const char* typeName, Setter&& set)
{
	std::shared_ptr<T> node;
	if (*handle == nullptr) {
		node = std::make_shared<T>();
	} else {
		node = getNodeAs<T>(*handle, typeName);
	}
	if (node->ctx) {
		node->ctx->synchronize();
	}
	set(*node);
	node->dirty = true;
	if (!node->lastUpdateContentOnly()) {
		node->markParamsChanged();
	}
	if (*handle == nullptr) {
		*handle = Nodes::add(node);
	}
}

Mat34 toMat(const rgl_mat3x4f& m)
{
	Mat34 r;
	std::memcpy(r.m, m.value, sizeof(r.m));
	return r;
}

void releaseGraph(const std::shared_ptr<Node>& node)
{
	if (node->ctx) {
		node->ctx->detachAndDestroy();
	}
	for (auto& n : node->disconnectConnectedNodes()) {
		Nodes::map().erase(n.get());
	}
}

// Bytes of a points-from-array input, as the tape stores it (0 when the arguments are invalid).
size_t tapePointBytes(const void* points, int32_t count, const rgl_field_t* fields, int32_t fieldCount)
{
	if (points == nullptr || fields == nullptr || count <= 0 || fieldCount <= 0) {
		return 0;
	}
	try {
		return (size_t) count * rgl::pointSize(std::vector<rgl_field_t>(fields, fields + fieldCount));
	}
	catch (std::exception&) {
		return 0;
	}
}

[[noreturn]] void notImplemented(const char* what)
{
	throw NotImplemented(format("%s is not implemented by this GB300 build", what));
}

// Default noise seed, as random as the reference's std::random_device seeding.
uint64_t randomSeed()
{
	std::random_device rd;
	return ((uint64_t) rd() << 32) ^ (uint64_t) rd();
}

} // namespace

// ================================================================ general

RGL_API rgl_status_t rgl_get_version_info(int32_t* out_major, int32_t* out_minor, int32_t* out_patch)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_major != nullptr);
		CHECK_ARG(out_minor != nullptr);
		CHECK_ARG(out_patch != nullptr);
		*out_major = RGL_VERSION_MAJOR;
		*out_minor = RGL_VERSION_MINOR;
		*out_patch = RGL_VERSION_PATCH;
	});
	RGL_TAPE_RECORD(T::num(out_major ? *out_major : 0), T::num(out_minor ? *out_minor : 0), T::num(out_patch ? *out_patch : 0));
	return status;
}

RGL_API rgl_status_t rgl_get_extension_info(rgl_extension_t extension, int32_t* out_available)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(0 <= extension && extension < RGL_EXTENSION_COUNT);
		CHECK_ARG(out_available != nullptr);
		*out_available = 0; // PCL, ROS2, UDP and weather extensions are not part of this build
	});
	RGL_TAPE_RECORD(T::num(extension), T::num(out_available ? *out_available : 0));
	return status;
}

RGL_API rgl_status_t rgl_configure_logging(rgl_log_level_t log_level, const char* log_file_path, bool use_stdout)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(0 <= log_level && log_level <= 6);
		logConfigure((int) log_level, log_file_path, use_stdout);
	});
	RGL_TAPE_RECORD(T::num(log_level), T::text(log_file_path), T::flag(use_stdout));
	return status;
}

RGL_API void rgl_get_last_error_string(const char** out_error_string)
{
	if (out_error_string == nullptr) {
		return;
	}
	*out_error_string = lastErrorString();
}

RGL_API rgl_status_t rgl_cleanup(void)
{
	const rgl_status_t status = safeCall([&]() {
		Batches::map().clear();
		Servers::map().clear();
		while (!Nodes::map().empty()) {
			auto node = Nodes::map().begin()->second;
			releaseGraph(node);
		}
		for (auto& c : std::vector<std::shared_ptr<GraphRunCtx>>(GraphRunCtx::instances())) {
			c->detachAndDestroy();
		}
		Scene::defaultScene().clear();
		for (auto& kv : Scenes::map()) {
			kv.second->clear();
			kv.second->releaseDevice();
		}
		Scenes::map().clear();
		Entities::map().clear();
		Meshes::map().clear();
		Textures::map().clear();
	});
	RGL_TAPE_RECORD();
	return status;
}

// ================================================================ mesh

RGL_API rgl_status_t rgl_mesh_create(rgl_mesh_t* out_mesh, const rgl_vec3f* vertices, int32_t vertex_count,
                                     const rgl_vec3i* indices, int32_t index_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_mesh != nullptr);
		CHECK_ARG(vertices != nullptr);
		CHECK_ARG(vertex_count > 0);
		CHECK_ARG(indices != nullptr);
		CHECK_ARG(index_count > 0);
		GraphRunCtx::synchronizeAll();
		*out_mesh = Meshes::add(std::make_shared<Mesh>(vertices, vertex_count, indices, index_count));
	});
	RGL_TAPE_RECORD(T::handle(out_mesh ? *out_mesh : nullptr), T::arr(vertices, vertex_count), T::num(vertex_count), T::arr(indices, index_count), T::num(index_count));
	return status;
}

RGL_API rgl_status_t rgl_mesh_set_texture_coords(rgl_mesh_t mesh, const rgl_vec2f* uvs, int32_t uv_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(mesh != nullptr);
		CHECK_ARG(uvs != nullptr);
		CHECK_ARG(uv_count > 0);
		GraphRunCtx::synchronizeAll();
		Meshes::get(mesh, "Mesh")->setTexCoords(uvs, uv_count);
	});
	RGL_TAPE_RECORD(T::handle(mesh), T::arr(uvs, uv_count), T::num(uv_count));
	return status;
}

RGL_API rgl_status_t rgl_mesh_set_bone_weights(rgl_mesh_t mesh, const rgl_bone_weights_t* bone_weights, int32_t bone_weights_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(mesh != nullptr);
		CHECK_ARG(bone_weights != nullptr);
		CHECK_ARG(bone_weights_count > 0);
		GraphRunCtx::synchronizeAll();
		Meshes::get(mesh, "Mesh")->setBoneWeights(bone_weights, bone_weights_count);
	});
	RGL_TAPE_RECORD(T::handle(mesh), T::arr(bone_weights, bone_weights_count), T::num(bone_weights_count));
	return status;
}

RGL_API rgl_status_t rgl_mesh_set_restposes(rgl_mesh_t mesh, const rgl_mat3x4f* restposes, int32_t bones_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(mesh != nullptr);
		CHECK_ARG(restposes != nullptr);
		CHECK_ARG(bones_count > 0);
		GraphRunCtx::synchronizeAll();
		Meshes::get(mesh, "Mesh")->setRestposes(restposes, bones_count);
	});
	RGL_TAPE_RECORD(T::handle(mesh), T::arr(restposes, bones_count), T::num(bones_count));
	return status;
}

RGL_API rgl_status_t rgl_mesh_destroy(rgl_mesh_t mesh)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(mesh != nullptr);
		GraphRunCtx::synchronizeAll();
		Meshes::release(mesh, "Mesh");
	});
	RGL_TAPE_RECORD(T::handle(mesh));
	return status;
}

RGL_API rgl_status_t rgl_mesh_is_alive(rgl_mesh_t mesh, bool* out_alive)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_alive != nullptr);
		*out_alive = Meshes::contains(mesh);
	});
	RGL_TAPE_RECORD(T::handle(mesh), T::flag(out_alive && *out_alive));
	return status;
}

// ================================================================ entity

RGL_API rgl_status_t rgl_entity_create(rgl_entity_t* out_entity, rgl_scene_t scene, rgl_mesh_t mesh)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_entity != nullptr);
		CHECK_ARG(mesh != nullptr);
		GraphRunCtx::synchronizeAll();
		auto m = Meshes::get(mesh, "Mesh");
		auto sc = sceneOf(scene);
		auto e = std::make_shared<Entity>(m, sc.get());
		sc->addEntity(e);
		*out_entity = Entities::add(e);
	});
	RGL_TAPE_RECORD(T::handle(out_entity ? *out_entity : nullptr), T::handle(scene), T::handle(mesh));
	return status;
}

RGL_API rgl_status_t rgl_entity_destroy(rgl_entity_t entity)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(entity != nullptr);
		GraphRunCtx::synchronizeAll();
		auto e = Entities::get(entity, "Entity");
		e->scene->removeEntity(e.get());
		Entities::release(entity, "Entity");
	});
	RGL_TAPE_RECORD(T::handle(entity));
	return status;
}

RGL_API rgl_status_t rgl_entity_set_transform(rgl_entity_t entity, const rgl_mat3x4f* transform)
{
	const rgl_status_t status = safeCallKeepingValidation([&]() {
		CHECK_ARG(entity != nullptr);
		CHECK_ARG(transform != nullptr);
		GraphRunCtx::synchronizeAll();
		Entities::get(entity, "Entity")->setTransform(toMat(*transform));
	});
	RGL_TAPE_RECORD(T::handle(entity), T::arr(transform, 1));
	return status;
}

RGL_API rgl_status_t rgl_entity_set_pose_world(rgl_entity_t entity, const rgl_mat3x4f* pose, int32_t bones_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(entity != nullptr);
		CHECK_ARG(pose != nullptr);
		CHECK_ARG(bones_count > 0);
		// The entity's BLAS is rebuilt in place: nothing may still be reading it.
		GraphRunCtx::synchronizeAll();
		RGL_CHECK_CUDA(cudaDeviceSynchronize());
		Entities::get(entity, "Entity")->setPoseAndAnimate(pose, bones_count);
	});
	RGL_TAPE_RECORD(T::handle(entity), T::arr(pose, bones_count), T::num(bones_count));
	return status;
}

RGL_API rgl_status_t rgl_entity_set_id(rgl_entity_t entity, int32_t id)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(entity != nullptr);
		CHECK_ARG(id != RGL_ENTITY_INVALID_ID);
		GraphRunCtx::synchronizeAll();
		Entities::get(entity, "Entity")->setId(id);
	});
	RGL_TAPE_RECORD(T::handle(entity), T::num(id));
	return status;
}

RGL_API rgl_status_t rgl_entity_set_intensity_texture(rgl_entity_t entity, rgl_texture_t texture)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(entity != nullptr);
		CHECK_ARG(texture != nullptr);
		GraphRunCtx::synchronizeAll();
		Entities::get(entity, "Entity")->setIntensityTexture(Textures::get(texture, "Texture"));
	});
	RGL_TAPE_RECORD(T::handle(entity), T::handle(texture));
	return status;
}

RGL_API rgl_status_t rgl_entity_set_laser_retro(rgl_entity_t entity, float retro)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(entity != nullptr);
		GraphRunCtx::synchronizeAll();
		Entities::get(entity, "Entity")->setLaserRetro(retro);
	});
	RGL_TAPE_RECORD(T::handle(entity), T::real(retro));
	return status;
}

RGL_API rgl_status_t rgl_entity_apply_external_animation(rgl_entity_t entity, const rgl_vec3f* vertices, int32_t vertex_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(entity != nullptr);
		CHECK_ARG(vertices != nullptr);
		CHECK_ARG(vertex_count > 0);
		GraphRunCtx::synchronizeAll();
		RGL_CHECK_CUDA(cudaDeviceSynchronize());
		Entities::get(entity, "Entity")->applyExternalAnimation(vertices, vertex_count);
	});
	RGL_TAPE_RECORD(T::handle(entity), T::arr(vertices, vertex_count), T::num(vertex_count));
	return status;
}

RGL_API rgl_status_t rgl_entity_is_alive(rgl_entity_t entity, bool* out_alive)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_alive != nullptr);
		*out_alive = Entities::contains(entity);
	});
	RGL_TAPE_RECORD(T::handle(entity), T::flag(out_alive && *out_alive));
	return status;
}

// ================================================================ texture

RGL_API rgl_status_t rgl_texture_create(rgl_texture_t* out_texture, const void* texels, int32_t width, int32_t height)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_texture != nullptr);
		CHECK_ARG(texels != nullptr);
		CHECK_ARG(width > 0);
		CHECK_ARG(height > 0);
		*out_texture = Textures::add(std::make_shared<Texture>(texels, width, height));
	});
	RGL_TAPE_RECORD(T::handle(out_texture ? *out_texture : nullptr), T::bin(texels, texels && width > 0 && height > 0 ? (size_t) width * height : 0),
	                T::num(width), T::num(height));
	return status;
}

RGL_API rgl_status_t rgl_texture_destroy(rgl_texture_t texture)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(texture != nullptr);
		GraphRunCtx::synchronizeAll();
		Textures::release(texture, "Texture");
	});
	RGL_TAPE_RECORD(T::handle(texture));
	return status;
}

RGL_API rgl_status_t rgl_texture_is_alive(rgl_texture_t texture, bool* out_alive)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_alive != nullptr);
		*out_alive = Textures::contains(texture);
	});
	RGL_TAPE_RECORD(T::handle(texture), T::flag(out_alive && *out_alive));
	return status;
}

// ================================================================ scene

RGL_API rgl_status_t rgl_scene_set_time(rgl_scene_t scene, uint64_t nanoseconds)
{
	const rgl_status_t status = safeCall([&]() {
		GraphRunCtx::synchronizeAll();
		sceneOf(scene)->setTime(nanoseconds);
	});
	RGL_TAPE_RECORD(T::handle(scene), T::unum(nanoseconds));
	return status;
}

// ================================================================ graph

RGL_API rgl_status_t rgl_graph_run(rgl_node_t raw_node)
{
	const rgl_status_t status = safeCallKeepingValidation([&]() {
		CHECK_ARG(raw_node != nullptr);
		auto node = getNode(raw_node);
		if (!node->ctx) {
			GraphRunCtx::createAndAttach(node);
		}
		node->ctx->run();
	});
	RGL_TAPE_RECORD(T::handle(raw_node));
	return status;
}

RGL_API rgl_status_t rgl_graph_destroy(rgl_node_t raw_node)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(raw_node != nullptr);
		releaseGraph(getNode(raw_node));
	});
	RGL_TAPE_RECORD(T::handle(raw_node));
	return status;
}

RGL_API rgl_status_t rgl_graph_get_result_size(rgl_node_t node, rgl_field_t field, int32_t* out_count, int32_t* out_size_of)
{
	const rgl_status_t status = safeCallKeepingValidation([&]() {
		CHECK_ARG(node != nullptr);
		auto pn = getNodeAs<PointsNode>(node, "IPointsNode");
		if (pn->dirty || !pn->ctx) {
			throw InvalidPipeline(format("Cannot get results from %s; it hasn't been run yet, or the run has failed", pn->name()));
		}
		pn->ctx->synchronize();
		int32_t count = (int32_t) pn->pointCountHost();
		int32_t size = (int32_t) pn->fieldPointSize(field);
		if (out_count != nullptr) {
			*out_count = count;
		}
		if (out_size_of != nullptr) {
			*out_size_of = size;
		}
	});
	RGL_TAPE_RECORD(T::handle(node), T::num(field), T::num(out_count ? *out_count : 0), T::num(out_size_of ? *out_size_of : 0));
	return status;
}

RGL_API rgl_status_t rgl_graph_get_result_data(rgl_node_t node, rgl_field_t field, void* dst)
{
	const rgl_status_t status = safeCallKeepingValidation([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(dst != nullptr);
		auto pn = getNodeAs<PointsNode>(node, "IPointsNode");
		if (!pn->hasField(field)) {
			throw InvalidPipeline(format("node %s does not provide field %s", pn->name(), fieldName(field)));
		}
		if (pn->dirty || !pn->ctx) {
			throw InvalidPipeline(format("Cannot get results from %s; it hasn't been run yet, or the run has failed", pn->name()));
		}
		pn->ctx->synchronize();
		size_t count = pn->pointCountHost();
		size_t bytes = count * pn->fieldPointSize(field);
		if (bytes == 0) {
			return;
		}
		const void* src = pn->fieldDev(field);
		RGL_CHECK_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
	});
	RGL_TAPE_RECORD(T::handle(node), T::num(field), T::handle(dst));
	return status;
}

RGL_API rgl_status_t rgl_graph_node_add_child(rgl_node_t parent, rgl_node_t child)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(parent != nullptr);
		CHECK_ARG(child != nullptr);
		CHECK_ARG(parent != child);
		getNode(parent)->addChild(getNode(child));
	});
	RGL_TAPE_RECORD(T::handle(parent), T::handle(child));
	return status;
}

RGL_API rgl_status_t rgl_graph_node_remove_child(rgl_node_t parent, rgl_node_t child)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(parent != nullptr);
		CHECK_ARG(child != nullptr);
		getNode(parent)->removeChild(getNode(child));
	});
	RGL_TAPE_RECORD(T::handle(parent), T::handle(child));
	return status;
}

RGL_API rgl_status_t rgl_graph_node_set_priority(rgl_node_t node, int32_t priority)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		auto n = getNode(node);
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setPriority(priority);
	});
	RGL_TAPE_RECORD(T::handle(node), T::num(priority));
	return status;
}

RGL_API rgl_status_t rgl_graph_node_get_priority(rgl_node_t node, int32_t* out_priority)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(out_priority != nullptr);
		*out_priority = getNode(node)->priority;
	});
	RGL_TAPE_RECORD(T::handle(node), T::num(out_priority ? *out_priority : 0));
	return status;
}

// ================================================================ ray nodes

RGL_API rgl_status_t rgl_node_rays_from_mat3x4f(rgl_node_t* node, const rgl_mat3x4f* rays, int32_t ray_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(rays != nullptr);
		CHECK_ARG(ray_count > 0);
		createOrUpdateNode<FromMat3x4fRaysNode>(node, "FromMat3x4fRaysNode",
		                                        [&](FromMat3x4fRaysNode& n) { n.setParameters(rays, (size_t) ray_count); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(rays, ray_count), T::num(ray_count));
	return status;
}

RGL_API rgl_status_t rgl_node_rays_set_ring_ids(rgl_node_t* node, const int32_t* ring_ids, int32_t ring_ids_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(ring_ids != nullptr);
		CHECK_ARG(ring_ids_count > 0);
		createOrUpdateNode<SetRingIdsRaysNode>(node, "SetRingIdsRaysNode",
		                                       [&](SetRingIdsRaysNode& n) { n.setParameters(ring_ids, (size_t) ring_ids_count); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(ring_ids, ring_ids_count), T::num(ring_ids_count));
	return status;
}

RGL_API rgl_status_t rgl_node_rays_set_range(rgl_node_t* node, const rgl_vec2f* ranges, int32_t ranges_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(ranges != nullptr);
		CHECK_ARG(ranges_count > 0);
		createOrUpdateNode<SetRangeRaysNode>(node, "SetRangeRaysNode",
		                                     [&](SetRangeRaysNode& n) { n.setParameters(ranges, (size_t) ranges_count); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(ranges, ranges_count), T::num(ranges_count));
	return status;
}

RGL_API rgl_status_t rgl_node_rays_set_time_offsets(rgl_node_t* node, const float* offsets, int32_t offsets_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(offsets != nullptr);
		CHECK_ARG(offsets_count > 0);
		createOrUpdateNode<SetTimeOffsetsRaysNode>(node, "SetTimeOffsetsRaysNode",
		                                           [&](SetTimeOffsetsRaysNode& n) { n.setParameters(offsets, (size_t) offsets_count); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(offsets, offsets_count), T::num(offsets_count));
	return status;
}

RGL_API rgl_status_t rgl_node_rays_transform(rgl_node_t* node, const rgl_mat3x4f* transform)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(transform != nullptr);
		Mat34 tf = toMat(*transform);
		createOrUpdateNode<TransformRaysNode>(node, "TransformRaysNode", [&](TransformRaysNode& n) { n.setParameters(tf); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(transform, 1));
	return status;
}

// ================================================================ point nodes

RGL_API rgl_status_t rgl_node_points_transform(rgl_node_t* node, const rgl_mat3x4f* transform)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(transform != nullptr);
		Mat34 tf = toMat(*transform);
		createOrUpdateNode<TransformPointsNode>(node, "TransformPointsNode", [&](TransformPointsNode& n) { n.setParameters(tf); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(transform, 1));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace(rgl_node_t* node, rgl_scene_t scene)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		auto sc = sceneOf(scene);
		createOrUpdateNode<RaytraceNode>(node, "RaytraceNode", [&](RaytraceNode& n) {
			n.sceneRef = sc;
			n.scene = sc.get();
		});
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::handle(scene));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace_configure_velocity(rgl_node_t node, const rgl_vec3f* linear_velocity,
                                                          const rgl_vec3f* angular_velocity)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(linear_velocity != nullptr);
		CHECK_ARG(angular_velocity != nullptr);
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setVelocity(rgl::v3(linear_velocity->value[0], linear_velocity->value[1], linear_velocity->value[2]),
		               rgl::v3(angular_velocity->value[0], angular_velocity->value[1], angular_velocity->value[2]));
	});
	RGL_TAPE_RECORD(T::handle(node), T::arr(linear_velocity, 1), T::arr(angular_velocity, 1));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace_configure_distortion(rgl_node_t node, bool enable)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setDistortion(enable);
	});
	RGL_TAPE_RECORD(T::handle(node), T::flag(enable));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace_configure_non_hits(rgl_node_t node, float nearDistance, float farDistance)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setNonHits(nearDistance, farDistance);
		n->markParamsChanged();
	});
	RGL_TAPE_RECORD(T::handle(node), T::real(nearDistance), T::real(farDistance));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace_configure_mask(rgl_node_t node, const int8_t* rays_mask, int32_t rays_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(rays_mask != nullptr);
		CHECK_ARG(rays_count > 0);
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setRayMask(rays_mask, (size_t) rays_count); // staged with the job at every run
	});
	RGL_TAPE_RECORD(T::handle(node), T::arr(rays_mask, rays_count), T::num(rays_count));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace_configure_beam_divergence(rgl_node_t node, float horizontal_beam_divergence,
                                                                 float vertical_beam_divergence)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG((horizontal_beam_divergence > 0.0f && vertical_beam_divergence > 0.0f) ||
		          (horizontal_beam_divergence == 0.0f && vertical_beam_divergence == 0.0f));
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setBeamDivergence(horizontal_beam_divergence, vertical_beam_divergence);
		n->markParamsChanged();
	});
	RGL_TAPE_RECORD(T::handle(node), T::real(horizontal_beam_divergence), T::real(vertical_beam_divergence));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace_configure_default_intensity(rgl_node_t node, float default_intensity)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(default_intensity >= 0.0f);
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setDefaultIntensity(default_intensity);
		n->markParamsChanged();
	});
	RGL_TAPE_RECORD(T::handle(node), T::real(default_intensity));
	return status;
}

RGL_API rgl_status_t rgl_node_raytrace_configure_return_mode(rgl_node_t node, rgl_return_mode_t return_mode)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(return_mode != RGL_RETURN_UNKNOWN);
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setReturnMode((int32_t) return_mode);
		n->dirty = true;
		n->markParamsChanged();
	});
	RGL_TAPE_RECORD(T::handle(node), T::num(return_mode));
	return status;
}

RGL_API rgl_status_t rgl_node_points_format(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(fields != nullptr);
		CHECK_ARG(field_count > 0);
		std::vector<rgl_field_t> f(fields, fields + field_count);
		createOrUpdateNode<FormatPointsNode>(node, "FormatPointsNode", [&](FormatPointsNode& n) { n.setParameters(f); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(fields, field_count), T::num(field_count));
	return status;
}

RGL_API rgl_status_t rgl_node_points_yield(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(fields != nullptr);
		CHECK_ARG(field_count > 0);
		std::vector<rgl_field_t> f(fields, fields + field_count);
		createOrUpdateNode<YieldPointsNode>(node, "YieldPointsNode", [&](YieldPointsNode& n) { n.setParameters(f); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(fields, field_count), T::num(field_count));
	return status;
}

RGL_API rgl_status_t rgl_node_points_compact_by_field(rgl_node_t* node, rgl_field_t field)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(field == RGL_FIELD_IS_HIT_I32 || field == RGL_FIELD_IS_GROUND_I32);
		createOrUpdateNode<CompactByFieldPointsNode>(node, "CompactByFieldPointsNode",
		                                             [&](CompactByFieldPointsNode& n) { n.setParameters(field); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::num(field));
	return status;
}

RGL_API rgl_status_t rgl_node_points_spatial_merge(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(fields != nullptr);
		CHECK_ARG(field_count > 0);
		std::vector<rgl_field_t> f(fields, fields + field_count);
		createOrUpdateNode<SpatialMergePointsNode>(node, "SpatialMergePointsNode", [&](SpatialMergePointsNode& n) { n.setParameters(f); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(fields, field_count), T::num(field_count));
	return status;
}

RGL_API rgl_status_t rgl_node_points_temporal_merge(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(fields != nullptr);
		CHECK_ARG(field_count > 0);
		std::vector<rgl_field_t> f(fields, fields + field_count);
		createOrUpdateNode<TemporalMergePointsNode>(node, "TemporalMergePointsNode", [&](TemporalMergePointsNode& n) { n.setParameters(f); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(fields, field_count), T::num(field_count));
	return status;
}

RGL_API rgl_status_t rgl_node_points_from_array(rgl_node_t* node, const void* points, int32_t points_count, const rgl_field_t* fields,
                                                int32_t field_count)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(points != nullptr);
		CHECK_ARG(points_count > 0);
		CHECK_ARG(fields != nullptr);
		CHECK_ARG(field_count > 0);
		std::vector<rgl_field_t> f(fields, fields + field_count);
		createOrUpdateNode<FromArrayPointsNode>(node, "FromArrayPointsNode",
		                                        [&](FromArrayPointsNode& n) { n.setParameters(points, (size_t) points_count, f); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::bin(points, tapePointBytes(points, points_count, fields, field_count)), T::num(points_count), T::arr(fields, field_count), T::num(field_count));
	return status;
}

RGL_API rgl_status_t rgl_node_points_radar_postprocess(rgl_node_t* node, const rgl_radar_scope_t* radar_scopes,
                                                       int32_t radar_scopes_count, float ray_azimuth_step, float ray_elevation_step,
                                                       float frequency, float power_transmitted, float cumulative_device_gain,
                                                       float received_noise_mean, float received_noise_st_dev)
{
	return safeCall([&]() {
		CHECK_ARG(radar_scopes != nullptr);
		CHECK_ARG(radar_scopes_count > 0);
		notImplemented("rgl_node_points_radar_postprocess");
	});
}

RGL_API rgl_status_t rgl_node_points_radar_track_objects(rgl_node_t* node, float object_distance_threshold,
                                                         float object_azimuth_threshold, float object_elevation_threshold,
                                                         float object_radial_speed_threshold, float max_matching_distance,
                                                         float max_prediction_time_frame, float movement_sensitivity)
{
	return safeCall([&]() {
		CHECK_ARG(node != nullptr);
		notImplemented("rgl_node_points_radar_track_objects");
	});
}

RGL_API rgl_status_t rgl_node_points_radar_set_classes(rgl_node_t node, const int32_t* entity_ids,
                                                       const rgl_radar_object_class_t* object_classes, int32_t count)
{
	return safeCall([&]() {
		CHECK_ARG(node != nullptr);
		notImplemented("rgl_node_points_radar_set_classes");
	});
}

RGL_API rgl_status_t rgl_node_points_filter_ground(rgl_node_t* node, const rgl_vec3f* sensor_up_vector, float ground_angle_threshold)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(ground_angle_threshold >= 0);
		CHECK_ARG(sensor_up_vector != nullptr);
		const rgl::Vec3 up = rgl::v3(sensor_up_vector->value[0], sensor_up_vector->value[1], sensor_up_vector->value[2]);
		createOrUpdateNode<FilterGroundPointsNode>(node, "FilterGroundPointsNode",
		                                           [&](FilterGroundPointsNode& n) { n.setParameters(up, ground_angle_threshold); });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::arr(sensor_up_vector, 1), T::real(ground_angle_threshold));
	return status;
}

RGL_API rgl_status_t rgl_node_gaussian_noise_angular_ray(rgl_node_t* node, float mean, float st_dev, rgl_axis_t rotation_axis)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(st_dev >= 0);
		CHECK_ARG((rotation_axis == RGL_AXIS_X) || (rotation_axis == RGL_AXIS_Y) || (rotation_axis == RGL_AXIS_Z));
		bool created = *node == nullptr;
		createOrUpdateNode<GaussianNoiseAngularRaysNode>(node, "GaussianNoiseAngularRaysNode", [&](GaussianNoiseAngularRaysNode& n) {
			n.setParameters(mean, st_dev, rotation_axis);
			if (created) {
				n.setSeed(randomSeed(), 0);
			}
		});
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::real(mean), T::real(st_dev), T::num(rotation_axis));
	return status;
}

RGL_API rgl_status_t rgl_node_gaussian_noise_angular_hitpoint(rgl_node_t* node, float mean, float st_dev, rgl_axis_t rotation_axis)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(st_dev >= 0);
		CHECK_ARG((rotation_axis == RGL_AXIS_X) || (rotation_axis == RGL_AXIS_Y) || (rotation_axis == RGL_AXIS_Z));
		bool created = *node == nullptr;
		createOrUpdateNode<GaussianNoiseAngularHitpointNode>(node, "GaussianNoiseAngularHitpointNode",
		                                                     [&](GaussianNoiseAngularHitpointNode& n) {
			                                                     n.setParameters(mean, st_dev, rotation_axis);
			                                                     if (created) {
				                                                     n.setSeed(randomSeed(), 0);
			                                                     }
		                                                     });
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::real(mean), T::real(st_dev), T::num(rotation_axis));
	return status;
}

RGL_API rgl_status_t rgl_node_gaussian_noise_distance(rgl_node_t* node, float mean, float st_dev_base, float st_dev_rise_per_meter)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(st_dev_base >= 0);
		CHECK_ARG(st_dev_rise_per_meter >= 0);
		bool created = *node == nullptr;
		createOrUpdateNode<GaussianNoiseDistanceNode>(node, "GaussianNoiseDistanceNode", [&](GaussianNoiseDistanceNode& n) {
			n.setParameters(mean, st_dev_base, st_dev_rise_per_meter);
			if (created) {
				n.setSeed(randomSeed(), 0);
			}
		});
	});
	RGL_TAPE_RECORD(T::handle(node ? *node : nullptr), T::real(mean), T::real(st_dev_base), T::real(st_dev_rise_per_meter));
	return status;
}

RGL_API rgl_status_t rgl_node_is_alive(rgl_node_t node, bool* out_alive)
{
	const rgl_status_t status = safeCall([&]() {
		CHECK_ARG(out_alive != nullptr);
		*out_alive = Nodes::contains(node);
	});
	RGL_TAPE_RECORD(T::handle(node), T::flag(out_alive && *out_alive));
	return status;
}

// ================================================================ tape extension (not part of this build)

RGL_API rgl_status_t rgl_tape_record_begin(const char* path)
{
	return safeCall([&]() {
		CHECK_ARG(path != nullptr);
		CHECK_ARG(path[0] != '\0');
		T::beginRecording(path);
	});
}

RGL_API rgl_status_t rgl_tape_record_end()
{
	return safeCall([&]() { T::endRecording(); });
}

RGL_API rgl_status_t rgl_tape_record_is_active(bool* is_active)
{
	return safeCall([&]() {
		CHECK_ARG(is_active != nullptr);
		*is_active = T::recording();
	});
}

RGL_API rgl_status_t rgl_tape_play(const char* path)
{
	return safeCall([&]() {
		CHECK_ARG(path != nullptr);
		CHECK_ARG(path[0] != '\0');
		T::play(path);
	});
}

// ================================================================ GB300 extensions

RGL_API rgl_status_t rgl_gb300_node_gaussian_noise_set_seed(rgl_node_t node, uint64_t seed, uint64_t frame)
{
	return safeCall([&]() {
		CHECK_ARG(node != nullptr);
		auto n = getNode(node);
		if (n->ctx) {
			n->ctx->synchronize();
		}
		// Seed and frame are staged before every run: no recapture needed.
		if (auto a = std::dynamic_pointer_cast<GaussianNoiseAngularRaysNode>(n)) {
			a->setSeed(seed, frame);
		} else if (auto b = std::dynamic_pointer_cast<GaussianNoiseAngularHitpointNode>(n)) {
			b->setSeed(seed, frame);
		} else if (auto c = std::dynamic_pointer_cast<GaussianNoiseDistanceNode>(n)) {
			c->setSeed(seed, frame);
		} else {
			throw InvalidAPIObject(format("RGL API Error: Node type mismatch: expected a Gaussian noise node, got %s", n->name()));
		}
	});
}

RGL_API rgl_status_t rgl_gb300_node_raytrace_configure_beam_samples(rgl_node_t node, int32_t layers, int32_t vertices)
{
	return safeCall([&]() {
		CHECK_ARG(node != nullptr);
		CHECK_ARG(layers > 0);
		CHECK_ARG(vertices > 0);
		CHECK_ARG(1 + layers * vertices <= kMaxBeamSamples);
		auto n = getNodeAs<RaytraceNode>(node, "RaytraceNode");
		if (n->ctx) {
			n->ctx->synchronize();
		}
		n->setBeamSamples(layers, vertices);
		n->markParamsChanged();
	});
}

RGL_API rgl_status_t rgl_gb300_configure_timing(bool enable)
{
	return safeCall([&]() {
		GraphRunCtx::synchronizeAll();
		setTimingEnabled(enable);
	});
}

RGL_API rgl_status_t rgl_gb300_graph_get_timing(rgl_node_t node, float* out_run_ms, float* out_trace_ms)
{
	return safeCallKeepingValidation([&]() {
		CHECK_ARG(node != nullptr);
		auto n = getNode(node);
		if (!n->ctx) {
			throw InvalidPipeline(format("%s has not been run", n->name()));
		}
		n->ctx->synchronize();
		if (out_run_ms) {
			*out_run_ms = n->ctx->lastRunMs;
		}
		if (out_trace_ms) {
			*out_trace_ms = n->ctx->lastTraceMs;
		}
	});
}

RGL_API rgl_status_t rgl_gb300_graph_sync(rgl_node_t node)
{
	return safeCallKeepingValidation([&]() {
		CHECK_ARG(node != nullptr);
		auto n = getNode(node);
		if (n->ctx) {
			n->ctx->synchronize();
		}
	});
}

RGL_API rgl_status_t rgl_gb300_get_kernel_launch_count(uint64_t* out_count)
{
	return safeCallKeepingValidation([&]() {
		CHECK_ARG(out_count != nullptr);
		*out_count = launchCount();
	});
}

RGL_API rgl_status_t rgl_gb300_device_info(int32_t* out_sm_count, int32_t* out_cc)
{
	return safeCall([&]() {
		int dev = 0;
		RGL_CHECK_CUDA(cudaGetDevice(&dev));
		cudaDeviceProp p{};
		RGL_CHECK_CUDA(cudaGetDeviceProperties(&p, dev));
		if (out_sm_count) {
			*out_sm_count = p.multiProcessorCount;
		}
		if (out_cc) {
			*out_cc = p.major * 10 + p.minor;
		}
	});
}

RGL_API rgl_status_t rgl_gb300_scene_get_stats(int64_t* out_node_bytes, int64_t* out_triangle_bytes, int32_t* out_instances)
{
	return safeCall([&]() {
		GraphRunCtx::synchronizeAll();
		int64_t nb = 0, tb = 0;
		Scene::defaultScene().stats(nb, tb);
		if (out_node_bytes) {
			*out_node_bytes = nb;
		}
		if (out_triangle_bytes) {
			*out_triangle_bytes = tb;
		}
		if (out_instances) {
			*out_instances = (int32_t) Scene::defaultScene().entityCount();
		}
	});
}

RGL_API rgl_status_t rgl_gb300_configure_blas_builder(int32_t builder)
{
	return safeCall([&]() {
		CHECK_ARG(builder == RGL_GB300_BLAS_DEVICE_SAH || builder == RGL_GB300_BLAS_HOST_SAH || builder == RGL_GB300_BLAS_DEVICE_LBVH);
		setBlasBuilder(builder);
	});
}

RGL_API rgl_status_t rgl_gb300_get_blas_build_stats(int64_t* out_builds, double* out_total_ms)
{
	return safeCall([&]() {
		int64_t builds = 0;
		double ms = 0.0;
		blasBuildStats(builds, ms);
		if (out_builds) {
			*out_builds = builds;
		}
		if (out_total_ms) {
			*out_total_ms = ms;
		}
	});
}

// Allocation-free compaction (include/rgl/api/extensions/gb300.h). Status handling as safeCall() but
// without its first-call CUDA initialisation, which calls cudaFree(nullptr): this entry point uses the
// caller's current device and context as they are.
RGL_API rgl_status_t rgl_gb300_compact_by_flags_noalloc(const int32_t* flags, const void* src, int32_t count,
                                                        int32_t element_size, void* dst, int32_t* out_count, void* stream)
{
	if (!recoverable(lastStatus)) {
		return updateState(RGL_INVALID_STATE);
	}
	try {
		CHECK_ARG(out_count != nullptr);
		*out_count = compactNoAlloc(flags, src, count, element_size, dst, static_cast<cudaStream_t>(stream));
	}
	catch (InvalidAPIObject& e) {
		return updateState(RGL_INVALID_API_OBJECT, std::string(e.what()));
	}
	catch (std::invalid_argument& e) {
		return updateState(RGL_INVALID_ARGUMENT, std::string(e.what()));
	}
	catch (std::exception& e) {
		return updateState(RGL_INTERNAL_EXCEPTION, std::string(e.what()));
	}
	catch (...) {
		return updateState(RGL_INTERNAL_EXCEPTION, std::string("exceptional exception"));
	}
	return updateState(RGL_SUCCESS);
}

RGL_API rgl_status_t rgl_gb300_configure_cuda_graphs(bool enable)
{
	return safeCall([&]() {
		GraphRunCtx::synchronizeAll();
		setCudaGraphsEnabled(enable);
	});
}

RGL_API rgl_status_t rgl_gb300_graph_get_capture_stats(rgl_node_t node, int64_t* out_captures, int64_t* out_replays)
{
	return safeCall([&]() {
		CHECK_ARG(node != nullptr);
		auto n = getNode(node);
		if (out_captures) {
			*out_captures = n->ctx ? (int64_t) n->ctx->captures : 0;
		}
		if (out_replays) {
			*out_replays = n->ctx ? (int64_t) n->ctx->replays : 0;
		}
	});
}

// ---------------------------------------------------------------- batched multi-sensor frames

RGL_API rgl_status_t rgl_gb300_batch_create(rgl_gb300_batch_t* out_batch, const rgl_node_t* nodes, int32_t node_count)
{
	return safeCall([&]() {
		CHECK_ARG(out_batch != nullptr);
		CHECK_ARG(nodes != nullptr);
		CHECK_ARG(node_count > 0);
		CHECK_ARG(node_count <= rgl::kMaxBatchJobs);
		std::vector<Node::Ptr> anchors;
		for (int32_t i = 0; i < node_count; ++i) {
			CHECK_ARG(nodes[i] != nullptr);
			anchors.push_back(getNode(nodes[i]));
		}
		*out_batch = Batches::add(std::make_shared<BatchRun>(std::move(anchors)));
	});
}

RGL_API rgl_status_t rgl_gb300_batch_run(rgl_gb300_batch_t batch)
{
	return safeCallKeepingValidation([&]() {
		CHECK_ARG(batch != nullptr);
		Batches::get(batch, "Batch")->run();
	});
}

RGL_API rgl_status_t rgl_gb300_batch_destroy(rgl_gb300_batch_t batch)
{
	return safeCall([&]() {
		CHECK_ARG(batch != nullptr);
		Batches::get(batch, "Batch")->synchronize();
		Batches::release(batch, "Batch");
	});
}

RGL_API rgl_status_t rgl_gb300_batch_configure_schedule(rgl_gb300_batch_t batch, bool autotune, int32_t block, int32_t packing,
                                                        int32_t order, int32_t chunk, int32_t regs)
{
	return safeCall([&]() {
		CHECK_ARG(batch != nullptr);
		CHECK_ARG(block == 64 || block == 128 || block == 256);
		CHECK_ARG(packing == rgl::kPackLaneGroup || packing == rgl::kPackSerial);
		CHECK_ARG(order >= rgl::kOrderNatural && order <= rgl::kOrderElevation);
		CHECK_ARG(chunk >= 1 && chunk <= 64);
		CHECK_ARG(regs == 64 || regs == 80 || regs == 96 || regs == 128);
		auto b = Batches::get(batch, "Batch");
		b->synchronize();
		b->autotune = autotune;
		if (!autotune) {
			b->schedule = rgl::BatchSchedule{block, packing, order, chunk, regs};
		}
	});
}

RGL_API rgl_status_t rgl_gb300_batch_get_schedule(rgl_gb300_batch_t batch, int32_t* out_block, int32_t* out_packing, int32_t* out_order,
                                                  int32_t* out_chunk, int32_t* out_regs)
{
	return safeCall([&]() {
		CHECK_ARG(batch != nullptr);
		auto b = Batches::get(batch, "Batch");
		const rgl::BatchSchedule s = b->schedule;
		if (out_block) *out_block = s.block;
		if (out_packing) *out_packing = s.packing;
		if (out_order) *out_order = s.order;
		if (out_chunk) *out_chunk = s.chunk;
		if (out_regs) *out_regs = s.regs;
	});
}

RGL_API rgl_status_t rgl_gb300_batch_configure_waves(rgl_gb300_batch_t batch, int32_t waves)
{
	return safeCall([&]() {
		CHECK_ARG(batch != nullptr);
		CHECK_ARG(waves >= 0 && waves <= rgl::kMaxBatchJobs);
		auto b = Batches::get(batch, "Batch");
		b->synchronize();
		b->wavesWanted = waves;
	});
}

RGL_API rgl_status_t rgl_gb300_batch_get_waves(rgl_gb300_batch_t batch, int32_t* out_waves)
{
	return safeCall([&]() {
		CHECK_ARG(batch != nullptr);
		CHECK_ARG(out_waves != nullptr);
		auto b = Batches::get(batch, "Batch");
		*out_waves = std::max(0, b->waveCount());
	});
}

RGL_API rgl_status_t rgl_gb300_batch_get_tuning(rgl_gb300_batch_t batch, int32_t capacity, int32_t* out_schedules, float* out_ms,
                                                int32_t* out_count)
{
	return safeCall([&]() {
		CHECK_ARG(batch != nullptr);
		CHECK_ARG(capacity >= 0);
		CHECK_ARG(capacity == 0 || (out_schedules != nullptr && out_ms != nullptr));
		auto b = Batches::get(batch, "Batch");
		b->synchronize();
		const auto& t = b->lastTuning;
		for (size_t i = 0; i < t.size() && (int32_t) i < capacity; ++i) {
			const rgl::BatchSchedule& s = t[i].s;
			int32_t* o = out_schedules + 5 * i;
			o[0] = s.block;
			o[1] = s.packing;
			o[2] = s.order;
			o[3] = s.chunk;
			o[4] = s.regs;
			out_ms[i] = t[i].ms;
		}
		if (out_count) {
			*out_count = (int32_t) t.size();
		}
	});
}

RGL_API rgl_status_t rgl_gb300_batch_get_stats(rgl_gb300_batch_t batch, float* out_frame_ms, float* out_trace_ms, int64_t* out_beams,
                                               int64_t* out_rays, int64_t* out_captures, int64_t* out_replays, int64_t* out_tunings)
{
	return safeCallKeepingValidation([&]() {
		CHECK_ARG(batch != nullptr);
		auto b = Batches::get(batch, "Batch");
		b->synchronize();
		if (out_frame_ms) *out_frame_ms = b->lastFrameMs;
		if (out_trace_ms) *out_trace_ms = b->lastTraceMs;
		if (out_beams) *out_beams = b->beams;
		if (out_rays) *out_rays = b->rays;
		if (out_captures) *out_captures = (int64_t) b->captures;
		if (out_replays) *out_replays = (int64_t) b->replays;
		if (out_tunings) *out_tunings = (int64_t) b->tunings;
	});
}

// ---------------------------------------------------------------- resident scenes

RGL_API rgl_status_t rgl_gb300_scene_create(rgl_scene_t* out_scene)
{
	return safeCall([&]() {
		CHECK_ARG(out_scene != nullptr);
		*out_scene = Scenes::add(std::make_shared<Scene>());
	});
}

RGL_API rgl_status_t rgl_gb300_scene_destroy(rgl_scene_t scene)
{
	return safeCall([&]() {
		CHECK_ARG(scene != nullptr);
		auto sc = Scenes::get(scene, "Scene");
		GraphRunCtx::synchronizeAll();
		for (auto it = Entities::map().begin(); it != Entities::map().end();) {
			it = (it->second->scene == sc.get()) ? Entities::map().erase(it) : std::next(it);
		}
		sc->clear();
		sc->releaseDevice();
		Scenes::release(scene, "Scene");
	});
}

RGL_API rgl_status_t rgl_gb300_scene_get_stats_of(rgl_scene_t scene, int64_t* out_node_bytes, int64_t* out_triangle_bytes,
                                                 int32_t* out_instances)
{
	return safeCall([&]() {
		auto sc = sceneOf(scene);
		int64_t nb = 0, tb = 0;
		sc->stats(nb, tb);
		if (out_node_bytes) *out_node_bytes = nb;
		if (out_triangle_bytes) *out_triangle_bytes = tb;
		if (out_instances) *out_instances = (int32_t) sc->entityCount();
	});
}

// ---------------------------------------------------------------- serving loop

RGL_API rgl_status_t rgl_gb300_server_create(rgl_gb300_server_t* out_server, int64_t hbm_budget_bytes, int32_t max_in_flight_batches)
{
	return safeCall([&]() {
		CHECK_ARG(out_server != nullptr);
		CHECK_ARG(hbm_budget_bytes > 0);
		CHECK_ARG(max_in_flight_batches >= 1 && max_in_flight_batches <= 8);
		*out_server = Servers::add(std::make_shared<Server>(hbm_budget_bytes, max_in_flight_batches));
	});
}

RGL_API rgl_status_t rgl_gb300_server_destroy(rgl_gb300_server_t server)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		Servers::release(server, "Server");
	});
}

RGL_API rgl_status_t rgl_gb300_server_add_pattern(rgl_gb300_server_t server, const rgl_mat3x4f* rays, int32_t ray_count,
                                                  int32_t* out_pattern)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		CHECK_ARG(rays != nullptr);
		CHECK_ARG(ray_count > 0);
		CHECK_ARG(out_pattern != nullptr);
		*out_pattern = Servers::get(server, "Server")->addPattern(rays, ray_count);
	});
}

RGL_API rgl_status_t rgl_gb300_server_submit(rgl_gb300_server_t server, rgl_scene_t scene, int32_t pattern,
                                             const rgl_mat3x4f* sensor_pose, rgl_return_mode_t return_mode, float min_range,
                                             float max_range, int64_t* out_request)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		CHECK_ARG(sensor_pose != nullptr);
		CHECK_ARG(out_request != nullptr);
		CHECK_ARG(return_mode != RGL_RETURN_UNKNOWN);
		CHECK_ARG(!std::isnan(min_range) && !std::isnan(max_range) && min_range >= 0.0f && min_range <= max_range);
		auto srv = Servers::get(server, "Server");
		*out_request = srv->submit(sceneOf(scene), pattern, toMat(*sensor_pose), (int32_t) return_mode, min_range, max_range);
	});
}

RGL_API rgl_status_t rgl_gb300_server_wait(rgl_gb300_server_t server, int64_t request, float timeout_ms, bool* out_done)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		const bool done = Servers::get(server, "Server")->wait(request, timeout_ms);
		if (out_done) {
			*out_done = done;
		}
	});
}

RGL_API rgl_status_t rgl_gb300_server_take_completed(rgl_gb300_server_t server, int64_t* out_requests, int32_t capacity,
                                                     int32_t* out_count)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		CHECK_ARG(out_requests != nullptr);
		CHECK_ARG(capacity > 0);
		CHECK_ARG(out_count != nullptr);
		*out_count = Servers::get(server, "Server")->takeCompleted(out_requests, capacity);
	});
}

RGL_API rgl_status_t rgl_gb300_server_wait_completed(rgl_gb300_server_t server, float timeout_ms, int64_t* out_requests, int32_t capacity,
                                                     int32_t* out_count)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		CHECK_ARG(out_requests != nullptr);
		CHECK_ARG(capacity > 0);
		CHECK_ARG(out_count != nullptr);
		*out_count = Servers::get(server, "Server")->waitCompleted(out_requests, capacity, timeout_ms);
	});
}

RGL_API rgl_status_t rgl_gb300_server_get_result_size(rgl_gb300_server_t server, int64_t request, rgl_field_t field,
                                                      int32_t* out_count, int32_t* out_size_of)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		int32_t c = 0, sz = 0;
		Servers::get(server, "Server")->resultSize(request, field, c, sz);
		if (out_count) *out_count = c;
		if (out_size_of) *out_size_of = sz;
	});
}

RGL_API rgl_status_t rgl_gb300_server_get_result_data(rgl_gb300_server_t server, int64_t request, rgl_field_t field, void* out_data)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		CHECK_ARG(out_data != nullptr);
		Servers::get(server, "Server")->resultData(request, field, out_data);
	});
}

RGL_API rgl_status_t rgl_gb300_server_get_result_host(rgl_gb300_server_t server, int64_t request, rgl_field_t field,
                                                      const void** out_data, int32_t* out_count)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		CHECK_ARG(out_data != nullptr);
		int32_t c = 0;
		*out_data = Servers::get(server, "Server")->resultHost(request, field, c);
		if (out_count) *out_count = c;
	});
}

RGL_API rgl_status_t rgl_gb300_server_get_request_timing(rgl_gb300_server_t server, int64_t request, double* out_queued_s,
                                                         double* out_total_s)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		double q = 0, t = 0;
		Servers::get(server, "Server")->timing(request, q, t);
		if (out_queued_s) *out_queued_s = q;
		if (out_total_s) *out_total_s = t;
	});
}

RGL_API rgl_status_t rgl_gb300_server_release(rgl_gb300_server_t server, int64_t request)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		Servers::get(server, "Server")->release(request);
	});
}

RGL_API rgl_status_t rgl_gb300_server_drain(rgl_gb300_server_t server)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		Servers::get(server, "Server")->drain();
	});
}

RGL_API rgl_status_t rgl_gb300_server_configure_schedule(rgl_gb300_server_t server, int32_t block, int32_t order, int32_t chunk,
                                                         int32_t regs, int64_t max_batch_beams)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		CHECK_ARG(block == 64 || block == 128 || block == 256);
		CHECK_ARG(order >= rgl::kOrderNatural && order <= rgl::kOrderElevation);
		CHECK_ARG(chunk >= 1 && chunk <= 64);
		CHECK_ARG(regs == 64 || regs == 80 || regs == 96 || regs == 128);
		CHECK_ARG(max_batch_beams >= 1);
		Servers::get(server, "Server")->configure(rgl::BatchSchedule{block, rgl::kPackLaneGroup, order, chunk, regs}, max_batch_beams);
	});
}

RGL_API rgl_status_t rgl_gb300_server_get_stats(rgl_gb300_server_t server, int64_t* out_submitted, int64_t* out_completed,
                                                int64_t* out_failed, int64_t* out_batches, int64_t* out_requests_in_batches,
                                                int64_t* out_peak_reserved_bytes, int64_t* out_device_us)
{
	return safeCall([&]() {
		CHECK_ARG(server != nullptr);
		const Server::Stats s = Servers::get(server, "Server")->stats();
		if (out_submitted) *out_submitted = s.submitted;
		if (out_completed) *out_completed = s.completed;
		if (out_failed) *out_failed = s.failed;
		if (out_batches) *out_batches = s.batches;
		if (out_requests_in_batches) *out_requests_in_batches = s.jobsInBatches;
		if (out_peak_reserved_bytes) *out_peak_reserved_bytes = s.peakReserved;
		if (out_device_us) *out_device_us = (int64_t) (s.deviceSeconds * 1e6);
	});
}

RGL_API rgl_status_t rgl_gb300_server_get_batch_times(rgl_gb300_server_t server, bool reset, float* out_max_ms, int64_t* out_over_5ms,
                                                      int64_t* out_batches)
{
	return safeCallKeepingValidation([&]() {
		CHECK_ARG(server != nullptr);
		const Server::BatchTimes t = Servers::get(server, "Server")->batchTimes(reset);
		for (int k = 0; k < 3; ++k) {
			if (out_max_ms) out_max_ms[k] = t.maxMs[k];
			if (out_over_5ms) out_over_5ms[k] = t.over5ms[k];
		}
		if (out_batches) *out_batches = t.batches;
	});
}

RGL_API rgl_status_t rgl_gb300_configure_trace_schedule(int32_t block, int32_t packing, int32_t chunk, int32_t regs)
{
	return safeCall([&]() {
		CHECK_ARG(block == 64 || block == 128 || block == 256);
		CHECK_ARG(packing == rgl::kPackLaneGroup || packing == rgl::kPackSerial);
		CHECK_ARG(chunk >= 1 && chunk <= 64);
		CHECK_ARG(regs == 64 || regs == 80 || regs == 96 || regs == 128);
		GraphRunCtx::synchronizeAll();
		setTraceSchedule(rgl::BatchSchedule{block, packing, traceSchedule().order, chunk, regs});
		// Captured runs baked the old schedule into their launches.
		for (auto& kv : Nodes::map()) {
			if (std::dynamic_pointer_cast<RaytraceNode>(kv.second)) {
				kv.second->markParamsChanged();
			}
		}
	});
}

RGL_API rgl_status_t rgl_gb300_configure_trace_order(int32_t order)
{
	return safeCall([&]() {
		CHECK_ARG(order >= rgl::kOrderNatural && order <= rgl::kOrderElevation);
		GraphRunCtx::synchronizeAll();
		rgl::BatchSchedule sch = traceSchedule();
		sch.order = order;
		setTraceSchedule(sch);
	});
}
