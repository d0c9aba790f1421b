/*
 * RGL C API — GB300-native implementation.
 *
 * This header declares the same C ABI as RobotecGPULidar v0.19.0
 * (reference: include/rgl/api/core.h:52-1198): every function name, argument
 * list, enum value and POD struct layout is kept identical so that an engine
 * plugin built against RGL links against libRobotecGPULidar.so from this
 * project without source changes.  Only the implementation behind it differs
 * (hand-written sm_103a CUDA instead of OptiX).
 *
 * Conventions shared with the reference:
 *  - every call returns rgl_status_t, except rgl_get_last_error_string;
 *  - input arrays are copied before the call returns, the caller keeps ownership;
 *  - node-creating calls follow the create-or-modify idiom: *node == NULL creates
 *    a node, otherwise the existing node is re-parameterised;
 *  - results are read into caller buffers sized with rgl_graph_get_result_size.
 *
 * Beside the ray-casting path this library implements ring ids, time offsets,
 * ray masks, velocities and velocity distortion, external and skeleton mesh
 * animation, intensity textures, laser retro, spatial and temporal merges,
 * points from arrays, the ground filter and tape record/playback. The radar
 * nodes are exported with the reference's signatures and return
 * RGL_NOT_IMPLEMENTED.
 */
#pragma once

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#include <type_traits>
#define NO_MANGLING extern "C"
#else
#define NO_MANGLING
#endif

#if defined RGL_STATIC
#define RGL_VISIBLE
#elif defined _WIN32 || defined __CYGWIN__
#define RGL_VISIBLE __declspec(dllexport)
#else
#define RGL_VISIBLE __attribute__((visibility("default")))
#endif

#define RGL_API NO_MANGLING RGL_VISIBLE

/* Version of the API this library implements (reference core.h:52-54). */
#define RGL_VERSION_MAJOR 0
#define RGL_VERSION_MINOR 19
#define RGL_VERSION_PATCH 0

/* Entity id written for non-hits, and id of entities that never got one (reference core.h:57-62). */
#define RGL_ENTITY_INVALID_ID 0
#define RGL_DEFAULT_ENTITY_ID 268435455

/* ---- POD types (fixed layout, reference core.h:67-160) ---- */

typedef struct
{
	float value[2];
} rgl_vec2f;

typedef struct
{
	float value[3];
} rgl_vec3f;

typedef struct
{
	int32_t value[3];
} rgl_vec3i;

/* Row-major 3x4 affine matrix: value[row][col]; column 3 is the translation. */
typedef struct
{
	float value[3][4];
} rgl_mat3x4f;

typedef struct
{
	float begin_distance;
	float end_distance;
	float distance_separation_threshold;
	float radial_speed_separation_threshold;
	float azimuth_separation_threshold;
} rgl_radar_scope_t;

typedef struct
{
	float weights[4];
	int32_t bone_indexes[4];
} rgl_bone_weights_t;

#ifdef __cplusplus
static_assert(sizeof(rgl_vec2f) == 8 && std::is_trivial<rgl_vec2f>::value, "rgl_vec2f layout");
static_assert(sizeof(rgl_vec3f) == 12 && std::is_trivial<rgl_vec3f>::value, "rgl_vec3f layout");
static_assert(sizeof(rgl_vec3i) == 12 && std::is_trivial<rgl_vec3i>::value, "rgl_vec3i layout");
static_assert(sizeof(rgl_mat3x4f) == 48 && std::is_trivial<rgl_mat3x4f>::value, "rgl_mat3x4f layout");
static_assert(sizeof(rgl_radar_scope_t) == 20, "rgl_radar_scope_t layout");
static_assert(sizeof(rgl_bone_weights_t) == 32, "rgl_bone_weights_t layout");
#endif

typedef enum : int32_t
{
	RGL_RADAR_CLASS_CAR = 0,
	RGL_RADAR_CLASS_TRUCK,
	RGL_RADAR_CLASS_MOTORCYCLE,
	RGL_RADAR_CLASS_BICYCLE,
	RGL_RADAR_CLASS_PEDESTRIAN,
	RGL_RADAR_CLASS_ANIMAL,
	RGL_RADAR_CLASS_HAZARD,
	RGL_RADAR_CLASS_UNKNOWN,
	RGL_RADAR_CLASS_COUNT
} rgl_radar_object_class_t;

/* ---- Opaque handles (reference core.h:199-224) ---- */
typedef struct Mesh* rgl_mesh_t;
typedef struct Entity* rgl_entity_t;
typedef struct Texture* rgl_texture_t;
typedef struct Node* rgl_node_t;
typedef struct Scene* rgl_scene_t;

typedef enum : int32_t
{
	RGL_EXTENSION_PCL = 0,
	RGL_EXTENSION_ROS2 = 1,
	RGL_EXTENSION_UDP = 2,
	RGL_EXTENSION_WEATHER = 3,
	RGL_EXTENSION_COUNT
} rgl_extension_t;

/* Status codes (reference core.h:244-327). Recoverable: INVALID_ARGUMENT, INVALID_API_OBJECT,
 * INVALID_PIPELINE, INVALID_FILE_PATH, NOT_IMPLEMENTED, TAPE/UDP/ROS2 errors. Any other error
 * latches the library into RGL_INVALID_STATE. */
typedef enum : int32_t
{
	RGL_SUCCESS = 0,
	RGL_INVALID_ARGUMENT,
	RGL_INVALID_STATE,
	RGL_LOGGING_ERROR,
	RGL_INVALID_API_OBJECT,
	RGL_INVALID_FILE_PATH,
	RGL_TAPE_ERROR,
	RGL_UDP_ERROR,
	RGL_ROS2_ERROR,
	RGL_INVALID_PIPELINE,
	RGL_INITIALIZATION_ERROR,
	RGL_NOT_IMPLEMENTED = 404,
	RGL_INTERNAL_EXCEPTION = 500,
} rgl_status_t;

typedef enum : int32_t
{
	RGL_LOG_LEVEL_ALL = 0,
	RGL_LOG_LEVEL_TRACE = 0,
	RGL_LOG_LEVEL_DEBUG = 1,
	RGL_LOG_LEVEL_INFO = 2,
	RGL_LOG_LEVEL_WARN = 3,
	RGL_LOG_LEVEL_ERROR = 4,
	RGL_LOG_LEVEL_CRITICAL = 5,
	RGL_LOG_LEVEL_OFF = 6,
	RGL_LOG_LEVEL_COUNT = 7
} rgl_log_level_t;

/* Point fields (reference core.h:348-450). Sizes in bytes: XYZ 12, INTENSITY_F32 4, INTENSITY_U8 1,
 * IS_HIT 4, IS_GROUND 4, RAY_IDX 4, ENTITY_ID 4, DISTANCE 4, AZIMUTH 4, ELEVATION 4, RING_ID 2,
 * RETURN_TYPE 1, TIME_STAMP_F64 8, TIME_STAMP_U32 4, velocities 12, RADIAL_SPEED 4, POWER 4, RCS 4,
 * NOISE 4, SNR 4, NORMAL 12, INCIDENT_ANGLE 4, RAY_POSE 48, LASER_RETRO 4, paddings 1/2/4. */
typedef enum : int32_t
{
	RGL_FIELD_XYZ_VEC3_F32 = 1,
	RGL_FIELD_INTENSITY_F32,
	RGL_FIELD_INTENSITY_U8,
	RGL_FIELD_IS_HIT_I32,
	RGL_FIELD_IS_GROUND_I32,
	RGL_FIELD_RAY_IDX_U32,
	RGL_FIELD_ENTITY_ID_I32,
	RGL_FIELD_DISTANCE_F32,
	RGL_FIELD_AZIMUTH_F32,
	RGL_FIELD_ELEVATION_F32,
	RGL_FIELD_RING_ID_U16,
	RGL_FIELD_RETURN_TYPE_U8,
	RGL_FIELD_TIME_STAMP_F64,
	RGL_FIELD_TIME_STAMP_U32,
	RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32,
	RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32,
	RGL_FIELD_RADIAL_SPEED_F32,
	RGL_FIELD_POWER_F32,
	RGL_FIELD_RCS_F32,
	RGL_FIELD_NOISE_F32,
	RGL_FIELD_SNR_F32,
	RGL_FIELD_NORMAL_VEC3_F32,
	RGL_FIELD_INCIDENT_ANGLE_F32,
	RGL_FIELD_RAY_POSE_MAT3x4_F32,
	RGL_FIELD_LASER_RETRO_F32,
	RGL_FIELD_PADDING_8 = 1024,
	RGL_FIELD_PADDING_16,
	RGL_FIELD_PADDING_32,
	RGL_FIELD_DYNAMIC_FORMAT = 13842,
} rgl_field_t;

/* Return-mode encoding (reference core.h:452-504): bits 24..31 hold the number of returns per beam,
 * byte k (bits 8k..8k+7) holds the type of return k. */
const int32_t RGL_RETURN_MODE_BIT_SHIFT = 24;
const int32_t RGL_RETURN_MODE_SINGLE = 1 << RGL_RETURN_MODE_BIT_SHIFT;
const int32_t RGL_RETURN_MODE_DUAL = 2 << RGL_RETURN_MODE_BIT_SHIFT;
const int32_t RGL_RETURN_TYPE_BIT_SHIFT = 8;

typedef enum : uint8_t
{
	RGL_RETURN_TYPE_UNKNOWN = 0,
	RGL_RETURN_TYPE_STRONGEST = 1,
	RGL_RETURN_TYPE_LAST = 2,
	RGL_RETURN_TYPE_SECOND = 3,
	RGL_RETURN_TYPE_FIRST = 4,
	RGL_RETURN_TYPE_SECOND_STRONGEST = 5,
} rgl_return_type_t;

typedef enum : int32_t
{
	RGL_RETURN_UNKNOWN = RGL_RETURN_TYPE_UNKNOWN,
	RGL_RETURN_FIRST = RGL_RETURN_MODE_SINGLE | RGL_RETURN_TYPE_FIRST,
	RGL_RETURN_SECOND = RGL_RETURN_MODE_SINGLE | RGL_RETURN_TYPE_SECOND,
	RGL_RETURN_LAST = RGL_RETURN_MODE_SINGLE | RGL_RETURN_TYPE_LAST,
	RGL_RETURN_STRONGEST = RGL_RETURN_MODE_SINGLE | RGL_RETURN_TYPE_STRONGEST,
	RGL_RETURN_LAST_STRONGEST = RGL_RETURN_MODE_DUAL | (RGL_RETURN_TYPE_LAST) |
	                            (RGL_RETURN_TYPE_STRONGEST << RGL_RETURN_TYPE_BIT_SHIFT),
	RGL_RETURN_FIRST_LAST = RGL_RETURN_MODE_DUAL | (RGL_RETURN_TYPE_FIRST) | (RGL_RETURN_TYPE_LAST << RGL_RETURN_TYPE_BIT_SHIFT),
	RGL_RETURN_FIRST_STRONGEST = RGL_RETURN_MODE_DUAL | (RGL_RETURN_TYPE_FIRST) |
	                             (RGL_RETURN_TYPE_STRONGEST << RGL_RETURN_TYPE_BIT_SHIFT),
	RGL_RETURN_STRONGEST_SECOND_STRONGEST = RGL_RETURN_MODE_DUAL | (RGL_RETURN_TYPE_STRONGEST) |
	                                        (RGL_RETURN_TYPE_SECOND_STRONGEST << RGL_RETURN_TYPE_BIT_SHIFT),
	RGL_RETURN_FIRST_SECOND = RGL_RETURN_MODE_DUAL | (RGL_RETURN_TYPE_FIRST) |
	                          (RGL_RETURN_TYPE_SECOND << RGL_RETURN_TYPE_BIT_SHIFT),
} rgl_return_mode_t;

typedef enum : int32_t
{
	RGL_AXIS_X = 1,
	RGL_AXIS_Y = 2,
	RGL_AXIS_Z = 3,
} rgl_axis_t;

/* ---- General (reference core.h:526-560; src/api/apiCore.cpp:33-164) ---- */
RGL_API rgl_status_t rgl_get_version_info(int32_t* out_major, int32_t* out_minor, int32_t* out_patch);
RGL_API rgl_status_t rgl_get_extension_info(rgl_extension_t extension, int32_t* out_available);
RGL_API rgl_status_t rgl_configure_logging(rgl_log_level_t log_level, const char* log_file_path, bool use_stdout);
RGL_API void rgl_get_last_error_string(const char** out_error_string);
RGL_API rgl_status_t rgl_cleanup(void);

/* ---- Mesh (reference core.h:562-615; apiCore.cpp:172-275) ---- */
RGL_API rgl_status_t rgl_mesh_create(rgl_mesh_t* out_mesh, const rgl_vec3f* vertices, int32_t vertex_count,
                                     const rgl_vec3i* indices, int32_t index_count);
RGL_API rgl_status_t rgl_mesh_set_texture_coords(rgl_mesh_t mesh, const rgl_vec2f* uvs, int32_t uv_count);
RGL_API rgl_status_t rgl_mesh_set_bone_weights(rgl_mesh_t mesh, const rgl_bone_weights_t* bone_weights,
                                               int32_t bone_weights_count);
RGL_API rgl_status_t rgl_mesh_set_restposes(rgl_mesh_t mesh, const rgl_mat3x4f* restposes, int32_t bones_count);
RGL_API rgl_status_t rgl_mesh_destroy(rgl_mesh_t mesh);
RGL_API rgl_status_t rgl_mesh_is_alive(rgl_mesh_t mesh, bool* out_alive);

/* ---- Entity (reference core.h:617-700; apiCore.cpp:291-445) ---- */
RGL_API rgl_status_t rgl_entity_create(rgl_entity_t* out_entity, rgl_scene_t scene, rgl_mesh_t mesh);
RGL_API rgl_status_t rgl_entity_destroy(rgl_entity_t entity);
RGL_API rgl_status_t rgl_entity_set_transform(rgl_entity_t entity, const rgl_mat3x4f* transform);
RGL_API rgl_status_t rgl_entity_set_pose_world(rgl_entity_t entity, const rgl_mat3x4f* pose, int32_t bones_count);
RGL_API rgl_status_t rgl_entity_set_id(rgl_entity_t entity, int32_t id);
RGL_API rgl_status_t rgl_entity_set_intensity_texture(rgl_entity_t entity, rgl_texture_t texture);
RGL_API rgl_status_t rgl_entity_set_laser_retro(rgl_entity_t entity, float retro);
RGL_API rgl_status_t rgl_entity_apply_external_animation(rgl_entity_t entity, const rgl_vec3f* vertices, int32_t vertex_count);
RGL_API rgl_status_t rgl_entity_is_alive(rgl_entity_t entity, bool* out_alive);

/* ---- Texture (reference core.h:702-730) ---- */
RGL_API rgl_status_t rgl_texture_create(rgl_texture_t* out_texture, const void* texels, int32_t width, int32_t height);
RGL_API rgl_status_t rgl_texture_destroy(rgl_texture_t texture);
RGL_API rgl_status_t rgl_texture_is_alive(rgl_texture_t texture, bool* out_alive);

/* ---- Scene (reference core.h:732-742) ---- */
RGL_API rgl_status_t rgl_scene_set_time(rgl_scene_t scene, uint64_t nanoseconds);

/* ---- Ray nodes (reference core.h:744-815) ---- */
RGL_API rgl_status_t rgl_node_rays_from_mat3x4f(rgl_node_t* node, const rgl_mat3x4f* rays, int32_t ray_count);
RGL_API rgl_status_t rgl_node_rays_set_ring_ids(rgl_node_t* node, const int32_t* ring_ids, int32_t ring_ids_count);
RGL_API rgl_status_t rgl_node_rays_set_range(rgl_node_t* node, const rgl_vec2f* ranges, int32_t ranges_count);
RGL_API rgl_status_t rgl_node_rays_set_time_offsets(rgl_node_t* node, const float* offsets, int32_t offsets_count);
RGL_API rgl_status_t rgl_node_rays_transform(rgl_node_t* node, const rgl_mat3x4f* transform);

/* ---- Point / raytrace nodes (reference core.h:817-1095) ---- */
RGL_API rgl_status_t rgl_node_points_transform(rgl_node_t* node, const rgl_mat3x4f* transform);
RGL_API rgl_status_t rgl_node_raytrace(rgl_node_t* node, rgl_scene_t scene);
RGL_API rgl_status_t rgl_node_raytrace_configure_velocity(rgl_node_t node, const rgl_vec3f* linear_velocity,
                                                          const rgl_vec3f* angular_velocity);
RGL_API rgl_status_t rgl_node_raytrace_configure_distortion(rgl_node_t node, bool enable);
RGL_API rgl_status_t rgl_node_raytrace_configure_non_hits(rgl_node_t node, float nearDistance, float farDistance);
RGL_API rgl_status_t rgl_node_raytrace_configure_mask(rgl_node_t node, const int8_t* rays_mask, int32_t rays_count);
RGL_API rgl_status_t rgl_node_raytrace_configure_beam_divergence(rgl_node_t node, float horizontal_beam_divergence,
                                                                 float vertical_beam_divergence);
RGL_API rgl_status_t rgl_node_raytrace_configure_default_intensity(rgl_node_t node, float default_intensity);
RGL_API rgl_status_t rgl_node_raytrace_configure_return_mode(rgl_node_t node, rgl_return_mode_t return_mode);
RGL_API rgl_status_t rgl_node_points_format(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count);
RGL_API rgl_status_t rgl_node_points_yield(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count);
RGL_API rgl_status_t rgl_node_points_compact_by_field(rgl_node_t* node, rgl_field_t field);
RGL_API rgl_status_t rgl_node_points_spatial_merge(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count);
RGL_API rgl_status_t rgl_node_points_temporal_merge(rgl_node_t* node, const rgl_field_t* fields, int32_t field_count);
RGL_API rgl_status_t rgl_node_points_from_array(rgl_node_t* node, const void* points, int32_t points_count,
                                                const rgl_field_t* fields, int32_t field_count);
RGL_API rgl_status_t rgl_node_points_radar_postprocess(rgl_node_t* node, const rgl_radar_scope_t* radar_scopes,
                                                       int32_t radar_scopes_count, float ray_azimuth_step,
                                                       float ray_elevation_step, float frequency, float power_transmitted,
                                                       float cumulative_device_gain, float received_noise_mean,
                                                       float received_noise_st_dev);
RGL_API rgl_status_t rgl_node_points_radar_track_objects(rgl_node_t* node, float object_distance_threshold,
                                                         float object_azimuth_threshold, float object_elevation_threshold,
                                                         float object_radial_speed_threshold, float max_matching_distance,
                                                         float max_prediction_time_frame, float movement_sensitivity);
RGL_API rgl_status_t rgl_node_points_radar_set_classes(rgl_node_t node, const int32_t* entity_ids,
                                                       const rgl_radar_object_class_t* object_classes, int32_t count);
RGL_API rgl_status_t rgl_node_points_filter_ground(rgl_node_t* node, const rgl_vec3f* sensor_up_vector,
                                                   float ground_angle_threshold);
RGL_API rgl_status_t rgl_node_gaussian_noise_angular_ray(rgl_node_t* node, float mean, float st_dev, rgl_axis_t rotation_axis);
RGL_API rgl_status_t rgl_node_gaussian_noise_angular_hitpoint(rgl_node_t* node, float mean, float st_dev,
                                                              rgl_axis_t rotation_axis);
RGL_API rgl_status_t rgl_node_gaussian_noise_distance(rgl_node_t* node, float mean, float st_dev_base,
                                                      float st_dev_rise_per_meter);
RGL_API rgl_status_t rgl_node_is_alive(rgl_node_t node, bool* out_alive);

/* ---- Graph (reference core.h:1097-1198) ---- */
RGL_API rgl_status_t rgl_graph_run(rgl_node_t node);
RGL_API rgl_status_t rgl_graph_destroy(rgl_node_t node);
RGL_API rgl_status_t rgl_graph_get_result_size(rgl_node_t node, rgl_field_t field, int32_t* out_count, int32_t* out_size_of);
RGL_API rgl_status_t rgl_graph_get_result_data(rgl_node_t node, rgl_field_t field, void* data);
RGL_API rgl_status_t rgl_graph_node_add_child(rgl_node_t parent, rgl_node_t child);
RGL_API rgl_status_t rgl_graph_node_remove_child(rgl_node_t parent, rgl_node_t child);
RGL_API rgl_status_t rgl_graph_node_set_priority(rgl_node_t node, int32_t priority);
RGL_API rgl_status_t rgl_graph_node_get_priority(rgl_node_t node, int32_t* out_priority);
