/*
 * Additive entry points of the GB300 build. None of them has a counterpart in RobotecGPULidar's C API;
 * existing callers never need them, and every reference call keeps its meaning without them.
 */
#pragma once

#include <rgl/api/core.h>

/*
 * Makes a Gaussian noise node reproducible. The reference seeds its noise from std::random_device
 * (src/graph/NodesCore.hpp:536,563,590), so two runs never agree; this build draws each normal from
 * Philox4x32-10 keyed by (seed, noise kind, point or ray index, frame) and advances `frame` by one on
 * every graph run. Without this call a node gets a random seed, as in the reference.
 * Applies to nodes created by rgl_node_gaussian_noise_angular_ray / _angular_hitpoint / _distance.
 */
RGL_API rgl_status_t rgl_gb300_node_gaussian_noise_set_seed(rgl_node_t node, uint64_t seed, uint64_t frame);

/*
 * Sets the beam-divergence sub-ray pattern of a raytrace node: one primary ray plus `layers` rings of
 * `vertices` rays each (sample index 1 + layer * vertices + vertex, ring l scaled by 1 - l/layers).
 * The default, 3 x 19 (58 samples per beam), is the reference's fixed pattern
 * (src/gpu/MultiReturn.hpp:19-21); e.g. 1 x 4 gives 5 samples per beam. At most 63 extra rays.
 * Only used when a beam divergence is configured.
 */
RGL_API rgl_status_t rgl_gb300_node_raytrace_configure_beam_samples(rgl_node_t node, int32_t layers, int32_t vertices);

/* Enables CUDA-event timing of graph runs (whole run and traversal kernel). */
RGL_API rgl_status_t rgl_gb300_configure_timing(bool enable);

/* Device time of the last completed run of the node's graph, in milliseconds (timing enabled). */
RGL_API rgl_status_t rgl_gb300_graph_get_timing(rgl_node_t node, float* out_run_ms, float* out_trace_ms);

/*
 * Enables or disables CUDA-graph execution of graph runs (default: enabled, or disabled by the
 * environment variable RGL_GB300_CUDA_GRAPH=0). When enabled, a run's device work is captured into a
 * CUDA graph once and replayed by later runs until a node's parameters, links or buffers change.
 */
RGL_API rgl_status_t rgl_gb300_configure_cuda_graphs(bool enable);

/* Number of captures and replays performed for the node's graph so far. */
RGL_API rgl_status_t rgl_gb300_graph_get_capture_stats(rgl_node_t node, int64_t* out_captures, int64_t* out_replays);

/*
 * Traversal schedule of graph runs (rgl_graph_run). Every raytrace runs on the persistent traversal
 * kernel of batched frames as a one-job launch; this sets its block size (64, 128, 256), packing
 * (0: a beam's sub-rays on adjacent lanes, walking the scene together; 1: one lane per beam), tasks
 * per fetch (1..64) and register budget (64, 80, 96, 128). The default is 256, 0, 1, 128. Changes speed
 * only, never results.
 */
RGL_API rgl_status_t rgl_gb300_configure_trace_schedule(int32_t block, int32_t packing, int32_t chunk, int32_t regs);

/*
 * Beam visiting order of graph runs: 0 as given, 1 sorted by octahedral direction key, 2 by Morton key
 * of a probe point along the ray, 3 by elevation of the world direction, then azimuth (the rows of a
 * scan; the default). A run computes the order (one key kernel and one
 * sort) when its ray count, ray buffer or this setting changed, and keeps it for later ray contents
 * of the same count. Changes speed only, never results.
 */
RGL_API rgl_status_t rgl_gb300_configure_trace_order(int32_t order);

/* Waits until the last run of the node's graph completed (rgl_graph_get_result_* also wait). */
RGL_API rgl_status_t rgl_gb300_graph_sync(rgl_node_t node);

/* Number of CUDA kernels this library launched since it was loaded. */
RGL_API rgl_status_t rgl_gb300_get_kernel_launch_count(uint64_t* out_count);

/*
 * Size of the default scene's acceleration structure after the last raytrace: bytes of BLAS wide nodes
 * and triangle records over all distinct meshes, and the number of entities (instances).
 */
RGL_API rgl_status_t rgl_gb300_scene_get_stats(int64_t* out_node_bytes, int64_t* out_triangle_bytes, int32_t* out_instances);

/*
 * Builder of mesh BLASes (acceleration structures over a mesh's triangles), for meshes whose BLAS is
 * built after the call. No counterpart in the reference, whose OptiX GAS build
 * (src/scene/GASBuilder.hpp:31-100) has no choice of builder.
 *   RGL_GB300_BLAS_DEVICE_SAH   (default) binned SAH topology built on the device, then the 8-wide collapse
 *   RGL_GB300_BLAS_HOST_SAH     the same binned SAH tree built on the host and uploaded
 *   RGL_GB300_BLAS_DEVICE_LBVH  Morton codes, onesweep radix sort and LBVH on the device (as for animated entities)
 */
#define RGL_GB300_BLAS_DEVICE_SAH 0
#define RGL_GB300_BLAS_HOST_SAH 1
#define RGL_GB300_BLAS_DEVICE_LBVH 2
RGL_API rgl_status_t rgl_gb300_configure_blas_builder(int32_t builder);

/* Number of mesh BLAS builds since the library was loaded and their total wall time (ms, host clock,
 * the build's device work waited for). */
RGL_API rgl_status_t rgl_gb300_get_blas_build_stats(int64_t* out_builds, double* out_total_ms);

/* SM count and compute capability (major * 10 + minor) of the device in use. */
RGL_API rgl_status_t rgl_gb300_device_info(int32_t* out_sm_count, int32_t* out_compute_capability);

/*
 * Compaction for callers that cannot allocate device memory. No counterpart in the reference API.
 *
 * Engines that give the library only buffers they pre-allocated from their own pool, and real-time
 * loops that must never enter the CUDA allocator (cudaMalloc/cudaFree may synchronise the device),
 * cannot use the graph API's compaction: it allocates its look-back scratch on first use. This call
 * keeps that scratch in a fixed array inside the library and calls no cudaMalloc, cudaFree or
 * allocating routine. It copies the elements of `src` whose int32 flag is non-zero, in order, to `dst`:
 *   flags, src, dst   device pointers: `count` flags, `count * element_size` bytes in, room for as many out
 *   out_count         host pointer, receives the number of elements kept
 *   stream            a cudaStream_t, or NULL for the default stream; the call waits for its work on it
 * Limits: count <= 16,777,216 (larger counts return RGL_INVALID_ARGUMENT), element_size 1..256 bytes.
 * The fixed array (65,548 bytes) stays resident on every device that loads the library until exit.
 * The first call on a device looks up the array's device address, so make it before any stream capture.
 * Under CUDA's lazy module loading (the default) that first call also makes the driver load the
 * library's device code and the array on the device, which the driver allocates; callers that must
 * allocate nothing at run time make one warm-up call at initialisation. Later calls allocate nothing.
 * All calls share the array and clear what they use when they start; calls whose GPU work overlaps
 * (other streams or host threads) race on it and must be serialised by the caller.
 */
RGL_API rgl_status_t rgl_gb300_compact_by_flags_noalloc(const int32_t* flags, const void* src, int32_t count,
                                                        int32_t element_size, void* dst, int32_t* out_count, void* stream);

/*
 * Batched multi-sensor frames. The reference has no batched form: every sensor's graph runs on its
 * own with rgl_graph_run (src/api/apiCore.cpp:530-544).
 *
 * A batch is a list of ordinary graphs, given by any one node of each; each graph must hold exactly
 * one raytrace node (the graphs may trace different scenes). rgl_gb300_batch_run runs one frame:
 * every graph is validated and prepared as by rgl_graph_run, then CUDA graphs hold the frame's
 * device work (instance upload and TLAS refit after rgl_entity_set_transform, every graph's nodes,
 * and one persistent traversal launch per wave of sensors, see rgl_gb300_batch_configure_waves).
 * They are captured on the first frame and replayed while nothing structural changes. Results are read per graph with
 * rgl_graph_get_result_size/_data and equal what rgl_graph_run of that graph alone writes.
 * At most 1024 graphs per batch. Destroy a batch before destroying its graphs.
 */
typedef struct BatchRun* rgl_gb300_batch_t;

RGL_API rgl_status_t rgl_gb300_batch_create(rgl_gb300_batch_t* out_batch, const rgl_node_t* nodes, int32_t node_count);
RGL_API rgl_status_t rgl_gb300_batch_run(rgl_gb300_batch_t batch);
RGL_API rgl_status_t rgl_gb300_batch_destroy(rgl_gb300_batch_t batch);

/*
 * Traversal schedule of a batch. With `autotune` (the default) the library times a staged set of
 * candidates on the first frame of every new batch shape (per-graph ray and sample counts) and keeps
 * the fastest; otherwise the given schedule is used:
 *   block    threads per block: 64, 128 or 256
 *   packing  0: a beam's sub-rays on adjacent lanes, walking the scene together; 1: one lane per
 *            beam, sub-rays in turn
 *   order    beam visiting order. 0: as given; 1: sorted by octahedral direction; 2: by Morton code
 *            of a probe point; 3: by elevation, then azimuth (the rows of a scan)
 *   chunk    tasks (one warp's beams each) taken per fetch from the shared work counter, 1..64
 *   regs     registers per thread: 64, 80, 96 or 128 (fewer registers, more resident warps)
 * The schedule changes speed only, never results.
 */
RGL_API rgl_status_t rgl_gb300_batch_configure_schedule(rgl_gb300_batch_t batch, bool autotune, int32_t block, int32_t packing,
                                                        int32_t order, int32_t chunk, int32_t regs);
RGL_API rgl_status_t rgl_gb300_batch_get_schedule(rgl_gb300_batch_t batch, int32_t* out_block, int32_t* out_packing,
                                                  int32_t* out_order, int32_t* out_chunk, int32_t* out_regs);

/*
 * Waves of a batch frame. The frame's graphs are cut, in batch order, into `waves` contiguous runs of
 * about equal traced rays, each traced by its own persistent launch (which starts while the previous
 * one drains) and followed by its graphs' later nodes; a graph's results are ready, and
 * rgl_graph_get_result_* returns, once its wave's later nodes end, so reads of the first graphs
 * overlap the device work of the rest. 0 (the default) picks one wave per 2 Mi traced rays, at most
 * 16; the count never exceeds the number of graphs. get_waves gives the count of the last frame (0
 * before the first). Changes speed and result latency only, never results.
 */
RGL_API rgl_status_t rgl_gb300_batch_configure_waves(rgl_gb300_batch_t batch, int32_t waves);
RGL_API rgl_status_t rgl_gb300_batch_get_waves(rgl_gb300_batch_t batch, int32_t* out_waves);

/*
 * The candidates timed by the batch's last tuning, in the order tried: five int32 per candidate
 * (block, packing, order, chunk, regs) into out_schedules and its traversal time (ms, best of its
 * repetitions) into out_ms, at most `capacity` candidates; out_count receives the number tried
 * (0 before any tuning). No counterpart in the reference, which has no batched traversal.
 */
RGL_API rgl_status_t rgl_gb300_batch_get_tuning(rgl_gb300_batch_t batch, int32_t capacity, int32_t* out_schedules, float* out_ms,
                                                int32_t* out_count);

/*
 * Statistics of a batch: device time of the last completed frame and of its traversal launch (ms),
 * beams and traced rays (beams x sub-rays) of the last frame, and the number of captures, replays and
 * tunings so far. Waits for the last frame.
 */
RGL_API rgl_status_t rgl_gb300_batch_get_stats(rgl_gb300_batch_t batch, float* out_frame_ms, float* out_trace_ms, int64_t* out_beams,
                                               int64_t* out_rays, int64_t* out_captures, int64_t* out_replays, int64_t* out_tunings);

/*
 * Resident scenes. The reference accepts only NULL (its one default scene) wherever an rgl_scene_t is
 * passed (src/api/apiCore.cpp:297,516,922). This build also accepts scenes made here: rgl_entity_create,
 * rgl_scene_set_time and rgl_node_raytrace take them, and NULL keeps meaning the default scene. Meshes
 * (and their acceleration structures) are shared by all scenes. Destroying a scene destroys its
 * entities; raytrace nodes that trace it keep an empty scene.
 */
RGL_API rgl_status_t rgl_gb300_scene_create(rgl_scene_t* out_scene);
RGL_API rgl_status_t rgl_gb300_scene_destroy(rgl_scene_t scene);
/* As rgl_gb300_scene_get_stats, for any scene (NULL: the default scene). */
RGL_API rgl_status_t rgl_gb300_scene_get_stats_of(rgl_scene_t scene, int64_t* out_node_bytes, int64_t* out_triangle_bytes,
                                                 int32_t* out_instances);

/*
 * Serving loop. No counterpart in the reference, whose clients run one rgl_graph_run per scan.
 *
 * Robots register their ray patterns (sensor-local rgl_mat3x4f rays, as for rgl_node_rays_from_mat3x4f)
 * once; the patterns stay on the device. A scan request names a scene, a pattern, the sensor pose,
 * a return mode and a range. A scheduler thread admits requests first come first served while the
 * bytes of admitted requests (24 B per point of device buffers while on the GPU and 20 B per point of
 * pinned host results until released; points = rays x returns) stay within `hbm_budget_bytes` and
 * fewer than `max_in_flight_batches` batches run,
 * and launches all admitted requests as one batch (one persistent traversal launch plus one segmented
 * compaction). Requests arriving meanwhile go into the next batch (continuous batching).
 *
 * A request's result is XYZ_VEC3_F32, DISTANCE_F32 and ENTITY_ID_I32 of its hit points, in point order:
 * the same bytes as the graph rays_from_mat3x4f(pattern) -> rays_transform(pose) ->
 * rays_set_range({min, max}) -> raytrace(scene, mode) -> points_compact_by_field(IS_HIT) -> yield.
 * Scenes used by a server must not be modified while it has requests (rgl_gb300_server_drain first).
 */
typedef struct Server* rgl_gb300_server_t;

RGL_API rgl_status_t rgl_gb300_server_create(rgl_gb300_server_t* out_server, int64_t hbm_budget_bytes, int32_t max_in_flight_batches);
RGL_API rgl_status_t rgl_gb300_server_destroy(rgl_gb300_server_t server);
RGL_API rgl_status_t rgl_gb300_server_add_pattern(rgl_gb300_server_t server, const rgl_mat3x4f* rays, int32_t ray_count,
                                                  int32_t* out_pattern);
RGL_API rgl_status_t rgl_gb300_server_submit(rgl_gb300_server_t server, rgl_scene_t scene, int32_t pattern,
                                             const rgl_mat3x4f* sensor_pose, rgl_return_mode_t return_mode, float min_range,
                                             float max_range, int64_t* out_request);
/* Waits up to timeout_ms (negative: without limit) for a request; *out_done tells whether it completed. */
RGL_API rgl_status_t rgl_gb300_server_wait(rgl_gb300_server_t server, int64_t request, float timeout_ms, bool* out_done);
/* Moves up to `capacity` ids of requests completed since the last call into out_requests. */
RGL_API rgl_status_t rgl_gb300_server_take_completed(rgl_gb300_server_t server, int64_t* out_requests, int32_t capacity,
                                                     int32_t* out_count);
/* As rgl_gb300_server_take_completed, but first waits up to timeout_ms for a completed request. */
RGL_API rgl_status_t rgl_gb300_server_wait_completed(rgl_gb300_server_t server, float timeout_ms, int64_t* out_requests, int32_t capacity,
                                                     int32_t* out_count);
RGL_API rgl_status_t rgl_gb300_server_get_result_size(rgl_gb300_server_t server, int64_t request, rgl_field_t field,
                                                      int32_t* out_count, int32_t* out_size_of);
RGL_API rgl_status_t rgl_gb300_server_get_result_data(rgl_gb300_server_t server, int64_t request, rgl_field_t field, void* out_data);
/*
 * Host address of a completed request's field and its element count. Results are written by the GPU
 * straight into the server's pinned host memory, so this needs no copy; the address stays valid
 * until rgl_gb300_server_release.
 */
RGL_API rgl_status_t rgl_gb300_server_get_result_host(rgl_gb300_server_t server, int64_t request, rgl_field_t field,
                                                      const void** out_data, int32_t* out_count);
/* Seconds from submission to admission into a batch, and from submission to completion. */
RGL_API rgl_status_t rgl_gb300_server_get_request_timing(rgl_gb300_server_t server, int64_t request, double* out_queued_s,
                                                         double* out_total_s);
/* Frees a completed request's result (waits for it first if it is still running). */
RGL_API rgl_status_t rgl_gb300_server_release(rgl_gb300_server_t server, int64_t request);
/* Waits until no request is pending or running. */
RGL_API rgl_status_t rgl_gb300_server_drain(rgl_gb300_server_t server);

/*
 * Traversal schedule of the server's batches (block, order, chunk and regs as for
 * rgl_gb300_batch_configure_schedule; order 0 casts a pattern's beams in the given order, 1 and 2 in
 * its octahedral direction order, 3 in its scan-row order: elevation, then azimuth) and the most beams
 * coalesced into one batch (>= 1; a single larger request still forms a batch of its own). Applies to
 * batches launched afterwards; changes speed only, never results. Defaults: 256, 3, 1, 128 and 4 Mi
 * beams.
 */
RGL_API rgl_status_t rgl_gb300_server_configure_schedule(rgl_gb300_server_t server, int32_t block, int32_t order, int32_t chunk,
                                                         int32_t regs, int64_t max_batch_beams);
/* Counters: requests submitted, completed (including failed), failed; batches launched and the requests
 * they held; the largest admitted byte total; the summed device time of the batches in microseconds. */
RGL_API rgl_status_t rgl_gb300_server_get_stats(rgl_gb300_server_t server, int64_t* out_submitted, int64_t* out_completed,
                                                int64_t* out_failed, int64_t* out_batches, int64_t* out_requests_in_batches,
                                                int64_t* out_peak_reserved_bytes, int64_t* out_device_us);

/*
 * Phases of the batches retired since the last call with `reset` (or since creation), on the device's
 * clock, three entries each: traversal and compaction (launch to kept counts published), the server's
 * reaction (counts published to the first result copy enqueued), the result copies. out_max_ms gets
 * the longest of each phase, out_over_5ms how many batches spent more than 5 ms in it.
 */
RGL_API rgl_status_t rgl_gb300_server_get_batch_times(rgl_gb300_server_t server, bool reset, float* out_max_ms, int64_t* out_over_5ms,
                                                      int64_t* out_batches);
