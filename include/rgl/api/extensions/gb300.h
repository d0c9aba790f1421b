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

/* Waits until the last run of the node's graph completed (rgl_graph_get_result_* also wait). */
RGL_API rgl_status_t rgl_gb300_graph_sync(rgl_node_t node);

/* Number of CUDA kernels this library launched since it was loaded. */
RGL_API rgl_status_t rgl_gb300_get_kernel_launch_count(uint64_t* out_count);

/*
 * Size of the default scene's acceleration structure after the last raytrace: bytes of BLAS wide nodes
 * and triangle records over all distinct meshes, and the number of entities (instances).
 */
RGL_API rgl_status_t rgl_gb300_scene_get_stats(int64_t* out_node_bytes, int64_t* out_triangle_bytes, int32_t* out_instances);

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
 * All calls share the array and clear what they use when they start; calls whose GPU work overlaps
 * (other streams or host threads) race on it and must be serialised by the caller.
 */
RGL_API rgl_status_t rgl_gb300_compact_by_flags_noalloc(const int32_t* flags, const void* src, int32_t count,
                                                        int32_t element_size, void* dst, int32_t* out_count, void* stream);
