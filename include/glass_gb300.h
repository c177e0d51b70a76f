/*
 * glass_gb300.h - C ABI of the GB300-native resident light-stack library.
 *
 * This header is the drop-in boundary.  GLASS reaches its CUDA backend through
 * one Python module name, `_glass_cuda_native`, imported lazily by
 * src/glass_cuda.py:31-44 and exercised through the pybind11 module defined in
 * cpp/src/native_bindings.cpp:20383-21200.  This library replaces that module
 * with a plain C ABI; glass_gb300/_glass_cuda_native.py is the ctypes shim that
 * presents the same Python names on top of it.  Each declaration below names
 * the reference entry point it replaces.
 *
 * Conventions (all functions):
 *   - return int status: GG_OK (0) or a negative GG_ERR_* code; the message of
 *     the last failure on the calling thread is available from gg_last_error();
 *   - all pointers named host_* are caller-owned host buffers (pinned or
 *     pageable), all pointers named dev_* are device pointers;
 *   - float32 / uint16 / int16 / uint8 / int64 / float64 only, C-contiguous;
 *   - a gg_stack is not thread-safe; distinct stacks may be used from distinct
 *     threads.  Work is enqueued on the stack's stream; functions that return
 *     host data synchronise that stream before returning.
 */
#ifndef GLASS_GB300_H
#define GLASS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mapped by the shim onto Python exceptions) ----------- */
#define GG_OK 0
#define GG_ERR_INVALID_ARGUMENT (-1) /* ValueError  (std::invalid_argument in the reference) */
#define GG_ERR_OUT_OF_RANGE (-2)     /* IndexError  (std::out_of_range)                      */
#define GG_ERR_RUNTIME (-3)          /* RuntimeError (state errors, e.g. frames not loaded)  */
#define GG_ERR_CUDA (-4)             /* RuntimeError (check_cuda, native_bindings.cpp:1011)  */
#define GG_ERR_NO_DEVICE (-5)        /* RuntimeError: no CUDA device                          */
#define GG_ERR_OUT_OF_MEMORY (-6)    /* MemoryError                                           */
#define GG_ERR_TIMEOUT (-7)          /* a bounded device-side wait ran out                    */

/* ---- enumerations -------------------------------------------------------- */
#define GG_REJECT_NONE 0        /* weighted mean, cpu/integration.py:106-118                 */
#define GG_REJECT_SIGMA_CLIP 1  /* median centre / std scale, engine/rejection.py:47-49      */
#define GG_REJECT_WINSORIZED 2  /* engine/rejection.py:39-44, 54-60, 219-297                */
#define GG_REJECT_LINEAR_FIT 3  /* linear-fit clipping; no counterpart in the reference      */

#define GG_COUNT_F32 0 /* count maps as float32 (cpu/integration.py:100-110)          */
#define GG_COUNT_U16 1 /* count maps as uint16 (count_map_dtype="uint16")              */

#define GG_INTERP_NEAREST 0 /* integer translations (cpu/warp.py:6-22), engine/warp.py:87-96 */
#define GG_INTERP_BILINEAR 1
#define GG_INTERP_LANCZOS3 3

/* ---- library / device ---------------------------------------------------- */
/* Library ABI version (major*10000 + minor*100 + patch). */
int gg_version(int* version);
/* Copies the last error message of the calling thread (NUL-terminated). */
int gg_last_error(char* buf, size_t cap);
/* Number of CUDA kernels this library has launched in this process
 * (instrumentation; no reference counterpart). */
int gg_kernel_launches(int64_t* count);
/* Replaces `cuda_available()` (native_bindings.cpp module def; glass_cuda.py:62). */
int gg_cuda_available(int* available);
/* Replaces `list_devices()` / `get_device_info(i)` (glass_cuda.py:184-212). */
typedef struct {
  char name[256];
  int major;
  int minor;
  int multiprocessor_count;
  int64_t total_global_mem;
  int64_t l2_cache_bytes;
  int64_t shared_mem_per_block_optin;
} gg_device_info_t;
int gg_device_count(int* count);
int gg_device_info(int device, gg_device_info_t* info);
/* Replaces `host_pinned_empty_{f32,u8}` (glass_cuda.py:215-226). */
int gg_host_alloc_pinned(size_t bytes, void** host_ptr);
int gg_host_free_pinned(void* host_ptr);

/* ---- calibration parameters --------------------------------------------- */
/* Mirrors CalibrationParameters (native_bindings.cpp:15138-15158) and the CPU
 * policy fields read by cpu/calibration.py:51-76.  dark_scale is the already
 * resolved light/dark exposure ratio (1 when scaling is off). */
typedef struct {
  int master_dark_includes_bias;
  float dark_scale;
  float flat_floor;
  float pedestal;
} gg_calib_params_t;

/* Standalone calibrate (replaces module `calibrate_tile_f32`,
 * glass_cuda.py:477-508 → calibration_kernels.cu:5-43).  Any master may be NULL. */
int gg_calibrate_tile_f32(const float* host_light, const float* host_bias, const float* host_dark,
                          const float* host_flat, int64_t n, const gg_calib_params_t* params,
                          float* host_out);

/* ---- resident stack ------------------------------------------------------ */
typedef struct gg_stack gg_stack;

typedef struct {
  int64_t frame_count;
  int64_t height;
  int64_t width;
  int64_t pixels_per_frame;
  int64_t frame_stride;   /* elements between frame slots (padded to 64) */
  int64_t slot_count;     /* frame slots incl. spare warp targets        */
  int64_t loaded_count;
  int64_t bytes_allocated;
  int64_t warp_scratch_bytes;
  int64_t host_pinned_bytes;
  int64_t calibration_lane_count;
  int64_t warp_coverage_frame_count;
  int has_bias;
  int has_dark;
  int has_flat;
} gg_stack_info_t;

/* Replaces ResidentCalibratedStack(frame_count, height, width)
 * (native_bindings.cpp:2917-2934; glass_cuda.py:2661). */
int gg_stack_create(int64_t frame_count, int64_t height, int64_t width, gg_stack** out);
int gg_stack_destroy(gg_stack* stack);
/* Replaces the read-only properties (native_bindings.cpp:20624-20645). */
int gg_stack_info(const gg_stack* stack, gg_stack_info_t* info);
/* Runs the stack's work on the given cudaStream_t (NULL: the stack's own stream). */
int gg_stack_set_stream(gg_stack* stack, void* cuda_stream);
int gg_stack_synchronize(gg_stack* stack);

/* Replaces set_calibration_masters(bias, dark, flat); NULL clears a master. */
int gg_stack_set_masters(gg_stack* stack, const float* host_bias, const float* host_dark,
                         const float* host_flat);
/* Replaces upload_calibrated_frame(i, frame). */
int gg_stack_upload_frame(gg_stack* stack, int64_t index, const float* host_frame);
/* Replaces download_frame_tile(i, x0, y0, x1, y1) (row-major (y1-y0, x1-x0)). */
int gg_stack_download_frame_tile(gg_stack* stack, int64_t index, int64_t x0, int64_t y0, int64_t x1,
                                 int64_t y1, float* host_out);
/* Replaces download_frames_tile(indices, x0, y0, x1, y1). */
int gg_stack_download_frames_tile(gg_stack* stack, const int64_t* indices, int64_t count, int64_t x0,
                                  int64_t y0, int64_t x1, int64_t y1, float* host_out);

/* Fused uint16 decode + calibrate of `count` frames from host memory
 * (replaces calibrate_frames_fits_u16be_bzero_* native_bindings.cpp:7422-8094 and
 * calibration_kernels.cu:110-153).  host_raw holds count*H*W uint16 samples;
 * big_endian_bzero=1 means FITS BITPIX=16 big-endian bytes with BZERO 32768,
 * 0 means native-endian unsigned values.  Copies overlap the decode kernels. */
int gg_stack_calibrate_u16(gg_stack* stack, const int64_t* indices, int64_t count, const void* host_raw,
                           int big_endian_bzero, const gg_calib_params_t* params);
/* Same with the raw frames already in device memory (count*H*W uint16). */
int gg_stack_calibrate_u16_device(gg_stack* stack, const int64_t* indices, int64_t count,
                                  const void* dev_raw, int big_endian_bzero,
                                  const gg_calib_params_t* params);
/* Staged ingest (no counterpart in the reference, whose resident path reads,
 * uploads and calibrates frame by frame): gg_stack_upload_raw_u16 enqueues
 * the host-to-device copies of `count` frames (host_raw: page-locked,
 * count*H*W uint16 in the order of indices) into a device staging copy of
 * the stack's raw samples (allocated on first use: frames*H*W*2 bytes) on
 * the stack's copy stream and returns at once; gg_stack_calibrate_u16_staged
 * then calibrates any subset of the staged frames on the stack stream, each
 * launch waiting (on the device) only for its own frames' copies.  A caller
 * uploads a whole stack and processes it chunk by chunk while the later
 * chunks are still in flight.  A frame's staged samples may be uploaded
 * again once its calibration has been enqueued. */
int gg_stack_upload_raw_u16(gg_stack* stack, const int64_t* indices, int64_t count, const void* host_raw);
int gg_stack_calibrate_u16_staged(gg_stack* stack, const int64_t* indices, int64_t count, int big_endian_bzero,
                                  const gg_calib_params_t* params);
/* Replaces calibrate_frame(i, light_f32, t_L, t_D, policy) (native_bindings.cpp:5979). */
int gg_stack_calibrate_f32(gg_stack* stack, int64_t index, const float* host_light,
                           const gg_calib_params_t* params);

/* Replaces frame_global_stats(i) (native_bindings.cpp:10569-10640). */
typedef struct {
  double mean;
  double std;
  int64_t valid_pixels;
  int64_t total_pixels;
} gg_frame_stats_t;
int gg_stack_frame_stats(gg_stack* stack, const int64_t* indices, int64_t count, gg_frame_stats_t* out);

/* Frame weights computed on the device into the stack's weight vector
 * (used by gg_stack_integrate_device_weights with dev_weights = NULL).
 * GG_WEIGHTS_SIMPLE_SNR: w = max(|mean|/std, eps) (1/eps when std <= eps, 0
 * without valid pixels) - resident_cuda.py:1948-1956 with the statistics of
 * frame_global_stats, times the prior (a per-frame multiplier such as the
 * registration-agreement weight multiplier, resident_cuda.py:12800-12804);
 * GG_WEIGHTS_PRIOR: w = prior.  A frame whose prior is not finite and
 * positive gets weight 0.  host_prior (frame_count) may be NULL;
 * host_weights_out (frame_count) may be NULL to stay asynchronous. */
#define GG_WEIGHTS_PRIOR 0
#define GG_WEIGHTS_SIMPLE_SNR 1
int gg_stack_compute_weights(gg_stack* stack, int mode, const float* host_prior, float eps,
                             float* host_weights_out);

/* Frame statistics (same results as gg_stack_frame_stats) for callers that
 * cannot allocate device memory: plugins whose host application owns every
 * device allocation, real-time loops that forbid allocation after start-up.
 * No counterpart in the reference.  It allocates nothing: the reduction
 * scratch is a fixed 193.5 KiB __device__ array that every GPU loading this
 * library reserves until exit.  `frame_count` frames of `pixels` float32
 * samples start `frame_stride` elements apart at dev_frames (device memory of
 * the stream's device).  At most 64 frames per call (larger counts are
 * rejected with GG_ERR_INVALID_ARGUMENT).  The first call on a device
 * resolves and caches the scratch address; after a device / primary-context
 * reset that address is stale and the entry point must not be called again.
 * Calls share the scratch, so calls that overlap on the GPU race.  Copies the
 * results back and synchronises cuda_stream (NULL: legacy default stream of
 * the current device) before returning, so it cannot run while cuda_stream is
 * being captured: such a call returns GG_ERR_INVALID_ARGUMENT before
 * enqueuing anything and the capture stays valid. */
int gg_frames_stats_f32_noalloc(const float* dev_frames, int64_t frame_count, int64_t pixels,
                                int64_t frame_stride, void* cuda_stream, gg_frame_stats_t* out);

/* ---- integration --------------------------------------------------------- */
typedef struct {
  int rejection;             /* GG_REJECT_*                                  */
  float low_sigma;
  float high_sigma;
  int min_samples;           /* guard, cpu/integration.py:85-99              */
  float max_reject_fraction;
  int count_dtype;           /* GG_COUNT_*                                   */
  int linear_fit_iterations; /* GG_REJECT_LINEAR_FIT only                    */
} gg_integrate_params_t;

/* Rejection + weighted integration of all frames into the stack's six output
 * maps (master f32, weight f32, coverage, low, high count maps, DQ int16).
 * Replaces integrate_mean / integrate_sigma_clip /
 * integrate_hardened_winsorized_sigma (native_bindings.cpp:13227, 13395-14337;
 * integration_kernels.cu:1610-1638, 1743-1902, 2292-2836) with the CPU
 * semantics of cpu/integration.py:36-118.  host_weights may be NULL (unit).
 * Asynchronous: results stay on the device until gg_stack_download_maps. */
int gg_stack_integrate(gg_stack* stack, const float* host_weights, const gg_integrate_params_t* params);
/* Same with the weights already on the device (float32[frame_count]); NULL
 * uses the weights of the last gg_stack_compute_weights. */
int gg_stack_integrate_device_weights(gg_stack* stack, const void* dev_weights,
                                      const gg_integrate_params_t* params);
/* Fused warp + integration: the maps of integrating every frame warped
 * through its forward matrix (float64 row-major 3x3 per frame, moving ->
 * reference; invalid samples excluded) without writing warped frames, plus
 * the geometric coverage (frames with a valid sample per pixel).  Replaces
 * integrate_matrix_warped_{mean,sigma_clip} (glass_cuda.py:5142-5287;
 * integration_kernels.cu:3840-4123).  interpolation GG_INTERP_BILINEAR or
 * GG_INTERP_LANCZOS3; rejection NONE, SIGMA_CLIP or WINSORIZED; at most 512
 * frames (above 32 one warp per pixel over a sampled tile).  host_weights
 * may be NULL (unit).  Asynchronous. */
int gg_stack_integrate_warped(gg_stack* stack, const double* host_matrices, int interpolation,
                              float clamping_threshold, const float* host_weights,
                              const gg_integrate_params_t* params);
/* Geometric coverage (float32 H*W) of the last fused warp-integration. */
int gg_stack_download_fused_coverage(gg_stack* stack, float* host_out);
/* Tile-local weighted integration (integrate_tile_local_mean / _sigma_clip,
 * native_bindings.cpp:12998-13210, 14337-14630; integration_kernels.cu:
 * 1658-1711, 3622-3796).  mode 0 mean, 1 sigma clip, 2 winsorized sigma
 * clip; host_weights may be NULL (1); host_target_mask: frame_count bytes
 * (at least one set); host_tile_extents: tile_count x (x0, y0, x1, y1)
 * half-open, inside the image, not overlapping; multipliers finite >= 0.
 * At most 128 frames and 2048 tiles.  Maps as float32 counts
 * (gg_stack_download_maps with GG_COUNT_F32). */
int gg_stack_integrate_tile_local(gg_stack* stack, int mode, const float* host_weights,
                                  const uint8_t* host_target_mask, const int32_t* host_tile_extents,
                                  const float* host_multipliers, int32_t tile_count, float low_sigma,
                                  float high_sigma);
/* Several resident stacks (same device, each at most 32 frames; frame
 * counts and shapes may differ) integrated in one launch of the column
 * kernel, each with the device weights of its last gg_stack_compute_weights
 * and the same rejection parameters; the maps land in each stack as after
 * gg_stack_integrate_device_weights.  Enqueued on the first stack's stream,
 * ordered after and before the other stacks' streams.  No reference
 * counterpart (the reference integrates one group at a time). */
int gg_stacks_integrate_batch(gg_stack* const* stacks, int32_t count, const gg_integrate_params_t* params);
/* gg_stack_integrate_warped with the weights of the last
 * gg_stack_compute_weights (left on the device; no host round trip). */
int gg_stack_integrate_warped_device_weights(gg_stack* stack, const double* host_matrices, int interpolation,
                                             float clamping_threshold, const gg_integrate_params_t* params);

/* CUDA graph of the resident step with fixed matrices (no reference
 * counterpart; the reference launches every kernel from the host):
 * calibrate all frames from uint16 frames already on the device (dev_raw,
 * frame-major, H*W each, read at every replay) -> frame weights (weighting =
 * GG_WEIGHTS_PRIOR (unit) or GG_WEIGHTS_SIMPLE_SNR, on the device) -> fused
 * warp + rejection + integration through host_matrices (as
 * gg_stack_integrate_warped; at most 512 frames).  Capture runs the sequence
 * once eagerly first.  gg_stack_graph_launch replays it on the stack's
 * stream (asynchronous; maps as after gg_stack_integrate_warped). */
int gg_stack_graph_capture_step(gg_stack* stack, const void* dev_raw, const double* host_matrices, int interpolation,
                                float clamping_threshold, int weighting, const gg_calib_params_t* calib,
                                const gg_integrate_params_t* params);
int gg_stack_graph_launch(gg_stack* stack);

/* ---- local normalisation (resident grid_mean_std / global_mean_std) -------
 * Replaces frame_pair_grid_stats[_batch], apply_grid_normalization_frame[s]
 * and apply_global_normalization_frame (native_bindings.cpp:10645-11200;
 * resident_cuda.py:12902-13060).  Tiles of tile_h x tile_w pixels from the
 * top-left corner, rows = ceil(H / tile_h), cols = ceil(W / tile_w).
 * gg_stack_pair_grid_stats: per source frame and tile, over the pixels finite
 * in both frames, float32 mean / std of source and reference (float64 sums,
 * std = sqrt(max(sum2/n - mean^2, 0))) and the pixel count; outputs are
 * count x rows x cols (any may be NULL). */
int gg_stack_pair_grid_stats(gg_stack* stack, int64_t reference_index, const int64_t* sources, int64_t count,
                             int32_t tile_h, int32_t tile_w, float* host_source_mean, float* host_source_std,
                             float* host_reference_mean, float* host_reference_std, uint64_t* host_valid);
/* In place v * scale + offset (float32 multiply then add) with the tile's
 * coefficients, count x grid_rows x grid_cols; pixels past the grid use its
 * last row / column. */
int gg_stack_apply_grid_normalization(gg_stack* stack, const int64_t* indices, int64_t count,
                                      const float* host_scales, const float* host_offsets, int32_t grid_rows,
                                      int32_t grid_cols, int32_t tile_h, int32_t tile_w);
/* The resident sequence on the device: statistics, coefficients (empty tile
 * 1 / 0; std <= eps: 1 / ref_mean - src_mean; else ref_std / src_std,
 * ref_mean - src_mean * scale in float32) and the in-place apply for every
 * source frame (not the reference); update_weights = 1 zeroes the device
 * frame weight of a source without any paired finite pixel.  Asynchronous
 * unless host_scales / host_offsets (count x rows x cols) are requested. */
int gg_stack_local_normalize_grid(gg_stack* stack, int64_t reference_index, const int64_t* sources, int64_t count,
                                  int32_t tile_h, int32_t tile_w, double eps, int update_weights, float* host_scales,
                                  float* host_offsets);
int gg_stack_apply_global_normalization(gg_stack* stack, int64_t index, float scale, float offset);

/* Launch-shape autotuner (no reference counterpart).  Kernels with
 * equivalent launch shapes (the fused warp-integration's pixel tile, the
 * alignment-metric kernel's CTA bands) time their candidates with CUDA
 * events on the first eager call for a problem shape and keep the fastest;
 * calls during stream capture use the kept or default choice.  On by
 * default (GG_AUTOTUNE=0 in the environment starts it off). */
int gg_autotune_set_enabled(int enabled);
int gg_autotune_clear(void);
int gg_autotune_count(int32_t* out);
/* Entry `index`: kernel family, shape key and chosen candidate (NUL-
 * terminated, truncated to the buffer lengths), its time per launch in ms
 * and the number of candidates. */
int gg_autotune_entry(int32_t index, char* kernel, size_t kernel_len, char* shape, size_t shape_len, char* choice,
                      size_t choice_len, float* best_ms, int32_t* candidates);
int gg_stack_graph_kernel_count(gg_stack* stack, int* out);
int gg_stack_graph_destroy(gg_stack* stack);

/* Several stacks in one CUDA graph (batched uneven stacks; no counterpart in
 * the reference).  Each step names a stack, its uint16 frames in device
 * memory (frame_count frames, frame-major), its forward matrices (moving ->
 * reference, frame_count row-major 3x3 float64; identity matrices are not
 * warped), interpolation, weighting, calibration and integration parameters.
 * The capture runs every step once eagerly (buffers, autotuner), then records
 * calibrate -> weights -> warp -> rejection + integration of every stack, in
 * order, on cuda_stream (NULL: the first stack's stream); a launch replays
 * them all.  The graph owns the warp descriptors; it uses each stack's
 * frames, weights and maps, which later calls may read or overwrite between
 * replays.  Destroy the graph before its stacks. */
typedef struct gg_stacks_graph gg_stacks_graph;
typedef struct {
  gg_stack* stack;
  const void* dev_raw;
  const double* host_matrices;
  int32_t interpolation;        /* GG_INTERP_BILINEAR or GG_INTERP_LANCZOS3 */
  float clamping_threshold;     /* < 0: no clamp */
  int32_t weighting;            /* GG_WEIGHTS_PRIOR (unit) or GG_WEIGHTS_SIMPLE_SNR */
  gg_calib_params_t calib;
  gg_integrate_params_t integrate;
} gg_stack_step_t;
int gg_stacks_graph_capture(const gg_stack_step_t* steps, int32_t count, void* cuda_stream, gg_stacks_graph** out);
int gg_stacks_graph_launch(gg_stacks_graph* graph);
int gg_stacks_graph_kernel_count(gg_stacks_graph* graph, int32_t* out);
int gg_stacks_graph_destroy(gg_stacks_graph* graph);
/* Downloads the maps of the last integration; any pointer may be NULL.  Count
 * maps are float32 or uint16 per the count_dtype used. */
int gg_stack_download_maps(gg_stack* stack, float* host_master, float* host_weight, void* host_coverage,
                           void* host_low, void* host_high, int16_t* host_dq);

/* Device pointers of the stack's buffers, for zero-copy consumers. */
typedef struct {
  void* slots;          /* float32 frame slots                                   */
  void* slot_of_frame;  /* int32[frame_count] device table frame -> slot          */
  void* master;
  void* weight;
  void* coverage;
  void* low;
  void* high;
  void* dq;
  void* warp_coverage;  /* float32 coverage accumulator                           */
} gg_stack_device_ptrs_t;
int gg_stack_device_ptrs(gg_stack* stack, gg_stack_device_ptrs_t* out);
/* Device address of loaded frame `index` (H*W float32, row-major) as of the
 * moment of the call: synchronises the stack's stream; a later warp of that
 * frame moves it to another slot.  No reference counterpart (views of
 * resident frames for the differentiable warp). */
int gg_stack_frame_device_ptr(gg_stack* stack, int64_t index, float** out);
/* The device frame weights (last gg_stack_compute_weights, as updated by
 * gg_stack_local_normalize_grid), frame_count float32; synchronises. */
int gg_stack_download_weights(gg_stack* stack, float* host_out);

/* ---- star detection ------------------------------------------------------ */
/* Parameters of detect_stars (cpu/star_detect.py:121-132).  background /
 * noise: NaN estimates them (median / 1.4826*MAD of the finite pixels). */
typedef struct {
  float threshold_sigma;   /* 5.0   */
  int max_stars;           /* 500, at most 4096 */
  int window_radius;       /* 4     */
  float min_separation_px; /* 2.0   */
  float background;        /* NaN   */
  float noise;             /* NaN   */
  /* Registration catalog (the first 80 detected stars, brightest first, as
   * cpu/registration.py:37-39 takes them) optionally skips stars whose
   * fwhm < catalog_min_fwhm or eccentricity > catalog_max_eccentricity
   * (undefined values fail an active test).  0 and 1 (or more) switch the
   * tests off, which is the reference's behaviour.  No reference counterpart:
   * a shape filter against cosmic-ray hits as bright as stars. */
  float catalog_min_fwhm;
  float catalog_max_eccentricity;
  /* Background mesh (no reference counterpart; 0 = the reference's global
   * median / MAD).  mesh_cell in [8, 64]: the frame is cut into cells of
   * mesh_cell x mesh_cell pixels from the top-left corner (edge cells
   * smaller); each cell's finite pixels give a float64 median and noise
   * 1.4826 * MAD (1 when the MAD is 0; NaN for a cell without finite
   * pixels); background and noise at a pixel are the bilinear interpolation
   * between cell centres (clamped at the border), the threshold there is
   * background + k * max(noise, 1e-6) compared in float64, and each star is
   * measured against the interpolated background and noise at its peak.
   * background / noise must then be NaN. */
  int32_t mesh_cell;
} gg_star_params_t;

/* One star (cpu/star_detect.py:8-18); fwhm / eccentricity NaN when undefined. */
typedef struct {
  double x;
  double y;
  double flux;
  double peak;
  double fwhm;
  double eccentricity;
  double snr;
  double sharpness;
  int32_t npix;
  int32_t pad;
} gg_star_t;

typedef struct {
  float median;
  float mad;
  double noise;
  double threshold;
  int64_t candidates;
  int64_t valid_pixels;
} gg_star_frame_info_t;

/* detect_stars for `count` resident frames (star_detect.py:121-168; reference
 * device path: star_detect_kernels.cu, native_bindings.cpp:12123).  host_stars
 * receives count * max_stars records (brightest first), host_counts the stars
 * per frame; host_info (may be NULL) the background statistics.  The
 * catalogs also stay on the device for registration. */
int gg_stack_detect_stars(gg_stack* stack, const int64_t* indices, int64_t count, const gg_star_params_t* params,
                          gg_star_t* host_stars, int32_t* host_counts, gg_star_frame_info_t* host_info);

/* ---- grid star catalogs ---------------------------------------------------- */
typedef struct {
  float threshold;            /* candidates are interior local maxima > threshold */
  int grid_cols;              /* cells: x in [c*W/cols, (c+1)*W/cols), same for y */
  int grid_rows;
  int candidates_per_cell;    /* best K per cell (value desc, y asc, x asc), <= 3072 */
  int max_output_candidates;  /* kept after the separation scan, <= 8192          */
  float min_separation_px;
  int centroid_radius;        /* 0: no centroid; window radius (clamped to 1..8) */
  int centroid_background;    /* 0: window median, 1: frame global mean           */
} gg_grid_catalog_params_t;

/* Deterministic grid catalogs of `count` resident frames: per-cell top-K local
 * maxima, merged in value order, greedy minimum-separation scan, optional
 * windowed centroid.  Replaces ResidentCalibratedStack.
 * star_grid_top_nms_candidates_batch_deterministic_centroid and its siblings
 * (native_bindings.cpp:12622-12645 over the batch driver :12211-12616; kernels
 * star_detect_kernels.cu:40-101, 317-742).  host_catalog receives five planes
 * of count * max_output_candidates float32 each: x, y (after the centroid),
 * value, x and y before the centroid; host_status (may be NULL) count *
 * max_output_candidates centroid flags (1 = moved); host_counts count pairs
 * (candidates in the frame, kept).  Synchronises the stack's stream. */
int gg_stack_star_grid_catalog(gg_stack* stack, const int64_t* indices, int64_t count,
                               const gg_grid_catalog_params_t* params, float* host_catalog, uint8_t* host_status,
                               int32_t* host_counts);

/* ---- raw FITS read queue (RawFitsReadQueue, native_bindings.cpp:2605-2915,
 * 20417-20429) ---------------------------------------------------------------
 * Host worker threads read [data_offset, data_offset + byte_count) of a file
 * into host_out (normally pinned memory for the u16 decode + calibration
 * entry points); completions come back in finishing order.  A failed read
 * is reported by gg_read_queue_wait as GG_ERR_RUNTIME (the completion is
 * still filled and consumed). */
typedef struct gg_read_queue gg_read_queue;
typedef struct {
  uint64_t frame_index;
  uint64_t bytes_read;
  double file_open_s;
  double file_read_s;
  double total_s;
} gg_read_completion_t;
typedef struct {
  uint64_t worker_count;
  uint64_t submitted_count;
  uint64_t completed_count;
  uint64_t queued_count;
  uint64_t active_count;
  uint64_t ready_count;
  uint64_t requested_bytes;
  int32_t closed;
  int32_t pad;
} gg_read_queue_stats_t;
int gg_read_queue_create(int32_t workers, gg_read_queue** out);
int gg_read_queue_submit(gg_read_queue* queue, uint64_t frame_index, const char* path, uint64_t data_offset,
                         uint64_t byte_count, void* host_out, uint64_t* pending_after);
/* timeout_s < 0 waits without limit; *has_completion = 0 on time-out or
 * when the queue is closed and drained. */
int gg_read_queue_wait(gg_read_queue* queue, double timeout_s, gg_read_completion_t* out, int32_t* has_completion);
int gg_read_queue_stats(gg_read_queue* queue, gg_read_queue_stats_t* out);
int gg_read_queue_close(gg_read_queue* queue);
int gg_read_queue_destroy(gg_read_queue* queue);

/* ---- source DQ: isolated cosmetic defects ----------------------------------
 * Replaces apply_isolated_cosmetic_threshold_mask_frame(s) and the
 * star-protected variant (resident_source_dq.py:825-1740; detection rules of
 * cpu/cosmetic.py:97-307): per frame, with the frame's robust median / sigma
 * (as detect_stars), isolated hot / cold pixels without enough same-side
 * neighbour support; star_protection = 1 keeps those within
 * star_protection_radius_px of catalog stars (threshold star_threshold_sigma,
 * 500 stars, npix >= star_min_pixels, sharpness <= star_max_sharpness).
 * apply = 1 sets the defects to NaN (no replacement); 0 only counts. */
typedef struct {
  float hot_sigma;                 /* 8    */
  float cold_sigma;                /* 8    */
  float structure_sigma;           /* 1.5  */
  int32_t min_neighbor_support;    /* 2    */
  int32_t star_protection;         /* 0/1  */
  float star_threshold_sigma;      /* 5    */
  float star_protection_radius_px; /* 3    */
  int32_t star_min_pixels;         /* 3    */
  float star_max_sharpness;        /* 0.95 */
  int32_t apply;                   /* 1    */
} gg_cosmetic_params_t;

typedef struct {
  int64_t hot_pixels;
  int64_t cold_pixels;
  int64_t candidate_hot_pixels;
  int64_t candidate_cold_pixels;
  int64_t star_protected_hot_pixels;
  int64_t star_protected_cold_pixels;
  double median;
  double sigma;
  int32_t star_count;
  int32_t pad;
} gg_cosmetic_result_t;

int gg_stack_cosmetic_mask(gg_stack* stack, const int64_t* indices, int64_t count,
                           const gg_cosmetic_params_t* params, gg_cosmetic_result_t* host_out);
/* Replaces apply_cosmetic_threshold_mask_frame(s) and
 * count_cosmetic_threshold_mask_frame(s) (native_bindings.cpp:3243-3400,
 * 4307-4620; kernels integration_kernels.cu:181-330): for frame indices[k]
 * a sample is non-finite, hot (> high_thresholds[k]) or cold
 * (< low_thresholds[k]), tested in that order; apply = 1 sets all three to
 * NaN (and counts the hot and cold ones in the frame's non-finite counter),
 * 0 only counts.  Thresholds may be infinite, not NaN, low <= high; at most
 * 65535 distinct frames.  host_counts (may be NULL) receives [count][3] =
 * hot, cold, non-finite.  Synchronises. */
int gg_stack_cosmetic_threshold(gg_stack* stack, const int64_t* indices, int64_t count, const float* low_thresholds,
                                const float* high_thresholds, int32_t apply, int64_t* host_counts);
/* apply_invalid_mask (integration_kernels.cu:159-179): frame `index` samples
 * whose host_mask byte (H*W) is non-zero become NaN; host_invalid_samples
 * (may be NULL) receives the number of flagged samples.  Synchronises. */
int gg_stack_apply_invalid_mask(gg_stack* stack, int64_t index, const uint8_t* host_mask,
                                int64_t* host_invalid_samples);

/* ---- registration (triangle asterisms) ----------------------------------- */
/* Point lists are (x, y) float64 pairs, brightest star first.  Catalogs hold
 * at most 80 stars. */
#define GG_TRANSFORM_TRANSLATION 0
#define GG_TRANSFORM_SIMILARITY 1
#define GG_TRANSFORM_AFFINE 2

/* Parameters of estimate_triangle_asterism_transform
 * (cpu/registration.py:361-373). */
typedef struct {
  int32_t transform_model;  /* GG_TRANSFORM_SIMILARITY (Procrustes fits) or GG_TRANSFORM_AFFINE
                               (least-squares affine fits, cpu/registration.py:106-119) */
  int32_t min_inliers;      /* 6 */
  double tolerance_px;      /* 3.0 */
  double descriptor_radius; /* 0.1 */
  int32_t max_stars;        /* 80, at most 80 */
  int32_t neighbors;        /* 5, at most 6 (values below 3 mean 3) */
  int32_t max_descriptors;  /* 1200 */
  int32_t max_candidates;   /* 1500, at most 2048 */
} gg_register_params_t;

/* StarRegistration (cpu/registration.py:11-20) without the warning strings. */
typedef struct {
  double matrix[9];         /* row-major 3x3, moving -> reference pixels */
  double rms_px;            /* NaN without pairs */
  int64_t best_candidate;   /* winning candidate (2 * match + orientation), -1 if none */
  int32_t inliers;          /* = matched_stars */
  int32_t status;           /* 1 "ok", 0 "failed" */
  int32_t descriptors_reference;
  int32_t descriptors_moving;
  int32_t matches;          /* descriptor matches scored */
  int32_t pad;
} gg_registration_t;

/* Replaces module triangle_asterism_descriptors_f32 (glass_cuda.py:1835-1902;
 * cpu/registration.py:273-303): local triangle descriptors of one catalog,
 * area-descending.  host_descriptors [count][2], host_indices [count][3] and
 * host_areas [count] may each be NULL; `capacity` rows are available. */
int gg_triangle_descriptors(const double* host_xy, int64_t n, int32_t max_stars, int32_t neighbors,
                            int32_t max_descriptors, double* host_descriptors, int32_t* host_indices,
                            double* host_areas, int64_t capacity, int64_t* count);
/* estimate_triangle_asterism_transform (cpu/registration.py:361-475) of two
 * host catalogs.  host_pairs (may be NULL) receives 80 (moving, reference)
 * index pairs, -1 past the inliers. */
int gg_register_star_lists(const double* host_ref_xy, int64_t n_ref, const double* host_mov_xy, int64_t n_mov,
                           const gg_register_params_t* params, gg_registration_t* host_out, int32_t* host_pairs);
/* Replaces module estimate_similarity_from_triangle_descriptors_f32
 * (glass_cuda.py:2054-2140): every descriptor pair within the radius, both
 * reference orientations, best by (pairs, rms), no refit. */
int gg_similarity_from_descriptors(const double* host_ref_xy, int64_t n_ref, const double* host_mov_xy,
                                   int64_t n_mov, const float* host_ref_desc, const int32_t* host_ref_idx,
                                   int64_t n_ref_desc, const float* host_mov_desc, const int32_t* host_mov_idx,
                                   int64_t n_mov_desc, double tolerance_px, double descriptor_radius,
                                   gg_registration_t* host_out, int32_t* host_pairs);
/* Registers resident frames to a resident reference frame from the catalogs
 * of their last gg_stack_detect_stars (the reference's resident triangle path,
 * resident_cuda.py:10790-11420).  host_out receives `count` results.
 * Synchronises the stack stream. */
int gg_stack_register_frames(gg_stack* stack, int64_t reference_index, const int64_t* indices, int64_t count,
                             const gg_register_params_t* params, gg_registration_t* host_out);

/* ---- alignment metrics and sub-pixel refinement ---------------------------- */
/* matrix_alignment_metrics_f32 (glass_cuda.py:706-768): bilinear warp of the
 * moving frame (fill 0) compared with the reference on every
 * sample_stride-th row and column. */
typedef struct {
  int64_t valid_pixels;
  int64_t sampled_pixels;
  int32_t sample_stride;
  int32_t pad;
  double rms;           /* NaN without valid samples */
  double mean_abs_diff; /* NaN without valid samples */
  double ncc;           /* NaN with <= 1 valid sample or a zero denominator */
} gg_alignment_metrics_t;

/* refine_matrix_translation_with_metrics_f32 (glass_cuda.py:771-900). */
typedef struct {
  double search_radius_px; /* 1.0    */
  double coarse_step_px;   /* 0.25   */
  double fine_radius_px;   /* 0.25   */
  double fine_step_px;     /* 0.0625 */
  int32_t coarse_sample_stride; /* 4 */
  int32_t final_sample_stride;  /* 1 */
} gg_refine_params_t;

typedef struct {
  double matrix[9];      /* refined matrix (float32 values), row-major */
  double dx_correction;  /* float32 value */
  double dy_correction;
  gg_alignment_metrics_t metrics; /* of the refined matrix at the last stride */
  int32_t coarse_candidates;
  int32_t fine_candidates;
} gg_refine_result_t;

/* estimate_translation_subpixel_ncc_f32 (glass_cuda.py:1131-1245). */
typedef struct {
  double dx;
  double dy;
  double score; /* best NCC, -inf when no candidate scored */
  int64_t candidate_count;
} gg_translation_ncc_t;

/* Metrics of one forward matrix (moving -> reference, float64 row-major 3x3)
 * per moving frame against a resident reference frame.  Replaces module
 * matrix_alignment_metrics_f32 (and its kernel warp_kernels.cu:1198-1323). */
int gg_stack_alignment_metrics(gg_stack* stack, int64_t reference_index, const int64_t* indices, int64_t count,
                               const double* host_matrices, int32_t sample_stride, gg_alignment_metrics_t* host_out);
/* Coarse-to-fine translation refinement of each moving frame's matrix
 * against the reference frame.  Replaces
 * refine_matrix_translation_candidates_batch_to_reference
 * (native_bindings.cpp:10186-10417) and module
 * refine_matrix_translation_with_metrics_f32 (glass_cuda.py:771-900). */
int gg_stack_refine_translation(gg_stack* stack, int64_t reference_index, const int64_t* indices, int64_t count,
                                const double* host_matrices, const gg_refine_params_t* params,
                                gg_refine_result_t* host_out);
/* Sub-pixel translation by NCC over a (2r+1)^2 grid of translations around
 * (center_dx, center_dy).  Replaces estimate_translation_subpixel_ncc_f32
 * (glass_cuda.py:1175-1245; registration_kernels.cu:127-233). */
int gg_stack_translation_ncc(gg_stack* stack, int64_t reference_index, int64_t moving_index, double center_dx,
                             double center_dy, int32_t radius_steps, double step, int32_t sample_stride,
                             gg_translation_ncc_t* host_out);

/* ---- warps --------------------------------------------------------------- */
/* Warps `count` resident frames in place through their forward matrices
 * (float64 row-major 3x3, moving -> reference; the kernel samples the source
 * at the float64 inverse).  Replaces apply_matrix_{bilinear,lanczos3}_frame(s)
 * (native_bindings.cpp:8900-9924, 9704; warp_kernels.cu:206-777).  Invalid
 * output pixels get `fill`; clamping_threshold < 0 disables the Lanczos3
 * overshoot clamp; track_coverage adds 1 to the warp-coverage accumulator for
 * every covered output pixel.  Asynchronous. */
int gg_stack_warp_frames(gg_stack* stack, const int64_t* indices, int64_t count, const double* host_matrices,
                         int interpolation, float fill, float clamping_threshold, int track_coverage);
/* Warp-coverage accumulator: reset_warp_coverage /
 * accumulate_full_warp_coverage_frame / warp_coverage_map. */
int gg_stack_reset_warp_coverage(gg_stack* stack);
int gg_stack_accumulate_full_warp_coverage_frame(gg_stack* stack);
int gg_stack_download_warp_coverage(gg_stack* stack, float* host_out);
/* 1 when the stack's frames are staged by TMA (width % 4 == 0). */
int gg_stack_tma_enabled(gg_stack* stack, int* enabled);
/* Standalone warp of one host image (module warp_matrix_{bilinear,lanczos3}_f32,
 * glass_cuda.py:595-706).  host_coverage (H*W float32) may be NULL. */
int gg_warp_matrix_f32(const float* host_in, int64_t height, int64_t width, const double* host_matrix,
                       int interpolation, float fill, float clamping_threshold, float* host_out,
                       float* host_coverage);

/* Replaces module `resident_dq_map_count_maps_i16` (glass_cuda.py:270-290;
 * resident_cuda.py:3110-3297): DQ bits from the output maps.  Any count map
 * pointer may be NULL; geometric may be NULL. */
int gg_dq_map_i16(const float* host_master, const float* host_weight, const float* host_coverage,
                  const float* host_low, const float* host_high, const float* host_geometric,
                  int64_t n, int64_t active_frame_count, int16_t* host_dq);

/* ---- differentiable affine warp (no reference counterpart: the adjoint
 * behind gradient-based registration refinement; forward semantics of
 * engine/warp.py:99-152 without the overshoot clamp) -------------------
 * host_theta: 6 float64 parameters of the INVERSE map (output -> source):
 * sx = t0 x + t1 y + t2, sy = t3 x + t4 y + t5.  Device pointers, row-major
 * float32 H x W, enqueued on cuda_stream (NULL: legacy default stream).
 * src_all_finite = 1 promises a source without NaN/Inf (fast Lanczos3 path). */
int gg_warp_affine_f32_device(const float* dev_src, int64_t height, int64_t width, const double* host_theta,
                              int interpolation, float fill, int src_all_finite, float* dev_out,
                              void* cuda_stream);
/* Adjoint of gg_warp_affine_f32_device for the incoming gradient dev_grad_out
 * (H x W float32; zero or non-finite entries are ignored, as are invalid
 * samples).  dev_grad_src (H x W float32, may be NULL) is ACCUMULATED into;
 * dev_grad_theta (6 float64 on the device, may be NULL) is overwritten. */
int gg_warp_affine_backward_f32_device(const float* dev_src, int64_t height, int64_t width, const double* host_theta,
                                       int interpolation, const float* dev_grad_out, float* dev_grad_src,
                                       double* dev_grad_theta, void* cuda_stream);

/* ---- gradient (Gauss-Newton) registration refinement on resident frames
 * (no reference counterpart: replaces the translation grid search of
 * refine_matrix_translation_candidates_batch_to_reference with the warp
 * adjoint's position derivatives).  Minimises
 * sum m_p (O_p(theta) - alpha a_p - beta)^2 over a sample grid of the
 * reference, O the moving frame sampled through the inverse affine theta,
 * m_p dropping invalid samples, residuals above
 * clip_sigma * sigma + mask_shift_px * min(|alpha| |grad a|, |grad O|) and
 * samples with |grad O| > 2 |alpha| |grad a| + 3 sigma (sigma = 1.4826 *
 * median |r| of the previous pass). */
typedef struct {
  int32_t transform_model; /* GG_TRANSFORM_TRANSLATION, _SIMILARITY or _AFFINE */
  int32_t interpolation;   /* GG_INTERP_BILINEAR or GG_INTERP_LANCZOS3 */
  int32_t sample_stride;   /* every stride-th column of the reference, 1..64 */
  int32_t row_stride;      /* every row_stride-th row, 0..4096; 0: sample_stride (a square grid) */
  int32_t stats_passes;    /* photometric offset / noise passes first, on a grid twice as coarse
                              (both steps; the row step alone when row_stride > 0), 1..16 */
  int32_t iterations;      /* Gauss-Newton steps, 1..100 */
  int32_t min_samples;     /* fewer kept samples fail the frame (>= 16) */
  int32_t reserved;        /* 0 */
  float clip_sigma;
  float mask_shift_px;
  double tolerance_px;     /* converged when a step moves no image corner farther */
  double max_step_px;      /* longer steps are scaled down to this */
} gg_gradient_refine_params_t;

typedef struct {
  double matrix[9];        /* refined moving -> reference (the input matrix on failure) */
  double alpha, beta;      /* photometric match: moving ~ alpha * reference + beta */
  double sigma;            /* residual scale used by the mask in the last step */
  double rms;              /* residual RMS over the kept samples, last pass */
  double last_step_px;
  int64_t samples;         /* kept samples, last pass */
  int32_t iterations;
  int32_t status;          /* 1 converged, 2 iteration cap, -1 too few samples, -2 singular system */
} gg_gradient_refine_result_t;

/* host_matrices: count x 9 affine moving -> reference starting matrices. */
int gg_stack_refine_gradient(gg_stack* stack, int64_t reference_index, const int64_t* moving, int64_t count,
                             const double* host_matrices, const gg_gradient_refine_params_t* params,
                             gg_gradient_refine_result_t* host_out);
/* One accumulation pass at given inverse parameters (count x 6) and
 * photometric state (count x 3: alpha, beta, sigma; sigma = +inf keeps every
 * valid sample): host_sums (count x 48) receives per job the upper triangle
 * of J^T J (36, row-major over (t0..t5, alpha, beta) in centred units
 * ((x - (W-1)/2) * 2 / max(W,H), likewise y)), J^T r (8), sum r^2, the kept
 * sample count and two zeros. */
int gg_stack_gradient_normal_equations(gg_stack* stack, int64_t reference_index, const int64_t* moving,
                                       int64_t count, const double* host_theta, const double* host_photometric,
                                       const gg_gradient_refine_params_t* params, double* host_sums);

#ifdef __cplusplus
}
#endif

#endif /* GLASS_GB300_H */
