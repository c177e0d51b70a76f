// Internal definition of the resident stack (opaque `gg_stack` in the C ABI).
//
// HBM layout
// ----------
// The stack owns `slot_count = frame_count + spare_count` frame slots in one
// allocation.  Each slot holds one float32 frame of H*W pixels, padded to a
// stride of 64 elements (256 B) so that every frame starts on a TMA- and
// vector-aligned boundary.  A device table `slot_of_frame[frame]` maps a
// logical frame to its slot.  Warps write each output frame into a spare slot
// and then swap the table entries, so a warp moves 8 B per pixel (read + write)
// instead of the 16 B that warp-to-scratch-then-copy-back costs.  The device
// table is the single source of truth; every kernel indexes frames through it
// and the host reads it back only for downloads.
#pragma once

#include <cuda.h>

#include <vector>

#include "common.cuh"

struct gg_stack {
  int device = 0;
  int64_t frames = 0;
  int64_t height = 0;
  int64_t width = 0;
  int64_t pixels = 0;
  int64_t stride = 0;   // elements between slots
  int64_t spares = 0;   // spare slots for warp outputs
  int64_t slots = 0;    // frames + spares

  float* d_slots = nullptr;
  int* d_slot_of_frame = nullptr;  // [frames]
  int* d_spare_slot = nullptr;     // [spares]

  std::vector<unsigned char> loaded;
  int64_t loaded_count = 0;

  // Per-frame count of non-finite samples, maintained by every kernel that
  // writes a frame.  The integrator reads it to pick NumPy's all-valid
  // statistics formulas (engine/rejection.py:39-44) without another pass.
  unsigned* d_frame_nonfinite = nullptr;

  // Calibration masters (float32, P each).
  float* d_bias = nullptr;
  float* d_dark = nullptr;
  float* d_flat = nullptr;
  bool has_bias = false;
  bool has_dark = false;
  bool has_flat = false;

  // Output maps of the last integration.
  float* d_master = nullptr;
  float* d_weight = nullptr;
  void* d_coverage = nullptr;  // 4 B/px capacity: float32 or uint16
  void* d_low = nullptr;
  void* d_high = nullptr;
  int16_t* d_dq = nullptr;
  int last_count_dtype = -1;

  // Warp coverage accumulator (geometric coverage), float32 per pixel.
  float* d_warp_coverage = nullptr;
  int64_t warp_coverage_frames = 0;

  // Raw uint16 staging lanes for calibration from host memory.
  static constexpr int kLanes = 2;
  static constexpr int kLaneFrames = 4;
  uint16_t* d_raw_lane[kLanes] = {nullptr, nullptr};
  void* h_pinned_lane[kLanes] = {nullptr, nullptr};
  size_t lane_bytes = 0;
  int next_lane = 0;
  cudaEvent_t lane_free[kLanes] = {nullptr, nullptr};
  cudaEvent_t lane_ready[kLanes] = {nullptr, nullptr};

  // Small device/pinned scratch (weights upload, reduction partials).
  float* d_weights = nullptr;          // [frames]
  float* h_weights_pinned = nullptr;   // [frames]
  double* d_partials = nullptr;        // reduction partials
  double* h_partials_pinned = nullptr;
  size_t partial_capacity = 0;         // doubles
  int* h_slot_table_pinned = nullptr;  // [frames]

  // Warp batches: per-item descriptors (device + pinned staging) and the TMA
  // descriptor of the slot pool viewed as a [slot][H][W] float32 tensor.
  void* d_warp_items = nullptr;
  void* h_warp_items = nullptr;
  int64_t warp_item_capacity = 0;
  cudaEvent_t warp_items_free = nullptr;
  CUtensorMap slot_tmap{};
  bool has_slot_tmap = false;

  // Device error word set by kernels whose bounded waits run out.
  int* d_error = nullptr;

  // Lazily created per-feature scratch (star detection, registration), freed
  // with the stack through their own release hooks.
  void* star_scratch = nullptr;
  void (*star_scratch_free)(void*) = nullptr;
  void* reg_scratch = nullptr;
  void (*reg_scratch_free)(void*) = nullptr;
  void* metric_scratch = nullptr;
  void (*metric_scratch_free)(void*) = nullptr;
  void* gn_scratch = nullptr;
  void (*gn_scratch_free)(void*) = nullptr;
  void* step_graph = nullptr;  // captured resident step (integrate.cu)
  void (*step_graph_free)(void*) = nullptr;
  void* ln_scratch = nullptr;  // local normalisation (localnorm.cu)
  void (*ln_scratch_free)(void*) = nullptr;
  void* raw_stage = nullptr;  // staged raw frames for pipelined ingest (calibrate.cu)
  void (*raw_stage_free)(void*) = nullptr;

  // Fused warp-integration: per-frame inverse matrices, per-frame
  // non-finite sample counts of the virtual warped stack and the geometric
  // coverage map of the last fused integration.
  void* d_fused_frames = nullptr;
  unsigned* d_fused_counts = nullptr;
  float* d_fused_geometric = nullptr;
  bool has_fused_geometric = false;

  // Per-frame registration catalogs: the brightest kCatalogPoints star
  // centroids of each frame's last detection (x, y float64) and their count.
  double* d_cat_xy = nullptr;
  int* d_cat_n = nullptr;

  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t copy_stream = nullptr;

  int64_t bytes_allocated = 0;
  int64_t host_pinned_bytes = 0;
};

namespace gg {

// Device helpers used across translation units.
void stack_activate(gg_stack* s);
void stack_require_index(const gg_stack* s, int64_t index);
void stack_require_loaded(const gg_stack* s, int64_t index, const char* what);
void stack_require_all_loaded(const gg_stack* s, const char* what);
void stack_mark_loaded(gg_stack* s, int64_t index);
// Reads the device frame->slot table into `out` (synchronises the stream).
void stack_read_slots(gg_stack* s, std::vector<int>& out);
void stack_ensure_maps(gg_stack* s);
void stack_ensure_partials(gg_stack* s, size_t doubles);
// Raises GG_ERR_TIMEOUT if a kernel reported a bounded wait running out
// (synchronises the stream), then clears the flag.
void stack_check_device_error(gg_stack* s);
// Encodes a TMA tensor map over the slot pool ([slot][H][W] float32).
bool make_slot_tensor_map(gg_stack* s, int box_w, int box_h);
// Registration catalog storage (allocated on first detection).
constexpr int kCatalogPoints = 80;
void ensure_catalog_storage(gg_stack* s);

// Kernel launchers (defined in the per-kernel translation units).
struct CalibLaunch {
  const uint16_t* raw;     // device, frames_in_batch * P samples (nullptr for f32 path)
  const float* light_f32;  // device, P samples (f32 path)
  int big_endian_bzero;
  int nframes;
  int frame[GG_MAX_BATCH_FRAMES];
};
void launch_calibrate(gg_stack* s, const CalibLaunch& job, const gg_calib_params_t& p);
void launch_count_nonfinite(gg_stack* s, int64_t frame);
void launch_frame_stats(gg_stack* s, const int64_t* indices, int64_t count, int blocks_per_frame);
void launch_integrate(gg_stack* s, const float* d_weights, const gg_integrate_params_t& p);

}  // namespace gg
