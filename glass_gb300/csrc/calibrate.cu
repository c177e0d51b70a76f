// Fused uint16 decode + bias/dark/flat calibration into the resident stack.
//
// Semantics follow the CPU oracle cpu/calibration.py:51-76 (which the
// reference CUDA kernels calibration_kernels.cu:5-43 and :110-153 implement):
//   v = light
//   if dark:  v = v - dark * dark_scale ; if !dark_includes_bias and bias: v = v - bias
//   elif bias: v = v - bias
//   if flat:  v = v / max(flat, flat_floor)
//   if pedestal != 0: v = v + pedestal
// Every operation is rounded separately (no FMA), as NumPy does.
//
// GB300 design: one launch calibrates a batch of up to GG_MAX_BATCH_FRAMES
// frames.  Each thread owns 8 consecutive pixels, loads the masters for them
// once (16-byte vector loads) and then streams the batch's frames through
// registers: 16 B of uint16 in and 32 B of float32 out per frame, so the
// masters cost 12 B per pixel per batch instead of per frame.  Raw frames
// arrive over PCIe/C2C on a copy stream into one of two lane buffers while the
// previous lane is being decoded (cudaEvent handshakes).
#include <algorithm>
#include <vector>

#include "stack.cuh"

namespace gg {

struct CalibArgs {
  const uint16_t* raw;     // nframes * P (nullptr -> light_f32)
  const float* light_f32;  // P (single frame)
  const float* bias;
  const float* dark;
  const float* flat;
  float* slots;
  const int* slot_of_frame;
  unsigned* nonfinite;
  int64_t stride;
  int64_t pixels;
  int nframes;
  int frame[GG_MAX_BATCH_FRAMES];
  int big_endian_bzero;
  int has_bias, has_dark, has_flat, dark_includes_bias;
  float dark_scale, flat_floor, pedestal;
};

__device__ __forceinline__ float calibrate_one(float v, float b, float d, float f, const CalibArgs& a) {
  if (a.has_dark) {
    v = __fsub_rn(v, __fmul_rn(d, a.dark_scale));
    if (!a.dark_includes_bias && a.has_bias) v = __fsub_rn(v, b);
  } else if (a.has_bias) {
    v = __fsub_rn(v, b);
  }
  if (a.has_flat) {
    // np.maximum(flat, floor): NaN propagates, anything below the floor is raised.
    v = __fdiv_rn(v, f < a.flat_floor ? a.flat_floor : f);
  }
  if (a.pedestal != 0.0f) v = __fadd_rn(v, a.pedestal);
  return v;
}

__device__ __forceinline__ float decode_u16(uint16_t raw, int big_endian_bzero) {
  if (big_endian_bzero) {
    const unsigned bits = ((static_cast<unsigned>(raw) & 0xffu) << 8) | (static_cast<unsigned>(raw) >> 8);
    return static_cast<float>(bits ^ 0x8000u);
  }
  return static_cast<float>(raw);
}

// Vector path: P % 8 == 0.  Thread t owns pixels [8t, 8t+8).
__global__ void __launch_bounds__(256) calibrate_u16_vec8_kernel(CalibArgs a) {
  const int64_t groups = a.pixels / 8;
  for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < groups;
       g += int64_t(gridDim.x) * blockDim.x) {
    const int64_t p0 = g * 8;
    float b[8], d[8], f[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) b[k] = d[k] = f[k] = 0.0f;
    if (a.has_bias) {
      const float4 u = __ldg(reinterpret_cast<const float4*>(a.bias + p0));
      const float4 v = __ldg(reinterpret_cast<const float4*>(a.bias + p0) + 1);
      b[0] = u.x; b[1] = u.y; b[2] = u.z; b[3] = u.w; b[4] = v.x; b[5] = v.y; b[6] = v.z; b[7] = v.w;
    }
    if (a.has_dark) {
      const float4 u = __ldg(reinterpret_cast<const float4*>(a.dark + p0));
      const float4 v = __ldg(reinterpret_cast<const float4*>(a.dark + p0) + 1);
      d[0] = u.x; d[1] = u.y; d[2] = u.z; d[3] = u.w; d[4] = v.x; d[5] = v.y; d[6] = v.z; d[7] = v.w;
    }
    if (a.has_flat) {
      const float4 u = __ldg(reinterpret_cast<const float4*>(a.flat + p0));
      const float4 v = __ldg(reinterpret_cast<const float4*>(a.flat + p0) + 1);
      f[0] = u.x; f[1] = u.y; f[2] = u.z; f[3] = u.w; f[4] = v.x; f[5] = v.y; f[6] = v.z; f[7] = v.w;
    }
    for (int fi = 0; fi < a.nframes; ++fi) {
      const uint4 r = __ldcs(reinterpret_cast<const uint4*>(a.raw + fi * a.pixels + p0));
      const uint16_t raw[8] = {static_cast<uint16_t>(r.x & 0xffffu), static_cast<uint16_t>(r.x >> 16),
                               static_cast<uint16_t>(r.y & 0xffffu), static_cast<uint16_t>(r.y >> 16),
                               static_cast<uint16_t>(r.z & 0xffffu), static_cast<uint16_t>(r.z >> 16),
                               static_cast<uint16_t>(r.w & 0xffffu), static_cast<uint16_t>(r.w >> 16)};
      float out[8];
      bool bad = false;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        out[k] = calibrate_one(decode_u16(raw[k], a.big_endian_bzero), b[k], d[k], f[k], a);
        bad |= !isfinite(out[k]);
      }
      float* dst = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frame[fi]]) * a.stride + p0;
      __stcs(reinterpret_cast<float4*>(dst), make_float4(out[0], out[1], out[2], out[3]));
      __stcs(reinterpret_cast<float4*>(dst) + 1, make_float4(out[4], out[5], out[6], out[7]));
      if (__any_sync(__activemask(), bad)) {
        int nbad = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) nbad += !isfinite(out[k]);
        if (nbad) atomicAdd(a.nonfinite + a.frame[fi], static_cast<unsigned>(nbad));
      }
    }
  }
}

// Scalar path for any P (odd shapes, float32 lights).
__global__ void __launch_bounds__(256) calibrate_scalar_kernel(CalibArgs a) {
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < a.pixels;
       p += int64_t(gridDim.x) * blockDim.x) {
    const float b = a.has_bias ? a.bias[p] : 0.0f;
    const float d = a.has_dark ? a.dark[p] : 0.0f;
    const float f = a.has_flat ? a.flat[p] : 0.0f;
    for (int fi = 0; fi < a.nframes; ++fi) {
      const float light = a.raw ? decode_u16(a.raw[fi * a.pixels + p], a.big_endian_bzero) : a.light_f32[p];
      const float out = calibrate_one(light, b, d, f, a);
      a.slots[static_cast<int64_t>(a.slot_of_frame[a.frame[fi]]) * a.stride + p] = out;
      warp_count_add(a.nonfinite + a.frame[fi], !isfinite(out));
    }
  }
}

__global__ void zero_counters_kernel(unsigned* counters, CalibArgs a) {
  if (threadIdx.x < a.nframes) counters[a.frame[threadIdx.x]] = 0u;
}

__global__ void __launch_bounds__(256) count_nonfinite_kernel(const float* frame, int64_t n, unsigned* counter) {
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n; p += int64_t(gridDim.x) * blockDim.x) {
    warp_count_add(counter, !isfinite(frame[p]));
  }
}

__global__ void __launch_bounds__(256) count_nonfinite_slot_kernel(const float* slots, const int* slot_of_frame,
                                                                   int64_t stride, int frame, int64_t n,
                                                                   unsigned* counters) {
  const float* src = slots + static_cast<int64_t>(slot_of_frame[frame]) * stride;
  for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n; p += int64_t(gridDim.x) * blockDim.x) {
    warp_count_add(counters + frame, !isfinite(src[p]));
  }
}

static CalibArgs make_args(gg_stack* s, const gg_calib_params_t& p) {
  CalibArgs a{};
  a.bias = s->d_bias;
  a.dark = s->d_dark;
  a.flat = s->d_flat;
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.nonfinite = s->d_frame_nonfinite;
  a.stride = s->stride;
  a.pixels = s->pixels;
  a.has_bias = s->has_bias;
  a.has_dark = s->has_dark;
  a.has_flat = s->has_flat;
  a.dark_includes_bias = p.master_dark_includes_bias;
  a.dark_scale = p.dark_scale;
  a.flat_floor = p.flat_floor;
  a.pedestal = p.pedestal;
  return a;
}

void launch_calibrate(gg_stack* s, const CalibLaunch& job, const gg_calib_params_t& p) {
  CalibArgs a = make_args(s, p);
  a.raw = job.raw;
  a.light_f32 = job.light_f32;
  a.big_endian_bzero = job.big_endian_bzero;
  a.nframes = job.nframes;
  for (int i = 0; i < job.nframes; ++i) a.frame[i] = job.frame[i];
  note_launch();
  zero_counters_kernel<<<1, 32, 0, s->stream>>>(s->d_frame_nonfinite, a);
  const bool aligned = (s->pixels % 8 == 0) && job.raw != nullptr &&
                       (reinterpret_cast<uintptr_t>(job.raw) % 16 == 0);
  if (aligned) {
    const unsigned grid = grid_for(static_cast<size_t>(s->pixels / 8), 256, 8);
    note_launch();
    calibrate_u16_vec8_kernel<<<grid, 256, 0, s->stream>>>(a);
  } else {
    const unsigned grid = grid_for(static_cast<size_t>(s->pixels), 256, 8);
    note_launch();
    calibrate_scalar_kernel<<<grid, 256, 0, s->stream>>>(a);
  }
  check_cuda(cudaGetLastError(), "calibrate kernel launch");
}

void launch_count_nonfinite(gg_stack* s, int64_t frame) {
  check_cuda(cudaMemsetAsync(s->d_frame_nonfinite + frame, 0, sizeof(unsigned), s->stream), "cudaMemsetAsync");
  const unsigned grid = grid_for(static_cast<size_t>(s->pixels), 256, 4);
  note_launch();
  count_nonfinite_slot_kernel<<<grid, 256, 0, s->stream>>>(s->d_slots, s->d_slot_of_frame, s->stride,
                                                           static_cast<int>(frame), s->pixels, s->d_frame_nonfinite);
  check_cuda(cudaGetLastError(), "count_nonfinite kernel launch");
}

static void validate_calib(const gg_calib_params_t* p) {
  require(p != nullptr, "calibration parameters are null");
  require(std::isfinite(p->dark_scale), "dark_scale must be finite");
  require(std::isfinite(p->flat_floor), "flat_floor must be finite");
  require(std::isfinite(p->pedestal), "pedestal must be finite");
}

static void ensure_lanes(gg_stack* s) {
  if (s->d_raw_lane[0] != nullptr) return;
  s->lane_bytes = static_cast<size_t>(gg_stack::kLaneFrames) * static_cast<size_t>(s->pixels) * 2;
  for (int i = 0; i < gg_stack::kLanes; ++i) {
    void* d = nullptr;
    check_cuda(cudaMalloc(&d, s->lane_bytes), "cudaMalloc(raw lane)");
    s->d_raw_lane[i] = static_cast<uint16_t*>(d);
    s->bytes_allocated += static_cast<int64_t>(s->lane_bytes);
    check_cuda(cudaHostAlloc(&s->h_pinned_lane[i], s->lane_bytes, cudaHostAllocPortable), "cudaHostAlloc(raw lane)");
    s->host_pinned_bytes += static_cast<int64_t>(s->lane_bytes);
  }
}

static bool is_pinned(const void* p) {
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeHost;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_calibrate_u16(gg_stack* s, const int64_t* indices, int64_t count, const void* host_raw,
                           int big_endian_bzero, const gg_calib_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && host_raw != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  validate_calib(params);
  for (int64_t k = 0; k < count; ++k) stack_require_index(s, indices[k]);
  stack_activate(s);
  ensure_lanes(s);
  const bool pinned = is_pinned(host_raw);
  const size_t frame_bytes = static_cast<size_t>(s->pixels) * 2;
  const auto* src = static_cast<const unsigned char*>(host_raw);
  int lane = s->next_lane;
  for (int64_t k0 = 0; k0 < count; k0 += gg_stack::kLaneFrames) {
    const int nb = static_cast<int>(std::min<int64_t>(gg_stack::kLaneFrames, count - k0));
    // The lane's previous decode must finish before its buffers are reused.
    check_cuda(cudaEventSynchronize(s->lane_free[lane]), "cudaEventSynchronize(lane)");
    const unsigned char* chunk = src + static_cast<size_t>(k0) * frame_bytes;
    const void* copy_src = chunk;
    if (!pinned) {
      std::memcpy(s->h_pinned_lane[lane], chunk, frame_bytes * nb);
      copy_src = s->h_pinned_lane[lane];
    }
    check_cuda(cudaStreamWaitEvent(s->copy_stream, s->lane_free[lane], 0), "cudaStreamWaitEvent");
    check_cuda(cudaMemcpyAsync(s->d_raw_lane[lane], copy_src, frame_bytes * nb, cudaMemcpyHostToDevice,
                               s->copy_stream),
               "cudaMemcpyAsync(raw lane)");
    check_cuda(cudaEventRecord(s->lane_ready[lane], s->copy_stream), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(s->stream, s->lane_ready[lane], 0), "cudaStreamWaitEvent");
    CalibLaunch job{};
    job.raw = s->d_raw_lane[lane];
    job.big_endian_bzero = big_endian_bzero;
    job.nframes = nb;
    for (int i = 0; i < nb; ++i) job.frame[i] = static_cast<int>(indices[k0 + i]);
    launch_calibrate(s, job, *params);
    check_cuda(cudaEventRecord(s->lane_free[lane], s->stream), "cudaEventRecord");
    lane = (lane + 1) % gg_stack::kLanes;
  }
  s->next_lane = lane;
  for (int64_t k = 0; k < count; ++k) stack_mark_loaded(s, indices[k]);
  GG_API_END
}

// ---- staged ingest: uploads run ahead of the per-frame stages ---------------
// A device copy of every frame's raw uint16 samples (frames x P) filled from
// pinned host memory on the copy stream, one event per frame when its copy
// has landed and one when its calibration has read it: the caller enqueues
// the uploads of a whole stack at once and calibrates (and processes) the
// frames in chunks while later chunks are still in flight.
struct RawStage {
  uint16_t* d_raw = nullptr;
  std::vector<cudaEvent_t> ready;     // the frame's upload has landed
  std::vector<cudaEvent_t> consumed;  // the frame's calibration has read it
  std::vector<unsigned char> uploaded;
};

static void raw_stage_release(RawStage* r) {
  if (r->d_raw) cudaFree(r->d_raw);
  for (cudaEvent_t e : r->ready) cudaEventDestroy(e);
  for (cudaEvent_t e : r->consumed) cudaEventDestroy(e);
  delete r;
}

static RawStage& raw_stage(gg_stack* s) {
  if (!s->raw_stage) {
    auto* r = new RawStage();
    s->raw_stage = r;
    s->raw_stage_free = [](void* q) { raw_stage_release(static_cast<RawStage*>(q)); };
    const size_t bytes = static_cast<size_t>(s->frames) * static_cast<size_t>(s->pixels) * 2;
    check_cuda(cudaMalloc(&r->d_raw, bytes), "cudaMalloc(raw staging)");
    s->bytes_allocated += static_cast<int64_t>(bytes);
    r->ready.assign(static_cast<size_t>(s->frames), nullptr);
    r->consumed.assign(static_cast<size_t>(s->frames), nullptr);
    r->uploaded.assign(static_cast<size_t>(s->frames), 0);
    for (int64_t k = 0; k < s->frames; ++k) {
      check_cuda(cudaEventCreateWithFlags(&r->ready[k], cudaEventDisableTiming), "cudaEventCreate(raw ready)");
      check_cuda(cudaEventCreateWithFlags(&r->consumed[k], cudaEventDisableTiming), "cudaEventCreate(raw read)");
    }
  }
  return *static_cast<RawStage*>(s->raw_stage);
}

int gg_stack_calibrate_u16_device(gg_stack* s, const int64_t* indices, int64_t count, const void* dev_raw,
                                  int big_endian_bzero, const gg_calib_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && dev_raw != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  validate_calib(params);
  for (int64_t k = 0; k < count; ++k) stack_require_index(s, indices[k]);
  stack_activate(s);
  const auto* raw = static_cast<const uint16_t*>(dev_raw);
  for (int64_t k0 = 0; k0 < count; k0 += GG_MAX_BATCH_FRAMES) {
    const int nb = static_cast<int>(std::min<int64_t>(GG_MAX_BATCH_FRAMES, count - k0));
    CalibLaunch job{};
    job.raw = raw + static_cast<size_t>(k0) * static_cast<size_t>(s->pixels);
    job.big_endian_bzero = big_endian_bzero;
    job.nframes = nb;
    for (int i = 0; i < nb; ++i) job.frame[i] = static_cast<int>(indices[k0 + i]);
    launch_calibrate(s, job, *params);
  }
  for (int64_t k = 0; k < count; ++k) stack_mark_loaded(s, indices[k]);
  GG_API_END
}

int gg_stack_upload_raw_u16(gg_stack* s, const int64_t* indices, int64_t count, const void* host_raw) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && host_raw != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  for (int64_t k = 0; k < count; ++k) stack_require_index(s, indices[k]);
  require(is_pinned(host_raw), "staged uploads need page-locked (pinned) host memory");
  stack_activate(s);
  RawStage& r = raw_stage(s);
  const size_t frame_bytes = static_cast<size_t>(s->pixels) * 2;
  const auto* src = static_cast<const unsigned char*>(host_raw);
  for (int64_t k = 0; k < count; ++k) {
    const int64_t f = indices[k];
    // the previous calibration of this frame must have read its staged copy
    check_cuda(cudaStreamWaitEvent(s->copy_stream, r.consumed[f], 0), "cudaStreamWaitEvent(raw read)");
    check_cuda(cudaMemcpyAsync(reinterpret_cast<unsigned char*>(r.d_raw) + static_cast<size_t>(f) * frame_bytes,
                               src + static_cast<size_t>(k) * frame_bytes, frame_bytes, cudaMemcpyHostToDevice,
                               s->copy_stream),
               "cudaMemcpyAsync(raw staging)");
    check_cuda(cudaEventRecord(r.ready[f], s->copy_stream), "cudaEventRecord(raw ready)");
    r.uploaded[f] = 1;
  }
  GG_API_END
}

int gg_stack_calibrate_u16_staged(gg_stack* s, const int64_t* indices, int64_t count, int big_endian_bzero,
                                  const gg_calib_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr, "null argument");
  require(count > 0, "indices must contain at least one frame index");
  validate_calib(params);
  for (int64_t k = 0; k < count; ++k) stack_require_index(s, indices[k]);
  require(s->raw_stage != nullptr, "no staged raw frames: call gg_stack_upload_raw_u16 first");
  RawStage& r = raw_stage(s);
  for (int64_t k = 0; k < count; ++k) require(r.uploaded[indices[k]] != 0, "frame has no staged raw samples");
  stack_activate(s);
  // runs of consecutive frame indices share one launch (their staged copies are contiguous)
  int64_t k0 = 0;
  while (k0 < count) {
    int64_t k1 = k0 + 1;
    while (k1 < count && k1 - k0 < GG_MAX_BATCH_FRAMES && indices[k1] == indices[k1 - 1] + 1) ++k1;
    for (int64_t k = k0; k < k1; ++k)
      check_cuda(cudaStreamWaitEvent(s->stream, r.ready[indices[k]], 0), "cudaStreamWaitEvent(raw ready)");
    CalibLaunch job{};
    job.raw = r.d_raw + static_cast<size_t>(indices[k0]) * static_cast<size_t>(s->pixels);
    job.big_endian_bzero = big_endian_bzero;
    job.nframes = static_cast<int>(k1 - k0);
    for (int64_t k = k0; k < k1; ++k) job.frame[k - k0] = static_cast<int>(indices[k]);
    launch_calibrate(s, job, *params);
    for (int64_t k = k0; k < k1; ++k)
      check_cuda(cudaEventRecord(r.consumed[indices[k]], s->stream), "cudaEventRecord(raw read)");
    k0 = k1;
  }
  for (int64_t k = 0; k < count; ++k) stack_mark_loaded(s, indices[k]);
  GG_API_END
}

int gg_stack_calibrate_f32(gg_stack* s, int64_t index, const float* host_light, const gg_calib_params_t* params) {
  GG_API_BEGIN
  require(s != nullptr && host_light != nullptr, "null argument");
  validate_calib(params);
  stack_require_index(s, index);
  stack_activate(s);
  // The float32 light is staged in stream-ordered pool memory.
  float* staging = nullptr;
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&staging), static_cast<size_t>(s->pixels) * 4, s->stream),
             "cudaMallocAsync(light)");
  check_cuda(cudaMemcpyAsync(staging, host_light, static_cast<size_t>(s->pixels) * 4, cudaMemcpyHostToDevice,
                             s->stream),
             "cudaMemcpyAsync(light)");
  CalibLaunch job{};
  job.light_f32 = staging;
  job.nframes = 1;
  job.frame[0] = static_cast<int>(index);
  launch_calibrate(s, job, *params);
  check_cuda(cudaFreeAsync(staging, s->stream), "cudaFreeAsync(light)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(calibrate)");
  stack_mark_loaded(s, index);
  GG_API_END
}

int gg_calibrate_tile_f32(const float* host_light, const float* host_bias, const float* host_dark,
                          const float* host_flat, int64_t n, const gg_calib_params_t* params, float* host_out) {
  GG_API_BEGIN
  require(host_light != nullptr && host_out != nullptr, "null argument");
  require(n >= 0, "n must be non-negative");
  validate_calib(params);
  if (n == 0) return GG_OK;
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs <= 0) {
    cudaGetLastError();
    fail(GG_ERR_NO_DEVICE, "no CUDA device is available");
  }
  const size_t bytes = static_cast<size_t>(n) * 4;
  float* d[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  unsigned* d_counter = nullptr;
  int* d_slot = nullptr;
  auto release = [&]() {
    for (float* p : d)
      if (p) cudaFree(p);
    if (d_counter) cudaFree(d_counter);
    if (d_slot) cudaFree(d_slot);
  };
  try {
    const float* srcs[4] = {host_light, host_bias, host_dark, host_flat};
    for (int i = 0; i < 4; ++i) {
      if (!srcs[i]) continue;
      check_cuda(cudaMalloc(&d[i], bytes), "cudaMalloc(calibrate tile)");
      check_cuda(cudaMemcpy(d[i], srcs[i], bytes, cudaMemcpyHostToDevice), "cudaMemcpy(calibrate tile)");
    }
    check_cuda(cudaMalloc(&d[4], bytes), "cudaMalloc(calibrate out)");
    check_cuda(cudaMalloc(&d_counter, sizeof(unsigned)), "cudaMalloc(counter)");
    check_cuda(cudaMalloc(&d_slot, sizeof(int)), "cudaMalloc(slot)");
    check_cuda(cudaMemset(d_counter, 0, sizeof(unsigned)), "cudaMemset");
    check_cuda(cudaMemset(d_slot, 0, sizeof(int)), "cudaMemset");
    CalibArgs a{};
    a.light_f32 = d[0];
    a.bias = d[1];
    a.dark = d[2];
    a.flat = d[3];
    a.slots = d[4];
    a.slot_of_frame = d_slot;
    a.nonfinite = d_counter;
    a.stride = n;
    a.pixels = n;
    a.nframes = 1;
    a.frame[0] = 0;
    a.has_bias = host_bias != nullptr;
    a.has_dark = host_dark != nullptr;
    a.has_flat = host_flat != nullptr;
    a.dark_includes_bias = params->master_dark_includes_bias;
    a.dark_scale = params->dark_scale;
    a.flat_floor = params->flat_floor;
    a.pedestal = params->pedestal;
    note_launch();
    calibrate_scalar_kernel<<<grid_for(static_cast<size_t>(n), 256, 4), 256>>>(a);
    check_cuda(cudaGetLastError(), "calibrate kernel launch");
    check_cuda(cudaMemcpy(host_out, d[4], bytes, cudaMemcpyDeviceToHost), "cudaMemcpy(calibrate out)");
  } catch (...) {
    release();
    throw;
  }
  release();
  GG_API_END
}

}  // extern "C"
