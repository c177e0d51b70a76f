// Grid local normalisation of registered frames to the reference frame (the
// resident grid_mean_std mode, tile 256 by default):
//
//   ln_pair_stats_kernel  one CTA per (tile, frame pair): sums of the source
//                         and reference pixels and their squares over the
//                         pixels finite in both (local_norm_kernels.cu:220-300),
//                         float-float per thread, float64 across the CTA;
//   ln_coeff_kernel       one thread per (pair, tile): mean = sum / n,
//                         std = sqrt(max(sum2 / n - mean^2, 0)) in float64,
//                         stored as float32 (native_bindings.cpp:10745-10760);
//                         coefficients (resident_cuda.py:1897-1927): empty
//                         tile scale 1 / offset 0; std <= eps on either side
//                         scale 1 / offset ref_mean - src_mean; else
//                         scale = ref_std / src_std, offset = ref_mean -
//                         src_mean * scale, float32 operations;
//   ln_apply_kernel       in place, v * scale + offset per tile (float32
//                         multiply, then add: cpu/local_norm.py:197-215).
//
// Traffic: the statistics read both frames of a pair (8 B per pixel), the
// apply reads and writes the source (8 B per pixel); both are HBM-bound
// streams (float-float accumulation keeps the statistics off the FP64 pipe).
#include <cmath>
#include <cstring>
#include <vector>

#include "stack.cuh"

namespace gg {

constexpr int kLnThreads = 256;

struct LnArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  int width, height;
  int tile_w, tile_h, cols, rows;
  int ref_frame;
  const int* frames;         // [pairs] source frames
  double* sums;              // [pairs][tiles][4]
  unsigned long long* counts;  // [pairs][tiles]
  float* stats;              // [pairs][tiles][4]: src mean, src std, ref mean, ref std
  float* scales;             // [pairs][tiles]
  float* offsets;
  unsigned long long* totals;  // [pairs] paired finite pixels of the frame
  double eps;
};

__global__ void __launch_bounds__(kLnThreads) ln_pair_stats_kernel(LnArgs a) {
  __shared__ double red[kLnThreads / 32][4];
  __shared__ unsigned long long redn[kLnThreads / 32];
  const int tile = blockIdx.x, pair = blockIdx.y;
  const int tx = tile % a.cols, ty = tile / a.cols;
  const int x0 = tx * a.tile_w, y0 = ty * a.tile_h;
  const int w = min(a.tile_w, a.width - x0), h = min(a.tile_h, a.height - y0);
  const float* src = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[pair]]) * a.stride;
  const float* ref = a.slots + static_cast<int64_t>(a.slot_of_frame[a.ref_frame]) * a.stride;
  FF s1, s2, r1, r2;
  unsigned n = 0;
  const int npx = w * h;
  for (int q = threadIdx.x; q < npx; q += kLnThreads) {
    const int y = y0 + q / w, x = x0 + q % w;
    const int64_t p = static_cast<int64_t>(y) * a.width + x;
    const float s = __ldcs(src + p), r = __ldcs(ref + p);
    if (isfinite(s) && isfinite(r)) {
      s1.add(s);
      s2.add_prod(s, s);
      r1.add(r);
      r2.add_prod(r, r);
      ++n;
    }
  }
  double v[4] = {static_cast<double>(s1.hi) + static_cast<double>(s1.lo),
                 static_cast<double>(s2.hi) + static_cast<double>(s2.lo),
                 static_cast<double>(r1.hi) + static_cast<double>(r1.lo),
                 static_cast<double>(r2.hi) + static_cast<double>(r2.lo)};
  unsigned long long nn = n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], off);
    nn += __shfl_xor_sync(0xffffffffu, nn, off);
  }
  if (lane == 0) {
    for (int i = 0; i < 4; ++i) red[warp][i] = v[i];
    redn[warp] = nn;
  }
  __syncthreads();
  const int64_t t = static_cast<int64_t>(pair) * a.cols * a.rows + tile;
  if (threadIdx.x < 4) {
    double acc = 0.0;
    for (int k = 0; k < kLnThreads / 32; ++k) acc += red[k][threadIdx.x];
    a.sums[t * 4 + threadIdx.x] = acc;
  } else if (threadIdx.x == 4) {
    unsigned long long acc = 0;
    for (int k = 0; k < kLnThreads / 32; ++k) acc += redn[k];
    a.counts[t] = acc;
  }
}

__global__ void ln_coeff_kernel(LnArgs a, int pairs) {
  const int tiles = a.cols * a.rows;
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<int64_t>(pairs) * tiles) return;
  const int pair = static_cast<int>(t / tiles);
  const unsigned long long c = a.counts[t];
  float sm = 0.0f, ss = 0.0f, rm = 0.0f, rs = 0.0f;
  float scale = 1.0f, offset = 0.0f;
  if (c > 0) {
    const double inv = 1.0 / static_cast<double>(c);
    const double* s = a.sums + t * 4;
    const double smd = s[0] * inv, rmd = s[2] * inv;
    const double sv = fmax(__dsub_rn(__dmul_rn(s[1], inv), __dmul_rn(smd, smd)), 0.0);
    const double rv = fmax(__dsub_rn(__dmul_rn(s[3], inv), __dmul_rn(rmd, rmd)), 0.0);
    sm = __double2float_rn(smd);
    ss = __double2float_rn(sqrt(sv));
    rm = __double2float_rn(rmd);
    rs = __double2float_rn(sqrt(rv));
    if (static_cast<double>(ss) <= a.eps || static_cast<double>(rs) <= a.eps) {
      offset = __fsub_rn(rm, sm);
    } else {
      scale = __fdiv_rn(rs, ss);
      offset = __fsub_rn(rm, __fmul_rn(sm, scale));
    }
    atomicAdd(a.totals + pair, c);
  }
  if (a.stats) {
    a.stats[t * 4 + 0] = sm;
    a.stats[t * 4 + 1] = ss;
    a.stats[t * 4 + 2] = rm;
    a.stats[t * 4 + 3] = rs;
  }
  a.scales[t] = scale;
  a.offsets[t] = offset;
}

// In place v * scale + offset for every pixel of each listed frame; frames
// whose pair had no finite pixel (totals == 0) are left as they are.
__global__ void __launch_bounds__(256) ln_apply_kernel(LnArgs a, int check_totals) {
  const int pair = blockIdx.y;
  if (check_totals && a.totals[pair] == 0) return;
  float* img = const_cast<float*>(a.slots) + static_cast<int64_t>(a.slot_of_frame[a.frames[pair]]) * a.stride;
  const float* sc = a.scales + static_cast<int64_t>(pair) * a.cols * a.rows;
  const float* of = a.offsets + static_cast<int64_t>(pair) * a.cols * a.rows;
  const int W = a.width;
  const int64_t P = static_cast<int64_t>(W) * a.height;
  for (int64_t p4 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * 4; p4 < P;
       p4 += static_cast<int64_t>(gridDim.x) * blockDim.x * 4) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t p = p4 + i;
      if (p >= P) break;
      const int y = static_cast<int>(p / W), x = static_cast<int>(p - static_cast<int64_t>(y) * W);
      const int t = min(y / a.tile_h, a.rows - 1) * a.cols + min(x / a.tile_w, a.cols - 1);
      img[p] = __fadd_rn(__fmul_rn(img[p], __ldg(sc + t)), __ldg(of + t));
    }
  }
}

__global__ void ln_zero_weights_kernel(const unsigned long long* totals, const int* frames, int pairs,
                                       float* weights) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < pairs && totals[i] == 0) weights[frames[i]] = 0.0f;
}

struct LnScratch {
  double* sums = nullptr;
  unsigned long long* counts = nullptr;
  float* stats = nullptr;
  float* scales = nullptr;
  float* offsets = nullptr;
  unsigned long long* totals = nullptr;
  int* frames = nullptr;
  int* h_frames = nullptr;  // pinned
  int64_t tile_cap = 0;     // pairs * tiles
  int pair_cap = 0;
};

static void ln_release(LnScratch& g) {
  void* d[] = {g.sums, g.counts, g.stats, g.scales, g.offsets, g.totals, g.frames};
  for (void* p : d)
    if (p) cudaFree(p);
  if (g.h_frames) cudaFreeHost(g.h_frames);
  g = LnScratch{};
}

static LnScratch& ln_scratch(gg_stack* s, int pairs, int64_t tiles) {
  if (!s->ln_scratch) {
    s->ln_scratch = new LnScratch();
    s->ln_scratch_free = [](void* q) {
      auto* g = static_cast<LnScratch*>(q);
      ln_release(*g);
      delete g;
    };
  }
  LnScratch& g = *static_cast<LnScratch*>(s->ln_scratch);
  const int64_t need = static_cast<int64_t>(pairs) * tiles;
  if (g.tile_cap < need || g.pair_cap < pairs) {
    check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(local norm scratch)");
    const int64_t tc = std::max(need, g.tile_cap);
    const int pc = std::max(pairs, g.pair_cap);
    ln_release(g);
    check_cuda(cudaMalloc(&g.sums, sizeof(double) * 4 * tc), "cudaMalloc(local norm sums)");
    check_cuda(cudaMalloc(&g.counts, sizeof(unsigned long long) * tc), "cudaMalloc(local norm counts)");
    check_cuda(cudaMalloc(&g.stats, sizeof(float) * 4 * tc), "cudaMalloc(local norm stats)");
    check_cuda(cudaMalloc(&g.scales, sizeof(float) * tc), "cudaMalloc(local norm scales)");
    check_cuda(cudaMalloc(&g.offsets, sizeof(float) * tc), "cudaMalloc(local norm offsets)");
    check_cuda(cudaMalloc(&g.totals, sizeof(unsigned long long) * pc), "cudaMalloc(local norm totals)");
    check_cuda(cudaMalloc(&g.frames, sizeof(int) * pc), "cudaMalloc(local norm frames)");
    check_cuda(cudaHostAlloc(reinterpret_cast<void**>(&g.h_frames), sizeof(int) * pc, cudaHostAllocDefault),
               "cudaHostAlloc(local norm frames)");
    g.tile_cap = tc;
    g.pair_cap = pc;
  }
  return g;
}

static LnArgs ln_args(gg_stack* s, int tile_h, int tile_w, int rows, int cols, int ref, LnScratch& g) {
  LnArgs a{};
  a.slots = s->d_slots;
  a.slot_of_frame = s->d_slot_of_frame;
  a.stride = s->stride;
  a.width = static_cast<int>(s->width);
  a.height = static_cast<int>(s->height);
  a.tile_w = tile_w;
  a.tile_h = tile_h;
  a.cols = cols;
  a.rows = rows;
  a.ref_frame = ref;
  a.frames = g.frames;
  a.sums = g.sums;
  a.counts = g.counts;
  a.stats = g.stats;
  a.scales = g.scales;
  a.offsets = g.offsets;
  a.totals = g.totals;
  return a;
}

static void upload_frames(gg_stack* s, LnScratch& g, const int64_t* idx, int64_t count) {
  for (int64_t k = 0; k < count; ++k) g.h_frames[k] = static_cast<int>(idx[k]);
  upload_params(s->stream, g.frames, g.h_frames, sizeof(int) * count, "cudaMemcpyAsync(local norm frames)");
}

static unsigned apply_grid_x(gg_stack* s, int pairs) {
  const int64_t want = static_cast<int64_t>(sm_count()) * 8 / std::max(pairs, 1) + 1;
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((s->pixels + 1023) / 1024, want)));
}

// statistics + coefficients (+ apply) for `count` source frames
static void ln_run(gg_stack* s, int64_t ref, const int64_t* sources, int64_t count, int tile_h, int tile_w, double eps,
                   bool apply, bool update_weights) {
  const int rows = static_cast<int>((s->height + tile_h - 1) / tile_h);
  const int cols = static_cast<int>((s->width + tile_w - 1) / tile_w);
  const int pairs = static_cast<int>(count);
  LnScratch& g = ln_scratch(s, pairs, static_cast<int64_t>(rows) * cols);
  upload_frames(s, g, sources, count);
  LnArgs a = ln_args(s, tile_h, tile_w, rows, cols, static_cast<int>(ref), g);
  a.eps = eps;
  check_cuda(cudaMemsetAsync(g.totals, 0, sizeof(unsigned long long) * pairs, s->stream), "cudaMemsetAsync(totals)");
  note_launch();
  ln_pair_stats_kernel<<<dim3(static_cast<unsigned>(rows * cols), static_cast<unsigned>(pairs)), kLnThreads, 0,
                         s->stream>>>(a);
  check_cuda(cudaGetLastError(), "ln_pair_stats launch");
  const int64_t tiles = static_cast<int64_t>(pairs) * rows * cols;
  note_launch();
  ln_coeff_kernel<<<static_cast<unsigned>((tiles + 255) / 256), 256, 0, s->stream>>>(a, pairs);
  check_cuda(cudaGetLastError(), "ln_coeff launch");
  if (apply) {
    note_launch();
    ln_apply_kernel<<<dim3(apply_grid_x(s, pairs), static_cast<unsigned>(pairs)), 256, 0, s->stream>>>(a, 1);
    check_cuda(cudaGetLastError(), "ln_apply launch");
  }
  if (update_weights) {
    note_launch();
    ln_zero_weights_kernel<<<(pairs + 127) / 128, 128, 0, s->stream>>>(g.totals, g.frames, pairs, s->d_weights);
    check_cuda(cudaGetLastError(), "ln_zero_weights launch");
  }
}

static void validate_tiles(int tile_h, int tile_w) {
  require(tile_h > 0 && tile_w > 0, "tile dimensions must be positive");
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_stack_pair_grid_stats(gg_stack* s, int64_t reference_index, const int64_t* sources, int64_t count,
                             int32_t tile_h, int32_t tile_w, float* host_source_mean, float* host_source_std,
                             float* host_reference_mean, float* host_reference_std, uint64_t* host_valid) {
  GG_API_BEGIN
  require(s != nullptr && sources != nullptr, "null argument");
  require(count > 0 && count <= 65535, "source count must be in [1, 65535]");
  validate_tiles(tile_h, tile_w);
  stack_require_loaded(s, reference_index, "grid local normalization reference statistics");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, sources[k], "grid local normalization statistics");
  stack_activate(s);
  ln_run(s, reference_index, sources, count, tile_h, tile_w, 1.0e-6, false, false);
  const int rows = static_cast<int>((s->height + tile_h - 1) / tile_h);
  const int cols = static_cast<int>((s->width + tile_w - 1) / tile_w);
  const int64_t tiles = count * rows * cols;
  LnScratch& g = *static_cast<LnScratch*>(s->ln_scratch);
  std::vector<float> st(static_cast<size_t>(tiles) * 4);
  std::vector<unsigned long long> cn(static_cast<size_t>(tiles));
  check_cuda(cudaMemcpyAsync(st.data(), g.stats, sizeof(float) * 4 * tiles, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(local norm stats)");
  check_cuda(cudaMemcpyAsync(cn.data(), g.counts, sizeof(unsigned long long) * tiles, cudaMemcpyDeviceToHost,
                             s->stream),
             "cudaMemcpyAsync(local norm counts)");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(local norm stats)");
  for (int64_t t = 0; t < tiles; ++t) {
    if (host_source_mean) host_source_mean[t] = st[static_cast<size_t>(t) * 4 + 0];
    if (host_source_std) host_source_std[t] = st[static_cast<size_t>(t) * 4 + 1];
    if (host_reference_mean) host_reference_mean[t] = st[static_cast<size_t>(t) * 4 + 2];
    if (host_reference_std) host_reference_std[t] = st[static_cast<size_t>(t) * 4 + 3];
    if (host_valid) host_valid[t] = cn[static_cast<size_t>(t)];
  }
  GG_API_END
}

int gg_stack_apply_grid_normalization(gg_stack* s, const int64_t* indices, int64_t count, const float* host_scales,
                                      const float* host_offsets, int32_t grid_rows, int32_t grid_cols,
                                      int32_t tile_h, int32_t tile_w) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && host_scales != nullptr && host_offsets != nullptr, "null argument");
  require(count > 0 && count <= 65535, "frame count must be in [1, 65535]");
  validate_tiles(tile_h, tile_w);
  require(grid_rows > 0 && grid_cols > 0, "coefficient grid must not be empty");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, indices[k], "grid local normalization");
  stack_activate(s);
  const int64_t tiles = static_cast<int64_t>(grid_rows) * grid_cols;
  LnScratch& g = ln_scratch(s, static_cast<int>(count), tiles);
  upload_frames(s, g, indices, count);
  upload_params(s->stream, g.scales, host_scales, sizeof(float) * tiles * count, "cudaMemcpyAsync(local norm scales)");
  upload_params(s->stream, g.offsets, host_offsets, sizeof(float) * tiles * count,
                "cudaMemcpyAsync(local norm offsets)");
  LnArgs a = ln_args(s, tile_h, tile_w, grid_rows, grid_cols, 0, g);
  note_launch();
  ln_apply_kernel<<<dim3(apply_grid_x(s, static_cast<int>(count)), static_cast<unsigned>(count)), 256, 0,
                    s->stream>>>(a, 0);
  check_cuda(cudaGetLastError(), "ln_apply launch");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(local norm apply)");
  GG_API_END
}

int gg_stack_local_normalize_grid(gg_stack* s, int64_t reference_index, const int64_t* sources, int64_t count,
                                  int32_t tile_h, int32_t tile_w, double eps, int update_weights, float* host_scales,
                                  float* host_offsets) {
  GG_API_BEGIN
  require(s != nullptr && sources != nullptr, "null argument");
  require(count > 0 && count <= 65535, "source count must be in [1, 65535]");
  validate_tiles(tile_h, tile_w);
  require(std::isfinite(eps) && eps >= 0.0, "eps must be finite and non-negative");
  stack_require_loaded(s, reference_index, "grid local normalization reference");
  for (int64_t k = 0; k < count; ++k) {
    stack_require_loaded(s, sources[k], "grid local normalization");
    require(sources[k] != reference_index, "the reference frame is not normalised to itself");
  }
  stack_activate(s);
  ln_run(s, reference_index, sources, count, tile_h, tile_w, eps, true, update_weights != 0);
  if (host_scales || host_offsets) {
    const int64_t tiles = count * ((s->height + tile_h - 1) / tile_h) * ((s->width + tile_w - 1) / tile_w);
    LnScratch& g = *static_cast<LnScratch*>(s->ln_scratch);
    if (host_scales)
      check_cuda(cudaMemcpyAsync(host_scales, g.scales, sizeof(float) * tiles, cudaMemcpyDeviceToHost, s->stream),
                 "cudaMemcpyAsync(local norm scales)");
    if (host_offsets)
      check_cuda(cudaMemcpyAsync(host_offsets, g.offsets, sizeof(float) * tiles, cudaMemcpyDeviceToHost, s->stream),
                 "cudaMemcpyAsync(local norm offsets)");
    check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(local norm coefficients)");
  }
  GG_API_END
}

int gg_stack_apply_global_normalization(gg_stack* s, int64_t index, float scale, float offset) {
  GG_API_BEGIN
  require(s != nullptr, "null argument");
  stack_require_loaded(s, index, "global local normalization");
  stack_activate(s);
  LnScratch& g = ln_scratch(s, 1, 1);
  upload_frames(s, g, &index, 1);
  upload_params(s->stream, g.scales, &scale, sizeof(float), "cudaMemcpyAsync(global scale)");
  upload_params(s->stream, g.offsets, &offset, sizeof(float), "cudaMemcpyAsync(global offset)");
  LnArgs a = ln_args(s, static_cast<int>(s->height), static_cast<int>(s->width), 1, 1, 0, g);
  note_launch();
  ln_apply_kernel<<<dim3(apply_grid_x(s, 1), 1), 256, 0, s->stream>>>(a, 0);
  check_cuda(cudaGetLastError(), "ln_apply launch");
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(global normalization)");
  GG_API_END
}

}  // extern "C"
