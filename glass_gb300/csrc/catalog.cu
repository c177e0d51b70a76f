// Grid star catalogs of resident frames: per-cell top-K local maxima, one
// flux-ordered merge, minimum-separation suppression and a windowed centroid.
//
// Semantics of the reference's deterministic grid catalog
// (star_detect_kernels.cu:40-101 local maximum and candidate order,
// :317-498 per-cell top-K, :500-605 sort, :607-648 suppression, :650-742
// centroid; batch driver native_bindings.cpp:12622-12645, 12211-12616):
//   - a candidate is an interior pixel whose value is finite, > threshold and
//     not below any of its 8 neighbours;
//   - the image is cut into grid_cols x grid_rows cells (cell x-range
//     [cx*W/cols, (cx+1)*W/cols), same for y); each cell keeps its best K
//     candidates, "better" meaning larger value, then smaller y, then smaller
//     x;
//   - all kept candidates are ordered by the same rule and scanned greedily:
//     a candidate is kept unless it lies closer than min_separation_px to an
//     already kept one, until max_output_candidates are kept;
//   - with centroid_radius > 0 every kept candidate moves to the centroid of
//     max(value - background, 0) over the window of that radius (at most 8)
//     around it, clipped to the frame; the background is the median of the
//     window's finite samples, or the frame's global mean of finite samples
//     when asked (falling back to the median when the frame has none).
//   - `count` is the number of candidates in the whole frame.
//
// GB300 form: one CTA per (cell, frame) streams its cell once, keeps the
// candidates as 64-bit keys (order-preserving value bits above the inverted
// pixel index, so "better" is "larger key") in shared memory and compacts to
// the best K whenever the buffer fills; one CTA per frame sorts the kept keys
// (bitonic, in shared memory when they fit, else in a global scratch) and one
// warp runs the suppression scan; one warp per kept star computes the
// centroid (window median by rank counting across the warp).
#include <cmath>
#include <vector>

#include "stack.cuh"

namespace gg {
namespace {

constexpr int kCellCap = 4096;        // keys a cell CTA buffers
constexpr int kCellThreads = 256;     // 32 x 8
constexpr int kTileRows = 32;         // rows of a tile: 4 per thread
constexpr int kTileKeys = kTileRows * 32;
constexpr int kMaxPerCell = kCellCap - kTileKeys;
constexpr int kMaxOutput = 8192;
constexpr int kSharedSortMax = 16384;  // keys sorted in shared memory (128 KiB)
constexpr int kSelectThreads = 1024;
constexpr int kMaxCentroidRadius = 8;
constexpr int kWindowMax = (2 * kMaxCentroidRadius + 1) * (2 * kMaxCentroidRadius + 1);

__device__ __forceinline__ unsigned ordered_bits(float v) {
  const unsigned u = __float_as_uint(v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float float_of_ordered(unsigned o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

__device__ __forceinline__ unsigned long long candidate_key(float value, unsigned pixel) {
  return (static_cast<unsigned long long>(ordered_bits(value)) << 32) | static_cast<unsigned long long>(~pixel);
}

// Bitonic sort of keys[0, n) into descending order (n a power of two) by all
// threads of the CTA.
__device__ void bitonic_desc(unsigned long long* keys, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int peer = i ^ j;
        if (peer > i) {
          const unsigned long long a = keys[i], b = keys[peer];
          // descending overall: blocks with (i & k) == 0 put the larger key first
          const bool swap = ((i & k) == 0) ? (a < b) : (a > b);
          if (swap) {
            keys[i] = b;
            keys[peer] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ int pow2_at_least(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

struct CellArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  const int* frames;
  int width, height;
  float threshold;
  int grid_cols, grid_rows, per_cell;
  unsigned long long* cell_keys;  // [frame][cell][per_cell]
  unsigned* found;                // [frame]
};

__global__ void __launch_bounds__(kCellThreads) grid_cell_topk_kernel(CellArgs a) {
  __shared__ unsigned long long buf[kCellCap];
  __shared__ int n;
  __shared__ unsigned long long cutoff;
  __shared__ unsigned local_found;
  const int cell = blockIdx.x;
  const int f = blockIdx.y;
  const int cells = a.grid_cols * a.grid_rows;
  const float* img = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[f]]) * a.stride;
  const int cx = cell % a.grid_cols, cy = cell / a.grid_cols;
  const int x0 = static_cast<int>((static_cast<int64_t>(cx) * a.width) / a.grid_cols);
  const int x1 = static_cast<int>((static_cast<int64_t>(cx + 1) * a.width) / a.grid_cols);
  const int y0 = static_cast<int>((static_cast<int64_t>(cy) * a.height) / a.grid_rows);
  const int y1 = static_cast<int>((static_cast<int64_t>(cy + 1) * a.height) / a.grid_rows);
  if (threadIdx.x == 0) {
    n = 0;
    cutoff = 0ull;
    local_found = 0u;
  }
  __syncthreads();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int W = a.width, H = a.height;
  // tiles of 32 rows x 32 columns (a warp per row, four rows per warp); a
  // tile adds at most kTileKeys keys, so the buffer is compacted to the best
  // `per_cell` keys whenever fewer than that many slots are left
  for (int ybase = y0; ybase < y1; ybase += kTileRows) {
    for (int xbase = x0; xbase < x1; xbase += 32) {
      const int x = xbase + tx;
#pragma unroll
      for (int r = 0; r < kTileRows / 8; ++r) {
        const int y = ybase + ty + 8 * r;
        if (y < y1 && x < x1 && x > 0 && y > 0 && x < W - 1 && y < H - 1) {
          const float* p = img + static_cast<int64_t>(y) * W + x;
          const float c = __ldg(p);
          if (isfinite(c) && c > a.threshold) {
            bool peak = true;
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
#pragma unroll
              for (int dx = -1; dx <= 1; ++dx) {
                if ((dx || dy) && c < __ldg(p + static_cast<int64_t>(dy) * W + dx)) peak = false;
              }
            }
            if (peak) {
              atomicAdd(&local_found, 1u);
              const unsigned long long key = candidate_key(c, static_cast<unsigned>(y) * static_cast<unsigned>(W) +
                                                                  static_cast<unsigned>(x));
              if (key > cutoff) buf[atomicAdd(&n, 1)] = key;
            }
          }
        }
      }
      __syncthreads();
      const int filled = n;
      __syncthreads();  // every thread has read `filled` before the next tile appends
      if (filled > kCellCap - kTileKeys) {
        const int m = pow2_at_least(filled);
        for (int i = filled + threadIdx.x; i < m; i += blockDim.x) buf[i] = 0ull;
        __syncthreads();
        bitonic_desc(buf, m);
        if (threadIdx.x == 0) {
          n = a.per_cell;
          cutoff = buf[a.per_cell - 1];
        }
        __syncthreads();
      }
    }
  }
  const int total = n;
  const int m = pow2_at_least(total > 0 ? total : 1);
  for (int i = total + threadIdx.x; i < m; i += blockDim.x) buf[i] = 0ull;
  __syncthreads();
  bitonic_desc(buf, m);
  unsigned long long* out = a.cell_keys + (static_cast<int64_t>(f) * cells + cell) * a.per_cell;
  for (int i = threadIdx.x; i < a.per_cell; i += blockDim.x) out[i] = i < total ? buf[i] : 0ull;
  if (threadIdx.x == 0) atomicAdd(a.found + f, local_found);
}

struct SelectArgs {
  const unsigned long long* cell_keys;  // [frame][entries]
  unsigned long long* sort_scratch;     // [frame][sort_n] when sort_n > kSharedSortMax, else null
  int entries, sort_n;
  int width;
  float min_sep2;
  int max_out;
  float* pre_x;  // [frame][max_out] candidate positions before the centroid
  float* pre_y;
  float* flux;
  int* stored;   // [frame]
};

__global__ void __launch_bounds__(kSelectThreads) catalog_select_kernel(SelectArgs a) {
  extern __shared__ unsigned long long sm[];
  const int f = blockIdx.x;
  const unsigned long long* src = a.cell_keys + static_cast<int64_t>(f) * a.entries;
  const bool in_shared = a.sort_scratch == nullptr;
  unsigned long long* keys = in_shared ? sm : a.sort_scratch + static_cast<int64_t>(f) * a.sort_n;
  float2* sel = reinterpret_cast<float2*>(in_shared ? sm + a.sort_n : sm);
  for (int i = threadIdx.x; i < a.sort_n; i += blockDim.x) keys[i] = i < a.entries ? src[i] : 0ull;
  __syncthreads();
  bitonic_desc(keys, a.sort_n);
  if (threadIdx.x >= 32) return;
  // greedy suppression scan in key order by one warp
  const int lane = threadIdx.x;
  const int64_t ob = static_cast<int64_t>(f) * a.max_out;
  int kept = 0;
  for (int i = 0; i < a.entries && kept < a.max_out; ++i) {
    const unsigned long long key = keys[i];
    if (key == 0ull) break;
    const unsigned pixel = ~static_cast<unsigned>(key & 0xffffffffull);
    const float x = static_cast<float>(pixel % static_cast<unsigned>(a.width));
    const float y = static_cast<float>(pixel / static_cast<unsigned>(a.width));
    bool clash = false;
    for (int j = lane; j < kept; j += 32) {
      const float dx = __fsub_rn(x, sel[j].x);
      const float dy = __fsub_rn(y, sel[j].y);
      if (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) < a.min_sep2) clash = true;
    }
    if (__any_sync(0xffffffffu, clash)) continue;
    if (lane == 0) {
      sel[kept] = make_float2(x, y);
      a.pre_x[ob + kept] = x;
      a.pre_y[ob + kept] = y;
      a.flux[ob + kept] = float_of_ordered(static_cast<unsigned>(key >> 32));
    }
    __syncwarp();
    ++kept;
  }
  if (lane == 0) a.stored[f] = kept;
}

// float32 global mean of each frame's finite samples from the frame-stats
// partials ([frame][block][sum, sum2, count]); NaN for a frame without any.
__global__ void frame_mean_kernel(const double* partials, int blocks, int count, float* mean) {
  const int f = blockIdx.x;
  if (f >= count) return;
  double s = 0.0, n = 0.0;
  for (int b = threadIdx.x; b < blocks; b += 32) {
    s += partials[(static_cast<int64_t>(f) * blocks + b) * 3];
    n += partials[(static_cast<int64_t>(f) * blocks + b) * 3 + 2];
  }
  for (int off = 16; off > 0; off >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, off);
    n += __shfl_xor_sync(0xffffffffu, n, off);
  }
  if (threadIdx.x == 0) mean[f] = n > 0.0 ? static_cast<float>(s / n) : __int_as_float(0x7fc00000);
}

struct CentroidArgs {
  const float* slots;
  const int* slot_of_frame;
  int64_t stride;
  const int* frames;
  int width, height, radius, max_out;
  const float* pre_x;
  const float* pre_y;
  const int* stored;
  const float* global_mean;  // [frame] or null (window median)
  float* out_x;
  float* out_y;
  unsigned char* status;
};

constexpr int kCentroidWarps = 4;

__global__ void __launch_bounds__(32 * kCentroidWarps) catalog_centroid_kernel(CentroidArgs a) {
  __shared__ float win[kCentroidWarps][kWindowMax];
  __shared__ float med[kCentroidWarps][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int f = blockIdx.y;
  const int i = blockIdx.x * kCentroidWarps + warp;
  if (i >= a.stored[f]) return;
  const int64_t o = static_cast<int64_t>(f) * a.max_out + i;
  const float px = a.pre_x[o], py = a.pre_y[o];
  a.out_x[o] = px;
  a.out_y[o] = py;
  if (lane == 0) a.status[o] = 0;
  const int cx = static_cast<int>(floorf(__fadd_rn(px, 0.5f)));
  const int cy = static_cast<int>(floorf(__fadd_rn(py, 0.5f)));
  if (cx < 0 || cx >= a.width || cy < 0 || cy >= a.height) return;
  const int r = min(max(a.radius, 1), kMaxCentroidRadius);
  const int x0 = max(0, cx - r), x1 = min(a.width - 1, cx + r);
  const int y0 = max(0, cy - r), y1 = min(a.height - 1, cy + r);
  const int ww = x1 - x0 + 1, count = ww * (y1 - y0 + 1);
  const float* img = a.slots + static_cast<int64_t>(a.slot_of_frame[a.frames[f]]) * a.stride;
  for (int k = lane; k < count; k += 32) win[warp][k] = __ldg(img + static_cast<int64_t>(y0 + k / ww) * a.width + x0 + k % ww);
  __syncwarp();
  float bg = a.global_mean ? a.global_mean[f] : __int_as_float(0x7fc00000);
  if (!isfinite(bg)) {
    int finite = 0;
    for (int k = lane; k < count; k += 32) finite += isfinite(win[warp][k]) ? 1 : 0;
    for (int off = 16; off > 0; off >>= 1) finite += __shfl_xor_sync(0xffffffffu, finite, off);
    if (finite == 0) return;
    // the value at sorted rank finite/2 (and finite/2 - 1 when even): rank of
    // a sample = samples below it + equal samples earlier in the window
    const int hi = finite / 2, lo = (finite & 1) ? hi : hi - 1;
    for (int k = lane; k < count; k += 32) {
      const float v = win[warp][k];
      if (!isfinite(v)) continue;
      int rank = 0;
      for (int j = 0; j < count; ++j) {
        const float u = win[warp][j];
        rank += (isfinite(u) && (u < v || (u == v && j < k))) ? 1 : 0;
      }
      if (rank == hi) med[warp][1] = v;
      if (rank == lo) med[warp][0] = v;
    }
    __syncwarp();
    bg = (finite & 1) ? med[warp][1] : __fmul_rn(0.5f, __fadd_rn(med[warp][0], med[warp][1]));
  }
  if (lane != 0) return;
  double sw = 0.0, sx = 0.0, sy = 0.0;
  for (int k = 0; k < count; ++k) {
    const float v = win[warp][k];
    if (!isfinite(v)) continue;
    const float w = fmaxf(__fsub_rn(v, bg), 0.0f);
    if (w <= 0.0f) continue;
    const double dw = static_cast<double>(w);
    sw += dw;
    sx = fma(static_cast<double>(x0 + k % ww), dw, sx);
    sy = fma(static_cast<double>(y0 + k / ww), dw, sy);
  }
  if (sw <= 0.0) return;
  a.out_x[o] = static_cast<float>(sx / sw);
  a.out_y[o] = static_cast<float>(sy / sw);
  a.status[o] = 1;
}

}  // namespace

void launch_frame_stats_partials(gg_stack* s, const int* d_frames, int count, int blocks, double* partials);

}  // namespace gg

using namespace gg;

extern "C" int gg_stack_star_grid_catalog(gg_stack* s, const int64_t* indices, int64_t count,
                                          const gg_grid_catalog_params_t* params, float* host_catalog,
                                          uint8_t* host_status, int32_t* host_counts) {
  GG_API_BEGIN
  require(s != nullptr && indices != nullptr && params != nullptr && host_catalog != nullptr &&
              host_counts != nullptr,
          "null argument");
  require(count > 0 && count <= 65535, "frame count must be in [1, 65535]");
  const gg_grid_catalog_params_t p = *params;
  require(p.grid_cols > 0 && p.grid_rows > 0 && p.candidates_per_cell > 0 && p.max_output_candidates > 0,
          "grid dimensions and candidate counts must be positive");
  require(p.min_separation_px >= 0.0f && std::isfinite(p.min_separation_px), "min_separation_px must be non-negative");
  require(p.candidates_per_cell <= kMaxPerCell, "candidates_per_cell must be at most 3072");
  require(p.max_output_candidates <= kMaxOutput, "max_output_candidates must be at most 8192");
  require(p.centroid_radius >= 0, "centroid_radius must be non-negative");
  require(p.centroid_background == 0 || p.centroid_background == 1, "centroid background must be 0 or 1");
  require(static_cast<int64_t>(p.grid_cols) * p.grid_rows <= 65535, "grid_cols * grid_rows must be at most 65535");
  require(s->pixels < 0xffffffffLL, "frame too large for the grid catalog");
  require(p.grid_cols <= s->width && p.grid_rows <= s->height, "grid finer than the frame");
  for (int64_t k = 0; k < count; ++k) stack_require_loaded(s, indices[k], "grid star catalog");
  stack_activate(s);
  const int cells = p.grid_cols * p.grid_rows;
  const int64_t entries = static_cast<int64_t>(cells) * p.candidates_per_cell;
  require(entries <= (int64_t{1} << 26), "grid_cols * grid_rows * candidates_per_cell is too large");
  int sort_n = 1;
  while (sort_n < entries) sort_n <<= 1;
  const bool shared_sort = sort_n <= kSharedSortMax;
  const int n = static_cast<int>(count);
  const int mo = p.max_output_candidates;

  // one stream-ordered workspace: frames | found | stored | mean | keys | [sort] | pre x,y | flux | x,y | status
  auto align = [](size_t v) { return (v + 255) & ~size_t(255); };
  const size_t off_found = align(sizeof(int) * n);
  const size_t off_stored = off_found + align(sizeof(unsigned) * n);
  const size_t off_mean = off_stored + align(sizeof(int) * n);
  const size_t off_keys = off_mean + align(sizeof(float) * n);
  const size_t off_sort = off_keys + align(sizeof(unsigned long long) * entries * n);
  const size_t off_pre = off_sort + (shared_sort ? 0 : align(sizeof(unsigned long long) * sort_n * n));
  const size_t cat = static_cast<size_t>(n) * mo;
  // catalog planes, each [frame][max_out]: x | y | flux | x before centroid | y before centroid
  const size_t off_status = off_pre + align(sizeof(float) * 5 * cat);
  const size_t total = off_status + align(cat);
  char* ws = nullptr;
  check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&ws), total, s->stream), "cudaMallocAsync(grid catalog)");
  struct Free {
    char* p;
    cudaStream_t st;
    ~Free() { cudaFreeAsync(p, st); }
  } release{ws, s->stream};
  int* d_frames = reinterpret_cast<int*>(ws);
  unsigned* d_found = reinterpret_cast<unsigned*>(ws + off_found);
  int* d_stored = reinterpret_cast<int*>(ws + off_stored);
  float* d_mean = reinterpret_cast<float*>(ws + off_mean);
  auto* d_keys = reinterpret_cast<unsigned long long*>(ws + off_keys);
  auto* d_sort = shared_sort ? nullptr : reinterpret_cast<unsigned long long*>(ws + off_sort);
  float* d_planes = reinterpret_cast<float*>(ws + off_pre);
  float* d_out_x = d_planes;
  float* d_out_y = d_planes + cat;
  float* d_flux = d_planes + 2 * cat;
  float* d_pre_x = d_planes + 3 * cat;
  float* d_pre_y = d_planes + 4 * cat;
  unsigned char* d_status = reinterpret_cast<unsigned char*>(ws + off_status);

  std::vector<int> frames(n);
  for (int k = 0; k < n; ++k) frames[k] = static_cast<int>(indices[k]);
  upload_params(s->stream, d_frames, frames.data(), sizeof(int) * n, "cudaMemcpyAsync(grid catalog frames)");
  check_cuda(cudaMemsetAsync(d_found, 0, sizeof(unsigned) * n, s->stream), "cudaMemsetAsync(grid catalog)");
  check_cuda(cudaMemsetAsync(d_planes, 0, sizeof(float) * 5 * cat, s->stream), "cudaMemsetAsync(grid catalog)");
  check_cuda(cudaMemsetAsync(d_status, 0, cat, s->stream), "cudaMemsetAsync(grid catalog)");

  CellArgs ca{s->d_slots, s->d_slot_of_frame, s->stride, d_frames, static_cast<int>(s->width),
              static_cast<int>(s->height), p.threshold, p.grid_cols, p.grid_rows, p.candidates_per_cell, d_keys,
              d_found};
  note_launch();
  grid_cell_topk_kernel<<<dim3(cells, n), kCellThreads, 0, s->stream>>>(ca);
  check_cuda(cudaGetLastError(), "grid_cell_topk launch");

  SelectArgs sa{d_keys, d_sort, static_cast<int>(entries), sort_n, static_cast<int>(s->width),
                p.min_separation_px * p.min_separation_px, mo, d_pre_x, d_pre_y, d_flux, d_stored};
  const size_t select_smem = (shared_sort ? sizeof(unsigned long long) * sort_n : 0) + sizeof(float2) * mo;
  check_cuda(cudaFuncSetAttribute(catalog_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(select_smem)),
             "cudaFuncSetAttribute(catalog_select)");
  note_launch();
  catalog_select_kernel<<<n, kSelectThreads, select_smem, s->stream>>>(sa);
  check_cuda(cudaGetLastError(), "catalog_select launch");

  if (p.centroid_radius > 0) {
    const float* mean = nullptr;
    if (p.centroid_background == 1) {
      const int blocks = 128;
      stack_ensure_partials(s, static_cast<size_t>(n) * blocks * 3);
      launch_frame_stats_partials(s, d_frames, n, blocks, s->d_partials);
      note_launch();
      frame_mean_kernel<<<n, 32, 0, s->stream>>>(s->d_partials, blocks, n, d_mean);
      check_cuda(cudaGetLastError(), "frame_mean launch");
      mean = d_mean;
    }
    CentroidArgs ce{s->d_slots, s->d_slot_of_frame, s->stride, d_frames, static_cast<int>(s->width),
                    static_cast<int>(s->height), p.centroid_radius, mo, d_pre_x, d_pre_y, d_stored, mean,
                    d_out_x, d_out_y, d_status};
    note_launch();
    catalog_centroid_kernel<<<dim3((mo + kCentroidWarps - 1) / kCentroidWarps, n), 32 * kCentroidWarps, 0,
                              s->stream>>>(ce);
    check_cuda(cudaGetLastError(), "catalog_centroid launch");
  } else {
    check_cuda(cudaMemcpyAsync(d_out_x, d_pre_x, sizeof(float) * 2 * cat, cudaMemcpyDeviceToDevice, s->stream),
               "cudaMemcpyAsync(grid catalog positions)");
  }
  std::vector<unsigned> found(n);
  std::vector<int> stored(n);
  check_cuda(cudaMemcpyAsync(found.data(), d_found, sizeof(unsigned) * n, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(grid catalog counts)");
  check_cuda(cudaMemcpyAsync(stored.data(), d_stored, sizeof(int) * n, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(grid catalog counts)");
  check_cuda(cudaMemcpyAsync(host_catalog, d_planes, sizeof(float) * 5 * cat, cudaMemcpyDeviceToHost, s->stream),
             "cudaMemcpyAsync(grid catalog)");
  if (host_status != nullptr) {
    check_cuda(cudaMemcpyAsync(host_status, d_status, cat, cudaMemcpyDeviceToHost, s->stream),
               "cudaMemcpyAsync(grid catalog status)");
  }
  check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize(grid catalog)");
  for (int k = 0; k < n; ++k) {
    host_counts[2 * k] = static_cast<int32_t>(found[k]);
    host_counts[2 * k + 1] = stored[k];
  }
  GG_API_END
}
