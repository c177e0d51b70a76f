// Shared device/host helpers for the GB300 resident light-stack library.
//
// Everything here is internal to libglass_gb300.so; the public surface is
// include/glass_gb300.h.  Error handling follows one rule: no C++ exception
// ever crosses the C ABI.  Internal code throws gg::Error, and every exported
// function wraps its body in GG_API_BEGIN / GG_API_END, which converts the
// exception into an int status plus a thread-local message.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "../../include/glass_gb300.h"

// Frames handled by one calibration launch (frame indices travel by value).
#define GG_MAX_BATCH_FRAMES 8

namespace gg {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

void set_last_error(int code, const char* msg);

[[noreturn]] inline void fail(int code, const std::string& msg) { throw Error(code, msg); }

inline void require(bool ok, const std::string& msg) {
  if (!ok) fail(GG_ERR_INVALID_ARGUMENT, msg);
}

inline void check_cuda(cudaError_t err, const char* what) {
  if (err != cudaSuccess) {
    const int code = (err == cudaErrorMemoryAllocation) ? GG_ERR_OUT_OF_MEMORY : GG_ERR_CUDA;
    fail(code, std::string(what) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) + ")");
  }
}

// Process-wide count of kernels this library has launched (gg_kernel_launches).
void note_launch(int n = 1);
long long launch_count();

// Stream-ordered host-to-device copy of a small block (launch descriptors,
// frame lists, per-frame priors) that keeps off the copy engines: up to
// kParamUploadMax bytes travel in the launch parameters of a one-CTA kernel,
// larger blocks fall back to cudaMemcpyAsync.  A copy-engine copy on the stack
// stream queues behind bulk copies already submitted to the same engine by
// another stream (the next step's raw frames on the copy stream), so a stage
// that needs a few hundred bytes of parameters would otherwise wait for
// gigabytes of unrelated upload.  The host block may be reused as soon as the
// call returns.
constexpr std::size_t kParamUploadMax = 64 * 1024;
void upload_params(cudaStream_t stream, void* dst, const void* src, std::size_t bytes, const char* what);

// Grid sizing for streaming kernels: a whole number of waves over the SMs.
int sm_count();
inline unsigned grid_for(std::size_t work_items, int threads, int ctas_per_sm = 8) {
  std::size_t blocks = (work_items + threads - 1) / threads;
  const std::size_t cap = static_cast<std::size_t>(sm_count()) * ctas_per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  return static_cast<unsigned>(blocks);
}

}  // namespace gg

#define GG_API_BEGIN try {
#define GG_API_END                                        \
  }                                                       \
  catch (const gg::Error& e) {                            \
    gg::set_last_error(e.code, e.what());                 \
    return e.code;                                        \
  }                                                       \
  catch (const std::bad_alloc&) {                         \
    gg::set_last_error(GG_ERR_OUT_OF_MEMORY, "host allocation failed"); \
    return GG_ERR_OUT_OF_MEMORY;                          \
  }                                                       \
  catch (const std::exception& e) {                       \
    gg::set_last_error(GG_ERR_RUNTIME, e.what());         \
    return GG_ERR_RUNTIME;                                \
  }                                                       \
  gg::set_last_error(GG_OK, "");                          \
  return GG_OK;

// ---------------------------------------------------------------------------
// Device arithmetic.  Every rounding step is spelled out with _rn intrinsics so
// that nvcc cannot contract a multiply and an add into an FMA: the CPU
// reference (NumPy) rounds after every operation and the rejection masks are
// required to agree bit for bit.
// ---------------------------------------------------------------------------
namespace gg {

__device__ __forceinline__ bool finitef(float v) { return isfinite(v); }

// Error-free transformation of a sum (Knuth TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Compensated ("float-float") accumulator.  hi + lo carries about 48
// significant bits, which is what the NumPy float64 sums of float32 samples
// need so that the final float32 rounding agrees.
struct FF {
  float hi = 0.0f;
  float lo = 0.0f;
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  // Adds an exact product a*b (TwoProd through one FMA).
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    add(p);
    lo = __fadd_rn(lo, pe);
  }
  __device__ __forceinline__ float value_f32() const { return __fadd_rn(hi, lo); }
};

// round_f32((hi + lo) / d) for a float32 denominator d (d > 0).
__device__ __forceinline__ float ff_div_f32(float hi, float lo, float d) {
  const float q = __fdiv_rn(hi, d);
  const float r = __fadd_rn(__fmaf_rn(-q, d, hi), lo);
  return __fadd_rn(q, __fdiv_rn(r, d));
}

// (hi + lo) / d as an unevaluated pair (q, ql): q + ql approximates the
// quotient to about 48 bits.
__device__ __forceinline__ void ff_div_pair(float hi, float lo, float d, float& q, float& ql) {
  q = __fdiv_rn(hi, d);
  const float r = __fadd_rn(__fmaf_rn(-q, d, hi), lo);
  ql = __fdiv_rn(r, d);
}

// round_f32((nh + nl) / (dh + dl)), dh > 0.
__device__ __forceinline__ float ff_div_ff(float nh, float nl, float dh, float dl) {
  const float q = __fdiv_rn(nh, dh);
  float r = __fmaf_rn(-q, dh, nh);
  r = __fadd_rn(r, nl);
  r = __fmaf_rn(-q, dl, r);
  return __fadd_rn(q, __fdiv_rn(r, dh));
}

// round_f32(sqrt(q + ql)) for q + ql >= 0.
__device__ __forceinline__ float ff_sqrt_f32(float q, float ql) {
  if (!(q > 0.0f)) {
    const float t = __fadd_rn(q, ql);
    return t > 0.0f ? __fsqrt_rn(t) : (t == 0.0f ? 0.0f : __fsqrt_rn(t));
  }
  const float s = __fsqrt_rn(q);
  const float e = __fadd_rn(__fmaf_rn(-s, s, q), ql);
  return __fadd_rn(s, __fdiv_rn(e, __fmul_rn(2.0f, s)));
}

// Squared deviation (x - (mh + ml))^2 accumulated into acc with ~48-bit
// precision.  The deviation is formed exactly by TwoSum and then squared by
// TwoProd plus the cross term.
__device__ __forceinline__ void ff_add_sqdev(FF& acc, float x, float mh, float ml) {
  float d, de;
  two_sum(x, -mh, d, de);
  de = __fsub_rn(de, ml);
  const float p = __fmul_rn(d, d);
  const float pe = __fmaf_rn(d, d, -p);
  acc.add(p);
  acc.lo = __fadd_rn(acc.lo, __fmaf_rn(__fmul_rn(2.0f, d), de, pe));
}

// Warp-aggregated counter increment (one atomic per warp).
__device__ __forceinline__ void warp_count_add(unsigned int* counter, bool pred) {
  const unsigned active = __activemask();
  const unsigned mask = __ballot_sync(active, pred);
  const int leader = __ffs(active) - 1;
  if ((threadIdx.x & 31) == leader && mask != 0u) atomicAdd(counter, static_cast<unsigned>(__popc(mask)));
}

}  // namespace gg
