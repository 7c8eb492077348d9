// Shared device helpers for the tTV-NESTA kernels: complex arithmetic on
// interleaved complex64 (float2), compile-time trigonometry for FFT twiddle
// constants, and a compile-time loop helper.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#define GBN_HD __host__ __device__

namespace gbn {

// ---------------------------------------------------------------------------
// Compile-time trigonometry (double precision).  Used only to bake twiddle
// constants into the register DFT code and to fill host-side twiddle tables.
// Angles are 2*pi*j/n with integer j, n: the argument is reduced exactly on
// integers to the nearest quarter turn, leaving |r| <= pi/4, and sin/cos of the
// remainder come from their Taylor series (25th order, error < 1e-25).
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double cx_sin_taylor(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int i = 1; i < 13; ++i) {
    term *= -x2 / double((2 * i) * (2 * i + 1));
    sum += term;
  }
  return sum;
}

constexpr double cx_cos_taylor(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int i = 1; i < 13; ++i) {
    term *= -x2 / double((2 * i - 1) * (2 * i));
    sum += term;
  }
  return sum;
}

// returns cos(2*pi*j/n) (want_sin == false) or sin(2*pi*j/n) (want_sin == true)
constexpr double cx_trig2pi(long long j, long long n, bool want_sin) {
  j %= n;
  if (j < 0) j += n;
  const long long q = (8 * j + n) / (2 * n);  // nearest quarter turn, 0..4
  const double r = kPi * double(4 * j - q * n) / double(2 * n);
  const double s = cx_sin_taylor(r), c = cx_cos_taylor(r);
  switch (q & 3) {
    case 0: return want_sin ? s : c;
    case 1: return want_sin ? c : -s;
    case 2: return want_sin ? -s : -c;
    default: return want_sin ? -c : s;
  }
}
constexpr double cx_cos2pi(long long j, long long n) { return cx_trig2pi(j, n, false); }
constexpr double cx_sin2pi(long long j, long long n) { return cx_trig2pi(j, n, true); }

// ---------------------------------------------------------------------------
// Compile-time loop: f(std::integral_constant<int, i>) for i in [B, E)
// ---------------------------------------------------------------------------
template <int B, int E, typename F>
GBN_HD __forceinline__ void sfor(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    sfor<B + 1, E>(static_cast<F&&>(f));
  }
}

// ---------------------------------------------------------------------------
// complex64 helpers
// ---------------------------------------------------------------------------
GBN_HD __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
GBN_HD __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
GBN_HD __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// Packed forms of cadd and csub: one FP32x2 instruction on sm_100 and later.
// Each lane rounds as the scalar operation does (a - b is a + (-b) in IEEE
// arithmetic), so the results are identical.
GBN_HD __forceinline__ float2 padd(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  return __fadd2_rn(a, b);
#else
  return cadd(a, b);
#endif
}
GBN_HD __forceinline__ float2 psub(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  return __fadd2_rn(a, make_float2(-b.x, -b.y));
#else
  return csub(a, b);
#endif
}
// a * b
GBN_HD __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
GBN_HD __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
// multiply by -i (forward-direction quarter turn) or +i
GBN_HD __forceinline__ float2 cmul_negi(float2 a) { return make_float2(a.y, -a.x); }
GBN_HD __forceinline__ float2 cmul_posi(float2 a) { return make_float2(-a.y, a.x); }

GBN_HD __forceinline__ float cabs2(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }

// ---------------------------------------------------------------------------
// Block-wide sum of one double per thread (all threads must call).  Returns the
// total in thread 0.  Warp partials are combined in a fixed order, so the
// result is deterministic for a fixed launch shape.
// ---------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sred /* >= NT/32 */) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sred[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NT / 32; ++i) t += sred[i];
  }
  return t;
}

// ---------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async, 16-byte granules).  Both
// addresses must be 16-byte aligned.  Copies issued between two commits form
// one group; wait<N> blocks until at most N groups are still in flight.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gmem_src) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace gbn
