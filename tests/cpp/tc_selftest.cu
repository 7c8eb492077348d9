// Self-test of the tcgen05 building blocks (opencliper_gb300/csrc/tc.cuh):
// one CTA stages fp16 A (128 x K) and B (N x K) in the K-major core-matrix
// layout, issues K/16 kind::f16 MMAs into a TMEM accumulator, and reads it back
// with tcgen05.ld; the result is compared with a double-precision GEMM of the
// same fp16 values on the host.  Every wait is bounded; a wait that runs out
// is reported as a failure.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tc.cuh"

using namespace gbn;

template <int N, int KC>
__global__ void __launch_bounds__(128) k_gemm(const __half* __restrict__ A, const __half* __restrict__ B,
                                              float* __restrict__ D, int* __restrict__ err) {
  constexpr uint32_t NCOLS = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm;
  unsigned char* sB = sm + 128 * KC * 2;
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  const int t = threadIdx.x, warp = t >> 5;
  for (int i = t; i < 128 * KC; i += 128)
    *reinterpret_cast<__half*>(sA + tc::kmajor_offset(i / KC, i % KC, KC)) = A[i];
  for (int i = t; i < N * KC; i += 128)
    *reinterpret_cast<__half*>(sB + tc::kmajor_offset(i / KC, i % KC, KC)) = B[i];
  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOLS);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  if (t == 0) {
    constexpr uint32_t idesc = tc::idesc_f16_f32(128, N);
    for (int ks = 0; ks < KC / 16; ++ks) {
      const uint64_t ad = tc::smem_desc(tc::smem_u32(sA) + ks * 256, 128, KC * 16);
      const uint64_t bd = tc::smem_desc(tc::smem_u32(sB) + ks * 256, 128, KC * 16);
      tc::mma_f16(taddr, ad, bd, idesc, ks > 0);
    }
    tc::mma_commit(&mbar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait(&mbar, 0, 1u << 22) ? 1 : 0);
  tc::fence_after_sync();
  if (ok) {
    float v[16];
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      tc::tmem_ld16(taddr + (uint32_t(32 * warp) << 16) + uint32_t(c0), v);
#pragma unroll
      for (int j = 0; j < 16; ++j) D[t * N + c0 + j] = v[j];
    }
  } else if (t == 0) {
    atomicExch(err, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOLS);
}

template <int N, int KC>
bool run_case(unsigned seed) {
  std::vector<__half> A(128 * KC), B(N * KC);
  std::vector<float> Af(A.size()), Bf(B.size());
  srand(seed);
  for (size_t i = 0; i < A.size(); ++i) {
    A[i] = __float2half(float(rand()) / RAND_MAX * 2.f - 1.f);
    Af[i] = __half2float(A[i]);
  }
  for (size_t i = 0; i < B.size(); ++i) {
    B[i] = __float2half(float(rand()) / RAND_MAX * 2.f - 1.f);
    Bf[i] = __half2float(B[i]);
  }
  __half *dA, *dB;
  float* dD;
  int* derr;
  cudaMalloc(&dA, A.size() * 2);
  cudaMalloc(&dB, B.size() * 2);
  cudaMalloc(&dD, 128 * N * 4);
  cudaMalloc(&derr, 4);
  cudaMemcpy(dA, A.data(), A.size() * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B.data(), B.size() * 2, cudaMemcpyHostToDevice);
  cudaMemset(dD, 0, 128 * N * 4);
  cudaMemset(derr, 0, 4);
  const int smem = (128 + N) * KC * 2;
  cudaFuncSetAttribute(k_gemm<N, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_gemm<N, KC><<<1, 128, smem>>>(dA, dB, dD, derr);
  cudaError_t e = cudaDeviceSynchronize();
  std::vector<float> D(128 * N);
  int herr = 0;
  cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(derr);
  if (e != cudaSuccess || herr) {
    printf("case N=%d K=%d: %s%s\n", N, KC, cudaGetErrorString(e), herr ? " (mbarrier wait ran out)" : "");
    return false;
  }
  double maxerr = 0, maxref = 0;
  for (int m = 0; m < 128; ++m)
    for (int n = 0; n < N; ++n) {
      double r = 0;
      for (int k = 0; k < KC; ++k) r += double(Af[m * KC + k]) * double(Bf[n * KC + k]);
      maxerr = std::fmax(maxerr, std::fabs(r - D[m * N + n]));
      maxref = std::fmax(maxref, std::fabs(r));
    }
  const double rel = maxerr / maxref;
  printf("case N=%d K=%d: max|D| %.3f max rel err %.3e %s\n", N, KC, maxref, rel, rel < 1e-5 ? "ok" : "FAIL");
  return rel < 1e-5;
}

// An mbarrier that nothing arrives at: the bounded wait gives up and reports
// it instead of hanging the CTA.
__global__ void k_wait_gives_up(int* __restrict__ out) {
  __shared__ uint64_t mbar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  const bool done = tc::mbar_wait(&mbar, 0, 1000);
  if (threadIdx.x == 0) *out = done ? 1 : 2;
}

bool run_wait_case() {
  int* d;
  int h = 0;
  cudaMalloc(&d, 4);
  cudaMemset(d, 0, 4);
  k_wait_gives_up<<<1, 32>>>(d);
  const cudaError_t e = cudaDeviceSynchronize();
  cudaMemcpy(&h, d, 4, cudaMemcpyDeviceToHost);
  cudaFree(d);
  const bool ok = e == cudaSuccess && h == 2;
  printf("bounded wait on an mbarrier nobody completes: %s\n", ok ? "gave up, ok" : "FAIL");
  return ok;
}

int main() {
  bool ok = run_wait_case();
  ok &= run_case<16, 32>(1);
  ok &= run_case<64, 64>(2);
  ok &= run_case<128, 128>(3);
  ok &= run_case<256, 32>(4);
  printf(ok ? "ALL OK\n" : "FAILED\n");
  return ok ? 0 : 1;
}
