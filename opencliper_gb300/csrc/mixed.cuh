// Shared definitions of the mixed-precision kernels (mixed.cu, and the
// tensor-core row-local iteration in mixed_rowlocal.cu): operand chunking of the
// kept-row DFT operands built by k_build_fk / k_build_fa, status codes and the
// split of FP32 values into fp16 hi + lo parts.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

namespace gbn {

// forward operand (k_build_fk): per frame, chunks of kTcKC real k (kTcHC image
// rows) of [hi | lo][npad x kTcKC], K-major
constexpr int kTcCols = 32;   // columns per CTA tile of k_fwd_cols_tc
constexpr int kTcCoils = 4;   // coils per CTA tile of k_fwd_cols_tc (rows m = coil * 32 + column)
constexpr int kTcKC = 32;     // real k per chunk
constexpr int kTcHC = kTcKC / 2;
constexpr int kTcAPart = 128 * kTcKC * 2;  // bytes of one A part (hi or lo) of a stage
constexpr uint32_t kWaitLimit = 1u << 24;
constexpr int kStatusTcWait = 3;  // NestaDevState::status: a tensor-core wait ran out
constexpr int kStatusTcRows = 4;  // NestaDevState::status: kept rows outgrew the DFT operand

constexpr int kTcStages = 2;  // shared-memory stages (A hi/lo + B hi/lo of one chunk each)

__host__ __device__ constexpr int stage_bytes(int npad) { return 2 * kTcAPart + 2 * npad * kTcKC * 2; }

// adjoint operand (k_build_fa): per frame and 128-row tile of H, chunks of
// kAcKC real k (kAcRows kept rows) of [hi | lo][128 x kAcKC], K-major
constexpr int kAcKC = 64;                  // real k per chunk
constexpr int kAcRows = kAcKC / 2;         // kept rows per chunk
constexpr int kAcCols = 8;                 // columns per CTA of k_inv_cols_tc
constexpr int kAcCoils = 8;                // coils per TMEM pass of k_inv_cols_tc
constexpr int kAcBatch = 2;                // coils combined per TMEM read
constexpr int kAcAPart = 128 * kAcKC * 2;  // bytes of one A part (hi or lo)
__host__ __device__ constexpr int ac_b_part(int n) { return n * kAcKC * 2; }
__host__ __device__ constexpr int ac_smem(int nmax) { return 2 * kAcAPart + 2 * ac_b_part(nmax); }

__device__ __forceinline__ uint32_t as_u32(__half2 h) { return *reinterpret_cast<const uint32_t*>(&h); }

// (re, im) -> hi = fp16 pair, lo = fp16 pair of the remainders (packed, re in
// the low half)
__device__ __forceinline__ void split_pair(float re, float im, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __floats2half2_rn(re, im);
  const float2 hf = __half22float2(h);
  hi = as_u32(h);
  lo = as_u32(__floats2half2_rn(re - hf.x, im - hf.y));
}

}  // namespace gbn
