// Mixed-precision form: the forward column transform on the tensor cores.
//
// k_fwd_cols_tc computes the same T = DFT_H(S_c x_f) on the kept k-space rows
// as k_fwd_cols, as a GEMM with split-precision fp16 operands and FP32
// accumulation in tensor memory:
//   D[m, n] = sum_k A[m, k] B[n, k]
//   m = (coil, column) of a CTA tile (4 coils x 32 columns = 128 rows),
//   k = 2h + {0: real, 1: imaginary} (K = 2H),
//   n = 2g + {0: real, 1: imaginary} of kept row g of the frame (N = 2G, padded
//       to a multiple of 16),
//   A[m, 2h + p] = the p part of sigma_m * x_f[h, w] S_c[h, w],
//   B = the real form of the kept rows of the DFT matrix, w^(row_g * h):
//       B[2g, 2h] = cos, B[2g, 2h+1] = -sin, B[2g+1, 2h] = sin, B[2g+1, 2h+1] = cos.
// Each operand is split into fp16 hi + lo parts (hi = fp16(v), lo = fp16(v - hi),
// 22 significant bits together) and D accumulates A_hi B_hi + A_lo B_hi +
// A_hi B_lo; the dropped A_lo B_lo term is below 2^-22 of the product.  The row
// scale sigma_m is a power of two chosen from the column maximum of |x_f| and of
// |S_c| so that every |A| < 2^14 (fp16 range) and is undone exactly in the
// epilogue.  B is prebuilt per frame (k_build_fk, double-precision twiddles) in
// the tensor core's K-major core-matrix layout, chunk by chunk, so each chunk is
// one contiguous copy.
//
// Pipeline per CTA: K runs in chunks of 16 values of h (32 real k) through
// two shared-memory stages; while the tensor core multiplies chunk j the
// threads form chunk j+1's A operand from prefetched x and S, and the B chunk
// is copied one chunk ahead.  One
// thread issues the MMAs; tcgen05.commit signals the stage's mbarrier.  All
// waits are bounded; a wait that runs out sets the instance's status and the
// CTA skips its output.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.h"
#include "inst.cuh"
#include "solver.h"
#include "tc.cuh"

namespace gbn {

namespace {

constexpr int kTcCols = 32;   // columns per CTA tile
constexpr int kTcCoils = 4;   // coils per CTA tile (rows m = coil * 32 + column)
constexpr int kTcKC = 32;     // real k per chunk
constexpr int kTcHC = kTcKC / 2;
constexpr int kTcAPart = 128 * kTcKC * 2;  // bytes of one A part (hi or lo) of a stage
constexpr uint32_t kWaitLimit = 1u << 24;
constexpr int kStatusTcWait = 3;  // NestaDevState::status: a tensor-core wait ran out
constexpr int kStatusTcRows = 4;  // NestaDevState::status: kept rows outgrew the DFT operand

constexpr int kTcStages = 2;  // shared-memory stages (A hi/lo + B hi/lo of one chunk each)

__host__ __device__ constexpr int stage_bytes(int npad) { return 2 * kTcAPart + 2 * npad * kTcKC * 2; }

__device__ __forceinline__ uint32_t as_u32(__half2 h) { return *reinterpret_cast<const uint32_t*>(&h); }

// (re, im) -> hi = fp16 pair, lo = fp16 pair of the remainders (packed, re in
// the low half)
__device__ __forceinline__ void split_pair(float re, float im, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __floats2half2_rn(re, im);
  const float2 hf = __half22float2(h);
  hi = as_u32(h);
  lo = as_u32(__floats2half2_rn(re - hf.x, im - hf.y));
}

}  // namespace

__global__ void __launch_bounds__(128, 4)
    k_fwd_cols_tc(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar[kTcStages];
  __shared__ uint32_t tslot;
  const int inst = find_inst(bm, blockIdx.z);
  const FusedArgs& a = tab[inst];
  NestaDevState* st = a.st;
  const int f = blockIdx.z - bm.fbase[inst], cg = blockIdx.y, w0 = blockIdx.x * kTcCols;
  const int W = a.W, H = a.H, C = a.C, F = a.F;
  const int c0 = cg * kTcCoils;
  if (c0 >= C || it > st->last_iter) return;
  const int npad = a.npad, nch = a.nch;
  const int sbytes = stage_bytes(npad);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int c = c0 + warp, w = w0 + lane;
  const bool valid = (c < C) && (w < W);
  const size_t N = size_t(W) * H;
  uint32_t ncols = 32;
  while (ncols < uint32_t(npad)) ncols <<= 1;

  if (warp == 0) {
    tc::tmem_alloc(&tslot, ncols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    for (int i = 0; i < kTcStages; ++i) tc::mbar_init(&mbar[i], 1);
    tc::fence_mbar_init();
  }
  // B chunks of this frame: [chunk][hi | lo][npad x kTcKC K-major]
  const unsigned char* fk = a.fk + size_t(f) * nch * (2 * npad * kTcKC * 2);
  auto issue_B = [&](int j, int s) {
    const unsigned char* src = fk + size_t(j) * (2 * npad * kTcKC * 2);
    unsigned char* dst = sm + s * sbytes + 2 * kTcAPart;
    for (int q = t; q < npad * kTcKC * 4 / 16; q += 128) cp_async16(dst + 16 * q, src + 16 * q);
  };
  issue_B(0, 0);
  cp_async_commit();
  const int rowbase = a.rowoff[f], G = a.rowoff[f + 1] - rowbase;
  grid_dep_wait();  // x_k and its column maxima come from the previous adjoint column pass
  grid_dep_release();

  // row scale: |x S| < 2^14 for this (coil, column)
  float sig = 1.f, isig = 1.f;
  if (valid) {
    const float p = a.colmax[size_t(it & 1) * F * W + size_t(f) * W + w] * a.smax[size_t(c) * W + w];
    if (p > 0.f) {
      int e;
      frexpf(p, &e);
      sig = ldexpf(1.f, 14 - e);
      isig = ldexpf(1.f, e - 14);
    }
  }
  // the next iteration's column maxima are accumulated by this iteration's adjoint pass
  if (cg == 0 && warp == 0 && w < W) a.colmax[size_t((it + 1) & 1) * F * W + size_t(f) * W + w] = 0.f;

  const float2* __restrict__ xk = (it & 1) ? a.xk1 : a.xk0;
  const size_t wc = size_t(valid ? w : 0);
  const float2* __restrict__ xcol = xk + size_t(f) * N + wc;                 // x_f[., w]
  const float2* __restrict__ xmcol = xk + size_t((f + F - 1) % F) * N + wc;  // x_{f-1}[., w]
  const float2* __restrict__ scol = a.S + size_t(valid ? c : 0) * N + wc;    // S_c[., w]
  // tTV partial sums (coil group 0): d = x_f - x_{f-1} over this column; warp k
  // takes the rows q = k (mod 4) of every chunk, so the four warps share it
  const bool tv = (cg == 0) && (w < W);
  const float inv_mu = 1.0f / st->mu;
  float su2 = 0.f, sud = 0.f;

  float2 px[kTcHC], ps[kTcHC], pt[kTcHC / 4], pm[kTcHC / 4];
  auto prefetch = [&](int j) {
    const int h0 = j * kTcHC;
#pragma unroll
    for (int q = 0; q < kTcHC; ++q) {
      const bool in = valid && (h0 + q < H);
      px[q] = in ? xcol[size_t(h0 + q) * W] : make_float2(0.f, 0.f);
      ps[q] = in ? scol[size_t(h0 + q) * W] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int e = 0; e < kTcHC / 4; ++e) {
      const int h = h0 + 4 * e + warp;
      const bool in = tv && h < H;
      pt[e] = in ? xcol[size_t(h) * W] : make_float2(0.f, 0.f);  // an L1 hit: the same row is in px
      pm[e] = in ? xmcol[size_t(h) * W] : make_float2(0.f, 0.f);
    }
  };
  prefetch(0);
  const uint32_t idesc = tc::idesc_f16_f32(128, npad);
  // chunk j uses stage j % 2; MMA(j) signals mbar[j % 2] (its (j / 2)-th
  // completion).  A(j) goes into stage j % 2 once MMA(j-2) is done (waited for
  // in chunk j-1); after forming it, MMA(j-1) is waited for and B(j+1) is
  // copied into the other stage, one chunk ahead of its use.
  bool ok = true;
  for (int j = 0; j < nch; ++j) {
    const int s = j & 1;
    unsigned char* stg = sm + s * sbytes;
    if (tv) {
#pragma unroll
      for (int e = 0; e < kTcHC / 4; ++e) {
        if (j * kTcHC + 4 * e + warp < H) {
          const float2 d = csub(pt[e], pm[e]);
          const float2 u = tv_normalize(d, inv_mu);
          su2 = fmaf(u.x, u.x, fmaf(u.y, u.y, su2));
          sud = fmaf(u.x, d.x, fmaf(u.y, d.y, sud));
        }
      }
    }
    // A operand of chunk j: 4 core-matrix K groups of 4 complex values each
#pragma unroll
    for (int gi = 0; gi < kTcKC / 8; ++gi) {
      uint32_t hw[4], lw[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 v = cmul(px[4 * gi + e], ps[4 * gi + e]);
        split_pair(v.x * sig, v.y * sig, hw[e], lw[e]);
      }
      const uint32_t off = tc::kmajor_offset(t, 8 * gi, kTcKC);
      *reinterpret_cast<uint4*>(stg + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
      *reinterpret_cast<uint4*>(stg + kTcAPart + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    }
    if (j + 1 < nch) prefetch(j + 1);
    if (j >= 1) ok = ok && tc::mbar_wait(&mbar[(j - 1) & 1], ((j - 1) >> 1) & 1, kWaitLimit);
    if (j + 1 < nch && ok) issue_B(j + 1, (j + 1) & 1);
    cp_async_commit();
    cp_async_wait<1>();  // B(j) has landed; B(j+1) may still be in flight
    tc::fence_proxy_async();
    tc::fence_before_sync();
    if (__syncthreads_and(ok ? 1 : 0) == 0) {
      ok = false;
      break;
    }
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t sa = tc::smem_u32(stg), sb = sa + 2 * kTcAPart;
      const uint32_t bpart = uint32_t(npad) * kTcKC * 2;
#pragma unroll
      for (int ks = 0; ks < kTcKC / 16; ++ks) {
        const uint64_t ahi = tc::smem_desc(sa + ks * 256, 128, kTcKC * 16);
        const uint64_t alo = tc::smem_desc(sa + kTcAPart + ks * 256, 128, kTcKC * 16);
        const uint64_t bhi = tc::smem_desc(sb + ks * 256, 128, kTcKC * 16);
        const uint64_t blo = tc::smem_desc(sb + bpart + ks * 256, 128, kTcKC * 16);
        tc::mma_f16(tslot, ahi, bhi, idesc, j > 0 || ks > 0);
        tc::mma_f16(tslot, alo, bhi, idesc, true);
        tc::mma_f16(tslot, ahi, blo, idesc, true);
      }
      tc::mma_commit(&mbar[s]);
    }
  }
  cp_async_wait<0>();
  if (ok) ok = tc::mbar_wait(&mbar[(nch - 1) & 1], ((nch - 1) >> 1) & 1, kWaitLimit);
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  tc::fence_after_sync();
  if (ok) {
    const uint32_t taddr = tslot + (uint32_t(32 * warp) << 16);
    float2* __restrict__ T = a.T;
    for (int col0 = 0; col0 < npad; col0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + uint32_t(col0), v);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int g = col0 / 2 + i;
        if (valid && g < G) T[(size_t(rowbase + g) * C + c) * W + w] = make_float2(v[2 * i] * isig, v[2 * i + 1] * isig);
      }
    }
  } else if (t == 0) {
    atomicExch(&st->status, kStatusTcWait);
  }
  if (cg == 0) {  // block-uniform
    __shared__ double red[2][4];
    double d2 = double(su2), dd = double(sud);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      d2 += __shfl_down_sync(0xffffffffu, d2, o);
      dd += __shfl_down_sync(0xffffffffu, dd, o);
    }
    if (lane == 0) {
      red[0][warp] = d2;
      red[1][warp] = dd;
    }
    __syncthreads();
    if (t == 0) {
      const int blk = f * gridDim.x + blockIdx.x;
      a.part_tv[2 * blk] = ((red[0][0] + red[0][1]) + red[0][2]) + red[0][3];
      a.part_tv[2 * blk + 1] = ((red[1][0] + red[1][1]) + red[1][2]) + red[1][3];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tslot, ncols);
}

// Kept-row DFT operand of every frame (see above), hi and lo parts.
// A frame with more kept rows than the operand was sized for (at batch
// creation) sets the instance's status instead of being truncated silently.
__global__ void k_build_fk(const int* __restrict__ rows_h, const int* __restrict__ rowoff, int F, int H, int npad,
                           int nch, unsigned char* __restrict__ fk, int* __restrict__ status) {
  const size_t per_chunk = size_t(npad) * kTcKC;  // elements of one part
  const size_t total = size_t(F) * nch * per_chunk;
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < F; f += gridDim.x * blockDim.x)
    if (2 * (rowoff[f + 1] - rowoff[f]) > npad) atomicExch(status, kStatusTcRows);
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int kk = int(i % kTcKC), n = int((i / kTcKC) % npad);
    const int j = int((i / per_chunk) % nch), f = int(i / (per_chunk * nch));
    const int h = j * kTcHC + kk / 2, p = kk & 1, g = n / 2, q = n & 1;
    const int base = rowoff[f], G = rowoff[f + 1] - base;
    double v = 0.0;
    if (h < H && g < G) {
      const long long idx = (long long)rows_h[base + g] * h % H;
      double sn, cs;
      sincospi(2.0 * double(idx) / double(H), &sn, &cs);
      sn = -sn;  // forward transform: w = exp(-2 pi i idx / H)
      v = (q == 0) ? (p == 0 ? cs : -sn) : (p == 0 ? sn : cs);
    }
    const __half hi = __double2half(v);
    const __half lo = __double2half(v - double(__half2float(hi)));
    unsigned char* chunk = fk + (size_t(f) * nch + j) * (2 * per_chunk * 2);
    const uint32_t off = tc::kmajor_offset(n, kk, kTcKC);
    *reinterpret_cast<__half*>(chunk + off) = hi;
    *reinterpret_cast<__half*>(chunk + per_chunk * 2 + off) = lo;
  }
}

// out[r * W + w] = max_h |in[(r * H + h) * W + w]|, for R planes (one thread per (r, w))
__global__ void k_colmax(const float2* __restrict__ in, int R, int H, int W, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= R * W) return;
  const int r = i / W, w = i % W;
  const float2* p = in + size_t(r) * H * W + w;
  float m = 0.f;
  for (int h = 0; h < H; ++h) {
    const float2 v = p[size_t(h) * W];
    m = fmaxf(m, sqrtf(fmaf(v.x, v.x, v.y * v.y)));
  }
  out[i] = m;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int mixed_prepare(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params& prm) {
  // kept rows of the current y and mask (the padded operand width is fixed here)
  cudaStream_t s = ctx->stream;
  ctx->launches += launch_pre(P, prm, s);
  std::vector<int> off(P->F + 1);
  cudaError_t e = cudaMemcpyAsync(off.data(), P->rowoff, sizeof(int) * (P->F + 1), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "mixed precision setup");
  int gmax = 0;
  for (int f = 0; f < P->F; ++f) gmax = std::max(gmax, off[f + 1] - off[f]);
  const int npad = std::max(16, (2 * gmax + 15) / 16 * 16);
  if (npad > 256)
    return set_error(GBN_ERR_UNSUPPORTED, "mixed precision: more than 128 kept rows in a frame (got " +
                                              std::to_string(gmax) + ")");
  const int nch = (P->H + kTcHC - 1) / kTcHC;
  const size_t fk_bytes = size_t(P->F) * nch * 2 * npad * kTcKC * 2;
  if (P->fk_bytes < fk_bytes) {
    if (P->fk) cudaFree(P->fk);
    P->fk = nullptr;
    P->fk_bytes = 0;
    if (cudaMalloc(&P->fk, fk_bytes) != cudaSuccess) {
      cudaGetLastError();
      return set_error(GBN_ERR_NOMEM, "mixed precision allocation failed");
    }
    P->fk_bytes = fk_bytes;
  }
  if (!P->colmax) {
    if (cudaMalloc(&P->colmax, sizeof(float) * 2 * P->F * P->W) != cudaSuccess ||
        cudaMalloc(&P->smax, sizeof(float) * P->C * P->W) != cudaSuccess) {
      cudaGetLastError();
      return set_error(GBN_ERR_NOMEM, "mixed precision allocation failed");
    }
  }
  P->npad = npad;
  P->nch = nch;
  return GBN_OK;
}

void mixed_args(gbn_problem* P, FusedArgs* a) {
  a->fk = P->fk;
  a->colmax = P->colmax;
  a->smax = P->smax;
  a->npad = P->npad;
  a->nch = P->nch;
  a->ntv = P->F * ((P->W + kTcCols - 1) / kTcCols);
}

// after the kept-row analysis: DFT operand and coil-map column maxima
int launch_mixed_setup(gbn_ctx* ctx, gbn_problem* P, cudaStream_t s) {
  const size_t total = size_t(P->F) * P->nch * P->npad * kTcKC;
  k_build_fk<<<int(std::min<size_t>((total + 255) / 256, size_t(ctx->nsm) * 8)), 256, 0, s>>>(
      P->rows_h, P->rowoff, P->F, P->H, P->npad, P->nch, P->fk, &P->st->status);
  k_colmax<<<(P->C * P->W + 127) / 128, 128, 0, s>>>(P->S, P->C, P->H, P->W, P->smax);
  return 2;
}

// after an outer-loop start (x_k = x_ref): column maxima of x_k for iteration 0
int launch_mixed_colmax(gbn_problem* P, cudaStream_t s) {
  k_colmax<<<(P->F * P->W + 127) / 128, 128, 0, s>>>(P->xk0, P->F, P->H, P->W, P->colmax);
  return 1;
}

dim3 fwd_cols_tc_grid(int W, int maxC, int frames) {
  return dim3((W + kTcCols - 1) / kTcCols, (maxC + kTcCoils - 1) / kTcCoils, frames);
}

// Dynamic shared memory of a launch whose instances have operands of at most
// npad_max rows: two stages, and at least enough that the CTAs resident on
// an SM never ask for more than its 512 TMEM columns (two CTAs of 256 columns).
int fwd_cols_tc_smem(int npad_max) {
  const int need = stage_bytes(npad_max) * kTcStages;
  return npad_max > 128 ? std::max(need, 80 * 1024) : need;
}

void launch_fwd_cols_tc(const FusedArgs* tab, const BatchMap& bm, int it, int npad_max, dim3 grid, cudaStream_t s) {
  static bool ok = false;
  allow_smem(k_fwd_cols_tc, fwd_cols_tc_smem(256), ok);
  launch_pdl(k_fwd_cols_tc, grid, 128, fwd_cols_tc_smem(npad_max), s, tab, bm, it);
}

}  // namespace gbn
