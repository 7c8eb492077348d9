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
#include "mixed.cuh"

namespace gbn {


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
// k_inv_cols_tc: the adjoint column pass with coil combination, the tTV
// gradient and the Nesterov update (the UPDATE form of k_inv_cols) with the
// column transform on the tensor cores.
//   Y[h, (c, w)] = sum_g exp(+2 pi i row_g h / H) T[g, c, w]       (real form)
//   D[m, n] = sum_k A[m, k] B[n, k],  m = h (128-row tile), k = 2g + p,
//   n = 2 (8 c + w) + q,
//   A[h, 2g] = cos, A[h, 2g+1] = sin                (static per frame, k_build_fa)
//   B[2(8c+w), 2g] = Tr, B[2(8c+w), 2g+1] = -Ti, B[2(8c+w)+1, 2g] = Ti,
//   B[2(8c+w)+1, 2g+1] = Tr                           (formed from T, scaled)
// then x = sum_c conj(S_c) Y_c straight from tensor memory.  A CTA takes one
// frame, 128 rows and 8 columns; coils go through TMEM 8 at a time (N <= 128).
// Operands are split fp16 hi + lo as in k_fwd_cols_tc; B is scaled by a power
// of two from the maximum |T| of the coil group (two passes over T), undone in
// the combination.  K runs in chunks of 32 kept rows (64 real k), one stage.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(128, 3)
    k_inv_cols_tc(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  __shared__ float s_red[4];
  const int inst = find_inst(bm, blockIdx.z);
  const FusedArgs& a = tab[inst];
  NestaDevState* st = a.st;
  const int f = blockIdx.z - bm.fbase[inst], ht = blockIdx.y, w0 = blockIdx.x * kAcCols;
  const int W = a.W, H = a.H, C = a.C, F = a.F;
  if (ht * 128 >= H) return;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int h = ht * 128 + t;
  const bool hrow = h < H;
  const size_t N = size_t(W) * H;
  const int ncg = (C + kAcCoils - 1) / kAcCoils;          // coil groups
  const int cg_n = (C + ncg - 1) / ncg;                   // coils per group (balanced)
  const int nmax = 16 * cg_n;                             // operand rows of a group
  uint32_t ncols = 32;
  while (ncols < uint32_t(nmax)) ncols <<= 1;
  if (warp == 0) {
    tc::tmem_alloc(&tslot, ncols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
  }
  const int nht = (H + 127) / 128, ncha = a.ncha;
  const unsigned char* fa = a.fa + (size_t(f) * nht + ht) * ncha * (2 * kAcAPart);
  auto issue_A = [&](int j) {
    const unsigned char* src = fa + size_t(j) * (2 * kAcAPart);
    for (int q = t; q < 2 * kAcAPart / 16; q += 128) cp_async16(sm + 16 * q, src + 16 * q);
  };
  issue_A(0);
  cp_async_commit();
  const int rowbase = a.rowoff[f], G = a.rowoff[f + 1] - rowbase;
  const int nch = (G + kAcRows - 1) / kAcRows;
  grid_dep_wait();  // T and the scalar state come from the row pass
  grid_dep_release();
  bool active = !(it > st->last_iter);  // uniform over the instance

  unsigned char* sB = sm + 2 * kAcAPart;
  float2 acc[kAcCols];
#pragma unroll
  for (int w = 0; w < kAcCols; ++w) acc[w] = make_float2(0.f, 0.f);
  bool ok = true;
  uint32_t phase = 0;
  for (int cg0 = 0; cg0 < C && active && ok; cg0 += cg_n) {
    const int cn = min(cg_n, C - cg0);
    const int n_rows = 16 * cn;  // operand rows of this group (multiple of 16)
    // pass 1: max |T| over the group's values (power-of-two scale of B)
    float mx = 0.f;
    for (int item = t; item < G * cn * kAcCols; item += 128) {
      const int w = item % kAcCols, c = cg0 + (item / kAcCols) % cn, g = item / (kAcCols * cn);
      const float2 v = a.T[(size_t(rowbase + g) * C + c) * W + w0 + w];
      mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_red[warp] = mx;
    __syncthreads();
    mx = fmaxf(fmaxf(s_red[0], s_red[1]), fmaxf(s_red[2], s_red[3]));
    float sig = 1.f, isig = 1.f;
    if (mx > 0.f) {
      int e;
      frexpf(mx, &e);
      sig = ldexpf(1.f, 14 - e);
      isig = ldexpf(1.f, e - 14);
    }
    const uint32_t idesc = tc::idesc_f16_f32(128, n_rows);
    for (int j = 0; j < nch && ok; ++j) {
      if (j > 0 || (cg0 > 0 && nch > 1)) {  // with one chunk, A stays from the first group
        issue_A(j);
        cp_async_commit();
      }
      // B chunk j: items (c, w, group of 4 kept rows) -> two operand rows x 16 bytes x 2 parts
      const int g0 = j * kAcRows;
      for (int item = t; item < cn * kAcCols * (kAcRows / 4); item += 128) {
        const int w = item % kAcCols, gq = (item / kAcCols) % (kAcRows / 4), cl = item / (kAcCols * (kAcRows / 4));
        uint32_t r0h[4], r0l[4], r1h[4], r1l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int g = g0 + 4 * gq + e;
          float2 v = make_float2(0.f, 0.f);
          if (g < G) v = a.T[(size_t(rowbase + g) * C + cg0 + cl) * W + w0 + w];
          v.x *= sig;
          v.y *= sig;
          uint32_t hp, lp;
          split_pair(v.x, -v.y, hp, lp);  // row q = 0: (Tr, -Ti)
          r0h[e] = hp;
          r0l[e] = lp;
          split_pair(v.y, v.x, hp, lp);   // row q = 1: (Ti, Tr)
          r1h[e] = hp;
          r1l[e] = lp;
        }
        const int n0 = 2 * (cl * kAcCols + w);
        const uint32_t o0 = tc::kmajor_offset(n0, 8 * gq, kAcKC), o1 = tc::kmajor_offset(n0 + 1, 8 * gq, kAcKC);
        *reinterpret_cast<uint4*>(sB + o0) = make_uint4(r0h[0], r0h[1], r0h[2], r0h[3]);
        *reinterpret_cast<uint4*>(sB + ac_b_part(n_rows) + o0) = make_uint4(r0l[0], r0l[1], r0l[2], r0l[3]);
        *reinterpret_cast<uint4*>(sB + o1) = make_uint4(r1h[0], r1h[1], r1h[2], r1h[3]);
        *reinterpret_cast<uint4*>(sB + ac_b_part(n_rows) + o1) = make_uint4(r1l[0], r1l[1], r1l[2], r1l[3]);
      }
      cp_async_wait<0>();
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      if (t == 0) {
        tc::fence_after_sync();
        const uint32_t sa = tc::smem_u32(sm), sb = tc::smem_u32(sB);
#pragma unroll
        for (int ks = 0; ks < kAcKC / 16; ++ks) {
          const uint64_t ahi = tc::smem_desc(sa + ks * 256, 128, kAcKC * 16);
          const uint64_t alo = tc::smem_desc(sa + kAcAPart + ks * 256, 128, kAcKC * 16);
          const uint64_t bhi = tc::smem_desc(sb + ks * 256, 128, kAcKC * 16);
          const uint64_t blo = tc::smem_desc(sb + ac_b_part(n_rows) + ks * 256, 128, kAcKC * 16);
          tc::mma_f16(tslot, ahi, bhi, idesc, j > 0 || ks > 0);
          tc::mma_f16(tslot, alo, bhi, idesc, true);
          tc::mma_f16(tslot, ahi, blo, idesc, true);
        }
        tc::mma_commit(&mbar);
      }
      ok = __syncthreads_and(tc::mbar_wait(&mbar, phase, kWaitLimit) ? 1 : 0) != 0;
      phase ^= 1u;
      tc::fence_after_sync();
    }
    if (!ok) break;
    // x += sum_c conj(S_c) Y_c for this group, from tensor memory, coils in
    // batches of kAcBatch: the next batch's S rows are loaded while the current
    // batch is combined, and a batch's TMEM columns are read with one wait
    const uint32_t taddr = tslot + (uint32_t(32 * warp) << 16);
    const float4* srow = reinterpret_cast<const float4*>(a.S + size_t(h < H ? h : 0) * W + w0);
    const size_t cstride = N / 2;  // float4 per coil plane
    float4 sb[2][kAcBatch][kAcCols / 2];
    auto load_s = [&](int slot, int c_first) {
#pragma unroll
      for (int k = 0; k < kAcBatch; ++k) {
        const int cl = c_first + k;
#pragma unroll
        for (int q = 0; q < kAcCols / 2; ++q)
          sb[slot][k][q] = (hrow && cl < cn) ? __ldg(srow + size_t(cg0 + cl) * cstride + q) : make_float4(0, 0, 0, 0);
      }
    };
    load_s(0, 0);
#pragma unroll
    for (int bi = 0; bi < kAcCoils / kAcBatch; ++bi) {  // unrolled: the buffer slot is a constant
      const int cb = bi * kAcBatch, slot = bi & 1;
      if (cb >= cn) break;
      if (cb + kAcBatch < cn) load_s(slot ^ 1, cb + kAcBatch);
      float v[kAcBatch][16];
#pragma unroll
      for (int k = 0; k < kAcBatch; ++k)
        if (cb + k < cn) tc::tmem_ld16_nowait(taddr + uint32_t(16 * (cb + k)), v[k]);
      tc::tmem_wait_ld();
#pragma unroll
      for (int k = 0; k < kAcBatch; ++k) {
        if (cb + k >= cn) break;
#pragma unroll
        for (int q = 0; q < kAcCols / 2; ++q) {
          const float4 s2 = sb[slot][k][q];
          const float yr0 = v[k][4 * q] * isig, yi0 = v[k][4 * q + 1] * isig;
          const float yr1 = v[k][4 * q + 2] * isig, yi1 = v[k][4 * q + 3] * isig;
          acc[2 * q].x = fmaf(s2.x, yr0, fmaf(s2.y, yi0, acc[2 * q].x));
          acc[2 * q].y = fmaf(s2.x, yi0, fmaf(-s2.y, yr0, acc[2 * q].y));
          acc[2 * q + 1].x = fmaf(s2.z, yr1, fmaf(s2.w, yi1, acc[2 * q + 1].x));
          acc[2 * q + 1].y = fmaf(s2.z, yi1, fmaf(-s2.w, yr1, acc[2 * q + 1].y));
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();  // tensor memory read before the next group's MMAs
    tc::fence_after_sync();
  }
  if (!ok && t == 0) atomicExch(&st->status, kStatusTcWait);

  if (active && ok) {
    // tTV gradient and Nesterov update of this row's 8 pixels (as k_inv_cols)
    const float2* __restrict__ xk = (it & 1) ? a.xk1 : a.xk0;
    float2* __restrict__ xn = (it & 1) ? a.xk0 : a.xk1;
    const float inv_mu = 1.0f / st->mu, lambda = st->lambda, nLmu1 = -st->Lmu1, apk = st->apk, tauk = st->tauk;
    const float omt = 1.0f - tauk, s_adj = a.s_adj;
    float cmx[kAcCols];
    if (hrow) {
      const size_t p0 = size_t(h) * W + w0;
      const size_t off0 = size_t(f) * N + p0, offm = size_t((f + F - 1) % F) * N + p0,
                   offp = size_t((f + 1) % F) * N + p0;
      float2 xa[kAcCols], xm[kAcCols], xp[kAcCols], wo[kAcCols], xr[kAcCols];
#pragma unroll
      for (int q = 0; q < kAcCols / 2; ++q) {
        const float4 va = *reinterpret_cast<const float4*>(xk + off0 + 2 * q);
        const float4 vm = *reinterpret_cast<const float4*>(xk + offm + 2 * q);
        const float4 vp = *reinterpret_cast<const float4*>(xk + offp + 2 * q);
        const float4 vw = *reinterpret_cast<const float4*>(a.wacc + off0 + 2 * q);
        const float4 vr = *reinterpret_cast<const float4*>(a.xref + off0 + 2 * q);
        xa[2 * q] = make_float2(va.x, va.y), xa[2 * q + 1] = make_float2(va.z, va.w);
        xm[2 * q] = make_float2(vm.x, vm.y), xm[2 * q + 1] = make_float2(vm.z, vm.w);
        xp[2 * q] = make_float2(vp.x, vp.y), xp[2 * q + 1] = make_float2(vp.z, vp.w);
        wo[2 * q] = make_float2(vw.x, vw.y), wo[2 * q + 1] = make_float2(vw.z, vw.w);
        xr[2 * q] = make_float2(vr.x, vr.y), xr[2 * q + 1] = make_float2(vr.z, vr.w);
      }
      float2 wn_out[kAcCols], xn_out[kAcCols];
#pragma unroll
      for (int w = 0; w < kAcCols; ++w) {
        const float2 u0 = tv_normalize(csub(xa[w], xm[w]), inv_mu);
        const float2 u1 = tv_normalize(csub(xp[w], xa[w]), inv_mu);
        const float2 adj = csub(u1, u0);
        const float2 ares = cscale(acc[w], s_adj);
        const float2 df = make_float2(__fadd_rn(__fmul_rn(-adj.x, lambda), ares.x),
                                      __fadd_rn(__fmul_rn(-adj.y, lambda), ares.y));
        const float2 yk = make_float2(fmaf(nLmu1, df.x, xa[w].x), fmaf(nLmu1, df.y, xa[w].y));
        const float2 wn = make_float2(fmaf(apk, df.x, wo[w].x), fmaf(apk, df.y, wo[w].y));
        const float2 zk = make_float2(fmaf(nLmu1, wn.x, xr[w].x), fmaf(nLmu1, wn.y, xr[w].y));
        xn_out[w] = make_float2(fmaf(omt, yk.x, tauk * zk.x), fmaf(omt, yk.y, tauk * zk.y));
        wn_out[w] = wn;
        cmx[w] = fmaf(xn_out[w].x, xn_out[w].x, xn_out[w].y * xn_out[w].y);
      }
#pragma unroll
      for (int q = 0; q < kAcCols / 2; ++q) {
        *reinterpret_cast<float4*>(a.wacc + off0 + 2 * q) =
            make_float4(wn_out[2 * q].x, wn_out[2 * q].y, wn_out[2 * q + 1].x, wn_out[2 * q + 1].y);
        *reinterpret_cast<float4*>(xn + off0 + 2 * q) =
            make_float4(xn_out[2 * q].x, xn_out[2 * q].y, xn_out[2 * q + 1].x, xn_out[2 * q + 1].y);
      }
    } else {
#pragma unroll
      for (int w = 0; w < kAcCols; ++w) cmx[w] = 0.f;
    }
    // column maxima of x_{k+1} for the next forward pass (rows of a warp are its lanes)
#pragma unroll
    for (int w = 0; w < kAcCols; ++w) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) cmx[w] = fmaxf(cmx[w], __shfl_xor_sync(0xffffffffu, cmx[w], o));
    }
    if (lane < kAcCols) {
      float m = 0.f;
#pragma unroll
      for (int w = 0; w < kAcCols; ++w)
        if (w == lane) m = cmx[w];
      atomicMax(reinterpret_cast<unsigned int*>(a.colmax) + size_t((it + 1) & 1) * F * W + size_t(f) * W + w0 + lane,
                __float_as_uint(sqrtf(m)));
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tslot, ncols);
  cp_async_wait<0>();
}

// Adjoint kept-row DFT operand of every frame: [frame][h tile][chunk][hi | lo]
// [128 rows x kAcKC], A[h, 2g] = cos, A[h, 2g+1] = sin of 2 pi row_g h / H.
__global__ void k_build_fa(const int* __restrict__ rows_h, const int* __restrict__ rowoff, int F, int H, int ncha,
                           unsigned char* __restrict__ fa) {
  const int nht = (H + 127) / 128;
  const size_t per_chunk = size_t(128) * kAcKC;
  const size_t total = size_t(F) * nht * ncha * per_chunk;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int kk = int(i % kAcKC), r = int((i / kAcKC) % 128);
    const size_t blk = i / per_chunk;  // (f * nht + ht) * ncha + j
    const int j = int(blk % ncha), ht = int((blk / ncha) % nht), f = int(blk / (size_t(ncha) * nht));
    const int h = ht * 128 + r, g = j * kAcRows + kk / 2, p = kk & 1;
    const int base = rowoff[f], G = rowoff[f + 1] - base;
    double v = 0.0;
    if (h < H && g < G) {
      const long long idx = (long long)rows_h[base + g] * h % H;
      double sn, cs;
      sincospi(2.0 * double(idx) / double(H), &sn, &cs);
      v = p == 0 ? cs : sn;
    }
    const __half hi = __double2half(v);
    const __half lo = __double2half(v - double(__half2float(hi)));
    unsigned char* chunk = fa + blk * (2 * per_chunk * 2);
    const uint32_t off = tc::kmajor_offset(r, kk, kAcKC);
    *reinterpret_cast<__half*>(chunk + off) = hi;
    *reinterpret_cast<__half*>(chunk + per_chunk * 2 + off) = lo;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int mixed_prepare(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params& prm, const float2* out) {
  // the tensor-core kernels read S and the image rows with 16-byte vector accesses
  if ((reinterpret_cast<uintptr_t>(P->S) | reinterpret_cast<uintptr_t>(out)) % 16 != 0)
    return set_error(GBN_ERR_INVALID, "mixed precision: sensitivity maps and output must be 16-byte aligned");
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
  // adjoint operand: 128-row tiles of H, chunks of kAcRows kept rows
  const int ncha = std::max(1, (gmax + kAcRows - 1) / kAcRows);
  const size_t fa_bytes = size_t(P->F) * ((P->H + 127) / 128) * ncha * (2 * kAcAPart);
  if (P->fa_bytes < fa_bytes) {
    if (P->fa) cudaFree(P->fa);
    P->fa = nullptr;
    P->fa_bytes = 0;
    if (cudaMalloc(&P->fa, fa_bytes) != cudaSuccess) {
      cudaGetLastError();
      return set_error(GBN_ERR_NOMEM, "mixed precision allocation failed");
    }
    P->fa_bytes = fa_bytes;
  }
  P->npad = npad;
  P->nch = nch;
  P->ncha = ncha;
  P->gmax = gmax;
  return GBN_OK;
}

// coils per TMEM pass of the adjoint kernel for C coils (balanced groups of <= 16)
static int ac_group(int C) {
  const int ncg = (C + kAcCoils - 1) / kAcCoils;
  return (C + ncg - 1) / ncg;
}

int inv_cols_tc_rows(int C) { return 16 * ac_group(C); }

void mixed_args(gbn_problem* P, FusedArgs* a) {
  a->fk = P->fk;
  a->colmax = P->colmax;
  a->smax = P->smax;
  a->npad = P->npad;
  a->nch = P->nch;
  a->fa = P->fa;
  a->ncha = P->ncha;
  a->ntv = P->F * ((P->W + kTcCols - 1) / kTcCols);
}

// after the kept-row analysis: DFT operand and coil-map column maxima
int launch_mixed_setup(gbn_ctx* ctx, gbn_problem* P, cudaStream_t s) {
  const size_t total = size_t(P->F) * P->nch * P->npad * kTcKC;
  k_build_fk<<<int(std::min<size_t>((total + 255) / 256, size_t(ctx->nsm) * 8)), 256, 0, s>>>(
      P->rows_h, P->rowoff, P->F, P->H, P->npad, P->nch, P->fk, &P->st->status);
  k_colmax<<<(P->C * P->W + 127) / 128, 128, 0, s>>>(P->S, P->C, P->H, P->W, P->smax);
  const size_t ta = size_t(P->F) * ((P->H + 127) / 128) * P->ncha * 128 * kAcKC;
  k_build_fa<<<int(std::min<size_t>((ta + 255) / 256, size_t(ctx->nsm) * 8)), 256, 0, s>>>(P->rows_h, P->rowoff, P->F,
                                                                                          P->H, P->ncha, P->fa);
  return 3;
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

dim3 inv_cols_tc_grid(int W, int H, int frames) { return dim3(W / kAcCols, (H + 127) / 128, frames); }

// shared memory for operands of at most nmax rows; as for the forward kernel,
// CTAs that take 256 TMEM columns are kept to two per SM
int inv_cols_tc_smem(int nmax) {
  const int need = ac_smem(nmax);
  return nmax > 128 ? std::max(need, 80 * 1024) : need;
}

void launch_inv_cols_tc(const FusedArgs* tab, const BatchMap& bm, int it, int nmax, dim3 grid, cudaStream_t s) {
  static bool ok = false;
  allow_smem(k_inv_cols_tc, inv_cols_tc_smem(256), ok);
  launch_pdl(k_inv_cols_tc, grid, 128, inv_cols_tc_smem(nmax), s, tab, bm, it);
}

void launch_fwd_cols_tc(const FusedArgs* tab, const BatchMap& bm, int it, int npad_max, dim3 grid, cudaStream_t s) {
  static bool ok = false;
  allow_smem(k_fwd_cols_tc, fwd_cols_tc_smem(256), ok);
  launch_pdl(k_fwd_cols_tc, grid, 128, fwd_cols_tc_smem(npad_max), s, tab, bm, it);
}

}  // namespace gbn
