// Mixed-precision row-local iteration: the inner iteration of rowlocal.cuh
// (one kernel per iteration for problems whose kept k-space rows are fully
// sampled or unsampled) with both column transforms on the tensor cores.
//
// For frame f and the 8 image columns w0..w0+7 of a CTA, with the coils taken
// in groups of cn (pairs p = (coil c, column w), p = 8 c_local + w):
//
//  1. forward GEMM (as k_fwd_cols_tc):
//       D1[p, 2j + q] = sum_{h, r} A1[p, 2h + r] B1[2j + q, 2h + r]
//     A1 = sigma_p (S_c x_f)[h, w] split into fp16 hi + lo (real form along
//     K = 2H), B1 = the frame's kept-row DFT operand (k_build_fk); D1 holds
//     sigma_p DFT_H(S_c x_f) on the kept rows j, one pair per TMEM lane.
//  2. residual, by the lane's own thread:
//       rho_j = W s t_j - IDFT_W(y)_j   (fully sampled kept row)
//       rho_j = -IDFT_W(y)_j             (kept row without samples)
//     rescaled by a power of two per pair and written as the B operand of
//     the adjoint GEMM, rows 2p: (Re rho, -Im rho), 2p+1: (Im rho, Re rho).
//  3. adjoint GEMM per 128-row tile of H (as k_inv_cols_tc):
//       D3[h, 2p + q] = sum_k A3[h, k] B3[2p + q, k],  A3 = the frame's
//     adjoint kept-row DFT operand (k_build_fa), so D3[h, 2p], D3[h, 2p+1]
//     are Re, Im of IDFT_H(rho_p)[h] (unscaled);
//  4. each thread owns image row h of the tile: x_grad[h, w] += sum_c
//     conj(S_c[h, w]) D3[h, (c, w)] straight from TMEM.
// After all coil groups: the tTV gradient and Nesterov update of the CTA's
// pixels, the tTV objective partial sums and the column maxima of x_{k+1}
// (the next iteration's operand scales), then the shared finish of
// rowlocal.cuh (last CTA: fixed-order reduction and scalar recurrence).
//
// All operands are split fp16 hi + lo with FP32 accumulation in TMEM
// (A_hi B_hi + A_lo B_hi + A_hi B_lo, 22 significant bits).  TMEM holds D1,
// then D3 of one row tile in the same columns: max(npad, 2 * pairs) <= 256
// columns, so two CTAs share an SM.  Every mbarrier wait is bounded; a wait
// that runs out sets the instance's status and the CTA still completes its
// barriers.
#include <algorithm>

#include "ctx.h"
#include "mixed.cuh"
#include "pdl.cuh"
#include "rowlocal.cuh"
#include "solver.h"
#include "tc.cuh"

namespace gbn {

namespace {

constexpr int kRtCols = 8;                       // image columns per CTA
constexpr int kRtNT = 128;                       // threads per CTA (one TMEM lane each)
constexpr int kRtA1Part = 128 * kTcKC * 2;       // bytes of one part of a forward A chunk (8 KB)
constexpr int kRtA3Bytes = 2 * kAcAPart;         // adjoint A chunk, hi + lo (32 KB)

constexpr int kRtB3Max = 64 * 1024;             // adjoint B operand: all its chunks of one coil group

// dynamic shared memory: two forward stages, aliased by the adjoint B operand
// once the forward GEMM is done, then one adjoint A chunk
__host__ __device__ constexpr int rt_stage_bytes(int npad) { return 2 * kRtA1Part + 2 * npad * kTcKC * 2; }
__host__ __device__ constexpr int rt_b3_chunk(int pairs) { return 2 * ac_b_part(2 * pairs); }
__host__ __device__ constexpr int rt_a3_offset(int npad_max) {
  const int r0 = 2 * rt_stage_bytes(npad_max) > kRtB3Max ? 2 * rt_stage_bytes(npad_max) : kRtB3Max;
  return (r0 + 1023) / 1024 * 1024;
}
__host__ __device__ constexpr int rt_smem(int npad_max) { return rt_a3_offset(npad_max) + kRtA3Bytes; }

// Coils per group of an instance with C coils and ncha adjoint chunks: 8 * cg
// pairs <= 128 TMEM lanes and the group's adjoint B operand within kRtB3Max,
// balanced over the groups.  A property of the instance alone, so a batch
// member sums its coils in the same order as a run of its own.
__host__ __device__ constexpr int rt_coils(int C, int ncha) {
  int cg = C < 16 ? (C > 1 ? C : 1) : 16;
  while (cg > 1 && ncha * rt_b3_chunk(kRtCols * cg) > kRtB3Max) --cg;
  const int ng = (C + cg - 1) / cg;
  return (C + ng - 1) / ng;
}

__device__ __forceinline__ float pow2_scale(float mx, float* inv) {
  float sig = 1.f;
  *inv = 1.f;
  if (mx > 0.f) {
    int e;
    frexpf(mx, &e);
    sig = ldexpf(1.f, 14 - e);
    *inv = ldexpf(1.f, e - 14);
  }
  return sig;
}

}  // namespace

// grid (W/8, 1, total frames), 128 threads; the launch's widest forward
// operand npad_max fixes the shared-memory layout
__global__ void __launch_bounds__(kRtNT, 2)
    k_iter_tc(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it, int npad_max) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar[3];  // 0, 1: forward stages; 2: adjoint GEMM
  __shared__ uint32_t tslot;
  __shared__ float s_isig3[128];  // per-pair scale of the adjoint B operand
  __shared__ float s_cmx[kRtNT / 32][kRtCols];
  __shared__ double sred[kRtNT / 32];
  __shared__ float fm[kFmeanCopy];

  const int inst = find_inst(bm, blockIdx.z);
  const FusedArgs& a = tab[inst];
  NestaDevState* st = a.st;
  const int f = blockIdx.z - bm.fbase[inst], w0 = blockIdx.x * kRtCols;
  const int W = a.W, H = a.H, C = a.C, F = a.F;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const size_t N = size_t(W) * H;
  const int npad = a.npad, nch = a.nch, ncha = a.ncha;
  const int rowbase = a.rowoff[f], G = a.rowoff[f + 1] - rowbase;
  const int nht = (H + 127) / 128;
  const int stg = rt_stage_bytes(npad);
  unsigned char* a3s = sm + rt_a3_offset(npad_max);
  const int cgmax = rt_coils(C, ncha);
  const unsigned char* fk = a.fk + size_t(f) * nch * (2 * npad * kTcKC * 2);
  const unsigned char* fa = a.fa + size_t(f) * nht * ncha * kRtA3Bytes;
  auto issue_B1 = [&](int j, int s) {
    const unsigned char* src = fk + size_t(j) * (2 * npad * kTcKC * 2);
    unsigned char* dst = sm + s * stg + 2 * kRtA1Part;
    for (int q = t; q < npad * kTcKC * 4 / 16; q += kRtNT) cp_async16(dst + 16 * q, src + 16 * q);
  };
  auto issue_A3 = [&](int ht, int j) {
    const unsigned char* src = fa + (size_t(ht) * ncha + j) * kRtA3Bytes;
    for (int q = t; q < kRtA3Bytes / 16; q += kRtNT) cp_async16(a3s + 16 * q, src + 16 * q);
  };
  issue_B1(0, 0);  // the DFT operand is an input of the whole solve
  cp_async_commit();
  grid_dep_wait();  // x_k, w_k, the column maxima and the scalar state come from the previous iteration
  grid_dep_release();

  // which update this launch computes (uniform over the instance)
  const int last = st->last_iter;
  bool fix = false;
  int itx = it;
  if (st->partial_rows) {
    if (t == 0 && blockIdx.x == 0 && f == 0 && it == 0) st->status = kStatusRowStructure;
    cp_async_wait<0>();
    return;
  }
  if (it > last) {
    if (!(st->fixup && it == last + 1)) {
      cp_async_wait<0>();
      return;
    }
    fix = true;
    itx = last;
  }

  uint32_t ncols = 32;
  while (ncols < uint32_t(max(npad, 2 * kRtCols * cgmax))) ncols <<= 1;
  if (warp == 0) {
    tc::tmem_alloc(&tslot, ncols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    for (int i = 0; i < 3; ++i) tc::mbar_init(&mbar[i], 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tslot;
  const uint32_t taddr = tbase + (uint32_t(32 * warp) << 16);  // this warp's TMEM lanes

  const float2* __restrict__ xk = (itx & 1) ? a.xk1 : a.xk0;
  float2* __restrict__ xn = (itx & 1) ? a.xk0 : a.xk1;
  const float2* __restrict__ wk = (itx & 1) ? a.wacc1 : a.wacc;
  float2* __restrict__ wn = (itx & 1) ? a.wacc : a.wacc1;
  const float* colmax_k = a.colmax + size_t(itx & 1) * F * W + size_t(f) * W;
  const float s_row = a.s_row;

  float2 acc[4][kRtCols];  // x_grad of rows h = 128 ht + t (H <= 512)
#pragma unroll
  for (int ht = 0; ht < 4; ++ht)
#pragma unroll
    for (int w = 0; w < kRtCols; ++w) acc[ht][w] = make_float2(0.f, 0.f);
  float racc = 0.f;
  bool ok = true;
  uint32_t ph = 0u;  // bit s: the phase parity next awaited on mbar[s]
  int q0 = 0;  // forward chunks issued so far (stage of chunk q is q & 1)

  for (int cg0 = 0; cg0 < C; cg0 += cgmax) {
    const int cn = min(cgmax, C - cg0), pairs = kRtCols * cn;
    const int cl = t / kRtCols, wl = t % kRtCols;
    const bool valid = t < pairs;
    const int c = cg0 + (valid ? cl : 0), w = w0 + wl;
    if (cg0 > 0) {  // the stages held the previous group's adjoint operand until its GEMMs finished
      issue_B1(0, q0 & 1);
      cp_async_commit();
    }
    // ---- 1. forward GEMM ------------------------------------------------
    float isig = 1.f;
    const float sig = valid ? pow2_scale(colmax_k[w] * a.smax[size_t(c) * W + w], &isig) : 1.f;
    const float2* __restrict__ xcol = xk + size_t(f) * N + w;
    const float2* __restrict__ scol = a.S + size_t(c) * N + w;
    float2 px[kTcHC], ps[kTcHC];
    auto prefetch = [&](int j) {
      const int h0 = j * kTcHC;
#pragma unroll
      for (int q = 0; q < kTcHC; ++q) {
        const bool in = valid && (h0 + q < H);
        px[q] = in ? xcol[size_t(h0 + q) * W] : make_float2(0.f, 0.f);
        ps[q] = in ? scol[size_t(h0 + q) * W] : make_float2(0.f, 0.f);
      }
    };
    prefetch(0);
    const uint32_t idesc1 = tc::idesc_f16_f32(128, npad);
    for (int j = 0; j < nch; ++j) {
      const int q = q0 + j, s = q & 1;
      unsigned char* stgp = sm + s * stg;
      // A1 chunk j (this thread's row): 4 core-matrix K groups of 4 complex values
#pragma unroll
      for (int gi = 0; gi < kTcKC / 8; ++gi) {
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float2 v = cmul(px[4 * gi + e], ps[4 * gi + e]);
          split_pair(v.x * sig, v.y * sig, hw[e], lw[e]);
        }
        const uint32_t off = tc::kmajor_offset(t, 8 * gi, kTcKC);
        *reinterpret_cast<uint4*>(stgp + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(stgp + kRtA1Part + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
      if (j + 1 < nch) prefetch(j + 1);
      if (j >= 1) {  // the MMAs of chunk q-1 are done: its stage takes B1 of chunk q+1
        const int sp = (q - 1) & 1;
        ok = tc::mbar_wait(&mbar[sp], (ph >> sp) & 1u, kWaitLimit) && ok;
        ph ^= 1u << sp;
      }
      if (j + 1 < nch) issue_B1(j + 1, (q + 1) & 1);
      cp_async_commit();
      cp_async_wait<1>();  // B1 of chunk q has landed
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      if (t == 0) {
        tc::fence_after_sync();
        const uint32_t sa = tc::smem_u32(stgp), sb = sa + 2 * kRtA1Part;
        const uint32_t bpart = uint32_t(npad) * kTcKC * 2;
#pragma unroll
        for (int ks = 0; ks < kTcKC / 16; ++ks) {
          const uint64_t ahi = tc::smem_desc(sa + ks * 256, 128, kTcKC * 16);
          const uint64_t alo = tc::smem_desc(sa + kRtA1Part + ks * 256, 128, kTcKC * 16);
          const uint64_t bhi = tc::smem_desc(sb + ks * 256, 128, kTcKC * 16);
          const uint64_t blo = tc::smem_desc(sb + bpart + ks * 256, 128, kTcKC * 16);
          tc::mma_f16(tbase, ahi, bhi, idesc1, j > 0 || ks > 0);
          tc::mma_f16(tbase, alo, bhi, idesc1, true);
          tc::mma_f16(tbase, ahi, blo, idesc1, true);
        }
        tc::mma_commit(&mbar[s]);
      }
    }
    {
      const int sl = (q0 + nch - 1) & 1;
      ok = tc::mbar_wait(&mbar[sl], (ph >> sl) & 1u, kWaitLimit) && ok;
      ph ^= 1u << sl;
    }
    q0 += nch;
    cp_async_wait<0>();
    tc::fence_after_sync();

    // ---- 2. residual -> adjoint B operand (this thread's pair) ------------
    const float2* __restrict__ yhat = a.T + (size_t(rowbase) * C + c) * W + w;  // IDFT_W(y) of kept row 0
    const size_t ystride = size_t(C) * W;
    auto rho_of = [&](const float* v, int i, int jrow) -> float2 {
      const float2 tv = make_float2(v[2 * i] * isig, v[2 * i + 1] * isig);
      const float2 yv = yhat[size_t(jrow) * ystride];
      return __ldg(a.row_full + rowbase + jrow) ? csub(cscale(tv, s_row), yv) : make_float2(-yv.x, -yv.y);
    };
    float mx = 0.f;
    for (int col0 = 0; col0 < 2 * G; col0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + uint32_t(col0), v);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int jrow = col0 / 2 + i;
        if (valid && jrow < G) {
          const float2 r = rho_of(v, i, jrow);
          if (!fix) racc = fmaf(r.x, r.x, fmaf(r.y, r.y, racc));
          mx = fmaxf(mx, fmaxf(fabsf(r.x), fabsf(r.y)));
        }
      }
    }
    float isig3 = 1.f;
    const float sig3 = pow2_scale(mx, &isig3);
    if (t < 128) s_isig3[t] = valid ? isig3 : 0.f;
    tc::fence_before_sync();
    __syncthreads();  // every forward stage is free: the adjoint B operand takes their place
    tc::fence_after_sync();
    const int n0 = 2 * t;  // B3 rows of this pair
    for (int col0 = 0; col0 < 2 * kAcRows * ncha; col0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + uint32_t(col0 < npad ? col0 : 0), v);
      if (valid) {
        const int jc = col0 / (2 * kAcRows);        // adjoint K chunk
        unsigned char* b3 = sm + jc * rt_b3_chunk(pairs);
        const int bpart3 = ac_b_part(2 * pairs);
#pragma unroll
        for (int gq = 0; gq < 2; ++gq) {  // 4 kept rows = 8 real k = one core-matrix K group
          uint32_t r0h[4], r0l[4], r1h[4], r1l[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int i = 4 * gq + e, jrow = col0 / 2 + i;
            float2 r = make_float2(0.f, 0.f);
            if (jrow < G && col0 < npad) r = rho_of(v, i, jrow);
            r.x *= sig3;
            r.y *= sig3;
            split_pair(r.x, -r.y, r0h[e], r0l[e]);  // row 2p: (Re, -Im)
            split_pair(r.y, r.x, r1h[e], r1l[e]);   // row 2p+1: (Im, Re)
          }
          const int kk = (col0 % (2 * kAcRows)) + 8 * gq;
          const uint32_t o0 = tc::kmajor_offset(n0, kk, kAcKC), o1 = tc::kmajor_offset(n0 + 1, kk, kAcKC);
          *reinterpret_cast<uint4*>(b3 + o0) = make_uint4(r0h[0], r0h[1], r0h[2], r0h[3]);
          *reinterpret_cast<uint4*>(b3 + bpart3 + o0) = make_uint4(r0l[0], r0l[1], r0l[2], r0l[3]);
          *reinterpret_cast<uint4*>(b3 + o1) = make_uint4(r1h[0], r1h[1], r1h[2], r1h[3]);
          *reinterpret_cast<uint4*>(b3 + bpart3 + o1) = make_uint4(r1l[0], r1l[1], r1l[2], r1l[3]);
        }
      }
    }

    // ---- 3./4. adjoint GEMM per row tile and the coil combination ----------
    const uint32_t idesc3 = tc::idesc_f16_f32(128, 2 * pairs);
#pragma unroll
    for (int ht = 0; ht < 4; ++ht) {  // unrolled: acc[ht] stays in registers
      if (ht >= nht) break;           // uniform over the CTA
      for (int jc = 0; jc < ncha; ++jc) {
        issue_A3(ht, jc);
        cp_async_commit();
        cp_async_wait<0>();
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();  // A3 chunk and B3 visible; the previous TMEM reads are done
        if (t == 0) {
          tc::fence_after_sync();
          const uint32_t sa = tc::smem_u32(a3s), sb = tc::smem_u32(sm + jc * rt_b3_chunk(pairs));
#pragma unroll
          for (int ks = 0; ks < kAcKC / 16; ++ks) {
            const uint64_t ahi = tc::smem_desc(sa + ks * 256, 128, kAcKC * 16);
            const uint64_t alo = tc::smem_desc(sa + kAcAPart + ks * 256, 128, kAcKC * 16);
            const uint64_t bhi = tc::smem_desc(sb + ks * 256, 128, kAcKC * 16);
            const uint64_t blo = tc::smem_desc(sb + ac_b_part(2 * pairs) + ks * 256, 128, kAcKC * 16);
            tc::mma_f16(tbase, ahi, bhi, idesc3, jc > 0 || ks > 0);
            tc::mma_f16(tbase, alo, bhi, idesc3, true);
            tc::mma_f16(tbase, ahi, blo, idesc3, true);
          }
          tc::mma_commit(&mbar[2]);
        }
        ok = tc::mbar_wait(&mbar[2], (ph >> 2) & 1u, kWaitLimit) && ok;
        ph ^= 4u;
        tc::fence_after_sync();
      }
      // x_grad[h, w] += sum_c conj(S_c[h, w]) Y_c[h, w] for this thread's row
      const int h = ht * 128 + t;
      const bool hrow = h < H;
      const float4* srow = reinterpret_cast<const float4*>(a.S + size_t(hrow ? h : 0) * W + w0);
      for (int k = 0; k < cn; ++k) {
        float v[16];
        tc::tmem_ld16(taddr + uint32_t(16 * k), v);
        if (hrow) {
          float4 s4[kRtCols / 2];
#pragma unroll
          for (int qq = 0; qq < kRtCols / 2; ++qq) s4[qq] = __ldg(srow + size_t(cg0 + k) * (N / 2) + qq);
#pragma unroll
          for (int qq = 0; qq < kRtCols / 2; ++qq) {
            const float i0 = s_isig3[k * kRtCols + 2 * qq], i1 = s_isig3[k * kRtCols + 2 * qq + 1];
            const float yr0 = v[4 * qq] * i0, yi0 = v[4 * qq + 1] * i0;
            const float yr1 = v[4 * qq + 2] * i1, yi1 = v[4 * qq + 3] * i1;
            float2& a0 = acc[ht][2 * qq];
            float2& a1 = acc[ht][2 * qq + 1];
            a0.x = fmaf(s4[qq].x, yr0, fmaf(s4[qq].y, yi0, a0.x));
            a0.y = fmaf(s4[qq].x, yi0, fmaf(-s4[qq].y, yr0, a0.y));
            a1.x = fmaf(s4[qq].z, yr1, fmaf(s4[qq].w, yi1, a1.x));
            a1.y = fmaf(s4[qq].z, yi1, fmaf(-s4[qq].w, yr1, a1.y));
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();  // TMEM read before the next tile's (or group's) MMAs
      tc::fence_after_sync();
    }
  }
  if (!ok && t == 0) atomicExch(&st->status, kStatusTcWait);

  // ---- tTV gradient, Nesterov update, objective terms, column maxima ---------
  const float inv_mu = 1.0f / st->mu, lambda = st->lambda, nLmu1 = -st->Lmu1;
  const float apk = fix ? st->apk : 0.5f * (float(itx) + 1.0f);
  const float tauk = fix ? st->tauk : 2.0f / (float(itx) + 3.0f);
  const float omt = 1.0f - tauk, s_adj = a.s_adj;
  float su2 = 0.f, sud = 0.f;
  float cmx[kRtCols];
#pragma unroll
  for (int w = 0; w < kRtCols; ++w) cmx[w] = 0.f;
#pragma unroll
  for (int ht = 0; ht < 4; ++ht) {
    const int h = ht * 128 + t;
    if (ht >= nht || h >= H) continue;
    const size_t p0 = size_t(h) * W + w0;
    const size_t off0 = size_t(f) * N + p0, offm = size_t((f + F - 1) % F) * N + p0,
                 offp = size_t((f + 1) % F) * N + p0;
    float2 xa[kRtCols], xm[kRtCols], xp[kRtCols], wo[kRtCols], xr[kRtCols];
#pragma unroll
    for (int q = 0; q < kRtCols / 2; ++q) {
      const float4 va = *reinterpret_cast<const float4*>(xk + off0 + 2 * q);
      const float4 vm = *reinterpret_cast<const float4*>(xk + offm + 2 * q);
      const float4 vp = *reinterpret_cast<const float4*>(xk + offp + 2 * q);
      const float4 vw = *reinterpret_cast<const float4*>(wk + off0 + 2 * q);
      const float4 vr = *reinterpret_cast<const float4*>(a.xref + off0 + 2 * q);
      xa[2 * q] = make_float2(va.x, va.y), xa[2 * q + 1] = make_float2(va.z, va.w);
      xm[2 * q] = make_float2(vm.x, vm.y), xm[2 * q + 1] = make_float2(vm.z, vm.w);
      xp[2 * q] = make_float2(vp.x, vp.y), xp[2 * q + 1] = make_float2(vp.z, vp.w);
      wo[2 * q] = make_float2(vw.x, vw.y), wo[2 * q + 1] = make_float2(vw.z, vw.w);
      xr[2 * q] = make_float2(vr.x, vr.y), xr[2 * q + 1] = make_float2(vr.z, vr.w);
    }
    float2 wn_out[kRtCols], xn_out[kRtCols];
#pragma unroll
    for (int w = 0; w < kRtCols; ++w) {
      const float2 d0 = csub(xa[w], xm[w]);
      const float2 u0 = tv_normalize(d0, inv_mu);
      const float2 u1 = tv_normalize(csub(xp[w], xa[w]), inv_mu);
      su2 = fmaf(u0.x, u0.x, fmaf(u0.y, u0.y, su2));  // Scnrm2(u), Cdotc(u, d) terms
      sud = fmaf(u0.x, d0.x, fmaf(u0.y, d0.y, sud));
      const float2 adj = csub(u1, u0);
      const float2 ares = cscale(acc[ht][w], s_adj);
      const float2 df = make_float2(__fadd_rn(__fmul_rn(-adj.x, lambda), ares.x),
                                    __fadd_rn(__fmul_rn(-adj.y, lambda), ares.y));
      const float2 yk = make_float2(fmaf(nLmu1, df.x, xa[w].x), fmaf(nLmu1, df.y, xa[w].y));
      const float2 wnv = make_float2(fmaf(apk, df.x, wo[w].x), fmaf(apk, df.y, wo[w].y));
      const float2 zk = make_float2(fmaf(nLmu1, wnv.x, xr[w].x), fmaf(nLmu1, wnv.y, xr[w].y));
      xn_out[w] = make_float2(fmaf(omt, yk.x, tauk * zk.x), fmaf(omt, yk.y, tauk * zk.y));
      wn_out[w] = wnv;
      cmx[w] = fmaxf(cmx[w], fmaf(xn_out[w].x, xn_out[w].x, xn_out[w].y * xn_out[w].y));
    }
#pragma unroll
    for (int q = 0; q < kRtCols / 2; ++q) {
      *reinterpret_cast<float4*>(wn + off0 + 2 * q) =
          make_float4(wn_out[2 * q].x, wn_out[2 * q].y, wn_out[2 * q + 1].x, wn_out[2 * q + 1].y);
      *reinterpret_cast<float4*>(xn + off0 + 2 * q) =
          make_float4(xn_out[2 * q].x, xn_out[2 * q].y, xn_out[2 * q + 1].x, xn_out[2 * q + 1].y);
    }
  }
  // column maxima of x_{k+1}: this CTA owns columns w0..w0+7 of frame f
#pragma unroll
  for (int w = 0; w < kRtCols; ++w) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cmx[w] = fmaxf(cmx[w], __shfl_xor_sync(0xffffffffu, cmx[w], o));
  }
  if (lane == 0) {
#pragma unroll
    for (int w = 0; w < kRtCols; ++w) s_cmx[warp][w] = cmx[w];
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
  if (t < kRtCols) {
    float m = 0.f;
    for (int k = 0; k < kRtNT / 32; ++k) m = fmaxf(m, s_cmx[k][t]);
    a.colmax[size_t((itx + 1) & 1) * F * W + size_t(f) * W + w0 + t] = sqrtf(m);
  }
  if (fix) return;

  const int blk = f * gridDim.x + blockIdx.x;
  const double pr = block_sum<kRtNT>(double(racc), sred);
  const double t1 = block_sum<kRtNT>(double(su2), sred);
  const double t2 = block_sum<kRtNT>(double(sud), sred);
  if (t == 0) {
    a.part_r[blk] = pr;
    a.part_tv[2 * blk] = t1;
    a.part_tv[2 * blk + 1] = t2;
  }
  if (rowlocal_last_cta(bm.ctl, inst, gridDim.x * unsigned(F)))
    rowlocal_finish<kRtNT>(a, st, bm.ctl, inst, it, apk, a.ntv, sred, fm);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
dim3 iter_tc_grid(int W, int frames) { return dim3(W / kRtCols, 1, frames); }

void launch_iter_tc(const FusedArgs* tab, const BatchMap& bm, int it, int npad_max, dim3 grid, cudaStream_t s) {
  static bool ok = false;
  if (!ok) {
    cudaFuncSetAttribute(k_iter_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, rt_smem(256));
    ok = true;
  }
  launch_pdl(k_iter_tc, grid, kRtNT, rt_smem(npad_max), s, tab, bm, it, npad_max);
}

}  // namespace gbn
