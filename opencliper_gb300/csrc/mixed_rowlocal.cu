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
#include <cudaTypedefs.h>

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
constexpr int kRtA1Stage = 2 * kRtA1Part;        // hi + lo
constexpr int kRtA3Bytes = 2 * kAcAPart;         // adjoint A chunk, hi + lo (32 KB)
constexpr int kRtB3Max = 64 * 1024;              // adjoint B operand: all its chunks of one coil group
constexpr int kRtR2 = kRtB3Max;                  // second region: IDFT_W(y) tile, adjoint A chunk, S ring
constexpr int kRtR2Bytes = 32 * 1024;
constexpr int kRtSlots = 4;                      // S ring of the coil combination: one coil per slot
constexpr int kRtSlotBytes = 128 * 64;           // 128 image rows x 8 complex columns
constexpr uint32_t kRtWaitPolls = 4096;          // suspending polls of one wait (~1 ms each at most)

// Shared memory (1024-aligned base):
//   forward GEMM: [0, 2 A1 stages) then a ring of nst stages, each
//     [x tile: 16 rows x 8 columns][S tile: cnmax coils x 16 rows x 8 columns]
//     [the frame's forward DFT operand chunk, npad rows hi | lo];
//   afterwards: [0, 64 KB) the adjoint B operand, [64 KB, 96 KB) the kept rows'
//   IDFT_W(y) tile, then one adjoint A chunk at a time, then the S ring.
__host__ __device__ constexpr int rt_ring_stage(int npad_max, int cnmax) {
  return 1024 + cnmax * 1024 + npad_max * kTcKC * 4;
}
__host__ __device__ constexpr int rt_nst(int npad_max, int cnmax) {
  return 2 * kRtA1Stage + 3 * rt_ring_stage(npad_max, cnmax) <= 100 * 1024 ? 3 : 2;
}
__host__ __device__ constexpr int rt_smem(int npad_max, int cnmax) {
  const int fwd = 2 * kRtA1Stage + rt_nst(npad_max, cnmax) * rt_ring_stage(npad_max, cnmax);
  return fwd > kRtR2 + kRtR2Bytes ? fwd : kRtR2 + kRtR2Bytes;
}
__host__ __device__ constexpr int rt_b3_chunk(int pairs) { return 2 * ac_b_part(2 * pairs); }

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

// grid (W/8, 1, total frames), 128 threads; npad_max and cnmax (the launch's
// widest forward operand and coil group) fix the shared-memory layout.  The
// register cap keeps two CTAs per SM (two CTAs of 255 registers a thread
// would need the whole register file, and the SM then keeps one).
__global__ void __maxnreg__(224)
    k_iter_tc(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it, int npad_max, int cnmax) {
  extern __shared__ __align__(1024) unsigned char sm[];
  // mbarriers: ring stages, forward MMAs (per A1 stage), adjoint A chunk,
  // adjoint MMAs, IDFT_W(y) tile, S ring slots
  __shared__ uint64_t bar_full[3], bar_mma[2], bar_a3, bar_mma3, bar_y, bar_s[kRtSlots];
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
  const int cgmax = rt_coils(C, ncha);  // this instance's coils per group (the S and IDFT_W(y) boxes)
  const int rs = rt_ring_stage(npad_max, cnmax), nst = rt_nst(npad_max, cnmax);
  unsigned char* ring = sm + 2 * kRtA1Stage;
  unsigned char* r2 = sm + kRtR2;
  const unsigned char* fk = a.fk + size_t(f) * nch * (2 * npad * kTcKC * 2);
  const unsigned char* fa = a.fa + size_t(f) * nht * ncha * kRtA3Bytes;
  grid_dep_wait();  // x_k, w_k, the column maxima and the scalar state come from the previous iteration
  grid_dep_release();

  // which update this launch computes (uniform over the instance)
  const int last = st->last_iter;
  bool fix = false;
  int itx = it;
  if (st->partial_rows) {
    if (t == 0 && blockIdx.x == 0 && f == 0 && it == 0) st->status = kStatusRowStructure;
    return;
  }
  if (it > last) {
    if (!(st->fixup && it == last + 1)) return;
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
    for (int i = 0; i < 3; ++i) tc::mbar_init(&bar_full[i], 1);
    for (int i = 0; i < 2; ++i) tc::mbar_init(&bar_mma[i], 1);
    tc::mbar_init(&bar_a3, 1);
    tc::mbar_init(&bar_mma3, 1);
    tc::mbar_init(&bar_y, 1);
    for (int i = 0; i < kRtSlots; ++i) tc::mbar_init(&bar_s[i], 1);
    tc::fence_mbar_init();
    tc::tmap_acquire(&a.tm_x[itx & 1]);
    tc::tmap_acquire(&a.tm_s);
    tc::tmap_acquire(&a.tm_se);
    tc::tmap_acquire(&a.tm_y);
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
  const CUtensorMap* tmx = &a.tm_x[itx & 1];
  const float s_row = a.s_row;

  // barrier phases: bits 0-2 ring stages, 3-4 forward MMAs, 5 adjoint A, 6
  // adjoint MMAs, 7 IDFT_W(y), 8-11 S slots
  uint32_t ph = 0u;
  bool ok = true;
  auto waitb = [&](uint64_t* b, int bit) {
    ok = tc::mbar_wait_sleep(b, (ph >> bit) & 1u, kRtWaitPolls) && ok;
    ph ^= 1u << bit;
  };

  float2 acc[4][kRtCols];  // x_grad of rows h = 128 ht + t (H <= 512)
#pragma unroll
  for (int ht = 0; ht < 4; ++ht)
#pragma unroll
    for (int w = 0; w < kRtCols; ++w) acc[ht][w] = make_float2(0.f, 0.f);
  float racc = 0.f;
  int q0 = 0;  // forward chunks so far: ring stage q % nst, A1 stage q & 1

  for (int cg0 = 0; cg0 < C; cg0 += cgmax) {
    const int cn = min(cgmax, C - cg0), pairs = kRtCols * cn;
    const int cl = t / kRtCols, wl = t % kRtCols;
    const bool valid = t < pairs;
    const int c = cg0 + (valid ? cl : 0), w = w0 + wl;
    const uint32_t chunk_bytes = 1024u + uint32_t(cgmax) * 1024u + uint32_t(npad) * kTcKC * 4u;
    // the forward operands of chunk j (x, S of the group, DFT rows) into ring stage sidx (thread 0)
    auto load_chunk = [&](int j, int sidx) {
      unsigned char* sp = ring + sidx * rs;
      tc::mbar_arrive_expect_tx(&bar_full[sidx], chunk_bytes);
      tc::tma_load_3d(sp, tmx, 2 * w0, kTcHC * j, f, &bar_full[sidx]);
      tc::tma_load_3d(sp + 1024, &a.tm_s, 2 * w0, kTcHC * j, cg0, &bar_full[sidx]);
      tc::bulk_g2s(sp + 1024 + cnmax * 1024, fk + size_t(j) * (2 * npad * kTcKC * 2), uint32_t(npad) * kTcKC * 4u,
                   &bar_full[sidx]);
    };
    if (t == 0)
      for (int i = 0; i < nst && i < nch; ++i) load_chunk(i, (q0 + i) % nst);

    // ---- 1. forward GEMM ------------------------------------------------
    float isig = 1.f;
    const float sig = valid ? pow2_scale(colmax_k[w] * a.smax[size_t(c) * W + w], &isig) : 1.f;
    const uint32_t idesc1 = tc::idesc_f16_f32(128, npad);
    for (int j = 0; j < nch; ++j) {
      const int q = q0 + j, sidx = q % nst, a1 = q & 1;
      waitb(&bar_full[sidx], sidx);
      const unsigned char* sp = ring + sidx * rs;
      const float2* xs = reinterpret_cast<const float2*>(sp);                          // [16 rows][8]
      const float2* ss = reinterpret_cast<const float2*>(sp + 1024) + cl * kTcHC * 8;  // [coil][16 rows][8]
      unsigned char* a1p = sm + a1 * kRtA1Stage;
#pragma unroll
      for (int gi = 0; gi < kTcKC / 8; ++gi) {
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int r = 4 * gi + e;
          const float2 v = valid ? cmul(xs[r * 8 + wl], ss[r * 8 + wl]) : make_float2(0.f, 0.f);
          split_pair(v.x * sig, v.y * sig, hw[e], lw[e]);
        }
        const uint32_t off = tc::kmajor_offset(t, 8 * gi, kTcKC);
        *reinterpret_cast<uint4*>(a1p + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(a1p + kRtA1Part + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();  // A1 chunk complete; the ring stage's x and S are consumed
      if (t == 0) {
        tc::fence_after_sync();
        const uint32_t sa = tc::smem_u32(a1p), sb = tc::smem_u32(sp + 1024 + cnmax * 1024);
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
        tc::mma_commit(&bar_mma[a1]);
      }
      if (j >= 1) {  // the MMAs of chunk q-1: their A1 stage and ring stage are free again
        waitb(&bar_mma[(q - 1) & 1], 3 + ((q - 1) & 1));
        if (t == 0 && j - 1 + nst < nch) load_chunk(j - 1 + nst, (q - 1) % nst);
      }
    }
    waitb(&bar_mma[(q0 + nch - 1) & 1], 3 + ((q0 + nch - 1) & 1));
    q0 += nch;
    tc::fence_after_sync();
    // the kept rows' IDFT_W(y) of this group's coils: [G rows][cgmax coils][8 columns]
    if (t == 0) {
      tc::mbar_arrive_expect_tx(&bar_y, uint32_t(a.gmax_box) * uint32_t(cgmax) * 64u);
      tc::tma_load_3d(r2, &a.tm_y, 2 * w0, cg0, rowbase, &bar_y);
    }
    waitb(&bar_y, 7);

    // ---- 2. residual -> adjoint B operand (this thread's pair) ------------
    const float2* ys = reinterpret_cast<const float2*>(r2) + cl * 8 + wl;  // + j * cgmax * 8
    auto rho_of = [&](const float* v, int i, int jrow) -> float2 {
      const float2 tv = make_float2(v[2 * i] * isig, v[2 * i + 1] * isig);
      const float2 yv = ys[jrow * cgmax * 8];
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
    s_isig3[t] = valid ? isig3 : 0.f;
    const int n0 = 2 * t;  // B3 rows of this pair
    for (int col0 = 0; col0 < 2 * kAcRows * ncha; col0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + uint32_t(col0 < npad ? col0 : 0), v);
      if (valid) {
        const int jc = col0 / (2 * kAcRows);  // adjoint K chunk
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
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();  // B3 complete; the IDFT_W(y) tile and D1 are no longer read
    tc::fence_after_sync();

    // ---- 3./4. adjoint GEMM per row tile and the coil combination ----------
    const uint32_t idesc3 = tc::idesc_f16_f32(128, 2 * pairs);
#pragma unroll
    for (int ht = 0; ht < 4; ++ht) {  // unrolled: acc[ht] stays in registers
      if (ht >= nht) break;           // uniform over the CTA
      for (int jc = 0; jc < ncha; ++jc) {
        if (t == 0) {
          tc::mbar_arrive_expect_tx(&bar_a3, kRtA3Bytes);
          tc::bulk_g2s(r2, fa + (size_t(ht) * ncha + jc) * kRtA3Bytes, kRtA3Bytes, &bar_a3);
        }
        waitb(&bar_a3, 5);
        if (t == 0) {
          const uint32_t sa = tc::smem_u32(r2), sb = tc::smem_u32(sm + jc * rt_b3_chunk(pairs));
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
          tc::mma_commit(&bar_mma3);
        }
        waitb(&bar_mma3, 6);  // the MMAs read the A chunk: the region is free again
        tc::fence_after_sync();
      }
      // S of this row tile, one coil per ring slot (thread 0 issues, all wait)
      auto load_s = [&](int k) {
        tc::mbar_arrive_expect_tx(&bar_s[k % kRtSlots], kRtSlotBytes);
        tc::tma_load_3d(r2 + (k % kRtSlots) * kRtSlotBytes, &a.tm_se, 2 * w0, 128 * ht, cg0 + k, &bar_s[k % kRtSlots]);
      };
      if (t == 0)
        for (int k = 0; k < kRtSlots && k < cn; ++k) load_s(k);
      // x_grad[h, w] += sum_c conj(S_c[h, w]) Y_c[h, w] for this thread's row
      const int h = ht * 128 + t;
      const bool hrow = h < H;
      for (int k = 0; k < cn; ++k) {
        float v[16];
        tc::tmem_ld16(taddr + uint32_t(16 * k), v);
        waitb(&bar_s[k % kRtSlots], 8 + (k % kRtSlots));
        const float4* srow = reinterpret_cast<const float4*>(r2 + (k % kRtSlots) * kRtSlotBytes) + t * 4;
        if (hrow) {
#pragma unroll
          for (int qq = 0; qq < kRtCols / 2; ++qq) {
            const float4 s4 = srow[qq];
            const float i0 = s_isig3[k * kRtCols + 2 * qq], i1 = s_isig3[k * kRtCols + 2 * qq + 1];
            const float yr0 = v[4 * qq] * i0, yi0 = v[4 * qq + 1] * i0;
            const float yr1 = v[4 * qq + 2] * i1, yi1 = v[4 * qq + 3] * i1;
            float2& a0 = acc[ht][2 * qq];
            float2& a1 = acc[ht][2 * qq + 1];
            a0.x = fmaf(s4.x, yr0, fmaf(s4.y, yi0, a0.x));
            a0.y = fmaf(s4.x, yi0, fmaf(-s4.y, yr0, a0.y));
            a1.x = fmaf(s4.z, yr1, fmaf(s4.w, yi1, a1.x));
            a1.y = fmaf(s4.z, yi1, fmaf(-s4.w, yr1, a1.y));
          }
        }
        if (k + kRtSlots < cn) {
          __syncthreads();  // every thread read this slot
          if (t == 0) load_s(k + kRtSlots);
        }
      }
      tc::fence_before_sync();
      __syncthreads();  // TMEM and the S slots read before the next tile's (or group's) loads and MMAs
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
    rowlocal_finish<kRtNT>(a, st, bm.ctl, inst, it, apk, a.ntv, a.ntv, sred, fm);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// float32 tensor of dims (d0 innermost, d1, d2), dense, box (b0, b1, b2);
// elements outside the tensor read as zero
bool encode3d(CUtensorMap* m, const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint32_t b0, uint32_t b1,
              uint32_t b2) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {d0, d1, d2};
  const cuuint64_t strides[2] = {d0 * 4, d0 * d1 * 4};
  const cuuint32_t box[3] = {b0, b1, b2};
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Coils per group of an instance (the S and IDFT_W(y) boxes of its tensor maps).
int iter_tc_coils(int C, int ncha) { return rt_coils(C, ncha); }

// Whether the tensor-core row-local iteration takes a prepared problem (its
// IDFT_W(y) tile must fit the 32 KB region); encodes its tensor maps.
bool iter_tc_prepare(gbn_problem* P) {
  const int cg = rt_coils(P->C, P->ncha);
  P->tmaps_ok = false;
  if (P->gmax < 1 || P->gmax > 256 || P->gmax * cg * 64 > kRtR2Bytes) return false;
  const uint64_t W2 = uint64_t(2) * P->W;
  bool ok = encode3d(&P->tm_x[0], P->xk0, W2, P->H, P->F, 2 * kRtCols, kTcHC, 1) &&
            encode3d(&P->tm_x[1], P->xk1, W2, P->H, P->F, 2 * kRtCols, kTcHC, 1) &&
            encode3d(&P->tm_s, P->S, W2, P->H, P->C, 2 * kRtCols, kTcHC, cg) &&
            encode3d(&P->tm_se, P->S, W2, P->H, P->C, 2 * kRtCols, 128, 1) &&
            encode3d(&P->tm_y, P->T, W2, P->C, P->T_rows, 2 * kRtCols, cg, P->gmax);
  P->tmaps_ok = ok;
  return ok;
}

void iter_tc_args(gbn_problem* P, FusedArgs* a) {
  a->tm_x[0] = P->tm_x[0];
  a->tm_x[1] = P->tm_x[1];
  a->tm_s = P->tm_s;
  a->tm_se = P->tm_se;
  a->tm_y = P->tm_y;
  a->gmax_box = P->gmax;
  a->ntv = P->F * (P->W / kRtCols);  // one partial sum per (frame, 8 columns)
}

dim3 iter_tc_grid(int W, int frames) { return dim3(W / kRtCols, 1, frames); }

void launch_iter_tc(const FusedArgs* tab, const BatchMap& bm, int it, int npad_max, int cnmax, dim3 grid,
                    cudaStream_t s) {
  static bool ok = false;
  if (!ok) {
    cudaFuncSetAttribute(k_iter_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, rt_smem(256, 16));
    // the whole unified memory as shared memory: two CTAs of ~100 KB per SM
    cudaFuncSetAttribute(k_iter_tc, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    ok = true;
  }
  launch_pdl(k_iter_tc, grid, kRtNT, rt_smem(npad_max, cnmax), s, tab, bm, it, npad_max, cnmax);
}

}  // namespace gbn
