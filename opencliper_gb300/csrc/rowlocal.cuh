// Row-local tTV-NESTA iteration: one fused kernel per inner iteration for
// problems whose kept k-space rows are each either fully sampled or not
// sampled at all (every Cartesian phase-encode mask, i.e. every row mask of
// SamplingMasksData, SamplingMasksData.cpp:389-441).
//
// For such a row the mask does not vary along the readout (W) axis, so the
// row transform of the residual and its inverse cancel:
//   IDFT_W( s * DFT_W(t) - y )  =  W*s*t - IDFT_W(y)          (fully sampled row)
//   IDFT_W( 0 * DFT_W(t) - y )  =  -IDFT_W(y)                 (row kept for its data only)
// with t the column transform DFT_H(S_c x_f) of that row and s = 1/sqrt(N) the
// reference's forward scale (NestaUp.cpp:712-718).  IDFT_W(y) of every kept
// row is what the setup's adjoint row pass leaves in T when it forms
// x0 = E^H y, and it stays there for the whole solve.  The residual's norm
// follows from Parseval: ||s DFT_W(t) - y||^2 = ||W s t - IDFT_W(y)||^2 / W.
// So E^H(E x - y) (NestaUp.cpp:710-756) becomes a per-column operation:
//   rho = W s DFT_H(S_c x_f)[kept rows] - IDFT_W(y)[kept rows]
//   A^H r = (sqrt(N)/N) sum_c conj(S_c) IDFT_H(rho)
// and the whole inner iteration runs in one kernel.
//
// k_iter_cols<H, MOTION>: grid (W/kWB, 2, frames) in clusters of 2 along y;
// CTA = (frame, 8 columns, half of the coils), 128 threads (160 at H = 288,
// 320).  Per coil: forward column DFT of
// S_c x_f (dit2<A,B>), residual on the kept rows, inverse column DFT
// (dit2<B,A> of the conjugate) and conj(S_c) accumulation.  The forward
// pass-2 item (w, k1) holds rows k1 + A*k2, exactly the rows the inverse
// pass-1 item s' = k1 needs, so the residual never leaves registers.  The two
// coil halves are summed through distributed shared memory, then the tTV
// gradient (temporalTV.cl:78-107 with NestaUp's negation, vectorNormalization.cl
// :42-56) and the Nesterov update (NestaUp.cpp:758-875) finish each pixel.
// The tTV objective terms (Scnrm2, Cdotc of NestaUp.cpp:686-691; each CTA of
// the pair over half of the tile) and ||r||^2 are written as fixed-slot
// partial sums; the last CTA of an instance reduces them in fixed order and
// runs the scalar recurrence (nesta_scalar_step).  Register budgets per length
// (x and the accumulators in registers or in tensor memory) are set by
// iter_cols_tmem / iter_cols_threads / iter_cols_min_blocks below.
//
// The update of iteration k uses apk = (k+1)/2 and tauk = 2/(k+3), what the
// scalar recurrence yields unless the stopping test fires for the second time
// at k; then the reference updates with k = maxIter and stops
// (NestaUp.cpp:808-831).  x and w are ping-pong buffers, so the launch after
// such an iteration (its index is last_iter + 1) recomputes that update from
// the unchanged x_k and w_k with the recurrence's weights ("fixup" mode).
#pragma once

#include "nesta_kernels.cuh"
#include "tc.cuh"

namespace gbn {

constexpr int kStatusRowStructure = 7;  // NestaDevState::status: a kept row is partly sampled (row-local path)

// Block-wide sums of three doubles per thread, in thread 0: each summed as
// block_sum sums one (same order), with one pair of barriers for the three.
// sred holds 3 * NT/32 doubles.
template <int NT>
__device__ __forceinline__ void rowlocal_block_sum3(double a, double b, double c, double* sred, double* ra, double* rb,
                                                    double* rc) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    sred[wid] = a;
    sred[NT / 32 + wid] = b;
    sred[2 * (NT / 32) + wid] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0, tc = 0.0;
#pragma unroll
    for (int i = 0; i < NT / 32; ++i) {
      ta += sred[i];
      tb += sred[NT / 32 + i];
      tc += sred[2 * (NT / 32) + i];
    }
    *ra = ta;
    *rb = tb;
    *rc = tc;
  }
}

// Counts this CTA as finished for instance `inst` (after thread 0 stored its
// partial sums) and tells every thread whether it was the instance's last of
// `total` CTAs.  All threads call it.  Only thread 0's stores need to be
// visible before the count (the other threads' image stores are read by the
// next launch), so only thread 0 fences.
__device__ __forceinline__ bool rowlocal_last_cta(ClassCtl* ctl, int inst, unsigned total) {
  __shared__ int s_fin;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_fin = (atomicAdd(&ctl->done[inst], 1u) + 1u == total) ? 1 : 0;
  }
  __syncthreads();
  return s_fin != 0;
}

// The instance's last CTA of a row-local iteration: reduces the fixed-slot
// partial sums (ntv (||u||^2, Re<u,d>) pairs, npr sums of |rho|^2) in fixed
// order and runs the scalar recurrence; ||E x - y||^2 = sum |rho|^2 / W
// (Parseval along the rows).  `apk_used` is the weight the CTAs updated with:
// when the recurrence's differs, the stopping test fired for the second time
// and the next launch recomputes this iteration's update.  All NT threads call it.
template <int NT>
__device__ void rowlocal_finish(const FusedArgs& a, NestaDevState* st, ClassCtl* ctl, int inst, int it, float apk_used,
                                int ntv, int npr, double* sred, float* fm) {
  const int t = threadIdx.x;
  __threadfence();
  if (t < kFmeanCopy && t < st->miniter) fm[t] = __ldcg(a.fmean + t);
  constexpr int U = 8;
  double s1 = 0.0, s2 = 0.0, s3 = 0.0;
  const double2* ptv = reinterpret_cast<const double2*>(a.part_tv);
  for (int i0 = 0; i0 < ntv; i0 += U * NT) {
    double2 vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * NT + t;
      vv[u] = (i < ntv) ? __ldcg(ptv + i) : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      s1 += vv[u].x;
      s2 += vv[u].y;
    }
  }
  for (int i0 = 0; i0 < npr; i0 += U * NT) {
    double vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int i = i0 + u * NT + t;
      vv[u] = (i < npr) ? __ldcg(a.part_r + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) s3 += vv[u];
  }
  s1 = block_sum<NT>(s1, sred);
  s2 = block_sum<NT>(s2, sred);
  s3 = block_sum<NT>(s3, sred);
  if (t == 0) {
    nesta_scalar_step(st, a.fmean, fm, it, s1, s2, s3 / double(a.W));
    if (st->apk != apk_used) st->fixup = 1;
    ctl->done[inst] = 0;
  }
}

// Kept rows per frame whose IDFT_W(y) k_iter_cols<L> stages: a quarter of the
// rows (every Cartesian mask at R >= 4), at least 32 for short columns.
constexpr int iter_cols_rcap(int L) { return L / 4 > (L < 32 ? L : 32) ? L / 4 : (L < 32 ? L : 32); }

// Twiddle m of a thread's item from its row of M consecutive values (16-byte
// aligned when M is even): pairs come from one 16-byte shared load.
template <int M>
__device__ __forceinline__ float2 twiddle(const float2* row, int m) {
  if constexpr (M % 2 == 0) {
    const float4 q = reinterpret_cast<const float4*>(row)[m >> 1];
    return (m & 1) ? make_float2(q.z, q.w) : make_float2(q.x, q.y);
  } else {
    return row[m];
  }
}

// Lengths whose x values and coil accumulators live in tensor memory instead
// of registers: first factors above 16 with one pass-1 and one inverse pass-2
// item per thread (H = 288, 320, 336, 384).  With the registers this frees and
// a single S buffer, three CTAs share an SM at H = 320 and 384 instead of two
// (measured: 1.28x at 384 x 384).  At H = 256 the register form is faster.
constexpr bool iter_cols_tmem(int L) { return split_a(L) > 16 && kWB * split_b(L) == kColNT; }

// Calls fn(offset, count) for consecutive pieces of F TMEM columns: pieces of
// 16, then one each of 8, 4 and 2 as F requires (F even); every piece starts
// at a multiple of its size.
template <int F, typename Fn>
__device__ __forceinline__ void tmem_pieces(Fn&& fn) {
  static_assert(F % 2 == 0, "whole complex values");
  sfor<0, F / 16>([&](auto qc) {
    fn(std::integral_constant<int, 16 * decltype(qc)::value>{}, std::integral_constant<int, 16>{});
  });
  constexpr int o8 = F / 16 * 16, o4 = o8 + ((F - o8) & 8), o2 = o4 + ((F - o4) & 4);
  if constexpr ((F - o8) & 8) fn(std::integral_constant<int, o8>{}, std::integral_constant<int, 8>{});
  if constexpr ((F - o4) & 4) fn(std::integral_constant<int, o4>{}, std::integral_constant<int, 4>{});
  if constexpr ((F - o2) & 2) fn(std::integral_constant<int, o2>{}, std::integral_constant<int, 2>{});
}
template <int N>
__device__ __forceinline__ void tmem_ld_n(uint32_t taddr, float* v) {
  if constexpr (N == 16) tc::tmem_ld16(taddr, v);
  else tc::tmem_ld_small<N>(taddr, v);
}
template <int N>
__device__ __forceinline__ void tmem_st_n(uint32_t taddr, const float* v) {
  if constexpr (N == 16) tc::tmem_st16(taddr, v);
  else tc::tmem_st_small<N>(taddr, v);
}
constexpr int iter_cols_sbufs(int L) { return iter_cols_tmem(L) ? 1 : 2; }

// Threads per CTA: 128, or for the tensor-memory lengths one per pass-2 item
// (kWB * A of them, rounded up to whole warps) where three such CTAs still fit
// at 128 registers a thread (H = 288, 320: 160 threads).  With 128 threads
// those items fall twice to some threads and the pass waits for them; more
// threads at fewer CTAs per SM measured slower (H = 384: 288 us per iteration
// with 192 threads at two CTAs, against 280 us).  The pass-1 and pass-3 items
// (kWB * B = 128) stay on warps 0-3, whose tensor-memory lanes hold their state.
// Short columns with at most 64 pass-2 items (A <= 8: H = 64, 96, 128 ...)
// run 64 threads with two pass-1 and pass-3 items each, so no thread idles in
// pass 2, at twice the CTAs per SM.
constexpr int iter_cols_threads(int L) {
  return (iter_cols_tmem(L) && (kWB * split_a(L) + 31) / 32 * 32 * 3 * 128 <= 65536) ? (kWB * split_a(L) + 31) / 32 * 32
         : (!iter_cols_tmem(L) && kWB * split_a(L) <= 64 && kWB * split_b(L) == kColNT) ? 64
                                                                                        : kColNT;
}

// Shared-memory bytes of k_iter_cols<L> (the layout of IterColsSmem<L>).
constexpr int iter_cols_bytes(int L) {
  const int a = split_a(L), b = split_b(L);
  const int ex = (a * col_ks(b) > b * col_ks(a)) ? a * col_ks(b) : b * col_ks(a);
  return (iter_cols_sbufs(L) * L * kWB + 2 * iter_cols_rcap(L) * kWB + ex + b * (a + 2) + a * (b + 2)) * 8 + L * 4 +
         3 * (iter_cols_threads(L) / 32) * 8 + kFmeanCopy * 4 + 16;
}

template <int H>
struct IterColsSmem {
  static constexpr int A = Split<H>::A, B = Split<H>::B;
  static constexpr int NT = iter_cols_threads(H);   // threads per CTA
  static constexpr int NI3 = cdiv(kWB * B, NT);     // inverse pass-2 items per thread
  static constexpr int XST = NI3 == 1 ? kWB * B : NT;  // stride of the accumulator exchange
  static constexpr int KSF = col_ks(B);  // forward exchange: slot (k1, s*kWB + w), k1 < A
  static constexpr int KSI = col_ks(A);  // inverse exchange: slot (k1', s'*kWB + w), k1' < B
  static constexpr int EXN = (A * KSF > B * KSI) ? A * KSF : B * KSI;
  static constexpr int RCAP = iter_cols_rcap(H);         // kept rows whose IDFT_W(y) is staged
  static constexpr int SB = iter_cols_sbufs(H);          // S buffers: 2 (next coil copied during this one) or 1
  static constexpr int S_OFF = 0;                        // float2 [SB][H][kWB]
  static constexpr int Y_OFF = S_OFF + SB * H * kWB;     // float2 [2][RCAP][kWB]
  static constexpr int EX_OFF = Y_OFF + 2 * RCAP * kWB;  // float2 [EXN]
  // twiddles: B rows of A (forward first pass, one row per item s) and A rows
  // of B (inverse first pass, one per item k1), each row padded by one 16-byte
  // pair so that the rows a warp reads at once sit in different banks
  static constexpr int TWF = A + 2, TWI = B + 2;
  static constexpr int TW_OFF = EX_OFF + EXN;
  static constexpr int TWI_OFF = B * TWF;                // inverse rows, from TW_OFF
  static constexpr int F2_END = TW_OFF + TWI_OFF + A * TWI;
  static constexpr int BYTES = F2_END * 8 + H * 4 + 3 * (NT / 32) * 8 + kFmeanCopy * 4 + 16;
  static_assert(NI3 * A * XST <= SB * H * kWB, "accumulator exchange must fit the S buffers");
  static_assert(BYTES == iter_cols_bytes(H), "layout and byte count agree");
  static_assert(TW_OFF % 2 == 0, "twiddle rows start on 16-byte boundaries");
};


// CTAs per SM the launch bounds ask for.  With x and the accumulators in
// tensor memory, as many as shared memory allows and keep 128 registers a
// thread (at most three); otherwise a
// first factor A <= 16 keeps the per-thread state (x at the pass-1 items, the
// accumulators, one pass-2 item) within 168 registers at three CTAs per SM,
// and longer first factors hold more per thread at the two CTAs per SM (one
// past 448) their shared memory allows, with up to 255 registers a thread.
constexpr int iter_cols_min_blocks(int H) {
  if (iter_cols_tmem(H)) {
    const int by_smem = (228 * 1024) / (iter_cols_bytes(H) + 1024);
    const int by_regs = 65536 / (iter_cols_threads(H) * 128);  // at least 128 registers a thread
    const int m = by_smem < by_regs ? by_smem : by_regs;
    return m < 3 ? m : 3;
  }
  if (iter_cols_threads(H) == 64) return 6;
  return split_a(H) <= 16 ? 3 : (iter_cols_bytes(H) + 1024 <= 114 * 1024 ? 2 : 1);
}

// Lengths that run the row-local iteration; the others (whose per-thread
// state would spill) run the three-pass iteration.
constexpr bool iter_cols_ok(int H) {
  return split_a(H) != 0 && (split_a(H) <= 16 || (split_b(H) >= 8 && split_b(H) <= 16 && split_a(H) <= 24) ||
                             (iter_cols_tmem(H) && split_a(H) <= 32));
}

// MOTION: the motion-compensated form (tTV gradient M^T(tTVadj u) and the
// tTV sums from the motion kernels launched before it).
template <int H, bool MOTION>
__global__ void __cluster_dims__(1, 2, 1) __launch_bounds__(iter_cols_threads(H), iter_cols_min_blocks(H))
    k_iter_cols(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it) {
  using L = IterColsSmem<H>;
  constexpr int A = L::A, B = L::B, KSF = L::KSF, KSI = L::KSI, RCAP = L::RCAP, NT = L::NT;
  constexpr int N1 = kWB * B;  // forward pass-1 items (w, s), s < B: rows B*n1 + s
  constexpr int N2 = kWB * A;  // forward pass-2 = inverse pass-1 items (w, k1), k1 < A: rows k1 + A*k2
  constexpr int N3 = kWB * B;  // inverse pass-2 items (w, k1'), k1' < B: rows k1' + B*k2
  constexpr int NI1 = cdiv(N1, NT), NI2 = cdiv(N2, NT), NI3 = cdiv(N3, NT);
  // tensor memory: columns [0, 2A) x at the pass-1 item, [ACC0, ACC0 + 2A) the accumulators
  constexpr bool TM = iter_cols_tmem(H);
  constexpr int ACC0 = (2 * A + 15) / 16 * 16;
  constexpr uint32_t TCOLS = (ACC0 + 2 * A <= 32) ? 32u : (ACC0 + 2 * A <= 64) ? 64u : 128u;
  static_assert(!TM || (N1 == kColNT && N3 == kColNT && NI1 == 1 && NI3 == 1 && ACC0 + 2 * A <= 128),
                "one pass-1 and one pass-3 item on each thread of warps 0-3");
  __shared__ uint32_t tslot;
  extern __shared__ float4 smem4[];
  float2* Sb = reinterpret_cast<float2*>(smem4) + L::S_OFF;
  float2* Yb = reinterpret_cast<float2*>(smem4) + L::Y_OFF;
  float2* ex = reinterpret_cast<float2*>(smem4) + L::EX_OFF;
  float2* tws = reinterpret_cast<float2*>(smem4) + L::TW_OFF;
  int* rcode = reinterpret_cast<int*>(reinterpret_cast<float2*>(smem4) + L::F2_END);
  double* sred = reinterpret_cast<double*>(rcode + H);
  float* fm = reinterpret_cast<float*>(sred + 3 * (NT / 32));
  namespace cgr = cooperative_groups;
  cgr::cluster_group cluster = cgr::this_cluster();

  const int inst = find_inst(bm, blockIdx.z);
  const FusedArgs& a = tab[inst];
  NestaDevState* st = a.st;
  const int t = threadIdx.x;
  const int half = blockIdx.y, f = blockIdx.z - bm.fbase[inst], w0 = blockIdx.x * kWB;
  const int W = a.W, C = a.C, F = a.F;
  const size_t N = size_t(a.N);
  const int rowbase = a.rowoff[f];
  const int nrows = a.rowoff[f + 1] - rowbase;
  // kept rows fit the shared buffers: a frame with more runs the three-pass
  // iteration (the row analysis counts it in partial_rows, checked below)
  const bool staged = nrows <= RCAP;
  const int cmid = (C + 1) / 2;
  const int cbeg = half ? cmid : 0, cend = half ? C : cmid;

  // S and IDFT_W(y) (in T since the setup) are inputs of the whole solve: they
  // are staged before the dependency wait
  // this thread's 16-byte granules of an S tile: rows srow + i*RSTEP, columns
  // 2*spart, 2*spart + 1 (the granule pattern repeats every RSTEP rows)
  constexpr int GPR = kWB / 2, RSTEP = NT / GPR;
  const int srow = t / GPR, spart = t % GPR;
  const float2* const s_src0 = a.S + size_t(srow) * W + w0 + 2 * spart;
  const float2* const t_src0 = a.T + size_t(rowbase) * C * W + w0;
  auto issue_S = [&](int c, int buf) {
    float2* dst = Sb + (L::SB == 2 ? buf : 0) * H * kWB;
    if constexpr (H % RSTEP == 0) {
      const float2* src = s_src0 + size_t(c) * N;
      float2* d0 = dst + srow * kWB + 2 * spart;
#pragma unroll
      for (int i = 0; i < H / RSTEP; ++i) cp_async16(d0 + i * RSTEP * kWB, src + size_t(i) * RSTEP * W);
    } else {
      const float2* src = a.S + size_t(c) * N + w0;
      for (int q = t; q < H * GPR; q += NT) {
        const int row = q / GPR, part = q % GPR;
        cp_async16(dst + row * kWB + 2 * part, src + size_t(row) * W + 2 * part);
      }
    }
  };
  auto issue_Y = [&](int c, int buf) {
    if (staged) {
      const float2* src = t_src0 + size_t(c) * W;
      float2* dst = Yb + buf * RCAP * kWB;
      for (int q = t; q < nrows * (kWB / 2); q += NT) {
        const int j = q / (kWB / 2), part = q % (kWB / 2);
        cp_async16(dst + j * kWB + 2 * part, src + size_t(j) * C * W + 2 * part);
      }
    }
  };
  if (cbeg < cend) {
    issue_S(cbeg, 0);
    issue_Y(cbeg, 0);
  }
  cp_async_commit();
  // row codes: j >= 0 fully sampled kept row j; -2 - j kept row j without
  // samples (data only); -1 not kept
  for (int i = t; i < H; i += NT) {
    const int j = a.rowmap[f * H + i];
    rcode[i] = (j < 0) ? -1 : (a.row_full[rowbase + j] ? j : -2 - j);
  }
  // twiddles, stored per item so that a thread reads its own as consecutive
  // pairs: row s, entry k1 = w_H^(s*k1) (forward first pass) and row k1,
  // entry k1' = w_H^(k1*k1') (inverse first pass); the global table holds them
  // as [k1*B + s] and [H + k1'*A + k1]
  for (int d = t; d < L::TWI_OFF + A * L::TWI; d += NT) {
    if (d < L::TWI_OFF) {
      const int s = d / L::TWF, k1 = d % L::TWF;
      if (k1 < A) tws[d] = __ldg(a.twH + k1 * B + s);
    } else {
      const int k1 = (d - L::TWI_OFF) / L::TWI, k1p = (d - L::TWI_OFF) % L::TWI;
      if (k1p < B) tws[d] = __ldg(a.twH + H + k1p * A + k1);
    }
  }
  // Plain form: x_k, w_k and the scalar state come from the previous launch,
  // the previous iteration.  Motion-compensated form: the launch before this
  // one is M^T(tTVadj u) (k_mc_adjoint, after the fused tTV kernel that also
  // writes the objective's tTV sums), which only the update below reads, after
  // a later wait; the previous iteration is three launches back and complete
  // when this kernel starts (both motion kernels release their successors only
  // after their own waits).
  constexpr bool motion = MOTION;
  if constexpr (!motion) grid_dep_wait();
  grid_dep_release();

  // which update this launch computes (uniform over the instance, so over each cluster)
  const int last = st->last_iter;
  bool fix = false;
  int itx = it;
  if (st->partial_rows) {  // the data changed under a captured row-local solve
    if (t == 0 && half == 0 && blockIdx.x == 0 && f == 0 && it == 0) st->status = kStatusRowStructure;
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
  const float2* __restrict__ xk = (itx & 1) ? a.xk1 : a.xk0;
  float2* __restrict__ xn = (itx & 1) ? a.xk0 : a.xk1;
  const float2* __restrict__ wk = (itx & 1) ? a.wacc1 : a.wacc;
  float2* __restrict__ wn = (itx & 1) ? a.wacc : a.wacc1;
  const float2* __restrict__ x = xk + size_t(f) * N;
  const float inv_mu = 1.0f / st->mu;

  uint32_t tl = 0;  // this thread's TMEM lane
  if constexpr (TM) {
    if (t < 32) {
      tc::tmem_alloc(&tslot, TCOLS);
      tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    tl = tslot + (uint32_t(32 * (t >> 5)) << 16);
  }
  // x_k at this thread's forward pass-1 items, reused for every coil
  float2 xv[NI1][A];
#pragma unroll
  for (int ii = 0; ii < NI1; ++ii) {
    const int i = t + ii * NT;
    if (i < N1) {
      const int w = i % kWB, s = i / kWB;
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) xv[ii][n1] = x[size_t(B * n1 + s) * W + w0 + w];
    }
  }

  float2 acc[NI3][A];
#pragma unroll
  for (int ii = 0; ii < NI3; ++ii)
#pragma unroll
    for (int k2 = 0; k2 < A; ++k2) acc[ii][k2] = make_float2(0.f, 0.f);
  if constexpr (TM) {  // x and the zeroed accumulators move to tensor memory for the coil loop
    if (t < N1) tmem_pieces<2 * A>([&](auto oc, auto nc) {
      constexpr int o = decltype(oc)::value, n = decltype(nc)::value;
      float xf[n], zf[n];
#pragma unroll
      for (int e = 0; e < n / 2; ++e) {
        xf[2 * e] = xv[0][o / 2 + e].x;
        xf[2 * e + 1] = xv[0][o / 2 + e].y;
        zf[2 * e] = zf[2 * e + 1] = 0.f;
      }
      tmem_st_n<n>(tl + o, xf);
      tmem_st_n<n>(tl + ACC0 + o, zf);
    });
    if (t < N1) tc::tmem_wait_st();
  }
  const float s_row = a.s_row;
  float racc = 0.f;
  // kept rows of each pass-2 item (w, k1): bit k2 for row k1 + A*k2
  __syncthreads();  // row codes written
  unsigned kept[NI2];
#pragma unroll
  for (int ii = 0; ii < NI2; ++ii) {
    kept[ii] = 0u;
    const int k1 = (t + ii * NT) / kWB;
    if (t + ii * NT < N2) {
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) kept[ii] |= (rcode[k1 + A * k2] != -1 ? 1u : 0u) << k2;
    }
  }

  for (int c = cbeg; c < cend; ++c) {
    const int buf = (c - cbeg) & 1;
    cp_async_wait<0>();
    __syncthreads();  // coil c staged; the previous coil's inverse pass 2 has read the exchange
    if (c + 1 < cend) {
      if constexpr (L::SB == 2) issue_S(c + 1, buf ^ 1);  // one buffer: copied once this coil's pass 2 read S
      issue_Y(c + 1, buf ^ 1);
    }
    cp_async_commit();
    const float2* Sc = Sb + (L::SB == 2 ? buf : 0) * H * kWB;
    const float2* Yc = Yb + buf * RCAP * kWB;
    // forward pass 1: S_c x_f, DFT_A, twiddles
#pragma unroll
    for (int ii = 0; ii < NI1; ++ii) {
      const int i = t + ii * NT;
      if (i < N1) {
        const int w = i % kWB, s = i / kWB;
        float2 v[A];
        if constexpr (TM) {
          tmem_pieces<2 * A>([&](auto oc, auto nc) {
            constexpr int o = decltype(oc)::value, n = decltype(nc)::value;
            float xf[n];
            tmem_ld_n<n>(tl + o, xf);
#pragma unroll
            for (int e = 0; e < n / 2; ++e)
              v[o / 2 + e] = cmul(make_float2(xf[2 * e], xf[2 * e + 1]), Sc[(B * (o / 2 + e) + s) * kWB + w]);
          });
        } else {
#pragma unroll
          for (int n1 = 0; n1 < A; ++n1) v[n1] = cmul(xv[ii][n1], Sc[(B * n1 + s) * kWB + w]);
        }
        dft<A>(v);
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) ex[k1 * KSF + s * kWB + w] = (k1 == 0) ? v[k1] : cmul(v[k1], twiddle<A>(tws + s * L::TWF, k1));
      }
    }
    __syncthreads();
    // forward pass 2 (DFT_B: row k1 + A*k2) and the residual on the kept rows
    float2 r[NI2][B];
#pragma unroll
    for (int ii = 0; ii < NI2; ++ii) {
      const int i = t + ii * NT;
      if (i < N2) {
        const int w = i % kWB, k1 = i / kWB;
#pragma unroll
        for (int s = 0; s < B; ++s) r[ii][s] = ex[k1 * KSF + s * kWB + w];
        dft<B>(r[ii]);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) {
          float2 q = make_float2(0.f, 0.f);
          if (kept[ii] & (1u << k2)) {
            const int code = rcode[k1 + A * k2];
            const int j = code >= 0 ? code : -2 - code;
            const float2 yv = Yc[j * kWB + w];
            q = (code >= 0) ? csub(cscale(r[ii][k2], s_row), yv) : make_float2(-yv.x, -yv.y);
            racc = fmaf(q.x, q.x, fmaf(q.y, q.y, racc));
          }
          r[ii][k2] = conjf2(q);  // the inverse transform runs on the conjugate
        }
      }
    }
    __syncthreads();  // every forward pass-2 read of the exchange is done
    // inverse pass 1 on the same items: DFT_B over rows A*n1 + k1, twiddles
#pragma unroll
    for (int ii = 0; ii < NI2; ++ii) {
      const int i = t + ii * NT;
      if (i < N2) {
        const int w = i % kWB, k1 = i / kWB;
        dft<B>(r[ii]);
#pragma unroll
        for (int k1p = 0; k1p < B; ++k1p)
          ex[k1p * KSI + k1 * kWB + w] = (k1p == 0) ? r[ii][k1p] : cmul(r[ii][k1p], twiddle<B>(tws + L::TWI_OFF + k1 * L::TWI, k1p));
      }
    }
    __syncthreads();
    // inverse pass 2 (DFT_A: row k1' + B*k2) and conj(S_c) accumulation
#pragma unroll
    for (int ii = 0; ii < NI3; ++ii) {
      const int i = t + ii * NT;
      if (i < N3) {
        const int w = i % kWB, k1p = i / kWB;
        float2 v[A];
#pragma unroll
        for (int s = 0; s < A; ++s) v[s] = ex[k1p * KSI + s * kWB + w];
        dft<A>(v);
        // conj(v) * conj(S) == conj(v * S), formed as cmul's negated imaginary part
        auto term = [&](int k2) {
          const float2 sv = Sc[(k1p + B * k2) * kWB + w];
          return make_float2(fmaf(v[k2].x, sv.x, -v[k2].y * sv.y), fmaf(-v[k2].x, sv.y, -(v[k2].y * sv.x)));
        };
        if constexpr (TM) {
          tc::tmem_wait_st();  // the previous coil's accumulator stores
          tmem_pieces<2 * A>([&](auto oc, auto nc) {
            constexpr int o = decltype(oc)::value, n = decltype(nc)::value;
            float af[n];
            tmem_ld_n<n>(tl + ACC0 + o, af);
#pragma unroll
            for (int e = 0; e < n / 2; ++e) {
              const float2 sum = padd(make_float2(af[2 * e], af[2 * e + 1]), term(o / 2 + e));
              af[2 * e] = sum.x;
              af[2 * e + 1] = sum.y;
            }
            tmem_st_n<n>(tl + ACC0 + o, af);
          });
        } else {
#pragma unroll
          for (int k2 = 0; k2 < A; ++k2) acc[ii][k2] = padd(acc[ii][k2], term(k2));
        }
      }
    }
    if constexpr (L::SB == 1) {  // one S buffer: the next coil's copy starts once every thread has read this one
      if (c + 1 < cend) {
        __syncthreads();
        issue_S(c + 1, 0);
        cp_async_commit();
      }
    }
  }
  if constexpr (TM) {  // x and the accumulators back to registers; the tensor memory is released
    if (t < N1) tc::tmem_wait_st();
    if (t < N1) tmem_pieces<2 * A>([&](auto oc, auto nc) {
      constexpr int o = decltype(oc)::value, n = decltype(nc)::value;
      float xf[n], af[n];
      tmem_ld_n<n>(tl + o, xf);
      tmem_ld_n<n>(tl + ACC0 + o, af);
#pragma unroll
      for (int e = 0; e < n / 2; ++e) {
        xv[0][o / 2 + e] = make_float2(xf[2 * e], xf[2 * e + 1]);
        acc[0][o / 2 + e] = make_float2(af[2 * e], af[2 * e + 1]);
      }
    });
    tc::fence_before_sync();
    __syncthreads();
    if (t < 32) tc::tmem_dealloc(tslot, TCOLS);
  }

  // tTV objective partial sums over the tile, each CTA of the pair over half
  // of its pass-1 items (s < B/2 for the first, whole warps); not in fixup mode
  float su2 = 0.f, sud = 0.f;
  if (!fix && !motion) {  // the motion-compensated form has them from k_mc_tv
    const float2* __restrict__ xm = xk + size_t((f + F - 1) % F) * N;
#pragma unroll
    for (int ii = 0; ii < NI1; ++ii) {
      const int i = t + ii * NT;
      if (i < N1 && ((i / kWB < B / 2) == (half == 0))) {
        const int w = i % kWB, s = i / kWB;
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) {
          const float2 d = csub(xv[ii][n1], xm[size_t(B * n1 + s) * W + w0 + w]);
          const float2 u = tv_normalize(d, inv_mu);
          su2 = fmaf(u.x, u.x, fmaf(u.y, u.y, su2));
          sud = fmaf(u.x, d.x, fmaf(u.y, d.y, sud));
        }
      }
    }
  }

  // This CTA finishes half of the tile's rows (k2 < A/2 for the first).  The
  // update's operands at those rows (x_k and its neighbouring frames, w_k,
  // x_ref: independent of the accumulators) are requested between the two
  // halves of the cluster barrier below, so that they arrive during the
  // exchange.
  constexpr int KH = A / 2, KM = A - KH;
  const int kb = half ? KH : 0, ke = half ? A : KH;
  const size_t offm = size_t((f + F - 1) % F) * N, off0 = size_t(f) * N, offp = size_t((f + 1) % F) * N;
  // Sum the two halves' accumulators through distributed shared memory.
  cp_async_wait<0>();
  __syncthreads();
  float2* mine = Sb;
#pragma unroll
  for (int ii = 0; ii < NI3; ++ii)
#pragma unroll
    for (int k2 = 0; k2 < A; ++k2)  // the rows the other CTA finishes
      if ((k2 < kb || k2 >= ke) && t + ii * NT < N3) mine[(ii * A + k2) * L::XST + t] = acc[ii][k2];
  // the cluster barrier in two halves: the arrive publishes this CTA's rows
  // (release), the update's operands are requested while the partner gets
  // there, and the wait makes the partner's rows visible (acquire)
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  // (x_k, w_k and x_ref for every form with one pass-3 item per thread and
  // A <= 24 at 168 registers a thread; the neighbouring frames too for the
  // plain form at A <= 16; the rest after the exchange)
  constexpr bool PRE = NI3 == 1 && (A <= 16 || (A <= 24 && NT == kColNT));
  constexpr bool PRE_T = PRE && !MOTION && A <= 16;
  float2 pxa[PRE ? KM : 1], pxm[PRE ? KM : 1], pxp[PRE ? KM : 1], pwo[PRE ? KM : 1], pxr[PRE ? KM : 1];
  if constexpr (PRE) {
    if (t < N3) {
      const int w = t % kWB, k1p = t / kWB;
#pragma unroll
      for (int k = 0; k < KM; ++k) {
        if (kb + k < ke) {
          const size_t p = size_t(k1p + B * (kb + k)) * W + w0 + w;
          pxa[k] = xk[off0 + p];
          if constexpr (PRE_T) {
            pxm[k] = xk[offm + p];
            pxp[k] = xk[offp + p];
          }
          pwo[k] = wk[off0 + p];
          pxr[k] = a.xref[off0 + p];
        }
      }
    }
  }

  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
  const float2* other = cluster.map_shared_rank(mine, half ^ 1);
#pragma unroll
  for (int ii = 0; ii < NI3; ++ii)
#pragma unroll
    for (int k2 = 0; k2 < A; ++k2)
      if (k2 >= kb && k2 < ke && t + ii * NT < N3) {
        const float2 o = other[(ii * A + k2) * L::XST + t];
        acc[ii][k2] = half ? cadd(o, acc[ii][k2]) : cadd(acc[ii][k2], o);
      }
  // the partner may still be reading this CTA's rows: signal that this CTA's
  // reads are done now (their values are already consumed above, so the
  // arrive needs no release fence), and wait for the partner's before exiting
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");

  // tTV gradient and Nesterov update of this CTA's rows
  if constexpr (motion) grid_dep_wait();  // M^T(tTVadj u) of x_k
  const float s_adj = a.s_adj;
  const float lambda = st->lambda, nLmu1 = -st->Lmu1;
  const float apk = fix ? st->apk : 0.5f * (float(itx) + 1.0f);  // nesta_scalar_step's weights for k = itx
  const float tauk = fix ? st->tauk : 2.0f / (float(itx) + 3.0f);
  const float omt = 1.0f - tauk;
  // the update of one pixel: x_k, its neighbours in time (or M^T(tTVadj u)),
  // w_k, x_ref and the accumulated A^H r
  auto update = [&](size_t p, float2 xa, float2 xm, float2 xp, float2 wo, float2 xr, float2 accv) {
    // operator_tTVadj gives u_{f+1} - u_f of the normalised temporal
    // differences; NestaUp negates it, scales by lambda, adds A^H r
    float2 adj;
    if constexpr (motion) {
      adj = xm;
    } else {
      const float2 u0 = tv_normalize(csub(xa, xm), inv_mu);
      const float2 u1 = tv_normalize(csub(xp, xa), inv_mu);
      adj = csub(u1, u0);
    }
    const float2 ares = cscale(accv, s_adj);
    const float2 df = make_float2(__fadd_rn(__fmul_rn(-adj.x, lambda), ares.x),
                                  __fadd_rn(__fmul_rn(-adj.y, lambda), ares.y));
    const float2 yk = make_float2(fmaf(nLmu1, df.x, xa.x), fmaf(nLmu1, df.y, xa.y));
    const float2 wnv = make_float2(fmaf(apk, df.x, wo.x), fmaf(apk, df.y, wo.y));
    const float2 zk = make_float2(fmaf(nLmu1, wnv.x, xr.x), fmaf(nLmu1, wnv.y, xr.y));
    wn[off0 + p] = wnv;
    xn[off0 + p] = make_float2(fmaf(omt, yk.x, tauk * zk.x), fmaf(omt, yk.y, tauk * zk.y));
  };
  if constexpr (PRE) {
    if (t < N3) {
      float2 af[KM];  // the accumulators of this CTA's rows
      if (half == 0) {
#pragma unroll
        for (int k = 0; k < KH; ++k) af[k] = acc[0][k];
      } else {
#pragma unroll
        for (int k = 0; k < KM; ++k) af[k] = acc[0][KH + k];
      }
      const int w = t % kWB, k1p = t / kWB;
      if constexpr (!PRE_T) {
#pragma unroll
        for (int k = 0; k < KM; ++k) {
          if (kb + k < ke) {
            const size_t p = size_t(k1p + B * (kb + k)) * W + w0 + w;
            if constexpr (motion) {
              pxm[k] = a.grad_ext[off0 + p];  // M^T (tTVadj u) of the motion-compensated form
            } else {
              pxm[k] = xk[offm + p];
              pxp[k] = xk[offp + p];
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < KM; ++k)
        if (kb + k < ke) update(size_t(k1p + B * (kb + k)) * W + w0 + w, pxa[k], pxm[k], pxp[k], pwo[k], pxr[k], af[k]);
    }
  }
  constexpr int BATCH = A <= 16 ? 8 : 4;  // one round of loads for a CTA's 8 rows at A = 16
#pragma unroll
  for (int ii = 0; ii < (PRE ? 0 : NI3); ++ii) {
    const int i = t + ii * NT;
    if (i < N3) {
      const int w = i % kWB, k1p = i / kWB;
#pragma unroll
      for (int k0 = 0; k0 < A; k0 += BATCH) {
        float2 xa[BATCH], xm[BATCH], xp[BATCH], wo[BATCH], xr[BATCH];
#pragma unroll
        for (int b = 0; b < BATCH; ++b) {
          const int k2 = k0 + b;
          if (k2 < A && k2 >= kb && k2 < ke) {
            const size_t p = size_t(k1p + B * k2) * W + w0 + w;
            xa[b] = xk[off0 + p];
            if constexpr (motion) {
              xm[b] = a.grad_ext[off0 + p];  // M^T (tTVadj u) of the motion-compensated form
            } else {
              xm[b] = xk[offm + p];
              xp[b] = xk[offp + p];
            }
            wo[b] = wk[off0 + p];
            xr[b] = a.xref[off0 + p];
          }
        }
#pragma unroll
        for (int b = 0; b < BATCH; ++b) {
          const int k2 = k0 + b;
          if (k2 < A && k2 >= kb && k2 < ke)
            update(size_t(k1p + B * k2) * W + w0 + w, xa[b], xm[b], xp[b], wo[b], xr[b], acc[ii][k2]);
        }
      }
    }
  }
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
  if (fix) return;

  // fixed-slot partial sums: ||rho||^2 of this CTA, the tTV terms of the tile
  const int blk = f * gridDim.x + blockIdx.x;
  double pr, t1, t2;
  rowlocal_block_sum3<NT>(double(racc), double(su2), double(sud), sred, &pr, &t1, &t2);
  if (t == 0) {
    if (!motion) {  // the motion-compensated form's come from k_mc_tv, in the same buffer
      a.part_tv[2 * (2 * blk + half)] = t1;
      a.part_tv[2 * (2 * blk + half) + 1] = t2;
    }
    a.part_r[2 * blk + half] = pr;
  }
  if (rowlocal_last_cta(bm.ctl, inst, 2u * gridDim.x * unsigned(F)))
    rowlocal_finish<NT>(a, st, bm.ctl, inst, it, apk, motion ? a.ntv : 2 * F * int(gridDim.x),
                            2 * F * int(gridDim.x), sred, fm);
}

}  // namespace gbn
