// Fused per-iteration kernels of the tTV-NESTA solver and the dense FFT
// passes, templated on the transform length.  Instantiated for every supported
// size by inst_*.cu.
//
// Data flow of one inner iteration (NestaUp.cpp:651-880 restated):
//   k_fwd_cols  x_k, S      -> T = DFT_H(S_c x_f) on the kept k-space rows only
//                              (+ partial sums of ||u||^2, Re<u,d>, u = D x_k normalised)
//   k_rows      T, y, mask  -> r = mask*DFT_W(T)/sqrt(N) - y ;  T = IDFT_W(r)
//                              (+ ||r||^2; last block runs the scalar recurrence)
//   k_inv_cols  T, S, x_k   -> A^H r = sum_c conj(S_c) IDFT_H(T) ; tTV gradient and
//                              the Nesterov update x_{k+1}, w_{k+1}
// Column transforms run first in the forward direction so that only the kept
// (sampled) phase-encode rows ever leave the column pass: T holds G*C rows, not
// F*C*H.  The adjoint column transform reads only those rows (others are zero).
//
// Latency hiding: global loads for the next coil (k_fwd_cols, k_inv_cols) or
// for the residual's data row (k_rows) are issued before the current stage's
// arithmetic and barriers, so they are in flight while it runs.
#pragma once

#include <cooperative_groups.h>

#include "fft.cuh"
#include "pdl.cuh"
#include "types.h"

namespace gbn {

constexpr int kWB = 8;       // columns per CTA in the column kernels
constexpr int kColNT = 128;  // threads per CTA in the column kernels
constexpr int kRowNT = 128;  // threads per CTA in the row kernels
constexpr int kRowWarps = kRowNT / 32;


template <int L>
struct Split {
  static constexpr int A = split_a(L);
  static constexpr int B = split_b(L);
  static_assert(A * B == L && A >= 1 && B >= 1, "unsupported transform length");
};

// smallest v' >= v with v' % 16 == 8 (in 8-byte words): staggers groups of
// lanes across the two halves of the shared-memory bank space
constexpr int pad_to_8mod16(int v) { return v + ((8 - v % 16) + 16) % 16; }
constexpr int odd_up(int v) { return (v % 2) ? v : v + 1; }
constexpr int cdiv(int a, int b) { return (a + b - 1) / b; }
// exchange-slot stride between k1 groups of the column kernels (kWB lanes each)
constexpr int col_ks(int q) { return (q * kWB) % 16 == 8 ? q * kWB : q * kWB + 8; }

__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// instance owning grid z index `z` (largest i with fbase[i] <= z)
__device__ __forceinline__ int find_inst(const BatchMap& bm, int z) {
  int lo = 0, hi = bm.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bm.fbase[mid] <= z) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// d / max(mu, |d|) (vectorNormalization.cl:42-56) as d * min(1/mu, 1/|d|):
// one reciprocal square root instead of a square root and two divisions
// (within 2 ulp; d = 0 gives 0).
__device__ __forceinline__ float2 tv_normalize(float2 d, float inv_mu) {
  const float s = fminf(inv_mu, rsqrtf(fmaf(d.x, d.x, d.y * d.y)));
  return make_float2(d.x * s, d.y * s);
}

// ---------------------------------------------------------------------------
// Reference scalar recurrence of one inner iteration: objective, stopping test
// and the Nesterov weights (NestaUp.cpp:791-831), executed by one thread.
// Arithmetic types follow the reference: host floats, std::pow in double.
// ---------------------------------------------------------------------------
// `fm` is a copy of the first min(miniter, kFmeanCopy) entries of fmean.
constexpr int kFmeanCopy = 64;
__device__ inline void nesta_scalar_step(NestaDevState* gst, float* fmean, const float* fm, int it, double su2,
                                         double sud, double sr2) {
  // work on a register copy: one batch of loads instead of a chain of round trips
  NestaDevState loc = *gst;
  NestaDevState* st = &loc;
  const float normUk = float(sqrt(su2));  // Scnrm2(u)
  const float fxdot = float(sud);         // real part of Cdotc(u, d)
  const float l2 = float(sr2);            // Scsum(|res|^2)
  const float mu = st->mu;
  // std::pow(normUk, 2) of a float is exactly its square in double
  const double nu2 = double(normUk) * double(normUk);
  const float l1term = float(double(fxdot) - double(mu / 2.0f) * nu2);
  const float fx = 0.5f * l2 + st->lambda * l1term;
  int k = it;
  float qp = st->qp;
  if (st->stoptest == 1) {
    const int m = st->miniter;
    bool brk = false;
    if (k >= m) {
      float s = 0.0f;
      for (int ne = 0; ne < m; ++ne) {
        const int idx = m - ne - 1;
        s += (idx < kFmeanCopy) ? fm[idx] : fmean[idx];
      }
      s = s / float(unsigned(m));
      qp = (s - fx) / s;
      if (qp <= st->tolVar) {
        if (st->qpDone) k = st->maxIter;  // reference sets k = maxIter: this update is the last
        st->qpDone = 1;
        brk = true;
      }
    } else {
      qp = (m - 1 < kFmeanCopy) ? fm[m - 1] : fmean[m - 1];
    }
    if (!brk) fmean[(m - 1) - int(unsigned(k + 1) % unsigned(m))] = fx;
  }
  const float apk = 0.5f * (float(k) + 1.0f);
  st->Ak = st->Ak + apk;
  const float tauk = 2.0f / (float(k) + 3.0f);
  st->apk = apk;
  st->tauk = tauk;
  st->qp = qp;
  st->fx = fx;
  st->normUk = normUk;
  st->fxdot = fxdot;
  st->l2term = l2;
  st->iters_total += 1;
  if (k >= st->maxIter) st->last_iter = it;  // later inner iterations of this outer loop are skipped
  *gst = loc;
}

// ===========================================================================
// K1: forward column pass.  grid = (W/kWB, coil groups, F), dynamic smem.
// dit2<A,B> along H: pass-1 items (w, s), s < B, hold rows B*n1 + s; pass-2
// items (w, k1), k1 < A, produce rows k1 + A*k2.  The S tile of the next coil
// is copied asynchronously into a second shared buffer while the current coil
// is transformed.
// ===========================================================================
template <int H>
struct FwdColsSmem {
  static constexpr int A = Split<H>::A, B = Split<H>::B, KS = col_ks(B);
  static constexpr int S_OFF = 0;                        // float2 [2][H][kWB]
  static constexpr int EX_OFF = S_OFF + 2 * H * kWB;     // float2 [A*KS]
  static constexpr int F2_END = EX_OFF + A * KS;
  static constexpr int BYTES = F2_END * 8 + (kColNT / 32) * 8 + H * 4;
};

// power-of-two lengths up to 256 fit 4 CTAs per SM without spilling
constexpr int fwd_min_blocks(int H) { return (H <= 256 && (H & (H - 1)) == 0) ? 4 : 1; }

template <int H>
__global__ void __launch_bounds__(kColNT, fwd_min_blocks(H))
    k_fwd_cols(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it, int coils_per_block) {
  using L = FwdColsSmem<H>;
  constexpr int A = L::A, B = L::B, KS = L::KS;
  constexpr int N1 = kWB * B, N2 = kWB * A;
  constexpr int NI1 = cdiv(N1, kColNT), NI2 = cdiv(N2, kColNT);
  extern __shared__ float4 smem4[];
  float2* Sb = reinterpret_cast<float2*>(smem4) + L::S_OFF;
  float2* ex = reinterpret_cast<float2*>(smem4) + L::EX_OFF;
  double* sred = reinterpret_cast<double*>(reinterpret_cast<float2*>(smem4) + L::F2_END);
  int* rmap = reinterpret_cast<int*>(sred + kColNT / 32);

  const int inst = find_inst(bm, blockIdx.z);
  const FusedArgs& a = tab[inst];
  const NestaDevState* st = a.st;
  const int t = threadIdx.x;
  const int f = blockIdx.z - bm.fbase[inst], cg = blockIdx.y, w0 = blockIdx.x * kWB;
  const int W = a.W, C = a.C, F = a.F;
  const int c0 = cg * coils_per_block;
  if (c0 >= C || it > st->last_iter) return;
  const int c1 = min(C, c0 + coils_per_block);
  const size_t N = size_t(a.N);
  const float2* __restrict__ xk = (it & 1) ? a.xk1 : a.xk0;
  const float2* __restrict__ x = xk + size_t(f) * N;

  auto issue_S = [&](int c, int buf) {
    const float2* src = a.S + size_t(c) * N + w0;
    float2* dst = Sb + buf * H * kWB;
    for (int q = t; q < H * (kWB / 2); q += kColNT) {
      const int row = q / (kWB / 2), part = q % (kWB / 2);
      cp_async16(dst + row * kWB + 2 * part, src + size_t(row) * W + 2 * part);
    }
    cp_async_commit();
  };
  issue_S(c0, 0);

  for (int i = t; i < H; i += kColNT) rmap[i] = a.rowmap[f * H + i];
  const int rowbase = a.rowoff[f];
  grid_dep_wait();  // x_k comes from the previous adjoint column pass
  grid_dep_release();

  // x_k for this thread's pass-1 items, reused for every coil
  float2 xv[NI1][A];
#pragma unroll
  for (int ii = 0; ii < NI1; ++ii) {
    const int i = t + ii * kColNT;
    if (i < N1) {
      const int w = i % kWB, s = i / kWB;
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) xv[ii][n1] = x[size_t(B * n1 + s) * W + w0 + w];
    }
  }

  // Partial sums of the tTV objective terms over this CTA's tile (coil group 0
  // only): d = x_f - x_{f-1} (temporalTV.cl:49-76), u = d / max(mu, |d|)
  // (vectorNormalization.cl:42-56), sum |u|^2 (Scnrm2) and Re<u,d> (Cdotc).
  // (with motion compensation the gradient kernel writes these sums instead)
  float su2 = 0.f, sud = 0.f;
  const bool tv_here = (cg == 0) && !a.tv_src;
  if (tv_here) {
    const float2* __restrict__ xm = xk + size_t((f + F - 1) % F) * N;
    const float inv_mu = 1.0f / st->mu;
#pragma unroll
    for (int ii = 0; ii < NI1; ++ii) {
      const int i = t + ii * kColNT;
      if (i < N1) {
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

  // inter-pass twiddles of this thread's pass-1 items, identical for every coil
  float2 twr[NI1][A];
#pragma unroll
  for (int ii = 0; ii < NI1; ++ii) {
    const int i = t + ii * kColNT;
    const int s = (i < N1) ? i / kWB : 0;
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) twr[ii][k1] = __ldg(a.twH + k1 * B + s);
  }

  for (int c = c0; c < c1; ++c) {
    const int buf = (c - c0) & 1;
    cp_async_wait<0>();
    __syncthreads();  // S tile of coil c visible; previous coil's pass 2 finished
    if (c + 1 < c1) issue_S(c + 1, buf ^ 1);
    const float2* Sc = Sb + buf * H * kWB;
#pragma unroll
    for (int ii = 0; ii < NI1; ++ii) {
      const int i = t + ii * kColNT;
      if (i < N1) {
        const int w = i % kWB, s = i / kWB;
        float2 v[A];
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) v[n1] = cmul(xv[ii][n1], Sc[(B * n1 + s) * kWB + w]);
        dft<A>(v);
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) ex[k1 * KS + s * kWB + w] = (k1 == 0) ? v[k1] : cmul(v[k1], twr[ii][k1]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int ii = 0; ii < NI2; ++ii) {
      const int i = t + ii * kColNT;
      if (i < N2) {
        const int w = i % kWB, k1 = i / kWB;
        float2 v[B];
#pragma unroll
        for (int s = 0; s < B; ++s) v[s] = ex[k1 * KS + s * kWB + w];
        dft<B>(v);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) {
          const int j = rmap[k1 + A * k2];
          if (j >= 0) a.T[(size_t(rowbase + j) * C + c) * W + w0 + w] = v[k2];
        }
      }
    }
  }

  if (tv_here) {
    const double t1 = block_sum<kColNT>(double(su2), sred);
    const double t2 = block_sum<kColNT>(double(sud), sred);
    if (t == 0) {
      const int blk = f * gridDim.x + blockIdx.x;
      a.part_tv[2 * blk] = t1;
      a.part_tv[2 * blk + 1] = t2;
    }
  }
}

// ===========================================================================
// K2: row pass over kept rows in steps of RPC rows taken by a persistent grid
// from a device counter; the next step's rows (T, y, mask) are staged into
// shared memory with cp.async while the current step is transformed.
//   RESID: r = mask * DFT_W(T)/sqrt(N) - y, T = IDFT_W(r), ||r||^2 partials.
//   !RESID (adjoint of the data, x0 = E^H y): T = IDFT_W(y).
// ===========================================================================
template <int W>
struct RowCfg {
  static constexpr int A = Split<W>::A, B = Split<W>::B;
  static constexpr int MX = A > B ? A : B;
  static constexpr int RPC = (kRowNT / MX) > 0 ? kRowNT / MX : 1;  // rows per CTA step
  static constexpr int S1 = odd_up(B), RS1 = pad_to_8mod16(A * S1);   // forward slots (k1, s)
  static constexpr int S2 = odd_up(A), RS2 = pad_to_8mod16(B * S2);   // inverse slots (k1', s')
  static constexpr int EXN = RPC * (RS1 > RS2 ? RS1 : RS2);           // shared exchange buffer
};

template <int W, bool RESID>
struct RowsSmem {
  using R = RowCfg<W>;
  static constexpr int Y_OFF = 0;                                 // float2 [2][RPC][W]
  static constexpr int T_OFF = Y_OFF + 2 * R::RPC * W;            // float2 [RPC][W] (RESID)
  static constexpr int EX_OFF = T_OFF + (RESID ? R::RPC * W : 0); // float2 [EXN]
  static constexpr int F2_END = EX_OFF + R::EXN;
  static constexpr int M_BYTES = RESID ? 2 * R::RPC * W : 0;      // uint8 [2][RPC][W]
  static constexpr int BYTES = F2_END * 8 + (kRowNT / 32) * 8 + M_BYTES + 16;
};

template <int W, bool RESID>
__global__ void __launch_bounds__(kRowNT)
    k_rows(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it) {
  using R = RowCfg<W>;
  using L = RowsSmem<W, RESID>;
  constexpr int A = R::A, B = R::B, RPC = R::RPC;
  extern __shared__ float4 smem4[];
  float2* Yb = reinterpret_cast<float2*>(smem4) + L::Y_OFF;
  float2* Tb = reinterpret_cast<float2*>(smem4) + L::T_OFF;
  float2* ex = reinterpret_cast<float2*>(smem4) + L::EX_OFF;
  double* sred = reinterpret_cast<double*>(reinterpret_cast<float2*>(smem4) + L::F2_END);
  uint8_t* Mb = reinterpret_cast<uint8_t*>(sred + kRowNT / 32);
  __shared__ int s_fin, s_last;
  __shared__ int s_q[2];                    // claimed steps: current and next
  __shared__ int sb[kMaxBatch + 1];         // step_base of the launch's instances
  __shared__ int sn[kMaxBatch];             // their kept rows x coils
  __shared__ unsigned char sact[kMaxBatch];  // instance runs this iteration
  // rows of the two staged steps: data row, mask row (nullptr: fully sampled)
  __shared__ const float2* meta_y[2][RPC];
  __shared__ const uint8_t* meta_m[2][RPC];

  const int n = bm.n;
  if (RESID && n == 1 && it > tab[0].st->last_iter) return;  // uniform: the only instance has finished
  const int t = threadIdx.x;
  for (int i = t; i <= n; i += kRowNT) {
    sb[i] = bm.ctl->step_base[i];
    if (i < n) {
      sn[i] = bm.ctl->nitems[i];
      sact[i] = (!RESID || it <= tab[i].st->last_iter) ? 1 : 0;
    }
  }
  __syncthreads();
  const int nsteps = sb[n];
  auto inst_of = [&](int step) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sb[mid] <= step) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  };
  // Dynamic assignment from the group's step counter, one step ahead: while
  // a CTA transforms step k it already knows step k+1 (whose rows it is
  // staging) and claims step k+2.  Steps of instances that have finished their
  // iterations are skipped by moving the counter past them.  (thread 0)
  ClassCtl* ctl = bm.ctl;
  auto claim = [&]() {
    int s = atomicAdd(&ctl->row_next, 1);
    if (RESID && n > 1) {
      while (s < nsteps) {
        const int i = inst_of(s);
        if (sact[i]) break;
        atomicMax(&ctl->row_next, sb[i + 1]);
        s = atomicAdd(&ctl->row_next, 1);
      }
    }
    return s;
  };

  // Row lookups of step `step` for row r (thread r < RPC): data and mask rows.
  struct RowRef {
    const float2* y;
    const uint8_t* m;
  };
  auto lookup = [&](int step, int r) {
    RowRef rr{nullptr, nullptr};
    if (step < nsteps) {
      const int i = inst_of(step);
      const FusedArgs& ai = tab[i];
      const int item = (step - sb[i]) * RPC + r;
      if (item < sn[i]) {
        const int C = ai.C, H = ai.H, g = item / C, c = item % C;
        const int f = __ldg(ai.rows_f + g), h = __ldg(ai.rows_h + g);
        rr.y = ai.y + ((size_t(f) * C + c) * H + h) * size_t(W);
        if (RESID && !__ldg(ai.row_full + g)) rr.m = ai.mask + (size_t(f) * H + h) * size_t(W);
      }
    }
    return rr;
  };
  // copies of the staged rows of a step (metadata in slot `buf`)
  auto issue_y = [&](int buf) {
#pragma unroll
    for (int r = 0; r < RPC; ++r) {
      const float2* ys = meta_y[buf][r];
      const uint8_t* ms = meta_m[buf][r];
      if (ys) {
        for (int part = t; part < W / 2; part += kRowNT)
          cp_async16(Yb + (buf * RPC + r) * W + 2 * part, ys + 2 * part);
        if (RESID && ms) {
          for (int part = t; part < W / 8; part += kRowNT)
            cp_async8(Mb + (buf * RPC + r) * W + 8 * part, ms + 8 * part);
        }
      }
    }
  };
  auto issue_T = [&](int step) {
    const int i = inst_of(step);
    const int base = (step - sb[i]) * RPC, nitems = sn[i];
    const float2* T = tab[i].T;
    for (int q = t; q < RPC * (W / 2); q += kRowNT) {
      const int r = q / (W / 2), part = q % (W / 2), item = base + r;
      if (item < nitems) cp_async16(Tb + r * W + 2 * part, T + size_t(item) * W + 2 * part);
    }
  };

  if (t == 0) {
    s_q[0] = claim();
    s_q[1] = claim();
  }
  __syncthreads();
  int step = s_q[0];
  if (t < RPC) {
    const RowRef rr = lookup(step, t);
    meta_y[0][t] = rr.y;
    meta_m[0][t] = rr.m;
  }
  // inter-pass twiddles: RPC * max(A, B) <= kRowNT, so every thread has at
  // most one item per pass and keeps it at every step (pass A: s = t % B,
  // backward pass 1: k1 = t % A); their twiddles live in registers
  static_assert(RPC * B <= kRowNT && RPC * A <= kRowNT, "one item per thread and pass");
  const float2* __restrict__ twW = tab[0].twW;
  float2 twa[A], twb[B];
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) twa[k1] = __ldg(twW + k1 * B + (t % B));
#pragma unroll
  for (int k1p = 0; k1p < B; ++k1p) twb[k1p] = __ldg(twW + W + k1p * A + (t % A));
  __syncthreads();
  if (step < nsteps) issue_y(0);  // data rows: inputs, not written by the predecessor
  grid_dep_wait();
  grid_dep_release();
  if (RESID && step < nsteps) issue_T(step);
  cp_async_commit();
  const float s_fwd = tab[0].s_fwd;
  int buf = 0;
  int run = 0;  // steps of the current instance since the last count

  while (step < nsteps) {
    const int next = s_q[buf ^ 1];
    // the next step's row lookups and the claim of the one after are in
    // flight while this step is transformed
    const RowRef nref = (t < RPC) ? lookup(next, t) : RowRef{nullptr, nullptr};
    const int after = (t == 0 && next < nsteps) ? claim() : nsteps;
    const int inst = inst_of(step);
    const FusedArgs& ai = tab[inst];
    const int lstep = step - sb[inst];
    const int base = lstep * RPC, nitems = sn[inst], C = ai.C;
    cp_async_wait<0>();
    __syncthreads();  // rows of `step` visible; slot buf^1 and the exchange are free
    const float2* Yc = Yb + buf * RPC * W;
    const uint8_t* Mc = Mb + buf * RPC * W;

    if constexpr (RESID) {
      for (int i = t; i < RPC * B; i += kRowNT) {
        const int r = i / B, s = i % B;
        if (base + r >= nitems) continue;
        float2 v[A];
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) v[n1] = Tb[r * W + B * n1 + s];
        dft<A>(v);
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) ex[r * R::RS1 + k1 * R::S1 + s] = (k1 == 0) ? v[k1] : cmul(v[k1], twa[k1]);
      }
    }
    if (t < RPC) {
      meta_y[buf ^ 1][t] = nref.y;
      meta_m[buf ^ 1][t] = nref.m;
    }
    if (t == 0) s_q[buf] = after;  // every thread read s_q before the first barrier
    __syncthreads();  // Tb consumed, exchange filled, next step's rows known
    if (next < nsteps) {
      issue_y(buf ^ 1);
      if (RESID) issue_T(next);
    }
    cp_async_commit();
    // pass B (+ residual) and the first pass of the backward row transform;
    // each thread has at most one item
    const int r = t / A, k1 = t % A, q = base + r;
    const bool has = (t < RPC * A) && (q < nitems);
    float racc = 0.f;
    float2 v[B];
    if (has) {
      if constexpr (RESID) {
#pragma unroll
        for (int s = 0; s < B; ++s) v[s] = ex[r * R::RS1 + k1 * R::S1 + s];
      }
    }
    if constexpr (RESID) __syncthreads();  // exchange reused by the backward pass
    if (has) {
      if constexpr (RESID) {
        const bool full = meta_m[buf][r] == nullptr;
        dft<B>(v);  // v[k2] = X[k1 + A*k2]
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) {
          const int kx = k1 + A * k2;
          float2 m = cscale(v[k2], s_fwd);
          if (!full && Mc[r * W + kx] == 0) m = make_float2(0.f, 0.f);
          const float2 rr = csub(m, Yc[r * W + kx]);
          racc = fmaf(rr.x, rr.x, fmaf(rr.y, rr.y, racc));
          v[k2] = conjf2(rr);
        }
      } else {
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) v[k2] = conjf2(Yc[r * W + k1 + A * k2]);
      }
      // backward = conj(forward(conj)); forward dit2<B,A>, pass-1 item s' = k1
      dft<B>(v);
#pragma unroll
      for (int k1p = 0; k1p < B; ++k1p)
        ex[r * R::RS2 + k1p * R::S2 + k1] = (k1p == 0) ? v[k1p] : cmul(v[k1p], twb[k1p]);
    }
    __syncthreads();
    for (int i = t; i < RPC * B; i += kRowNT) {
      const int rr = i / B, k1p = i % B, qq = base + rr;
      if (qq >= nitems) continue;
      float2 u[A];
#pragma unroll
      for (int sp = 0; sp < A; ++sp) u[sp] = ex[rr * R::RS2 + k1p * R::S2 + sp];
      dft<A>(u);
      float2* __restrict__ dst = ai.T + size_t(qq) * W;
#pragma unroll
      for (int k2p = 0; k2p < A; ++k2p) dst[k1p + B * k2p] = conjf2(u[k2p]);
    }

    if constexpr (RESID) {
      // ||r||^2 of this step, one partial per warp (fixed slots, so the final
      // sum does not depend on which CTA ran which step)
      double pr = double(racc);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) pr += __shfl_down_sync(0xffffffffu, pr, o);
      if ((t & 31) == 0) ai.part_r[lstep * kRowWarps + (t >> 5)] = pr;
      ++run;
      // at the end of a run of steps of one instance, count them; the CTA that
      // completes the instance reduces its partial sums and runs its scalar
      // recurrence
      const int nst = sb[inst + 1] - sb[inst];
      const bool run_ends = (next >= nsteps) || (inst_of(next) != inst);
      if (run_ends) {
        if ((t & 31) == 0) __threadfence();  // this warp's partials before the count
        __syncthreads();
        if (t == 0) {
          const unsigned dn = atomicAdd(&ctl->done[inst], unsigned(run));
          s_fin = (dn + unsigned(run) == unsigned(nst)) ? 1 : 0;
        }
        run = 0;
        __syncthreads();
      }
      if (run_ends && s_fin) {
        __threadfence();
        NestaDevState* st = ai.st;
        __shared__ float fm[kFmeanCopy];
        if (t < kFmeanCopy && t < st->miniter) fm[t] = __ldcg(ai.fmean + t);
        // loads of each batch are issued together; the summation order is fixed
        constexpr int U = 16;
        double su2 = 0.0, sud = 0.0, sr2 = 0.0;
        const double2* ptv = reinterpret_cast<const double2*>(ai.part_tv);
        const int ntv = ai.ntv;
        for (int i0 = 0; i0 < ntv; i0 += U * kRowNT) {
          double2 vv[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int i = i0 + u * kRowNT + t;
            vv[u] = (i < ntv) ? __ldcg(ptv + i) : make_double2(0.0, 0.0);
          }
#pragma unroll
          for (int u = 0; u < U; ++u) {
            su2 += vv[u].x;
            sud += vv[u].y;
          }
        }
        const int npr = nst * kRowWarps;
        for (int i0 = 0; i0 < npr; i0 += 2 * U * kRowNT) {
          double vv[2 * U];
#pragma unroll
          for (int u = 0; u < 2 * U; ++u) {
            const int i = i0 + u * kRowNT + t;
            vv[u] = (i < npr) ? __ldcg(ai.part_r + i) : 0.0;
          }
#pragma unroll
          for (int u = 0; u < 2 * U; ++u) sr2 += vv[u];
        }
        su2 = block_sum<kRowNT>(su2, sred);
        sud = block_sum<kRowNT>(sud, sred);
        sr2 = block_sum<kRowNT>(sr2, sred);
        if (t == 0) {
          nesta_scalar_step(st, ai.fmean, fm, it, su2, sud, sr2);
          ctl->done[inst] = 0;
        }
        __syncthreads();
      }
    }
    step = next;
    buf ^= 1;
  }
  cp_async_wait<0>();

  // the last CTA to finish resets the step counter for the next launch
  if (t == 0) {
    __threadfence();
    s_last = (atomicAdd(&ctl->ticket, 1u) == gridDim.x - 1) ? 1 : 0;
    if (s_last) {
      ctl->row_next = 0;
      ctl->ticket = 0;
    }
  }
}

// ===========================================================================
// K3: adjoint column pass with coil combination, plus (UPDATE) the tTV
// gradient and the Nesterov update, or (!UPDATE) x0 = E^H y into x_ref.
// grid = (W/kWB, 2, F) in clusters of 2 CTAs along y: the two CTAs of a
// cluster share one (frame, 8-column) tile and take the first and second half
// of the coils; their accumulators are summed through distributed shared
// memory and each CTA then finishes half of the tile's rows.
// backward transform along H = conj(forward dit2<B,A>(conj)): pass-1 items
// (w, s), s < A, hold rows A*n1 + s; pass-2 items (w, k1'), k1' < B, produce
// rows k1' + B*k2.  The next coil's S tile and kept T rows are copied
// asynchronously into second shared buffers while the current coil runs.
// ===========================================================================
template <int H>
struct InvColsSmem {
  static constexpr int A = Split<H>::A, B = Split<H>::B, KS = col_ks(A);
  static constexpr int RCAP = H / 2;                     // kept rows staged in shared memory
  static constexpr int S_OFF = 0;                        // float2 [2][H][kWB]
  static constexpr int T_OFF = S_OFF + 2 * H * kWB;      // float2 [2][RCAP][kWB] (kept rows, compact)
  static constexpr int EX_OFF = T_OFF + 2 * RCAP * kWB;  // float2 [B*KS]
  static constexpr int F2_END = EX_OFF + B * KS;
  static constexpr int BYTES = F2_END * 8 + H * 4;
  static_assert(cdiv(kWB * B, kColNT) * A * kColNT <= 2 * H * kWB, "accumulator exchange must fit the S buffers");
};

template <int H, bool UPDATE>
__global__ void __cluster_dims__(1, 2, 1) __launch_bounds__(kColNT)
    k_inv_cols(const FusedArgs* __restrict__ tab, const __grid_constant__ BatchMap bm, int it) {
  using L = InvColsSmem<H>;
  constexpr int A = L::A, B = L::B, KS = L::KS, RCAP = L::RCAP;
  constexpr int N1 = kWB * A, N2 = kWB * B;
  constexpr int NI1 = cdiv(N1, kColNT), NI2 = cdiv(N2, kColNT);
  extern __shared__ float4 smem4[];
  float2* Sb = reinterpret_cast<float2*>(smem4) + L::S_OFF;
  float2* Tb = reinterpret_cast<float2*>(smem4) + L::T_OFF;
  float2* ex = reinterpret_cast<float2*>(smem4) + L::EX_OFF;
  int* rmap = reinterpret_cast<int*>(reinterpret_cast<float2*>(smem4) + L::F2_END);
  namespace cgr = cooperative_groups;
  cgr::cluster_group cluster = cgr::this_cluster();

  const int inst = find_inst(bm, blockIdx.z);
  const FusedArgs& a = tab[inst];
  const NestaDevState* st = a.st;
  const int t = threadIdx.x;
  const int half = blockIdx.y, f = blockIdx.z - bm.fbase[inst], w0 = blockIdx.x * kWB;
  const int W = a.W, C = a.C, F = a.F;
  const size_t N = size_t(a.N);
  const int rowbase = a.rowoff[f];
  const int nrows = a.rowoff[f + 1] - rowbase;
  const bool staged = nrows <= RCAP;  // kept rows fit the shared buffers (uniform per CTA)
  const int cmid = (C + 1) / 2;
  const int cbeg = half ? cmid : 0, cend = half ? C : cmid;

  auto issue_S = [&](int c, int buf) {
    const float2* src = a.S + size_t(c) * N + w0;
    float2* dst = Sb + buf * H * kWB;
    for (int q = t; q < H * (kWB / 2); q += kColNT) {
      const int row = q / (kWB / 2), part = q % (kWB / 2);
      cp_async16(dst + row * kWB + 2 * part, src + size_t(row) * W + 2 * part);
    }
  };
  auto issue_T = [&](int c, int buf) {
    if (staged) {
      const float2* tsrc = a.T + (size_t(rowbase) * C + c) * W + w0;
      float2* tdst = Tb + buf * RCAP * kWB;
      for (int q = t; q < nrows * (kWB / 2); q += kColNT) {
        const int j = q / (kWB / 2), part = q % (kWB / 2);
        cp_async16(tdst + j * kWB + 2 * part, tsrc + size_t(j) * C * W + 2 * part);
      }
    }
  };
  if (cbeg < cend) issue_S(cbeg, 0);
  for (int i = t; i < H; i += kColNT) rmap[i] = a.rowmap[f * H + i];
  grid_dep_wait();  // T and the scalar state come from the row pass
  grid_dep_release();
  if (UPDATE && it > st->last_iter) {  // uniform over the instance, so over each cluster
    cp_async_commit();
    cp_async_wait<0>();
    return;
  }
  if (cbeg < cend) issue_T(cbeg, 0);
  cp_async_commit();

  float2 acc[NI2][A];
#pragma unroll
  for (int ii = 0; ii < NI2; ++ii)
#pragma unroll
    for (int k2 = 0; k2 < A; ++k2) acc[ii][k2] = make_float2(0.f, 0.f);
  __syncthreads();
  // inter-pass twiddles of this thread's pass-1 items, identical for every coil
  float2 twr[NI1][B];
#pragma unroll
  for (int ii = 0; ii < NI1; ++ii) {
    const int i = t + ii * kColNT;
    const int s = (i < N1) ? i / kWB : 0;
#pragma unroll
    for (int k1p = 0; k1p < B; ++k1p) twr[ii][k1p] = __ldg(a.twH + H + k1p * A + s);
  }

  for (int c = cbeg; c < cend; ++c) {
    const int buf = (c - cbeg) & 1;
    cp_async_wait<0>();
    __syncthreads();  // coil c staged; previous coil's pass 2 finished
    if (c + 1 < cend) {
      issue_S(c + 1, buf ^ 1);
      issue_T(c + 1, buf ^ 1);
    }
    cp_async_commit();
    const float2* Tc = Tb + buf * RCAP * kWB;
    const float2* Sc = Sb + buf * H * kWB;
#pragma unroll
    for (int ii = 0; ii < NI1; ++ii) {
      const int i = t + ii * kColNT;
      if (i < N1) {
        const int w = i % kWB, s = i / kWB;
        int jv[B];
#pragma unroll
        for (int n1 = 0; n1 < B; ++n1) jv[n1] = rmap[A * n1 + s];
        float2 v[B];
#pragma unroll
        for (int n1 = 0; n1 < B; ++n1) {
          float2 e = make_float2(0.f, 0.f);
          if (jv[n1] >= 0)
            e = staged ? Tc[jv[n1] * kWB + w] : a.T[(size_t(rowbase + jv[n1]) * C + c) * W + w0 + w];
          v[n1] = conjf2(e);
        }
        dft<B>(v);
#pragma unroll
        for (int k1p = 0; k1p < B; ++k1p)
          ex[k1p * KS + s * kWB + w] = (k1p == 0) ? v[k1p] : cmul(v[k1p], twr[ii][k1p]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int ii = 0; ii < NI2; ++ii) {
      const int i = t + ii * kColNT;
      if (i < N2) {
        const int w = i % kWB, k1p = i / kWB;
        float2 v[A];
#pragma unroll
        for (int s = 0; s < A; ++s) v[s] = ex[k1p * KS + s * kWB + w];
        dft<A>(v);
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2) {
          // conj(v) * conj(S) == conj(v * S)
          const float2 p = cmul(v[k2], Sc[(k1p + B * k2) * kWB + w]);
          acc[ii][k2].x += p.x;
          acc[ii][k2].y -= p.y;
        }
      }
    }
  }

  // Sum the two halves' accumulators: each CTA publishes its partial sums in
  // its own (now idle) S buffers and reads its partner's for the rows it
  // finishes (k2 < A/2 for the first CTA, the rest for the second).
  cp_async_wait<0>();
  __syncthreads();
  float2* mine = Sb;
#pragma unroll
  for (int ii = 0; ii < NI2; ++ii)
#pragma unroll
    for (int k2 = 0; k2 < A; ++k2) mine[(ii * A + k2) * kColNT + t] = acc[ii][k2];
  cluster.sync();
  const float2* other = cluster.map_shared_rank(mine, half ^ 1);
  constexpr int KH = A / 2;
  const int kb = half ? KH : 0, ke = half ? A : KH;
#pragma unroll
  for (int ii = 0; ii < NI2; ++ii)
#pragma unroll
    for (int k2 = 0; k2 < A; ++k2)
      if (k2 >= kb && k2 < ke) {
        // fixed summation order (first half of the coils, then the second)
        const float2 o = other[(ii * A + k2) * kColNT + t];
        acc[ii][k2] = half ? cadd(o, acc[ii][k2]) : cadd(acc[ii][k2], o);
      }
  cluster.sync();  // partner finished reading this CTA's buffers

  const float s_adj = a.s_adj;
  if constexpr (!UPDATE) {
#pragma unroll
    for (int ii = 0; ii < NI2; ++ii) {
      const int i = t + ii * kColNT;
      if (i < N2) {
        const int w = i % kWB, k1p = i / kWB;
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2)
          if (k2 >= kb && k2 < ke)
            a.xref[size_t(f) * N + size_t(k1p + B * k2) * W + w0 + w] = cscale(acc[ii][k2], s_adj);
      }
    }
  } else {
    // the epilogue is instantiated twice (MC: the tTV gradient comes from
    // M^T of the motion-compensated form), so the uniform branch stays out of
    // the per-element loop
    const float2* __restrict__ xk = (it & 1) ? a.xk1 : a.xk0;
    float2* __restrict__ xn = (it & 1) ? a.xk0 : a.xk1;
    const size_t offm = size_t((f + F - 1) % F) * N, off0 = size_t(f) * N, offp = size_t((f + 1) % F) * N;
    const float inv_mu = 1.0f / st->mu, lambda = st->lambda, nLmu1 = -st->Lmu1, apk = st->apk, tauk = st->tauk;
    const float omt = 1.0f - tauk;
    float cmx = 0.f;  // max |x_{k+1}|^2 of this thread's column (mixed form)
    constexpr int BATCH = 4;  // outputs whose global loads are issued together
    auto epilogue = [&](auto mc_tag) {
      constexpr bool MC = decltype(mc_tag)::value;
#pragma unroll
    for (int ii = 0; ii < NI2; ++ii) {
      const int i = t + ii * kColNT;
      if (i < N2) {
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
              if constexpr (MC) {
                xm[b] = a.grad_ext[off0 + p];  // M^T (tTVadj u) of the motion-compensated form
              } else {
                xm[b] = xk[offm + p];
                xp[b] = xk[offp + p];
              }
              wo[b] = a.wacc[off0 + p];
              xr[b] = a.xref[off0 + p];
            }
          }
#pragma unroll
          for (int b = 0; b < BATCH; ++b) {
            const int k2 = k0 + b;
            if (k2 < A && k2 >= kb && k2 < ke) {
              const size_t p = size_t(k1p + B * k2) * W + w0 + w;
              // operator_tTVadj gives u_{f+1} - u_f of the normalised temporal
              // differences; NestaUp negates it, scales by lambda, adds A^H r
              float2 adj;
              if constexpr (MC) {
                adj = xm[b];
              } else {
                const float2 u0 = tv_normalize(csub(xa[b], xm[b]), inv_mu);
                const float2 u1 = tv_normalize(csub(xp[b], xa[b]), inv_mu);
                adj = csub(u1, u0);
              }
              const float2 ares = cscale(acc[ii][k2], s_adj);
              const float2 df = make_float2(__fadd_rn(__fmul_rn(-adj.x, lambda), ares.x),
                                            __fadd_rn(__fmul_rn(-adj.y, lambda), ares.y));
              const float2 yk = make_float2(fmaf(nLmu1, df.x, xa[b].x), fmaf(nLmu1, df.y, xa[b].y));
              const float2 wn = make_float2(fmaf(apk, df.x, wo[b].x), fmaf(apk, df.y, wo[b].y));
              const float2 zk = make_float2(fmaf(nLmu1, wn.x, xr[b].x), fmaf(nLmu1, wn.y, xr[b].y));
              const float2 xnew = make_float2(fmaf(omt, yk.x, tauk * zk.x), fmaf(omt, yk.y, tauk * zk.y));
              a.wacc[off0 + p] = wn;
              xn[off0 + p] = xnew;
              cmx = fmaxf(cmx, fmaf(xnew.x, xnew.x, xnew.y * xnew.y));
            }
          }
        }
      }
    }
    };
    if (a.grad_ext)
      epilogue(std::true_type{});
    else
      epilogue(std::false_type{});
    if (a.colmax) {
      // column maxima for the next tensor-core forward pass: lanes l, l^8,
      // l^16, l^24 share a column (i % kWB)
      cmx = fmaxf(cmx, __shfl_xor_sync(0xffffffffu, cmx, 8));
      cmx = fmaxf(cmx, __shfl_xor_sync(0xffffffffu, cmx, 16));
      if ((t & 31) < kWB)
        atomicMax(reinterpret_cast<unsigned int*>(a.colmax) + size_t((it + 1) & 1) * F * W + size_t(f) * W + w0 + (t & 31),
                  __float_as_uint(sqrtf(cmx)));
    }
  }
}

// ===========================================================================
// Dense FFT passes (the FFT process on full KData/XData buffers):
// rows along W, then columns along H.  Forward code only; the backward
// transform is conj(forward(conj(x))).  In place is allowed (out == in).
// ===========================================================================
template <int W>
__global__ void __launch_bounds__(kRowNT) k_fft_rows_dense(const float2* in, float2* out, int nrows, int inv,
                                                           float scale, const float2* twW) {
  using R = RowCfg<W>;
  constexpr int A = R::A, B = R::B, RPC = R::RPC;
  __shared__ float2 ex1[RPC * R::RS1];
  __shared__ float2 tw[W];
  const int t = threadIdx.x;
  for (int i = t; i < W; i += kRowNT) tw[i] = twW[i];
  __syncthreads();
  const float sg = inv ? -1.f : 1.f;
  for (int base = blockIdx.x * RPC; base < nrows; base += gridDim.x * RPC) {
    for (int i = t; i < RPC * B; i += kRowNT) {
      const int r = i / B, s = i % B, q = base + r;
      if (q >= nrows) continue;
      const float2* __restrict__ src = in + size_t(q) * W;
      float2 v[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) {
        const float2 e = src[B * n1 + s];
        v[n1] = make_float2(e.x, sg * e.y);
      }
      dft<A>(v);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) ex1[r * R::RS1 + k1 * R::S1 + s] = (k1 == 0) ? v[k1] : cmul(v[k1], tw[k1 * B + s]);
    }
    __syncthreads();
    for (int i = t; i < RPC * A; i += kRowNT) {
      const int r = i / A, k1 = i % A, q = base + r;
      if (q >= nrows) continue;
      float2 v[B];
#pragma unroll
      for (int s = 0; s < B; ++s) v[s] = ex1[r * R::RS1 + k1 * R::S1 + s];
      dft<B>(v);
      float2* __restrict__ dst = out + size_t(q) * W;
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) dst[k1 + A * k2] = make_float2(v[k2].x * scale, sg * v[k2].y * scale);
    }
    __syncthreads();
  }
}

// grid = (W/kWB, nimg)
template <int H>
__global__ void __launch_bounds__(kColNT) k_fft_cols_dense(const float2* in, float2* out, int W, int inv, float scale,
                                                           const float2* twH) {
  constexpr int A = Split<H>::A, B = Split<H>::B;
  constexpr int KS = col_ks(B);
  constexpr int N1 = kWB * B, N2 = kWB * A;
  __shared__ float2 ex[A * KS];
  __shared__ float2 tw[H];
  const int t = threadIdx.x;
  const int w0 = blockIdx.x * kWB;
  const size_t off = size_t(blockIdx.y) * H * W;
  for (int i = t; i < H; i += kColNT) tw[i] = twH[i];
  __syncthreads();
  const float sg = inv ? -1.f : 1.f;
  for (int i = t; i < N1; i += kColNT) {
    const int w = i % kWB, s = i / kWB;
    float2 v[A];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) {
      const float2 e = in[off + size_t(B * n1 + s) * W + w0 + w];
      v[n1] = make_float2(e.x, sg * e.y);
    }
    dft<A>(v);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) ex[k1 * KS + s * kWB + w] = (k1 == 0) ? v[k1] : cmul(v[k1], tw[k1 * B + s]);
  }
  __syncthreads();
  for (int i = t; i < N2; i += kColNT) {
    const int w = i % kWB, k1 = i / kWB;
    float2 v[B];
#pragma unroll
    for (int s = 0; s < B; ++s) v[s] = ex[k1 * KS + s * kWB + w];
    dft<B>(v);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2)
      out[off + size_t(k1 + A * k2) * W + w0 + w] = make_float2(v[k2].x * scale, sg * v[k2].y * scale);
  }
}

}  // namespace gbn
