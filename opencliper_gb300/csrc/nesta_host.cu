// tTV-NESTA solver: launch sequence of NestaUp::launch
// (src/processes/nesta/NestaUp.cpp:442-910) on one CUDA stream with all scalar
// bookkeeping kept on the device, plus the non-templated kernels (kept-row
// analysis, initial maxima, power-method norm estimate, scalar setup).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>

#include "ctx.h"
#include "nesta_kernels.cuh"
#include "rowlocal.cuh"
#include "solver.h"

namespace gbn {

constexpr int kNeIters = 100;  // myNormest maxiter (NestaUp.cpp:294)
constexpr int kNeNT = 256;

// ---------------------------------------------------------------------------
// drand48 jump-ahead (host and device)
// ---------------------------------------------------------------------------
constexpr uint64_t kMask48 = (1ULL << 48) - 1;
constexpr uint64_t kRandA = 0x5DEECE66DULL, kRandC = 0xBULL;

__host__ __device__ inline Lcg48 lcg_compose(Lcg48 first, Lcg48 second) {
  // x -> second(first(x)) = sa*(fa*x + fc) + sc
  return Lcg48{(second.a * first.a) & kMask48, (second.a * first.c + second.c) & kMask48};
}
__host__ __device__ inline Lcg48 lcg_jump_k(uint64_t k) {
  Lcg48 r{1, 0}, b{kRandA, kRandC};
  while (k) {
    if (k & 1) r = lcg_compose(r, b);
    b = lcg_compose(b, b);
    k >>= 1;
  }
  return r;
}
Lcg48 lcg48_jump(uint64_t k) { return lcg_jump_k(k); }
uint64_t lcg48_apply(const Lcg48& j, uint64_t x) { return (j.a * x + j.c) & kMask48; }

// ---------------------------------------------------------------------------
// Kept k-space rows: a row (f, h) is carried by the solver when its mask row
// has any sampled pixel or any coil holds a nonzero datum there.  Rows that are
// neither contribute exactly zero to E^H(Ex - y) and to ||Ex - y||^2.
// flags: 0 not kept, 1 kept with sampled pixels, 2 kept for its data only;
// full: every pixel of the mask row sampled.  grid = (H, F)
// ---------------------------------------------------------------------------
__global__ void k_rowflags(const float2* __restrict__ y, const uint8_t* __restrict__ mask, int W, int H, int F, int C,
                           int* __restrict__ flags, int* __restrict__ full) {
  const int h = blockIdx.x, f = blockIdx.y, t = threadIdx.x;
  const uint8_t* m = mask + (size_t(f) * H + h) * W;
  int any = 0, all = 1;
  for (int w = t; w < W; w += blockDim.x) {
    const int nz = m[w] != 0;
    any |= nz;
    all &= nz;
  }
  any = __syncthreads_or(any);
  all = __syncthreads_and(all);
  const int sampled = any;
  if (!any) {
    for (int c = 0; c < C && !any; ++c) {
      const float4* yr = reinterpret_cast<const float4*>(y + ((size_t(f) * C + c) * H + h) * W);
      int nz = 0;
      for (int i = t; i < W / 2; i += blockDim.x) {
        const float4 v = yr[i];
        nz |= (v.x != 0.f) | (v.y != 0.f) | (v.z != 0.f) | (v.w != 0.f);
      }
      any = __syncthreads_or(nz);
    }
  }
  if (t == 0) {
    flags[f * H + h] = sampled ? 1 : (any ? 2 : 0);
    full[f * H + h] = all;
  }
}

constexpr int kStatusRowsOverflow = 6;  // NestaDevState::status: kept rows beyond the row buffer were dropped

// one CTA of 512 threads (H <= 512): per-frame prefix numbering of kept rows;
// rows beyond the row buffer's capacity `cap` are dropped (rowmap -1) and
// reported in *status; *partial counts what keeps a problem off the
// row-local iteration: kept rows whose mask row is sampled in part, and
// frames with more kept rows than that iteration stages (iter_cols_rcap)
__global__ void __launch_bounds__(512) k_rowscan(const int* __restrict__ flags, const int* __restrict__ full, int H,
                                                 int F, int* __restrict__ rowmap, int* __restrict__ rowoff,
                                                 int* __restrict__ rows_h, int* __restrict__ rows_f,
                                                 int* __restrict__ row_full, int cap, int* __restrict__ status,
                                                 int* __restrict__ partial) {
  __shared__ int wsum[16];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  int base = 0, npart = 0, nwide = 0;
  bool dropped = false;
  for (int f = 0; f < F; ++f) {
    const int fl = (t < H) ? flags[f * H + t] : 0;
    npart += __syncthreads_count(t < H && fl == 1 && !full[f * H + t]);
    const unsigned bal = __ballot_sync(0xffffffffu, fl);
    const int pre = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    int woff = 0, tot = 0;
    for (int i = 0; i < 16; ++i) {
      if (i < wid) woff += wsum[i];
      tot += wsum[i];
    }
    const int room = max(0, cap - base);
    if (t < H) {
      const int j = (fl && woff + pre < room) ? woff + pre : -1;
      rowmap[f * H + t] = j;
      if (j >= 0) {
        rows_h[base + j] = t;
        rows_f[base + j] = f;
        row_full[base + j] = full[f * H + t];
      }
    }
    if (t == 0) rowoff[f] = base;
    dropped |= tot > room;
    nwide += tot > iter_cols_rcap(H);
    base += min(tot, room);
    __syncthreads();
  }
  if (t == 0) {
    rowoff[F] = base;
    *partial = npart + nwide;
    if (dropped) atomicExch(status, kStatusRowsOverflow);
  }
}

// every row kept, in natural order (SimpleMRIRecon: fully sampled data)
__global__ void k_rows_identity(int H, int F, int* __restrict__ rowmap, int* __restrict__ rowoff,
                                int* __restrict__ rows_h, int* __restrict__ rows_f, int* __restrict__ row_full) {
  const int n = H * F;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    rowmap[i] = i % H;
    rows_h[i] = i % H;
    rows_f[i] = i / H;
    row_full[i] = 1;
  }
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f <= F; f += gridDim.x * blockDim.x) rowoff[f] = f * H;
}

// ---------------------------------------------------------------------------
// Instance tables of a launch group.  k_store_args writes one entry from its
// by-value parameter (no host buffer has to outlive the call); k_group_init
// numbers the row-pass steps of every instance from its kept-row count and
// clears the group's counters.
// ---------------------------------------------------------------------------
__global__ void k_store_args(FusedArgs* __restrict__ dst, FusedArgs v) { *dst = v; }
__global__ void k_set_u64(unsigned long long* dst, unsigned long long v) { *dst = v; }

__global__ void k_group_init(const FusedArgs* __restrict__ tab, int n, int rpc, ClassCtl* __restrict__ ctl) {
  if (threadIdx.x == 0) {
    int base = 0;
    for (int i = 0; i < n; ++i) {
      const FusedArgs& a = tab[i];
      const int items = a.rowoff[a.F] * a.C;
      ctl->step_base[i] = base;
      ctl->nitems[i] = items;
      base += (items + rpc - 1) / rpc;
    }
    ctl->step_base[n] = base;
    ctl->row_next = 0;
    ctl->ticket = 0;
  }
  for (int i = threadIdx.x; i < kMaxBatch; i += blockDim.x) ctl->done[i] = 0;
}

// ---------------------------------------------------------------------------
// State initialisation from the launch parameters (one thread).
// ---------------------------------------------------------------------------
__global__ void k_state_init(NestaDevState* st, gbn_nesta_params p) {
  NestaDevState s;
  memset(&s, 0, sizeof(s));
  s.lambda_i = p.lambda_i;
  s.mu_f = p.mu_f;
  s.La = p.La;
  s.tolVar_in = p.tolVar;
  s.maxIntIter = int(p.maxIntIter);
  s.maxIter = int(p.maxIter);
  s.stoptest = int(p.stoptest);
  s.miniter = int(p.miniter);
  s.last_iter = -1;
  *st = s;
}

// ---------------------------------------------------------------------------
// max|x0| and max|U x0| (NestaUp.cpp:521-568: ComplexAbs + host loop).  Values
// are non-negative, so float order equals unsigned order of their bits.
// ---------------------------------------------------------------------------
// xu: the image the sparsity operator is applied to (x itself, or M x with
// motion compensation)
__global__ void __launch_bounds__(256) k_maxima(const float2* __restrict__ x, const float2* __restrict__ xu, int N,
                                                int F, NestaDevState* st) {
  __shared__ float s1[8], s2[8];
  const size_t total = size_t(N) * F;
  float m1 = 0.f, m2 = 0.f;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int f = int(i / N);
    const size_t p = i - size_t(f) * N;
    const float2 a = x[i];
    const float2 d = csub(xu[i], xu[size_t((f + F - 1) % F) * N + p]);
    m1 = fmaxf(m1, sqrtf(a.x * a.x + a.y * a.y));
    m2 = fmaxf(m2, sqrtf(d.x * d.x + d.y * d.y));
  }
  m1 = warp_max(m1);
  m2 = warp_max(m2);
  if ((threadIdx.x & 31) == 0) {
    s1[threadIdx.x >> 5] = m1;
    s2[threadIdx.x >> 5] = m2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < 8; ++i) {
      m1 = fmaxf(m1, s1[i]);
      m2 = fmaxf(m2, s2[i]);
    }
    atomicMax(&st->maxX_bits, __float_as_uint(m1));
    atomicMax(&st->maxUX_bits, __float_as_uint(m2));
  }
}

// ---------------------------------------------------------------------------
// Power method for ||U|| (myNormest, NestaUp.cpp:291-439).
//
// The start vector is all ones, so U x = 0 exactly and the reference always
// restarts from r = (drand48(), 0) drawn in [frame][row][col] order
// (NestaUp.cpp:369-385).  From there e_1 = ||r|| and, for m >= 1,
// e_{m+1} = ||D b_m|| / ||b_m|| with b_1 = D^T r and b_{m+1} = D^T D b_m
// (the reference's per-iteration normalisations and the sign of its adjoint
// kernel cancel in these ratios).  D acts along frames only, so every pixel's
// frame vector evolves independently: one thread per pixel advances it in
// registers (scaled by 1/4 per step, exact in binary floating point, to stay
// in range) and per-step sums of ||b_m||^2 and ||D b_m||^2 are reduced per
// block.  Steps run in chunks; after each chunk k_normest_check replays the
// reference's stopping rule on the sums available so far and, once it has
// stopped, later chunks return immediately.
// part layout: [block][step - m_begin (+1 for the first chunk)][2]; in the
// first chunk slot 0 holds ||r||^2.
// ---------------------------------------------------------------------------
constexpr int kNeChunks = 3;
constexpr int kNeBounds[kNeChunks + 1] = {1, 17, 49, kNeIters};
constexpr int kNeMaxSlots = 52;  // largest chunk (51 steps) + ||r||^2 slot

template <int FMAX>
__global__ void __launch_bounds__(kNeNT) k_normest_chunk(int N, int F, RandStart rs,
                                                         unsigned long long jumpN_a, unsigned long long jumpN_c,
                                                         int m_begin, int m_end, float* __restrict__ bstore,
                                                         double* __restrict__ part, const NestaDevState* st) {
  __shared__ float sw[kNeNT / 32][kNeMaxSlots][2];
  if (st->ne_done) return;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int p = blockIdx.x * kNeNT + t;
  const bool act = p < N;
  const int slot0 = (m_begin == 1) ? 1 : 0;
  float b[FMAX], d[FMAX];
  if (m_begin == 1) {
    const unsigned long long x0 = rs.p ? ((rs.ja * *rs.p + rs.jc) & kMask48) : rs.x0;
    // element (f, p) is draw number f*N + p + 1 after the state x0
    const Lcg48 jp = lcg_jump_k(uint64_t(act ? p : 0) + 1);
    uint64_t X = (jp.a * x0 + jp.c) & kMask48;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
      if (f < F && act) {
        d[f] = __double2float_rn(double(X) * 0x1p-48);
        X = (jumpN_a * X + jumpN_c) & kMask48;
      } else {
        d[f] = 0.f;
      }
    }
    float s0 = 0.f;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) s0 = fmaf(d[f], d[f], s0);
    // b_1 = D^T r: (D^T v)_f = v_f - v_{f+1 mod F}
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
      const float nx = (f + 1 < FMAX && f + 1 < F) ? d[(f + 1) % FMAX] : d[0];
      b[f] = (f < F) ? d[f] - nx : 0.f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s0 += __shfl_down_sync(0xffffffffu, s0, o);
    if (lane == 0) {
      sw[wid][0][0] = s0;
      sw[wid][0][1] = 0.f;
    }
  } else {
#pragma unroll
    for (int f = 0; f < FMAX; ++f) b[f] = (f < F && act) ? bstore[size_t(f) * N + p] : 0.f;
  }
  for (int m = m_begin; m < m_end; ++m) {
    float last = b[0];
#pragma unroll
    for (int f = 1; f < FMAX; ++f)
      if (f == F - 1) last = b[f];
    float sb = 0.f, sd = 0.f;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
      const float pv = (f == 0) ? last : b[(f + FMAX - 1) % FMAX];
      d[f] = (f < F) ? b[f] - pv : 0.f;
      sb = fmaf(b[f], b[f], sb);
      sd = fmaf(d[f], d[f], sd);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sb += __shfl_down_sync(0xffffffffu, sb, o);
      sd += __shfl_down_sync(0xffffffffu, sd, o);
    }
    if (lane == 0) {
      sw[wid][slot0 + m - m_begin][0] = sb;
      sw[wid][slot0 + m - m_begin][1] = sd;
    }
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
      const float nx = (f + 1 < FMAX && f + 1 < F) ? d[(f + 1) % FMAX] : d[0];
      b[f] = (f < F) ? (d[f] - nx) * 0.25f : 0.f;
    }
  }
  if (m_end < kNeIters && act) {
#pragma unroll
    for (int f = 0; f < FMAX; ++f)
      if (f < F) bstore[size_t(f) * N + p] = b[f];
  }
  __syncthreads();
  const int nslots = slot0 + m_end - m_begin;
  for (int i = t; i < nslots * 2; i += kNeNT) {
    double s = 0.0;
    for (int w = 0; w < kNeNT / 32; ++w) s += double(sw[w][i >> 1][i & 1]);
    part[size_t(blockIdx.x) * kNeMaxSlots * 2 + i] = s;
  }
}

// one CTA: reduce the chunk's per-block sums (one warp per sum) and continue
// the reference's convergence loop (NestaUp.cpp:325-431)
__global__ void __launch_bounds__(256) k_normest_check(const double* __restrict__ part, int nblk, int m_begin,
                                                       int m_end, int N, int F, NestaDevState* st) {
  __shared__ double tot[kNeMaxSlots * 2];
  if (st->ne_done) return;
  const int slot0 = (m_begin == 1) ? 1 : 0;
  const int nsum = (slot0 + m_end - m_begin) * 2;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = wid; i < nsum; i += blockDim.x / 32) {
    double s = 0.0;
    for (int b = lane; b < nblk; b += 32) s += part[size_t(b) * kNeMaxSlots * 2 + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) tot[i] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const float tol = 1e-3f;
    float e, e0;
    int cnt;
    if (m_begin == 1) {
      e = sqrtf(float(unsigned(N) * unsigned(F)));  // ||ones||
      e0 = 0.f;
      cnt = 0;
    } else {
      e = st->ne_e;
      e0 = st->ne_e0;
      cnt = st->ne_cnt;
    }
    bool stopped = false;
    for (;;) {
      if (!(fabsf(e - e0) > tol * e && cnt < kNeIters)) {
        stopped = true;
        break;
      }
      if (cnt > 0 && cnt >= m_end) break;  // needs steps of a later chunk
      const float en = (cnt == 0) ? float(sqrt(tot[0]))
                                  : float(sqrt(tot[2 * (slot0 + cnt - m_begin) + 1] / tot[2 * (slot0 + cnt - m_begin)]));
      e0 = e;
      e = en;
      ++cnt;
    }
    st->ne_e = e;
    st->ne_e0 = e0;
    st->ne_cnt = cnt;
    if (stopped) {
      st->normU = e;
      st->normest_iters = cnt;
      st->ne_done = 1;
    }
  }
}

// ---------------------------------------------------------------------------
// Derived constants (NestaUp.cpp:570-583), one thread.
// ---------------------------------------------------------------------------
__global__ void k_setup(NestaDevState* st) {
  NestaDevState& s = *st;
  s.maxX = __uint_as_float(s.maxX_bits);
  s.maxUX = __uint_as_float(s.maxUX_bits);
  s.lambda = s.lambda_i * s.maxX;
  s.muf = s.mu_f * s.maxX;
  s.mu0 = float(0.9 * double(s.maxUX));
  const float muL = s.lambda / s.La;
  if (muL > s.mu0) s.mu0 = muL;
  s.gamma = float(pow(double(s.muf / s.mu0), 1.0 / double(unsigned(s.maxIntIter))));
  s.mu = s.mu0;
  s.gammat = float(pow(double(s.tolVar_in) / 0.1, 1.0 / double(unsigned(s.maxIntIter))));
  s.tolVar = 0.1f;
}

// Start of an outer (continuation) loop (NestaUp.cpp:604-648):
// mu and tolVar updates, Lmu, w = 0, x_k = x_ref.
__global__ void k_outer_begin(NestaDevState* st, int nl, float* fmean, const float2* __restrict__ xref,
                              float2* __restrict__ xk0, float2* __restrict__ wacc, size_t n) {
  if (nl > st->maxIntIter) {
    // this instance has run all its outer loops (a batch runs the largest count)
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->outer_active = 0;
      st->last_iter = -1;
    }
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    NestaDevState& s = *st;
    s.outer_active = 1;
    s.nl = nl;
    s.mu = s.mu * s.gamma;
    s.tolVar = s.tolVar * s.gammat;
    s.Ak = 0.0f;
    float Lmu = s.normU / s.mu;
    if (s.miniter > 0) fmean[s.miniter - 1] = float(LONG_MAX);
    Lmu = s.lambda * Lmu + s.La;
    s.Lmu = Lmu;
    s.Lmu1 = 1.0f / Lmu;
    s.qpDone = 0;
    s.fixup = 0;
    s.last_iter = s.maxIter - 1;
  }
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    xk0[i] = xref[i];
    wacc[i] = make_float2(0.f, 0.f);
  }
}

// End of an outer loop: x_ref = x_k (NestaUp.cpp:889).
__global__ void k_outer_end(const NestaDevState* st, const float2* __restrict__ xk0, const float2* __restrict__ xk1,
                            float2* __restrict__ xref, size_t n) {
  if (!st->outer_active) return;
  const float2* src = ((st->last_iter + 1) & 1) ? xk1 : xk0;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    xref[i] = src[i];
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {

template <typename T>
int grow(T*& p, int& cap, int need) {
  if (need <= cap) return GBN_OK;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  if (cudaMalloc(&p, sizeof(T) * size_t(need)) != cudaSuccess) {
    cudaGetLastError();
    return set_error(GBN_ERR_NOMEM, "workspace allocation failed");
  }
  cap = need;
  return GBN_OK;
}

int normest_fmax(int F) {
  for (int m : {8, 16, 24, 32, 40, 48, 64})
    if (F <= m) return m;
  return 0;
}

void launch_normest_chunk(int fmax, int nblk, cudaStream_t s, int N, int F, const RandStart& x0, const Lcg48& jN, int mb,
                          int me, float* bstore, double* part, const NestaDevState* st) {
#define GBN_NE_CASE(M)                                                                                  \
  case M:                                                                                               \
    k_normest_chunk<M><<<nblk, kNeNT, 0, s>>>(N, F, x0, jN.a, jN.c, mb, me, bstore, part, st); \
    break;
  switch (fmax) {
    GBN_NE_CASE(8)
    GBN_NE_CASE(16)
    GBN_NE_CASE(24)
    GBN_NE_CASE(32)
    GBN_NE_CASE(40)
    GBN_NE_CASE(48)
    default:
      k_normest_chunk<64><<<nblk, kNeNT, 0, s>>>(N, F, x0, jN.a, jN.c, mb, me, bstore, part, st);
  }
#undef GBN_NE_CASE
}

}  // namespace

int problem_alloc(gbn_problem* P) {
  const size_t FH = size_t(P->F) * P->H;
  const size_t X = size_t(P->F) * P->H * P->W;
  const size_t K = X * P->C;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  A((void**)&P->flags, FH * sizeof(int));
  A((void**)&P->full_fh, FH * sizeof(int));
  A((void**)&P->rowmap, FH * sizeof(int));
  A((void**)&P->rowoff, (P->F + 1) * sizeof(int));
  A((void**)&P->rows_h, FH * sizeof(int));
  A((void**)&P->rows_f, FH * sizeof(int));
  A((void**)&P->row_full, FH * sizeof(int));
  A((void**)&P->T, K * sizeof(float2));
  P->T_rows = FH;
  A((void**)&P->xk0, X * sizeof(float2));
  A((void**)&P->xk1, X * sizeof(float2));
  A((void**)&P->wacc, X * sizeof(float2));
  A((void**)&P->wacc1, X * sizeof(float2));
  A((void**)&P->st, sizeof(NestaDevState));
  A((void**)&P->d_args, sizeof(FusedArgs));
  A((void**)&P->ctl, sizeof(ClassCtl));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(GBN_ERR_NOMEM, std::string("problem workspace allocation failed: ") + cudaGetErrorString(e));
  }
  return GBN_OK;
}

void launch_row_analysis(gbn_problem* P, cudaStream_t s);

// Shrinks (or grows) the row buffer T to the rows the current y and mask keep
// plus `headroom` (at most every row); returns the kept rows in *kept.
int problem_fit_rows(gbn_problem* P, int headroom, int* kept) {
  if (headroom < 0) return set_error(GBN_ERR_INVALID, "headroom must be >= 0");
  if (P->in_batches > 0)
    return set_error(GBN_ERR_INVALID, "fit rows: the problem belongs to a live batch (destroy it first)");
  cudaStream_t s = P->ctx->stream;
  cudaError_t e = cudaMemsetAsync(&P->st->status, 0, sizeof(int), s);
  const size_t saved = P->T_rows;
  P->T_rows = size_t(P->F) * P->H;  // count every kept row
  if (e == cudaSuccess) {
    launch_row_analysis(P, s);
    int g = 0;
    if ((e = cudaMemcpyAsync(&g, P->rowoff + P->F, sizeof(int), cudaMemcpyDeviceToHost, s)) == cudaSuccess &&
        (e = cudaStreamSynchronize(s)) == cudaSuccess) {
      const size_t want = std::min<size_t>(size_t(P->F) * P->H, size_t(g) + size_t(headroom));
      if (want != saved) {
        float2* nt = nullptr;
        if ((e = cudaMalloc(&nt, std::max<size_t>(want, 1) * P->C * P->W * sizeof(float2))) == cudaSuccess) {
          cudaFree(P->T);
          P->T = nt;
          P->T_rows = want;
          if (kept) *kept = g;
          return GBN_OK;
        }
      } else {
        P->T_rows = saved;
        if (kept) *kept = g;
        return GBN_OK;
      }
    }
  }
  P->T_rows = saved;
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? set_error(GBN_ERR_NOMEM, "row buffer allocation failed")
                                        : cuda_status(e, "fit rows");
}

void motion_free(gbn_problem* P);

void problem_free(gbn_problem* P) {
  void* ptrs[] = {P->flags, P->full_fh, P->rowmap, P->rowoff,  P->rows_h, P->rows_f,  P->row_full, P->T,
                  P->xk0,   P->xk1,     P->wacc,   P->wacc1,  P->st,      P->fmean,  P->part_tv, P->part_r,   P->part_ne,
                  P->ne_b,  P->d_args,  P->ctl,      P->fk,     P->colmax, P->smax,   P->fa};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  motion_free(P);
}

// Kept-row analysis for the current contents of y and mask (device only).
void launch_row_analysis(gbn_problem* P, cudaStream_t s) {
  k_rowflags<<<dim3(P->H, P->F), 128, 0, s>>>(P->y, P->mask, P->W, P->H, P->F, P->C, P->flags, P->full_fh);
  k_rowscan<<<1, 512, 0, s>>>(P->flags, P->full_fh, P->H, P->F, P->rowmap, P->rowoff, P->rows_h, P->rows_f,
                              P->row_full, int(P->T_rows), &P->st->status, &P->st->partial_rows);
}

FusedArgs make_args(gbn_problem* P, float2* xref) {
  gbn_ctx* ctx = P->ctx;
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.W = P->W;
  a.H = P->H;
  a.F = P->F;
  a.C = P->C;
  a.N = P->W * P->H;
  a.y = P->y;
  a.S = P->S;
  a.mask = P->mask;
  a.rowmap = P->rowmap;
  a.rowoff = P->rowoff;
  a.rows_h = P->rows_h;
  a.rows_f = P->rows_f;
  a.row_full = P->row_full;
  a.T = P->T;
  a.xk0 = P->xk0;
  a.xk1 = P->xk1;
  a.xref = xref;
  a.wacc = P->wacc;
  a.wacc1 = P->wacc1;
  a.st = P->st;
  a.fmean = P->fmean;
  a.part_tv = P->part_tv;
  a.part_r = P->part_r;
  a.twH = ctx_twiddles(ctx, P->H);
  a.twW = ctx_twiddles(ctx, P->W);
  const unsigned N = unsigned(P->W) * unsigned(P->H);
  a.s_fwd = float(1.0 / std::sqrt(double(N)));               // NestaUp.cpp:712: 1/(sqrt(cols*rows*slices))
  a.s_adj = std::sqrt(float(N)) * (1.0f / float(N));        // NestaUp.cpp:749 sqrt(float(N)) times clFFT 1/N
  a.s_row = float(double(P->W) * double(a.s_fwd));
  a.ntv = P->F * (P->W / kWB);
  return a;
}

BatchMap single_map(int F, ClassCtl* ctl) {
  BatchMap bm;
  memset(&bm, 0, sizeof(bm));
  bm.n = 1;
  bm.fbase[0] = 0;
  bm.fbase[1] = F;
  bm.ctl = ctl;
  return bm;
}

int validate_problem_dims(int W, int H, int F, int C) {
  if (W <= 0 || H <= 0 || F <= 0 || C <= 0) return set_error(GBN_ERR_INVALID, "dimensions must be positive");
  if (W % 8 != 0) return set_error(GBN_ERR_INVALID, "NDArray dimension 0 (width) is not multiple of 8");
  if (!find_size(W) || !find_size(H))
    return set_error(GBN_ERR_UNSUPPORTED,
                     "FFT lengths must be 7-smooth multiples of 8 in [8, 512] (got W=" + std::to_string(W) +
                         ", H=" + std::to_string(H) + ")");
  return GBN_OK;
}

int run_prepare(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params* prm) {
  if (!ctx || !P || !prm) return set_error(GBN_ERR_INVALID, "null argument");
  if (P->F < 2) return set_error(GBN_ERR_INVALID, "temporal TV needs at least 2 frames (F=1 makes ||U|| undefined)");
  if (prm->stoptest == 1 && prm->miniter == 0) return set_error(GBN_ERR_INVALID, "miniter must be >= 1 when stoptest == 1");
  if (!normest_fmax(P->F)) return set_error(GBN_ERR_UNSUPPORTED, "more than 64 frames is not supported");
  const SizeKernels* kh = find_size(P->H);
  const SizeKernels* kw = find_size(P->W);
  if (!kh || !kw) return set_error(GBN_ERR_UNSUPPORTED, "unsupported FFT length");
  const int W = P->W, H = P->H, F = P->F, C = P->C, N = W * H;
  const long long steps_max = ((long long)F * H * C + kw->rows_per_cta - 1) / kw->rows_per_cta;
  const int nblk_ne = (N + kNeNT - 1) / kNeNT;
  int rc;
  if ((rc = grow(P->fmean, P->fmean_cap, std::max<int>(1, int(prm->miniter)))) != GBN_OK) return rc;
  // one (|u|^2, Re<u,d>) pair per (frame, 8-column tile) and coil half (row-local iteration)
  if ((rc = grow(P->part_tv, P->part_tv_cap, 4 * F * (W / kWB))) != GBN_OK) return rc;
  if ((rc = grow(P->part_r, P->part_r_cap, std::max(int(steps_max) * kRowWarps, 2 * F * (W / kWB)))) != GBN_OK)
    return rc;
  if ((rc = grow(P->part_ne, P->part_ne_cap, nblk_ne * kNeMaxSlots * 2)) != GBN_OK) return rc;
  if ((rc = grow(P->ne_b, P->ne_b_cap, N * F)) != GBN_OK) return rc;
  return GBN_OK;
}

int row_grid(gbn_ctx* ctx, const SizeKernels* kw, bool resid, long long steps, int k2_per_sm) {
  const int per_sm = std::max(1, std::min(k2_per_sm, kw->rows_occupancy(resid)));
  return int(std::max<long long>(1, std::min<long long>(steps, (long long)ctx->nsm * per_sm)));
}

int launch_store_args(FusedArgs* dst, const FusedArgs& a, cudaStream_t s) {
  k_store_args<<<1, 1, 0, s>>>(dst, a);
  return 1;
}

int launch_group_init(const FusedArgs* tab, int n, int rows_per_cta, ClassCtl* ctl, cudaStream_t s) {
  k_group_init<<<1, 64, 0, s>>>(tab, n, rows_per_cta, ctl);
  return 1;
}

int launch_set_rand(unsigned long long* dst, unsigned long long v, cudaStream_t s) {
  k_set_u64<<<1, 1, 0, s>>>(dst, v);
  return 1;
}

int launch_pre(gbn_problem* P, const gbn_nesta_params& prm, cudaStream_t s) {
  k_state_init<<<1, 1, 0, s>>>(P->st, prm);
  launch_row_analysis(P, s);
  return 3;
}

namespace {
int elementwise_grid(gbn_ctx* ctx, size_t n) { return int(std::min<size_t>((n + 255) / 256, size_t(ctx->nsm) * 8)); }
}  // namespace

int launch_constants(gbn_ctx* ctx, gbn_problem* P, const float2* xref, const RandStart& rs, cudaStream_t s) {
  const int N = P->W * P->H, F = P->F;
  const int nblk_ne = (N + kNeNT - 1) / kNeNT;
  // maxima, norm estimate, constants (NestaUp.cpp:521-583)
  k_maxima<<<elementwise_grid(ctx, size_t(N) * F), 256, 0, s>>>(xref, xref, N, F, P->st);
  const Lcg48 jN = lcg_jump_k(uint64_t(N));
  for (int ch = 0; ch < kNeChunks; ++ch) {
    launch_normest_chunk(normest_fmax(F), nblk_ne, s, N, F, rs, jN, kNeBounds[ch], kNeBounds[ch + 1], P->ne_b,
                         P->part_ne, P->st);
    k_normest_check<<<1, 256, 0, s>>>(P->part_ne, nblk_ne, kNeBounds[ch], kNeBounds[ch + 1], N, F, P->st);
  }
  k_setup<<<1, 1, 0, s>>>(P->st);
  return 2 + 2 * kNeChunks;
}

int launch_maxima(gbn_ctx* ctx, gbn_problem* P, const float2* x0, const float2* xu, cudaStream_t s) {
  const size_t X = size_t(P->W) * P->H * P->F;
  k_maxima<<<elementwise_grid(ctx, X), 256, 0, s>>>(x0, xu, P->W * P->H, P->F, P->st);
  return 1;
}

int launch_setup(gbn_problem* P, cudaStream_t s) {
  k_setup<<<1, 1, 0, s>>>(P->st);
  return 1;
}

int launch_outer_begin(gbn_ctx* ctx, gbn_problem* P, int nl, const float2* xref, cudaStream_t s) {
  const size_t X = size_t(P->W) * P->H * P->F;
  k_outer_begin<<<elementwise_grid(ctx, X), 256, 0, s>>>(P->st, nl, P->fmean, xref, P->xk0, P->wacc, X);
  return 1;
}

int launch_outer_end(gbn_ctx* ctx, gbn_problem* P, float2* xref, cudaStream_t s) {
  const size_t X = size_t(P->W) * P->H * P->F;
  k_outer_end<<<elementwise_grid(ctx, X), 256, 0, s>>>(P->st, P->xk0, P->xk1, xref, X);
  return 1;
}

int read_stats(gbn_problem* P, cudaStream_t s, gbn_nesta_stats* stats) {
  NestaDevState h;
  int G = 0;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(&h, P->st, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_status(e, "stats copy");
  if ((e = cudaMemcpyAsync(&G, P->rowoff + P->F, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_status(e, "stats copy");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e, "nesta run");
  stats->normU = h.normU;
  stats->maxX = h.maxX;
  stats->maxUX = h.maxUX;
  stats->lambda = h.lambda;
  stats->muf = h.muf;
  stats->mu0 = h.mu0;
  stats->mu_final = h.mu;
  stats->tolVar_final = h.tolVar;
  stats->fx_final = h.fx;
  stats->qp_final = h.qp;
  stats->inner_iters = h.iters_total;
  stats->normest_iters = h.normest_iters;
  stats->kept_rows = G;
  stats->status = h.status;
  return GBN_OK;
}

int nesta_run_mc(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params* prm, float2* x_out);

// pinned read-back slot and event of the per-run row-structure check (first use)
int partial_flag_ready(gbn_ctx* ctx) {
  if (ctx->host_partial) return GBN_OK;
  cudaError_t e = cudaHostAlloc(&ctx->host_partial, sizeof(int), cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_partial, cudaEventDisableTiming);
  return cuda_status(e, "pinned row-structure flag");
}

int nesta_run(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params* prm, float2* x_out, gbn_nesta_stats* stats) {
  if (!x_out) return set_error(GBN_ERR_INVALID, "null argument");
  int rc = run_prepare(ctx, P, prm);
  if (rc != GBN_OK) return rc;
  if (P->mc_on) {
    if ((rc = nesta_run_mc(ctx, P, prm, x_out)) != GBN_OK) return rc;
    return stats ? read_stats(P, ctx->stream, stats) : GBN_OK;
  }
  const SizeKernels* kh = find_size(P->H);
  const SizeKernels* kw = find_size(P->W);
  const int W = P->W, H = P->H, F = P->F, C = P->C;
  cudaStream_t s = ctx->stream;
  int cpb, k2;
  tuning_for(ctx, W, H, F, C, &cpb, &k2);
  cpb = std::max(1, std::min(cpb, C));
  const dim3 g1(W / kWB, (C + cpb - 1) / cpb, F);
  const long long steps = ((long long)F * H * C + kw->rows_per_cta - 1) / kw->rows_per_cta;
  const int g2 = row_grid(ctx, kw, true, steps, k2), g2a = row_grid(ctx, kw, false, steps, k2);
  const dim3 g3(W / kWB, 2, F);  // clusters of 2 along y
  const FusedArgs a = make_args(P, x_out);
  const FusedArgs* tab = P->d_args;
  const BatchMap bm = single_map(F, P->ctl);

  // the row-local iteration needs every kept row fully sampled or unsampled:
  // the row analysis's count of partly sampled rows comes back to pinned
  // host memory while the setup below is queued, and is read before the
  // iterations are
  const bool check_rows = ctx->row_local && kh->iter_cols;
  int rc2 = check_rows ? partial_flag_ready(ctx) : GBN_OK;
  if (rc2 != GBN_OK) return rc2;
  cudaError_t ef = cudaSuccess;
  int n_setup = 0;
  GBN_LAUNCH(ctx, GBN_PROF_SETUP, n_setup, {
    n_setup += launch_pre(P, *prm, s);
    if (check_rows) {
      ef = cudaMemcpyAsync(ctx->host_partial, &P->st->partial_rows, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (ef == cudaSuccess) ef = cudaEventRecord(ctx->ev_partial, s);
    }
    n_setup += launch_store_args(P->d_args, a, s);
    n_setup += launch_group_init(tab, 1, kw->rows_per_cta, P->ctl, s);
    // x0 = E^H y (NestaUp.cpp:465-486); T keeps IDFT_W(y) of the kept rows
    kw->rows(tab, bm, 0, false, g2a, s);
    kh->inv_cols(tab, bm, 0, false, g3, s);
    n_setup += 2;
    n_setup += launch_constants(ctx, P, x_out, RandStart{ctx->rand48, nullptr, 1, 0}, s);
    ctx->rand48 = lcg48_apply(lcg_jump_k(uint64_t(W) * uint64_t(H) * uint64_t(F)), ctx->rand48);
  });
  if (ef != cudaSuccess) return cuda_status(ef, "row structure read-back");
  bool row_local = false;
  if (ctx->row_local && kh->iter_cols) {
    if ((ef = cudaEventSynchronize(ctx->ev_partial)) != cudaSuccess) return cuda_status(ef, "row structure read-back");
    row_local = *ctx->host_partial == 0;
  }
  // stopping test on: one more launch per outer loop recomputes the last
  // update if the rule stops the loop (row-local iteration only)
  const unsigned n_iter_launch = prm->maxIter + ((row_local && prm->stoptest == 1) ? 1u : 0u);

  for (unsigned nl = 1; nl <= prm->maxIntIter; ++nl) {
    GBN_LAUNCH(ctx, GBN_PROF_OUTER, 1, launch_outer_begin(ctx, P, int(nl), x_out, s));
    if (row_local) {
      for (unsigned it = 0; it < n_iter_launch; ++it)
        GBN_LAUNCH(ctx, GBN_PROF_ITER, 1, kh->iter_cols(tab, bm, int(it), false, g3, s));
    } else {
      for (unsigned it = 0; it < prm->maxIter; ++it) {
        GBN_LAUNCH(ctx, GBN_PROF_FWD_COLS, 1, kh->fwd_cols(tab, bm, int(it), cpb, g1, s));
        GBN_LAUNCH(ctx, GBN_PROF_ROWS, 1, kw->rows(tab, bm, int(it), true, g2, s));
        GBN_LAUNCH(ctx, GBN_PROF_INV_COLS, 1, kh->inv_cols(tab, bm, int(it), true, g3, s));
      }
    }
    GBN_LAUNCH(ctx, GBN_PROF_OUTER, 1, launch_outer_end(ctx, P, x_out, s));
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "nesta launch");
  if (stats) return read_stats(P, s, stats);
  return GBN_OK;
}

// Adjoint-only pass (rows without residual, then columns without update) of
// one instance with every row kept: SimpleMRIRecon.  `ws` provides the
// intermediates and tables (simple_recon_bytes); no allocation happens here.
size_t simple_recon_bytes(int W, int H, int F, int C) {
  const size_t FH = size_t(F) * H, K = FH * C * W;
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  return up(K * sizeof(float2)) + up((4 * FH + F + 1) * sizeof(int)) + up(sizeof(NestaDevState)) +
         up(sizeof(FusedArgs)) + up(sizeof(ClassCtl));
}

int simple_recon_in(gbn_ctx* ctx, void* ws, const float2* y, const float2* S, float2* x, int W, int H, int F, int C,
                    bool tables_valid) {
  const SizeKernels* kh = find_size(H);
  const SizeKernels* kw = find_size(W);
  if (!kh || !kw) return set_error(GBN_ERR_UNSUPPORTED, "unsupported FFT length");
  const size_t FH = size_t(F) * H, K = FH * C * W;
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  unsigned char* b = static_cast<unsigned char*>(ws);
  float2* T = reinterpret_cast<float2*>(b);
  b += up(K * sizeof(float2));
  int* rowmap = reinterpret_cast<int*>(b);
  int* rows_h = rowmap + FH;
  int* rows_f = rows_h + FH;
  int* row_full = rows_f + FH;
  int* rowoff = row_full + FH;
  b += up((4 * FH + F + 1) * sizeof(int));
  NestaDevState* st = reinterpret_cast<NestaDevState*>(b);
  b += up(sizeof(NestaDevState));
  FusedArgs* tab = reinterpret_cast<FusedArgs*>(b);
  b += up(sizeof(FusedArgs));
  ClassCtl* ctl = reinterpret_cast<ClassCtl*>(b);
  cudaStream_t s = ctx->stream;
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.W = W;
  a.H = H;
  a.F = F;
  a.C = C;
  a.N = W * H;
  a.y = y;
  a.S = S;
  a.rowmap = rowmap;
  a.rowoff = rowoff;
  a.rows_h = rows_h;
  a.rows_f = rows_f;
  a.row_full = row_full;
  a.T = T;
  a.xref = x;
  a.st = st;
  a.twH = ctx_twiddles(ctx, H);
  a.twW = ctx_twiddles(ctx, W);
  a.s_adj = 1.0f / float(W * H);  // clFFT BACKWARD scale
  a.ntv = F * (W / kWB);
  const long long steps = ((long long)FH * C + kw->rows_per_cta - 1) / kw->rows_per_cta;
  const int g2 = row_grid(ctx, kw, false, steps, ctx->k2_ctas_per_sm);
  const BatchMap bm = single_map(F, ctl);
  // the tables persist in `ws`, and the row pass leaves its control block
  // ready for the next launch
  const int n_tables = tables_valid ? 0 : 3;
  GBN_LAUNCH(ctx, GBN_PROF_SETUP, n_tables + 2, {
    if (!tables_valid) {
      k_rows_identity<<<int(std::min<size_t>((FH + 255) / 256, 1024)), 256, 0, s>>>(H, F, rowmap, rowoff, rows_h,
                                                                                    rows_f, row_full);
      k_store_args<<<1, 1, 0, s>>>(tab, a);
      k_group_init<<<1, 64, 0, s>>>(tab, 1, kw->rows_per_cta, ctl);
    }
    kw->rows(tab, bm, 0, false, g2, s);
    kh->inv_cols(tab, bm, 0, false, dim3(W / kWB, 2, F), s);
  });
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "simple recon launch");
  return GBN_OK;
}

// SimpleMRIRecon: x = sum_c conj(S_c) ifft2(y_c) through the adjoint row and
// column passes with every row kept, working memory from the context scratch.
int simple_recon(gbn_ctx* ctx, const float2* y, const float2* S, float2* x, int W, int H, int F, int C) {
  if (!find_size(H) || !find_size(W)) return set_error(GBN_ERR_UNSUPPORTED, "unsupported FFT length");
  void* scr = nullptr;
  const bool mine = ctx->scratch_user == kScratchSimple;
  const int rc = ctx_scratch(ctx, simple_recon_bytes(W, H, F, C), &scr, kScratchSimple);
  if (rc != GBN_OK) {
    // a failed allocation freed the old scratch: a later one at the same
    // address holds no tables
    ctx->simple_key = gbn_ctx::SimpleKey{};
    return rc;
  }
  gbn_ctx::SimpleKey& k = ctx->simple_key;
  const bool same = mine && k.y == y && k.S == S && k.x == x && k.ws == scr && k.W == W && k.H == H && k.F == F &&
                    k.C == C;
  const int rc2 = simple_recon_in(ctx, scr, y, S, x, W, H, F, C, same);
  if (rc2 == GBN_OK) {
    k.y = y;
    k.S = S;
    k.x = x;
    k.ws = scr;
    k.W = W;
    k.H = H;
    k.F = F;
    k.C = C;
  } else {
    k = gbn_ctx::SimpleKey{};
  }
  return rc2;
}

}  // namespace gbn
