// Motion-compensated tTV-NESTA (NestaUp with argsMC != nullptr): the sparsity
// operator becomes U x = tTV(M x) and U^T u = M^T tTVadj(u) (NestaUp.cpp:
// 201-278), where M warps every frame by bilinear interpolation on a deformed
// mesh (MotionCompensation.cpp:57-78; optimizer.cl:832-877) and M^T scatters
// back with the same weights (AdjointMotionCompensation.cpp:59-86;
// optimizer.cl:880-937; initialize.cl:55-80).  The solve starts from the image
// already in the output buffer (the reference skips x0 = E^H y with argsMC,
// NestaUp.cpp:483-486).
//
// Both operators run as gathers over tables built from the meshes at the
// start of each run:
//  * inv[p]: the rectangle entry whose warped value lands on pixel p (the
//    last one in the reference's work-item order when several do), or -1:
//    (M x)[f][p] = inv[p] < 0 ? x[f][p] : bilinear x[f] at that entry;
//  * per target pixel and frame, the list of (entry, corner) pairs the
//    scatter would add there, in the reference's work-item order, with each
//    entry's source pixel and fractional position: (M^T g)[q] = (q in the
//    rectangle ? 0 : g[q]) + sum of (g[src] * fa) * fb, each product and sum
//    rounded as the kernel's.
// So M^T is deterministic and equals an in-order scatter bit for bit, where
// the reference's atomic scatter depends on the order of its atomics.
//
// Per inner iteration: k_mc_tv (M x_k for three frames on the fly, D, the
// Huber normalisation, g = D^T u and the objective's partial sums),
// k_mc_adjoint (M^T g), and the data term with the update.  For row masks the
// last is the one-kernel row-local iteration (rowlocal.cuh), launched after
// the two on one stream; its update waits for M^T g, its tTV gradient.
// Otherwise it is the fused forward column and row passes as in the plain form
// (the forward pass skips its tTV sums) and the adjoint column pass, which
// takes M^T g; k_mc_tv and k_mc_adjoint then run on a side stream beside the
// forward column pass, events ordering them after the previous iterate and
// before the row and adjoint column passes.  The power method ||U|| cannot use the plain form's per-pixel
// recurrence (M mixes pixels), so it runs myNormest's loop step for step on
// the device (k_ne_*), the host reading the stop flag once per eight steps.
//
// Bounds: the reference reads the image at the interpolation corners without
// checks; here a corner or target outside the image skips that pixel and sets
// the instance's status (kStatusMotionRange) instead of reading out of range.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.h"
#include "inst.cuh"
#include "solver.h"

namespace gbn {

int op_ttv(gbn_ctx* ctx, int dir, const float2* in, float2* out, int W, int H, int F);
Lcg48 lcg48_jump(uint64_t k);
uint64_t lcg48_apply(const Lcg48& j, uint64_t x);

// tables of one problem's meshes (rebuilt at every run)
struct McTables {
  int* inv = nullptr;         // [H*W] rectangle entry landing on each pixel, -1 none
  int* cnt = nullptr;         // [F*H*W] contributions per target (then fill cursors)
  int* off = nullptr;         // [F*H*W + 1] exclusive prefix sums of cnt
  int* bsum = nullptr;        // [scan blocks] block totals of the prefix sum
  int* key = nullptr;         // [4 * l1 * l2 * F] contributions grouped by target, sorted by entry * 4 + corner,
                              // then rewritten to (the entry's pixel R1*W + R2) * 4 + corner
  int* srcmap = nullptr;      // [H*W] pixel each entry (by its R1*W + R2) reads in the adjoint
  float2* wts = nullptr;      // [F][H*W] (Whh, Wvv): each entry's fractional position in frame f
  int* csrc = nullptr;        // [4 * l1 * l2 * F] per contribution: the pixel the adjoint reads
  float2* cw = nullptr;       // [4 * l1 * l2 * F] per contribution: its two weights (fa, fb)
  double* tvpart = nullptr;   // [F * pixel blocks][2] partial sums of the fused tTV kernel
  size_t x = 0, entries = 0;  // F*H*W and l1*l2 the buffers were sized for
  int nbp = 0, nscan = 0;
};

namespace {

constexpr int kStatusMotionRange = 5;  // NestaDevState::status: a mesh point outside the image
constexpr int kNT = 256;
constexpr int kScanItems = 4;                   // prefix-sum elements per thread
constexpr int kScanBlock = kNT * kScanItems;    // per block
constexpr int kTvFrames = 2;                    // frames per thread of the fused tTV kernel

// rows r1b .. r1b+l1-1 and columns r2b .. r2b+l2-1 of the rectangle
// (Interpolator.cpp:63-87: margins H/40 and W/40 in integer division)
struct McRect {
  int r1b, l1, r2b, l2;
};

McRect mc_rect(int W, int H, const int* bb) {
  const int m0 = H / 40, m1 = W / 40;
  McRect r;
  r.l1 = (bb[3] + m0 + 1) - (bb[1] - m0 - 1) + 1;
  r.l2 = (bb[2] + m1 + 1) - (bb[0] - m1 - 1) + 1;
  r.r1b = (bb[1] - m0 - 1) - 1;
  r.r2b = (bb[0] - m1 - 1) - 1;
  return r;
}

bool rect_ok(const McRect& r, int W, int H) {
  return r.l1 > 0 && r.l2 > 0 && r.r1b >= 0 && r.r2b >= 0 && r.r1b + r.l1 <= H && r.r2b + r.l2 <= W;
}

// deformed position of rectangle entry e = i + l1*j in frame k (0-based) and
// its upper-left interpolation corner
struct McPoint {
  float nh, nv;
  int ph, pv;
  bool ok;
};

__device__ __forceinline__ int entry_offset(McRect r, int e, int W) {
  const int i = e % r.l1, j = e / r.l1;
  return (r.r2b + j) + (r.r1b + i) * W;  // (row R1, column R2) in a [H][W] plane
}

__device__ __forceinline__ McPoint mc_point(const float* __restrict__ xn, int xo, int k, int W, int H, int F) {
  const size_t HW = size_t(H) * W;
  McPoint q;
  q.nh = xn[xo + k * HW] - 1.f;
  q.nv = xn[xo + k * HW + HW * F] - 1.f;
  q.ph = int(floorf(q.nh));
  q.pv = int(floorf(q.nv));
  q.ok = q.ph >= 0 && q.ph + 1 < W && q.pv >= 0 && q.pv + 1 < H;
  return q;
}

// p*u + q*v with both products and the sum rounded separately
__device__ __forceinline__ float lin2(float p, float u, float q, float v) {
  return __fadd_rn(__fmul_rn(p, u), __fmul_rn(q, v));
}

// the interpolator's value (optimizer.cl:832-877) at q from frame xf, in the
// kernel's order with separately rounded products and sums: with motion
// compensation the power method starts from this interpolation's rounding
// residue on a constant image, so ||U|| depends on these exact bits
__device__ __forceinline__ float2 bilinear(const float2* __restrict__ xf, const McPoint& q, int W) {
  const float2 i1 = xf[q.ph + size_t(q.pv) * W], i2 = xf[q.ph + 1 + size_t(q.pv) * W];
  const float2 i3 = xf[q.ph + size_t(q.pv + 1) * W], i4 = xf[q.ph + 1 + size_t(q.pv + 1) * W];
  const float a = float(q.ph + 1) - q.nh, b = q.nh - float(q.ph);
  const float c = float(q.pv + 1) - q.nv, d = q.nv - float(q.pv);
  const float2 aux1 = make_float2(lin2(a, i1.x, b, i2.x), lin2(a, i1.y, b, i2.y));
  const float2 aux2 = make_float2(lin2(a, i3.x, b, i4.x), lin2(a, i3.y, b, i4.y));
  return make_float2(lin2(c, aux1.x, d, aux2.x), lin2(c, aux1.y, d, aux2.y));
}

// (M x)[k][p]
__device__ __forceinline__ float2 warp_at(const float2* __restrict__ x, const float* __restrict__ xn, McRect r, int e,
                                          int p, int k, int W, int H, int F, int* __restrict__ status) {
  const float2* xf = x + size_t(k) * H * W;
  if (e < 0) return xf[p];
  const McPoint q = mc_point(xn, entry_offset(r, e, W), k, W, H, F);
  if (!q.ok) {
    atomicExch(status, kStatusMotionRange);
    return xf[p];
  }
  return bilinear(xf, q, W);
}

// ---- table construction ------------------------------------------------------
// inv[ver*W + hor] = the largest entry e whose original-mesh point is (hor, ver);
// srcmap[R1*W + R2] = that pixel (-1 outside the image)
__global__ void k_mc_inv(const int* __restrict__ xm, McRect r, int W, int H, int* __restrict__ inv,
                         int* __restrict__ srcmap, int* __restrict__ status) {
  const int E = r.l1 * r.l2;
  const size_t HW = size_t(H) * W;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    const int R1 = r.r1b + e % r.l1, R2 = r.r2b + e / r.l1;
    const int hor = xm[R1 + size_t(R2) * H] - 1, ver = xm[R1 + size_t(R2) * H + HW] - 1;
    if (hor < 0 || hor >= W || ver < 0 || ver >= H) {
      srcmap[R1 * W + R2] = -1;
      atomicExch(status, kStatusMotionRange);
      continue;
    }
    srcmap[R1 * W + R2] = ver * W + hor;
    atomicMax(inv + size_t(ver) * W + hor, e);
  }
}

// the (entry, frame) pairs that scatter: target pixel (its original-mesh point) in the image, corners too
__device__ __forceinline__ bool scatter_point(const float* __restrict__ xn, const int* __restrict__ xm, McRect r, int e,
                                              int k, int W, int H, int F, McPoint* q, int* src) {
  const size_t HW = size_t(H) * W;
  const int R1 = r.r1b + e % r.l1, R2 = r.r2b + e / r.l1;
  const int hor = xm[R1 + size_t(R2) * H] - 1, ver = xm[R1 + size_t(R2) * H + HW] - 1;
  *q = mc_point(xn, R2 + R1 * W, k, W, H, F);
  *src = ver * W + hor;
  return q->ok && hor >= 0 && hor < W && ver >= 0 && ver < H;
}

__global__ void k_mc_count(const float* __restrict__ xn, const int* __restrict__ xm, McRect r, int W, int H, int F,
                           int* __restrict__ cnt, int* __restrict__ status) {
  const int E = r.l1 * r.l2;
  const size_t HW = size_t(H) * W, n = size_t(E) * F;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < n; t += size_t(gridDim.x) * blockDim.x) {
    const int e = int(t % E), k = int(t / E);
    McPoint q;
    int src;
    if (!scatter_point(xn, xm, r, e, k, W, H, F, &q, &src)) {
      atomicExch(status, kStatusMotionRange);
      continue;
    }
    int* c = cnt + k * HW + size_t(q.pv) * W + q.ph;
    atomicAdd(c, 1);
    atomicAdd(c + 1, 1);
    atomicAdd(c + W, 1);
    atomicAdd(c + W + 1, 1);
  }
}

// exclusive prefix sum of n ints in three launches: per-block scan, scan of the
// block totals, add
__device__ __forceinline__ int block_exclusive_scan(int v, int* swarp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) swarp[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < int(blockDim.x >> 5) ? swarp[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += u;
    }
    if (lane < int(blockDim.x >> 5)) swarp[lane] = wi - w;
    if (lane == int(blockDim.x >> 5) - 1) *total = wi;
  }
  __syncthreads();
  return swarp[wid] + incl - v;
}

__global__ void __launch_bounds__(kNT) k_scan_blocks(const int* __restrict__ in, size_t n, int* __restrict__ out,
                                                      int* __restrict__ bsum) {
  __shared__ int swarp[kNT / 32];
  __shared__ int total;
  const size_t base = size_t(blockIdx.x) * kScanBlock + size_t(threadIdx.x) * kScanItems;
  int v[kScanItems], s = 0;
#pragma unroll
  for (int u = 0; u < kScanItems; ++u) {
    v[u] = base + u < n ? in[base + u] : 0;
    s += v[u];
  }
  int run = block_exclusive_scan(s, swarp, &total);
#pragma unroll
  for (int u = 0; u < kScanItems; ++u) {
    if (base + u < n) out[base + u] = run;
    run += v[u];
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// one block: exclusive scan of the nb block totals in place; out[n] = the grand total
__global__ void __launch_bounds__(1024) k_scan_totals(int* __restrict__ bsum, int nb, int* __restrict__ out, size_t n) {
  __shared__ int swarp[32];
  __shared__ int total;
  int carry = 0;
  for (int b0 = 0; b0 < nb; b0 += 1024) {
    const int b = b0 + int(threadIdx.x);
    const int v = b < nb ? bsum[b] : 0;
    const int ex = block_exclusive_scan(v, swarp, &total);
    if (b < nb) bsum[b] = carry + ex;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_scan_add(int* __restrict__ out, size_t n, const int* __restrict__ bsum) {
  const size_t i = size_t(blockIdx.x) * kScanBlock + threadIdx.x;
  const int add = bsum[blockIdx.x];
#pragma unroll
  for (int u = 0; u < kScanItems; ++u)
    if (i + size_t(u) * kNT < n) out[i + size_t(u) * kNT] += add;
}

// the contributions of every scattering (entry, frame) to its four corners,
// and the entry's fractional position (Whh, Wvv) the weights derive from
__global__ void k_mc_fill(const float* __restrict__ xn, const int* __restrict__ xm, McRect r, int W, int H, int F,
                          const int* __restrict__ off, int* __restrict__ cur, int* __restrict__ key,
                          float2* __restrict__ wts) {
  const int E = r.l1 * r.l2;
  const size_t HW = size_t(H) * W, n = size_t(E) * F;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < n; t += size_t(gridDim.x) * blockDim.x) {
    const int e = int(t % E), k = int(t / E);
    McPoint q;
    int src;
    if (!scatter_point(xn, xm, r, e, k, W, H, F, &q, &src)) continue;
    wts[k * HW + entry_offset(r, e, W)] = make_float2(q.nh - float(q.ph), q.nv - float(q.pv));
    const size_t q00 = k * HW + size_t(q.pv) * W + q.ph;
    const size_t tq[4] = {q00, q00 + 1, q00 + W, q00 + W + 1};
#pragma unroll
    for (int c = 0; c < 4; ++c) key[off[tq[c]] + atomicAdd(cur + tq[c], 1)] = e * 4 + c;
  }
}

// each target's contributions into key order (lists are short: insertion sort)
__global__ void k_mc_sort(const int* __restrict__ off, int* __restrict__ key, size_t n) {
  for (size_t q = blockIdx.x * size_t(blockDim.x) + threadIdx.x; q < n; q += size_t(gridDim.x) * blockDim.x) {
    const int b = off[q], e = off[q + 1];
    for (int i = b + 1; i < e; ++i) {
      const int v = key[i];
      int j = i - 1;
      while (j >= b && key[j] > v) {
        key[j + 1] = key[j];
        --j;
      }
      key[j + 1] = v;
    }
  }
}

// sorted keys entry * 4 + corner -> (the entry's pixel R1*W + R2) * 4 + corner,
// so that neighbouring targets read neighbouring table entries
__global__ void k_mc_rekey(int* __restrict__ key, const int* __restrict__ total, McRect r, int W) {
  const size_t n = size_t(*total);  // contributions filled (off[F*H*W])
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const int k = key[i];
    key[i] = entry_offset(r, k >> 2, W) * 4 + (k & 3);
  }
}

// per contribution, what the adjoint gathers need: the pixel it reads and its
// two weights fa = Whh or 1 - Whh (corner bit 0), fb = Wvv or 1 - Wvv (bit 1),
// rounded as optimizer.cl:880-937 forms them
__global__ void k_mc_pack(const int* __restrict__ off, const int* __restrict__ key, const int* __restrict__ srcmap,
                          const float2* __restrict__ wts, int* __restrict__ csrc, float2* __restrict__ cw, size_t X,
                          size_t HW) {
  for (size_t q = blockIdx.x * size_t(blockDim.x) + threadIdx.x; q < X; q += size_t(gridDim.x) * blockDim.x) {
    const float2* wk = wts + (q / HW) * HW;
    for (int c = off[q], ce = off[q + 1]; c < ce; ++c) {
      const int kc = key[c], e = kc >> 2;
      const float2 w = wk[e];
      csrc[c] = srcmap[e];
      cw[c] = make_float2((kc & 1) ? w.x : __fsub_rn(1.f, w.x), (kc & 2) ? w.y : __fsub_rn(1.f, w.y));
    }
  }
}

// ---- the operators -------------------------------------------------------------
// out = M x (MotionCompensation: copy, then the interpolator), one thread per pixel
__global__ void k_mc_warp(const float2* __restrict__ x, float2* __restrict__ out, const float* __restrict__ xn,
                          const int* __restrict__ inv, McRect r, int W, int H, int F, int* __restrict__ status) {
  const size_t HW = size_t(H) * W, n = HW * F;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < n; t += size_t(gridDim.x) * blockDim.x) {
    const int p = int(t % HW), k = int(t / HW);
    out[t] = warp_at(x, xn, r, inv[p], p, k, W, H, F, status);
  }
}

// out = M^T g (AdjointMotionCompensation: copy, zero the rectangle, scatter),
// one thread per target, contributions in the reference's order; corner c of
// an entry's square gets (g * fa) * fb with fa = Whh or 1 - Whh (c & 1), fb =
// Wvv or 1 - Wvv (c & 2), as optimizer.cl:880-937 rounds them.  Loads of up to
// four contributions are issued before any of them is accumulated.
__global__ void __launch_bounds__(kNT) k_mc_adjoint(const float2* __restrict__ g, float2* __restrict__ out,
                                                     const int* __restrict__ off, const int* __restrict__ csrc,
                                                     const float2* __restrict__ cw, McRect r, int W, int H, int F,
                                                     int pdl) {
  if (pdl) {
    grid_dep_wait();  // g comes from the fused tTV kernel two launches back
    grid_dep_release();
  }
  const size_t HW = size_t(H) * W, n = HW * F;
  const size_t q = blockIdx.x * size_t(kNT) + threadIdx.x;
  if (q >= n) return;
  const int p = int(q % HW), row = p / W, col = p % W;
  const bool in_rect = row >= r.r1b && row < r.r1b + r.l1 && col >= r.r2b && col < r.r2b + r.l2;
  int c = __ldg(off + q);
  const int ce = __ldg(off + q + 1);
  float2 acc = in_rect ? make_float2(0.f, 0.f) : g[q];
  const size_t k = q / HW;
  const float2* gk = g + k * HW;
  while (c < ce) {
    const int m = min(4, ce - c);
    float2 w[4], v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (u < m) {
        w[u] = __ldg(cw + c + u);
        v[u] = gk[__ldg(csrc + c + u)];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (u < m) {
        acc.x = __fadd_rn(acc.x, __fmul_rn(__fmul_rn(v[u].x, w[u].x), w[u].y));
        acc.y = __fadd_rn(acc.y, __fmul_rn(__fmul_rn(v[u].y, w[u].x), w[u].y));
      }
    }
    c += m;
  }
  out[q] = acc;
}

// g = tTVadj(normalise(D M x)) (temporalTV.cl:78-107 sign: u_{f+1} - u_f) and
// the objective's partial sums of |u|^2 and Re<u, d> per (frame, block of 256
// pixels).  grid (ceil(H*W/256), ceil(F/kTvFrames)); each thread warps its
// pixel for kTvFrames+2 consecutive frames (periodic in f) and slides over them.
// Inner iteration `it` reads x_it from the ping-pong pair (x0, x1); past the
// outer loop's last iteration it does nothing, except in the launch that
// recomputes the last update (row-local iteration, fixup), which reads x_last.
__global__ void __launch_bounds__(kNT) k_mc_tv(const float2* __restrict__ x0, const float2* __restrict__ x1, int it,
                                                const float* __restrict__ xn, const int* __restrict__ inv, McRect r,
                                                const NestaDevState* __restrict__ st, float2* __restrict__ g,
                                                double* __restrict__ part, int W, int H, int F,
                                                int* __restrict__ status) {
  __shared__ double sred[2 * kTvFrames][kNT / 32];
  const int HW = H * W;
  const int p = blockIdx.x * kNT + threadIdx.x;
  const bool live = p < HW;
  const int e = live ? __ldg(inv + p) : -1;
  const int f0 = blockIdx.y * kTvFrames, f1 = min(F, f0 + kTvFrames);
  grid_dep_wait();  // x_k comes from the previous iteration's update
  grid_dep_release();
  const int last = st->last_iter;
  int itx = it;
  if (it > last) {  // uniform over the grid
    if (!(st->fixup && it == last + 1)) return;
    itx = last;
  }
  const float2* __restrict__ x = (itx & 1) ? x1 : x0;
  const float inv_mu = 1.0f / st->mu;
  float su2[kTvFrames], sud[kTvFrames];
#pragma unroll
  for (int u = 0; u < kTvFrames; ++u) su2[u] = sud[u] = 0.f;
  if (live) {
    // M x_k at this pixel for frames f0-1 .. f1 (periodic): positions, then
    // corners, then values, so that the loads of all frames are in flight together
    constexpr int NW = kTvFrames + 2;
    const int nw = f1 - f0 + 2;
    int fr[NW];
#pragma unroll
    for (int u = 0; u < NW; ++u) fr[u] = (f0 - 1 + u + F) % F;
    float2 w[NW];
    if (e < 0) {
#pragma unroll
      for (int u = 0; u < NW; ++u)
        if (u < nw) w[u] = x[size_t(fr[u]) * HW + p];
    } else {
      const int xo = entry_offset(r, e, W);
      McPoint q[NW];
#pragma unroll
      for (int u = 0; u < NW; ++u)
        if (u < nw) q[u] = mc_point(xn, xo, fr[u], W, H, F);
#pragma unroll
      for (int u = 0; u < NW; ++u) {
        if (u < nw) {
          const float2* xf = x + size_t(fr[u]) * HW;
          if (q[u].ok) {
            w[u] = bilinear(xf, q[u], W);
          } else {
            atomicExch(status, kStatusMotionRange);
            w[u] = xf[p];
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kTvFrames; ++u) {
      const int f = f0 + u;
      if (f < f1) {
        const float2 d0 = csub(w[u + 1], w[u]);
        const float2 u0 = tv_normalize(d0, inv_mu);
        const float2 u1 = tv_normalize(csub(w[u + 2], w[u + 1]), inv_mu);
        su2[u] = fmaf(u0.x, u0.x, u0.y * u0.y);
        sud[u] = fmaf(u0.x, d0.x, u0.y * d0.y);
        g[size_t(f) * HW + p] = csub(u1, u0);
      }
    }
  }
  // fixed-order reduction: FP32 warp shuffles (32 values), then the warps in
  // order in FP64 (FP64 throughput is a small fraction of FP32's here)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int u = 0; u < kTvFrames; ++u) {
    float a = su2[u], b = sud[u];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      sred[2 * u][wid] = double(a);
      sred[2 * u + 1][wid] = double(b);
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * kTvFrames) {
    const int u = threadIdx.x >> 1;
    if (f0 + u < f1) {
      double t = 0.0;
#pragma unroll
      for (int w = 0; w < kNT / 32; ++w) t += sred[threadIdx.x][w];
      part[2 * (size_t(f0 + u) * gridDim.x + blockIdx.x) + (threadIdx.x & 1)] = t;
    }
  }
}

// ---- the power method's vector operations ----------------------------------------
__global__ void k_fill(float2* __restrict__ v, size_t n, float2 value) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) v[i] = value;
}
// sum of |v|^2 and of |Re| + |Im|: FP32 within a thread's few elements and
// a warp, FP64 across warps and blocks; per-block partials in fixed slots
// (blocks stride over the vector in a fixed order, so the sums are
// deterministic)
__device__ __forceinline__ void warp_sums_to_block(float s2, float s1, double* sred2, double* sred1, double* part) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sred2[wid] = double(s2);
    sred1[wid] = double(s1);
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    const double* r = threadIdx.x == 0 ? sred2 : sred1;
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kNT / 32; ++w) t += r[w];
    part[2 * blockIdx.x + threadIdx.x] = t;
  }
}
int grid1(gbn_ctx* ctx, size_t n) { return int(std::min<size_t>((n + kNT - 1) / kNT, size_t(ctx->nsm) * 8)); }

// ---- the power method on the device ------------------------------------------------
// myNormest's loop (NestaUp.cpp:291-439) with U = tTV M and U^T = M^T tTVadj,
// driven by a device-side state so that steps are enqueued in chunks without
// host round trips.  Each step: U x (warp, tTV, partial sums of |Sx|^2 and
// |Re|+|Im|), a scalar kernel (restart test, e), the drand48 restart (only when
// U x is exactly zero), U^T Sx (tTVadj and the ordered M^T gather, partial
// sums), a scalar kernel (||x||, the stopping test).  x is stored unscaled; its
// scale 1/||x|| is applied as each value is read, which rounds exactly as a
// separate scaling pass would.
struct McNe {
  float e, e0, s;          // current and previous ||U x||, scale of the stored x
  int cnt, done, restart;  // steps taken, stop flag, restart in the current step
  int nrestart;            // restarts so far (each consumed F*H*W drand48 draws)
  int pad;
  unsigned long long rand;  // drand48 state
};
constexpr int kPartDoubles = 2 * 1024 + 2 + 8;  // block partials, two totals, the McNe state
static_assert(sizeof(McNe) <= 8 * sizeof(double), "McNe fits its slot");
constexpr float kNeTol = 1e-3f;
constexpr int kNeMax = 100;

__device__ __forceinline__ McNe* ne_state(double* part) { return reinterpret_cast<McNe*>(part + 2 * 1024 + 2); }

// (M (s x))[k][p] for the stored, unscaled x
__device__ __forceinline__ float2 warp_scaled(const float2* __restrict__ x, float sc, const float* __restrict__ xn, McRect r,
                                             int e, int p, int k, int W, int H, int F, int* __restrict__ status) {
  const float2* xf = x + size_t(k) * H * W;
  if (e >= 0) {
    const McPoint q = mc_point(xn, entry_offset(r, e, W), k, W, H, F);
    if (q.ok) {
      const float2 i1 = cscale(xf[q.ph + size_t(q.pv) * W], sc), i2 = cscale(xf[q.ph + 1 + size_t(q.pv) * W], sc);
      const float2 i3 = cscale(xf[q.ph + size_t(q.pv + 1) * W], sc);
      const float2 i4 = cscale(xf[q.ph + 1 + size_t(q.pv + 1) * W], sc);
      const float a = float(q.ph + 1) - q.nh, b = q.nh - float(q.ph);
      const float c = float(q.pv + 1) - q.nv, d = q.nv - float(q.pv);
      const float2 aux1 = make_float2(lin2(a, i1.x, b, i2.x), lin2(a, i1.y, b, i2.y));
      const float2 aux2 = make_float2(lin2(a, i3.x, b, i4.x), lin2(a, i3.y, b, i4.y));
      return make_float2(lin2(c, aux1.x, d, aux2.x), lin2(c, aux1.y, d, aux2.y));
    }
    atomicExch(status, kStatusMotionRange);
  }
  return cscale(xf[p], sc);
}

__global__ void k_ne_init(double* part, float e, unsigned long long rand) {
  McNe* ne = ne_state(part);
  ne->e = e;
  ne->e0 = 0.f;
  ne->s = 1.0f / e;
  ne->cnt = 0;
  ne->done = !(fabsf(e - 0.f) > kNeTol * e && 0 < kNeMax);
  ne->restart = 0;
  ne->nrestart = 0;
  ne->rand = rand;
}

// Sx = tTV(M (s x)), partial sums
__global__ void __launch_bounds__(kNT) k_ne_u(const float2* __restrict__ x, float2* __restrict__ Sx,
                                               const float* __restrict__ xn, const int* __restrict__ inv, McRect r,
                                               int W, int H, int F, double* __restrict__ part, int* __restrict__ status) {
  __shared__ double sred2[kNT / 32], sred1[kNT / 32];
  const McNe* ne = ne_state(part);
  if (ne->done) return;
  const float sc = ne->s;
  const size_t HW = size_t(H) * W, n = HW * F;
  float s2 = 0.f, s1 = 0.f;
  for (size_t i = blockIdx.x * size_t(kNT) + threadIdx.x; i < n; i += size_t(gridDim.x) * kNT) {
    const int p = int(i % HW), k = int(i / HW);
    const int e = inv[p];
    const float2 w0 = warp_scaled(x, sc, xn, r, e, p, k, W, H, F, status);
    const float2 wm = warp_scaled(x, sc, xn, r, e, p, (k + F - 1) % F, W, H, F, status);
    const float2 a = csub(w0, wm);
    Sx[i] = a;
    s2 = fmaf(a.x, a.x, fmaf(a.y, a.y, s2));
    s1 += fabsf(a.x) + fabsf(a.y);
  }
  warp_sums_to_block(s2, s1, sred2, sred1, part);
}

// sums of the block partials: each thread a strided subset in order, then
// the threads in order
__device__ __forceinline__ void ne_totals(const double* __restrict__ part, int nblk, double* sred, double* t2, double* t1) {
  double s2 = 0.0, s1 = 0.0;
  for (int b = threadIdx.x; b < nblk; b += kNT) {
    s2 += part[2 * b];
    s1 += part[2 * b + 1];
  }
  *t2 = block_sum<kNT>(s2, sred);
  *t1 = block_sum<kNT>(s1, sred);
}

// e0 = e; restart test (Scasum(U x) == 0, NestaUp.cpp:369-385); e = ||U x||
__global__ void __launch_bounds__(kNT) k_ne_s1(double* part, int nblk) {
  __shared__ double sred[kNT / 32];
  McNe* ne = ne_state(part);
  if (ne->done) return;
  double t2, t1;
  ne_totals(part, nblk, sred, &t2, &t1);
  if (threadIdx.x == 0) {
    ne->e0 = ne->e;
    ne->restart = (t1 == 0.0) ? 1 : 0;
    if (!ne->restart) ne->e = float(sqrt(t2));
  }
}

// restart: Sx = (drand48(), 0) in element order, partial sums
__global__ void __launch_bounds__(kNT) k_ne_restart(float2* __restrict__ Sx, size_t n, double* __restrict__ part) {
  __shared__ double sred2[kNT / 32], sred1[kNT / 32];
  const McNe* ne = ne_state(part);
  if (ne->done || !ne->restart) return;
  const unsigned long long x0 = ne->rand;
  float s2 = 0.f, s1 = 0.f;
  for (size_t i = blockIdx.x * size_t(kNT) + threadIdx.x; i < n; i += size_t(gridDim.x) * kNT) {
    unsigned long long ra = 1, rc = 0, ba = 0x5DEECE66DULL, bc = 0xBULL, k = i + 1;
    const unsigned long long mask = (1ULL << 48) - 1;
    while (k) {
      if (k & 1) {
        rc = (ba * rc + bc) & mask;
        ra = (ba * ra) & mask;
      }
      bc = (ba * bc + bc) & mask;
      ba = (ba * ba) & mask;
      k >>= 1;
    }
    const float2 a = make_float2(__double2float_rn(double((ra * x0 + rc) & mask) * 0x1p-48), 0.f);
    Sx[i] = a;
    s2 = fmaf(a.x, a.x, fmaf(a.y, a.y, s2));
    s1 += fabsf(a.x) + fabsf(a.y);
  }
  warp_sums_to_block(s2, s1, sred2, sred1, part);
}

// after a restart: e = ||Sx||, the generator moved past the n draws
__global__ void __launch_bounds__(kNT) k_ne_s1b(double* part, int nblk, unsigned long long ja, unsigned long long jc) {
  __shared__ double sred[kNT / 32];
  McNe* ne = ne_state(part);
  if (ne->done || !ne->restart) return;
  double t2, t1;
  ne_totals(part, nblk, sred, &t2, &t1);
  if (threadIdx.x == 0) {
    ne->e = float(sqrt(t2));
    ne->rand = (ja * ne->rand + jc) & ((1ULL << 48) - 1);
    ne->nrestart += 1;
  }
}

// x = M^T tTVadj(Sx) (operatorUt without negation), partial sums
__global__ void __launch_bounds__(kNT) k_ne_ut(const float2* __restrict__ Sx, float2* __restrict__ x,
                                                const int* __restrict__ off, const int* __restrict__ csrc,
                                                const float2* __restrict__ cw, McRect r, int W, int H, int F,
                                                double* __restrict__ part) {
  __shared__ double sred2[kNT / 32], sred1[kNT / 32];
  const McNe* ne = ne_state(part);
  if (ne->done) return;
  const size_t HW = size_t(H) * W, n = HW * F;
  float s2 = 0.f, s1 = 0.f;
  for (size_t q = blockIdx.x * size_t(kNT) + threadIdx.x; q < n; q += size_t(gridDim.x) * kNT) {
    const int p = int(q % HW), row = p / W, col = p % W;
    const size_t k = q / HW;
    const float2* u0 = Sx + k * HW;                   // tTVadj: u_{f+1} - u_f
    const float2* u1 = Sx + size_t((k + 1) % F) * HW;
    const bool in_rect = row >= r.r1b && row < r.r1b + r.l1 && col >= r.r2b && col < r.r2b + r.l2;
    float2 acc = in_rect ? make_float2(0.f, 0.f) : csub(u1[p], u0[p]);
    for (int c = off[q], ce = off[q + 1]; c < ce; ++c) {
      const float2 w = __ldg(cw + c);
      const int src = __ldg(csrc + c);
      const float2 v = csub(u1[src], u0[src]);
      acc.x = __fadd_rn(acc.x, __fmul_rn(__fmul_rn(v.x, w.x), w.y));
      acc.y = __fadd_rn(acc.y, __fmul_rn(__fmul_rn(v.y, w.x), w.y));
    }
    x[q] = acc;
    s2 = fmaf(acc.x, acc.x, fmaf(acc.y, acc.y, s2));
    s1 += fabsf(acc.x) + fabsf(acc.y);
  }
  warp_sums_to_block(s2, s1, sred2, sred1, part);
}

// ||x||, the scale of the next step, the stopping test
__global__ void __launch_bounds__(kNT) k_ne_s2(double* part, int nblk) {
  __shared__ double sred[kNT / 32];
  McNe* ne = ne_state(part);
  if (ne->done) return;
  double t2, t1;
  ne_totals(part, nblk, sred, &t2, &t1);
  if (threadIdx.x == 0) {
    const float nx = float(sqrt(t2));
    ne->s = 1.0f / nx;
    ne->cnt += 1;
    ne->done = !(fabsf(ne->e - ne->e0) > kNeTol * ne->e && ne->cnt < kNeMax);
  }
}

__global__ void k_ne_finish(const double* part, NestaDevState* st) {
  const McNe* ne = ne_state(const_cast<double*>(part));
  st->normU = ne->e;
  st->normest_iters = ne->cnt;
  st->ne_done = 1;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void tables_free(McTables* t) {
  void* ptrs[] = {t->inv, t->cnt, t->off, t->bsum, t->key, t->srcmap, t->wts, t->tvpart, t->csrc, t->cw};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  *t = McTables{};
}

// buffers for F*H*W pixels and E rectangle entries (kept when large enough)
int tables_alloc(McTables* t, int W, int H, int F, int E) {
  const size_t HW = size_t(H) * W, X = HW * F;
  const int nbp = int((HW + kNT - 1) / kNT);
  if (t->inv && t->x == X && size_t(E) <= t->entries) return GBN_OK;
  tables_free(t);
  t->x = X;
  t->entries = size_t(E);
  t->nbp = nbp;
  t->nscan = int((X + kScanBlock - 1) / kScanBlock);
  cudaError_t e = cudaMalloc(&t->inv, HW * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&t->cnt, X * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&t->off, (X + 1) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&t->bsum, size_t(t->nscan) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&t->key, 4 * size_t(E) * F * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&t->srcmap, HW * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&t->wts, X * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&t->tvpart, 2 * size_t(F) * nbp * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&t->csrc, 4 * size_t(E) * F * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&t->cw, 4 * size_t(E) * F * sizeof(float2));
  if (e != cudaSuccess) {
    cudaGetLastError();
    tables_free(t);
    return set_error(GBN_ERR_NOMEM, "motion compensation table allocation failed");
  }
  return GBN_OK;
}

// builds inv and the contribution lists from the meshes (asynchronous on s)
int tables_build(gbn_ctx* ctx, McTables* t, const float* xn, const int* xm, const McRect& r, int W, int H, int F,
                 int* status, cudaStream_t s) {
  const size_t HW = size_t(H) * W, X = HW * F;
  const int E = r.l1 * r.l2;
  cudaError_t e = cudaMemsetAsync(t->inv, 0xFF, HW * sizeof(int), s);  // -1
  if (e == cudaSuccess) e = cudaMemsetAsync(t->cnt, 0, X * sizeof(int), s);
  if (e != cudaSuccess) return cuda_status(e, "motion compensation tables");
  k_mc_inv<<<grid1(ctx, size_t(E)), kNT, 0, s>>>(xm, r, W, H, t->inv, t->srcmap, status);
  k_mc_count<<<grid1(ctx, size_t(E) * F), kNT, 0, s>>>(xn, xm, r, W, H, F, t->cnt, status);
  k_scan_blocks<<<t->nscan, kNT, 0, s>>>(t->cnt, X, t->off, t->bsum);
  k_scan_totals<<<1, 1024, 0, s>>>(t->bsum, t->nscan, t->off, X);
  k_scan_add<<<t->nscan, kNT, 0, s>>>(t->off, X, t->bsum);
  if ((e = cudaMemsetAsync(t->cnt, 0, X * sizeof(int), s)) != cudaSuccess)
    return cuda_status(e, "motion compensation tables");
  k_mc_fill<<<grid1(ctx, size_t(E) * F), kNT, 0, s>>>(xn, xm, r, W, H, F, t->off, t->cnt, t->key, t->wts);
  k_mc_sort<<<grid1(ctx, X), kNT, 0, s>>>(t->off, t->key, X);
  k_mc_rekey<<<grid1(ctx, 4 * size_t(E) * F), kNT, 0, s>>>(t->key, t->off + X, r, W);
  k_mc_pack<<<grid1(ctx, X), kNT, 0, s>>>(t->off, t->key, t->srcmap, t->wts, t->csrc, t->cw, X, HW);
  ctx->launches += 10;
  return GBN_OK;
}

}  // namespace

void motion_free(gbn_problem* P) {
  if (P->mc_tab) {
    tables_free(P->mc_tab);
    delete P->mc_tab;
    P->mc_tab = nullptr;
  }
  void* ptrs[] = {P->mc_xw, P->mc_g, P->mc_gm, P->mc_part};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  P->mc_xw = P->mc_g = P->mc_gm = nullptr;
  P->mc_part = nullptr;
}

int motion_set(gbn_problem* P, const float* xn, const int* xmesh, const int* bb) {
  if (!xn && !xmesh && !bb) {
    P->mc_on = false;
    return GBN_OK;
  }
  if (!xn || !xmesh || !bb) return set_error(GBN_ERR_INVALID, "motion compensation needs xn, the mesh and the bounding box");
  const McRect r = mc_rect(P->W, P->H, bb);
  if (!rect_ok(r, P->W, P->H))
    return set_error(GBN_ERR_INVALID, "motion compensation: bounding box plus margins leaves the image");
  const size_t X = size_t(P->W) * P->H * P->F;
  if (!P->mc_xw) {
    cudaError_t e = cudaMalloc(&P->mc_xw, X * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&P->mc_g, X * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&P->mc_gm, X * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&P->mc_part, kPartDoubles * sizeof(double));
    if (e != cudaSuccess) {
      cudaGetLastError();
      motion_free(P);
      return set_error(GBN_ERR_NOMEM, "motion compensation workspace allocation failed");
    }
  }
  if (!P->mc_tab) P->mc_tab = new McTables();
  const int rc = tables_alloc(P->mc_tab, P->W, P->H, P->F, r.l1 * r.l2);
  if (rc != GBN_OK) return rc;
  P->mc_xn = xn;
  P->mc_xmesh = xmesh;
  std::memcpy(P->mc_bb, bb, sizeof(P->mc_bb));
  P->mc_on = true;
  return GBN_OK;
}

namespace {

// out = M in
void mc_apply(gbn_ctx* ctx, gbn_problem* P, const float2* in, float2* out, cudaStream_t s) {
  const size_t X = size_t(P->W) * P->H * P->F;
  const McRect r = mc_rect(P->W, P->H, P->mc_bb);
  k_mc_warp<<<grid1(ctx, X), kNT, 0, s>>>(in, out, P->mc_xn, P->mc_tab->inv, r, P->W, P->H, P->F, &P->st->status);
  ctx->launches += 1;
}

// myNormest (NestaUp.cpp:291-439) with U = tTV M, U^T = M^T tTVadj: steps on
// the device (k_ne_*), enqueued kNeChunk at a time; the host reads each
// chunk's stop flag while the next chunk runs
int mc_normest(gbn_ctx* ctx, gbn_problem* P, cudaStream_t s) {
  constexpr int kNeChunk = 8;
  const int W = P->W, H = P->H, F = P->F;
  const size_t X = size_t(W) * H * F;
  const McTables* t = P->mc_tab;
  const McRect r = mc_rect(W, H, P->mc_bb);
  float2 *x = P->mc_gm, *Sx = P->mc_g;
  const int nblk = std::min(1024, grid1(ctx, X));
  const float e_init = float(std::sqrt(double(X)));  // ||ones||
  const Lcg48 jX = lcg48_jump(uint64_t(X));
  k_fill<<<grid1(ctx, X), kNT, 0, s>>>(x, X, make_float2(1.f, 0.f));
  k_ne_init<<<1, 1, 0, s>>>(P->mc_part, e_init, (unsigned long long)ctx->rand48);
  ctx->launches += 2;
  // chunks of steps with one chunk of lookahead: the host waits for chunk
  // c-1's stop flag (pinned, copied behind it) while chunk c runs
  int rc = host_flags_ready(ctx);
  if (rc != GBN_OK) return rc;
  const McNe* dne = reinterpret_cast<const McNe*>(P->mc_part + 2 * 1024 + 2);
  cudaError_t e = cudaSuccess;
  int chunk = 0;
  for (int steps = 0; steps < kNeMax; ++chunk) {
    for (int k = 0; k < kNeChunk && steps < kNeMax; ++k, ++steps) {
      k_ne_u<<<nblk, kNT, 0, s>>>(x, Sx, P->mc_xn, t->inv, r, W, H, F, P->mc_part, &P->st->status);
      k_ne_s1<<<1, kNT, 0, s>>>(P->mc_part, nblk);
      k_ne_restart<<<nblk, kNT, 0, s>>>(Sx, X, P->mc_part);
      k_ne_s1b<<<1, kNT, 0, s>>>(P->mc_part, nblk, (unsigned long long)jX.a, (unsigned long long)jX.c);
      k_ne_ut<<<nblk, kNT, 0, s>>>(Sx, x, t->off, t->csrc, t->cw, r, W, H, F, P->mc_part);
      k_ne_s2<<<1, kNT, 0, s>>>(P->mc_part, nblk);
      ctx->launches += 6;
    }
    if ((e = cudaMemcpyAsync(&ctx->host_flags[chunk & 1], &dne->done, sizeof(int), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaEventRecord(ctx->ev_flag[chunk & 1], s)) != cudaSuccess)
      return cuda_status(e, "power method");
    if (chunk > 0) {
      if ((e = cudaEventSynchronize(ctx->ev_flag[(chunk - 1) & 1])) != cudaSuccess) return cuda_status(e, "power method");
      if (ctx->host_flags[(chunk - 1) & 1]) break;
    }
  }
  struct {
    int nrestart;
  } h{0};
  if ((e = cudaMemcpyAsync(&h.nrestart, &dne->nrestart, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_status(e, "power method");
  for (int i = 0; i < h.nrestart; ++i) ctx->rand48 = lcg48_apply(jX, ctx->rand48);
  k_ne_finish<<<1, 1, 0, s>>>(P->mc_part, P->st);
  ctx->launches += 1;
  return GBN_OK;
}

}  // namespace

// MotionCompensation (dir = GBN_TTV_FORWARD) or AdjointMotionCompensation
// (GBN_TTV_ADJOINT) of one XData [F][H][W] as a single operator.
int motion_op(gbn_ctx* ctx, int dir, const float2* in, float2* out, const float* xn, const int* xm, const int* bb,
              int W, int H, int F) {
  const McRect r = mc_rect(W, H, bb);
  if (!rect_ok(r, W, H))
    return set_error(GBN_ERR_INVALID, "motion compensation: bounding box plus margins leaves the image");
  if (in == out) return set_error(GBN_ERR_INVALID, "motion compensation: input and output must differ");
  void* scr = nullptr;
  int rc = ctx_scratch(ctx, sizeof(int), &scr);
  if (rc != GBN_OK) return rc;
  int* status = static_cast<int*>(scr);
  cudaStream_t s = ctx->stream;
  McTables t;
  if ((rc = tables_alloc(&t, W, H, F, r.l1 * r.l2)) != GBN_OK) return rc;
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), s);
  if (e != cudaSuccess) rc = cuda_status(e, "motion compensation");
  if (rc == GBN_OK) rc = tables_build(ctx, &t, xn, xm, r, W, H, F, status, s);
  if (rc == GBN_OK) {
    const size_t X = size_t(W) * H * F;
    if (dir == GBN_TTV_FORWARD)
      k_mc_warp<<<grid1(ctx, X), kNT, 0, s>>>(in, out, xn, t.inv, r, W, H, F, status);
    else
      k_mc_adjoint<<<int((X + kNT - 1) / kNT), kNT, 0, s>>>(in, out, t.off, t.csrc, t.cw, r, W, H, F, 0);
    ctx->launches += 1;
  }
  int h = 0;
  if (rc == GBN_OK) {
    if ((e = cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s)) == cudaSuccess)
      e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_status(e, "motion compensation");
  } else {
    cudaStreamSynchronize(s);
  }
  tables_free(&t);
  if (rc == GBN_OK && h) return set_error(GBN_ERR_INVALID, "motion compensation: a mesh point interpolates outside the image");
  return rc;
}

// The motion-compensated solve of problem P; x_out holds the starting image.
int nesta_run_mc(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params* prm, float2* x_out) {
  const SizeKernels* kh = find_size(P->H);
  const SizeKernels* kw = find_size(P->W);
  const int W = P->W, H = P->H, F = P->F, C = P->C;
  cudaStream_t s = ctx->stream;
  McTables* t = P->mc_tab;
  const McRect r = mc_rect(W, H, P->mc_bb);
  int cpb, k2;
  tuning_for(ctx, W, H, F, C, &cpb, &k2);
  cpb = std::max(1, std::min(cpb, C));
  const dim3 g1(W / kWB, (C + cpb - 1) / cpb, F);
  const long long steps = ((long long)F * H * C + kw->rows_per_cta - 1) / kw->rows_per_cta;
  const int g2 = row_grid(ctx, kw, true, steps, k2);
  const dim3 g3(W / kWB, 2, F);
  const dim3 gtv(t->nbp, (F + kTvFrames - 1) / kTvFrames);
  const int gadj = int((size_t(W) * H * F + kNT - 1) / kNT);
  FusedArgs a = make_args(P, x_out);
  a.tv_src = P->mc_xw;  // marks the motion-compensated form: the forward pass skips its tTV sums
  a.grad_ext = P->mc_gm;
  a.part_tv = t->tvpart;
  a.ntv = F * t->nbp;
  const FusedArgs* tab = P->d_args;
  const BatchMap bm = single_map(F, P->ctl);
  int rc;
  // the row-local iteration (rowlocal.cuh) takes problems whose kept rows are
  // fully sampled or unsampled; the row analysis's result comes back to
  // pinned host memory while the setup is queued
  const bool check_rows = ctx->row_local && kh->iter_cols;
  if (check_rows && (rc = partial_flag_ready(ctx)) != GBN_OK) return rc;
  ctx->launches += launch_pre(P, *prm, s);
  cudaError_t ef = cudaSuccess;
  if (check_rows) {
    ef = cudaMemcpyAsync(ctx->host_partial, &P->st->partial_rows, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (ef == cudaSuccess) ef = cudaEventRecord(ctx->ev_partial, s);
    if (ef != cudaSuccess) return cuda_status(ef, "row structure read-back");
  }
  if ((rc = tables_build(ctx, t, P->mc_xn, P->mc_xmesh, r, W, H, F, &P->st->status, s)) != GBN_OK) return rc;
  ctx->launches += launch_store_args(P->d_args, a, s);
  ctx->launches += launch_group_init(tab, 1, kw->rows_per_cta, P->ctl, s);
  if (check_rows) {  // T = IDFT_W(y) of the kept rows, the row-local iteration's data term
    kw->rows(tab, bm, 0, false, row_grid(ctx, kw, false, steps, k2), s);
    ctx->launches += 1;
  }
  // maxima of x0 and of U x0 = tTV(M x0) (NestaUp.cpp:491, 521-568)
  mc_apply(ctx, P, x_out, P->mc_xw, s);
  ctx->launches += launch_maxima(ctx, P, x_out, P->mc_xw, s);
  if ((rc = mc_normest(ctx, P, s)) != GBN_OK) return rc;
  ctx->launches += launch_setup(P, s);
  // k_mc_tv and M^T g run on the side stream beside the forward pass: k_mc_tv
  // waits for the iterate (the previous adjoint column pass), the row pass
  // waits for k_mc_tv's objective sums, the adjoint column pass for M^T g
  cudaError_t se = cudaSuccess;
  if (!ctx->mc_stream) {
    se = cudaStreamCreateWithFlags(&ctx->mc_stream, cudaStreamNonBlocking);
    if (se == cudaSuccess) se = cudaEventCreateWithFlags(&ctx->ev_mc_x, cudaEventDisableTiming);
    if (se == cudaSuccess) se = cudaEventCreateWithFlags(&ctx->ev_mc_tv, cudaEventDisableTiming);
    if (se == cudaSuccess) se = cudaEventCreateWithFlags(&ctx->ev_mc_adj, cudaEventDisableTiming);
    if (se != cudaSuccess) return cuda_status(se, "motion-compensated side stream");
  }
  bool row_local = false;
  if (check_rows) {
    if ((ef = cudaEventSynchronize(ctx->ev_partial)) != cudaSuccess) return cuda_status(ef, "row structure read-back");
    row_local = *ctx->host_partial == 0;
  }
  if (row_local) {
    // per inner iteration, on one stream with programmatic dependent launch:
    // k_mc_tv (M x_k, D, normalisation, tTVadj, objective sums), M^T g, and the
    // one-kernel iteration, whose update waits for M^T g; one more launch per
    // outer loop recomputes the last update if the stopping rule ends the loop
    // (the update gathering M^T g itself, without k_mc_adjoint, measured
    // slower: 20.7 against 16.7 ms per reconstruction at 256x256x20, 12 coils)
    const unsigned n_iter_launch = prm->maxIter + (prm->stoptest == 1 ? 1u : 0u);
    for (unsigned nl = 1; nl <= prm->maxIntIter; ++nl) {
      ctx->launches += launch_outer_begin(ctx, P, int(nl), x_out, s);
      for (unsigned it = 0; it < n_iter_launch; ++it) {
        launch_pdl(k_mc_tv, gtv, kNT, 0, s, (const float2*)P->xk0, (const float2*)P->xk1, int(it),
                   (const float*)P->mc_xn, (const int*)t->inv, r, (const NestaDevState*)P->st, P->mc_g, t->tvpart, W,
                   H, F, &P->st->status);
        launch_pdl(k_mc_adjoint, dim3(gadj), kNT, 0, s, (const float2*)P->mc_g, P->mc_gm, (const int*)t->off,
                   (const int*)t->csrc, (const float2*)t->cw, r, W, H, F, 1);
        GBN_LAUNCH(ctx, GBN_PROF_ITER, 1, kh->iter_cols(tab, bm, int(it), true, g3, s));
        ctx->launches += 2;
      }
      ctx->launches += launch_outer_end(ctx, P, x_out, s);
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBN_OK : cuda_status(e, "motion-compensated nesta launch");
  }
  cudaStream_t aux = ctx->mc_stream;
  for (unsigned nl = 1; nl <= prm->maxIntIter; ++nl) {
    ctx->launches += launch_outer_begin(ctx, P, int(nl), x_out, s);
    for (unsigned it = 0; it < prm->maxIter; ++it) {
      cudaEventRecord(ctx->ev_mc_x, s);
      cudaStreamWaitEvent(aux, ctx->ev_mc_x, 0);
      k_mc_tv<<<gtv, kNT, 0, aux>>>(P->xk0, P->xk1, int(it), P->mc_xn, t->inv, r, P->st, P->mc_g, t->tvpart, W, H, F,
                                    &P->st->status);
      cudaEventRecord(ctx->ev_mc_tv, aux);
      k_mc_adjoint<<<gadj, kNT, 0, aux>>>(P->mc_g, P->mc_gm, t->off, t->csrc, t->cw, r, W, H, F, 0);
      cudaEventRecord(ctx->ev_mc_adj, aux);
      kh->fwd_cols(tab, bm, int(it), cpb, g1, s);
      cudaStreamWaitEvent(s, ctx->ev_mc_tv, 0);
      kw->rows(tab, bm, int(it), true, g2, s);
      cudaStreamWaitEvent(s, ctx->ev_mc_adj, 0);
      kh->inv_cols(tab, bm, int(it), true, g3, s);
      ctx->launches += 5;
    }
    ctx->launches += launch_outer_end(ctx, P, x_out, s);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBN_OK : cuda_status(e, "motion-compensated nesta launch");
}

}  // namespace gbn
