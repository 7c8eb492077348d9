// Motion-compensated tTV-NESTA (NestaUp with argsMC != nullptr): the sparsity
// operator becomes U x = tTV(M x) and U^T u = M^T tTVadj(u) (NestaUp.cpp:
// 201-278), where M warps every frame by bilinear interpolation on a deformed
// mesh (MotionCompensation.cpp:57-78; optimizer.cl:832-877) and M^T scatters
// back with the same weights (AdjointMotionCompensation.cpp:59-86;
// optimizer.cl:880-937; initialize.cl:55-80).  The solve starts from the image
// already in the output buffer (the reference skips x0 = E^H y with argsMC,
// NestaUp.cpp:483-486).
//
// Per inner iteration: x_w = M x_k (copy + gather), then one kernel forms the
// tTV gradient g = tTVadj(normalise(D x_w)) and the objective's partial sums,
// the fused forward column and row passes run as in the plain form (the
// forward pass skips its tTV sums), M^T g (copy, zero rectangle, scatter with
// atomic adds, as the reference) feeds the adjoint column pass, which takes it
// as its tTV gradient.  The power method ||U|| cannot use the plain form's
// per-pixel recurrence (M mixes pixels), so it runs myNormest's loop literally
// with one host read of the norms per step.
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

namespace {

constexpr int kStatusMotionRange = 5;  // NestaDevState::status: a mesh point outside the image
constexpr int kNT = 256;

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

struct McPoint {
  int hor, ver, ph, pv;  // target pixel, upper-left interpolation corner
  float nh, nv;          // deformed position (0-based)
  bool ok;
};

__device__ __forceinline__ McPoint mc_point(const float* __restrict__ xn, const int* __restrict__ xm, McRect r,
                                            int W, int H, int F, int i, int j, int k) {
  McPoint q;
  const int R1 = r.r1b + i, R2 = r.r2b + j;
  const size_t HW = size_t(H) * W;
  q.hor = xm[R1 + size_t(R2) * H] - 1;
  q.ver = xm[R1 + size_t(R2) * H + HW] - 1;
  q.nh = xn[R2 + size_t(R1) * W + k * HW] - 1.f;
  q.nv = xn[R2 + size_t(R1) * W + k * HW + HW * F] - 1.f;
  q.ph = int(floorf(q.nh));
  q.pv = int(floorf(q.nv));
  q.ok = q.hor >= 0 && q.hor < W && q.ver >= 0 && q.ver < H && q.ph >= 0 && q.ph + 1 < W && q.pv >= 0 && q.pv + 1 < H;
  return q;
}

// p*u + q*v with both products and the sum rounded separately
__device__ __forceinline__ float lin2(float p, float u, float q, float v) {
  return __fadd_rn(__fmul_rn(p, u), __fmul_rn(q, v));
}

// interpolator (optimizer.cl:832-877); `out` already holds a copy of `in`
__global__ void k_mc_warp(const float2* __restrict__ in, float2* __restrict__ out, const float* __restrict__ xn,
                          const int* __restrict__ xm, McRect r, int W, int H, int F, int* __restrict__ status) {
  const size_t n = size_t(r.l1) * r.l2 * F;
  const size_t HW = size_t(H) * W;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < n; t += size_t(gridDim.x) * blockDim.x) {
    const int i = int(t % r.l1), j = int((t / r.l1) % r.l2), k = int(t / (size_t(r.l1) * r.l2));
    const McPoint q = mc_point(xn, xm, r, W, H, F, i, j, k);
    if (!q.ok) {
      atomicExch(status, kStatusMotionRange);
      continue;
    }
    const float2* src = in + k * HW;
    const float2 i1 = src[q.ph + size_t(q.pv) * W], i2 = src[q.ph + 1 + size_t(q.pv) * W];
    const float2 i3 = src[q.ph + size_t(q.pv + 1) * W], i4 = src[q.ph + 1 + size_t(q.pv + 1) * W];
    const float a = float(q.ph + 1) - q.nh, b = q.nh - float(q.ph);
    const float c = float(q.pv + 1) - q.nv, d = q.nv - float(q.pv);
    // separately rounded products and sums (no contraction), in the kernel's
    // order: with motion compensation the power method starts from this
    // interpolation's rounding residue on a constant image, so ||U|| depends
    // on these exact bits
    const float2 aux1 = make_float2(lin2(a, i1.x, b, i2.x), lin2(a, i1.y, b, i2.y));
    const float2 aux2 = make_float2(lin2(a, i3.x, b, i4.x), lin2(a, i3.y, b, i4.y));
    out[k * HW + size_t(q.ver) * W + q.hor] = make_float2(lin2(c, aux1.x, d, aux2.x), lin2(c, aux1.y, d, aux2.y));
  }
}

// initZeroRect (initialize.cl:55-69)
__global__ void k_mc_zero_rect(float2* __restrict__ out, McRect r, int W, int H, int F) {
  const size_t n = size_t(r.l1) * r.l2 * F;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < n; t += size_t(gridDim.x) * blockDim.x) {
    const int i = int(t % r.l1), j = int((t / r.l1) % r.l2), k = int(t / (size_t(r.l1) * r.l2));
    out[k * size_t(H) * W + size_t(r.r1b + i) * W + (r.r2b + j)] = make_float2(0.f, 0.f);
  }
}

// adjointInterpolator (optimizer.cl:880-937): scatter with atomic adds
__global__ void k_mc_scatter(const float2* __restrict__ in, float2* __restrict__ out, const float* __restrict__ xn,
                             const int* __restrict__ xm, McRect r, int W, int H, int F, int* __restrict__ status) {
  const size_t n = size_t(r.l1) * r.l2 * F;
  const size_t HW = size_t(H) * W;
  float* o = reinterpret_cast<float*>(out);
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < n; t += size_t(gridDim.x) * blockDim.x) {
    const int i = int(t % r.l1), j = int((t / r.l1) % r.l2), k = int(t / (size_t(r.l1) * r.l2));
    const McPoint q = mc_point(xn, xm, r, W, H, F, i, j, k);
    if (!q.ok) {
      atomicExch(status, kStatusMotionRange);
      continue;
    }
    const float Wvv = q.nv - float(q.pv), Whh = q.nh - float(q.ph);
    const float2 i0 = in[k * HW + size_t(q.ver) * W + q.hor];
    const size_t p00 = k * HW + size_t(q.pv) * W + q.ph, p01 = p00 + 1, p10 = p00 + W, p11 = p10 + 1;
    atomicAdd(o + 2 * p00, i0.x * (1.f - Whh) * (1.f - Wvv));
    atomicAdd(o + 2 * p01, i0.x * Whh * (1.f - Wvv));
    atomicAdd(o + 2 * p10, i0.x * (1.f - Whh) * Wvv);
    atomicAdd(o + 2 * p11, i0.x * Whh * Wvv);
    atomicAdd(o + 2 * p00 + 1, i0.y * (1.f - Whh) * (1.f - Wvv));
    atomicAdd(o + 2 * p01 + 1, i0.y * Whh * (1.f - Wvv));
    atomicAdd(o + 2 * p10 + 1, i0.y * (1.f - Whh) * Wvv);
    atomicAdd(o + 2 * p11 + 1, i0.y * Whh * Wvv);
  }
}

// g = tTVadj(normalise(D x_w)) (temporalTV.cl:78-107 sign: u_{f+1} - u_f) and the
// objective's partial sums of |u|^2 and Re<u, d> per (frame, 8-column tile),
// the slots the forward column pass fills in the plain form.  grid (W/8, F)
__global__ void __launch_bounds__(128) k_mc_tv(const float2* __restrict__ xw, const NestaDevState* __restrict__ st,
                                               float2* __restrict__ g, double* __restrict__ part_tv, int W, int H,
                                               int F) {
  __shared__ double sred[4];
  const int f = blockIdx.y, w0 = blockIdx.x * 8, t = threadIdx.x;
  const size_t N = size_t(W) * H;
  const float2* x0 = xw + size_t(f) * N;
  const float2* xm = xw + size_t((f + F - 1) % F) * N;
  const float2* xp = xw + size_t((f + 1) % F) * N;
  const float inv_mu = 1.0f / st->mu;
  float su2 = 0.f, sud = 0.f;
  for (int q = t; q < 8 * H; q += 128) {
    const size_t p = size_t(q / 8) * W + w0 + (q % 8);
    const float2 a = x0[p];
    const float2 d0 = csub(a, xm[p]);
    const float2 u0 = tv_normalize(d0, inv_mu);
    const float2 u1 = tv_normalize(csub(xp[p], a), inv_mu);
    su2 = fmaf(u0.x, u0.x, fmaf(u0.y, u0.y, su2));
    sud = fmaf(u0.x, d0.x, fmaf(u0.y, d0.y, sud));
    g[size_t(f) * N + p] = csub(u1, u0);
  }
  const double t1 = block_sum<128>(double(su2), sred);
  const double t2 = block_sum<128>(double(sud), sred);
  if (t == 0) {
    const int slot = f * gridDim.x + blockIdx.x;
    part_tv[2 * slot] = t1;
    part_tv[2 * slot + 1] = t2;
  }
}

// the power method's vector operations
__global__ void k_fill(float2* __restrict__ v, size_t n, float2 value) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) v[i] = value;
}
__global__ void k_scale2(float2* __restrict__ v, size_t n, float s) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float2 a = v[i];
    v[i] = make_float2(a.x * s, a.y * s);
  }
}
// complexType(drand48(), 0) in element order (NestaUp.cpp:369-385): draw i+1 after x0
__global__ void k_fill_drand48(float2* __restrict__ v, size_t n, unsigned long long x0) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    // jump x0 by i+1 steps: X -> a X + c (mod 2^48)
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
    const unsigned long long X = (ra * x0 + rc) & mask;
    v[i] = make_float2(__double2float_rn(double(X) * 0x1p-48), 0.f);
  }
}
// sum of |v|^2 and of |Re| + |Im| in FP64: per-block partials in fixed slots
__global__ void __launch_bounds__(kNT) k_sums(const float2* __restrict__ v, size_t n, double* __restrict__ part) {
  __shared__ double sred[kNT / 32];
  double s2 = 0.0, s1 = 0.0;
  for (size_t i = blockIdx.x * size_t(kNT) + threadIdx.x; i < n; i += size_t(gridDim.x) * kNT) {
    const float2 a = v[i];
    s2 += double(a.x) * a.x + double(a.y) * a.y;
    s1 += double(fabsf(a.x)) + double(fabsf(a.y));
  }
  s2 = block_sum<kNT>(s2, sred);
  s1 = block_sum<kNT>(s1, sred);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s2;
    part[2 * blockIdx.x + 1] = s1;
  }
}
__global__ void k_sums_final(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s2 = 0.0, s1 = 0.0;
    for (int b = 0; b < nblk; ++b) {
      s2 += part[2 * b];
      s1 += part[2 * b + 1];
    }
    out[0] = s2;
    out[1] = s1;
  }
}
__global__ void k_set_normest(NestaDevState* st, float e, int iters) {
  st->normU = e;
  st->normest_iters = iters;
  st->ne_done = 1;
}

int grid1(gbn_ctx* ctx, size_t n) { return int(std::min<size_t>((n + kNT - 1) / kNT, size_t(ctx->nsm) * 8)); }

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int motion_set(gbn_problem* P, const float* xn, const int* xmesh, const int* bb) {
  if (!xn && !xmesh && !bb) {
    P->mc_on = false;
    return GBN_OK;
  }
  if (!xn || !xmesh || !bb) return set_error(GBN_ERR_INVALID, "motion compensation needs xn, the mesh and the bounding box");
  const McRect r = mc_rect(P->W, P->H, bb);
  if (r.l1 <= 0 || r.l2 <= 0 || r.r1b < 0 || r.r2b < 0 || r.r1b + r.l1 > P->H || r.r2b + r.l2 > P->W)
    return set_error(GBN_ERR_INVALID, "motion compensation: bounding box plus margins leaves the image");
  const size_t X = size_t(P->W) * P->H * P->F;
  if (!P->mc_xw) {
    cudaError_t e = cudaMalloc(&P->mc_xw, X * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&P->mc_g, X * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&P->mc_gm, X * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&P->mc_part, 2 * 1024 * sizeof(double) + 2 * sizeof(double));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(GBN_ERR_NOMEM, "motion compensation workspace allocation failed");
    }
  }
  P->mc_xn = xn;
  P->mc_xmesh = xmesh;
  std::memcpy(P->mc_bb, bb, sizeof(P->mc_bb));
  P->mc_on = true;
  return GBN_OK;
}

namespace {

// out = M in (copy, then the interpolator over the rectangle)
int mc_apply(gbn_ctx* ctx, gbn_problem* P, const float2* in, float2* out, cudaStream_t s) {
  const size_t X = size_t(P->W) * P->H * P->F;
  const McRect r = mc_rect(P->W, P->H, P->mc_bb);
  cudaError_t e = cudaMemcpyAsync(out, in, X * sizeof(float2), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "motion compensation copy");
  k_mc_warp<<<grid1(ctx, size_t(r.l1) * r.l2 * P->F), kNT, 0, s>>>(in, out, P->mc_xn, P->mc_xmesh, r, P->W, P->H, P->F,
                                                                    &P->st->status);
  ctx->launches += 1;
  return GBN_OK;
}

// out = M^T in (copy, zero the rectangle, scatter)
int mc_adjoint(gbn_ctx* ctx, gbn_problem* P, const float2* in, float2* out, cudaStream_t s) {
  const size_t X = size_t(P->W) * P->H * P->F;
  const McRect r = mc_rect(P->W, P->H, P->mc_bb);
  cudaError_t e = cudaMemcpyAsync(out, in, X * sizeof(float2), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "motion compensation copy");
  const int g = grid1(ctx, size_t(r.l1) * r.l2 * P->F);
  k_mc_zero_rect<<<g, kNT, 0, s>>>(out, r, P->W, P->H, P->F);
  k_mc_scatter<<<g, kNT, 0, s>>>(in, out, P->mc_xn, P->mc_xmesh, r, P->W, P->H, P->F, &P->st->status);
  ctx->launches += 2;
  return GBN_OK;
}

// (sum |v|^2, sum |Re| + |Im|) on the host (synchronises s)
int sums(gbn_ctx* ctx, gbn_problem* P, const float2* v, double out[2], cudaStream_t s) {
  const size_t X = size_t(P->W) * P->H * P->F;
  const int nblk = std::min(1024, grid1(ctx, X));
  k_sums<<<nblk, kNT, 0, s>>>(v, X, P->mc_part);
  k_sums_final<<<1, 32, 0, s>>>(P->mc_part, nblk, P->mc_part + 2 * 1024);
  ctx->launches += 2;
  cudaError_t e = cudaMemcpyAsync(out, P->mc_part + 2 * 1024, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? GBN_OK : cuda_status(e, "power method norms");
}

// myNormest (NestaUp.cpp:291-439) with U = tTV M, U^T = M^T tTVadj; float
// scalars as the reference, norms reduced in FP64
int mc_normest(gbn_ctx* ctx, gbn_problem* P, cudaStream_t s) {
  const int W = P->W, H = P->H, F = P->F;
  const size_t X = size_t(W) * H * F;
  float2 *x = P->mc_gm, *Sx = P->mc_g, *tmp = P->mc_xw;
  const float tol = 1e-3f;
  double sm[2];
  int rc;
  k_fill<<<grid1(ctx, X), kNT, 0, s>>>(x, X, make_float2(1.f, 0.f));
  ctx->launches += 1;
  if ((rc = sums(ctx, P, x, sm, s)) != GBN_OK) return rc;
  float e = float(std::sqrt(sm[0]));
  k_scale2<<<grid1(ctx, X), kNT, 0, s>>>(x, X, 1.0f / e);
  ctx->launches += 1;
  float e0 = 0.f;
  int cnt = 0;
  while (std::fabs(e - e0) > tol * e && cnt < 100) {
    e0 = e;
    if ((rc = mc_apply(ctx, P, x, tmp, s)) != GBN_OK) return rc;
    if ((rc = op_ttv(ctx, GBN_TTV_FORWARD, tmp, Sx, W, H, F)) != GBN_OK) return rc;
    if ((rc = sums(ctx, P, Sx, sm, s)) != GBN_OK) return rc;
    if (sm[1] == 0.0) {
      // restart from (drand48(), 0) in element order, as the reference
      k_fill_drand48<<<grid1(ctx, X), kNT, 0, s>>>(Sx, X, ctx->rand48);
      ctx->launches += 1;
      ctx->rand48 = lcg48_apply(lcg48_jump(uint64_t(X)), ctx->rand48);
      if ((rc = sums(ctx, P, Sx, sm, s)) != GBN_OK) return rc;
    }
    e = float(std::sqrt(sm[0]));
    if ((rc = op_ttv(ctx, GBN_TTV_ADJOINT, Sx, tmp, W, H, F)) != GBN_OK) return rc;
    if ((rc = mc_adjoint(ctx, P, tmp, x, s)) != GBN_OK) return rc;
    if ((rc = sums(ctx, P, x, sm, s)) != GBN_OK) return rc;
    const float nx = float(std::sqrt(sm[0]));
    k_scale2<<<grid1(ctx, X), kNT, 0, s>>>(x, X, 1.0f / nx);
    ctx->launches += 1;
    ++cnt;
  }
  k_set_normest<<<1, 1, 0, s>>>(P->st, e, cnt);
  ctx->launches += 1;
  return GBN_OK;
}

}  // namespace

// MotionCompensation (dir = GBN_TTV_FORWARD) or AdjointMotionCompensation
// (GBN_TTV_ADJOINT) of one XData [F][H][W] as a single operator.
int motion_op(gbn_ctx* ctx, int dir, const float2* in, float2* out, const float* xn, const int* xm, const int* bb,
              int W, int H, int F) {
  const McRect r = mc_rect(W, H, bb);
  if (r.l1 <= 0 || r.l2 <= 0 || r.r1b < 0 || r.r2b < 0 || r.r1b + r.l1 > H || r.r2b + r.l2 > W)
    return set_error(GBN_ERR_INVALID, "motion compensation: bounding box plus margins leaves the image");
  void* scr = nullptr;
  int rc = ctx_scratch(ctx, sizeof(int), &scr);
  if (rc != GBN_OK) return rc;
  int* status = static_cast<int*>(scr);
  cudaStream_t s = ctx->stream;
  const size_t X = size_t(W) * H * F;
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, in, X * sizeof(float2), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "motion compensation");
  const int g = grid1(ctx, size_t(r.l1) * r.l2 * F);
  if (dir == GBN_TTV_FORWARD) {
    k_mc_warp<<<g, kNT, 0, s>>>(in, out, xn, xm, r, W, H, F, status);
    ctx->launches += 1;
  } else {
    k_mc_zero_rect<<<g, kNT, 0, s>>>(out, r, W, H, F);
    k_mc_scatter<<<g, kNT, 0, s>>>(in, out, xn, xm, r, W, H, F, status);
    ctx->launches += 2;
  }
  int h = 0;
  if ((e = cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, s)) == cudaSuccess)
    e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "motion compensation");
  if (h) return set_error(GBN_ERR_INVALID, "motion compensation: a mesh point interpolates outside the image");
  return GBN_OK;
}

// The motion-compensated solve of problem P; x_out holds the starting image.
int nesta_run_mc(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params* prm, float2* x_out) {
  const SizeKernels* kh = find_size(P->H);
  const SizeKernels* kw = find_size(P->W);
  const int W = P->W, H = P->H, F = P->F, C = P->C, N = W * H;
  cudaStream_t s = ctx->stream;
  int cpb, k2;
  tuning_for(ctx, W, H, F, C, &cpb, &k2);
  cpb = std::max(1, std::min(cpb, C));
  const dim3 g1(W / kWB, (C + cpb - 1) / cpb, F);
  const long long steps = ((long long)F * H * C + kw->rows_per_cta - 1) / kw->rows_per_cta;
  const int g2 = row_grid(ctx, kw, true, steps, k2);
  const dim3 g3(W / kWB, 2, F);
  FusedArgs a = make_args(P, x_out);
  a.tv_src = P->mc_xw;
  a.grad_ext = P->mc_gm;
  const FusedArgs* tab = P->d_args;
  const BatchMap bm = single_map(F, P->ctl);
  int rc;
  ctx->launches += launch_pre(P, *prm, s);
  ctx->launches += launch_store_args(P->d_args, a, s);
  ctx->launches += launch_group_init(tab, 1, kw->rows_per_cta, P->ctl, s);
  // maxima of x0 and of U x0 = tTV(M x0) (NestaUp.cpp:491, 521-568)
  if ((rc = mc_apply(ctx, P, x_out, P->mc_xw, s)) != GBN_OK) return rc;
  ctx->launches += launch_maxima(ctx, P, x_out, P->mc_xw, s);
  if ((rc = mc_normest(ctx, P, s)) != GBN_OK) return rc;
  ctx->launches += launch_setup(P, s);
  for (unsigned nl = 1; nl <= prm->maxIntIter; ++nl) {
    ctx->launches += launch_outer_begin(ctx, P, int(nl), x_out, s);
    for (unsigned it = 0; it < prm->maxIter; ++it) {
      const float2* xk = (it & 1) ? P->xk1 : P->xk0;
      if ((rc = mc_apply(ctx, P, xk, P->mc_xw, s)) != GBN_OK) return rc;
      k_mc_tv<<<dim3(W / kWB, F), 128, 0, s>>>(P->mc_xw, P->st, P->mc_g, P->part_tv, W, H, F);
      kh->fwd_cols(tab, bm, int(it), cpb, g1, s);
      kw->rows(tab, bm, int(it), true, g2, s);
      if ((rc = mc_adjoint(ctx, P, P->mc_g, P->mc_gm, s)) != GBN_OK) return rc;
      kh->inv_cols(tab, bm, int(it), true, g3, s);
      ctx->launches += 4;
    }
    ctx->launches += launch_outer_end(ctx, P, x_out, s);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBN_OK : cuda_status(e, "motion-compensated nesta launch");
}

}  // namespace gbn
