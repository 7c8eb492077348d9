// GroupwiseRegistration (GroupwiseRegistration.cpp:550-618 with optimizer(),
// groupwiseRegistration/optimizer.cpp): B-spline groupwise registration of the
// frames of a reconstruction, producing the deformed mesh that the
// motion-compensated solve warps with.
//
// The reference runs ~35 kernels over ~40 work arrays, about 2,100 launches per
// gradient-descent iteration (four per control point).  Per quantity, what they
// compute is:
//   xn_d,f(p) = x_d(p) + sum_{a,b} T[d][f][cr(row)+b][cr(col)+a] B(row,b) B(col,a)
//               (bounding-box pixels; x elsewhere)
//   I_w,f     = bilinear(I_f, xn_f)            dx_d,f = bilinear(dI_f/d(col|row), xn_f)
//   V         = var_f I_w [+ smoothness terms of T when sumLambda() != 0]
//   H         = sum over the region of interest of V
//   dH[d][f][k][l] = sum over the 17x17 support of control point (k, l) of
//               ROI (2/F)(I_w - mean) dx_d S(i) S(j)
//   T        -= Wn (dH - mean_f dH),   Wn adapted by evolution()
// The reference's regularisation gradient (gradientRegularization,
// reduction7Dto6D, the reductionsum passes, gradientJointAux) is broadcast
// over frames before it enters dH, so the frame-mean projection of
// updateTransformation removes it: it changes T only by rounding, and is not
// computed here.  The smoothness terms still enter the metric when sumLambda()
// (an int accumulation of the weights, GroupwiseRegistration.cpp:440-442) is
// non-zero, with the reference's pairing of spline factors (optimizer.cl:
// 746-830) and at the transposed pixel (optimizer.cl:138-187).
//
// Here one iteration is four kernels:
//   k_reg_grad    one thread per (d, frame, control point, column offset): the
//                 support sums in the reference's order (auxiliarCost,
//                 cost6DReduction, cost6D)
//   k_reg_update  one thread per (d, frame, control point): the frame mean,
//                 Dif = Wn (dH - mean), T -= Dif (updateTransformation)
//   k_reg_warp    one thread per (bounding-box pixel, frame): xn, the warped
//                 frame, dx, the smoothness terms
//   k_reg_metric  one thread per bounding-box pixel: the frames' mean, V, dy,
//                 per-CTA partial sums of the metric; its last CTA sums the
//                 partials (H, |Dif|) and runs evolution() and stopCondition()
// iterations are enqueued eight at a time; the host reads the stop flag once
// per chunk.  This file is compiled without FMA contraction, so products and
// sums round separately as in the reference's kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.h"

namespace gbn {

namespace {

constexpr int kRegNT = 256;
constexpr int kRegMaxE1 = 4;  // spline orders up to 3
constexpr int kStatusRange = 5;
constexpr int kRegChunk = 8;

struct RegState {
  float Wn, p2, p4, Tdif, Hdif;
  int it;      // iterations completed
  int done;
  int status;
  int nmax;
  int flagW;
  unsigned arrived;  // CTAs of k_reg_metric done this iteration (the last one finishes the iteration)
};

// ---- groupwiseRegistration/bspline.cpp: bsplineN / b1splineN / b2splineN
// (t = 0, 1, 2) of orders 1 to 3, float results of the reference's float and
// double expressions, its constants included ----
float spline_e(int t, float x, int E) {
  if (E == 1) {
    if (t == 0) {
      if (x < 0 && x >= -1) return x + 1;
      if (x < 1 && x >= 0) return 1 - x;
      return 0;
    }
    if (t == 1) return (x < 0 && x >= -1) ? 1.f : ((x < 1 && x >= 0) ? -1.f : 0.f);
    return 0;
  }
  if (E == 2) {
    if (t == 0) {
      if (x < -0.5 && x >= -1.5) return float((4 * std::pow(double(x), 2) + double(12 * x) + 9) / 8);
      if (x < 0.5 && x >= -0.5) return float((-4 * std::pow(double(x), 2) + 3) / 4);
      if (x < 1.5 && x >= 0.5) return float((4 * std::pow(double(x), 2) - double(12 * x) + 9) / 8);
      return 0;
    }
    if (t == 1) {
      if (x < -0.5 && x >= -1.5) return (2 * x + 3) / 2;
      if (x < 0.5 && x >= -0.5) return -2 * x;
      if (x < 1.5 && x >= 0.5) return (42 * x - 3) / 2;
      return 0;
    }
    if (x < -0.5 && x >= -1.5) return 1;
    if (x < 0.5 && x >= -0.5) return -2;
    if (x < 1.5 && x >= 0.5) return 1;
    return 0;
  }
  if (t == 0) {
    const float v = std::fabs(x);
    if (v < 1) return float(0.5 * std::pow(double(v), 3) - std::pow(double(v), 2) + 0.6666);
    if (v >= 1 && v < 2) return (2 - v) * (2 - v) * (2 - v) / 6;
    return 0;
  }
  if (t == 1) {
    if (x <= 1 && x >= 0) return float(1.5 * std::pow(double(x), 2) - double(2 * x));
    if (x >= -1 && x < 0) return float(-1.5 * std::pow(double(x), 2) - double(2 * x));
    if (x > 1 && x < 2) return -(x - 2) * (x - 2) / 2;
    if (x < -1 && x > -2) return (x + 2) * (x + 2) / 2;
    return 0;
  }
  const float v = std::fabs(x);
  if (v < 1) return 3 * v - 2;
  if (v >= 1 && v < 2) return -v + 2;
  return 0;
}

struct RegGeom {
  int N = 0, F = 0, E = 3, Dp = 4, Cp = 0, dp = 0, area = 0, sum_lambda = 0;
  int bb[4] = {0, 0, 0, 0};
  int box0 = 0, box1 = 0;    // bounding box, 0-based inclusive (rows and columns alike)
  int rect0 = 0, rect1 = 0;  // margin rectangle of the interpolators
  std::vector<float> roi;    // [N][N]
  std::vector<int> cr;       // [N] first control point of each pixel (0-based)
  std::vector<float> B;      // [3][N][E+1] spline values at each pixel
  std::vector<float> S;      // [3][dp] spline values over a control point's support
  std::vector<int> sup;      // [Cp] first pixel of each support (0-based)
  float Wn0 = 0;
};

// init() and creabspline() (GroupwiseRegistration.cpp:92-190, creabspline.cpp)
int reg_geometry(int N, int F, const gbn_registration_params* p, RegGeom* g) {
  if (!p) return set_error(GBN_ERR_INVALID, "null registration parameters");
  if (N < 16 || N % 8 != 0) return set_error(GBN_ERR_UNSUPPORTED, "registration: N must be a multiple of 8, >= 16");
  if (F < 3) return set_error(GBN_ERR_UNSUPPORTED, "registration: at least 3 frames (the temporal terms use f-2)");
  if (p->E < 1 || p->E > 3) return set_error(GBN_ERR_UNSUPPORTED, "registration: spline orders 1 to 3");
  if (p->Dp[0] != p->Dp[1] || p->Dp[0] < 1)
    return set_error(GBN_ERR_UNSUPPORTED, "registration: equal positive control spacing in both directions only");
  if (p->radius <= 0)
    return set_error(GBN_ERR_UNSUPPORTED,
                     "registration: circular region of interest only (radius > 0); the reference's whole-box "
                     "mode stores a one-pixel bounding box");
  if (p->nmax < 1) return set_error(GBN_ERR_INVALID, "registration: nmax must be >= 1");
  g->N = N;
  g->F = F;
  g->E = p->E;
  g->Dp = p->Dp[0];
  // setMask (GroupwiseRegistration.cpp:486-531)
  const int radius2 = int(std::pow(p->radius, 2));
  const float center = float(N + 1) / 2;
  g->roi.assign(size_t(N) * N, 0.f);
  int mn = N, mx = -1, mnr = N, mxr = -1;
  for (int col = 0; col < N; ++col)
    for (int row = 0; row < N; ++row) {
      const float Cv = float(std::pow(1 - center + row, 2)), Dv = float(std::pow(1 - center + col, 2));
      if ((Cv + Dv) <= radius2) {
        g->roi[size_t(row) * N + col] = 1.f;
        mn = std::min(mn, col);
        mx = std::max(mx, col);
        mnr = std::min(mnr, row);
        mxr = std::max(mxr, row);
        g->area++;
      }
    }
  if (g->area == 0) return set_error(GBN_ERR_INVALID, "registration: empty region of interest");
  g->bb[0] = mn + 1;
  g->bb[1] = mnr + 1;
  g->bb[2] = mx + 1;
  g->bb[3] = mxr + 1;
  if (g->bb[0] != g->bb[1] || g->bb[2] != g->bb[3])
    return set_error(GBN_ERR_UNSUPPORTED, "registration: region of interest not symmetric");
  g->box0 = g->bb[0] - 1;
  g->box1 = g->bb[2] - 1;
  const int m = N / 40;
  g->rect0 = g->bb[1] - m - 2;
  g->rect1 = g->bb[3] + m;
  const float c = float(g->bb[0] + g->bb[2]) / 2;
  const float rp = float((p->E + 1) * g->Dp / 2);
  const int C0 = int(std::floor((std::fabs(c - float(g->bb[0])) + rp) / g->Dp));
  const int C1 = int(std::floor((std::fabs(c - float(g->bb[2])) + rp) / g->Dp));
  g->Cp = C0 + C1 + 1;
  g->dp = 2 * int(std::ceil(rp)) + 1;
  const int E1 = p->E + 1;
  // per-pixel control ranges and spline values (coef, BBAux)
  std::vector<int> kmin(N);
  // creabspline.cpp: odd orders floor((x - c) / Dp) - (E - 1) / 2, even orders
  // round((x - c) / Dp) - E / 2
  for (int q = 0; q < N; ++q) {
    const float u = (float(q + 1) - c) / g->Dp;
    kmin[q] = (p->E % 2) ? int(std::floor(u)) - (p->E - 1) / 2 : int(std::round(u)) - p->E / 2;
  }
  g->cr.resize(N);
  for (int q = 0; q < N; ++q) g->cr[q] = kmin[q] - kmin[g->bb[0]];
  g->B.assign(size_t(3) * N * E1, 0.f);
  for (int q = 0; q < N; ++q)
    for (int s = 0; s < E1; ++s) {
      const float arg = ((float(q + 1) - c) / float(g->Dp)) - float(kmin[q] + s);
      for (int t = 0; t < 3; ++t) g->B[(size_t(t) * N + q) * E1 + s] = spline_e(t, arg, g->E);
    }
  // control points and supports (ControlPointsLocation, coefg, BBAux1)
  g->sup.resize(g->Cp);
  std::vector<float> pu(g->Cp);
  for (int n = 0; n < g->Cp; ++n) {
    pu[n] = c + float(g->Dp * (n - C0));
    g->sup[n] = int(std::ceil(pu[n] - std::ceil(rp))) - 1;
  }
  if (g->dp > kRegNT) return set_error(GBN_ERR_UNSUPPORTED, "registration: control spacing too large");
  if (g->sup.front() < 0 || g->sup.back() + g->dp > N)
    return set_error(GBN_ERR_UNSUPPORTED, "registration: the control grid's supports leave the image");
  for (int q = g->box0; q <= g->box1; ++q)
    if (g->cr[q] < 0 || g->cr[q] + E1 > g->Cp)
      return set_error(GBN_ERR_UNSUPPORTED, "registration: a box pixel's control points leave the grid");
  g->S.assign(size_t(3) * g->dp, 0.f);
  for (int s = 0; s < g->dp; ++s) {
    const float arg = (float(g->sup[0] + 1 + s) - pu[0]) / float(g->Dp);
    for (int t = 0; t < 3; ++t) g->S[size_t(t) * g->dp + s] = spline_e(t, arg, g->E);
  }
  for (int n = 1; n < g->Cp; ++n)
    for (int s = 0; s < g->dp; ++s) {
      const float arg = (float(g->sup[n] + 1 + s) - pu[n]) / float(g->Dp);
      if (spline_e(0, arg, g->E) != g->S[s])
        return set_error(GBN_ERR_UNSUPPORTED, "registration: control supports not uniform");
    }
  if (g->rect0 < 0 || g->rect1 > N - 1) return set_error(GBN_ERR_UNSUPPORTED, "registration: margin leaves the image");
  int acc = 0;
  for (int i = 0; i < 4; ++i) acc = int(float(acc) + p->lambda[i]);
  g->sum_lambda = acc;
  g->Wn0 = p->W / g->area;
  return GBN_OK;
}

// ---- device ----
__global__ void k_reg_absmax(const float2* __restrict__ x, size_t n, unsigned* __restrict__ maxbits) {
  float m = 0.f;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float2 v = x[i];
    m = fmaxf(m, float(sqrt(double(v.x) * v.x + double(v.y) * v.y)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits, __float_as_uint(m));  // non-negative: bit order = value order
}

// DataNormalization (initialize.cl:87-102): I = (500 / max) |x|
__global__ void k_reg_normalize(const float2* __restrict__ x, const unsigned* __restrict__ maxbits, float* __restrict__ I,
                                size_t n) {
  const float factor = 500.f / __uint_as_float(*maxbits);
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float2 v = x[i];
    I[i] = factor * float(sqrt(double(v.x) * v.x + double(v.y) * v.y));
  }
}

// gradient (optimizer.cl:189-234): central differences, one-sided at the borders
__global__ void k_reg_imgrad(const float* __restrict__ I, float* __restrict__ d1, float* __restrict__ d2, int N, int F) {
  const size_t n = size_t(N) * N * F;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const int col = int(i % N), row = int((i / N) % N);
    const float* f = I + (i - size_t(row) * N - col);
    const size_t p = size_t(row) * N + col;
    d1[i] = col == 0 ? f[p + 1] - f[p] : col == N - 1 ? f[p] - f[p - 1] : (f[p + 1] - f[p - 1]) / 2;
    d2[i] = row == 0 ? f[p + N] - f[p] : row == N - 1 ? f[p] - f[p - N] : (f[p + N] - f[p - N]) / 2;
  }
}

struct RegArgs {
  int N, F, Cp, dp, box0, box1, E1, smooth, warp;
  float lam[4];
  float fac;  // 2 / F (GradientMetric.cpp:72)
  float Dp;
  const float* I;
  const float* d1;
  const float* d2;
  const float* roi;
  const int* cr;
  const float* B;  // [3][N][E1]
  const float* S;  // [3][dp]
  const int* sup;
  float* T;    // [2][F][Cp][Cp]
  float* dH;   // [2][F][Cp][Cp]
  float* Dif;  // [2][F][Cp][Cp]
  float* xn;   // [2][F][N][N]
  float* Iw;   // [F][N][N] (box pixels)
  float* dy;   // [F][N][N] (box pixels)
  float* dx;   // [2][F][N][N] (box pixels)
  float* sterm;  // [F][2][7][box pixels] weighted squared smoothness terms
  float* H;    // [nmax + 1]
  float* part_h;  // per-CTA partial sums of the metric (k_reg_metric)
  float* part_d;  // per-CTA partial sums of Dif^2 (k_reg_update)
  RegState* st;
};

// bilinear interpolation of img [N][N] at 1-based (xh, xv), as optimizer.cl's
// interpolator and gradientInterpolator round it; false when a corner leaves the image
__device__ __forceinline__ bool reg_bilinear(const float* __restrict__ img, int N, float xh, float xv, float* out) {
  const float nh = xh - 1, nv = xv - 1;
  const int ph = int(floorf(nh)), pv = int(floorf(nv));
  if (ph < 0 || pv < 0 || ph + 1 >= N || pv + 1 >= N) return false;
  const float i1 = img[ph + size_t(pv) * N], i2 = img[ph + 1 + size_t(pv) * N];
  const float i3 = img[ph + size_t(pv + 1) * N], i4 = img[ph + 1 + size_t(pv + 1) * N];
  const float a = float(ph + 1) - nh, b = nh - float(ph), cc = float(pv + 1) - nv, d = nv - float(pv);
  const float aux1 = a * i1 + b * i2, aux2 = a * i3 + b * i4;
  *out = cc * aux1 + d * aux2;
  return true;
}

// one thread per (bounding-box pixel, frame): xn, the warped frame, dx; the
// smoothness terms of that frame when enabled (7 per direction d, each already
// weighted and squared as sumLambdaMetric adds it)
__global__ void __launch_bounds__(kRegNT) k_reg_warp(RegArgs a) {
  if (a.st->done) return;
  const int L = a.box1 - a.box0 + 1;
  const int q = blockIdx.x * kRegNT + threadIdx.x;
  if (q >= L * L * a.F) return;
  const int pix = q % (L * L), f = q / (L * L);
  const int row = a.box0 + pix / L, col = a.box0 + pix % L;
  const int N = a.N, F = a.F, Cp = a.Cp, E1 = a.E1;
  const size_t NN = size_t(N) * N, p = size_t(row) * N + col;
  const int r0 = a.cr[row], c0 = a.cr[col];
  float br[kRegMaxE1], bc[kRegMaxE1];
#pragma unroll
  for (int s = 0; s < kRegMaxE1; ++s) {
    br[s] = s < E1 ? a.B[size_t(row) * E1 + s] : 0.f;
    bc[s] = s < E1 ? a.B[size_t(col) * E1 + s] : 0.f;
  }
  float u[2];
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    const float* Tf = a.T + (size_t(d) * F + f) * Cp * Cp;
    float acc = 0.f;
    for (int aa = 0; aa < E1; ++aa)    // column spline outer, row spline inner (Deformation)
      for (int b = 0; b < E1; ++b) acc = acc + Tf[(r0 + b) * Cp + c0 + aa] * (br[b] * bc[aa]);
    u[d] = acc;
  }
  const float xh = u[0] + float(col + 1), xv = u[1] + float(row + 1);
  a.xn[size_t(f) * NN + p] = xh;
  a.xn[(size_t(F) + f) * NN + p] = xv;
  float iw, g1, g2;
  bool ok = reg_bilinear(a.d1 + f * NN, N, xh, xv, &g1) && reg_bilinear(a.d2 + f * NN, N, xh, xv, &g2);
  if (a.warp)
    ok = ok && reg_bilinear(a.I + f * NN, N, xh, xv, &iw);
  else
    iw = a.I[f * NN + p];
  if (!ok) {
    atomicExch(&a.st->status, kStatusRange);
    iw = a.I[f * NN + p];
    g1 = g2 = 0.f;
  }
  a.dx[size_t(f) * NN + p] = g1;
  a.dx[(size_t(F) + f) * NN + p] = g2;
  a.Iw[f * NN + p] = iw;
  if (!a.smooth) return;
  // smoothness terms (Regularization): at the pixel with row `row` and column
  // `col` the reference pairs the row-direction control offset n with the
  // column pixel's spline and the column offset m with the row pixel's
  const float* B0 = a.B;
  const float* B1 = a.B + size_t(N) * E1;
  const float* B2 = a.B + 2 * size_t(N) * E1;
  const float Dp = a.Dp, Dp2 = a.Dp * a.Dp;
  const float l0 = a.lam[0], l1 = a.lam[1], l2 = a.lam[2], l3 = a.lam[3];
  for (int d = 0; d < 2; ++d) {
    const float* T0 = a.T + (size_t(d) * F + f) * Cp * Cp;
    const float* T1 = a.T + (size_t(d) * F + (f + F - 1) % F) * Cp * Cp;
    const float* T2 = a.T + (size_t(d) * F + (f + F - 2) % F) * Cp * Cp;
    float ax0 = 0.f, ax1 = 0.f, bx0 = 0.f, bx1 = 0.f, axy = 0.f, at = 0.f, at2 = 0.f;
    for (int mm = 0; mm < E1; ++mm)
      for (int n = 0; n < E1; ++n) {
        const float t0 = T0[(r0 + n) * Cp + c0 + mm];
        const float cB = B0[size_t(col) * E1 + n], cB1 = B1[size_t(col) * E1 + n], cB2 = B2[size_t(col) * E1 + n];
        const float rB = B0[size_t(row) * E1 + mm], rB1 = B1[size_t(row) * E1 + mm], rB2 = B2[size_t(row) * E1 + mm];
        ax0 = ax0 + t0 * (Dp * (cB * rB1));
        bx0 = bx0 + t0 * (Dp2 * (cB * rB2));
        ax1 = ax1 + t0 * (Dp * (cB1 * rB));
        bx1 = bx1 + t0 * (Dp2 * (cB2 * rB));
      }
    for (int mm = 0; mm < E1; ++mm)
      for (int n = 0; n < E1; ++n)
        axy = axy + T0[(r0 + n) * Cp + c0 + mm] * (Dp2 * (B1[size_t(col) * E1 + n] * B1[size_t(row) * E1 + mm]));
    for (int mm = 0; mm < E1; ++mm)
      for (int n = 0; n < E1; ++n) {
        const int ti = (r0 + n) * Cp + c0 + mm;
        const float bb = B0[size_t(col) * E1 + n] * B0[size_t(row) * E1 + mm];
        at = at + (T0[ti] - T1[ti]) * bb;
        at2 = float(double(at2) + (double(T0[ti]) - 2.0 * double(T1[ti]) + double(T2[ti])) * double(bb));
      }
    if (d == 0) ax0 = ax0 + 1.f;
    else ax1 = ax1 + 1.f;
    float* o = a.sterm + (size_t(f) * 2 + d) * 7 * L * L + pix;
    const size_t st = size_t(L) * L;
    o[0 * st] = (l1 * 2) * (axy * axy);
    o[1 * st] = l3 * (at2 * at2);
    o[2 * st] = l2 * (at * at);
    o[3 * st] = l0 * (ax0 * ax0);
    o[4 * st] = l1 * (bx0 * bx0);
    o[5 * st] = l0 * (ax1 * ax1);
    o[6 * st] = l1 * (bx1 * bx1);
  }
}

// sum of one float per thread of a kRegNT-thread CTA in a fixed order (warp
// shuffles, then the warps in order); the result in thread 0
__device__ __forceinline__ float reg_block_sum(float v, float* sw) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x == 0)
    for (int w = 0; w < kRegNT / 32; ++w) t = t + sw[w];
  return t;
}

// one thread per bounding-box pixel: the frames' mean, V, dy (metric,
// gradientMetric); with the smoothness terms, V at this pixel gains the
// smoothness sum of the transposed pixel in sumLambdaMetric's order (the
// reference adds each pixel's sum at the transposed position); the CTA's
// partial sum of V over the region of interest
__device__ void reg_finish(RegArgs& a, int it, int nh, int nd, float et, float eh, float* sw);

__global__ void __launch_bounds__(kRegNT) k_reg_metric(RegArgs a, int it, int nd, float et, float eh) {
  if (a.st->done) return;
  __shared__ float sw[kRegNT / 32];
  const int L = a.box1 - a.box0 + 1;
  const int pix = blockIdx.x * kRegNT + threadIdx.x;
  float h = 0.f;
  if (pix < L * L) {
    const int row = a.box0 + pix / L, col = a.box0 + pix % L;
    const int N = a.N, F = a.F;
    const size_t NN = size_t(N) * N, p = size_t(row) * N + col;
    float sum = 0.f;
    for (int f = 0; f < F; ++f) sum = sum + a.Iw[f * NN + p];
    const float mean = sum / F;
    float V = 0.f;
    for (int f = 0; f < F; ++f) {
      const float dl = a.Iw[f * NN + p] - mean;
      V = V + dl * dl;
      a.dy[f * NN + p] = dl * a.fac;
    }
    V = V / F;
    if (a.smooth) {
      const size_t st = size_t(L) * L;
      const int pt = (col - a.box0) * L + (row - a.box0);  // the transposed pixel
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f;
      for (int f = 0; f < F; ++f)
        for (int d = 0; d < 2; ++d) {
          const float* o = a.sterm + (size_t(f) * 2 + d) * 7 * st + pt;
          s2 = s2 + o[0 * st];
          s3 = s3 + o[1 * st];
          s4 = s4 + o[2 * st];
          s0 = s0 + o[3 * st];
          s1 = s1 + o[4 * st];
          s0 = s0 + o[5 * st];
          s1 = s1 + o[6 * st];
        }
      V = V + ((((s0 + s1) + s2) + s3) + s4);
    }
    h = V * a.roi[p];
  }
  const float t = reg_block_sum(h, sw);
  // the last CTA to finish reduces every CTA's partial sum (fixed order) and
  // runs evolution(): no separate launch
  __shared__ bool last;
  if (threadIdx.x == 0) {
    a.part_h[blockIdx.x] = t;
    __threadfence();
    last = atomicAdd(&a.st->arrived, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  reg_finish(a, it, int(gridDim.x), nd, et, eh, sw);
}

// dH for (d, frame, control point) in the reference's order (auxiliarCost,
// then cost6DReduction over the row offsets i of each column offset j, then
// cost6D over j): one thread per column offset sums its i in order, one
// thread per group then sums the column sums in order.  The region of interest
// is read at the pixel itself: the reference reads it at the transposed
// pixel, and the centred circle is symmetric.  Terms outside it add an exact
// zero (dy and dx are zero outside the bounding box), so every term is
// computed, without a branch.  DP > 0: the support width at compile time.
template <int DP>
__global__ void __launch_bounds__(kRegNT) k_reg_grad(RegArgs a) {
  if (a.st->done) return;
  __shared__ float cs[kRegNT];
  const int Cp = a.Cp, F = a.F, N = a.N, dp = DP > 0 ? DP : a.dp;
  const int gpc = kRegNT / dp;  // groups per CTA
  const int t = threadIdx.x, gl = t / dp, j = t % dp;
  const int grp = blockIdx.x * gpc + gl;
  const bool live = gl < gpc && grp < 2 * F * Cp * Cp;
  if (live) {
    const int lc = grp % Cp, kr = (grp / Cp) % Cp, f = (grp / (Cp * Cp)) % F, d = grp / (Cp * Cp * F);
    const size_t NN = size_t(N) * N;
    const int R = a.sup[kr], C = a.sup[lc];
    const float* dyf = a.dy + f * NN + C + j;
    const float* dxf = a.dx + (size_t(d) * F + f) * NN + C + j;
    const float* roi = a.roi + C + j;
    const float Sj = a.S[j];
    float c = 0.f;
    if constexpr (DP > 0) {
      float v[DP], m[DP];
#pragma unroll
      for (int i = 0; i < DP; ++i) {
        const size_t p = size_t(R + i) * N;
        v[i] = dyf[p] * dxf[p];
        m[i] = roi[p];
      }
#pragma unroll
      for (int i = 0; i < DP; ++i) c = c + (v[i] * (a.S[i] * Sj)) * m[i];
    } else {
      for (int i = 0; i < dp; ++i) {
        const size_t p = size_t(R + i) * N;
        c = c + ((dyf[p] * dxf[p]) * (a.S[i] * Sj)) * roi[p];
      }
    }
    cs[t] = c;
  }
  __syncthreads();
  if (live && j == 0) {
    float acc = 0.f;
    for (int jj = 0; jj < dp; ++jj) acc = acc + cs[gl * dp + jj];
    a.dH[grp] = acc;
  }
}

// updateTransformation (optimizer.cl:519-563): T -= Wn (dH - mean_f dH), one
// thread per (d, frame, control point), each summing its control point's
// frames in order for the mean; the CTA's partial sum of Dif^2
__global__ void __launch_bounds__(kRegNT) k_reg_update(RegArgs a) {
  if (a.st->done) return;
  __shared__ float sw[kRegNT / 32];
  const int Cp = a.Cp, F = a.F, CC = Cp * Cp;
  const int q = blockIdx.x * kRegNT + threadIdx.x;
  float dd = 0.f;
  if (q < 2 * F * CC) {
    const int cp = q % CC, d = q / (CC * F);
    float sum = 0.f;
    for (int f = 0; f < F; ++f) sum = sum + a.dH[(size_t(d) * F + f) * CC + cp];
    const float mean = sum / F;
    const float dif = a.st->Wn * (a.dH[q] - mean);
    a.Dif[q] = dif;
    a.T[q] = a.T[q] - dif;
    dd = dif * dif;
  }
  const float t = reg_block_sum(dd, sw);
  if (threadIdx.x == 0) a.part_d[blockIdx.x] = t;
}

// H and |Dif| from the partial sums of k_reg_metric and k_reg_update (fixed
// order), evolution() and stopCondition() (GroupwiseRegistration.cpp:451-478,
// 533-545); run by the last CTA of k_reg_metric.  it == 0: the unregistered
// metric and the thresholds.
__device__ void reg_finish(RegArgs& a, int it, int nh, int nd, float et, float eh, float* sw) {
  RegState* st = a.st;
  __syncthreads();  // sw reuse
  float h = 0.f, dd = 0.f;
  for (int q = threadIdx.x; q < nh; q += kRegNT) h = h + __ldcg(a.part_h + q);
  if (it > 0)
    for (int q = threadIdx.x; q < nd; q += kRegNT) dd = dd + __ldcg(a.part_d + q);
  const float H = reg_block_sum(h, sw);
  __syncthreads();
  const float D = reg_block_sum(dd, sw);
  if (threadIdx.x != 0) return;
  st->arrived = 0;
  a.H[it] = H;
  if (it == 0) {
    st->p2 = et * float(a.F * 2);
    st->p4 = H * eh;
    return;
  }
  const float Tdif = sqrtf(D);
  const float Hdif = a.H[it - 1] - H;
  if (st->flagW) st->Wn = Hdif > 0 ? float(double(st->Wn) * 1.2) : st->Wn / 2;
  st->Tdif = Tdif;
  st->Hdif = Hdif;
  st->it = it;
  if (it == st->nmax || (Tdif < st->p2 && Hdif < st->p4)) st->done = 1;
}

__global__ void k_reg_mesh(int* __restrict__ xmesh, float* __restrict__ xn, int N, int F) {
  const size_t NN = size_t(N) * N;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < NN; i += size_t(gridDim.x) * blockDim.x) {
    // ArgumentsMotionCompensation::xData: [2][N][N] with the first index the
    // column (x[i + j N] = j + 1 in plane 0, i + 1 in plane 1)
    const int a0 = int(i % N), b0 = int(i / N);
    if (xmesh) {
      xmesh[i] = b0 + 1;
      xmesh[NN + i] = a0 + 1;
    }
    const int row = b0, col = a0;
    for (int f = 0; f < F; ++f) {
      xn[size_t(f) * NN + i] = float(col + 1);
      xn[(size_t(F) + f) * NN + i] = float(row + 1);
    }
  }
}


// bump allocation of the work arrays in one block (256-byte aligned); a pass
// with a null base sizes the block
struct Carve {
  char* base;
  size_t off;
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + off);
    off += std::max<size_t>(n, 1) * sizeof(T);
    return p;
  }
};

}  // namespace

int registration_info(int N, int F, const gbn_registration_params* p, gbn_registration_info* info) {
  RegGeom g;
  const int rc = reg_geometry(N, F, p, &g);
  if (rc != GBN_OK) return rc;
  if (info) {
    info->cp = g.Cp;
    std::memcpy(info->bound_box, g.bb, sizeof(g.bb));
    info->area = g.area;
  }
  return GBN_OK;
}

int registration_run(gbn_ctx* ctx, const float2* images, int N, int F, const gbn_registration_params* prm,
                     const float* T_init, float* T_out, float* xn_out, int* xmesh_out, float* h_H,
                     gbn_registration_stats* stats) {
  RegGeom g;
  int rc = reg_geometry(N, F, prm, &g);
  if (rc != GBN_OK) return rc;
  cudaStream_t s = ctx->stream;
  const size_t NN = size_t(N) * N, X = NN * F, nT = size_t(2) * F * g.Cp * g.Cp;
  // all work arrays in one grow-only block of the context (no allocation
  // after the first call of a size)
  RegArgs a{};
  float *I, *d1, *d2, *roi, *B, *S, *dH, *Dif, *Iw, *dy, *dx, *H, *part_h, *part_d, *sterm = nullptr;
  int *cr, *sup;
  unsigned* maxbits;
  RegState* st;
  const size_t L2 = size_t(g.box1 - g.box0 + 1) * (g.box1 - g.box0 + 1);
  auto plan = [&](Carve& c) {
    I = c.take<float>(X);
    d1 = c.take<float>(X);
    d2 = c.take<float>(X);
    roi = c.take<float>(NN);
    B = c.take<float>(g.B.size());
    S = c.take<float>(g.S.size());
    dH = c.take<float>(nT);
    Dif = c.take<float>(nT);
    Iw = c.take<float>(X);
    dy = c.take<float>(X);
    dx = c.take<float>(2 * X);
    H = c.take<float>(size_t(prm->nmax) + 1);
    part_h = c.take<float>(L2 / kRegNT + 1);
    part_d = c.take<float>(nT / kRegNT + 1);
    sterm = g.sum_lambda != 0 ? c.take<float>(size_t(F) * 14 * L2) : nullptr;
    cr = c.take<int>(size_t(N));
    sup = c.take<int>(size_t(g.Cp));
    maxbits = c.take<unsigned>(1);
    st = c.take<RegState>(1);
  };
  Carve sizer{nullptr, 0};
  plan(sizer);
  void* block = nullptr;
  if ((rc = ctx_scratch(ctx, sizer.off, &block)) != GBN_OK) return rc;
  Carve carver{static_cast<char*>(block), 0};
  plan(carver);
  RegState h0{};
  h0.Wn = g.Wn0;
  h0.nmax = prm->nmax;
  h0.flagW = prm->flagW ? 1 : 0;
  cudaError_t e = cudaMemcpyAsync(roi, g.roi.data(), NN * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B, g.B.data(), g.B.size() * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S, g.S.data(), g.S.size() * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cr, g.cr.data(), N * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sup, g.sup.data(), g.Cp * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st, &h0, sizeof(h0), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(maxbits, 0, sizeof(unsigned), s);
  // the gradient reads dy and dx over whole supports, outside the bounding box
  // times a zero mask: zero there
  if (e == cudaSuccess) e = cudaMemsetAsync(dy, 0, X * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dx, 0, 2 * X * sizeof(float), s);
  // T_init may be T_out itself (a continuation in place)
  if (e == cudaSuccess && T_init != T_out)
    e = T_init ? cudaMemcpyAsync(T_out, T_init, nT * sizeof(float), cudaMemcpyDeviceToDevice, s)
               : cudaMemsetAsync(T_out, 0, nT * sizeof(float), s);
  if (e != cudaSuccess) return cuda_status(e, "registration setup");
  const int gx = int(std::min<size_t>((X + kRegNT - 1) / kRegNT, size_t(ctx->nsm) * 8));
  k_reg_absmax<<<gx, kRegNT, 0, s>>>(images, X, maxbits);
  {
    // DataNormalization divides by the largest modulus: frames that are all
    // zero (or not finite) have no registration
    unsigned mb = 0;
    if ((e = cudaMemcpyAsync(&mb, maxbits, sizeof(mb), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return cuda_status(e, "registration");
    float mx;
    std::memcpy(&mx, &mb, sizeof(mx));
    if (!(mx > 0.f) || !std::isfinite(mx)) return set_error(GBN_ERR_INVALID, "registration: frames all zero, or an infinite modulus");
  }
  k_reg_normalize<<<gx, kRegNT, 0, s>>>(images, maxbits, I, X);
  k_reg_imgrad<<<gx, kRegNT, 0, s>>>(I, d1, d2, N, F);
  k_reg_mesh<<<int(std::min<size_t>((NN + kRegNT - 1) / kRegNT, size_t(ctx->nsm) * 8)), kRegNT, 0, s>>>(xmesh_out,
                                                                                                       xn_out, N, F);
  ctx->launches += 4;
  a.N = N;
  a.F = F;
  a.Cp = g.Cp;
  a.dp = g.dp;
  a.box0 = g.box0;
  a.box1 = g.box1;
  a.E1 = g.E + 1;
  a.smooth = 0;
  a.warp = 0;
  for (int i = 0; i < 4; ++i) a.lam[i] = prm->lambda[i];
  a.fac = float(2.0 / F);
  a.Dp = float(g.Dp);
  a.I = I;
  a.d1 = d1;
  a.d2 = d2;
  a.roi = roi;
  a.cr = cr;
  a.B = B;
  a.S = S;
  a.sup = sup;
  a.T = T_out;
  a.dH = dH;
  a.Dif = Dif;
  a.xn = xn_out;
  a.Iw = Iw;
  a.dy = dy;
  a.dx = dx;
  a.sterm = sterm;
  a.H = H;
  a.part_h = part_h;
  a.part_d = part_d;
  a.st = st;
  const int L = g.box1 - g.box0 + 1;
  const int gp = (L * L + kRegNT - 1) / kRegNT;
  const int gw = (L * L * F + kRegNT - 1) / kRegNT;
  const int gpc = kRegNT / g.dp;
  const int gg = (2 * F * g.Cp * g.Cp + gpc - 1) / gpc;
  const int gu = int((nT + kRegNT - 1) / kRegNT);
  // the unregistered frames: metric H[0]; dx at the starting mesh (optimizer.cpp: InitIT, Metric, CostReduction)
  k_reg_warp<<<gw, kRegNT, 0, s>>>(a);
  k_reg_metric<<<gp, kRegNT, 0, s>>>(a, 0, gu, prm->et, prm->eh);
  ctx->launches += 2;
  a.warp = 1;
  a.smooth = g.sum_lambda != 0;
  // chunks of iterations with one chunk of lookahead: while the GPU runs chunk
  // c the host waits for chunk c-1's stop flag (copied to pinned memory behind
  // it), so the queue never drains; after the stop, the chunk already queued
  // returns at each kernel's entry
  if ((rc = host_flags_ready(ctx)) != GBN_OK) return rc;
  RegState hs{};
  int chunk = 0;
  for (int it = 1; it <= prm->nmax; ++chunk) {
    for (int k = 0; k < kRegChunk && it <= prm->nmax; ++k, ++it) {
      // plain launches: chained by programmatic dependent launch these small
      // grids ran slower (6.3 against 5.1 ms per registration at 256^2 x 20)
      if (g.dp == 17)
        k_reg_grad<17><<<gg, kRegNT, 0, s>>>(a);
      else
        k_reg_grad<0><<<gg, kRegNT, 0, s>>>(a);
      k_reg_update<<<gu, kRegNT, 0, s>>>(a);
      k_reg_warp<<<gw, kRegNT, 0, s>>>(a);
      k_reg_metric<<<gp, kRegNT, 0, s>>>(a, it, gu, prm->et, prm->eh);
      ctx->launches += 4;
    }
    if ((e = cudaMemcpyAsync(&ctx->host_flags[chunk & 1], &st->done, sizeof(int), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaEventRecord(ctx->ev_flag[chunk & 1], s)) != cudaSuccess)
      return cuda_status(e, "registration");
    if (chunk > 0) {
      if ((e = cudaEventSynchronize(ctx->ev_flag[(chunk - 1) & 1])) != cudaSuccess) return cuda_status(e, "registration");
      if (ctx->host_flags[(chunk - 1) & 1]) break;
    }
  }
  if ((e = cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_status(e, "registration");
  std::vector<float> hH(size_t(prm->nmax) + 1, 0.f);
  if ((e = cudaMemcpyAsync(hH.data(), H, hH.size() * sizeof(float), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_status(e, "registration");
  if (h_H) std::memcpy(h_H, hH.data(), hH.size() * sizeof(float));
  if (stats) {
    stats->iterations = hs.it;
    stats->H0 = hH[0];
    stats->H = hH[size_t(hs.it)];
    stats->Wn = hs.Wn;
    stats->Tdif = hs.Tdif;
    stats->status = hs.status;
  }
  return GBN_OK;
}

}  // namespace gbn
