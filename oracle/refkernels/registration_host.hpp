// GroupwiseRegistration run on the host with the reference's own kernels --
// TEST INFRASTRUCTURE (oracle).  Included at the end of harness.cpp, after the
// kernel sources (initialize.cl, optimizer.cl, creabspline.cl, reductions.cl).
//
// The host sequence restates GroupwiseRegistration::init / launch / evolution /
// setMask / stopCondition (GroupwiseRegistration.cpp:79-618), creabspline()
// (groupwiseRegistration/creabspline.cpp) and optimizer()
// (groupwiseRegistration/optimizer.cpp), with each Process::launch's NDRange
// and arguments (groupwiseRegistration/*/*.cpp, cited per call).  The B-spline
// basis functions restate groupwiseRegistration/bspline.cpp, constants
// included.  Every work array is laid out like the reference's Data objects:
// the dims/strides header of Data::calcDataDims / calcDataStrides
// (Data.cpp:1225-1343) in a header region rounded up to the device alignment,
// then each NDArray rounded up to the same alignment
// (DeviceDataProperties.cpp:156-230), so that the kernels' header reads
// (hostKernelFunctions.cl) see what they see on a device.  Work items run in
// order (gid0 fastest), so kernels whose work items race on a device give the
// in-order result here.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <numeric>

namespace reg {

constexpr size_t kAlign = 512;  // CL_DEVICE_MEM_BASE_ADDR_ALIGN (4096 bits) of the reference's GPUs

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// a Data object: NDArrays with their spatial dims, the temporal ("dynamic") dims
struct RD {
  std::vector<std::vector<cl_uint>> nd;
  std::vector<cl_uint> dyn;
  size_t es = 4;
  std::vector<cl_uint> w;
  std::vector<size_t> off;  // word offset of each NDArray's data
  void* p(size_t i = 0) { return w.data() + off.at(i); }
  float* f(size_t i = 0) { return reinterpret_cast<float*>(p(i)); }
  int* n(size_t i = 0) { return reinterpret_cast<int*>(p(i)); }
  cl_uint* u(size_t i = 0) { return reinterpret_cast<cl_uint*>(p(i)); }
  float2* c(size_t i = 0) { return reinterpret_cast<float2*>(p(i)); }
  size_t count(size_t i = 0) const {
    size_t k = 1;
    for (cl_uint d : nd.at(i)) k *= d;
    return k;
  }
  cl_uint dim(size_t d, size_t i = 0) const { return nd.at(i).at(d); }
};

RD make_rd(std::vector<std::vector<cl_uint>> nd, std::vector<cl_uint> dyn, size_t es) {
  RD d;
  d.nd = std::move(nd);
  d.dyn = std::move(dyn);
  d.es = es;
  bool eq = true;
  for (size_t i = 1; i < d.nd.size(); ++i) eq = eq && d.nd[i] == d.nd[0];
  std::vector<cl_uint> v = {cl_uint(d.nd[0].size()), eq ? 1u : 0u, 0u, cl_uint(d.dyn.size())};
  for (cl_uint t : d.dyn) v.push_back(t);
  for (size_t i = 0; i < (eq ? 1 : d.nd.size()); ++i)
    for (cl_uint x : d.nd[i]) v.push_back(x);
  for (size_t i = 0; i < (eq ? 1 : d.nd.size()); ++i) {
    cl_uint acc = 1;
    for (cl_uint x : d.nd[i]) {
      v.push_back(acc);
      acc *= x;
    }
    cl_uint last = cl_uint(round_up(acc, kAlign / es));
    v.push_back(last);
    for (size_t t = 1; t < d.dyn.size(); ++t) {
      last *= d.dyn[t - 1];
      v.push_back(last);
    }
  }
  const size_t hbytes = round_up((v.size() + 1) * 4, kAlign);
  size_t words = hbytes / 4;
  for (size_t i = 0; i < d.nd.size(); ++i) {
    d.off.push_back(words);
    words += round_up(d.count(i) * es, kAlign) / 4;
  }
  d.w.assign(words, 0u);
  std::memcpy(d.w.data(), v.data(), v.size() * 4);
  d.w[hbytes / 4 - 1] = cl_uint(hbytes);
  return d;
}

RD make_rd1(std::vector<cl_uint> dims, size_t es) { return make_rd({std::move(dims)}, {}, es); }

// ---- bspline.cpp: B-spline basis and derivatives, orders 1-3 ----
float bspline1(float x) { return (x < 1 && x >= -1) ? 1 - std::fabs(x) : 0; }
float bspline2(float x) {
  if (x < -0.5 && x >= -1.5) return (4 * std::pow(x, 2) + 12 * x + 9) / 8;
  if (x < 0.5 && x >= -0.5) return (-4 * std::pow(x, 2) + 3) / 4;
  if (x < 1.5 && x >= 0.5) return (4 * std::pow(x, 2) - 12 * x + 9) / 8;
  return 0;
}
float bspline3(float x) {
  const float val = std::fabs(x);
  if (val < 1) return 0.5 * std::pow(val, 3) - std::pow(val, 2) + 0.6666;
  if (val >= 1 && val < 2) return (2 - val) * (2 - val) * (2 - val) / 6;
  return 0;
}
float b1spline1(float x) { return (x < 0 && x >= -1) ? 1 : ((x < 1 && x >= 0) ? -1 : 0); }
float b1spline2(float x) {
  if (x < -0.5 && x >= -1.5) return (2 * x + 3) / 2;
  if (x < 0.5 && x >= -0.5) return -2 * x;
  if (x < 1.5 && x >= 0.5) return (42 * x - 3) / 2;
  return 0;
}
float b1spline3(float x) {
  if (x <= 1 && x >= 0) return 1.5 * std::pow(x, 2) - 2 * x;
  if (x >= -1 && x < 0) return -1.5 * std::pow(x, 2) - 2 * x;
  if (x > 1 && x < 2) return -(x - 2) * (x - 2) / 2;
  if (x < -1 && x > -2) return (x + 2) * (x + 2) / 2;
  return 0;
}
float b2spline2(float x) {
  if (x < -0.5 && x >= -1.5) return 1;
  if (x < 0.5 && x >= -0.5) return -2;
  if (x < 1.5 && x >= 0.5) return 1;
  return 0;
}
float b2spline3(float x) {
  const float val = std::fabs(x);
  if (val < 1) return 3 * val - 2;
  if (val >= 1 && val < 2) return -val + 2;
  return 0;
}
float bsplineN(float x, int n) { return n == 1 ? bspline1(x) : n == 2 ? bspline2(x) : bspline3(x); }
float b1splineN(float x, int n) { return n == 1 ? b1spline1(x) : n == 2 ? b1spline2(x) : b1spline3(x); }
float b2splineN(float x, int n) { return n == 2 ? b2spline2(x) : n == 3 ? b2spline3(x) : 0.f; }

struct Params {
  float W;
  int flagW, radius, E, Dp0, Dp1, nmax;
  float et, eh;
  float lambda[4];
};

}  // namespace reg

extern "C" {

// GroupwiseRegistration on F frames of N x N complex images (frame-major,
// column fastest).  Outputs: T [C1 * C0 * F * 2] (the control-point
// displacements), xn [N * N * F * 2] (the deformed mesh), H [nmax + 1] (the
// metric per iteration), bb [4] (1-based bounding box), info [4] = {iterations,
// C0 (= Cp0), C1 (= Cp1), areaX}, wn = the final weight.  T_init: starting
// displacements in T's layout, or NULL for zeros.  Returns 0, or -1
// when the control grid or its supports leave the image (the reference reads
// outside its buffers there).
int ref_registration(const float* images, int N, int F, const reg::Params* prm, float* T_out, float* xn_out,
                     float* H_out, int* bb_out, int* info, float* wn_out, size_t T_cap, const float* T_init) {
  using namespace reg;
  const cl_uint nROWS = N, nCOLS = N, nFRAMES = F, nt = 2;
  if (N % 8 != 0 || F < 3) return -1;  // frames contiguous at the device alignment; shiftTAux needs 3 frames
  // ---- init() (GroupwiseRegistration.cpp:92-400) ----
  RD input = make_rd(std::vector<std::vector<cl_uint>>(F, {nCOLS, nROWS}), {nFRAMES}, 8);
  for (int f = 0; f < F; ++f) std::memcpy(input.p(f), images + size_t(f) * N * N * 2, size_t(N) * N * 8);
  RD normInputData = make_rd(input.nd, input.dyn, 8), transformedData = make_rd(input.nd, input.dyn, 8);
  std::vector<cl_uint> bound_box(4);
  std::vector<cl_uint> mask(size_t(nROWS) * nCOLS, 0);
  int areaX = 0;
  if (prm->radius != 0) {
    // setMask (GroupwiseRegistration.cpp:486-531)
    const int radius2 = std::pow(prm->radius, 2);
    const float center[2] = {float(nROWS + 1) / 2, float(nCOLS + 1) / 2};
    cl_uint min_fil1 = nCOLS, max_fil1 = 0, min_col1 = nROWS, max_col1 = 0;
    for (cl_uint i = 0; i < nCOLS; i++) {
      for (cl_uint j = 0; j < nROWS; j++) {
        const float Cv = std::pow(1 - center[0] + j, 2), Dv = std::pow(1 - center[1] + i, 2);
        if ((Cv + Dv) <= radius2) {
          mask[i + j * nCOLS] = 1;
          if (i < min_fil1) min_fil1 = i;
          if (j < min_col1) min_col1 = j;
          if (i > max_fil1) max_fil1 = i;
          if (j > max_col1) max_col1 = j;
          areaX++;
        }
      }
    }
    bound_box = {min_fil1 + 1, min_col1 + 1, max_fil1 + 1, max_col1 + 1};
  } else {
    const int Nh = prm->Dp0 * (prm->E + 1), Nv = prm->Dp1 * (prm->E + 1);
    for (cl_uint i = Nv; i < nROWS - Nv; i++)
      for (cl_uint j = Nh; j < nCOLS - Nh; j++) {
        mask[j + i * nCOLS] = 1;
        areaX++;
      }
    bound_box = {cl_uint(Nv + 1), nROWS - Nv, cl_uint(Nh + 1), nCOLS - Nh};
  }
  RD maskData = make_rd1({nROWS, nROWS}, 4);
  std::memcpy(maskData.p(), mask.data(), mask.size() * 4);
  const cl_uint longr1 = bound_box[2] - bound_box[0] + 1, longr2 = bound_box[3] - bound_box[1] + 1;
  const cl_uint margin[3] = {cl_uint(std::ceil(nCOLS / 40)), cl_uint(std::ceil(nROWS / 40)),
                             cl_uint(std::ceil(nFRAMES / 40))};
  const cl_uint longr1margin = (bound_box[3] + margin[0] + 1) - (bound_box[1] - margin[0] - 1) + 1;
  const cl_uint longr2margin = (bound_box[2] + margin[1] + 1) - (bound_box[0] - margin[1] - 1) + 1;
  float Wn = prm->W / areaX;
  RD xData = make_rd1({nROWS, nROWS, 2}, 4);
  for (cl_uint i = 0; i < nCOLS; i++)
    for (cl_uint j = 0; j < nROWS; j++) {
      xData.u()[i + j * nCOLS + 0 * nROWS * nCOLS] = j + 1;
      xData.u()[i + j * nCOLS + 1 * nROWS * nCOLS] = i + 1;
    }
  const cl_uint E = prm->E;
  const int Dp[2] = {prm->Dp0, prm->Dp1};
  float c[2], rp[2];
  int Cc[2][2];
  c[0] = float(bound_box[0] + bound_box[2]) / 2;
  c[1] = float(bound_box[1] + bound_box[3]) / 2;
  rp[0] = (E + 1) * Dp[0] / 2;
  rp[1] = (E + 1) * Dp[1] / 2;
  for (cl_uint l = 0; l < nt; l++)
    for (cl_uint b = 0; b < 2; b++) Cc[l][b] = std::floor((std::abs(c[l] - bound_box[l + b * 2]) + rp[l]) / Dp[l]);
  const cl_uint dp0 = cl_uint(2 * std::ceil(rp[0]) + 1), dp1 = cl_uint(2 * std::ceil(rp[1]) + 1);
  const cl_uint Cp1 = cl_uint(Cc[1][0] + Cc[1][1] + 1), Cp0 = cl_uint(Cc[0][0] + Cc[0][1] + 1);
  if (Cp0 != Cp1 || dp0 != dp1) return -1;  // the reference's kernels assume a square grid here
  {
    // every support of the control grid inside the image
    const float lo = c[0] + Dp[0] * (-Cc[0][0]) - std::ceil(rp[0]), hi = c[0] + Dp[0] * (Cc[0][1]) + std::ceil(rp[0]);
    const float lo1 = c[1] + Dp[1] * (-Cc[1][0]) - std::ceil(rp[1]), hi1 = c[1] + Dp[1] * (Cc[1][1]) + std::ceil(rp[1]);
    if (lo < 1 || lo1 < 1 || hi > N || hi1 > N) return -1;
  }
  if (T_cap < size_t(Cp1) * Cp0 * F * nt) return -1;
  RD coef = make_rd1({nCOLS, 2, nt}, 4);
  RD coefg = make_rd1({Cp1, 2, nt}, 4);
  RD puData = make_rd1({Cp0, Cp1, nt}, 4);
  RD auxBBallData = make_rd({{E + 1, E + 1, nCOLS, nROWS}, {E + 1, E + 1, nCOLS, nROWS, nt},
                             {E + 1, E + 1, nCOLS, nROWS, nt}, {E + 1, E + 1, nCOLS, nROWS}},
                            {4}, 4);
  RD BBall = make_rd({{nCOLS, nROWS, nFRAMES, nt, E + 1, E + 1}, {nCOLS, nROWS, nFRAMES, nt, E + 1, E + 1, 2},
                      {nCOLS, nROWS, nFRAMES, nt, E + 1, E + 1, 2}, {nCOLS, nROWS, nFRAMES, nt, E + 1, E + 1}},
                     {4}, 4);
  RD auxBBgallData = make_rd({{dp1, dp0, Cp1, Cp0, 2}, {dp1, dp0, Cp1, Cp0, 2}, {dp1, dp0, Cp1, Cp0}}, {3}, 4);
  RD aux1BBgallData = make_rd(
      {{dp1, dp0, Cp1, Cp0, 2, nFRAMES, 2}, {dp1, dp0, Cp1, Cp0, 2, nFRAMES, 2}, {dp1, dp0, Cp1, Cp0, nFRAMES, 2}}, {3},
      4);
  RD BBgall = make_rd({{dp1, dp0, Cp1, Cp0}, {dp1, dp0, nFRAMES, Cp1, Cp0, 2, 2}, {dp1, dp0, nFRAMES, Cp1, Cp0, 2, 2},
                       {dp1, dp0, nFRAMES, Cp1, Cp0, 2}},
                      {4}, 4);
  RD TAuxData = make_rd({{longr2, longr1, nFRAMES, nt, E + 1, E + 1}, {longr1, longr2, nFRAMES, nt, E + 1, E + 1},
                         {longr1, longr2, nFRAMES, nt, E + 1, E + 1}, {longr1, longr2, nFRAMES, nt, E + 1, E + 1}},
                        {4}, 4);
  RD VData = make_rd1({nCOLS, nROWS}, 4);
  RD dtauallData = make_rd({{nCOLS, nROWS, nFRAMES, nt, 2}, {nCOLS, nROWS, nFRAMES, nt, 2}, {nCOLS, nROWS, nFRAMES, nt},
                            {nCOLS, nROWS, nFRAMES, nt}, {nCOLS, nROWS, nFRAMES, nt}},
                           {5}, 4);
  RD dthetaallData = make_rd({{dp1, dp0, nFRAMES, Cp1, Cp0, nt, 2}, {dp1, dp0, nFRAMES, Cp1, Cp0, nt, 2},
                              {dp1, dp0, nFRAMES, Cp1, Cp0, nt}, {dp1, dp0, nFRAMES, Cp1, Cp0, nt},
                              {dp1, dp0, nFRAMES, Cp1, Cp0, nt}},
                             {5}, 4);
  RD HData = make_rd1({cl_uint(prm->nmax + 1)}, 4);
  RD dallData = make_rd({{nCOLS, nROWS, nFRAMES, 2}, {nCOLS, nROWS, nFRAMES, 2}}, {2}, 4);
  RD dxData = make_rd1({nCOLS, nROWS, nFRAMES, 2}, 4);
  RD dyData = make_rd1({nCOLS, nROWS, nFRAMES}, 4);
  RD xnData = make_rd1({nCOLS, nROWS, nFRAMES, nt}, 4);
  RD auxData = make_rd1({dp1, dp0, nFRAMES, Cp1, Cp0, nt}, 4);
  RD aux1Data = make_rd1({dp1, dp0, nFRAMES, Cp1, Cp0}, 4);
  RD aux2Data = make_rd1({dp1, dp0, Cp1, Cp0}, 4);
  RD AuxData = make_rd1({dp1, dp0, nFRAMES, Cp1, Cp0}, 4);
  RD dVData = make_rd({{dp1, dp0, nFRAMES, Cp1, Cp0, nt}, {dp1, dp0, Cp1, Cp0, nFRAMES, nt}}, {2}, 4);
  RD XauxData = make_rd1({dp1, dp0, nFRAMES, nt}, 4);
  RD cost1Data = make_rd1({dp1, dp0, nFRAMES, nt}, 4);
  RD cost2Data = make_rd1({dp1, nFRAMES, nt}, 4);
  RD dHData = make_rd1({Cp0, Cp1, nFRAMES, nt}, 4);
  RD DifData = make_rd1({Cp1, Cp0, nFRAMES, nt}, 4);
  // index lists: TransformationAux / Deformation / Regularization / SumLambdaMetric
  // ::init (bounding box rows and columns), GradientInterpolator / Interpolator
  // ::init (the margin rectangle)
  std::vector<int> r1(longr1), r2(longr2), r1m(longr1margin), r2m(longr2margin);
  for (cl_uint i = 0; i < longr1; i++) r1[i] = (bound_box[0] - 1) + i;
  for (cl_uint i = 0; i < longr2; i++) r2[i] = (bound_box[1] - 1) + i;
  for (cl_uint i = 0; i < longr1margin; i++) r1m[i] = (bound_box[1] - margin[0] - 1) + i - 1;
  for (cl_uint i = 0; i < longr2margin; i++) r2m[i] = (bound_box[0] - margin[1] - 1) + i - 1;

  // ---- launch(): maximum modulus, DataNormalization (GroupwiseRegistration.cpp:556-600) ----
  float oldmax = 0.f;
  for (int f = 0; f < F; ++f) {
    float m = 0.f;
    for (size_t q = 0; q < size_t(N) * N; ++q) {
      const float2 v = input.c(f)[q];
      m = std::max(m, std::hypot(v.x, v.y));  // std::fabs(std::complex<float>) is cabsf, a hypotf
    }
    oldmax = f == 0 ? m : std::max(oldmax, m);
  }
  const float newmax = 500;
  ndrange(size_t(F) * N * N, 1, 1, [&] { dataNormalization(normInputData.c(), input.c(), oldmax, newmax); });

  // ---- creabspline() (creabspline.cpp) ----
  // ControlPointsLocation::launch: global (Cp0, Cp1)
  {
    std::vector<float> cbuf = {c[0], c[1]};
    std::vector<int> dpbuf = {Dp[0], Dp[1]};
    ndrange(Cp0, Cp1, 1,
            [&] { controlPointsLocation(puData.f(), Cc[0][0], Cc[1][0], cbuf.data(), dpbuf.data()); });
  }
  std::vector<float> coefv(size_t(nCOLS) * 2 * nt);
  const cl_uint cdim0 = nCOLS, cdim1 = 2;
  const cl_uint* x = xData.u();
  const cl_uint xd0 = nROWS, xd1 = nROWS;
  for (cl_uint b = 0; b < cdim1; b++) {
    for (cl_uint i = 0; i < cdim0; i++) {
      if (E % 2 != 0) {
        coefv[i + b * cdim0 + 0 * cdim0 * cdim1] =
            std::floor((x[0 + i * xd0 + 0 * xd0 * xd1] - c[0]) / Dp[0]) + ((E + std::pow(-1, b + 1)) / 2) * std::pow(-1, b + 1);
        coefv[i + b * cdim0 + 1 * cdim0 * cdim1] =
            std::floor((x[i + 0 * xd0 + 1 * xd0 * xd1] - c[1]) / Dp[1]) + ((E + std::pow(-1, b + 1)) / 2) * std::pow(-1, b + 1);
      } else {
        coefv[i + b * cdim0 + 0 * cdim0 * cdim1] =
            std::round((x[0 + i * xd0 + 0 * xd0 * xd1] - c[0]) / Dp[0]) + (E / 2) * std::pow(-1, b + 1);
        coefv[i + b * cdim0 + 1 * cdim0 * cdim1] =
            std::round((x[i + 0 * xd0 + 1 * xd0 * xd1] - c[1]) / Dp[1]) + (E / 2) * std::pow(-1, b + 1);
      }
    }
  }
  {
    // BBAux [nCOLS][E+1][3][nt] as the host fills it; CreateBB::launch: global (E+1, E+1, nCOLS*nROWS)
    RD BBAuxData = make_rd1({nCOLS, E + 1, 3, nt}, 4);
    float* BBAux = BBAuxData.f();
    const cl_uint bd1 = E + 1, bd0 = nCOLS, bd2 = 3;
    const cl_uint dataSize[2] = {nCOLS, nROWS};
    for (cl_uint l = 0; l < nt; l++) {
      for (cl_uint n = 0; n < dataSize[l]; n++) {
        const float c0 = coefv[n + 0 * cdim0 + l * cdim0 * cdim1], c1 = coefv[n + 1 * cdim0 + l * cdim0 * cdim1];
        for (int k = int(c0); k <= c1; k++) {
          const int xb = int(n + 1);
          const size_t base = size_t(((k - 1) - c0) + 1) + n * bd1 + l * bd1 * bd0 * bd2;
          BBAux[base + 0 * bd1 * bd0] = bsplineN(((xb - c[l]) / Dp[l]) - k, E);
          BBAux[base + 1 * bd1 * bd0] = b1splineN(((xb - c[l]) / Dp[l]) - k, E);
          BBAux[base + 2 * bd1 * bd0] = b2splineN(((xb - c[l]) / Dp[l]) - k, E);
        }
      }
    }
    const cl_uint s0 = E + 1, s1 = E + 1, s2 = nCOLS, s3 = nROWS;
    ndrange(s0, s1, size_t(s2) * s3, [&] {
      createBB(auxBBallData.f(0), auxBBallData.f(1), auxBBallData.f(2), auxBBallData.f(3), BBAux, s2);
    });
  }
  {
    std::vector<float> coefbuffer(size_t(nCOLS) * 2 * nt);
    for (cl_uint i = 0; i < cdim0; i++)
      for (cl_uint b = 0; b < cdim1; b++)
        for (cl_uint l = 0; l < cdim1; l++)
          coefbuffer[i + b * cdim0 + l * cdim0 * cdim1] = coefv[i + b * cdim0 + l * cdim0 * cdim1] + 1 -
                                                          coefv[(bound_box[l]) + 0 * cdim0 + l * cdim0 * cdim1];
    std::memcpy(coef.f(), coefbuffer.data(), coefbuffer.size() * 4);
  }
  {
    // PermuteBB::launch: global (nCOLS*nROWS, F*nt, (E+1)*(E+1)), from the BB1 dims
    std::vector<int> dpbuf = {Dp[0], Dp[1]};
    ndrange(size_t(nCOLS) * nROWS, size_t(nFRAMES) * nt, size_t(E + 1) * (E + 1), [&] {
      permuteBB(BBall.f(0), BBall.f(1), BBall.f(2), BBall.f(3), auxBBallData.f(0), auxBBallData.f(1),
                auxBBallData.f(2), auxBBallData.f(3), dpbuf.data(), nCOLS, nFRAMES, E + 1);
    });
  }
  std::vector<float> coefgbuffer(size_t(Cp1) * 2 * nt);
  {
    const float* pu = puData.f();
    const cl_uint pd1 = Cp1, pd0 = Cp0, gd0 = Cp1, gd1 = 2;
    for (cl_uint i = 0; i < gd0; i++)
      for (cl_uint j = 0; j < gd1; j++) {
        coefgbuffer[i + j * gd0 + 0 * gd0 * gd1] =
            std::ceil(pu[i + 0 * pd1 + 0 * pd1 * pd0] - std::ceil(rp[0])) + j * 2 * std::ceil(rp[0]);
        coefgbuffer[i + j * gd0 + 1 * gd0 * gd1] =
            std::ceil(pu[0 + i * pd1 + 1 * pd1 * pd0] - std::ceil(rp[1])) + j * 2 * std::ceil(rp[1]);
      }
    const int limxy[2] = {int(Cp1), int(Cp0)};
    std::vector<float> xbis2(size_t(limxy[0]) * 2);
    for (int l = 0; l < 2; l++)
      for (int i = 0; i < limxy[l]; i++) {
        if (l == 0)
          xbis2[i + 0 * limxy[l]] = pu[i + 0 * pd1 + 0 * pd1 * pd0];
        else
          xbis2[i + 1 * limxy[l]] = pu[0 + i * pd1 + 1 * pd1 * pd0];
      }
    RD BBAux1Data = make_rd1({Cp1, dp0, 3, 2}, 4);
    float* BBAux1 = BBAux1Data.f();
    const cl_uint a1 = dp0, a0 = Cp1;  // BBAux1Data spatial dims 1 and 0
    for (cl_uint n = 0; n < gd0; n++) {
      const cl_uint idxcoefg = n;
      const float k0 = coefgbuffer[n + 0 * gd0], k1 = coefgbuffer[n + 1 * gd0];
      for (int k = int(k0); k <= k1; k++) {
        const size_t base = size_t(((k - 1) - coefgbuffer[idxcoefg]) + 1) + n * a1;
        BBAux1[base + 0 * a1 * a0 + 0 * a1 * a0 * 3] = bsplineN(((k - xbis2[n + 0 * limxy[0]]) / Dp[0]), E);
        BBAux1[base + 0 * a1 * a0 + 1 * a1 * a0 * 3] = bsplineN(((k - xbis2[n + 1 * limxy[0]]) / Dp[1]), E);
        BBAux1[base + 1 * a1 * a0 + 0 * a1 * a0 * 3] = b1splineN(((k - xbis2[n + 0 * limxy[0]]) / Dp[0]), E);
        BBAux1[base + 1 * a1 * a0 + 1 * a1 * a0 * 3] = b1splineN(((k - xbis2[n + 1 * limxy[0]]) / Dp[1]), E);
        BBAux1[base + 2 * a1 * a0 + 0 * a1 * a0 * 3] = b2splineN(((k - xbis2[n + 0 * limxy[0]]) / Dp[0]), E);
        BBAux1[base + 2 * a1 * a0 + 1 * a1 * a0 * 3] = b2splineN(((k - xbis2[n + 1 * limxy[0]]) / Dp[1]), E);
      }
    }
    // CreateBBg::launch: global (dp1, dp0, Cp1*Cp0), from the auxBB1g dims
    std::vector<int> dpbuf = {Dp[0], Dp[1]};
    ndrange(dp1, dp0, size_t(Cp1) * Cp0, [&] {
      createBBg(BBgall.f(0), auxBBgallData.f(0), auxBBgallData.f(1), auxBBgallData.f(2), BBAux1, dpbuf.data(), Cp1);
    });
  }
  // RepmatBBg::launch: global (dp1*dp0, Cp1*Cp0, 2*F), from the aux1BB1g dims
  ndrange(size_t(dp1) * dp0, size_t(Cp1) * Cp0, size_t(2) * nFRAMES, [&] {
    repmatBBg(aux1BBgallData.f(0), aux1BBgallData.f(1), aux1BBgallData.f(2), auxBBgallData.f(0), auxBBgallData.f(1),
              auxBBgallData.f(2), dp1, Cp1, 2, 2);
  });
  // PermuteBBg::launch: global (dp1*dp0, F*Cp1, Cp0*2), from the BB1g dims
  ndrange(size_t(dp1) * dp0, size_t(nFRAMES) * Cp1, size_t(Cp0) * 2, [&] {
    permuteBBg(BBgall.f(1), BBgall.f(2), BBgall.f(3), aux1BBgallData.f(0), aux1BBgallData.f(1), aux1BBgallData.f(2),
               dp1, nFRAMES, Cp0, 2);
  });
  {
    const cl_uint gd0 = Cp1, gd1 = 2, gd2 = nt;
    const cl_uint dataSize[2] = {nCOLS, nROWS};
    for (cl_uint i = 0; i < gd0; i++)
      for (cl_uint j = 0; j < gd1; j++)
        for (cl_uint l = 0; l < gd2; l++) {
          float& v = coefgbuffer[i + j * gd0 + l * gd0 * gd1];
          if (v < 1) v = 1;
          if (v > int(dataSize[l])) v = dataSize[l];
        }
    std::memcpy(coefg.f(), coefgbuffer.data(), coefgbuffer.size() * 4);
  }

  // ---- optimizer() (optimizer.cpp) ----
  // optimizer(): the given TData (a later motion iteration), else InitZero
  RD TData = make_rd1({Cp1, Cp0, nFRAMES, nt}, 4);
  if (T_init) std::memcpy(TData.f(), T_init, TData.count() * 4);
  std::vector<float> Hdif(prm->nmax), Tdif(prm->nmax);
  auto initZero = [&](RD& d) {
    for (size_t i = 0; i < d.nd.size(); ++i) {
      float* a = d.f(i);
      ndrange(d.count(i), 1, 1, [&] { ::initZero(a); });
    }
  };
  auto copyIT = [&] {  // CopyDataGPU::launch: global W*H*D*dynDims
    ndrange(size_t(N) * N * F, 1, 1, [&] { copyDataGPU(transformedData.c(), normInputData.c()); });
  };
  auto metricL = [&] {  // Metric::launch: global (dims0, dims1)
    ndrange(nCOLS, nROWS, 1, [&] { metric(VData.f(), transformedData.c()); });
  };
  auto costReductionL = [&](int iter) {  // CostReduction::launch: global dims0*dims1
    ndrange(size_t(nCOLS) * nROWS, 1, 1, [&] { costReduction(HData.f(), VData.f(), maskData.n(), iter); });
  };
  auto transformationAuxL = [&] {  // TransformationAux::launch
    const auto& ds = TAuxData.nd[0];
    ndrange(size_t(ds[0]) * ds[1], size_t(ds[2]) * ds[3], size_t(ds[4]) * ds[5], [&] {
      transformationAux(TAuxData.f(0), TData.f(), coef.f(), r1.data(), r2.data(), ds[0], ds[2], ds[4], nCOLS, Cp1,
                        Cp0);
    });
  };
  auto deformationL = [&] {  // Deformation::launch + DeformationAdjust::launch
    const auto& sb = BBall.nd[1];
    const auto& st = TAuxData.nd[0];
    ndrange(st[0], st[1], size_t(st[2]) * st[3], [&] {
      transformation(xnData.f(), TAuxData.f(0), BBall.f(0), r1.data(), r2.data(), st[2], sb[0], sb[1], sb[3], sb[4]);
    });
    const auto& dx = xnData.nd[0];
    ndrange(dx[0], dx[1], size_t(dx[2]) * dx[3], [&] { transformationAdjust(xnData.f(), xData.n()); });
  };
  // initial metric (optimizer.cpp: InitIT, InitZero dx / dtau, Metric, CostReduction, Gradient)
  int iter = 0;
  copyIT();
  initZero(dxData);
  initZero(dtauallData);
  metricL();
  costReductionL(iter);
  ndrange(nCOLS, nROWS, F, [&] { gradient(dallData.f(0), dallData.f(1), normInputData.c()); });
  const float p2 = prm->et * nFRAMES * nt;
  const float p4 = HData.f()[0] * prm->eh;
  bool stop = false;
  iter = 1;
  const float factor = 2.0 / nFRAMES;  // GradientMetric::launch (GradientMetric.cpp:72)
  while (!stop) {
    initZero(TAuxData);
    transformationAuxL();
    initZero(xnData);
    deformationL();
    // Initdx::launch: global (dims0, dims1, dims2) of dx
    ndrange(nCOLS, nROWS, nFRAMES, [&] { initdx(dxData.f(), dallData.f(0), dallData.f(1)); });
    // GradientInterpolator::launch: global (longr1margin, longr2margin, dims2 of dx)
    ndrange(longr1margin, longr2margin, nFRAMES, [&] {
      gradientInterpolator(dxData.f(), dallData.f(0), dallData.f(1), xnData.f(), xData.n(), r1m.data(), r2m.data());
    });
    // GradientMetric::launch: global (dims0, dims1, numFrames)
    ndrange(nCOLS, nROWS, nFRAMES, [&] { gradientMetric(dyData.f(), transformedData.c(), factor); });
    {
      // GradientRegularization::launch: global from the BB1g dims
      const auto& sg = BBgall.nd[1];
      const auto& sd = dtauallData.nd[0];
      ndrange(size_t(sg[0]) * sg[1], size_t(sg[2]) * sg[3], size_t(sg[4]) * sg[5], [&] {
        gradientRegularization(dthetaallData.f(0), dthetaallData.f(1), dthetaallData.f(2), dthetaallData.f(3),
                               dthetaallData.f(4), dtauallData.f(0), dtauallData.f(1), dtauallData.f(2),
                               dtauallData.f(3), dtauallData.f(4), coefg.f(), BBgall.f(0), BBgall.f(1), BBgall.f(2),
                               BBgall.f(3), sg[0], sg[2], sg[4], sd[0], sd[1]);
      });
    }
    {
      // Reduction7Dto6D::launch: global = product of the first six dthetax dims
      const auto& s = dthetaallData.nd[0];
      ndrange(size_t(s[0]) * s[1] * s[2] * s[3] * s[4] * s[5], 1, 1, [&] {
        reduction7Dto6D(auxData.f(), dthetaallData.f(0), dthetaallData.f(1), dthetaallData.f(2), dthetaallData.f(3),
                        dthetaallData.f(4), prm->lambda[0], prm->lambda[1], prm->lambda[2], prm->lambda[3]);
      });
    }
    // ReductionSum::launch (dim 5, then dim 2): global = output size
    ndrange(aux1Data.count(), 1, 1, [&] { reductionsum(aux1Data.f(), auxData.f(), 5); });
    ndrange(aux2Data.count(), 1, 1, [&] { reductionsum(aux2Data.f(), aux1Data.f(), 2); });
    {
      // GradientJointAux::launch: global (d0*d1, d2, d3*d4) of Aux
      const auto& s = AuxData.nd[0];
      ndrange(size_t(s[0]) * s[1], s[2], size_t(s[3]) * s[4], [&] { gradientJointAux(AuxData.f(), aux2Data.f()); });
    }
    {
      // GradientWithSmoothTerms::launch: global from the dV dims
      const auto& sv = dVData.nd[0];
      const auto& sg = BBgall.nd[1];
      const auto& sd = dxData.nd[0];
      ndrange(size_t(sv[0]) * sv[1], size_t(sv[2]) * sv[3], size_t(sv[4]) * sv[5], [&] {
        gradientJoint(dVData.f(0), dyData.f(), dxData.f(), BBgall.f(0), AuxData.f(), coefg.f(), sg[0], sg[2], sg[4],
                      sd[0], sd[1]);
      });
    }
    {
      // PermutedV::launch
      const auto& s = dVData.nd[0];
      ndrange(size_t(s[0]) * s[1], size_t(s[2]) * s[3], size_t(s[4]) * s[5],
              [&] { permutedV(dVData.f(1), dVData.f(0), s[0], s[2], s[4]); });
    }
    {
      const auto& s = dVData.nd[0];  // {dp1, dp0, F, Cp1, Cp0, nt}
      for (cl_uint k = 0; k < s[3]; k++) {
        for (cl_uint l = 0; l < s[4]; l++) {
          // AuxiliarMask / AuxiliarCost / Cost6DReduction / Cost6D ::launch
          ndrange(size_t(s[0]) * s[1], s[2], s[5], [&] {
            auxiliarMask(XauxData.f(), maskData.u(), coefg.f(), int(l), int(k), s[0], Cp1, 2);
          });
          ndrange(size_t(s[0]) * s[1], s[2], s[5], [&] {
            auxiliarCost(cost1Data.f(), dVData.f(1), XauxData.f(), int(l), int(k), s[0], s[3], s[4]);
          });
          ndrange(cost2Data.dim(0), cost2Data.dim(1), cost2Data.dim(2),
                  [&] { cost6DReduction(cost2Data.f(), cost1Data.f()); });
          ndrange(dHData.dim(2), dHData.dim(3), 1, [&] { cost6D(dHData.f(), cost2Data.f(), int(l), int(k)); });
        }
      }
    }
    {
      // UpdateTransformation::launch: global (d0, d1, d2*d3) of dH
      float wn = Wn;
      ndrange(dHData.dim(0), dHData.dim(1), size_t(dHData.dim(2)) * dHData.dim(3),
              [&] { updateTransformation(TData.f(), DifData.f(), dHData.f(), &wn); });
    }
    initZero(TAuxData);
    transformationAuxL();
    initZero(xnData);
    deformationL();
    {
      // PermuteTAux / ShiftTAux ::launch: global from the TAux original dims
      const auto& s = TAuxData.nd[0];
      ndrange(size_t(s[1]) * s[0], size_t(s[2]) * s[3], size_t(s[4]) * s[5],
              [&] { permuteTAux(TAuxData.f(1), TAuxData.f(0), s[1], s[2], s[4]); });
      ndrange(size_t(s[1]) * s[0], size_t(s[2]) * s[3], size_t(s[4]) * s[5],
              [&] { shiftTAux(TAuxData.f(2), TAuxData.f(3), TAuxData.f(1), s[1], s[2], s[4]); });
    }
    initZero(dtauallData);
    {
      // Regularization::launch: global (TAux dims1, dims0, dtau dims2*dims3)
      const auto& s = TAuxData.nd[0];
      const auto& sd = dtauallData.nd[0];
      ndrange(s[1], s[0], size_t(sd[2]) * sd[3], [&] {
        regularization(dtauallData.f(0), dtauallData.f(1), dtauallData.f(2), dtauallData.f(3), dtauallData.f(4),
                       TAuxData.f(2), TAuxData.f(3), TAuxData.f(1), BBall.f(0), BBall.f(1), BBall.f(2), BBall.f(3),
                       r1.data(), r2.data(), sd[0], sd[1], sd[2], s[4]);
      });
    }
    copyIT();
    {
      // Interpolator::launch: global (longr1margin, longr2margin, dynDims)
      ndrange(longr1margin, longr2margin, nFRAMES, [&] {
        interpolator(transformedData.c(), normInputData.c(), xnData.f(), xData.n(), r1m.data(), r2m.data());
      });
    }
    metricL();
    // sumLambda() accumulates the weights into an int (GroupwiseRegistration.cpp:440-442),
    // so weights below 1 each never add their terms to the metric
    if (std::accumulate(prm->lambda, prm->lambda + 4, 0) != 0) {
      // SumLambdaMetric::launch: global (longr1, longr2)
      const auto& sd = dtauallData.nd[0];
      ndrange(longr1, longr2, 1, [&] {
        sumLambdaMetric(VData.f(), sd[2], sd[3], dtauallData.f(0), dtauallData.f(1), dtauallData.f(2),
                        dtauallData.f(3), dtauallData.f(4), r1.data(), r2.data(), prm->lambda[0], prm->lambda[1],
                        prm->lambda[2], prm->lambda[3]);
      });
    }
    costReductionL(iter);
    // evolution (GroupwiseRegistration.cpp:451-478)
    {
      float sum_squares = 0.0f;
      for (size_t i = 0; i < DifData.count(); i++) sum_squares += DifData.f()[i] * DifData.f()[i];
      Tdif[iter - 1] = std::sqrt(sum_squares);
      Hdif[iter - 1] = HData.f()[iter - 1] - HData.f()[iter];
      if (prm->flagW) {
        if (Hdif[iter - 1] > 0)
          Wn = Wn * 1.2;
        else
          Wn = Wn / 2;
      }
    }
    stop = (prm->nmax == iter) || ((Tdif[iter - 1] < p2) && (Hdif[iter - 1] < p4));
    iter = iter + 1;
  }
  std::memcpy(T_out, TData.f(), TData.count() * 4);
  std::memcpy(xn_out, xnData.f(), xnData.count() * 4);
  std::memcpy(H_out, HData.f(), HData.count() * 4);
  for (int i = 0; i < 4; ++i) bb_out[i] = int(bound_box[i]);
  info[0] = iter - 1;
  info[1] = int(Cp0);
  info[2] = int(Cp1);
  info[3] = areaX;
  *wn_out = Wn;
  return 0;
}

}  // extern "C"
