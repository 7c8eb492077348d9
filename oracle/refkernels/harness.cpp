// Host harness running the reference's own OpenCL kernels on the CPU -- TEST
// INFRASTRUCTURE (oracle).  The kernel and accessor sources are compiled as
// they lie in the reference tree (src/kernels/*.cl); this file only lays out
// buffers the way DeviceDataProperties does (dims/strides header before the
// data, the header's byte offset in the word just before the data,
// DeviceDataProperties.cpp:156-230 and 416-439; strides from
// Data::calcDataStrides, Data.cpp:1305-1343) and executes each kernel over its
// NDRange (global sizes from the Process::launch methods cited below).
#include <OpenCLIPER/kernels/hostKernelFunctions.h>

thread_local size_t gbnref_gid[3];
thread_local size_t gbnref_gsz[3];

#include "hostKernelFunctions.cl"
#include "temporalTV.cl"
#include "vectorNormalization.cl"
#include "complexElementProd.cl"
#include "xImageSum.cl"
#include "applyMask.cl"
#include "complexAbsPow2.cl"
#include "complexAbs.cl"
#include "rss.cl"
#include "initialize.cl"
#include "optimizer.cl"
#include "creabspline.cl"
#include "reductions.cl"

#include <vector>

namespace {

struct RefBuf {
  std::vector<cl_uint> words;
  size_t data_word = 0;
  void* data() { return words.data() + data_word; }
};

// header: [numSpatialDims=2, allSizesEqual=1, numCoils, numTemporalDims,
//          temporal sizes..., W, H, strides: 1, W, (coil stride N), (frame stride)]
RefBuf make(cl_uint W, cl_uint H, cl_uint C, cl_uint F, size_t elem_bytes, const void* src) {
  const cl_uint N = W * H;
  std::vector<cl_uint> hdr = {2u, 1u, C, F ? 1u : 0u};
  if (F) hdr.push_back(F);
  hdr.push_back(W);
  hdr.push_back(H);
  hdr.push_back(1u);
  hdr.push_back(W);
  hdr.push_back(N);                  // coil stride (KData) or frame stride (XData)
  if (C && F) hdr.push_back(N * C);  // frame stride of KData
  RefBuf b;
  b.data_word = ((hdr.size() + 1 + 3) / 4) * 4;
  const size_t n = size_t(N) * (C ? C : 1) * (F ? F : 1);
  const size_t data_words = (n * elem_bytes + 3) / 4;
  b.words.assign(b.data_word + data_words, 0u);
  std::memcpy(b.words.data(), hdr.data(), hdr.size() * 4);
  b.words[b.data_word - 1] = cl_uint(b.data_word * 4);
  if (src) std::memcpy(b.data(), src, n * elem_bytes);
  return b;
}

template <typename Fn>
void ndrange(size_t g0, size_t g1, size_t g2, Fn fn) {
  gbnref_gsz[0] = g0;
  gbnref_gsz[1] = g1;
  gbnref_gsz[2] = g2;
  for (size_t k = 0; k < g2; ++k)
    for (size_t j = 0; j < g1; ++j)
      for (size_t i = 0; i < g0; ++i) {
        gbnref_gid[0] = i;
        gbnref_gid[1] = j;
        gbnref_gid[2] = k;
        fn();
      }
}

}  // namespace

extern "C" {

// TemporalTV::launch (TemporalTV.cpp:59-86): global (W, H, D)
void ref_ttv(int forward, const float* in, float* out, int W, int H, int F) {
  RefBuf a = make(W, H, 0, F, 8, in), b = make(W, H, 0, F, 8, nullptr);
  ndrange(W, H, 1, [&] {
    if (forward)
      operator_tTV((float2*)a.data(), (float2*)b.data(), cl_uint(F));
    else
      operator_tTVadj((float2*)a.data(), (float2*)b.data(), cl_uint(F));
  });
  std::memcpy(out, b.data(), size_t(W) * H * F * 8);
}

// VectorNormalization::launch (VectorNormalization.cpp:56-87): global (W, H, F*D)
void ref_normalize(const float* in, float* out, int W, int H, int F, float mu) {
  RefBuf a = make(W, H, 0, F, 8, in), b = make(W, H, 0, F, 8, nullptr);
  ndrange(W, H, F, [&] { vectorNormalization((float2*)a.data(), (float2*)b.data(), mu); });
  std::memcpy(out, b.data(), size_t(W) * H * F * 8);
}

// ComplexElementProd::launch (ComplexElementProd.cpp:64-131): global W*H*D
void ref_sensmul(int conj, const float* in, int in_has_coils, const float* S, float* out, int W, int H, int F, int C) {
  RefBuf a = in_has_coils ? make(W, H, C, F, 8, in) : make(W, H, 0, F, 8, in);
  RefBuf s = make(W, H, C, 0, 8, S);
  RefBuf b = make(W, H, C, F, 8, nullptr);
  ndrange(size_t(W) * H, 1, 1, [&] {
    complexElementProd_kernel((complexType*)a.data(), (complexType*)s.data(), (complexType*)b.data(),
                              conj ? 0x80000000u : 0u);
  });
  std::memcpy(out, b.data(), size_t(W) * H * F * C * 8);
}

// XImageSum::launch (XImageSum.cpp:79-96): global W*H*D
void ref_coilsum(const float* in, float* out, int W, int H, int F, int C) {
  RefBuf a = make(W, H, C, F, 8, in), b = make(W, H, 0, F, 8, nullptr);
  ndrange(size_t(W) * H, 1, 1, [&] { xImageSum_kernel((complexType*)a.data(), (complexType*)b.data()); });
  std::memcpy(out, b.data(), size_t(W) * H * F * 8);
}

// ApplyMask::launch (ApplyMask.cpp:21-51): global = NDArray size, in place
void ref_mask(float* data, const unsigned char* mask, int W, int H, int F, int C) {
  RefBuf a = make(W, H, C, F, 8, data), m = make(W, H, 0, F, 1, mask);
  ndrange(size_t(W) * H, 1, 1, [&] { applyMask_complex((complexType*)a.data(), (const uchar*)m.data()); });
  std::memcpy(data, a.data(), size_t(W) * H * F * C * 8);
}

// ComplexAbsPow2 on KData (NestaUp.cpp:738-741), in place: global (W, H, D)
void ref_abs2(float* data, int W, int H, int F, int C) {
  RefBuf a = make(W, H, C, F, 8, data);
  ndrange(W, H, 1, [&] { ComplexAbsPow2((float2*)a.data(), (float2*)a.data()); });
  std::memcpy(data, a.data(), size_t(W) * H * F * C * 8);
}

// ComplexAbs on XData (NestaUp.cpp:523-530): global (W, H, D)
void ref_abs(const float* in, float* out, int W, int H, int F) {
  RefBuf a = make(W, H, 0, F, 8, in), b = make(W, H, 0, F, 8, nullptr);
  ndrange(W, H, 1, [&] { complexAbs((float2*)a.data(), (float2*)b.data()); });
  std::memcpy(out, b.data(), size_t(W) * H * F * 8);
}

// RSoS::launch (RSoS.cpp:58-85): global (W, H, dynamic dims), KData in, XData out
void ref_rss(const float* in, float* out, int W, int H, int F, int C) {
  RefBuf a = make(W, H, C, F, 8, in), b = make(W, H, 0, F, 8, nullptr);
  ndrange(W, H, F, [&] { rss_kernel((float2*)a.data(), (float2*)b.data()); });
  std::memcpy(out, b.data(), size_t(W) * H * F * 8);
}

// Row and column index lists of the motion-compensation rectangle, as
// Interpolator / AdjointInterpolator / InitZeroRect::launch build them
// (Interpolator.cpp:63-87): margins H/40, W/40 (integer division) around the
// 1-based bounding box bb.
struct McRect {
  std::vector<int> r1, r2;
};
McRect mc_rect(int W, int H, const int* bb) {
  const int m0 = int(std::ceil(cl_uint(H) / 40)), m1 = int(std::ceil(cl_uint(W) / 40));
  const int l1 = (bb[3] + m0 + 1) - (bb[1] - m0 - 1) + 1, l2 = (bb[2] + m1 + 1) - (bb[0] - m1 - 1) + 1;
  McRect r;
  for (int i = 0; i < l1; ++i) r.r1.push_back((bb[1] - m0 - 1) + i - 1);
  for (int j = 0; j < l2; ++j) r.r2.push_back((bb[0] - m1 - 1) + j - 1);
  return r;
}

// MotionCompensation::launch (MotionCompensation.cpp:57-78): copyDataGPU, then
// the interpolator over the rectangle.  xn [2][F][H][W], x [2][W][H] (1-based).
void ref_mc(const float* in, float* out, const float* xn, const int* x, int W, int H, int F, const int* bb) {
  RefBuf a = make(W, H, 0, F, 8, in), b = make(W, H, 0, F, 8, nullptr);
  ndrange(size_t(W) * H * F, 1, 1, [&] { copyDataGPU((float2*)b.data(), (float2*)a.data()); });
  McRect r = mc_rect(W, H, bb);
  ndrange(r.r1.size(), r.r2.size(), F, [&] {
    interpolator((float2*)b.data(), (float2*)a.data(), (float*)xn, (int*)x, r.r1.data(), r.r2.data());
  });
  std::memcpy(out, b.data(), size_t(W) * H * F * 8);
}

// AdjointMotionCompensation::launch (AdjointMotionCompensation.cpp:59-86):
// copyDataGPU, initZeroRect over the rectangle, then adjointInterpolator.
void ref_mc_adjoint(const float* in, float* out, const float* xn, const int* x, int W, int H, int F, const int* bb) {
  RefBuf a = make(W, H, 0, F, 8, in), b = make(W, H, 0, F, 8, nullptr);
  ndrange(size_t(W) * H * F, 1, 1, [&] { copyDataGPU((float2*)b.data(), (float2*)a.data()); });
  McRect r = mc_rect(W, H, bb);
  ndrange(r.r1.size(), r.r2.size(), F, [&] { initZeroRect((float2*)b.data(), r.r1.data(), r.r2.data()); });
  ndrange(r.r1.size(), r.r2.size(), F, [&] {
    adjointInterpolator((float2*)b.data(), (float2*)a.data(), (float*)xn, (int*)x, r.r1.data(), r.r2.data());
  });
  std::memcpy(out, b.data(), size_t(W) * H * F * 8);
}

}  // extern "C"

#include "registration_host.hpp"
