// Per-operator kernels: one entry per Process on the NESTA path, operating on
// the reference's dense layouts.  These back the operator-level C ABI and the
// C++ facade's sub-processes; the NESTA solver itself uses the fused kernels.
#include <algorithm>
#include <cmath>
#include <string>

#include "ctx.h"
#include "nesta_kernels.cuh"

namespace gbn {

namespace {
inline int grid_for(gbn_ctx* ctx, size_t n, int nt = 256) {
  return int(std::max<size_t>(1, std::min<size_t>((n + nt - 1) / nt, size_t(ctx->nsm) * 16)));
}
#define GRID_STRIDE(i, n) \
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < (n); i += size_t(gridDim.x) * blockDim.x)
}  // namespace

// temporalTV.cl:49-107.  One thread per (frame, pixel).
__global__ void k_ttv(const float2* __restrict__ in, float2* __restrict__ out, int N, int F, int forward) {
  const size_t n = size_t(N) * F;
  GRID_STRIDE(i, n) {
    const int f = int(i / N);
    const size_t p = i - size_t(f) * N;
    if (forward) {
      out[i] = csub(in[i], in[size_t((f + F - 1) % F) * N + p]);
    } else {
      out[i] = csub(in[size_t((f + 1) % F) * N + p], in[i]);
    }
  }
}

// vectorNormalization.cl:42-56: out = in / fmax(mu, length(in))
__global__ void k_normalize(const float2* in, float2* out, size_t n, float mu) {
  GRID_STRIDE(i, n) {
    const float2 v = in[i];
    const float m = fmaxf(mu, sqrtf(fmaf(v.x, v.x, v.y * v.y)));
    out[i] = make_float2(v.x / m, v.y / m);
  }
}

// complexElementProd.cl:42-76: out[f][c][p] = in[f][(c)][p] * (conj?)S[c][p]
__global__ void k_sensmul(const float2* in, int in_has_coils, const float2* __restrict__ S, float2* out, int N, int F,
                          int C, int conj) {
  const size_t n = size_t(N) * F * C;
  GRID_STRIDE(i, n) {
    const size_t p = i % N;
    const size_t fc = i / N;
    const int c = int(fc % C), f = int(fc / C);
    const float2 a = in_has_coils ? in[i] : in[size_t(f) * N + p];
    float2 s = S[size_t(c) * N + p];
    if (conj) s.y = -s.y;
    out[i] = make_float2(a.x * s.x - a.y * s.y, a.x * s.y + a.y * s.x);
  }
}

// xImageSum.cl:42-61: out[f][p] = sum over coils in order
__global__ void k_coilsum(const float2* __restrict__ in, float2* __restrict__ out, int N, int F, int C) {
  const size_t n = size_t(N) * F;
  GRID_STRIDE(i, n) {
    const int f = int(i / N);
    const size_t p = i - size_t(f) * N;
    float2 acc = make_float2(0.f, 0.f);
    for (int c = 0; c < C; ++c) acc = cadd(acc, in[(size_t(f) * C + c) * N + p]);
    out[i] = acc;
  }
}

// applyMask.cl:5-40
__global__ void k_mask(float2* data, const uint8_t* __restrict__ mask, int N, int F, int C) {
  const size_t n = size_t(N) * F * C;
  GRID_STRIDE(i, n) {
    const size_t p = i % N;
    const int f = int(i / (size_t(N) * C));
    if (mask[size_t(f) * N + p] == 0) data[i] = make_float2(0.f, 0.f);
  }
}

// SamplingMasksData.cpp:389-441: row value 1 -> 255, 0 -> 0, else error flag
__global__ void k_rowmask(const uint32_t* __restrict__ rm, uint8_t* __restrict__ pm, int W, int H, int F, int* bad) {
  const size_t n = size_t(W) * H * F;
  GRID_STRIDE(i, n) {
    const uint32_t v = rm[i / W];
    if (v > 1u) atomicExch(bad, 1);
    pm[i] = (v == 1u) ? uint8_t(255) : uint8_t(0);
  }
}

// complexAbs.cl:43-70 / complexAbsPow2.cl:43-71
__global__ void k_abs(const float2* in, float2* out, size_t n, int squared) {
  GRID_STRIDE(i, n) {
    const float2 v = in[i];
    const float a2 = v.x * v.x + v.y * v.y;
    out[i] = make_float2(squared ? a2 : sqrtf(a2), 0.f);
  }
}

__global__ void k_scale(float2* data, size_t n, float s) {
  GRID_STRIDE(i, n) data[i] = cscale(data[i], s);
}

// ---------------------------------------------------------------------------
int op_ttv(gbn_ctx* ctx, int dir, const float2* in, float2* out, int W, int H, int F) {
  if (in == out) return set_error(GBN_ERR_INVALID, "TemporalTV needs distinct input and output buffers");
  const size_t n = size_t(W) * H * F;
  k_ttv<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(in, out, W * H, F, dir == GBN_TTV_FORWARD);
  return cuda_status(cudaGetLastError(), "ttv");
}

int op_normalize(gbn_ctx* ctx, const float2* in, float2* out, size_t n, float mu) {
  k_normalize<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(in, out, n, mu);
  return cuda_status(cudaGetLastError(), "normalize");
}

int op_sensmul(gbn_ctx* ctx, int conj, const float2* in, int in_has_coils, const float2* S, float2* out, int W, int H,
               int F, int C) {
  if (!in_has_coils && in == out && C > 1)
    return set_error(GBN_ERR_INVALID, "XData input cannot alias the KData output");
  const size_t n = size_t(W) * H * F * C;
  k_sensmul<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(in, in_has_coils, S, out, W * H, F, C, conj);
  return cuda_status(cudaGetLastError(), "sensmul");
}

int op_coilsum(gbn_ctx* ctx, const float2* in, float2* out, int W, int H, int F, int C) {
  const size_t n = size_t(W) * H * F;
  k_coilsum<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(in, out, W * H, F, C);
  return cuda_status(cudaGetLastError(), "coilsum");
}

int op_mask(gbn_ctx* ctx, float2* data, const uint8_t* mask, int W, int H, int F, int C) {
  const size_t n = size_t(W) * H * F * C;
  k_mask<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(data, mask, W * H, F, C);
  return cuda_status(cudaGetLastError(), "mask");
}

int op_rowmask(gbn_ctx* ctx, const uint32_t* rm, uint8_t* pm, int W, int H, int F) {
  void* scr = nullptr;
  int rc = ctx_scratch(ctx, sizeof(int), &scr);
  if (rc != GBN_OK) return rc;
  int* bad = static_cast<int*>(scr);
  cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream);
  const size_t n = size_t(W) * H * F;
  k_rowmask<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(rm, pm, W, H, F, bad);
  int hbad = 0;
  cudaError_t e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "rowmask");
  if (hbad) return set_error(GBN_ERR_INVALID, "sampling mask data element must be 0 or 1");
  return GBN_OK;
}

// rss.cl:43-74 (RSoS): out[f][p] = (sqrt(sum_c |k[f][c][p]|^2), 0), the sum in
// coil order in FP32
__global__ void k_rss(const float2* __restrict__ k, float2* __restrict__ out, int N, int F, int C) {
  const size_t n = size_t(N) * F;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const size_t f = i / N, p = i - f * N;
    const float2* src = k + f * size_t(C) * N + p;
    float acc = 0.f;
    for (int c = 0; c < C; ++c) {
      const float2 v = src[size_t(c) * N];
      acc = __fadd_rn(acc, __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)));
    }
    out[i] = make_float2(sqrtf(acc), 0.f);
  }
}

int op_rss(gbn_ctx* ctx, const float2* k, float2* out, int W, int H, int F, int C) {
  k_rss<<<grid_for(ctx, size_t(W) * H * F), 256, 0, ctx->stream>>>(k, out, W * H, F, C);
  ctx->launches += 1;
  return cuda_status(cudaGetLastError(), "rss");
}

int op_fft2(gbn_ctx* ctx, int direction, const float2* in, float2* out, int W, int H, int batch);

// SimpleMRIReconSOS: backward FFT of every coil image into the context scratch
// (the input stays untouched), then the root sum of squares
int simple_recon_sos(gbn_ctx* ctx, const float2* y, float2* x, int W, int H, int F, int C) {
  void* scr = nullptr;
  int rc = ctx_scratch(ctx, size_t(W) * H * F * C * sizeof(float2), &scr);
  if (rc != GBN_OK) return rc;
  float2* t = static_cast<float2*>(scr);
  if ((rc = op_fft2(ctx, GBN_FFT_BACKWARD, y, t, W, H, F * C)) != GBN_OK) return rc;
  return op_rss(ctx, t, x, W, H, F, C);
}

int op_abs(gbn_ctx* ctx, const float2* in, float2* out, size_t n, int squared) {
  k_abs<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(in, out, n, squared);
  return cuda_status(cudaGetLastError(), "abs");
}

// 2-D FFT of `batch` W x H images: rows along W, then columns along H.
int op_fft2(gbn_ctx* ctx, int direction, const float2* in, float2* out, int W, int H, int batch) {
  const SizeKernels* kw = find_size(W);
  const SizeKernels* kh = find_size(H);
  if (!kw || !kh) return set_error(GBN_ERR_UNSUPPORTED, "unsupported FFT length");
  if (direction != GBN_FFT_FORWARD && direction != GBN_FFT_BACKWARD)
    return set_error(GBN_ERR_INVALID, "FFT direction must be FORWARD or BACKWARD");
  const int inv = direction == GBN_FFT_BACKWARD;
  const long long nrows = (long long)batch * H;
  const int g = int(std::max<long long>(1, std::min<long long>((nrows + kw->rows_per_cta - 1) / kw->rows_per_cta,
                                                                (long long)ctx->nsm * 8)));
  kw->fft_rows(in, out, int(nrows), inv, 1.0f, ctx_twiddles(ctx, W), g, ctx->stream);
  const float scale = inv ? 1.0f / float(W * H) : 1.0f;
  kh->fft_cols(out, out, W, batch, inv, scale, ctx_twiddles(ctx, H), ctx->stream);
  return cuda_status(cudaGetLastError(), "fft2");
}

// operatorA + 1/sqrt(N): k = mask * FFT2(S x) / sqrt(N)
int op_encode(gbn_ctx* ctx, const float2* x, const float2* S, const uint8_t* mask, float2* k, int W, int H, int F,
              int C) {
  int rc;
  if ((rc = op_sensmul(ctx, 0, x, 0, S, k, W, H, F, C)) != GBN_OK) return rc;
  if ((rc = op_fft2(ctx, GBN_FFT_FORWARD, k, k, W, H, F * C)) != GBN_OK) return rc;
  if ((rc = op_mask(ctx, k, mask, W, H, F, C)) != GBN_OK) return rc;
  const size_t n = size_t(W) * H * F * C;
  k_scale<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(k, n, float(1.0 / std::sqrt(double(unsigned(W * H)))));
  return cuda_status(cudaGetLastError(), "encode");
}

// sqrt(N) pre-scale + operatorAt: x = sum_c conj(S_c) IFFT2(sqrt(N) k_c)
int op_encode_adjoint(gbn_ctx* ctx, const float2* k, const float2* S, float2* x, int W, int H, int F, int C) {
  const size_t n = size_t(W) * H * F * C;
  void* scr = nullptr;
  int rc = ctx_scratch(ctx, n * sizeof(float2), &scr);
  if (rc != GBN_OK) return rc;
  float2* aux = static_cast<float2*>(scr);
  cudaError_t e = cudaMemcpyAsync(aux, k, n * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "encode_adjoint copy");
  k_scale<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(aux, n, std::sqrt(float(W * H)));
  if ((rc = op_fft2(ctx, GBN_FFT_BACKWARD, aux, aux, W, H, F * C)) != GBN_OK) return rc;
  if ((rc = op_sensmul(ctx, 1, aux, 1, S, aux, W, H, F, C)) != GBN_OK) return rc;
  return op_coilsum(ctx, aux, x, W, H, F, C);
}

}  // namespace gbn
