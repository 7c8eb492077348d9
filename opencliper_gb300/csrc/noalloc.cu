// SimpleMRIRecon without any device allocation.
//
// Some callers cannot call cudaMalloc at reconstruction time: code that runs
// while a stream is being captured into a CUDA graph (allocation is not a
// capturable operation), real-time reconstruction hosts that hand out device
// memory only from their own fixed pools, and plugins whose host application
// forbids allocation after start-up.  gbn_simple_recon_static serves them: the
// caller passes only the input k-space, the sensitivity maps and the output
// image, and the working memory comes from a fixed array compiled into the
// library (kStaticScratchBytes, about 8.2 MiB on every device that loads the
// library, held until the process exits).
//
// The scratch holds the row-pass intermediates (F*H*C*W complex values), the
// row tables and a small state block.  Every call reuses it: the state block
// is cleared at the start of each call, the rest is fully rewritten before it
// is read.  Calls whose work overlaps on the GPU (different streams, or several
// host threads) share the one array and race; serialise them.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "ctx.h"
#include "nesta_kernels.cuh"

namespace gbn {

void launch_rows_identity(int H, int F, int* rowmap, int* rowoff, int* rows_h, int* rows_f, int* row_full,
                          cudaStream_t s);

namespace {

// limits of the static scratch
constexpr size_t kStaticMaxT = size_t(1) << 20;  // complex elements of the intermediates: F*H*C*W
constexpr size_t kStaticMaxRows = 8192;          // F*H
constexpr size_t kStaticTBytes = kStaticMaxT * sizeof(float2);
constexpr size_t kStaticIntBytes = (4 * kStaticMaxRows + kStaticMaxRows + 1) * sizeof(int);
constexpr size_t kStaticStateOff = ((kStaticTBytes + kStaticIntBytes + 255) / 256) * 256;
constexpr size_t kStaticScratchBytes = kStaticStateOff + ((sizeof(NestaDevState) + 255) / 256) * 256;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// device address of g_static_scratch, resolved once per device
std::mutex g_static_mu;
void* g_static_addr[64] = {};

int static_scratch(int device, void** out) {
  if (device < 0 || device >= 64) return set_error(GBN_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_addr[device]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(static scratch)");
    g_static_addr[device] = ptr;
  }
  *out = g_static_addr[device];
  return GBN_OK;
}

}  // namespace

int simple_recon_static(gbn_ctx* ctx, const float2* y, const float2* S, float2* x, int W, int H, int F, int C) {
  const SizeKernels* kh = find_size(H);
  const SizeKernels* kw = find_size(W);
  if (!kh || !kw) return set_error(GBN_ERR_UNSUPPORTED, "unsupported FFT length");
  const size_t FH = size_t(F) * H, K = FH * C * W;
  if (K > kStaticMaxT || FH > kStaticMaxRows)
    return set_error(GBN_ERR_UNSUPPORTED,
                     "gbn_simple_recon_static: problem exceeds the static scratch (F*H*C*W <= " +
                         std::to_string(kStaticMaxT) + " and F*H <= " + std::to_string(kStaticMaxRows) +
                         "; got " + std::to_string(K) + " and " + std::to_string(FH) + ")");
  void* base = nullptr;
  int rc = static_scratch(ctx->device, &base);
  if (rc != GBN_OK) return rc;
  unsigned char* b = static_cast<unsigned char*>(base);
  float2* T = reinterpret_cast<float2*>(b);
  int* rowmap = reinterpret_cast<int*>(b + kStaticTBytes);
  int* rows_h = rowmap + kStaticMaxRows;
  int* rows_f = rows_h + kStaticMaxRows;
  int* row_full = rows_f + kStaticMaxRows;
  int* rowoff = row_full + kStaticMaxRows;
  NestaDevState* st = reinterpret_cast<NestaDevState*>(b + kStaticStateOff);
  cudaStream_t s = ctx->stream;
  // the row pass's work counter and ticket must start at zero on every call
  cudaError_t e = cudaMemsetAsync(st, 0, sizeof(NestaDevState), s);
  if (e != cudaSuccess) return cuda_status(e, "static scratch reset");

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
  const long long rows = (long long)FH * C;
  const int g2 = int(std::max<long long>(
      1, std::min<long long>((rows + kw->rows_per_cta - 1) / kw->rows_per_cta, (long long)ctx->nsm * ctx->k2_ctas_per_sm)));
  launch_rows_identity(H, F, rowmap, rowoff, rows_h, rows_f, row_full, s);
  kw->rows(a, 0, false, g2, s);
  kh->inv_cols(a, 0, false, dim3(W / kWB, 2, F), s);
  ctx->launches += 3;
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "static simple recon launch");
  return GBN_OK;
}

}  // namespace gbn

extern "C" GBN_API int gbn_simple_recon_static(gbn_ctx* ctx, const float* d_y, const float* d_S, float* d_x, int W,
                                               int H, int F, int C) {
  using namespace gbn;
  if (!ctx) return set_error(GBN_ERR_INVALID, "null context");
  if (!d_y || !d_x) return set_error(GBN_ERR_INVALID, "null buffer");
  if (!d_S) return set_error(GBN_ERR_INVALID, "missing sensitivity maps");
  if (W <= 0 || H <= 0 || F <= 0 || C <= 0) return set_error(GBN_ERR_INVALID, "dimensions must be positive");
  if (W % 8 != 0) return set_error(GBN_ERR_INVALID, "NDArray dimension 0 (width) is not multiple of 8");
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess || cur != ctx->device) {
    const cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  }
  return simple_recon_static(ctx, reinterpret_cast<const float2*>(d_y), reinterpret_cast<const float2*>(d_S),
                             reinterpret_cast<float2*>(d_x), W, H, F, C);
}
