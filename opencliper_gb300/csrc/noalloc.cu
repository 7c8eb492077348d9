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
// row tables, the one-entry instance table and the row pass's control block.
// Every call reuses it: kernels of the call rewrite the tables and reset the
// control block before anything reads them.  Calls whose work overlaps on the
// GPU (different streams, or several host threads) share the one array and
// race; serialise them.  The array's device address is resolved on the first
// call on each device and kept for the life of the process, so the entry point
// must not be used across cudaDeviceReset (nor may any other object of this
// library: contexts hold streams of the device's primary context).
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "ctx.h"
#include "nesta_kernels.cuh"

namespace gbn {

size_t simple_recon_bytes(int W, int H, int F, int C);
int simple_recon_in(gbn_ctx* ctx, void* ws, const float2* y, const float2* S, float2* x, int W, int H, int F, int C,
                    bool tables_valid);

namespace {

// limits of the static scratch
constexpr size_t kStaticMaxT = size_t(1) << 20;  // complex elements of the intermediates: F*H*C*W
constexpr size_t kStaticMaxRows = 8192;          // F*H
constexpr size_t kStaticTBytes = kStaticMaxT * sizeof(float2);
constexpr size_t kStaticIntBytes = ((5 * kStaticMaxRows + 1) * sizeof(int) + 255) / 256 * 256;
// state block, instance table and control block, each rounded to 256 bytes
constexpr size_t kStaticSmallBytes = 4096;
static_assert(((sizeof(NestaDevState) + 255) / 256 + (sizeof(FusedArgs) + 255) / 256 + (sizeof(ClassCtl) + 255) / 256) *
                      256 <= kStaticSmallBytes,
              "static scratch tail too small");
constexpr size_t kStaticScratchBytes = kStaticTBytes + kStaticIntBytes + kStaticSmallBytes;

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
  const size_t FH = size_t(F) * H, K = FH * C * W;
  if (K > kStaticMaxT || FH > kStaticMaxRows)
    return set_error(GBN_ERR_UNSUPPORTED,
                     "gbn_simple_recon_static: problem exceeds the static scratch (F*H*C*W <= " +
                         std::to_string(kStaticMaxT) + " and F*H <= " + std::to_string(kStaticMaxRows) +
                         "; got " + std::to_string(K) + " and " + std::to_string(FH) + ")");
  void* base = nullptr;
  const int rc = static_scratch(ctx->device, &base);
  if (rc != GBN_OK) return rc;
  if (simple_recon_bytes(W, H, F, C) > kStaticScratchBytes)
    return set_error(GBN_ERR_UNSUPPORTED, "gbn_simple_recon_static: problem exceeds the static scratch");
  return simple_recon_in(ctx, base, y, S, x, W, H, F, C, false);  // the array is shared between contexts
}

}  // namespace gbn

extern "C" GBN_API int gbn_simple_recon_static(gbn_ctx* ctx, const float* d_y, const float* d_S, float* d_x, int W,
                                               int H, int F, int C) {
  using namespace gbn;
  if (!ctx) return set_error(GBN_ERR_INVALID, "null context");
  if (!d_y || !d_x) return set_error(GBN_ERR_INVALID, "null buffer");
  if (!d_S) return set_error(GBN_ERR_INVALID, "missing sensitivity maps");
  int rc = check_dims(W, H, F, C);
  if (rc == GBN_OK) rc = check_fft(W, H);
  if (rc != GBN_OK) return rc;
  DeviceGuard guard(ctx->device);  // the caller's current device is restored on return
  return simple_recon_static(ctx, reinterpret_cast<const float2*>(d_y), reinterpret_cast<const float2*>(d_S),
                             reinterpret_cast<float2*>(d_x), W, H, F, C);
}
