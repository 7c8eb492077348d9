// C ABI (include/gbn.h): argument checking, status codes and error strings
// around the operator and solver entry points.
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "fft.cuh"

namespace gbn {

int op_ttv(gbn_ctx*, int, const float2*, float2*, int, int, int);
int op_normalize(gbn_ctx*, const float2*, float2*, size_t, float);
int op_sensmul(gbn_ctx*, int, const float2*, int, const float2*, float2*, int, int, int, int);
int op_coilsum(gbn_ctx*, const float2*, float2*, int, int, int, int);
int op_mask(gbn_ctx*, float2*, const uint8_t*, int, int, int, int);
int op_rowmask(gbn_ctx*, const uint32_t*, uint8_t*, int, int, int);
int op_abs(gbn_ctx*, const float2*, float2*, size_t, int);
int op_fft2(gbn_ctx*, int, const float2*, float2*, int, int, int);
int op_rss(gbn_ctx*, const float2*, float2*, int, int, int, int);
int simple_recon_sos(gbn_ctx*, const float2*, float2*, int, int, int, int);
int op_encode(gbn_ctx*, const float2*, const float2*, const uint8_t*, float2*, int, int, int, int);
int op_encode_adjoint(gbn_ctx*, const float2*, const float2*, float2*, int, int, int, int);
int simple_recon(gbn_ctx*, const float2*, const float2*, float2*, int, int, int, int);
int problem_alloc(gbn_problem*);
void problem_free(gbn_problem*);
int validate_problem_dims(int, int, int, int);
int nesta_run(gbn_ctx*, gbn_problem*, const gbn_nesta_params*, float2*, gbn_nesta_stats*);
int batch_create(gbn_ctx*, int, gbn_problem* const*, const gbn_nesta_params*, float* const*, int, gbn_batch**);
int batch_launch(gbn_batch*);
int batch_capture(gbn_batch*);
int batch_stats(gbn_batch*, int, gbn_nesta_stats*);
int batch_destroy(gbn_batch*);
gbn_ctx* batch_ctx(gbn_batch*);
int batch_groups(gbn_batch*, int*, int*);
int batch_group_info(gbn_batch*, int, int*, int*, int*, int*, int*);
int motion_set(gbn_problem*, const float*, const int*, const int*);
int problem_fit_rows(gbn_problem*, int, int*);
int motion_op(gbn_ctx*, int, const float2*, float2*, const float*, const int*, const int*, int, int, int);
int registration_info(int, int, const gbn_registration_params*, gbn_registration_info*);
int registration_run(gbn_ctx*, const float2*, int, int, const gbn_registration_params*, const float*, float*, float*,
                     int*, float*, gbn_registration_stats*);
int autotune(gbn_ctx*, int, const int*, const char*);
int autotune_load(gbn_ctx*, const char*);
void tuning_for(gbn_ctx*, int, int, int, int, int*, int*);
int read_stats(gbn_problem*, cudaStream_t, gbn_nesta_stats*);

namespace {
thread_local std::string g_err;

// cached device buffers of gbn_nesta_run_host
struct HostRunCache {
  int W = 0, H = 0, F = 0, C = 0;
  float2 *y = nullptr, *S = nullptr, *x = nullptr;
  uint8_t* mask = nullptr;
  gbn_problem* prob = nullptr;
};
std::vector<std::pair<gbn_ctx*, HostRunCache*>> g_host_cache;

void free_host_cache(gbn_ctx* ctx) {
  for (auto it = g_host_cache.begin(); it != g_host_cache.end(); ++it) {
    if (it->first != ctx) continue;
    HostRunCache* c = it->second;
    if (c->prob) {
      problem_free(c->prob);
      delete c->prob;
    }
    cudaFree(c->y);
    cudaFree(c->S);
    cudaFree(c->x);
    cudaFree(c->mask);
    delete c;
    g_host_cache.erase(it);
    return;
  }
}

#define CHECK_CTX(ctx) \
  if (!(ctx)) return set_error(GBN_ERR_INVALID, "null context"); \
  DeviceGuard guard_((ctx)->device)

}  // namespace

int set_error(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return GBN_OK;
  cudaGetLastError();
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? GBN_ERR_NOMEM : GBN_ERR_CUDA;
}

const float2* ctx_twiddles(gbn_ctx* ctx, int L) {
  auto it = ctx->tw.find(L);
  return it == ctx->tw.end() ? nullptr : it->second;
}

namespace {
cudaEvent_t prof_event(gbn_ctx* ctx) {
  cudaEvent_t ev = nullptr;
  if (!ctx->prof_pool.empty()) {
    ev = ctx->prof_pool.back();
    ctx->prof_pool.pop_back();
  } else if (cudaEventCreate(&ev) != cudaSuccess) {
    cudaGetLastError();
    ev = nullptr;
  }
  return ev;
}
}  // namespace

void prof_begin(gbn_ctx* ctx, int, cudaEvent_t* ev) {
  *ev = prof_event(ctx);
  if (*ev) cudaEventRecord(*ev, ctx->stream);
}

void prof_end(gbn_ctx* ctx, int kind, cudaEvent_t start) {
  cudaEvent_t stop = prof_event(ctx);
  if (!start || !stop) return;
  cudaEventRecord(stop, ctx->stream);
  ctx->prof_pending.push_back({kind, start, stop});
}

int prof_collect(gbn_ctx* ctx) {
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "profile collect");
  for (auto& p : ctx->prof_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess && p.kind >= 0 && p.kind < 8) {
      ctx->prof_ms[p.kind] += ms;
      ctx->prof_count[p.kind] += 1;
    }
    ctx->prof_pool.push_back(p.start);
    ctx->prof_pool.push_back(p.stop);
  }
  ctx->prof_pending.clear();
  cudaGetLastError();
  return GBN_OK;
}

int ctx_scratch(gbn_ctx* ctx, size_t bytes, void** out, int user) {
  ctx->scratch_user = user;
  if (bytes > ctx->scratch_bytes) {
    if (ctx->scratch) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->scratch);
    }
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&ctx->scratch, bytes);
    if (e != cudaSuccess) return cuda_status(e, "scratch allocation");
    ctx->scratch_bytes = bytes;
  }
  *out = ctx->scratch;
  return GBN_OK;
}

int host_flags_ready(gbn_ctx* ctx) {
  if (ctx->host_flags) return GBN_OK;
  cudaError_t e = cudaHostAlloc(&ctx->host_flags, 2 * sizeof(int), cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_flag[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_flag[1], cudaEventDisableTiming);
  return cuda_status(e, "pinned stop flags");
}

}  // namespace gbn

using namespace gbn;

extern "C" {

const char* gbn_last_error_string(void) { return g_err.c_str(); }
int gbn_version(void) { return GBN_VERSION; }
int gbn_supported_lengths(int* out, int cap) { return supported_sizes(out, cap); }

int gbn_ctx_create(int device, gbn_ctx** out) {
  if (!out) return set_error(GBN_ERR_INVALID, "null output pointer");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDeviceCount");
  if (device < 0 || device >= ndev) return set_error(GBN_ERR_INVALID, "no such device: " + std::to_string(device));
  DeviceGuard guard(device);
  if ((e = cudaSetDevice(device)) != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  gbn_ctx* ctx = new gbn_ctx();
  ctx->device = device;
  if ((e = cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    delete ctx;
    return cuda_status(e, "context setup");
  }
  // two-pass twiddle tables for every supported length L = A*B:
  // [k1*B + s] = w_L^(s*k1) (k1 < A, s < B) and [L + k1'*A + s'] = w_L^(s'*k1')
  // (k1' < B, s' < A), w_L^j = (cos, -sin)(2 pi j / L)
  int lens[64];
  const int nl = supported_sizes(lens, 64);
  size_t total = 0;
  for (int i = 0; i < nl; ++i) total += 2 * size_t(lens[i]);
  std::vector<float2> h(total);
  size_t off = 0;
  std::vector<size_t> offs(nl);
  auto w = [](long long j, long long L) { return make_float2(float(cx_cos2pi(j, L)), -float(cx_sin2pi(j, L))); };
  for (int i = 0; i < nl; ++i) {
    const int L = lens[i], A = split_a(L), B = split_b(L);
    offs[i] = off;
    for (int k1 = 0; k1 < A; ++k1)
      for (int s = 0; s < B; ++s) h[off + size_t(k1) * B + s] = w((long long)s * k1, L);
    for (int k1 = 0; k1 < B; ++k1)
      for (int s = 0; s < A; ++s) h[off + L + size_t(k1) * A + s] = w((long long)s * k1, L);
    off += 2 * size_t(L);
  }
  if ((e = cudaMalloc(&ctx->tw_block, total * sizeof(float2))) != cudaSuccess ||
      (e = cudaMemcpy(ctx->tw_block, h.data(), total * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return cuda_status(e, "twiddle tables");
  }
  for (int i = 0; i < nl; ++i) ctx->tw[lens[i]] = ctx->tw_block + offs[i];
  *out = ctx;
  return GBN_OK;
}

int gbn_ctx_destroy(gbn_ctx* ctx) {
  CHECK_CTX(ctx);
  cudaStreamSynchronize(ctx->stream);
  free_host_cache(ctx);
  for (auto& p : ctx->prof_pending) {
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  for (cudaEvent_t ev : ctx->prof_pool) cudaEventDestroy(ev);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->tw_block) cudaFree(ctx->tw_block);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  if (ctx->mc_stream) {
    cudaStreamSynchronize(ctx->mc_stream);
    cudaStreamDestroy(ctx->mc_stream);
  }
  if (ctx->host_flags) cudaFreeHost(ctx->host_flags);
  if (ctx->host_partial) cudaFreeHost(ctx->host_partial);
  if (ctx->ev_partial) cudaEventDestroy(ctx->ev_partial);
  for (cudaEvent_t x : ctx->ev_flag)
    if (x) cudaEventDestroy(x);
  if (ctx->ev_mc_x) cudaEventDestroy(ctx->ev_mc_x);
  if (ctx->ev_mc_tv) cudaEventDestroy(ctx->ev_mc_tv);
  if (ctx->ev_mc_adj) cudaEventDestroy(ctx->ev_mc_adj);
  if (ctx->ev_compute) cudaEventDestroy(ctx->ev_compute);
  if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
  delete ctx;
  return GBN_OK;
}

int gbn_ctx_get_stream(gbn_ctx* ctx, void** stream) {
  CHECK_CTX(ctx);
  if (!stream) return set_error(GBN_ERR_INVALID, "null output pointer");
  *stream = ctx->stream;
  return GBN_OK;
}

int gbn_ctx_set_stream(gbn_ctx* ctx, void* stream) {
  CHECK_CTX(ctx);
  if (stream) {
    if (ctx->own_stream) {
      cudaStreamSynchronize(ctx->stream);
      cudaStreamDestroy(ctx->stream);
    }
    ctx->stream = static_cast<cudaStream_t>(stream);
    ctx->own_stream = false;
  } else if (!ctx->own_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamCreate");
    ctx->own_stream = true;
  }
  return GBN_OK;
}

int gbn_ctx_sync(gbn_ctx* ctx) {
  CHECK_CTX(ctx);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess && ctx->copy_stream) e = cudaStreamSynchronize(ctx->copy_stream);
  if (e == cudaSuccess && ctx->mc_stream) e = cudaStreamSynchronize(ctx->mc_stream);
  return cuda_status(e, "stream synchronize");
}

int gbn_ctx_seed48(gbn_ctx* ctx, const unsigned short seed16v[3]) {
  CHECK_CTX(ctx);
  if (!seed16v) return set_error(GBN_ERR_INVALID, "null seed");
  ctx->rand48 = uint64_t(seed16v[0]) | (uint64_t(seed16v[1]) << 16) | (uint64_t(seed16v[2]) << 32);
  return GBN_OK;
}

int gbn_ctx_get_rand48(gbn_ctx* ctx, unsigned short state16v[3]) {
  CHECK_CTX(ctx);
  if (!state16v) return set_error(GBN_ERR_INVALID, "null output");
  state16v[0] = (unsigned short)(ctx->rand48 & 0xffff);
  state16v[1] = (unsigned short)((ctx->rand48 >> 16) & 0xffff);
  state16v[2] = (unsigned short)((ctx->rand48 >> 32) & 0xffff);
  return GBN_OK;
}

int gbn_ctx_set_tuning(gbn_ctx* ctx, const char* key, int value) {
  CHECK_CTX(ctx);
  if (!key) return set_error(GBN_ERR_INVALID, "null key");
  if (!std::strcmp(key, "mixed_adjoint_tc")) {
    if (value != 0 && value != 1) return set_error(GBN_ERR_INVALID, "mixed_adjoint_tc is 0 or 1");
    ctx->mixed_adjoint_tc = value;
    return GBN_OK;
  }
  if (!std::strcmp(key, "row_local")) {
    if (value != 0 && value != 1) return set_error(GBN_ERR_INVALID, "row_local is 0 or 1");
    ctx->row_local = value;
    return GBN_OK;
  }
  if (!std::strcmp(key, "mixed_fwd_tc")) {
    if (value < -1 || value > 1) return set_error(GBN_ERR_INVALID, "mixed_fwd_tc is -1, 0 or 1");
    ctx->mixed_fwd_tc = value;
    return GBN_OK;
  }
  if (value < 1) return set_error(GBN_ERR_INVALID, "tuning values must be >= 1");
  if (!std::strcmp(key, "k1_coils_per_block"))
    ctx->k1_coils_per_block = value;
  else if (!std::strcmp(key, "k2_ctas_per_sm"))
    ctx->k2_ctas_per_sm = value;
  else
    return set_error(GBN_ERR_INVALID, std::string("unknown tuning key: ") + key);
  return GBN_OK;
}

int gbn_ctx_launch_count(gbn_ctx* ctx, unsigned long long* count) {
  CHECK_CTX(ctx);
  if (!count) return set_error(GBN_ERR_INVALID, "null output pointer");
  *count = ctx->launches;
  return GBN_OK;
}

int gbn_ctx_profile(gbn_ctx* ctx, int enable) {
  CHECK_CTX(ctx);
  if (!enable && ctx->profile) {
    int rc = prof_collect(ctx);
    if (rc) return rc;
  }
  ctx->profile = enable != 0;
  return GBN_OK;
}

int gbn_ctx_profile_read(gbn_ctx* ctx, int kind, unsigned long long* launches, double* total_ms) {
  CHECK_CTX(ctx);
  if (kind < 0 || kind >= GBN_PROF_KINDS) return set_error(GBN_ERR_INVALID, "unknown profile kind");
  int rc = prof_collect(ctx);
  if (rc) return rc;
  if (launches) *launches = ctx->prof_count[kind];
  if (total_ms) *total_ms = ctx->prof_ms[kind];
  return GBN_OK;
}

int gbn_ctx_profile_reset(gbn_ctx* ctx) {
  CHECK_CTX(ctx);
  int rc = prof_collect(ctx);
  if (rc) return rc;
  for (int i = 0; i < 8; ++i) {
    ctx->prof_ms[i] = 0.0;
    ctx->prof_count[i] = 0;
  }
  return GBN_OK;
}

int gbn_alloc(gbn_ctx* ctx, size_t bytes, void** d_ptr) {
  CHECK_CTX(ctx);
  if (!d_ptr) return set_error(GBN_ERR_INVALID, "null output pointer");
  *d_ptr = nullptr;
  return cuda_status(cudaMalloc(d_ptr, bytes ? bytes : 1), "cudaMalloc");
}

int gbn_free(gbn_ctx* ctx, void* d_ptr) {
  CHECK_CTX(ctx);
  cudaStreamSynchronize(ctx->stream);
  return cuda_status(cudaFree(d_ptr), "cudaFree");
}

int gbn_upload(gbn_ctx* ctx, void* d_dst, const void* h_src, size_t bytes) {
  CHECK_CTX(ctx);
  if ((!d_dst || !h_src) && bytes) return set_error(GBN_ERR_INVALID, "null buffer");
  return cuda_status(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
}

int gbn_download(gbn_ctx* ctx, void* h_dst, const void* d_src, size_t bytes) {
  CHECK_CTX(ctx);
  if ((!h_dst || !d_src) && bytes) return set_error(GBN_ERR_INVALID, "null buffer");
  cudaError_t e = cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return cuda_status(e, "download");
}

int gbn_download_async(gbn_ctx* ctx, void* h_dst, const void* d_src, size_t bytes) {
  CHECK_CTX(ctx);
  if ((!h_dst || !d_src) && bytes) return set_error(GBN_ERR_INVALID, "null buffer");
  return cuda_status(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download");
}

namespace {
int copy_stream_ready(gbn_ctx* ctx) {
  if (ctx->copy_stream) return GBN_OK;
  DeviceGuard guard(ctx->device);
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_compute, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming);
  return cuda_status(e, "copy stream");
}
}  // namespace

int gbn_copy_upload(gbn_ctx* ctx, void* d_dst, const void* h_src, size_t bytes) {
  CHECK_CTX(ctx);
  if ((!d_dst || !h_src) && bytes) return set_error(GBN_ERR_INVALID, "null buffer");
  const int rc = copy_stream_ready(ctx);
  if (rc != GBN_OK) return rc;
  return cuda_status(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, ctx->copy_stream), "prefetch");
}

int gbn_copy_wait_compute(gbn_ctx* ctx) {
  CHECK_CTX(ctx);
  const int rc = copy_stream_ready(ctx);
  if (rc != GBN_OK) return rc;
  cudaError_t e = cudaEventRecord(ctx->ev_compute, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_compute, 0);
  return cuda_status(e, "copy stream wait");
}

int gbn_compute_wait_copy(gbn_ctx* ctx) {
  CHECK_CTX(ctx);
  const int rc = copy_stream_ready(ctx);
  if (rc != GBN_OK) return rc;
  cudaError_t e = cudaEventRecord(ctx->ev_copy, ctx->copy_stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->ev_copy, 0);
  return cuda_status(e, "compute stream wait");
}

int gbn_memset(gbn_ctx* ctx, void* d_dst, int value, size_t bytes) {
  CHECK_CTX(ctx);
  return cuda_status(cudaMemsetAsync(d_dst, value, bytes, ctx->stream), "memset");
}

int gbn_host_alloc(size_t bytes, void** h_ptr) {
  if (!h_ptr) return set_error(GBN_ERR_INVALID, "null output pointer");
  return cuda_status(cudaMallocHost(h_ptr, bytes ? bytes : 1), "cudaMallocHost");
}

int gbn_host_free(void* h_ptr) { return cuda_status(cudaFreeHost(h_ptr), "cudaFreeHost"); }

#define F2(p) reinterpret_cast<float2*>(p)
#define CF2(p) reinterpret_cast<const float2*>(p)
#define NONNULL2(a, b) \
  if (!(a) || !(b)) return set_error(GBN_ERR_INVALID, "null buffer")

int gbn_op_ttv(gbn_ctx* ctx, int direction, const float* d_in, float* d_out, int W, int H, int F) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  int rc = check_dims(W, H, F, 1);
  if (rc) return rc;
  if (direction != GBN_TTV_FORWARD && direction != GBN_TTV_ADJOINT)
    return set_error(GBN_ERR_INVALID, "TemporalTV direction must be FORWARD or ADJOINT");
  return op_ttv(ctx, direction, CF2(d_in), F2(d_out), W, H, F);
}

int gbn_op_normalize(gbn_ctx* ctx, const float* d_in, float* d_out, size_t n, float mu) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  return op_normalize(ctx, CF2(d_in), F2(d_out), n, mu);
}

int gbn_op_sensmul(gbn_ctx* ctx, int conjugate, const float* d_in, int in_has_coils, const float* d_S, float* d_out,
                   int W, int H, int F, int C) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  if (!d_S) return set_error(GBN_ERR_INVALID, "ComplexElementProd::launch: non-existing SensitivityMaps");
  int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  return op_sensmul(ctx, conjugate ? 1 : 0, CF2(d_in), in_has_coils ? 1 : 0, CF2(d_S), F2(d_out), W, H, F, C);
}

int gbn_op_coilsum(gbn_ctx* ctx, const float* d_in, float* d_out, int W, int H, int F, int C) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  return op_coilsum(ctx, CF2(d_in), F2(d_out), W, H, F, C);
}

int gbn_op_mask(gbn_ctx* ctx, float* d_data, const uint8_t* d_mask, int W, int H, int F, int C) {
  CHECK_CTX(ctx);
  if (!d_data) return set_error(GBN_ERR_INVALID, "null buffer");
  if (!d_mask) return set_error(GBN_ERR_INVALID, "Empty sampling masks data");
  int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  return op_mask(ctx, F2(d_data), d_mask, W, H, F, C);
}

int gbn_op_rowmask_to_pixelmask(gbn_ctx* ctx, const uint32_t* d_rowmask, uint8_t* d_pixmask, int W, int H, int F) {
  CHECK_CTX(ctx);
  NONNULL2(d_rowmask, d_pixmask);
  int rc = check_dims(W, H, F, 1);
  if (rc) return rc;
  return op_rowmask(ctx, d_rowmask, d_pixmask, W, H, F);
}

int gbn_op_abs(gbn_ctx* ctx, const float* d_in, float* d_out, size_t n) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  return op_abs(ctx, CF2(d_in), F2(d_out), n, 0);
}

int gbn_op_abs2(gbn_ctx* ctx, const float* d_in, float* d_out, size_t n) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  return op_abs(ctx, CF2(d_in), F2(d_out), n, 1);
}

int gbn_op_fft2(gbn_ctx* ctx, int direction, const float* d_in, float* d_out, int W, int H, int batch) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  int rc = check_dims(W, H, batch, 1);
  if (rc) return rc;
  if ((rc = check_fft(W, H))) return rc;
  return op_fft2(ctx, direction, CF2(d_in), F2(d_out), W, H, batch);
}

int gbn_op_encode(gbn_ctx* ctx, const float* d_x, const float* d_S, const uint8_t* d_mask, float* d_k, int W, int H,
                  int F, int C) {
  CHECK_CTX(ctx);
  NONNULL2(d_x, d_k);
  if (!d_S || !d_mask) return set_error(GBN_ERR_INVALID, "missing sensitivity maps or sampling masks");
  int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  if ((rc = check_fft(W, H))) return rc;
  return op_encode(ctx, CF2(d_x), CF2(d_S), d_mask, F2(d_k), W, H, F, C);
}

int gbn_op_encode_adjoint(gbn_ctx* ctx, const float* d_k, const float* d_S, float* d_x, int W, int H, int F, int C) {
  CHECK_CTX(ctx);
  NONNULL2(d_k, d_x);
  if (!d_S) return set_error(GBN_ERR_INVALID, "missing sensitivity maps");
  int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  if ((rc = check_fft(W, H))) return rc;
  return op_encode_adjoint(ctx, CF2(d_k), CF2(d_S), F2(d_x), W, H, F, C);
}

int gbn_simple_recon(gbn_ctx* ctx, const float* d_y, const float* d_S, float* d_x, int W, int H, int F, int C) {
  CHECK_CTX(ctx);
  NONNULL2(d_y, d_x);
  if (!d_S) return set_error(GBN_ERR_INVALID, "missing sensitivity maps");
  int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  if ((rc = check_fft(W, H))) return rc;
  return simple_recon(ctx, CF2(d_y), CF2(d_S), F2(d_x), W, H, F, C);
}

int gbn_op_rss(gbn_ctx* ctx, const float* d_k, float* d_x, int W, int H, int F, int C) {
  CHECK_CTX(ctx);
  NONNULL2(d_k, d_x);
  const int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  return op_rss(ctx, CF2(d_k), F2(d_x), W, H, F, C);
}

int gbn_simple_recon_sos(gbn_ctx* ctx, const float* d_y, float* d_x, int W, int H, int F, int C) {
  CHECK_CTX(ctx);
  NONNULL2(d_y, d_x);
  int rc = check_dims(W, H, F, C);
  if (rc) return rc;
  if ((rc = check_fft(W, H))) return rc;
  return simple_recon_sos(ctx, CF2(d_y), F2(d_x), W, H, F, C);
}

int gbn_problem_create(gbn_ctx* ctx, int W, int H, int F, int C, const float* d_y, const float* d_S,
                       const uint8_t* d_mask, gbn_problem** out) {
  CHECK_CTX(ctx);
  if (!out) return set_error(GBN_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (!d_y) return set_error(GBN_ERR_INVALID, "null KData buffer");
  if (!d_S) return set_error(GBN_ERR_INVALID, "ComplexElementProd::launch: non-existing SensitivityMaps");
  if (!d_mask) return set_error(GBN_ERR_INVALID, "Empty sampling masks data");
  int rc = validate_problem_dims(W, H, F, C);
  if (rc) return rc;
  gbn_problem* p = new gbn_problem();
  p->ctx = ctx;
  p->W = W;
  p->H = H;
  p->F = F;
  p->C = C;
  p->y = CF2(d_y);
  p->S = CF2(d_S);
  p->mask = d_mask;
  if ((rc = problem_alloc(p)) != GBN_OK) {
    problem_free(p);
    delete p;
    return rc;
  }
  *out = p;
  return GBN_OK;
}

int gbn_op_motion(gbn_ctx* ctx, int direction, const float* d_in, float* d_out, const float* d_xn, const int* d_xmesh,
                  const int bound_box[4], int W, int H, int F) {
  CHECK_CTX(ctx);
  NONNULL2(d_in, d_out);
  if (!d_xn || !d_xmesh || !bound_box) return set_error(GBN_ERR_INVALID, "null mesh or bounding box");
  if (direction != GBN_TTV_FORWARD && direction != GBN_TTV_ADJOINT)
    return set_error(GBN_ERR_INVALID, "direction must be FORWARD or ADJOINT");
  const int rc = check_dims(W, H, F, 1);
  if (rc) return rc;
  return motion_op(ctx, direction, CF2(d_in), F2(d_out), d_xn, d_xmesh, bound_box, W, H, F);
}

int gbn_registration_info_get(int N, int F, const gbn_registration_params* params, gbn_registration_info* info) {
  return registration_info(N, F, params, info);
}

int gbn_registration_run(gbn_ctx* ctx, const float* d_images, int N, int F, const gbn_registration_params* params,
                         const float* d_T_init, float* d_T, float* d_xn, int* d_xmesh, float* h_H,
                         gbn_registration_stats* stats) {
  CHECK_CTX(ctx);
  NONNULL2(d_images, d_T);
  if (!d_xn) return set_error(GBN_ERR_INVALID, "null deformed-mesh output");
  return registration_run(ctx, CF2(d_images), N, F, params, d_T_init, d_T, d_xn, d_xmesh, h_H, stats);
}

int gbn_problem_set_motion(gbn_problem* p, const float* d_xn, const int* d_xmesh, const int bound_box[4]) {
  if (!p) return set_error(GBN_ERR_INVALID, "null problem");
  DeviceGuard guard(p->ctx->device);
  return motion_set(p, d_xn, d_xmesh, bound_box);
}

int gbn_problem_fit_rows(gbn_problem* p, int headroom_rows, int* kept_rows) {
  if (!p) return set_error(GBN_ERR_INVALID, "null problem");
  DeviceGuard guard(p->ctx->device);
  return problem_fit_rows(p, headroom_rows, kept_rows);
}

int gbn_problem_destroy(gbn_problem* p) {
  if (!p) return GBN_OK;
  if (p->in_batches > 0)
    return set_error(GBN_ERR_INVALID, "the problem belongs to a live batch: destroy the batch first");
  DeviceGuard guard(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  problem_free(p);
  delete p;
  return GBN_OK;
}

int gbn_nesta_run(gbn_ctx* ctx, gbn_problem* p, const gbn_nesta_params* params, float* d_x, gbn_nesta_stats* stats) {
  CHECK_CTX(ctx);
  if (!p || !params || !d_x) return set_error(GBN_ERR_INVALID, "null argument");
  if (p->ctx != ctx) return set_error(GBN_ERR_INVALID, "problem belongs to another context");
  return nesta_run(ctx, p, params, F2(d_x), stats);
}

int gbn_nesta_run_host(gbn_ctx* ctx, int W, int H, int F, int C, const float* h_y, const float* h_S,
                       const uint8_t* h_mask, const gbn_nesta_params* params, float* h_x, gbn_nesta_stats* stats) {
  CHECK_CTX(ctx);
  if (!h_y || !h_S || !h_mask || !params || !h_x) return set_error(GBN_ERR_INVALID, "null argument");
  int rc = validate_problem_dims(W, H, F, C);
  if (rc) return rc;
  HostRunCache* c = nullptr;
  for (auto& e : g_host_cache)
    if (e.first == ctx) c = e.second;
  if (c && (c->W != W || c->H != H || c->F != F || c->C != C)) {
    free_host_cache(ctx);
    c = nullptr;
  }
  const size_t X = size_t(W) * H * F, K = X * C, S = size_t(W) * H * C;
  if (!c) {
    c = new HostRunCache();
    c->W = W;
    c->H = H;
    c->F = F;
    c->C = C;
    g_host_cache.emplace_back(ctx, c);
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc(&c->y, K * sizeof(float2))) != cudaSuccess ||
        (e = cudaMalloc(&c->S, S * sizeof(float2))) != cudaSuccess ||
        (e = cudaMalloc(&c->x, X * sizeof(float2))) != cudaSuccess || (e = cudaMalloc(&c->mask, X)) != cudaSuccess) {
      free_host_cache(ctx);
      return cuda_status(e, "host-run buffers");
    }
    if ((rc = gbn_problem_create(ctx, W, H, F, C, reinterpret_cast<const float*>(c->y),
                                 reinterpret_cast<const float*>(c->S), c->mask, &c->prob)) != GBN_OK) {
      free_host_cache(ctx);
      return rc;
    }
  }
  cudaStream_t s = ctx->stream;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(c->y, h_y, K * sizeof(float2), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(c->S, h_S, S * sizeof(float2), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(c->mask, h_mask, X, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_status(e, "upload");
  if ((rc = nesta_run(ctx, c->prob, params, c->x, nullptr)) != GBN_OK) return rc;
  if ((e = cudaMemcpyAsync(h_x, c->x, X * sizeof(float2), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_status(e, "download");
  if (stats) return read_stats(c->prob, s, stats);  // waits for the download too
  return cuda_status(cudaStreamSynchronize(s), "nesta run");
}

#define CHECK_BATCH(b) \
  if (!(b)) return set_error(GBN_ERR_INVALID, "null batch"); \
  DeviceGuard guard_(batch_ctx(b)->device)

int gbn_batch_create(gbn_ctx* ctx, int n, gbn_problem* const* problems, const gbn_nesta_params* params,
                     float* const* d_outputs, int precision_mode, gbn_batch** out) {
  CHECK_CTX(ctx);
  return batch_create(ctx, n, problems, params, d_outputs, precision_mode, out);
}

int gbn_batch_launch(gbn_batch* b) {
  CHECK_BATCH(b);
  return batch_launch(b);
}

int gbn_batch_capture(gbn_batch* b) {
  CHECK_BATCH(b);
  return batch_capture(b);
}

int gbn_batch_groups(gbn_batch* b, int* groups, int* tensor_core_groups) {
  CHECK_BATCH(b);
  return batch_groups(b, groups, tensor_core_groups);
}

int gbn_batch_group_info(gbn_batch* b, int g, int* W, int* H, int* members, int* member_idx, int* path) {
  CHECK_BATCH(b);
  return batch_group_info(b, g, W, H, members, member_idx, path);
}

int gbn_batch_stats(gbn_batch* b, int i, gbn_nesta_stats* stats) {
  CHECK_BATCH(b);
  return batch_stats(b, i, stats);
}

int gbn_batch_destroy(gbn_batch* b) {
  if (!b) return GBN_OK;
  DeviceGuard guard_(batch_ctx(b)->device);
  return batch_destroy(b);
}

int gbn_batch_run(gbn_ctx* ctx, int n, gbn_problem* const* problems, const gbn_nesta_params* params,
                  float* const* d_outputs, int precision_mode, gbn_nesta_stats* stats) {
  CHECK_CTX(ctx);
  gbn_batch* b = nullptr;
  int rc = batch_create(ctx, n, problems, params, d_outputs, precision_mode, &b);
  if (rc != GBN_OK) return rc;
  rc = batch_launch(b);
  for (int i = 0; rc == GBN_OK && stats && i < n; ++i) rc = batch_stats(b, i, &stats[i]);
  const int rd = batch_destroy(b);
  return rc != GBN_OK ? rc : rd;
}

int gbn_graph_capture(gbn_batch* b) { return gbn_batch_capture(b); }
int gbn_graph_replay(gbn_batch* b) { return gbn_batch_launch(b); }

int gbn_autotune(gbn_ctx* ctx, int n, const int* shapes, const char* cache_path) {
  CHECK_CTX(ctx);
  return autotune(ctx, n, shapes, cache_path);
}

int gbn_autotune_load(gbn_ctx* ctx, const char* cache_path) {
  CHECK_CTX(ctx);
  return autotune_load(ctx, cache_path);
}

int gbn_autotune_lookup(gbn_ctx* ctx, int W, int H, int F, int C, int* k1_coils_per_block, int* k2_ctas_per_sm) {
  CHECK_CTX(ctx);
  if (!k1_coils_per_block || !k2_ctas_per_sm) return set_error(GBN_ERR_INVALID, "null output pointer");
  tuning_for(ctx, W, H, F, C, k1_coils_per_block, k2_ctas_per_sm);
  return GBN_OK;
}

}  // extern "C"
