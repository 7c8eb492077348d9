// Launch-shape autotuner.
//
// The fused kernels' tile shapes are compile-time per transform length; what
// is chosen at run time is how the work of a problem is cut into CTAs: the
// number of coils each forward-column CTA transforms (k1_coils_per_block:
// fewer coils, more CTAs and more re-reads of x; more coils, fewer and longer
// CTAs) and how many persistent row-pass CTAs run per SM (k2_ctas_per_sm).
// Both shape the three-pass iteration only (the one-kernel row-local
// iteration has a fixed launch), so the tuner times that iteration:
// gbn_autotune measures every candidate pair on a synthetic problem of each
// requested shape (zero data with a 1/8 row mask: the kernels' cost does not
// depend on the values) and keeps the fastest in the context; single runs and
// batch groups look their shape up (tuning_for).  It also times the mixed
// form's three-pass iteration with the tensor-core forward pass against the
// plain FP32 kernels on the same shape (captured batches of one) and records
// which is faster (mixed_fwd_tc_for; mixed groups that the row-local
// iteration takes run it in FP32 and do not ask).  A text cache file keeps the results across processes:
//   # gbn autotune v2: W H F C k1_coils_per_block k2_ctas_per_sm us_per_iteration mixed_fwd_tc
//   256 256 20 12 4 3 121.5 0
// (v1 lines without the last column are read with mixed_fwd_tc unknown)
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "solver.h"

namespace gbn {

int problem_alloc(gbn_problem*);
void problem_free(gbn_problem*);
int validate_problem_dims(int, int, int, int);
int nesta_run(gbn_ctx*, gbn_problem*, const gbn_nesta_params*, float2*, gbn_nesta_stats*);
int batch_create(gbn_ctx*, int, gbn_problem* const*, const gbn_nesta_params*, float* const*, int, gbn_batch**);
int batch_capture(gbn_batch*);
int batch_launch(gbn_batch*);
int batch_destroy(gbn_batch*);

// nearest tuned entry with the same transform lengths (coils first, then frames)
const gbn_ctx::Tuned* nearest_tuned(gbn_ctx* ctx, int W, int H, int F, int C) {
  const auto it = ctx->tuned.find(std::make_tuple(W, H, F, C));
  if (it != ctx->tuned.end()) return &it->second;
  const gbn_ctx::Tuned* hit = nullptr;
  long best = -1;
  for (const auto& e : ctx->tuned) {
    if (std::get<0>(e.first) != W || std::get<1>(e.first) != H) continue;
    const long d = 1000L * std::abs(std::get<3>(e.first) - C) + std::abs(std::get<2>(e.first) - F);
    if (best < 0 || d < best) {
      best = d;
      hit = &e.second;
    }
  }
  return hit;
}

bool mixed_fwd_tc_for(gbn_ctx* ctx, int W, int H, int F, int C) {
  if (ctx->mixed_fwd_tc >= 0) return ctx->mixed_fwd_tc != 0;
  if (ctx->use_tuned) {
    const gbn_ctx::Tuned* t = nearest_tuned(ctx, W, H, F, C);
    if (t && t->tc >= 0) return t->tc != 0;
  }
  (void)W;
  return H >= 320;  // three-pass iteration, measured: FP32 faster at 256, tensor cores at 384
}

void tuning_for(gbn_ctx* ctx, int W, int H, int F, int C, int* cpb, int* k2) {
  *cpb = ctx->k1_coils_per_block;
  *k2 = ctx->k2_ctas_per_sm;
  if (!ctx->use_tuned) return;
  const gbn_ctx::Tuned* t = nearest_tuned(ctx, W, H, F, C);
  if (t) {
    *cpb = t->cpb;
    *k2 = t->k2;
  }
}

namespace {

// rows h < 8, h >= H-8 and h = f (mod 8) sampled
__global__ void k_tune_mask(uint8_t* __restrict__ m, int W, int H, int F) {
  const size_t n = size_t(W) * H * F;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const int h = int((i / W) % H), f = int(i / (size_t(W) * H));
    m[i] = (h < 8 || h >= H - 8 || (h % 8) == (f % 8)) ? 255 : 0;
  }
}

int load_cache(gbn_ctx* ctx, const char* path, bool must_exist) {
  FILE* fp = std::fopen(path, "r");
  if (!fp) {
    if (must_exist) return set_error(GBN_ERR_INVALID, std::string("cannot open tuning cache ") + path);
    return GBN_OK;
  }
  char line[256];
  while (std::fgets(line, sizeof(line), fp)) {
    if (line[0] == '#' || line[0] == '\n') continue;
    int W, H, F, C, cpb, k2, tc = -1;
    float us;
    const int got = std::sscanf(line, "%d %d %d %d %d %d %f %d", &W, &H, &F, &C, &cpb, &k2, &us, &tc);
    if (got >= 7 && cpb >= 1 && k2 >= 1)
      ctx->tuned[std::make_tuple(W, H, F, C)] = gbn_ctx::Tuned{cpb, k2, us, (got == 8 && tc >= -1 && tc <= 1) ? tc : -1};
  }
  std::fclose(fp);
  return GBN_OK;
}

int append_cache(const char* path, int W, int H, int F, int C, const gbn_ctx::Tuned& v) {
  FILE* probe = std::fopen(path, "r");
  const bool fresh = probe == nullptr;
  if (probe) std::fclose(probe);
  FILE* fp = std::fopen(path, "a");
  if (!fp) return set_error(GBN_ERR_INVALID, std::string("cannot write tuning cache ") + path);
  if (fresh)
    std::fprintf(fp, "# gbn autotune v2: W H F C k1_coils_per_block k2_ctas_per_sm us_per_iteration mixed_fwd_tc\n");
  std::fprintf(fp, "%d %d %d %d %d %d %.2f %d\n", W, H, F, C, v.cpb, v.k2, v.us, v.tc);
  std::fclose(fp);
  return GBN_OK;
}

// Times every candidate on a synthetic problem of the shape.
int tune_shape(gbn_ctx* ctx, int W, int H, int F, int C, gbn_ctx::Tuned* out) {
  int rc = validate_problem_dims(W, H, F, C);
  if (rc != GBN_OK) return rc;
  if (F < 2) return set_error(GBN_ERR_INVALID, "autotune: F must be >= 2");
  const SizeKernels* kw = find_size(W);
  const size_t X = size_t(W) * H * F, K = X * C;
  float2 *y = nullptr, *S = nullptr, *x = nullptr;
  uint8_t* m = nullptr;
  cudaError_t e;
  if ((e = cudaMalloc(&y, K * sizeof(float2))) != cudaSuccess || (e = cudaMalloc(&S, size_t(W) * H * C * sizeof(float2))) != cudaSuccess ||
      (e = cudaMalloc(&x, X * sizeof(float2))) != cudaSuccess || (e = cudaMalloc(&m, X)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(y);
    cudaFree(S);
    cudaFree(x);
    cudaFree(m);
    return set_error(GBN_ERR_NOMEM, "autotune allocation failed");
  }
  cudaStream_t s = ctx->stream;
  cudaMemsetAsync(y, 0, K * sizeof(float2), s);
  cudaMemsetAsync(S, 0, size_t(W) * H * C * sizeof(float2), s);
  k_tune_mask<<<int(std::min<size_t>((X + 255) / 256, size_t(ctx->nsm) * 8)), 256, 0, s>>>(m, W, H, F);
  gbn_problem* P = new gbn_problem();
  P->ctx = ctx;
  P->W = W;
  P->H = H;
  P->F = F;
  P->C = C;
  P->y = y;
  P->S = S;
  P->mask = m;
  rc = problem_alloc(P);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == GBN_OK && ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess))
    rc = cuda_status(e, "autotune events");
  // 40 inner iterations per timed run, so the per-run setup does not decide the ranking
  gbn_nesta_params prm{0.01f, 1e-3f, 1.0f, 1u, 3e-4f, 0, 40u, 0u, 7u};
  const int saved_cpb = ctx->k1_coils_per_block, saved_k2 = ctx->k2_ctas_per_sm;
  const bool saved_use = ctx->use_tuned, saved_prof = ctx->profile;
  const int saved_rl = ctx->row_local;
  const uint64_t saved_rand = ctx->rand48;
  ctx->use_tuned = false;
  ctx->profile = false;
  // the launch shapes and the tensor-core choice shape the three-pass
  // iteration (the row-local iteration has neither), so it is what is timed
  ctx->row_local = 0;
  gbn_ctx::Tuned best{saved_cpb, saved_k2, -1.f};
  std::vector<int> cpbs;
  for (int c : {1, 2, 3, 4, 6, 8})
    if (c <= C && std::find(cpbs.begin(), cpbs.end(), std::min(c, C)) == cpbs.end()) cpbs.push_back(c);
  const int occ = kw->rows_occupancy(true);
  for (int cpb : cpbs) {
    for (int k2 = 1; k2 <= std::max(1, occ) && rc == GBN_OK; ++k2) {
      ctx->k1_coils_per_block = cpb;
      ctx->k2_ctas_per_sm = k2;
      float ms_best = -1.f;
      for (int rep = 0; rep < 3 && rc == GBN_OK; ++rep) {
        cudaEventRecord(e0, s);
        rc = nesta_run(ctx, P, &prm, x, nullptr);
        cudaEventRecord(e1, s);
        if (rc != GBN_OK) break;
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
          rc = cuda_status(e, "autotune run");
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (ms_best < 0 || ms < ms_best)) ms_best = ms;  // first run warms up
      }
      const float us = ms_best * 1e3f / float(prm.maxIter);
      if (rc == GBN_OK && (best.us < 0 || us < best.us)) best = gbn_ctx::Tuned{cpb, k2, us};
    }
  }
  // the mixed form's tensor-core forward pass against the plain FP32 kernels:
  // captured batches of one with the launch shape just found, best of 3 replays
  if (rc == GBN_OK && best.us > 0.f) {
    ctx->k1_coils_per_block = best.cpb;
    ctx->k2_ctas_per_sm = best.k2;
    const int saved_tc = ctx->mixed_fwd_tc;
    float ms_mode[2] = {-1.f, -1.f};
    for (int mode = 0; mode < 2 && rc == GBN_OK; ++mode) {
      ctx->mixed_fwd_tc = mode;  // 0: FP32 kernels, 1: tensor-core forward
      gbn_batch* b = nullptr;
      float* xo = reinterpret_cast<float*>(x);
      int brc = batch_create(ctx, 1, &P, &prm, &xo, GBN_PRECISION_MIXED, &b);
      if (brc == GBN_OK) brc = batch_capture(b);
      for (int rep = 0; rep < 4 && brc == GBN_OK; ++rep) {
        cudaEventRecord(e0, s);
        brc = batch_launch(b);
        cudaEventRecord(e1, s);
        if (brc != GBN_OK) break;
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
          brc = cuda_status(e, "autotune batch");
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (ms_mode[mode] < 0 || ms < ms_mode[mode])) ms_mode[mode] = ms;
      }
      if (b) batch_destroy(b);
      // a shape the mixed form cannot take (too many kept rows per frame) stays on FP32
      if (brc != GBN_OK && mode == 1) ms_mode[1] = -1.f;
      else if (brc != GBN_OK) rc = brc;
    }
    ctx->mixed_fwd_tc = saved_tc;
    if (rc == GBN_OK && ms_mode[0] > 0.f) best.tc = (ms_mode[1] > 0.f && ms_mode[1] < ms_mode[0]) ? 1 : 0;
  }
  ctx->k1_coils_per_block = saved_cpb;
  ctx->k2_ctas_per_sm = saved_k2;
  ctx->use_tuned = saved_use;
  ctx->profile = saved_prof;
  ctx->row_local = saved_rl;
  ctx->rand48 = saved_rand;  // tuning runs do not consume the caller's drand48 sequence
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(s);
  problem_free(P);
  delete P;
  cudaFree(y);
  cudaFree(S);
  cudaFree(x);
  cudaFree(m);
  if (rc == GBN_OK) *out = best;
  return rc;
}

}  // namespace

int autotune(gbn_ctx* ctx, int n, const int* shapes, const char* cache_path) {
  if (n < 0 || (n > 0 && !shapes)) return set_error(GBN_ERR_INVALID, "autotune: bad shape list");
  int rc;
  if (cache_path && (rc = load_cache(ctx, cache_path, false)) != GBN_OK) return rc;
  for (int i = 0; i < n; ++i) {
    const int W = shapes[4 * i], H = shapes[4 * i + 1], F = shapes[4 * i + 2], C = shapes[4 * i + 3];
    const auto key = std::make_tuple(W, H, F, C);
    if (ctx->tuned.count(key)) continue;
    gbn_ctx::Tuned v;
    if ((rc = tune_shape(ctx, W, H, F, C, &v)) != GBN_OK) return rc;
    ctx->tuned[key] = v;
    if (cache_path && (rc = append_cache(cache_path, W, H, F, C, v)) != GBN_OK) return rc;
  }
  return GBN_OK;
}

int autotune_load(gbn_ctx* ctx, const char* cache_path) {
  if (!cache_path) return set_error(GBN_ERR_INVALID, "null cache path");
  return load_cache(ctx, cache_path, true);
}

}  // namespace gbn
