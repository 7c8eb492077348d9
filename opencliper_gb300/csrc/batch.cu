// Batched tTV-NESTA: many reconstructions of uneven size, frame count and coil
// count solved together, optionally captured into one CUDA graph.
//
// Problems are grouped by their transform lengths (W, H), at most kMaxBatch
// per group.  Each group has a device table of its instances (FusedArgs) and
// a control block, and every pass of an inner iteration is ONE launch over
// all of the group's frames: the column kernels map grid z to (instance,
// frame), the persistent row kernel numbers the steps of all instances in one
// sequence and runs each instance's scalar recurrence when its last step is
// done.  Instances that stop early (stoptest) or run fewer iterations skip
// their work inside the launches.  Groups run on their own streams, forked
// from and joined back to the context stream.
//
// FP32 groups whose members' kept rows are each fully sampled or unsampled
// (checked when the batch is created) run the one-kernel row-local iteration
// (rowlocal.cuh); a later replay whose data break that sets the members'
// status (7) and leaves their images unsolved.
//
// Power-method restart draws follow the reference's process-wide drand48
// sequence as if the problems were solved one after another in batch order:
// instance i starts sum_{j<i} W_j*H_j*F_j draws after the context state.  A
// captured graph reads that state from device memory, written just before
// each replay, so replays continue the sequence.
#include <algorithm>
#include <map>
#include <utility>
#include <vector>

#include "ctx.h"
#include "nesta_kernels.cuh"
#include "solver.h"

struct gbn_batch {
  gbn_ctx* ctx = nullptr;
  int precision = GBN_PRECISION_FP32;
  std::vector<gbn_problem*> probs;
  std::vector<gbn_nesta_params> prm;
  std::vector<float2*> out;
  std::vector<unsigned long long> rand_off;  // draws before instance i
  unsigned long long rand_total = 0;
  struct Group {
    int W = 0, H = 0;
    std::vector<int> idx;  // members (indices into probs)
    gbn::FusedArgs* tab = nullptr;
    gbn::ClassCtl* ctl = nullptr;
    gbn::BatchMap bm{};
    int cpb = 1, g2 = 1, g2a = 1;  // row grids with / without the residual
    int npad_max = 0;              // mixed form: widest forward DFT operand of the group
    int nmax_ac = 0;               // mixed form: widest adjoint B operand of the group
    dim3 g3tc;                     // mixed form: grid of the adjoint tensor-core kernel
    bool adjoint_tc = false;       // mixed form: adjoint column pass on the tensor cores
    bool tc = false;               // mixed form with the forward pass on the tensor cores (else plain FP32)
    bool row_local = false;        // one-kernel row-local iteration (every member's kept rows full or unsampled)
    bool row_local_tc = false;     // mixed form: the row-local iteration on the tensor cores (k_iter_tc)
    int ncha_max = 1;              // widest adjoint operand of the group
    int cnmax_tc = 1;              // widest coil group of the tensor-core row-local iteration
    dim3 g_tc;
    bool any_stoptest = false;     // some member runs the stopping test
    dim3 g1, g3;
    unsigned maxIntIter = 0, maxIter = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
  };
  std::vector<Group> groups;
  cudaEvent_t fork = nullptr;
  unsigned long long* d_rand = nullptr;  // generator state read by a captured graph
  cudaGraphExec_t graph = nullptr;
};

namespace gbn {

bool mixed_fwd_tc_for(gbn_ctx* ctx, int W, int H, int F, int C);  // autotune.cu

// mixed-precision form (mixed.cu)
int mixed_prepare(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params& prm, const float2* out);
int inv_cols_tc_rows(int C);
dim3 inv_cols_tc_grid(int W, int H, int frames);
void launch_inv_cols_tc(const FusedArgs* tab, const BatchMap& bm, int it, int nmax, dim3 grid, cudaStream_t s);
void mixed_args(gbn_problem* P, FusedArgs* a);
int launch_mixed_setup(gbn_ctx* ctx, gbn_problem* P, cudaStream_t s);
int launch_mixed_colmax(gbn_problem* P, cudaStream_t s);
dim3 fwd_cols_tc_grid(int W, int maxC, int frames);
void launch_fwd_cols_tc(const FusedArgs* tab, const BatchMap& bm, int it, int npad_max, dim3 grid, cudaStream_t s);
// tensor-core row-local iteration (mixed_rowlocal.cu)
int iter_tc_coils(int C, int ncha);
bool iter_tc_prepare(gbn_problem* P);
void iter_tc_args(gbn_problem* P, FusedArgs* a);
dim3 iter_tc_grid(int W, int frames);
void launch_iter_tc(const FusedArgs* tab, const BatchMap& bm, int it, int npad_max, int cnmax, dim3 grid,
                    cudaStream_t s);

namespace {

void batch_release(gbn_batch* b) {
  for (gbn_problem* P : b->probs) P->in_batches -= 1;
  b->probs.clear();
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (auto& g : b->groups) {
    if (g.tab) cudaFree(g.tab);
    if (g.ctl) cudaFree(g.ctl);
    if (g.stream) cudaStreamDestroy(g.stream);
    if (g.done) cudaEventDestroy(g.done);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->d_rand) cudaFree(b->d_rand);
}

// Enqueues the whole solve of every instance.  graph_mode: restart draws start
// from *d_rand (see above) instead of the host-side context state.
int batch_enqueue(gbn_batch* b, bool graph_mode) {
  gbn_ctx* ctx = b->ctx;
  cudaError_t e = cudaEventRecord(b->fork, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e, "batch fork");
  unsigned long long n_launch = 0;
  for (auto& g : b->groups) {
    if ((e = cudaStreamWaitEvent(g.stream, b->fork, 0)) != cudaSuccess) return cuda_status(e, "batch fork");
    cudaStream_t s = g.stream;
    const SizeKernels* kh = find_size(g.H);
    const SizeKernels* kw = find_size(g.W);
    const bool mixed = g.tc;
    for (int i : g.idx) {
      n_launch += launch_pre(b->probs[i], b->prm[i], s);
      if (mixed) n_launch += launch_mixed_setup(ctx, b->probs[i], s);
    }
    n_launch += launch_group_init(g.tab, int(g.idx.size()), kw->rows_per_cta, g.ctl, s);
    // x0 = E^H y of all members (NestaUp.cpp:465-486)
    kw->rows(g.tab, g.bm, 0, false, g.g2a, s);
    kh->inv_cols(g.tab, g.bm, 0, false, g.g3, s);
    n_launch += 2;
    for (int i : g.idx) {
      const Lcg48 j = lcg48_jump(b->rand_off[i]);
      const RandStart rs = graph_mode ? RandStart{0, b->d_rand, j.a, j.c}
                                      : RandStart{lcg48_apply(j, ctx->rand48), nullptr, 1, 0};
      n_launch += launch_constants(ctx, b->probs[i], b->out[i], rs, s);
    }
    for (unsigned nl = 1; nl <= g.maxIntIter; ++nl) {
      for (int i : g.idx) {
        n_launch += launch_outer_begin(ctx, b->probs[i], int(nl), b->out[i], s);
        if (mixed) n_launch += launch_mixed_colmax(b->probs[i], s);
      }
      if (g.row_local || g.row_local_tc) {
        // one launch more recomputes a member's last update when its stopping test ends the loop
        const unsigned nit = g.maxIter + (g.any_stoptest ? 1u : 0u);
        for (unsigned it = 0; it < nit; ++it) {
          if (g.row_local_tc)
            launch_iter_tc(g.tab, g.bm, int(it), g.npad_max, g.cnmax_tc, g.g_tc, s);
          else
            kh->iter_cols(g.tab, g.bm, int(it), false, g.g3, s);
        }
        n_launch += nit;
      }
      for (unsigned it = 0; it < ((g.row_local || g.row_local_tc) ? 0u : g.maxIter); ++it) {
        if (mixed)
          launch_fwd_cols_tc(g.tab, g.bm, int(it), g.npad_max, g.g1, s);
        else
          kh->fwd_cols(g.tab, g.bm, int(it), g.cpb, g.g1, s);
        kw->rows(g.tab, g.bm, int(it), true, g.g2, s);
        if (g.adjoint_tc)
          launch_inv_cols_tc(g.tab, g.bm, int(it), g.nmax_ac, g.g3tc, s);
        else
          kh->inv_cols(g.tab, g.bm, int(it), true, g.g3, s);
        n_launch += 3;
      }
      for (int i : g.idx) n_launch += launch_outer_end(ctx, b->probs[i], b->out[i], s);
    }
    if ((e = cudaEventRecord(g.done, s)) != cudaSuccess) return cuda_status(e, "batch join");
    if ((e = cudaStreamWaitEvent(ctx->stream, g.done, 0)) != cudaSuccess) return cuda_status(e, "batch join");
  }
  ctx->launches += n_launch;
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "batch launch");
  return GBN_OK;
}

}  // namespace

int batch_create(gbn_ctx* ctx, int n, gbn_problem* const* problems, const gbn_nesta_params* params,
                 float* const* outputs, int precision, gbn_batch** out) {
  if (!ctx || !problems || !params || !outputs || !out) return set_error(GBN_ERR_INVALID, "null argument");
  if (n <= 0) return set_error(GBN_ERR_INVALID, "batch needs at least one problem");
  if (precision != GBN_PRECISION_FP32 && precision != GBN_PRECISION_MIXED)
    return set_error(GBN_ERR_INVALID, "unknown precision mode");
  *out = nullptr;
  gbn_batch* b = new gbn_batch();
  b->ctx = ctx;
  b->precision = precision;
  int rc = GBN_OK;
  std::map<std::pair<int, int>, std::vector<int>> by_size;  // (W, H) -> members, in batch order
  std::vector<std::pair<int, int>> order;
  for (int i = 0; i < n && rc == GBN_OK; ++i) {
    gbn_problem* P = problems[i];
    if (!P || !outputs[i]) {
      rc = set_error(GBN_ERR_INVALID, "null problem or output in batch");
      break;
    }
    if (P->ctx != ctx) {
      rc = set_error(GBN_ERR_INVALID, "batch problems must belong to the batch's context");
      break;
    }
    for (int j = 0; j < i; ++j)
      if (problems[j] == P) rc = set_error(GBN_ERR_INVALID, "a problem appears twice in the batch");
    if (rc != GBN_OK) break;
    if (P->mc_on) {
      rc = set_error(GBN_ERR_UNSUPPORTED, "batches do not take motion-compensated problems (use gbn_nesta_run)");
      break;
    }
    if ((rc = run_prepare(ctx, P, &params[i])) != GBN_OK) break;
    b->probs.push_back(P);
    P->in_batches += 1;  // the batch's tables hold pointers into P's buffers
    b->prm.push_back(params[i]);
    b->out.push_back(reinterpret_cast<float2*>(outputs[i]));
    b->rand_off.push_back(b->rand_total);
    b->rand_total += (unsigned long long)P->W * P->H * P->F;
    const auto key = std::make_pair(P->W, P->H);
    auto& v = by_size[key];
    if (v.empty()) order.push_back(key);
    v.push_back(i);
  }
  cudaError_t e = cudaSuccess;
  if (rc == GBN_OK) {
    for (const auto& key : order) {
      const auto& members = by_size[key];
      for (size_t c0 = 0; c0 < members.size(); c0 += kMaxBatch) {
        gbn_batch::Group g;
        g.W = key.first;
        g.H = key.second;
        g.idx.assign(members.begin() + c0, members.begin() + std::min(members.size(), c0 + kMaxBatch));
        b->groups.push_back(g);
      }
    }
    if ((e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess)
      rc = cuda_status(e, "batch event");
    if (rc == GBN_OK && (e = cudaMalloc(&b->d_rand, sizeof(unsigned long long))) != cudaSuccess)
      rc = set_error(GBN_ERR_NOMEM, "batch allocation failed");
  }
  for (auto& g : b->groups) {
    if (rc != GBN_OK) break;
    const SizeKernels* kw = find_size(g.W);
    const int ng = int(g.idx.size());
    if ((e = cudaMalloc(&g.tab, sizeof(FusedArgs) * ng)) != cudaSuccess ||
        (e = cudaMalloc(&g.ctl, sizeof(ClassCtl))) != cudaSuccess) {
      cudaGetLastError();
      rc = set_error(GBN_ERR_NOMEM, "batch allocation failed");
      break;
    }
    if ((e = cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming)) != cudaSuccess) {
      rc = cuda_status(e, "batch stream");
      break;
    }
    memset(&g.bm, 0, sizeof(g.bm));
    g.bm.n = ng;
    g.bm.ctl = g.ctl;
    const SizeKernels* kh = find_size(g.H);
    // row analysis of every member (the setup's row kernels): whether all of
    // them keep only fully sampled or unsampled rows, within what the
    // row-local iteration stages
    auto rows_all_local = [&](bool* all) -> int {
      *all = true;
      for (int i : g.idx) {
        gbn_problem* P = b->probs[i];
        g.any_stoptest = g.any_stoptest || b->prm[i].stoptest == 1;
        ctx->launches += launch_pre(P, b->prm[i], ctx->stream);
        int part = 1;
        if ((e = cudaMemcpyAsync(&part, &P->st->partial_rows, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
          return cuda_status(e, "batch row analysis");
        *all = *all && part == 0;
      }
      return GBN_OK;
    };
    // FP32 groups, and mixed groups left to the automatic choice, run the FP32
    // row-local iteration where it applies: faster than every tensor-core form
    // measured (the tensor-core row-local iteration, and the three-pass
    // iteration with the tensor-core forward pass, at 256 and 384)
    bool analysed = false;
    if (kh->iter_cols && ctx->row_local && (precision == GBN_PRECISION_FP32 || ctx->mixed_fwd_tc < 0)) {
      bool all = false;
      if ((rc = rows_all_local(&all)) != GBN_OK) break;
      g.row_local = all;
      analysed = true;
    }
    if (precision == GBN_PRECISION_MIXED && !g.row_local) {
      int gF = 2, gC = 1;
      for (int i : g.idx) {
        gF = std::max(gF, b->probs[i]->F);
        gC = std::max(gC, b->probs[i]->C);
      }
      // the row-local iteration on the tensor cores when every member's kept
      // rows are fully sampled or unsampled; else the three-pass mixed form
      if (ctx->mixed_fwd_tc == 1 && ctx->row_local) {
        bool all = true;
        for (int i : g.idx) {
          gbn_problem* P = b->probs[i];
          // the operands (and the row analysis) of the tensor-core kernels; a
          // member they do not take (too many kept rows, unaligned buffers)
          // keeps the group on the three-pass form, which reports it
          const int rcp = mixed_prepare(ctx, P, b->prm[i], b->out[i]);
          if (rcp == GBN_ERR_NOMEM) {
            rc = rcp;
            break;
          }
          if (rcp != GBN_OK) {
            all = false;
            break;
          }
          int part = 1;
          if ((e = cudaMemcpy(&part, &P->st->partial_rows, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess) {
            rc = cuda_status(e, "batch row analysis");
            break;
          }
          // and the tensor maps of the tensor-core row-local iteration
          all = all && part == 0 && iter_tc_prepare(P);
          g.any_stoptest = g.any_stoptest || b->prm[i].stoptest == 1;
        }
        if (rc != GBN_OK) break;
        g.row_local_tc = all;
      }
      g.tc = g.row_local_tc || mixed_fwd_tc_for(ctx, g.W, g.H, gF, gC);
      for (int i : g.idx) {
        if (!g.tc || g.row_local_tc || rc != GBN_OK) break;
        rc = mixed_prepare(ctx, b->probs[i], b->prm[i], b->out[i]);
      }
      if (rc != GBN_OK) break;
    }
    int frames = 0, maxC = 1, maxF = 2;
    long long steps = 0;
    for (int k = 0; k < ng; ++k) {
      const int i = g.idx[k];
      gbn_problem* P = b->probs[i];
      g.bm.fbase[k] = frames;
      frames += P->F;
      maxC = std::max(maxC, P->C);
      maxF = std::max(maxF, P->F);
      steps += ((long long)P->F * P->H * P->C + kw->rows_per_cta - 1) / kw->rows_per_cta;
      g.maxIntIter = std::max(g.maxIntIter, b->prm[i].maxIntIter);
      g.maxIter = std::max(g.maxIter, b->prm[i].maxIter);
      FusedArgs fa = make_args(P, b->out[i]);
      if (g.tc) {
        mixed_args(P, &fa);
        g.npad_max = std::max(g.npad_max, P->npad);
        g.nmax_ac = std::max(g.nmax_ac, inv_cols_tc_rows(P->C));
        g.ncha_max = std::max(g.ncha_max, P->ncha);
        if (g.row_local_tc) {
          iter_tc_args(P, &fa);
          g.cnmax_tc = std::max(g.cnmax_tc, iter_tc_coils(P->C, P->ncha));
        }
      }
      ctx->launches += launch_store_args(g.tab + k, fa, ctx->stream);
    }
    g.bm.fbase[ng] = frames;
    int cpb, k2;
    tuning_for(ctx, g.W, g.H, maxF, maxC, &cpb, &k2);
    g.cpb = std::max(1, std::min(cpb, maxC));
    g.g1 = g.tc ? fwd_cols_tc_grid(g.W, maxC, frames) : dim3(g.W / kWB, (maxC + g.cpb - 1) / g.cpb, frames);
    g.g2 = row_grid(ctx, kw, true, steps, k2);
    g.g2a = row_grid(ctx, kw, false, steps, k2);
    g.g3 = dim3(g.W / kWB, 2, frames);
    g.g3tc = inv_cols_tc_grid(g.W, g.H, frames);
    g.adjoint_tc = g.tc && ctx->mixed_adjoint_tc != 0;
    if (g.row_local_tc) g.g_tc = iter_tc_grid(g.W, frames);
    // a mixed group with the FP32 kernels forced (mixed_fwd_tc = 0) runs them
    // as an FP32 group does
    if (precision == GBN_PRECISION_MIXED && !analysed && !g.tc && !g.row_local_tc && kh->iter_cols &&
        ctx->row_local) {
      bool all = false;
      if ((rc = rows_all_local(&all)) != GBN_OK) break;
      g.row_local = all;
    }
  }
  if (rc == GBN_OK && (e = cudaGetLastError()) != cudaSuccess) rc = cuda_status(e, "batch tables");
  if (rc != GBN_OK) {
    batch_release(b);
    delete b;
    return rc;
  }
  *out = b;
  return GBN_OK;
}

int batch_launch(gbn_batch* b) {
  if (!b) return set_error(GBN_ERR_INVALID, "null batch");
  gbn_ctx* ctx = b->ctx;
  int rc;
  if (b->graph) {
    ctx->launches += launch_set_rand(b->d_rand, ctx->rand48, ctx->stream);
    const cudaError_t e = cudaGraphLaunch(b->graph, ctx->stream);
    if (e != cudaSuccess) return cuda_status(e, "graph launch");
    rc = GBN_OK;
  } else {
    rc = batch_enqueue(b, false);
  }
  if (rc == GBN_OK) ctx->rand48 = lcg48_apply(lcg48_jump(b->rand_total), ctx->rand48);
  return rc;
}

int batch_capture(gbn_batch* b) {
  if (!b) return set_error(GBN_ERR_INVALID, "null batch");
  gbn_ctx* ctx = b->ctx;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  if (ctx->profile) return set_error(GBN_ERR_INVALID, "disable profiling before capturing a graph");
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return cuda_status(e, "begin capture");
  const unsigned long long launches0 = ctx->launches;
  const int rc = batch_enqueue(b, true);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &graph);
  ctx->launches = launches0;  // nothing ran yet
  if (rc != GBN_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_status(e, "end capture");
  e = cudaGraphInstantiate(&b->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->graph = nullptr;
    return cuda_status(e, "graph instantiate");
  }
  return GBN_OK;
}

int batch_stats(gbn_batch* b, int i, gbn_nesta_stats* stats) {
  if (!b || !stats) return set_error(GBN_ERR_INVALID, "null argument");
  if (i < 0 || i >= int(b->probs.size())) return set_error(GBN_ERR_INVALID, "batch index out of range");
  return read_stats(b->probs[i], b->ctx->stream, stats);
}

gbn_ctx* batch_ctx(gbn_batch* b) { return b->ctx; }

int batch_groups(gbn_batch* b, int* groups, int* tensor_core_groups) {
  if (!b) return set_error(GBN_ERR_INVALID, "null batch");
  int tc = 0;
  for (const auto& g : b->groups) tc += g.tc ? 1 : 0;  // tensor-core forward transform (three-pass or row-local)
  if (groups) *groups = int(b->groups.size());
  if (tensor_core_groups) *tensor_core_groups = tc;
  return GBN_OK;
}

int batch_group_info(gbn_batch* b, int g, int* W, int* H, int* members, int* member_idx, int* path) {
  if (!b) return set_error(GBN_ERR_INVALID, "null batch");
  if (g < 0 || g >= int(b->groups.size())) return set_error(GBN_ERR_INVALID, "group index out of range");
  const auto& G = b->groups[size_t(g)];
  if (W) *W = G.W;
  if (H) *H = G.H;
  if (members) *members = int(G.idx.size());
  if (member_idx)
    for (size_t k = 0; k < G.idx.size(); ++k) member_idx[k] = G.idx[k];
  if (path)
    *path = G.row_local_tc ? GBN_PATH_ROW_LOCAL_TC
            : G.row_local  ? GBN_PATH_ROW_LOCAL
            : G.tc         ? GBN_PATH_THREE_PASS_TC
                           : GBN_PATH_THREE_PASS;
  return GBN_OK;
}

int batch_destroy(gbn_batch* b) {
  if (!b) return GBN_OK;
  cudaStreamSynchronize(b->ctx->stream);  // work of this batch may still be queued
  batch_release(b);
  delete b;
  return GBN_OK;
}

}  // namespace gbn
