// Host-side building blocks of a tTV-NESTA solve, shared by the single-problem
// entry point (nesta_host.cu) and the batched / graph-captured form (batch.cu).
// Each launch_* helper enqueues kernels on stream `s` and returns how many it
// launched.
#pragma once

#include "ctx.h"

namespace gbn {

// launch `stmt` (n kernels) as part of profiled group `kind`
#define GBN_LAUNCH(ctx, kind, n, ...)                    \
  do {                                                  \
    cudaEvent_t ev_ = nullptr;                          \
    if ((ctx)->profile) prof_begin((ctx), (kind), &ev_); \
    __VA_ARGS__;                                        \
    if ((ctx)->profile) prof_end((ctx), (kind), ev_);   \
    (ctx)->launches += (n);                             \
  } while (0)

// Start state of the power method's restart draws: `x0`, or, when `p` is set,
// the state read from device memory at *p advanced by the jump (ja, jc), so a
// captured graph uses the generator state current at replay time.
struct RandStart {
  unsigned long long x0;
  const unsigned long long* p;
  unsigned long long ja, jc;
};

// Checks the parameters of a run of P and grows its workspace for them.
int run_prepare(gbn_ctx* ctx, gbn_problem* P, const gbn_nesta_params* prm);

// Instance-table entry of P writing its image (x_ref, the output XData) to xref.
FusedArgs make_args(gbn_problem* P, float2* xref);
BatchMap single_map(int F, ClassCtl* ctl);

// grid of the persistent row pass (length-W kernels `kw`) for `steps` steps:
// at most k2_per_sm CTAs per SM and no more than fit on the GPU at once
int row_grid(gbn_ctx* ctx, const SizeKernels* kw, bool resid, long long steps, int k2_per_sm);

// launch shapes for a problem shape: autotuned entry (exact, else nearest of
// the same W, H) or the context's defaults (autotune.cu)
void tuning_for(gbn_ctx* ctx, int W, int H, int F, int C, int* k1_coils_per_block, int* k2_ctas_per_sm);

int launch_store_args(FusedArgs* dst, const FusedArgs& a, cudaStream_t s);
int launch_group_init(const FusedArgs* tab, int n, int rows_per_cta, ClassCtl* ctl, cudaStream_t s);
// parameters into the state block, then the kept-row analysis of y and mask
int launch_pre(gbn_problem* P, const gbn_nesta_params& prm, cudaStream_t s);
// after x0 = E^H y is in xref: maxima, norm estimate and derived constants
int launch_constants(gbn_ctx* ctx, gbn_problem* P, const float2* xref, const RandStart& rs, cudaStream_t s);
// max|x0| and max|D xu| into the state block (xu = x0, or M x0 with motion compensation)
int launch_maxima(gbn_ctx* ctx, gbn_problem* P, const float2* x0, const float2* xu, cudaStream_t s);
// derived constants (lambda, mu0, gamma, ...) once ||U|| and the maxima are in the state
int launch_setup(gbn_problem* P, cudaStream_t s);
// start (w = 0, x_k = x_ref, mu/tolVar/Lmu) and end (x_ref = x_k) of outer loop nl
int launch_outer_begin(gbn_ctx* ctx, gbn_problem* P, int nl, const float2* xref, cudaStream_t s);
int launch_outer_end(gbn_ctx* ctx, gbn_problem* P, float2* xref, cudaStream_t s);
// pinned host slot and event for the per-run row-structure read-back (created on first use)
int partial_flag_ready(gbn_ctx* ctx);
// 1-thread kernel storing a 48-bit generator state (outside captured graphs)
int launch_set_rand(unsigned long long* dst, unsigned long long v, cudaStream_t s);

// Copies P's run statistics to the host (synchronises s).
int read_stats(gbn_problem* P, cudaStream_t s, gbn_nesta_stats* stats);

}  // namespace gbn
