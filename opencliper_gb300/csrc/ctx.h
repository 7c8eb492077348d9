// Library-private definitions of the context and problem objects behind the
// C ABI (include/gbn.h).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "gbn.h"
#include "registry.h"
#include "types.h"

struct gbn_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host->device prefetches (created on first use)
  cudaEvent_t ev_compute = nullptr, ev_copy = nullptr;  // ordering points between the two streams
  // side stream of the motion-compensated solve: M^T runs beside the forward
  // and row passes (created on first use)
  cudaStream_t mc_stream = nullptr;
  cudaEvent_t ev_mc_x = nullptr, ev_mc_tv = nullptr, ev_mc_adj = nullptr;
  // pinned stop flags read one chunk behind the queue (device-driven loops)
  int* host_flags = nullptr;
  cudaEvent_t ev_flag[2] = {nullptr, nullptr};
  bool own_stream = true;
  int nsm = 0;
  std::map<int, float2*> tw;          // device twiddle tables, one per supported length
  float2* tw_block = nullptr;         // single allocation holding all tables
  uint64_t rand48 = 0x1234ABCD330EULL;  // drand48 state (glibc default before any seeding)
  void* scratch = nullptr;            // grow-only scratch for per-operator entry points
  size_t scratch_bytes = 0;
  int scratch_user = 0;               // entry point that used the scratch last (kScratch*)
  // SimpleMRIRecon keeps its tables (identity row map, instance entry, control
  // block) in the scratch: a call with the same shape, buffers and scratch,
  // with no other user of the scratch in between, launches only the two passes
  struct SimpleKey {
    const void* y = nullptr;
    const void* S = nullptr;
    const void* x = nullptr;
    const void* ws = nullptr;
    int W = 0, H = 0, F = 0, C = 0;
  } simple_key;
  int k1_coils_per_block = 4;         // tuning: coils per CTA in the forward column pass
  int k2_ctas_per_sm = 4;             // tuning: persistent CTAs per SM in the row pass
  int mixed_adjoint_tc = 0;           // tuning: mixed form runs the adjoint column pass on the tensor cores
  int row_local = 1;                  // tuning: fused row-local iteration when every kept row is fully sampled
                                      // or unsampled (0: always the three-pass iteration)
  int* host_partial = nullptr;        // pinned: partly sampled kept rows of the current run (read per run)
  cudaEvent_t ev_partial = nullptr;
  int mixed_fwd_tc = -1;              // tuning: mixed form's forward pass on the tensor cores: 1 always, 0 never,
                                      // -1 per shape (autotuned where measured, else H >= 320)
  // autotuned launch shapes per problem shape (W, H, F, C) (autotune.cu)
  struct Tuned {
    int cpb, k2;
    float us;     // measured time per inner iteration
    int tc = -1;  // mixed form: tensor-core forward faster (1) or not (0); -1 not measured
  };
  std::map<std::tuple<int, int, int, int>, Tuned> tuned;
  bool use_tuned = true;
  unsigned long long launches = 0;    // kernels launched by this context
  // event profiling of kernel groups (reference: ProcessCore::getKernelGroupExecutionTimes)
  bool profile = false;
  struct ProfEntry {
    int kind;
    cudaEvent_t start, stop;
  };
  std::vector<ProfEntry> prof_pending;
  std::vector<cudaEvent_t> prof_pool;
  double prof_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned long long prof_count[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

namespace gbn {
struct McTables;
}

struct gbn_problem {
  gbn_ctx* ctx = nullptr;
  int W = 0, H = 0, F = 0, C = 0;
  const float2* y = nullptr;          // caller's KData, not owned
  const float2* S = nullptr;          // caller's sensitivity maps, not owned
  const uint8_t* mask = nullptr;      // caller's pixel mask, not owned
  // owned workspace
  int* flags = nullptr;               // [F*H]
  int* full_fh = nullptr;             // [F*H]
  int* rowmap = nullptr;              // [F*H]
  int* rowoff = nullptr;              // [F+1]
  int* rows_h = nullptr;              // [F*H]
  int* rows_f = nullptr;              // [F*H]
  int* row_full = nullptr;            // [F*H]
  float2* T = nullptr;                // [T_rows][C][W] kept rows of the row pass
  size_t T_rows = 0;                  // rows T holds (F*H unless fitted with gbn_problem_fit_rows)
  int in_batches = 0;                 // live batches holding this problem's buffers
  float2* xk0 = nullptr;
  float2* xk1 = nullptr;
  float2* wacc = nullptr;
  float2* wacc1 = nullptr;
  gbn::NestaDevState* st = nullptr;
  float* fmean = nullptr;
  int fmean_cap = 0;
  double* part_tv = nullptr;
  int part_tv_cap = 0;
  double* part_r = nullptr;
  int part_r_cap = 0;
  double* part_ne = nullptr;          // power-method partial sums
  int part_ne_cap = 0;
  float* ne_b = nullptr;              // power-method frame vectors between chunks [F][N]
  int ne_b_cap = 0;
  // mixed-precision form (mixed.cu)
  unsigned char* fk = nullptr;        // kept-row DFT operand
  size_t fk_bytes = 0;
  float* colmax = nullptr;            // [2][F][W]
  float* smax = nullptr;              // [C][W]
  int npad = 0, nch = 0;
  unsigned char* fa = nullptr;        // adjoint kept-row DFT operand
  size_t fa_bytes = 0;
  int ncha = 0;
  int gmax = 0;                       // most kept rows of a frame (fixed when the mixed operands are built)
  bool tmaps_ok = false;              // tensor maps of the tensor-core row-local iteration encoded
  CUtensorMap tm_x[2], tm_s, tm_se, tm_y;
  // motion-compensated form (motion.cu): caller's meshes, not owned
  bool mc_on = false;
  const float* mc_xn = nullptr;       // deformed mesh [2][F][H][W], 1-based
  const int* mc_xmesh = nullptr;      // original mesh [2][W][H], 1-based
  int mc_bb[4] = {0, 0, 0, 0};        // bounding box (1-based)
  float2* mc_xw = nullptr;            // M x_k
  float2* mc_g = nullptr;             // tTVadj(normalise(D M x_k))
  float2* mc_gm = nullptr;            // M^T of it
  double* mc_part = nullptr;          // power-method norm partials
  gbn::McTables* mc_tab = nullptr;    // gather tables of the meshes (motion.cu)
  gbn::FusedArgs* d_args = nullptr;   // one-entry instance table of the fused kernels
  gbn::ClassCtl* ctl = nullptr;       // row-pass control block
};

namespace gbn {

// error helpers (capi.cu)
int set_error(int code, const std::string& msg);
// allocates ctx->host_flags (2 pinned ints) and ctx->ev_flag on first use
int host_flags_ready(gbn_ctx* ctx);
int cuda_status(cudaError_t e, const char* what);

// Makes `dev` current for the lifetime of the guard and restores the caller's
// device on every return path.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// argument checks shared by the C ABI entry points
inline int check_dims(int W, int H, int F, int C) {
  if (W <= 0 || H <= 0 || F <= 0 || C <= 0) return set_error(GBN_ERR_INVALID, "dimensions must be positive");
  if (W % 8 != 0) return set_error(GBN_ERR_INVALID, "NDArray dimension 0 (width) is not multiple of 8");
  return GBN_OK;
}
inline int check_fft(int W, int H) {
  if (!find_size(W) || !find_size(H))
    return set_error(GBN_ERR_UNSUPPORTED, "FFT lengths must be 7-smooth multiples of 8 in [8, 512] (got W=" +
                                              std::to_string(W) + ", H=" + std::to_string(H) + ")");
  return GBN_OK;
}

// twiddle table for length L (nullptr when unsupported)
const float2* ctx_twiddles(gbn_ctx* ctx, int L);
// grow-only scratch of at least `bytes`, recorded as used by `user`
constexpr int kScratchOther = 0, kScratchSimple = 1;
int ctx_scratch(gbn_ctx* ctx, size_t bytes, void** out, int user = kScratchOther);

// event-profiling helpers: bracket one launch of kernel group `kind`
void prof_begin(gbn_ctx* ctx, int kind, cudaEvent_t* ev);
void prof_end(gbn_ctx* ctx, int kind, cudaEvent_t ev);
int prof_collect(gbn_ctx* ctx);

// drand48 arithmetic on 48-bit states (POSIX: X' = (0x5DEECE66D X + 0xB) mod 2^48)
struct Lcg48 {
  uint64_t a, c;  // X -> a*X + c (mod 2^48)
};
Lcg48 lcg48_jump(uint64_t k);
uint64_t lcg48_apply(const Lcg48& j, uint64_t x);

}  // namespace gbn
