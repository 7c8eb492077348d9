// Structures shared by host and device code of the tTV-NESTA solver.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace gbn {

// Scalar state of one NESTA reconstruction, kept in device memory so that the
// whole solve runs without host round trips.  Field meanings follow the local
// variables of NestaUp::launch (src/processes/nesta/NestaUp.cpp:442-910).
struct NestaDevState {
  // launch parameters (NestaUp::LaunchParameters, NestaUp.hpp:67-83)
  float lambda_i, mu_f, La, tolVar_in;
  int maxIntIter, maxIter, stoptest, miniter;

  // initial maxima (NestaUp.cpp:521-568), as float bit patterns for atomicMax
  unsigned int maxX_bits, maxUX_bits;

  // derived constants (NestaUp.cpp:572-583)
  float maxX, maxUX, lambda, muf, mu0, normU, gamma, gammat;
  int normest_iters;

  // per outer (continuation) loop (NestaUp.cpp:604-648)
  float mu, tolVar, Lmu, Lmu1, Ak;
  int nl;

  // per inner iteration (NestaUp.cpp:651-880)
  int last_iter;  // index of the last inner iteration that runs in this outer loop
  int qpDone;
  float qp, fx, apk, tauk;
  float normUk, fxdot, l2term;
  int outer_active;       // this instance runs the current outer loop

  // power-method progress across chunks
  int ne_done, ne_cnt;
  float ne_e, ne_e0;

  // row-local iteration (rowlocal.cuh): the update of iteration last_iter
  // must be recomputed with the stopping rule's weights; kept rows that are
  // partly sampled (they need the row pass)
  int fixup;
  int partial_rows;

  // statistics
  int iters_total;
  int status;
};

// Arguments of the fused per-iteration kernels (passed by value).
struct FusedArgs {
  int W, H, F, C, N;
  const float2* y;        // KData [F][C][H][W], zero-copy
  const float2* S;        // SensitivityMaps [C][H][W]
  const uint8_t* mask;    // pixel mask [F][H][W] (0 = not sampled)
  // kept k-space rows (rows with any sampled pixel or any nonzero datum)
  const int* rowmap;      // [F][H] -> index j within the frame, or -1
  const int* rowoff;      // [F+1] prefix count of kept rows; G = rowoff[F]
  const int* rows_h;      // [G] row (phase-encode line) of kept row g
  const int* rows_f;      // [G] frame of kept row g
  const int* row_full;    // [G] 1 when the pixel mask row is entirely sampled
  float2* T;              // intermediates [G][C][W]
  float2* xk0;            // x_k ping
  float2* xk1;            // x_k pong
  float2* xref;           // x_ref == output XData [F][H][W]
  float2* wacc;           // Nesterov weighted gradient sum w_k
  float2* wacc1;          // second w buffer: the row-local iteration reads w_k and writes w_{k+1}
  NestaDevState* st;
  float* fmean;           // [miniter] rolling objective buffer
  double* part_tv;        // [ntv][2] partial sums of ||u||^2 and Re<u,d>, one per (frame, column tile)
  double* part_r;         // [row steps] partial sums of ||E x - y||^2, one per row-pass step
  // Twiddle tables for the two-pass transforms, forward sign, 2L entries per
  // length: [k1*B + s] = w_L^(s*k1) (k1 < A, s < B), then [L + k1'*A + s'] =
  // w_L^(s'*k1') (k1' < B, s' < A), laid out so that the lanes of a warp read
  // consecutive words.
  const float2* twH;
  const float2* twW;
  float s_fwd;            // 1/sqrt(N) as the reference computes it (double -> float)
  float s_adj;            // sqrt(N)/N: the reference's sqrt(N) pre-scale times clFFT's 1/N
  float s_row;            // W * s_fwd: the row transforms' round trip on a fully sampled row
  int ntv;                // number of tTV partial sums (F * W/8; mixed form F * ceil(W/32))
  // mixed-precision form (nullptr / 0 otherwise)
  const unsigned char* fk;  // kept-row DFT operand, fp16 hi/lo, per frame and chunk
  float* colmax;          // [2][F][W] column maxima of |x_k| (iteration parity)
  const float* smax;      // [C][W] column maxima of |S_c|
  int npad, nch;          // forward operand rows (2G padded to 16) and K chunks
  const unsigned char* fa;  // adjoint kept-row DFT operand, fp16 hi/lo, per frame, row tile and chunk
  int ncha;               // adjoint K chunks (32 kept rows each)
  // motion-compensated form (nullptr otherwise): tv_src = M x_k, whose tTV
  // objective sums a separate kernel writes (the forward column pass skips
  // them), and grad_ext = M^T (tTVadj u), the tTV gradient the adjoint column
  // pass takes instead of forming it from x_k
  const float2* tv_src;
  const float2* grad_ext;
  // tensor-core row-local iteration (mixed_rowlocal.cu): tensor maps of x_k
  // (ping, pong), of S for the forward chunks and for the adjoint row tiles,
  // and of the kept rows' IDFT_W(y) in T; zero when unused
  CUtensorMap tm_x[2];
  CUtensorMap tm_s;
  CUtensorMap tm_se;
  CUtensorMap tm_y;
  int gmax_box;           // kept rows per box of tm_y (the most kept rows of a frame)
};

// Instances covered by one launch of the fused kernels.  All of them share the
// transform lengths (W, H); frames of instance i occupy grid z indices
// [fbase[i], fbase[i+1]).
constexpr int kMaxBatch = 64;

// Device-resident control block of one launch group (one set of instances).
struct ClassCtl {
  int row_next;                   // dynamic step counter of the row pass
  unsigned int ticket;            // CTAs of the row pass that have finished
  int step_base[kMaxBatch + 1];   // prefix sums of the instances' row-pass steps
  int nitems[kMaxBatch];          // kept rows x coils of each instance
  unsigned int done[kMaxBatch];   // finished row-pass steps of each instance in this launch
};

struct BatchMap {
  int n;                          // instances
  int fbase[kMaxBatch + 1];       // prefix sums of their frame counts
  ClassCtl* ctl;
};

}  // namespace gbn
