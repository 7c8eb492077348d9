// Per-transform-length kernel table.  Each supported length L (see
// fft_size_ok) has one entry with host launchers for the templated kernels.
#pragma once

#include <cuda_runtime.h>
#include "types.h"

namespace gbn {

struct SizeKernels {
  int L;
  // The fused kernels take a device table of instances (all with H = L for the
  // column passes, W = L for the row pass) and the launch's BatchMap.
  // forward column pass (k_fwd_cols<L>), grid (W/8, coil groups, total frames)
  void (*fwd_cols)(const FusedArgs* tab, const BatchMap& bm, int it, int coils_per_block, dim3 grid, cudaStream_t s);
  // row pass (k_rows<L, resid>), 1-D persistent grid
  void (*rows)(const FusedArgs* tab, const BatchMap& bm, int it, bool resid, int grid, cudaStream_t s);
  // adjoint column pass (k_inv_cols<L, update>), grid (W/8, 2, total frames) in clusters of 2
  void (*inv_cols)(const FusedArgs* tab, const BatchMap& bm, int it, bool update, dim3 grid, cudaStream_t s);
  // dense FFT passes
  void (*fft_rows)(const float2* in, float2* out, int nrows, int inv, float scale, const float2* tw, int grid,
                   cudaStream_t s);
  void (*fft_cols)(const float2* in, float2* out, int W, int nimg, int inv, float scale, const float2* tw,
                   cudaStream_t s);
  // row-local inner iteration (k_iter_cols<L, motion>), grid (W/8, 2, total
  // frames) in clusters of 2; nullptr for lengths that run only the three-pass
  // iteration
  void (*iter_cols)(const FusedArgs* tab, const BatchMap& bm, int it, bool motion, dim3 grid, cudaStream_t s);
  int rows_per_cta;  // rows processed per CTA step by the row kernels
  int (*rows_occupancy)(bool resid);  // resident row-kernel CTAs per SM
};

// Returns the table entry for length L or nullptr when L is unsupported.
const SizeKernels* find_size(int L);

// Lengths with an entry, ascending.
int supported_sizes(int* out, int cap);

}  // namespace gbn
