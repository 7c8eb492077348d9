// Host launchers for the templated kernels of one transform length.
#pragma once

#include "nesta_kernels.cuh"
#include "registry.h"
#include "rowlocal.cuh"

namespace gbn {

// opt a kernel into more than 48 KB of dynamic shared memory (once)
template <typename K>
inline void allow_smem(K kernel, int bytes, bool& done) {
  if (!done) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done = true;
  }
}


template <int L>
struct Launchers {
  static void fwd_cols(const FusedArgs* tab, const BatchMap& bm, int it, int cpb, dim3 grid, cudaStream_t s) {
    static bool ok = false;
    allow_smem(k_fwd_cols<L>, FwdColsSmem<L>::BYTES, ok);
    launch_pdl(k_fwd_cols<L>, grid, kColNT, FwdColsSmem<L>::BYTES, s, tab, bm, it, cpb);
  }
  // resident CTAs per SM of the row kernel (queried once)
  static int rows_occupancy(bool resid) {
    static int occ1 = 0, occ0 = 0;
    int& o = resid ? occ1 : occ0;
    if (o == 0) {
      static bool ok1 = false, ok0 = false;
      int nb = 0;
      if (resid) {
        allow_smem(k_rows<L, true>, RowsSmem<L, true>::BYTES, ok1);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_rows<L, true>, kRowNT, RowsSmem<L, true>::BYTES);
      } else {
        allow_smem(k_rows<L, false>, RowsSmem<L, false>::BYTES, ok0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_rows<L, false>, kRowNT, RowsSmem<L, false>::BYTES);
      }
      o = nb > 0 ? nb : 1;
    }
    return o;
  }
  static void rows(const FusedArgs* tab, const BatchMap& bm, int it, bool resid, int grid, cudaStream_t s) {
    static bool ok1 = false, ok0 = false;
    if (resid) {
      allow_smem(k_rows<L, true>, RowsSmem<L, true>::BYTES, ok1);
      launch_pdl(k_rows<L, true>, dim3(grid), kRowNT, RowsSmem<L, true>::BYTES, s, tab, bm, it);
    } else {
      allow_smem(k_rows<L, false>, RowsSmem<L, false>::BYTES, ok0);
      launch_pdl(k_rows<L, false>, dim3(grid), kRowNT, RowsSmem<L, false>::BYTES, s, tab, bm, it);
    }
  }
  static void inv_cols(const FusedArgs* tab, const BatchMap& bm, int it, bool update, dim3 grid, cudaStream_t s) {
    static bool ok1 = false, ok0 = false;
    if (update) {
      allow_smem(k_inv_cols<L, true>, InvColsSmem<L>::BYTES, ok1);
      launch_pdl(k_inv_cols<L, true>, grid, kColNT, InvColsSmem<L>::BYTES, s, tab, bm, it);
    } else {
      allow_smem(k_inv_cols<L, false>, InvColsSmem<L>::BYTES, ok0);
      launch_pdl(k_inv_cols<L, false>, grid, kColNT, InvColsSmem<L>::BYTES, s, tab, bm, it);
    }
  }
  static void iter_cols(const FusedArgs* tab, const BatchMap& bm, int it, bool motion, dim3 grid, cudaStream_t s) {
    if constexpr (iter_cols_ok(L)) {
      static bool ok0 = false, ok1 = false;
      if (motion) {
        allow_smem(k_iter_cols<L, true>, IterColsSmem<L>::BYTES, ok1);
        launch_pdl(k_iter_cols<L, true>, grid, IterColsSmem<L>::NT, IterColsSmem<L>::BYTES, s, tab, bm, it);
      } else {
        allow_smem(k_iter_cols<L, false>, IterColsSmem<L>::BYTES, ok0);
        launch_pdl(k_iter_cols<L, false>, grid, IterColsSmem<L>::NT, IterColsSmem<L>::BYTES, s, tab, bm, it);
      }
    }
  }
  static void fft_rows(const float2* in, float2* out, int nrows, int inv, float scale, const float2* tw, int grid,
                       cudaStream_t s) {
    k_fft_rows_dense<L><<<grid, kRowNT, 0, s>>>(in, out, nrows, inv, scale, tw);
  }
  static void fft_cols(const float2* in, float2* out, int W, int nimg, int inv, float scale, const float2* tw,
                       cudaStream_t s) {
    k_fft_cols_dense<L><<<dim3(W / kWB, nimg), kColNT, 0, s>>>(in, out, W, inv, scale, tw);
  }
  static SizeKernels entry() {
    static_assert(fft_size_ok(L), "unsupported transform length");
    return SizeKernels{L, &fwd_cols, &rows, &inv_cols, &fft_rows, &fft_cols,
                       iter_cols_ok(L) ? &iter_cols : nullptr, RowCfg<L>::RPC, &rows_occupancy};
  }
};

}  // namespace gbn

// Defines gbn::register_sizes_<TAG>(SizeKernels* out) returning the count.
#define GBN_SIZE_TU(TAG, ...)                                              \
  namespace gbn {                                                          \
  int register_sizes_##TAG(SizeKernels* out) {                             \
    const SizeKernels e[] = {__VA_ARGS__};                                 \
    const int n = int(sizeof(e) / sizeof(e[0]));                           \
    for (int i = 0; i < n; ++i) out[i] = e[i];                             \
    return n;                                                              \
  }                                                                        \
  }
#define GBN_L(L) gbn::Launchers<L>::entry()
