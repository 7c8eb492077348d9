// Host-side check of the row-local kernel's per-length shape rules
// (rowlocal.cuh): for every length that runs the row-local iteration, one
// line "L A B threads bytes smem_ctas tmem_cols rcap" on stdout.  Built with
// nvcc and run on the host only (no kernel is launched).
#include <cstdio>

#include "rowlocal.cuh"

using namespace gbn;

int main() {
  for (int L = 8; L <= 512; L += 8) {
    if (!fft_size_ok(L) || !iter_cols_ok(L)) continue;
    const int a = split_a(L), b = split_b(L);
    const int bytes = iter_cols_bytes(L);
    const int ctas = (228 * 1024) / (bytes + 1024);
    int tcols = 0;
    if (iter_cols_tmem(L)) {
      const int acc0 = (2 * a + 15) / 16 * 16;
      tcols = (acc0 + 2 * a <= 32) ? 32 : (acc0 + 2 * a <= 64) ? 64 : 128;
    }
    std::printf("%d %d %d %d %d %d %d %d\n", L, a, b, iter_cols_threads(L), bytes, ctas, tcols, iter_cols_rcap(L));
  }
  return 0;
}
