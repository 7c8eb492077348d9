// Collects the per-length kernel tables of the instantiation units.
#include <mutex>

#include "registry.h"

namespace gbn {

int register_sizes_a(SizeKernels* out);
int register_sizes_b(SizeKernels* out);
int register_sizes_c(SizeKernels* out);
int register_sizes_d(SizeKernels* out);
int register_sizes_e(SizeKernels* out);
int register_sizes_f(SizeKernels* out);

namespace {
SizeKernels g_tab[64];
int g_n = 0;
std::once_flag g_once;

void build() {
  int n = 0;
  n += register_sizes_a(g_tab + n);
  n += register_sizes_b(g_tab + n);
  n += register_sizes_c(g_tab + n);
  n += register_sizes_d(g_tab + n);
  n += register_sizes_e(g_tab + n);
  n += register_sizes_f(g_tab + n);
  // ascending order
  for (int i = 1; i < n; ++i)
    for (int j = i; j > 0 && g_tab[j - 1].L > g_tab[j].L; --j) {
      const SizeKernels t = g_tab[j];
      g_tab[j] = g_tab[j - 1];
      g_tab[j - 1] = t;
    }
  g_n = n;
}
}  // namespace

const SizeKernels* find_size(int L) {
  std::call_once(g_once, build);
  for (int i = 0; i < g_n; ++i)
    if (g_tab[i].L == L) return &g_tab[i];
  return nullptr;
}

int supported_sizes(int* out, int cap) {
  std::call_once(g_once, build);
  for (int i = 0; i < g_n && i < cap; ++i) out[i] = g_tab[i].L;
  return g_n;
}

}  // namespace gbn
