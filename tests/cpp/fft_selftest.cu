// Host-side check of the register DFTs and of the two-pass split used by the
// column and row kernels: every supported length is transformed with the same
// index arithmetic as the kernels (forward dit2<A,B>, backward dit2<B,A> on the
// forward output distribution) and compared with a direct double-precision DFT.
// Build: nvcc -std=c++17 --expt-relaxed-constexpr -x cu fft_selftest.cu
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "../../opencliper_gb300/csrc/fft.cuh"

using namespace gbn;

static std::vector<double> naive(const std::vector<float2>& x, bool inv) {
  const int L = int(x.size());
  std::vector<double> out(2 * L);
  for (int k = 0; k < L; ++k) {
    long double re = 0, im = 0;
    for (int n = 0; n < L; ++n) {
      const long double ang = (inv ? 2.0L : -2.0L) * 3.14159265358979323846264338327950288L * ((long long)n * k % L) / L;
      re += x[n].x * cosl(ang) - x[n].y * sinl(ang);
      im += x[n].x * sinl(ang) + x[n].y * cosl(ang);
    }
    out[2 * k] = double(re);
    out[2 * k + 1] = double(im);
  }
  return out;
}

static double relerr(const std::vector<float2>& got, const std::vector<double>& ref) {
  double num = 0, den = 0;
  for (size_t i = 0; i < got.size(); ++i) {
    const double dx = got[i].x - ref[2 * i], dy = got[i].y - ref[2 * i + 1];
    num += dx * dx + dy * dy;
    den += ref[2 * i] * ref[2 * i] + ref[2 * i + 1] * ref[2 * i + 1];
  }
  return std::sqrt(num / den);
}

template <int N>
static double check_dft() {
  std::vector<float2> x(N);
  for (int i = 0; i < N; ++i) x[i] = make_float2(float(std::rand()) / RAND_MAX - 0.5f, float(std::rand()) / RAND_MAX - 0.5f);
  const std::vector<double> ref = naive(x, false);
  float2 a[N];
  for (int i = 0; i < N; ++i) a[i] = x[i];
  dft<N>(a);
  std::vector<float2> got(a, a + N);
  return relerr(got, ref);
}

// same arithmetic as k_fft_*_dense / k_fwd_cols pass 1+2 and k_rows' inverse
template <int L>
static bool check_len() {
  constexpr int A = split_a(L), B = split_b(L);
  std::vector<float2> tw(L);
  for (int j = 0; j < L; ++j) tw[j] = make_float2(float(cx_cos2pi(j, L)), -float(cx_sin2pi(j, L)));
  std::vector<float2> x(L);
  for (int i = 0; i < L; ++i) x[i] = make_float2(float(std::rand()) / RAND_MAX - 0.5f, float(std::rand()) / RAND_MAX - 0.5f);
  // forward dit2<A,B>
  std::vector<float2> ex(L), X(L);
  for (int s = 0; s < B; ++s) {
    float2 v[A];
    for (int n1 = 0; n1 < A; ++n1) v[n1] = x[B * n1 + s];
    dft<A>(v);
    for (int k1 = 0; k1 < A; ++k1) ex[k1 * B + s] = (k1 == 0) ? v[k1] : cmul(v[k1], tw[s * k1]);
  }
  for (int k1 = 0; k1 < A; ++k1) {
    float2 v[B];
    for (int s = 0; s < B; ++s) v[s] = ex[k1 * B + s];
    dft<B>(v);
    for (int k2 = 0; k2 < B; ++k2) X[k1 + A * k2] = v[k2];
  }
  const double ef = relerr(X, naive(x, false));
  // backward on X: conj, forward dit2<B,A> (pass-1 item s' = k1 holds X[A*n1 + k1]), conj
  std::vector<float2> ex2(L), y(L);
  for (int k1 = 0; k1 < A; ++k1) {
    float2 v[B];
    for (int k2 = 0; k2 < B; ++k2) v[k2] = make_float2(X[k1 + A * k2].x, -X[k1 + A * k2].y);
    dft<B>(v);
    for (int k1p = 0; k1p < B; ++k1p) ex2[k1p * A + k1] = (k1p == 0) ? v[k1p] : cmul(v[k1p], tw[k1 * k1p]);
  }
  for (int k1p = 0; k1p < B; ++k1p) {
    float2 v[A];
    for (int sp = 0; sp < A; ++sp) v[sp] = ex2[k1p * A + sp];
    dft<A>(v);
    for (int k2p = 0; k2p < A; ++k2p) y[k1p + B * k2p] = make_float2(v[k2p].x, -v[k2p].y);
  }
  const double eb = relerr(y, naive(X, true));
  const bool ok = ef < 2e-6 && eb < 2e-6;
  std::printf("L=%3d A=%2d B=%2d fwd=%.2e bwd=%.2e %s\n", L, A, B, ef, eb, ok ? "ok" : "FAIL");
  return ok;
}

template <int... Ls>
static bool check_all(std::integer_sequence<int, Ls...>) {
  bool ok = true;
  ((ok = check_len<Ls>() && ok), ...);
  return ok;
}

int main() {
  std::srand(1234);
  bool ok = true;
  double e;
#define D(N) e = check_dft<N>(); std::printf("dft<%d> err=%.2e\n", N, e); ok = ok && e < 2e-6;
  D(2) D(3) D(4) D(5) D(6) D(7) D(8) D(9) D(10) D(12) D(14) D(15) D(16) D(18) D(20) D(21) D(24) D(25) D(27) D(28) D(30) D(32)
#undef D
  ok = check_all(std::integer_sequence<int, 8, 16, 24, 32, 40, 48, 56, 64, 72, 80, 96, 112, 120, 128, 144, 160, 168, 192, 200,
                                       216, 224, 240, 256, 280, 288, 320, 336, 360, 384, 392, 400, 432, 448, 480, 504, 512>{}) && ok;
  std::printf(ok ? "ALL OK\n" : "FAILURES\n");
  return ok ? 0 : 1;
}
