// Register-resident small DFTs and the two-pass split used by the column and
// row FFT stages.
//
// Conventions follow the reference FFT process (src/processes/FFT.cpp:374-525,
// clFFT C2C interleaved): FORWARD is X[k] = sum_n x[n] e^{-2*pi*i*n*k/L},
// unscaled; BACKWARD uses e^{+2*pi*i*n*k/L} and is computed here as
// conj(FORWARD(conj(x))).  Scale factors are applied by the callers (the
// reference's 1/N on BACKWARD is folded into neighbouring arithmetic).
//
// A length-L transform is split as L = P*Q.  "dit2<P,Q>" semantics:
//   pass 1, item s in [0,Q): holds v[n1] = x[Q*n1 + s], n1 in [0,P); computes a
//            P-point DFT, multiplies output k1 by w_L^{s*k1}, and writes it to
//            the exchange slot (k1, s);
//   pass 2, item k1 in [0,P): reads slots (k1, s) for s in [0,Q), computes a
//            Q-point DFT; output k2 is X[k1 + P*k2].
// The forward column/row transforms use (P,Q) = (A,B) of split_of<L>; the
// inverse transforms use (B,A), whose pass-1 input distribution is exactly the
// forward pass-2 output distribution, so no reordering is ever needed.
#pragma once

#include "common.cuh"

namespace gbn {

// ---------------------------------------------------------------------------
// Size rules
// ---------------------------------------------------------------------------
constexpr bool is_7smooth(int n) {
  if (n < 1) return false;
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

// Split L = A * B with B preferably 16 (then 8, then other divisors) and both
// factors <= 32 so that each thread's DFT stays in registers.
constexpr int split_b(int L) {
  if (L % 16 == 0 && L / 16 <= 32) return 16;
  if (L % 8 == 0 && L / 8 <= 32) return 8;
  constexpr int pref[] = {24, 12, 20, 28, 18, 14, 30, 21, 15, 10, 9, 7, 6, 5, 4, 3, 2};
  for (int d : pref)
    if (L % d == 0 && L / d <= 32) return d;
  return 0;
}
constexpr int split_a(int L) { return split_b(L) ? L / split_b(L) : 0; }

// Sizes accepted by the fused and per-operator FFT paths: multiples of 8 (the
// reference requires the first spatial dimension to be a multiple of 8,
// Data.cpp:1360-1372), 7-smooth (clFFT radices 2,3,5,7), 8..512.
constexpr bool fft_size_ok(int L) { return L >= 8 && L <= 512 && L % 8 == 0 && is_7smooth(L) && split_b(L) != 0; }

// ---------------------------------------------------------------------------
// Multiply by the compile-time forward twiddle w_N^J = e^{-2*pi*i*J/N};
// trivial angles avoid multiplications.
// ---------------------------------------------------------------------------
template <int N, int J>
GBN_HD __forceinline__ float2 twc(float2 a) {
  constexpr int j = ((J % N) + N) % N;
  if constexpr (j == 0) {
    return a;
  } else if constexpr (2 * j == N) {
    return make_float2(-a.x, -a.y);
  } else if constexpr (4 * j == N) {
    return cmul_negi(a);
  } else if constexpr (4 * j == 3 * N) {
    return cmul_posi(a);
  } else {
    constexpr float c = float(cx_cos2pi(j, N));
    constexpr float s = -float(cx_sin2pi(j, N));
    return make_float2(fmaf(a.x, c, -a.y * s), fmaf(a.x, s, a.y * c));
  }
}

template <int N>
constexpr int first_radix() {
  return (N % 4 == 0) ? 4 : (N % 2 == 0) ? 2 : (N % 3 == 0) ? 3 : (N % 5 == 0) ? 5 : (N % 7 == 0) ? 7 : N;
}

// ---------------------------------------------------------------------------
// In-register forward DFT of N points, natural order in and out.  The backward
// transform is obtained by conjugating input and output.
// ---------------------------------------------------------------------------
template <int N>
GBN_HD __forceinline__ void dft(float2* a) {
  if constexpr (N == 1) {
  } else if constexpr (N == 2) {
    const float2 t = a[1];
    a[1] = psub(a[0], t);
    a[0] = padd(a[0], t);
  } else if constexpr (N == 4) {
    // packed adds where both operands are whole complex values; the -i turn
    // swaps components, so those two outputs stay scalar
    const float2 s02 = padd(a[0], a[2]), d02 = psub(a[0], a[2]);
    const float2 s13 = padd(a[1], a[3]), d13 = psub(a[1], a[3]);
    const float2 r = cmul_negi(d13);
    a[0] = padd(s02, s13);
    a[2] = psub(s02, s13);
    a[1] = cadd(d02, r);
    a[3] = csub(d02, r);
  } else if constexpr (N == 3 || N == 5 || N == 7) {
    // Odd prime: X_k = a0 + sum_m cos(2pi m k/N)(a_m + a_{N-m}) -/+ i sin(2pi m k/N)(a_m - a_{N-m})
    constexpr int M = (N - 1) / 2;
    float2 sp[M], sm[M];
    float2 x0 = a[0];
    sfor<0, M>([&](auto mc) {
      constexpr int m = decltype(mc)::value;
      sp[m] = cadd(a[m + 1], a[N - 1 - m]);
      sm[m] = csub(a[m + 1], a[N - 1 - m]);
      x0 = cadd(x0, sp[m]);
    });
    float2 out[N];
    out[0] = x0;
    sfor<1, M + 1>([&](auto kc) {
      constexpr int k = decltype(kc)::value;
      float2 re = a[0];
      float2 im = make_float2(0.f, 0.f);
      sfor<0, M>([&](auto mc) {
        constexpr int m = decltype(mc)::value;
        constexpr float c = float(cx_cos2pi((m + 1) * k, N));
        constexpr float s = float(cx_sin2pi((m + 1) * k, N));
        re.x = fmaf(c, sp[m].x, re.x);
        re.y = fmaf(c, sp[m].y, re.y);
        im.x = fmaf(s, sm[m].x, im.x);
        im.y = fmaf(s, sm[m].y, im.y);
      });
      // X_k = re - i*im, X_{N-k} = re + i*im
      const float2 mi = cmul_negi(im);
      out[k] = cadd(re, mi);
      out[N - k] = csub(re, mi);
    });
    sfor<0, N>([&](auto ic) { a[decltype(ic)::value] = out[decltype(ic)::value]; });
  } else {
    // Cooley-Tukey N = P*Q: n = Q*n1 + n2, k = k1 + P*k2.
    constexpr int P = first_radix<N>();
    constexpr int Q = N / P;
    static_assert(P * Q == N && P > 1 && Q > 1, "unsupported DFT size");
    float2 b[N];
    sfor<0, Q>([&](auto n2c) {
      constexpr int n2 = decltype(n2c)::value;
      float2 t[P];
      sfor<0, P>([&](auto n1c) { t[decltype(n1c)::value] = a[Q * decltype(n1c)::value + n2]; });
      dft<P>(t);
      sfor<0, P>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        b[k1 * Q + n2] = twc<N, n2 * k1>(t[k1]);
      });
    });
    sfor<0, P>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      dft<Q>(&b[k1 * Q]);
      sfor<0, Q>([&](auto k2c) { a[k1 + P * decltype(k2c)::value] = b[k1 * Q + decltype(k2c)::value]; });
    });
  }
}

}  // namespace gbn
