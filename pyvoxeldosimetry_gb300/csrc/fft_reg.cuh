// Register-resident mixed-radix DFTs and the two-level ("four-step") FFT used
// by the fast convolution passes.
//
// RDft<N> computes an N-point DFT (N = 2^a 3^b 5^c 7^d, N <= 32) entirely in
// registers: composite N = A * B is split Cooley-Tukey style into A DFTs of
// length B, twiddles W_N^(a k), and B DFTs of length A.  All indices are
// compile-time constants (static_for over std::integral_constant) and the
// twiddles are constexpr values computed from a Taylor series of sin/cos with
// exact integer quadrant reduction, so they become immediate operands.
//
// four_step<A, B> does a length L = A * B FFT of TXX independent columns held by
// TXX * max(A, B) threads: thread (c, j) with j < A holds x[j + A b] (b < B),
// computes the B-point DFT in registers, multiplies by W_L^(j k), writes to a
// shared-memory exchange tile, and thread (c, j) with j < B reads back the A
// values of index j and finishes with an A-point DFT: it then holds
// X[j + B q] (q < A).  One shared-memory round trip per transform.
#pragma once

#include <type_traits>
#include <utility>

#include "pvd_common.cuh"

namespace pvd {

// ---------------------------------------------------------------------------
// compile-time loops
// ---------------------------------------------------------------------------
template <class F, int... I>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

// ---------------------------------------------------------------------------
// constexpr cos/sin of 2 pi j / n
// ---------------------------------------------------------------------------
constexpr double kPiD = 3.14159265358979323846264338327950288;

constexpr double cx_sin_poly(double x) {  // |x| <= pi/4: Taylor series to x^27
  double x2 = x * x, t = x, s = x;
  for (int k = 1; k <= 13; ++k) {
    t *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
    s += t;
  }
  return s;
}
constexpr double cx_cos_poly(double x) {  // |x| <= pi/4: Taylor series to x^26
  double x2 = x * x, t = 1.0, s = 1.0;
  for (int k = 1; k <= 13; ++k) {
    t *= -x2 / ((2.0 * k - 1.0) * (2.0 * k));
    s += t;
  }
  return s;
}
struct CS {
  double c, s;
};
// angle 2 pi j / n = (pi/2) (q + r/n) with |r/n| <= 1/2 (integer reduction)
constexpr CS cx_cossin(long long j, long long n) {
  long long jj = ((j % n) + n) % n;
  long long q = (4 * jj + n / 2) / n;
  long long r = 4 * jj - q * n;
  double y = (kPiD / 2.0) * (double)r / (double)n;
  double c = cx_cos_poly(y), s = cx_sin_poly(y);
  switch (q & 3) {
    case 0: return CS{c, s};
    case 1: return CS{-s, c};
    case 2: return CS{-c, -s};
    default: return CS{s, -c};
  }
}

// v * W_N^J, W = exp(-2 pi i / N) (conjugate for INV)
template <int N, int J, bool INV>
__device__ __forceinline__ float2 twc(float2 v) {
  constexpr int jj = J % N;
  if constexpr (jj == 0) {
    return v;
  } else if constexpr (4 * jj == N) {  // -i (fwd) / +i (inv)
    return mul_mi<INV>(v);
  } else if constexpr (2 * jj == N) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (4 * jj == 3 * N) {  // +i (fwd) / -i (inv)
    return mul_mi<!INV>(v);
  } else {
    constexpr CS cs = cx_cossin(jj, N);
    constexpr float c = (float)cs.c;
    constexpr float s = INV ? (float)cs.s : (float)(-cs.s);
    return make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
  }
}

// ---------------------------------------------------------------------------
// register DFTs
// ---------------------------------------------------------------------------
template <int N>
struct SplitOf {
  static constexpr bool base = (N == 2 || N == 3 || N == 4 || N == 5 || N == 7 || N == 8);
  static constexpr int A = base ? N : (N % 4 == 0) ? 4 : (N % 2 == 0) ? 2 : (N % 3 == 0) ? 3 : (N % 5 == 0) ? 5 : 7;
};

template <int N, bool INV, bool BASE = SplitOf<N>::base>
struct RDft;

template <bool INV>
struct RDft<1, INV, false> {
  static __device__ __forceinline__ void run(float2*) {}
};

template <int N, bool INV>
struct RDft<N, INV, true> {
  static __device__ __forceinline__ void run(float2* v) { Dft<N, INV>::run(v); }
};

template <int N, bool INV>
struct RDft<N, INV, false> {
  static __device__ __forceinline__ void run(float2* v) {
    constexpr int A = SplitOf<N>::A;
    constexpr int B = N / A;
    static_assert(A * B == N && A > 1 && B > 1, "RDft: N must factor into 2, 3, 5, 7");
    float2 t[N];
    static_for<A>([&](auto ia) {
      constexpr int a = decltype(ia)::value;
      float2 u[B];
      static_for<B>([&](auto ib) {
        constexpr int b = decltype(ib)::value;
        u[b] = v[a + A * b];
      });
      RDft<B, INV>::run(u);
      static_for<B>([&](auto ik) {
        constexpr int k = decltype(ik)::value;
        t[a * B + k] = twc<N, a * k, INV>(u[k]);
      });
    });
    static_for<B>([&](auto ik) {
      constexpr int k = decltype(ik)::value;
      float2 u[A];
      static_for<A>([&](auto ia) {
        constexpr int a = decltype(ia)::value;
        u[a] = t[a * B + k];
      });
      RDft<A, INV>::run(u);
      static_for<A>([&](auto iq) {
        constexpr int q = decltype(iq)::value;
        v[k + B * q] = u[q];
      });
    });
  }
};

// ---------------------------------------------------------------------------
// two-level FFT across threads (see file comment).  `ex` holds A*B*TXX float2;
// `tw` holds W_L^n, n < L (forward sign).  ALIAS: `ex` may alias memory the
// threads read their inputs from (an extra barrier separates the two).
// Ends with every thread past its exchange read; callers barrier before
// reusing `ex`.
// ---------------------------------------------------------------------------
template <int A, int B, bool INV, int TXX, bool ALIAS>
__device__ __forceinline__ void four_step(float2 (&v)[B], float2 (&w)[A], float2* __restrict__ ex,
                                          const float2* __restrict__ tw, int c, int j) {
  if (j < A) RDft<B, INV>::run(v);
  if constexpr (ALIAS) __syncthreads();
  if (j < A) {
    static_for<B>([&](auto ik) {
      constexpr int k = decltype(ik)::value;
      float2 t = v[k];
      if constexpr (k > 0) {
        float2 ww = tw[j * k];
        if (INV) ww.y = -ww.y;
        t = cmul(t, ww);
      }
      ex[(j * B + k) * TXX + c] = t;
    });
  }
  __syncthreads();
  if (j < B) {
    static_for<A>([&](auto ia) {
      constexpr int a = decltype(ia)::value;
      w[a] = ex[(a * B + j) * TXX + c];
    });
    RDft<A, INV>::run(w);
  }
}

}  // namespace pvd
