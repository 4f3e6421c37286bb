// In-register DFT butterflies and in-place shared-memory FFT passes for the
// 3/2-padded lines (length M = 3N/2 = 2^a 3^b) of the DNS step.
//
// Layout convention (all kernels): a tile of V independent lines sits in
// shared memory as [slot][v] (v fastest), slot = k + k / RP (one pad slot per
// RP slots, RP = radix of the last DIF pass, even, so the stride-1 middle pass
// is bank-conflict free).  Consecutive lanes own the V lines of one butterfly,
// so they share one twiddle load.
//
// Transform structure (mixed radix R0..R{NP-1}, M = prod R):
//   DIF pass p : span L_p = M / (R0..R{p-1}), stride S_p = L_p / R_p;
//                y = DFT_R(x[base + j S]);  y_k *= W_L^{i k};  stored in place.
//                natural order in -> digit-reversed order out.
//   DIT pass p : the transpose: x_k *= W_L^{i k};  y = DFT_R(x);  in place.
//                digit-reversed in -> natural out (passes run NP-1 .. 0).
// The last DIF pass and the first DIT pass share their butterflies, so a
// pointwise operation between an inverse and a forward transform (the
// products, or the spectral update) is fused into a single smem round trip.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <utility>

#include "pal_consts.h"

namespace pal {

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };
template <typename T> using cplx = typename Cplx<T>::type;

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return {a.x + b.x, a.y + b.y}; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return {a.x - b.x, a.y - b.y}; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
  return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}

// Multiply by W_R^(SIGN*E) = cos(2 pi E/R) + i SIGN sin(2 pi E/R), all compile time.
template <int R, int E, int SIGN, typename C>
__device__ __forceinline__ C twc(C a) {
  using T = decltype(a.x);
  constexpr int e = ((E % R) + R) % R;
  if constexpr (e == 0) {
    return a;
  } else if constexpr ((4 * e) % R == 0) {
    constexpr int q = 4 * e / R;  // quarter turns
    if constexpr (q == 2) {
      return C{-a.x, -a.y};
    } else if constexpr ((q == 1) == (SIGN > 0)) {
      return C{-a.y, a.x};  // * (+i)
    } else {
      return C{a.y, -a.x};  // * (-i)
    }
  } else if constexpr ((8 * e) % R == 0) {
    constexpr int q = 8 * e / R;  // odd multiple of pi/4
    constexpr T h = T(0.7071067811865475244008443621);
    constexpr T c = (q == 1 || q == 7) ? h : -h;
    constexpr T s0 = (q == 1 || q == 3) ? h : -h;
    constexpr T s = SIGN > 0 ? s0 : -s0;
    return C{c * a.x - s * a.y, s * a.x + c * a.y};
  } else {
    constexpr T c = T(Trig<R>::c[e]);
    constexpr T s = SIGN > 0 ? T(Trig<R>::s[e]) : T(-Trig<R>::s[e]);
    return C{c * a.x - s * a.y, s * a.x + c * a.y};
  }
}

template <int R, int SIGN, typename C> struct Dft;

template <int SIGN, typename C> struct Dft<1, SIGN, C> {
  static __device__ __forceinline__ void run(C*) {}
};
template <int SIGN, typename C> struct Dft<2, SIGN, C> {
  static __device__ __forceinline__ void run(C* x) {
    C a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  }
};
template <int SIGN, typename C> struct Dft<3, SIGN, C> {
  static __device__ __forceinline__ void run(C* x) {
    using T = decltype(x[0].x);
    constexpr T h = T(0.8660254037844386467637232);  // sin(2 pi / 3)
    C t = cadd(x[1], x[2]);
    C d = csub(x[1], x[2]);
    C m = {x[0].x - T(0.5) * t.x, x[0].y - T(0.5) * t.y};
    C r = SIGN > 0 ? C{-h * d.y, h * d.x} : C{h * d.y, -h * d.x};
    x[0] = cadd(x[0], t);
    x[1] = cadd(m, r);
    x[2] = csub(m, r);
  }
};
template <int SIGN, typename C> struct Dft<4, SIGN, C> {
  static __device__ __forceinline__ void run(C* x) {
    C a = cadd(x[0], x[2]), b = csub(x[0], x[2]);
    C c = cadd(x[1], x[3]), d = csub(x[1], x[3]);
    C e = SIGN > 0 ? C{-d.y, d.x} : C{d.y, -d.x};
    x[0] = cadd(a, c);
    x[2] = csub(a, c);
    x[1] = cadd(b, e);
    x[3] = csub(b, e);
  }
};

template <int R, int A, int SIGN, typename C, int... I>
__device__ __forceinline__ void inner_twiddles(C* y, std::integer_sequence<int, I...>) {
  ((y[I] = twc<R, (I / A) * (I % A), SIGN>(y[I])), ...);
}

// R = A*B: n = B n1 + n2, k = k1 + A k2 (four-step inside registers).
template <int A, int B, int SIGN, typename C>
__device__ __forceinline__ void dft_ab(C* x) {
  constexpr int R = A * B;
  C y[R];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    C t[A];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) t[n1] = x[B * n1 + n2];
    Dft<A, SIGN, C>::run(t);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = t[k1];
  }
  inner_twiddles<R, A, SIGN>(y, std::make_integer_sequence<int, R>{});
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) {
    C t[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) t[n2] = y[n2 * A + k1];
    Dft<B, SIGN, C>::run(t);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) x[k1 + A * k2] = t[k2];
  }
}

// R = A*B with gcd(A, B) = 1 (Good-Thomas prime-factor mapping): input
// n = (B n1 + A n2) mod R, output k with k = k1 (mod A), k = k2 (mod B).  Then
// W_R^(n k) = W_A^(n1 k1) W_B^(n2 k2): a 2D DFT with no twiddles between the
// factors; both index maps are compile-time register renamings.
template <int A, int B>
constexpr int crt_index(int k1, int k2) {
  int k = 0;
  while (k % A != k1 || k % B != k2) ++k;
  return k;
}
// the output slot as a template constant, so no index is formed at run time
template <int A, int B, int K1, int K2>
struct Crt {
  static constexpr int value = crt_index<A, B>(K1, K2);
};
template <int A, int B, int K1, typename C, int... K2>
__device__ __forceinline__ void pfa_store(C* x, const C* t, std::integer_sequence<int, K2...>) {
  ((x[Crt<A, B, K1, K2>::value] = t[K2]), ...);
}
template <int A, int B, int SIGN, typename C, int K1>
__device__ __forceinline__ void pfa_column(C* x, const C* y) {
  C t[B];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) t[n2] = y[n2 * A + K1];
  Dft<B, SIGN, C>::run(t);
  pfa_store<A, B, K1>(x, t, std::make_integer_sequence<int, B>{});
}
template <int A, int B, int SIGN, typename C, int... K1>
__device__ __forceinline__ void pfa_columns(C* x, const C* y, std::integer_sequence<int, K1...>) {
  (pfa_column<A, B, SIGN, C, K1>(x, y), ...);
}
template <int A, int B, int SIGN, typename C>
__device__ __forceinline__ void dft_pfa(C* x) {
  constexpr int R = A * B;
  C y[R];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    C t[A];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) t[n1] = x[(B * n1 + A * n2) % R];
    Dft<A, SIGN, C>::run(t);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = t[k1];
  }
  pfa_columns<A, B, SIGN, C>(x, y, std::make_integer_sequence<int, A>{});
}

#define PAL_COMPOSITE(R_, A_, B_)                                                         \
  template <int SIGN, typename C> struct Dft<R_, SIGN, C> {                               \
    static __device__ __forceinline__ void run(C* x) { dft_ab<A_, B_, SIGN, C>(x); }      \
  };
#define PAL_PRIME_FACTOR(R_, A_, B_)                                                      \
  template <int SIGN, typename C> struct Dft<R_, SIGN, C> {                               \
    static __device__ __forceinline__ void run(C* x) { dft_pfa<A_, B_, SIGN, C>(x); }     \
  };
PAL_PRIME_FACTOR(6, 2, 3)
PAL_COMPOSITE(8, 2, 4)
PAL_PRIME_FACTOR(12, 3, 4)
PAL_COMPOSITE(16, 4, 4)
PAL_PRIME_FACTOR(24, 3, 8)
PAL_COMPOSITE(32, 4, 8)
PAL_PRIME_FACTOR(48, 3, 16)
PAL_COMPOSITE(64, 8, 8)
#undef PAL_COMPOSITE
#undef PAL_PRIME_FACTOR

// ---------------------------------------------------------------------------
// Plan: compile-time radix list for one line length.
template <int M_, int... Rs>
struct Plan {
  static constexpr int M = M_;
  static constexpr int NP = sizeof...(Rs);
  static constexpr int R[NP] = {Rs...};
  static constexpr int RP = R[NP - 1];
  static constexpr int prod() {
    int p = 1;
    for (int q = 0; q < NP; ++q) p *= R[q];
    return p;
  }
  static_assert(prod() == M_, "radices must multiply to M");
  static_assert(NP >= 2, "at least two passes");
  static_assert(RP % 2 == 0, "last radix must be even (bank-conflict-free padding)");
  // span of pass p (the sub-transform length it works on) and its stride
  static constexpr int span(int p) {
    int L = M;
    for (int q = 0; q < p; ++q) L /= R[q];
    return L;
  }
  static constexpr int stride(int p) { return span(p) / R[p]; }
  static constexpr int weight(int p) {  // frequency weight of digit p
    int w = 1;
    for (int q = 0; q < p; ++q) w *= R[q];
    return w;
  }
  static constexpr int PADM = M + M / RP;
  static __device__ __forceinline__ int phys(int k) { return k + k / RP; }
  // physical slot stride of pass p (every stride but the last is a multiple of RP)
  static constexpr int pstride(int p) { return stride(p) == 1 ? 1 : stride(p) + stride(p) / RP; }
  // twiddle tables: pass p holds W_{L_p}^(i k) as [i][k], i < S_p, k < R_p
  static constexpr int tw_off(int p) {
    int o = 0;
    for (int q = 0; q < p; ++q) o += stride(q) * R[q];
    return o;
  }
  static constexpr int TW_TOTAL = tw_off(NP);
  static constexpr int TW_MODE = 0;  // full [i][k] tables
  // frequency index of the DIF output stored at position pos (every constant
  // is a template-time value, so no radix table is touched at run time)
  template <int Q>
  static __device__ __forceinline__ void freq_digits(int& pos, int& f) {
    if constexpr (Q < NP) {
      constexpr int s = stride(Q);
      constexpr int w = weight(Q);
      const int k = pos / s;
      pos -= k * s;
      f += k * w;
      freq_digits<Q + 1>(pos, f);
    }
  }
  static __device__ __forceinline__ int freq(int pos) {
    int f = 0;
    freq_digits<0>(pos, f);
    return f;
  }
  // Butterfly-major order of the DIF output.  The butterfly b of the last DIF
  // pass holds the frequencies freq(b RP) + j FSTEP, j < RP; mid_perm(f) is the
  // index j FSTEP + b of frequency f, so that consecutive butterflies (lanes)
  // visiting the same j touch consecutive indices.
  static constexpr int FSTEP = M / RP;
  template <int Q>
  static __device__ __forceinline__ void perm_digits(int& f, int& pos) {
    if constexpr (Q >= 0) {
      constexpr int w = weight(Q);
      constexpr int s = stride(Q);
      const int k = f / w;
      f -= k * w;
      pos += k * s;
      perm_digits<Q - 1>(f, pos);
    }
  }
  static __device__ __forceinline__ int mid_perm(int f) {
    int pos = 0;
    perm_digits<NP - 1>(f, pos);
    return (pos % RP) * FSTEP + pos / RP;
  }
};

// The same plan with compact twiddle tables: per pass and butterfly only
// (W^i, W^4i); the other powers are formed in registers (at most two products
// of powers of the loaded values), trading load instructions for FMAs.
template <class PL>
struct Rec : PL {
  static constexpr int TW_MODE = 1;
  static constexpr int tw_off(int p) {
    int o = 0;
    for (int q = 0; q < p; ++q) o += 2 * PL::stride(q);
    return o;
  }
  static constexpr int TW_TOTAL = tw_off(PL::NP);
};

// Compact tables for pass 0 (large stride) and full tables for the later
// passes, stored transposed as [k/2][i] pairs (W^(2k' i), W^((2k'+1) i)) so the
// lanes of a warp, which hold consecutive butterflies i, read consecutive
// 16-byte entries.  The later passes have small strides (tables of a few KB
// that stay in L1), and each of their butterflies then spends R/2 loads
// instead of the products that form the powers.  FP32 only.
template <class PL>
struct RecT : PL {
  static constexpr int TW_MODE = 2;
  static constexpr int tw_off(int p) {
    int o = 0;
    for (int q = 0; q < p; ++q) o += q == 0 ? 2 * PL::stride(q) : PL::stride(q) * PL::R[q];
    return o;
  }
  static constexpr int TW_TOTAL = tw_off(PL::NP);
};

// x * W^(SIGN) where w = exp(-2 pi i e / L) is a forward-table entry.
template <int SIGN, typename C>
__device__ __forceinline__ C twmul(C x, C w) {
  if constexpr (SIGN > 0) {
    return cmulc(x, w);
  } else {
    return cmul(x, w);
  }
}

// The R twiddles of butterfly i of a pass, as 128-bit loads (row i of the table).
template <int R>
__device__ __forceinline__ void load_tw(const float2* __restrict__ t, float2 (&w)[R]) {
  static_assert(R % 2 == 0, "even radix");
#pragma unroll
  for (int q = 0; q < R / 2; ++q) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(t) + q);
    w[2 * q] = make_float2(v.x, v.y);
    w[2 * q + 1] = make_float2(v.z, v.w);
  }
}
template <int R>
__device__ __forceinline__ void load_tw(const double2* __restrict__ t, double2 (&w)[R]) {
#pragma unroll
  for (int q = 0; q < R; ++q) w[q] = __ldg(t + q);
}
template <int R, int SIGN, typename C>
__device__ __forceinline__ void apply_tw(C (&x)[R], const C* __restrict__ t) {
  if constexpr (R % 2 == 0 && sizeof(C) == 8) {  // FP32: pairs of twiddles per 128-bit load
    C w[R];
    load_tw<R>(t, w);
#pragma unroll
    for (int k = 1; k < R; ++k) x[k] = twmul<SIGN>(x[k], w[k]);
  } else {
#pragma unroll
    for (int k = 1; k < R; ++k) x[k] = twmul<SIGN>(x[k], __ldg(t + k));
  }
}

// Twiddles W^(k i), k = 1..R-1, from w1 = W^i and w4 = W^(4i): k = 4a + b,
// W^(ki) = (W^(4i))^a * (W^i)^b with the powers built by repeated products.
template <int R, int SIGN, typename C>
__device__ __forceinline__ void apply_tw_rec(C (&x)[R], C w1, C w4) {
  using T = decltype(w1.x);
  C pb[4];
  pb[0] = C{T(1), T(0)};
  pb[1] = w1;
  pb[2] = cmul(w1, w1);
  pb[3] = cmul(pb[2], w1);
  constexpr int NA = (R + 3) / 4;
  C pa[NA > 1 ? NA : 2];
  pa[0] = C{T(1), T(0)};
  pa[1] = w4;
#pragma unroll
  for (int a = 2; a < NA; ++a) pa[a] = (a % 2 == 0) ? cmul(pa[a / 2], pa[a / 2]) : cmul(pa[a - 1], w4);
#pragma unroll
  for (int k = 1; k < R; ++k) {
    const int a = k / 4, b = k % 4;
    const C t = (a == 0) ? pb[b] : (b == 0 ? pa[a] : cmul(pa[a], pb[b]));
    x[k] = twmul<SIGN>(x[k], t);
  }
}

// Twiddles of butterfly i of pass P, in the plan's table mode.
template <class PL, int P, int SIGN, int R, typename C>
__device__ __forceinline__ void pass_tw(C (&x)[R], const C* __restrict__ tw, int i) {
  if constexpr (PL::TW_MODE == 0) {
    apply_tw<R, SIGN>(x, tw + PL::tw_off(P) + i * R);
  } else if constexpr (PL::TW_MODE == 2 && P >= 1) {
    static_assert(sizeof(C) == 8 && R % 2 == 0, "transposed pair tables are FP32, even radix");
    constexpr int S = PL::stride(P);
    const float4* __restrict__ t = reinterpret_cast<const float4*>(tw + PL::tw_off(P)) + i;
#pragma unroll
    for (int k2 = 0; k2 < R / 2; ++k2) {
      const float4 v = __ldg(t + k2 * S);
      if (k2 > 0) x[2 * k2] = twmul<SIGN>(x[2 * k2], C{v.x, v.y});
      x[2 * k2 + 1] = twmul<SIGN>(x[2 * k2 + 1], C{v.z, v.w});
    }
  } else {
    const C* t = tw + PL::tw_off(P) + 2 * i;
    C w1, w4;
    if constexpr (sizeof(C) == 8) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(t));
      w1 = C{v.x, v.y};
      w4 = C{v.z, v.w};
    } else {
      w1 = __ldg(t);
      w4 = __ldg(t + 1);
    }
    apply_tw_rec<R, SIGN>(x, w1, w4);
  }
}

// One DIF pass p over a [slot][v] tile in shared memory.
template <typename T, class PL, int V, int NT, int P, int SIGN>
__device__ __forceinline__ void dif_pass(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  using C = cplx<T>;
  constexpr int R = PL::R[P];
  constexpr int L = PL::span(P);
  constexpr int S = L / R;
  constexpr int SP = PL::pstride(P);
  constexpr int NB = V * (PL::M / R);
  for (int w = tid; w < NB; w += NT) {
    const int v = w % V;
    const int b = w / V;
    const int blk = b / S;
    const int i = b - blk * S;
    C* p = sm + PL::phys(blk * L + i) * V + v;
    C x[R];
#pragma unroll
    for (int j = 0; j < R; ++j) x[j] = p[j * SP * V];
    Dft<R, SIGN, C>::run(x);
    if constexpr (S > 1) pass_tw<PL, P, SIGN>(x, tw, i);
#pragma unroll
    for (int k = 0; k < R; ++k) p[k * SP * V] = x[k];
  }
}

// One DIT pass p (transpose of the DIF pass).
template <typename T, class PL, int V, int NT, int P, int SIGN>
__device__ __forceinline__ void dit_pass(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  using C = cplx<T>;
  constexpr int R = PL::R[P];
  constexpr int L = PL::span(P);
  constexpr int S = L / R;
  constexpr int SP = PL::pstride(P);
  constexpr int NB = V * (PL::M / R);
  for (int w = tid; w < NB; w += NT) {
    const int v = w % V;
    const int b = w / V;
    const int blk = b / S;
    const int i = b - blk * S;
    C* p = sm + PL::phys(blk * L + i) * V + v;
    C x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = p[k * SP * V];
    if constexpr (S > 1) pass_tw<PL, P, SIGN>(x, tw, i);
    Dft<R, SIGN, C>::run(x);
#pragma unroll
    for (int j = 0; j < R; ++j) p[j * SP * V] = x[j];
  }
}

// Angle (in units of pi) of table entry e: W_{L_p}^(i k) = exp(-2 pi i (M/L_p) i k / M).
template <class PL, int Q>
__device__ __forceinline__ double tw_angle(int e) {
  if constexpr (Q < PL::NP) {
    constexpr int off = PL::tw_off(Q);
    constexpr int R = PL::R[Q];
    constexpr int S = PL::stride(Q);
    constexpr int step = PL::M / PL::span(Q);
    constexpr bool FULL_T = PL::TW_MODE == 2 && Q >= 1;      // transposed [k/2][i] pairs
    constexpr int W = (PL::TW_MODE == 0 || FULL_T) ? R : 2;  // entries per butterfly
    if (e < off + S * W) {
      int i, k;
      if constexpr (FULL_T) {
        const int r = e - off;
        const int k2 = r / (2 * S);
        i = (r - k2 * 2 * S) / 2;
        k = 2 * k2 + (r & 1);
      } else {
        i = (e - off) / W;
        const int c = (e - off) - i * W;
        k = PL::TW_MODE == 0 ? c : (c == 0 ? 1 : 4);
      }
      return 2.0 * (double)((long long)step * i * k) / (double)PL::M;
    }
    return tw_angle<PL, Q + 1>(e);
  }
  return 0.0;
}

// Fill every pass table, evaluated in double and rounded once to T.
template <typename T, class PL>
__global__ void k_twiddles(cplx<T>* tw) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= PL::TW_TOTAL) return;
  double sn, cs;
  sincospi(tw_angle<PL, 0>(e), &sn, &cs);
  tw[e] = cplx<T>{T(cs), T(-sn)};
}

// DIF passes FROM..TO-1 (each followed by a barrier).
template <typename T, class PL, int V, int NT, int SIGN, int P, int TO>
__device__ __forceinline__ void dif_range(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  if constexpr (P < TO) {
    dif_pass<T, PL, V, NT, P, SIGN>(sm, tw, tid);
    __syncthreads();
    dif_range<T, PL, V, NT, SIGN, P + 1, TO>(sm, tw, tid);
  }
}
// DIT passes P down to TO (inclusive), each followed by a barrier.
template <typename T, class PL, int V, int NT, int SIGN, int P, int TO>
__device__ __forceinline__ void dit_range(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  if constexpr (P >= TO) {
    dit_pass<T, PL, V, NT, P, SIGN>(sm, tw, tid);
    __syncthreads();
    dit_range<T, PL, V, NT, SIGN, P - 1, TO>(sm, tw, tid);
  }
}

}  // namespace pal
