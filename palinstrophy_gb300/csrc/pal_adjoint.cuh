// Discrete adjoint of one LS-IMEX-RK3 stage at fixed dt.
//
// Forward stage (see k_col): U = Inv(om_in); (u, v) = P(U) = C2R2(pad U);
// a = u^2 - v^2, b = u v; (A, B) = Q(a, b) = gather(R2C2 a, R2C2 b);
// fn = divxz (GA A + (G^2 - A^2) B) (row N/2 zero);
// om_out = D (c1 om_in + c2 fn + c3 f_in), f_out = fn, D = 1/(1 + K2 h2).
//
// With the real inner product <x, y> = Re sum conj(x) y the transposes are
//   P^T(lam) = w' R2C2(lam) at the kept modes,  Q^T(lam) = C2R2(pad(lam / w')),
// w' = 1 for kx = 0 and 2 otherwise (C2R2 counts each kx >= 1 mode twice),
// and for the complex scalings (Inv, GA, c1 D, ...) the conjugate scaling.
// One adjoint stage is three kernels with the forward step's FFT machinery:
//   k_adj_col_in  : lam_fn = c2 D lam_om + lam_f; lam_om <- c1 D lam_om,
//                   lam_f <- c3 D lam_om; (lam_A, lam_B)/w' padded, inverse z-FFT
//   k_adj_row     : inverse x of the lam planes and of the stage's velocity
//                   planes, lam_u = 2u lam_a + v lam_b, lam_v = -2v lam_a + u lam_b,
//                   forward x, unpack
//   k_adj_col_out : forward z-FFT, lam_om += conj(Inv) (w' lam_U, w' lam_V)
// (the stage's velocity planes come from k_col_inv on the stored om_in).
#pragma once
#include "pal_kernels.cuh"

namespace pal {

template <typename T>
struct StageCoef {
  T h1, h2, c2, c3, divxz;
};

template <typename T, int M>
__device__ __forceinline__ StageCoef<T> stage_coef(const StepArgs& a) {
  const double dt = a.sc->dt, visc = a.sc->visc;
  StageCoef<T> c;
  c.h1 = T((a.beta * dt) * visc);
  c.h2 = T((a.alpha * dt) * visc);
  c.c2 = T(a.alpha * dt);
  c.c3 = T(a.beta * dt);
  const T m32 = T(M);
  c.divxz = T(1) / (m32 * m32);
  return c;
}

template <typename T, class PL, int NT>
__global__ void __launch_bounds__(NT) k_adj_col_in(StepArgs a) {
  using C = cplx<T>;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int M = PL::M, V = 2, N = 2 * M / 3, Nh = M / 3;
  const int tid = threadIdx.x, kx = blockIdx.x;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  C* __restrict__ lom = static_cast<C*>(a.om) + (size_t)kx * N;
  C* __restrict__ lf = static_cast<C*>(a.fnm1) + (size_t)kx * N;
  const StageCoef<T> cf = stage_coef<T, M>(a);
  const T ax = T(kx);
  const T inv_w = kx == 0 ? T(1) : T(0.5);
  for (int pos = tid; pos < M; pos += NT) {
    const int f = PL::freq(pos);
    C la = {T(0), T(0)}, lb = {T(0), T(0)};
    if (f < Nh || f >= N) {
      const int z = f < Nh ? f : f - Nh;
      const T gz = T(z < Nh ? z : z - N);
      const T K2 = ax * ax + gz * gz;
      const T D = T(1) / (T(1) + K2 * cf.h2);
      const T c1 = T(1) - K2 * cf.h1;
      const C lw = lom[z], lff = lf[z];
      const C lfn = {cf.c2 * D * lw.x + lff.x, cf.c2 * D * lw.y + lff.y};
      lom[z] = C{c1 * D * lw.x, c1 * D * lw.y};
      lf[z] = C{cf.c3 * D * lw.x, cf.c3 * D * lw.y};
      if (z != Nh) {
        const T sa = cf.divxz * (gz * ax) * inv_w, sb = cf.divxz * (gz * gz - ax * ax) * inv_w;
        la = C{sa * lfn.x, sa * lfn.y};
        lb = C{sb * lfn.x, sb * lfn.y};
      }
    }
    sm[PL::phys(pos) * V + 0] = la;
    sm[PL::phys(pos) * V + 1] = lb;
  }
  __syncthreads();
  dit_range<T, PL, V, NT, +1, PL::NP - 1, 0>(sm, tw, tid);
  C* __restrict__ x0 = static_cast<C*>(a.w0) + (size_t)kx * M;
  C* __restrict__ x1 = static_cast<C*>(a.w1) + (size_t)kx * M;
  for (int w = tid; w < V * M; w += NT) {
    const int v = w & 1, k = w >> 1;
    (v == 0 ? x0 : x1)[k] = sm[PL::phys(k) * V + v];
  }
}

template <typename T, class PL, int V, int NT>
__global__ void __launch_bounds__(NT) k_adj_row(StepArgs a) {
  using C = cplx<T>;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* lam = reinterpret_cast<C*>(smraw);
  C* vel = lam + PL::PADM * V;
  constexpr int M = PL::M, Nh = M / 3;
  const int tid = threadIdx.x, z0 = blockIdx.x * V;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  row_first_pass<T, PL, V, NT>(a, lam, z0, tid, a.w0, a.w1);
  row_first_pass<T, PL, V, NT>(a, vel, z0, tid, a.y0, a.y1);
  dif_range<T, PL, V, NT, +1, 1, PL::NP>(lam, tw, tid);
  dif_range<T, PL, V, NT, +1, 1, PL::NP>(vel, tw, tid);
  for (int w = tid; w < V * M; w += NT) {
    const int v = w % V, pos = w / V;
    const int s = PL::phys(pos) * V + v;
    const C l = lam[s], q = vel[s];
    // l = (lam_a, lam_b), q = (u, v) at this physical point
    lam[s] = C{T(2) * q.x * l.x + q.y * l.y, -T(2) * q.y * l.x + q.x * l.y};
  }
  __syncthreads();
  dit_range<T, PL, V, NT, -1, PL::NP - 1, 0>(lam, tw, tid);
  C* __restrict__ x0 = static_cast<C*>(a.w0);
  C* __restrict__ x1 = static_cast<C*>(a.w1);
  for (int w = tid; w < V * Nh; w += NT) {
    const int v = w % V, k = w / V;
    const C p = lam[PL::phys(k) * V + v];
    const C q = lam[PL::phys(k == 0 ? 0 : M - k) * V + v];
    x0[(size_t)k * M + z0 + v] = C{T(0.5) * (p.x + q.x), T(0.5) * (p.y - q.y)};
    x1[(size_t)k * M + z0 + v] = C{T(0.5) * (p.y + q.y), T(-0.5) * (p.x - q.x)};
  }
}

template <typename T, class PL, int NT>
__global__ void __launch_bounds__(NT) k_adj_col_out(StepArgs a) {
  using C = cplx<T>;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int M = PL::M, V = 2, N = 2 * M / 3, Nh = M / 3;
  const int tid = threadIdx.x, kx = blockIdx.x;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  const C* __restrict__ x0 = static_cast<const C*>(a.w0) + (size_t)kx * M;
  const C* __restrict__ x1 = static_cast<const C*>(a.w1) + (size_t)kx * M;
  for (int w = tid; w < V * M; w += NT) {
    const int v = w & 1, k = w >> 1;
    sm[PL::phys(k) * V + v] = (v == 0 ? x0 : x1)[k];
  }
  __syncthreads();
  dif_range<T, PL, V, NT, -1, 0, PL::NP>(sm, tw, tid);
  C* __restrict__ lom = static_cast<C*>(a.om) + (size_t)kx * N;
  const T ax = T(kx);
  const T wgt = kx == 0 ? T(1) : T(2);
  for (int pos = tid; pos < M; pos += NT) {
    const int f = PL::freq(pos);
    if (!(f < Nh || f >= N)) continue;
    const int z = f < Nh ? f : f - Nh;
    const C lu = sm[PL::phys(pos) * V + 0], lv = sm[PL::phys(pos) * V + 1];
    const T gz = T(z < Nh ? z : z - N);
    C add = {T(0), T(0)};
    if (kx >= 1) {
      const T ik = T(1) / (ax * ax + gz * gz);
      // conj(-i gz/K2) w' lu + conj(i ax/K2) w' lv = i (gz w'/K2) lu - i (ax w'/K2) lv
      const T su = gz * ik * wgt, sv = ax * ik * wgt;
      add = C{-su * lu.y + sv * lv.y, su * lu.x - sv * lv.x};
    } else if (z >= 1) {
      const T ig = T(1) / gz;  // conj(-i/gz) = i/gz
      add = C{-ig * lu.y, ig * lu.x};
    }
    const C o = lom[z];
    lom[z] = C{o.x + add.x, o.y + add.y};
  }
}

// Loss gradient seed: lam_om = w' K2 om (L = 1/2 sum w' K2 |om|^2), lam_f = 0.
template <typename T>
__global__ void k_adj_seed(const cplx<T>* __restrict__ om, cplx<T>* __restrict__ lom, cplx<T>* __restrict__ lf, int N,
                           double* loss_part) {
  using C = cplx<T>;
  const int Nh = N >> 1;
  const long long total = (long long)N * Nh;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int kx = int(i / N), z = int(i - (long long)kx * N);
    const T gz = T(z < Nh ? z : z - N);
    const T K2 = T(kx) * T(kx) + gz * gz;
    const T w = kx == 0 ? T(1) : T(2);
    const C o = om[i];
    lom[i] = C{w * K2 * o.x, w * K2 * o.y};
    lf[i] = C{T(0), T(0)};
    acc += 0.5 * (double)w * (double)K2 * ((double)o.x * (double)o.x + (double)o.y * (double)o.y);
  }
  __shared__ double red[8];
  double v[1] = {acc};
  block_sum<256, 1>(v, red, threadIdx.x);
  if (threadIdx.x == 0) loss_part[blockIdx.x] = v[0];
}

}  // namespace pal
