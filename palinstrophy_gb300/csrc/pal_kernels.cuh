// Fused kernels of the GB300 DNS step.
//
// Device state of one field (element type T = float or double):
//   om, fnm1 : [kx][z]  (N/2 lines of N)      spectral vorticity / last nonlinear term
//   w0, w1   : [kx][z]  (N/2 lines of M)      the work planes, holding either
//               U-state: velocity (u^, v^) after the inverse z-transform, or
//               P-state: products after the forward x-transform,
//                        A = F_x(u^2 - v^2), B = F_x(u v).
// One stage of a step is two launches:
//   k_row : per tile of V physical rows z: Hermitian-packed inverse x-FFT
//           (u + i v), products, packed forward x-FFT, unpack A, B  (U -> P)
//   k_col : per column kx: forward z-FFT of A and B, nonlinear term, CNAB2 /
//           IMEX-RK3 update of om/fnm1, omega -> (u^, v^), de-aliasing pad,
//           inverse z-FFT (P -> U)
// The reference's STEP2B/STEP3/STEP2A split (turbo_simulator.py:1378-2100)
// maps onto this as: k_row = STEP2A row half + STEP2B products + STEP2B row
// half; k_col = STEP2B column half + STEP3 + STEP2A column half.
#pragma once
#include <cuda.h>  // CUtensorMap (types only; descriptors are encoded through the runtime's driver entry point)
#include <math.h>

#include "pal_fft.cuh"

namespace pal {

enum : int {
  F_STATS = 1,      // k_row / k_phys: CFL max and sum(u^2+v^2) reduction
  F_UPDATE_DT = 2,  // ... and the NEXTDT update of dt, cn from that CFLM
  F_ADVANCE = 4,    // k_col: t += dt, it += 1 in the epilogue
  F_CNM1 = 8,       // k_col: cnm1 = cn in the epilogue (CNAB2)
  F_PHYS = 16,      // k_phys: store the physical u, v planes
  // k_col, LS-IMEX-RK3 stages on butterfly-major om / fnm1 (om_p, fm_p):
  F_NO_FM_IN = 32,  // the update does not read fnm1 (its weight c3 is 0: first stage)
  F_Q_IN = 64,      // om holds q = (1 - K2 h1) om + c3 fnm1 of this stage; fnm1 is not read
  F_Q_OUT = 128,    // write the next stage's q (weights from beta_next) into om, not om and fn
  F_DIAG = 256,     // k_phys: the diagnostic sum of u^2+v^2, compensated FP64 (else a plain sum)
  // FP32 row pass of a batched ensemble, NEXTDT every step: instead of the
  // block reductions and the last-block epilogue of F_STATS, each warp folds
  // its max |u|+|v| into DevScalars::step_max (an atomic max on the float's
  // bits) and a non-finite sum into `nonfinite`; no barrier, fence or ticket.
  F_STATS_MAX = 512,
  // k_col: this step's dt and cn are the NEXTDT of step_max (as F_STATS |
  // F_UPDATE_DT would have set them), formed by every block from the device
  // scalars; the pass that ends the step (F_ADVANCE / F_CNM1) stores them,
  // with CFLM and max |u|+|v|, and clears step_max.
  F_DT_FROM_MAX = 1024,
};

// Device-resident scalars, FP64 in both precisions.
struct DevScalars {
  double dt, cn, cnm1, t;
  double visc, cflnum;
  double cflm, mean_speed2, maxabs;
  double E, L, Z, P, kmax2;
  long long it;
  int nonfinite;
  int wait_timeout;  // set by a kernel whose bounded wait for its own bulk copies ran out
  unsigned int row_counter, col_counter, diag_counter;
  unsigned int step_max;  // F_STATS_MAX: bits of this step's max |u|+|v| (a float, >= 0)
};

struct StepArgs {
  void* w0;
  void* w1;
  void* om;
  void* fnm1;
  const void* tw;   // M forward twiddles exp(-2 pi i m / M)
  const void* src;  // k_col_inv: velocity low band, reference layout (2, N, N/2)
  void* phys;       // k_phys: physical planes (2, M, M)
  DevScalars* sc;
  double* part;     // per-block reduction partials
  int N;
  int flags;
  double h1, h2;    // implicit factors: rhs = 1 - K2*h1, den = 1 + K2*h2 (if from_dt == 0)
  double c2, c3;    // explicit weights of fn and fnm1
  double alpha, beta;
  double beta_next;  // RK3: beta of the next stage (F_Q_OUT)
  int scheme;       // 0 = CNAB2 (coefficients from device dt/cnm1), 1 = RK3 stage
  // Batched ensembles: blockIdx.y selects the member; every per-member array
  // advances by its stride (in elements) and sc by one DevScalars per member.
  int members;      // grid.y of the launch (>= 1)
  long long ms_w, ms_om, ms_part, ms_phys, ms_src;
  const void* y0;   // adjoint: the forward velocity planes of the stage
  const void* y1;
  int ahead;        // resident blocks of one wave (L2-prefetch candidates; 0 = none)
  void* om_p;       // om / fnm1 in the column plan's butterfly-major order (N/2 x M)
  void* fm_p;
  const struct TmaMaps* tmaps;  // host: descriptors of w0 / w1 for the row pass's bulk copies
  const struct TmaMaps* cmaps;  // host: descriptors of w0 / w1 for the column pass's bulk copies
  // Test switch: 1 gives the first bounded wait for a tile's bulk copies no polls,
  // so the kernel takes its report path (wait_timeout) and then waits for the
  // copies with the normal bound before it uses the tile.
  int dbg_wait0;
};

// Groups per TMA box of the planar column tile: the largest divisor of the
// group count g that is at most 256 (a box dimension's limit).
__host__ __device__ constexpr int col_box_groups(int g) {
  int b = g < 256 ? g : 256;
  while (b > 1 && g % b != 0) --b;
  return b;
}

// Rows per TMA box of the row tiles: the largest power of two up to 256 that
// divides the N/2 stored rows (box dimensions are at most 256).
__host__ __device__ constexpr int tma_box_rows(int nh) {
  int b = 256;
  while (b > 1 && nh % b != 0) b /= 2;
  return b;
}

// TMA descriptors of the two work planes, each a 3D view (2M floats, N/2 rows,
// members) with a (2V floats, tma_box_rows(N/2) rows, 1) box: one box is that
// many rows of one row tile.  Passed to the row kernel as a __grid_constant__
// parameter.
struct TmaMaps {  // aligned as CUtensorMap
  CUtensorMap w0, w1;
};

// A block's place in its pass: x = tile or column index within the member,
// y = member, nx = blocks per member (the count the last-block reductions wait
// for).  A kernel launched for one group takes it from blockIdx / gridDim
// (hw_blk); the ensemble's one-launch passes decode it from a block table.
struct Blk {
  int x, y, nx;
};
__device__ __forceinline__ Blk hw_blk() { return Blk{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x}; }

// Member view of the arguments for member m.
__device__ __forceinline__ StepArgs member_args(const StepArgs& a, size_t esz, long long m) {
  if (m == 0) return a;
  StepArgs b = a;
  b.w0 = static_cast<char*>(a.w0) + m * a.ms_w * esz;
  b.w1 = static_cast<char*>(a.w1) + m * a.ms_w * esz;
  b.om = static_cast<char*>(a.om) + m * a.ms_om * esz;
  b.fnm1 = static_cast<char*>(a.fnm1) + m * a.ms_om * esz;
  if (a.om_p) b.om_p = static_cast<char*>(a.om_p) + m * a.ms_w * esz;  // N/2 x M per member, as w0
  if (a.fm_p) b.fm_p = static_cast<char*>(a.fm_p) + m * a.ms_w * esz;
  if (a.phys) b.phys = static_cast<char*>(a.phys) + m * a.ms_phys * (esz / 2);
  if (a.src) b.src = static_cast<const char*>(a.src) + m * a.ms_src * esz;
  b.sc = a.sc + m;
  b.part = a.part + m * a.ms_part;
  return b;
}
// ... for block row blockIdx.y.
__device__ __forceinline__ StepArgs member_args(const StepArgs& a, size_t esz) {
  return member_args(a, esz, (long long)blockIdx.y);
}

constexpr double kPi = 3.14159265358979323846;

// --------------------------------------------------------------------------
// Block reductions (deterministic: fixed tree order)
template <int NT, int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* red /* K*NT/32 */, int tid) {
#pragma unroll
  for (int q = 0; q < K; ++q) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
  }
  constexpr int NW = NT / 32;
  if ((tid & 31) == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) red[q * NW + (tid >> 5)] = v[q];
  }
  __syncthreads();
  if (tid < 32) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      double s = tid < NW ? red[q * NW + tid] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      v[q] = s;
    }
  }
  __syncthreads();
}

template <int NT>
__device__ __forceinline__ double block_max(double m, double* red, int tid) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  constexpr int NW = NT / 32;
  if ((tid & 31) == 0) red[tid >> 5] = m;
  __syncthreads();
  if (tid < 32) {
    double s = tid < NW ? red[tid] : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, off));
    m = s;
  }
  __syncthreads();
  return m;
}

// block_max and block_sum<NT, 1> of one value pair in one pass (one shared
// round trip instead of two), with the same tree order as each of them.
template <int NT>
__device__ __forceinline__ void block_maxsum(double& m, double& s, double* red /* 2*NT/32 */, int tid) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    s += __shfl_xor_sync(0xffffffffu, s, off);
  }
  constexpr int NW = NT / 32;
  if ((tid & 31) == 0) {
    red[tid >> 5] = m;
    red[NW + (tid >> 5)] = s;
  }
  __syncthreads();
  if (tid < 32) {
    double mm = tid < NW ? red[tid] : 0.0;
    double ss = tid < NW ? red[NW + tid] : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mm = fmax(mm, __shfl_xor_sync(0xffffffffu, mm, off));
      ss += __shfl_xor_sync(0xffffffffu, ss, off);
    }
    m = mm;
    s = ss;
  }
  __syncthreads();
}

// Compensated FP64 summation: s + c carries the running sum, c the exact
// rounding errors of the additions into s (TwoSum, which needs no ordering of
// the operands' magnitudes).
__device__ __forceinline__ void csum_add(double& s, double& c, double x) {
  const double t = s + x;
  const double bp = t - s;
  c += (s - (t - bp)) + (x - bp);
  s = t;
}

// Block-wide compensated sum of K pairs (s, c): every level of the tree adds
// the s parts with TwoSum and the c parts plainly.  Threads 0..31 hold s + c
// in s on return.
template <int NT, int K>
__device__ __forceinline__ void block_csum(double (&s)[K], double (&c)[K], double* red /* 2*K*NT/32 */, int tid) {
#pragma unroll
  for (int q = 0; q < K; ++q) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double so = __shfl_xor_sync(0xffffffffu, s[q], off);
      const double co = __shfl_xor_sync(0xffffffffu, c[q], off);
      csum_add(s[q], c[q], so);
      c[q] += co;
    }
  }
  constexpr int NW = NT / 32;
  if ((tid & 31) == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      red[(2 * q) * NW + (tid >> 5)] = s[q];
      red[(2 * q + 1) * NW + (tid >> 5)] = c[q];
    }
  }
  __syncthreads();
  if (tid < 32) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      double ss = tid < NW ? red[(2 * q) * NW + tid] : 0.0;
      double cc = tid < NW ? red[(2 * q + 1) * NW + tid] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const double so = __shfl_xor_sync(0xffffffffu, ss, off);
        const double co = __shfl_xor_sync(0xffffffffu, cc, off);
        csum_add(ss, cc, so);
        cc += co;
      }
      s[q] = ss + cc;
      c[q] = 0.0;
    }
  }
  __syncthreads();
}

// Returns true in every thread of the block that finished last of the nx
// blocks counting on `counter`.  Whatever the last block reads of the others
// (their partials) is written by their thread 0 before the call, so thread 0
// alone fences before it takes its ticket; the CTA barrier before it orders
// the rest of the block's work.
__device__ __forceinline__ bool last_block(unsigned int* counter, int tid, int nx) {
  __shared__ int is_last;
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned int ticket = atomicAdd(counter, 1u);
    is_last = (ticket == (unsigned)nx - 1u);
  }
  __syncthreads();
  return is_last != 0;
}
// ... of the blocks of this member (grid row).
__device__ __forceinline__ bool last_block(unsigned int* counter, int tid) {
  return last_block(counter, tid, (int)gridDim.x);
}

// Physical-space statistics of one block: (max |u|+|v|, sum u^2+v^2) -> partials;
// the last block reduces all partials in a fixed order and applies NEXTDT.  With
// COMP the sum arrives as a thread's compensated pair (sum, comp) and stays
// compensated through the block tree and the reduction of the partials (the
// diagnostic sum); without it the sum is a plain FP64 tree, enough for the
// finiteness check of the NEXTDT statistics and far cheaper in FP64 issue slots,
// which matters for small tiles that take the statistics every step.
template <int NT, bool COMP>
__device__ void finish_stats(const StepArgs& a, double mx, double sum, double comp, int M, int tid, const Blk& bk) {
  __shared__ double red[2 * (NT / 32)];
  double s1[1] = {sum}, c1[1] = {comp};
  if constexpr (COMP) {
    mx = block_max<NT>(mx, red, tid);
    block_csum<NT, 1>(s1, c1, red, tid);
  } else {
    block_maxsum<NT>(mx, s1[0], red, tid);
  }
  if (tid == 0) {
    a.part[2 * bk.x] = mx;
    a.part[2 * bk.x + 1] = s1[0];
  }
  const bool last = last_block(&a.sc->row_counter, tid, bk.nx);
  if (!last) return;
  const int nb = bk.nx;
  double m2 = 0.0, s2[1] = {0.0}, c2[1] = {0.0};
  for (int q = tid; q < nb; q += NT) {
    m2 = fmax(m2, __ldcg(a.part + 2 * q));
    if constexpr (COMP)
      csum_add(s2[0], c2[0], __ldcg(a.part + 2 * q + 1));
    else
      s2[0] += __ldcg(a.part + 2 * q + 1);
  }
  if constexpr (COMP) {
    m2 = block_max<NT>(m2, red, tid);
    block_csum<NT, 1>(s2, c2, red, tid);
  } else {
    block_maxsum<NT>(m2, s2[0], red, tid);
  }
  if (tid == 0) {
    DevScalars* sc = a.sc;
    const double cflm = m2 * (double(a.N) / (2.0 * kPi));
    sc->maxabs = m2;
    sc->cflm = cflm;
    sc->mean_speed2 = s2[0] / (double(M) * double(M));
    if (!isfinite(s2[0])) sc->nonfinite = 1;
    if ((a.flags & F_UPDATE_DT) && cflm > 0.0 && sc->dt > 0.0) {
      const double cfl = cflm * sc->dt * kPi;
      const double cn = 0.8 + 0.2 * (sc->cflnum / cfl);
      sc->cn = cn;
      sc->dt = sc->dt * cn;
    }
    sc->row_counter = 0u;
  }
}

// F_STATS_MAX epilogue of a row tile (FP32): the warp's max |u|+|v| into
// step_max, a non-finite sum into `nonfinite`.  Non-negative floats order as
// their bit patterns, so the atomic max of the bits is the max of the values,
// whatever the order the warps arrive in.
__device__ __forceinline__ void mark_step_max(const StepArgs& a, float mx, float acc, int tid) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  const bool bad = __any_sync(0xffffffffu, !isfinite(acc));
  if ((tid & 31) == 0) {
    atomicMax(&a.sc->step_max, __float_as_uint(mx));
    if (bad) atomicOr(&a.sc->nonfinite, 1);
  }
}

// NEXTDT from step_max (F_DT_FROM_MAX), the same arithmetic as finish_stats's
// last block: the step's dt and cn, CFLM and max |u|+|v|.
struct NextDt {
  double dt, cn, cflm, maxabs;
};
__device__ __forceinline__ NextDt nextdt_from_mark(const StepArgs& a) {
  const DevScalars* sc = a.sc;
  NextDt r;
  r.maxabs = double(__uint_as_float(sc->step_max));
  r.cflm = r.maxabs * (double(a.N) / (2.0 * kPi));
  r.dt = sc->dt;
  r.cn = sc->cn;
  if (r.cflm > 0.0 && sc->dt > 0.0) {
    const double cfl = r.cflm * sc->dt * kPi;
    r.cn = 0.8 + 0.2 * (sc->cflnum / cfl);
    r.dt = sc->dt * r.cn;
  }
  return r;
}

// --------------------------------------------------------------------------
// First DIF pass of the inverse x-transform, reading the U planes directly:
// Z[k] = u^[k] + i v^[k] (k < N/2; real parts only at k = 0),
// Z[M-k] = conj(u^[k]) + i conj(v^[k]), zero elsewhere (the 3/2 pad).
template <typename T, class PL, int V, int NT>
__device__ __forceinline__ void row_first_pass(const StepArgs& a, cplx<T>* sm, int z0, int tid,
                                               const void* p0 = nullptr, const void* p1 = nullptr) {
  using C = cplx<T>;
  constexpr int M = PL::M;
  constexpr int R = PL::R[0];
  constexpr int S = M / R;
  const C* __restrict__ w0 = static_cast<const C*>(p0 ? p0 : a.w0);
  const C* __restrict__ w1 = static_cast<const C*>(p1 ? p1 : a.w1);
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  constexpr int Nh = M / 3;
  for (int w = tid; w < V * S; w += NT) {
    const int v = w % V;
    const int i = w / V;
    const int z = z0 + v;
    C x[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int k = i + j * S;
      C zz = {T(0), T(0)};
      if (j * S >= Nh && j * S + S - 1 <= M - Nh) {
        // whole row segment inside the 3/2 pad: zero
      } else if (k < Nh) {
        const C u = w0[(size_t)k * M + z];
        const C q = w1[(size_t)k * M + z];
        zz = (k == 0) ? C{u.x, q.x} : C{u.x - q.y, u.y + q.x};
      } else if (k > M - Nh) {
        const int m = M - k;
        const C u = w0[(size_t)m * M + z];
        const C q = w1[(size_t)m * M + z];
        zz = C{u.x + q.y, q.x - u.y};
      }
      x[j] = zz;
    }
    Dft<R, +1, C>::run(x);
    pass_tw<PL, 0, +1>(x, tw, i);
    C* p = sm + PL::phys(i) * V + v;
#pragma unroll
    for (int k = 0; k < R; ++k) p[k * PL::pstride(0) * V] = x[k];
  }
  __syncthreads();
}

// Bulk tensor stores (TMA) from shared memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* smem, int x, int y, int z) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(map), "r"(s),
               "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void tma_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void tma_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Bulk tensor loads (TMA) into shared memory, completed on an mbarrier.
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_3d(const CUtensorMap* map, void* smem, unsigned long long* bar, int x, int y,
                                            int z) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(d),
      "l"(map), "r"(b), "r"(x), "r"(y), "r"(z)
      : "memory");
}
// Wait for phase `parity` of the mbarrier with non-blocking polls
// (mbarrier.test_wait), giving up after max_iter of them: a bound in time even
// if the expected transaction count were never reached.
__device__ __forceinline__ bool mbar_test_wait(unsigned long long* bar, unsigned parity, int max_iter) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  for (int i = 0; i < max_iter; ++i) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Wait for phase `parity` of the mbarrier, giving up after max_iter polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int max_iter) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  for (int i = 0; i < max_iter; ++i) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// First inverse DIF pass with each U-state row read once.  Butterfly i holds
// z[i + j S]; the mirrored entry z[M - k] = conj(u^[k]) + i conj(v^[k]) of a
// row k = i + j S < N/2 sits in butterfly S - i at index R-1-j.  Butterflies 0
// and S/2 are their own partners (at index (R-j) mod R and R-1-j).  Work item
// q < S/2 takes the pair (q, S - q), item 0 the two self-paired butterflies
// (0, S/2), so every item is two DFTs, V S / 2 items in all, and every row
// below N/2 is loaded by exactly one thread: half the global loads of an
// unpaired first pass.
template <typename T, class PL, int V, int NT>
__device__ __forceinline__ void row_first_pass_paired(const StepArgs& a, cplx<T>* sm, int z0, int tid) {
  using C = cplx<T>;
  constexpr int M = PL::M;
  constexpr int R = PL::R[0];
  constexpr int S = M / R;
  constexpr int SP = PL::pstride(0);
  constexpr int Nh = M / 3;
  constexpr int NQ = S / 2;
  static_assert(S % 2 == 0 && R % 2 == 0, "paired first pass needs an even stride and radix");
  const C* __restrict__ w0 = static_cast<const C*>(a.w0);
  const C* __restrict__ w1 = static_cast<const C*>(a.w1);
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  for (int w = tid; w < V * NQ; w += NT) {
    const int v = w % V;
    const int q = w / V;
    const bool self = q == 0;
    const int i2 = self ? S / 2 : S - q;
    const size_t col = (size_t)z0 + v;
    C x[R], y[R];
#pragma unroll
    for (int j = 0; j < R; ++j) x[j] = y[j] = C{T(0), T(0)};
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j * S >= Nh) continue;  // folded at compile time
      const int k1 = q + j * S;
      if (j * S + S - 1 < Nh || k1 < Nh) {
        const C u = w0[(size_t)k1 * M + col], qv = w1[(size_t)k1 * M + col];
        const C m = C{u.x + qv.y, qv.x - u.y};
        if (self) {
          if (j == 0) {
            x[0] = C{u.x, qv.x};
          } else {
            x[j] = C{u.x - qv.y, u.y + qv.x};
            x[(R - j) % R] = m;
          }
        } else {
          x[j] = C{u.x - qv.y, u.y + qv.x};
          y[R - 1 - j] = m;
        }
      }
      const int k2 = i2 + j * S;
      if (j * S + S - 1 < Nh || k2 < Nh) {
        const C u = w0[(size_t)k2 * M + col], qv = w1[(size_t)k2 * M + col];
        const C m = C{u.x + qv.y, qv.x - u.y};
        y[j] = C{u.x - qv.y, u.y + qv.x};
        if (self) y[R - 1 - j] = m;
        else x[R - 1 - j] = m;
      }
    }
    Dft<R, +1, C>::run(x);
    pass_tw<PL, 0, +1>(x, tw, q);
    {
      C* p = sm + PL::phys(q) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) p[k * SP * V] = x[k];
    }
    Dft<R, +1, C>::run(y);
    pass_tw<PL, 0, +1>(y, tw, i2);
    {
      C* p = sm + PL::phys(i2) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) p[k * SP * V] = y[k];
    }
  }
  __syncthreads();
}

// The paired first pass with its U-state rows brought in by the TMA unit: one
// elected thread issues 3D bulk tensor loads of the tile's rows below N/2
// (256-row boxes of both planes) into the tile region, laid out [plane][k][v];
// every thread reads its item's rows from there into registers, a barrier
// frees the region, and the DFTs write the tile as in row_first_pass_paired.
// No thread spends load instructions or LSU queue entries on global memory.
template <typename T, class PL, int V, int NT>
__device__ __forceinline__ void row_first_pass_tma(const StepArgs& a, cplx<T>* sm, int z0, int tid,
                                                   const TmaMaps& maps, unsigned long long* bar, int member) {
  using C = cplx<T>;
  constexpr int M = PL::M;
  constexpr int R = PL::R[0];
  constexpr int S = M / R;
  constexpr int SP = PL::pstride(0);
  constexpr int Nh = M / 3;
  constexpr int NQ = S / 2;
  constexpr int BOX = tma_box_rows(Nh);
  // one item per thread; threads beyond the V*NQ items only join the barriers
  static_assert(sizeof(C) == 8 && V * NQ <= NT && BOX >= 32, "one item per thread, FP32, boxes of 32+ rows");
  static_assert(S % 2 == 0 && R % 2 == 0, "paired first pass needs an even stride and radix");
  const bool live = V * NQ == NT || tid < V * NQ;
  const C* stg = sm;  // [plane][k < N/2][v]
  if (tid == 0) {
    mbar_expect_tx(bar, 2u * Nh * V * (unsigned)sizeof(C));
#pragma unroll 1
    for (int bx = 0; bx < Nh / BOX; ++bx) {
      tma_load_3d(&maps.w0, sm + (size_t)bx * BOX * V, bar, 2 * z0, bx * BOX, member);
      tma_load_3d(&maps.w1, sm + (size_t)(Nh + bx * BOX) * V, bar, 2 * z0, bx * BOX, member);
    }
  }
  if (!mbar_wait(bar, 0, a.dbg_wait0 ? 0 : 1 << 22)) {
    // the copies did not complete in time: report it and wait (bounded) for them
    // before the shared memory is used or released
    if (tid == 0) atomicExch(&a.sc->wait_timeout, 1);
    mbar_wait(bar, 0, 1 << 22);
  }
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  const int v = tid % V;
  const int q = tid / V;
  const bool self = q == 0;
  const int i2 = self ? S / 2 : S - q;
  C x[R], y[R];
#pragma unroll
  for (int j = 0; j < R; ++j) x[j] = y[j] = C{T(0), T(0)};
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (j * S >= Nh || !live) continue;  // the first test folds at compile time
    const int k1 = q + j * S;
    if (j * S + S - 1 < Nh || k1 < Nh) {
      const C u = stg[(size_t)k1 * V + v], qv = stg[(size_t)(Nh + k1) * V + v];
      const C m = C{u.x + qv.y, qv.x - u.y};
      if (self) {
        if (j == 0) {
          x[0] = C{u.x, qv.x};
        } else {
          x[j] = C{u.x - qv.y, u.y + qv.x};
          x[(R - j) % R] = m;
        }
      } else {
        x[j] = C{u.x - qv.y, u.y + qv.x};
        y[R - 1 - j] = m;
      }
    }
    const int k2 = i2 + j * S;
    if (j * S + S - 1 < Nh || k2 < Nh) {
      const C u = stg[(size_t)k2 * V + v], qv = stg[(size_t)(Nh + k2) * V + v];
      const C m = C{u.x + qv.y, qv.x - u.y};
      y[j] = C{u.x - qv.y, u.y + qv.x};
      if (self) y[R - 1 - j] = m;
      else x[R - 1 - j] = m;
    }
  }
  __syncthreads();  // every staged row is in registers: the tile is free
  if (live) {
    Dft<R, +1, C>::run(x);
    pass_tw<PL, 0, +1>(x, tw, q);
    {
      C* p = sm + PL::phys(q) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) p[k * SP * V] = x[k];
    }
    Dft<R, +1, C>::run(y);
    pass_tw<PL, 0, +1>(y, tw, i2);
    {
      C* p = sm + PL::phys(i2) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) p[k * SP * V] = y[k];
    }
  }
  __syncthreads();
}

// Last forward DIT pass of the row kernel fused with the Hermitian unpack.
// Butterfly i produces P[i + j S]; the conjugate partner P[M - i - j S] sits in
// butterfly S - i at index R-1-j (for i = 0 in butterfly 0 at (R-j) mod R, for
// i = S/2 in butterfly S/2 at R-1-j), so one thread transforms the pair
// (q, S - q), or (0, S/2) for q = 0, and writes
// A = (P[k] + conj P[M-k]) / 2 and B = (P[k] - conj P[M-k]) / (2i) for k < N/2
// straight to the work planes.  Outputs with N/2 <= k <= M - N/2 are never formed.
template <typename T, class PL, int V, int NT>
__device__ __forceinline__ void row_last_pass_paired(const StepArgs& a, cplx<T>* sm, int z0, int tid) {
  using C = cplx<T>;
  constexpr int M = PL::M;
  constexpr int R = PL::R[0];
  constexpr int S = M / R;
  constexpr int SP = PL::pstride(0);
  constexpr int Nh = M / 3;
  constexpr int NQ = S / 2;
  static_assert(S % 2 == 0 && R % 2 == 0, "paired unpack needs an even stride and radix");
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  C* __restrict__ w0 = static_cast<C*>(a.w0);
  C* __restrict__ w1 = static_cast<C*>(a.w1);
  for (int w = tid; w < V * NQ; w += NT) {
    const int v = w % V;
    const int q = w / V;
    const bool self = q == 0;
    const int i2 = self ? S / 2 : S - q;
    C y1[R], y2[R];
    {
      const C* p = sm + PL::phys(q) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) y1[k] = p[k * SP * V];
      pass_tw<PL, 0, -1>(y1, tw, q);
      Dft<R, -1, C>::run(y1);
    }
    {
      const C* p = sm + PL::phys(i2) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) y2[k] = p[k * SP * V];
      pass_tw<PL, 0, -1>(y2, tw, i2);
      Dft<R, -1, C>::run(y2);
    }
    const size_t col = (size_t)z0 + v;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j * S >= Nh) continue;  // folded at compile time
      const int k1 = q + j * S;
      if (j * S + S - 1 < Nh || k1 < Nh) {
        const C p = y1[j];
        const C c = self ? y1[(R - j) % R] : y2[R - 1 - j];
        w0[(size_t)k1 * M + col] = C{T(0.5) * (p.x + c.x), T(0.5) * (p.y - c.y)};
        w1[(size_t)k1 * M + col] = C{T(0.5) * (p.y + c.y), T(-0.5) * (p.x - c.x)};
      }
      const int k2 = i2 + j * S;
      if (j * S + S - 1 < Nh || k2 < Nh) {
        const C p = y2[j];
        const C c = self ? y2[R - 1 - j] : y1[R - 1 - j];
        w0[(size_t)k2 * M + col] = C{T(0.5) * (p.x + c.x), T(0.5) * (p.y - c.y)};
        w1[(size_t)k2 * M + col] = C{T(0.5) * (p.y + c.y), T(-0.5) * (p.x - c.x)};
      }
    }
  }
}


// The paired last pass with the stores handed to the TMA unit: each thread
// (one item, V S / 2 == NT) keeps its A, B rows in registers, the block
// rewrites the tile as dense [plane][row][v] boxes and one thread issues the
// bulk tensor stores, so no thread spends issue slots or LSU queue entries on
// the plane writes and they drain while the next tile starts.
template <typename T, class PL, int V, int NT>
__device__ __forceinline__ void row_last_pass_tma(const StepArgs& a, cplx<T>* sm, int z0, int tid,
                                                  const TmaMaps& maps, int member) {
  using C = cplx<T>;
  constexpr int M = PL::M;
  constexpr int R = PL::R[0];
  constexpr int S = M / R;
  constexpr int SP = PL::pstride(0);
  constexpr int Nh = M / 3;
  constexpr int NQ = S / 2;
  constexpr int JN = (Nh + S - 1) / S;  // j with j S < N/2
  constexpr int BOX = tma_box_rows(Nh);
  // one item per thread; threads beyond the V*NQ items only join the barriers
  static_assert(sizeof(C) == 8 && V * NQ <= NT && BOX >= 32, "one item per thread, FP32, boxes of 32+ rows");
  static_assert(size_t(2) * Nh * V <= size_t(PL::PADM) * V, "staging fits in the tile");
  const bool live = V * NQ == NT || tid < V * NQ;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  const int v = tid % V;
  const int q = live ? tid / V : 0;
  const bool self = q == 0;
  const int i2 = self ? S / 2 : S - q;
  C y1[R], y2[R];
  {
    const C* p = sm + PL::phys(q) * V + v;
#pragma unroll
    for (int k = 0; k < R; ++k) y1[k] = p[k * SP * V];
    pass_tw<PL, 0, -1>(y1, tw, q);
    Dft<R, -1, C>::run(y1);
  }
  {
    const C* p = sm + PL::phys(i2) * V + v;
#pragma unroll
    for (int k = 0; k < R; ++k) y2[k] = p[k * SP * V];
    pass_tw<PL, 0, -1>(y2, tw, i2);
    Dft<R, -1, C>::run(y2);
  }
  C A1[JN], B1[JN], A2[JN], B2[JN];
#pragma unroll
  for (int j = 0; j < JN; ++j) {
    const C p1 = y1[j], c1 = self ? y1[(R - j) % R] : y2[R - 1 - j];
    A1[j] = C{T(0.5) * (p1.x + c1.x), T(0.5) * (p1.y - c1.y)};
    B1[j] = C{T(0.5) * (p1.y + c1.y), T(-0.5) * (p1.x - c1.x)};
    const C p2 = y2[j], c2 = self ? y2[R - 1 - j] : y1[R - 1 - j];
    A2[j] = C{T(0.5) * (p2.x + c2.x), T(0.5) * (p2.y - c2.y)};
    B2[j] = C{T(0.5) * (p2.y + c2.y), T(-0.5) * (p2.x - c2.x)};
  }
  __syncthreads();  // every read of the tile is done: reuse it as the staging area
  C* stg = sm;      // [plane][k < N/2][v]
#pragma unroll
  for (int j = 0; j < JN; ++j) {
    if (!live) break;
    const int k1 = q + j * S, k2 = i2 + j * S;
    if (k1 < Nh) {
      stg[(size_t)k1 * V + v] = A1[j];
      stg[(size_t)(Nh + k1) * V + v] = B1[j];
    }
    if (k2 < Nh) {
      stg[(size_t)k2 * V + v] = A2[j];
      stg[(size_t)(Nh + k2) * V + v] = B2[j];
    }
  }
  fence_proxy_async_smem();
  __syncthreads();
  if (tid == 0) {
#pragma unroll 1
    for (int bx = 0; bx < Nh / BOX; ++bx) {
      tma_store_3d(&maps.w0, stg + (size_t)bx * BOX * V, 2 * z0, bx * BOX, member);
      tma_store_3d(&maps.w1, stg + (size_t)(Nh + bx * BOX) * V, 2 * z0, bx * BOX, member);
    }
    tma_commit();
    tma_wait_read();  // the shared memory stays the block's until the engine has read it
  }
}

// L2 prefetch helpers.  `cp.async.bulk.prefetch.L2` pulls a contiguous,
// 16-byte aligned range into L2 without occupying registers or the LSU queue;
// `prefetch.global.L2` does one line.  Both are hints with no visible effect.
__device__ __forceinline__ void l2_prefetch_bulk(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void l2_prefetch_line(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// The middle of the row pass: last inverse DIF pass -> products -> first
// forward DIT pass, one smem round trip.  NEXTDT needs the CFL maximum; the
// sum of u^2 + v^2 here only serves the finiteness check (a NaN drops out of a
// max), so it is a plain sum in the working precision.  The diagnostic
// mean(u^2 + v^2) is k_phys's compensated FP64 sum (pal_diagnostics).
template <typename T, class PL, int V, int NT>
__device__ __forceinline__ void row_products(cplx<T>* sm, int tid, bool stats, T& mx, T& acc) {
  using C = cplx<T>;
  constexpr int R = PL::RP;
  constexpr int NB = V * (PL::M / R);
  for (int w = tid; w < NB; w += NT) {
    const int v = w % V;
    const int b = w / V;
    C* p = sm + b * (R + 1) * V + v;
    C x[R];
#pragma unroll
    for (int j = 0; j < R; ++j) x[j] = p[j * V];
    Dft<R, +1, C>::run(x);
    if (stats) {
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const T u = x[j].x, q = x[j].y;
        mx = fmax(mx, fabs(u) + fabs(q));
        acc = fma(u, u, fma(q, q, acc));
      }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const T u = x[j].x, q = x[j].y;
      x[j] = C{u * u - q * q, u * q};
    }
    Dft<R, -1, C>::run(x);
#pragma unroll
    for (int j = 0; j < R; ++j) p[j * V] = x[j];
  }
  __syncthreads();
}

// k_row: U-state rows -> P-state rows (products), optional CFL statistics.
// PF bit 0: the tile one wave ahead (blockIdx.x + a.ahead) is pulled into L2
// first, so that the block that will run it finds its rows there.
// PF bit 1: the first pass reads every U-state row once (row_first_pass_paired).
// PF bit 2 (value 4): the last pass stores through the TMA unit (row_last_pass_tma).
// PF bit 3 (value 8): the first pass loads through the TMA unit (row_first_pass_tma).
// PF bit 5 (value 32): with bit 0, the prefetched tile is two waves ahead.
// PF bit 4 (value 16): registers are capped so that as many blocks share an SM
// as its shared memory holds tiles (row_tiles_per_sm); without it the
// launch bound names no block count and the compiler chooses.
template <typename T, class PL, int V>
constexpr int row_tiles_per_sm() {
  // 228 KB of shared memory per SM, 1 KB of it reserved per block, plus the
  // block's static shared memory (mbarrier, reduction scratch)
  return int(size_t(228 * 1024) / (size_t(PL::PADM) * V * sizeof(cplx<T>) + 1024 + 256));
}
// ENS: the ensemble's one-launch row pass, which honours F_STATS_MAX.
template <typename T, class PL, int V, int NT, int PF, bool ENS = false>
__device__ __forceinline__ void row_body(const StepArgs& a0, const TmaMaps& maps, const Blk bk) {
  using C = cplx<T>;
  const StepArgs a = member_args(a0, sizeof(C), bk.y);
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int M = PL::M;
  const int tid = threadIdx.x;
  const int z0 = bk.x * V;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);

  if constexpr ((PF & 1) != 0) {
    const int nb = bk.x + a.ahead;
    if (a.ahead > 0 && nb < bk.nx) {
      constexpr int Nh = M / 3;
      const cplx<T>* w0 = static_cast<const cplx<T>*>(a.w0) + (size_t)nb * V;
      const cplx<T>* w1 = static_cast<const cplx<T>*>(a.w1) + (size_t)nb * V;
      for (int r = tid; r < 2 * Nh; r += NT) l2_prefetch_line((r < Nh ? w0 : w1) + (size_t)(r < Nh ? r : r - Nh) * M);
    }
  }
  if constexpr ((PF & 8) != 0) {
    __shared__ __align__(8) unsigned long long tma_bar;
    if (tid == 0) mbar_init(&tma_bar, 1);
    __syncthreads();
    row_first_pass_tma<T, PL, V, NT>(a, sm, z0, tid, maps, &tma_bar, bk.y);
  } else if constexpr ((PF & 2) != 0) {
    row_first_pass_paired<T, PL, V, NT>(a, sm, z0, tid);
  } else {
    row_first_pass<T, PL, V, NT>(a, sm, z0, tid);
  }
  dif_range<T, PL, V, NT, +1, 1, PL::NP - 1>(sm, tw, tid);
  const bool stats = (a.flags & (ENS ? (F_STATS | F_STATS_MAX) : F_STATS)) != 0;
  T mx = T(0), acc = T(0);
  row_products<T, PL, V, NT>(sm, tid, stats, mx, acc);
  if constexpr (sizeof(C) == 8) {
    dit_range<T, PL, V, NT, -1, PL::NP - 2, 1>(sm, tw, tid);
    if constexpr ((PF & 4) != 0)
      row_last_pass_tma<T, PL, V, NT>(a, sm, z0, tid, maps, bk.y);
    else
      row_last_pass_paired<T, PL, V, NT>(a, sm, z0, tid);
  } else {
    dit_range<T, PL, V, NT, -1, PL::NP - 2, 0>(sm, tw, tid);
    // unpack P = FFT(a + i b) into A = F(a), B = F(b) for kx < N/2 and store
    C* __restrict__ w0 = static_cast<C*>(a.w0);
    C* __restrict__ w1 = static_cast<C*>(a.w1);
    constexpr int Nh = M / 3;
    for (int w = tid; w < V * Nh; w += NT) {
      const int v = w % V;
      const int k = w / V;
      const C p = sm[PL::phys(k) * V + v];
      const C q = sm[PL::phys(k == 0 ? 0 : M - k) * V + v];
      w0[(size_t)k * M + z0 + v] = C{T(0.5) * (p.x + q.x), T(0.5) * (p.y - q.y)};
      w1[(size_t)k * M + z0 + v] = C{T(0.5) * (p.y + q.y), T(-0.5) * (p.x - q.x)};
    }
  }
  if constexpr (ENS && sizeof(T) == 4) {
    if (a.flags & F_STATS)
      finish_stats<NT, false>(a, double(mx), double(acc), 0.0, M, tid, bk);
    else if (a.flags & F_STATS_MAX)
      mark_step_max(a, mx, acc, tid);
  } else {
    if (stats) finish_stats<NT, false>(a, double(mx), double(acc), 0.0, M, tid, bk);
  }
}
template <typename T, class PL, int V, int NT, int PF>
__global__ void __launch_bounds__(NT, (PF & 16) ? row_tiles_per_sm<T, PL, V>() : 0)
    k_row(StepArgs a0, const __grid_constant__ TmaMaps maps) {
  row_body<T, PL, V, NT, PF>(a0, maps, hw_blk());
}

// k_phys: U-state rows -> physical u, v (statistics, optional plane store).
template <typename T, class PL, int V, int NT>
__device__ __forceinline__ void phys_body(const StepArgs& a0, const Blk bk) {
  using C = cplx<T>;
  const StepArgs a = member_args(a0, sizeof(C), bk.y);
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int M = PL::M;
  const int tid = threadIdx.x;
  const int z0 = bk.x * V;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  row_first_pass<T, PL, V, NT>(a, sm, z0, tid);
  dif_range<T, PL, V, NT, +1, 1, PL::NP>(sm, tw, tid);
  T mx = T(0), accp = T(0);
  double acc = 0.0, comp = 0.0;  // F_DIAG: compensated FP64 sum of u^2 + v^2
  T* __restrict__ ph = static_cast<T*>(a.phys);
  const bool store = (a.flags & F_PHYS) != 0;
  const bool diag = (a.flags & F_DIAG) != 0;
  for (int w = tid; w < V * M; w += NT) {
    const int v = w % V;
    const int pos = w / V;
    const C val = sm[PL::phys(pos) * V + v];
    mx = fmax(mx, fabs(val.x) + fabs(val.y));
    if (diag) {
      const double du = double(val.x), dq = double(val.y);
      csum_add(acc, comp, fma(du, du, dq * dq));
    } else {
      accp = fma(val.x, val.x, fma(val.y, val.y, accp));  // finiteness check only
    }
    if (store) {
      const int n = PL::freq(pos);
      ph[(size_t)(z0 + v) * M + n] = val.x;
      ph[(size_t)M * M + (size_t)(z0 + v) * M + n] = val.y;
    }
  }
  if (diag)
    finish_stats<NT, true>(a, double(mx), acc, comp, M, tid, bk);
  else
    finish_stats<NT, false>(a, double(mx), double(accp), 0.0, M, tid, bk);
}
template <typename T, class PL, int V, int NT>
__global__ void __launch_bounds__(NT) k_phys(StepArgs a0) {
  phys_body<T, PL, V, NT>(a0, hw_blk());
}

// --------------------------------------------------------------------------
// Spectral update of one mode (kx, z) and the omega -> velocity inversion.
// CNAB2 (turbo_simulator.py:1642-1652) and LS-IMEX-RK3 (1826-1837) share the
// form  om' = [(1 - K2 h1) om + c2 fn + c3 fnm1] / (1 + K2 h2).
template <typename T>
struct ModeCoef {
  T h1, h2, c2, c3, divxz;
  T h1n, c3n;  // the next RK3 stage's h1 and c3 (F_Q_OUT)
};

// 16-byte asynchronous global -> shared copies (Ampere+ cp.async).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Implicit / explicit weights of the column update, formed in FP64 from the
// device scalars: CNAB2 (turbo_simulator.py:1745-1752) or one RK3 stage.
// ENS: the ensemble's one-launch column pass, which honours F_DT_FROM_MAX.
template <typename T, bool ENS = false>
__device__ __forceinline__ ModeCoef<T> col_coef(const StepArgs& a, int N) {
  ModeCoef<T> cf;
  const DevScalars* sc = a.sc;
  double dt = sc->dt;
  if constexpr (ENS) {
    if (a.flags & F_DT_FROM_MAX) dt = nextdt_from_mark(a).dt;
  }
  const double visc = sc->visc;
  double h1, h2, c2, c3;
  if (a.scheme == 0) {
    const double cnm1 = sc->cnm1;
    h1 = h2 = (0.5 * visc) * dt;
    c2 = (0.5 * dt) * (2.0 + cnm1);
    c3 = (-0.5 * dt) * cnm1;
  } else {
    h1 = (a.beta * dt) * visc;
    h2 = (a.alpha * dt) * visc;
    c2 = a.alpha * dt;
    c3 = a.beta * dt;
  }
  cf.h1n = a.scheme == 0 ? T(0) : T((a.beta_next * dt) * visc);
  cf.c3n = a.scheme == 0 ? T(0) : T(a.beta_next * dt);
  cf.h1 = T(h1);
  cf.h2 = T(h2);
  cf.c2 = T(c2);
  cf.c3 = T(c3);
  const T m32 = T(1.5) * T(N);
  cf.divxz = T(1) / (m32 * m32);
  return cf;
}

// The coefficients formed once per block: col_coef's FP64 arithmetic (and the
// FP64 division of F_DT_FROM_MAX) is uniform across the block, and FP64 issue
// is scarce, so warp 0 alone forms them and thread 0 leaves them in shared
// memory; the block reads them after its next barrier.
template <typename T, bool ENS>
__device__ __forceinline__ void col_coef_shared(const StepArgs& a, int N, int tid, ModeCoef<T>* s) {
  if (tid < 32) {
    const ModeCoef<T> c = col_coef<T, ENS>(a, N);
    if (tid == 0) *s = c;
  }
}

// Planar column tile for bulk tensor copies: plane v (A / u^, B / v^) starts at
// v * PB; within a plane, position k sits at k + 2 (k / RP), i.e. every RP
// positions (RP complex = 48 floats) are followed by 2 pad slots.  A group of
// RP + 2 slots is then one 52-float row of a TMA box over a 48-float tensor
// dimension: loads fill the pads with zeros and stores skip them.  The plane
// stride keeps both planes 128-byte aligned.
template <class PL>
struct ColPlanar {
  static constexpr int RP = PL::RP;
  static constexpr int PADM = PL::M + 2 * (PL::M / RP);         // slots per plane
  static constexpr int PB = ((PADM * 8 + 127) / 128) * 128 / 8;  // plane stride (FP32 complex)
  static constexpr int G = PL::M / RP;                          // groups per plane
  static constexpr int GBOX = col_box_groups(G);                // groups per TMA box
  static __device__ __forceinline__ int phys(int k) { return k + 2 * (k / RP); }
  static constexpr int pstride(int p) { return PL::stride(p) == 1 ? 1 : PL::stride(p) + 2 * (PL::stride(p) / RP); }
  static constexpr bool fits = PL::M % RP == 0 && G % GBOX == 0 && (2 * RP + 4) * 4 % 16 == 0;  // whole groups, boxes
};

// Middle of the column pass: last forward DIF -> nonlinear term, update,
// inversion -> first inverse DIT.  The two lanes of a butterfly hold A and B;
// lane 0 updates the even positions and lane 1 the odd ones, trading operands
// and results by shuffle.  When 3 divides the radix, the de-aliased band
// (frequencies N/2 .. N-1, the middle third of the positions) is known at
// compile time and skipped.  om / fm are read from s_om / s_fm when SMEM_OM.
// With PERM, om / fm are columns in butterfly-major order (Plan::mid_perm):
// the lanes of a warp then read and write consecutive elements.  With HOIST a
// lane requests all its om / fm values before the butterfly's shared-memory
// loads and DFT, so their latency overlaps that work (the update loop stores
// to om / fm, so the compiler cannot move later loads above earlier stores).
//
// Within an LS-IMEX-RK3 step the stage update
//   om' = ((1 - K2 h1) om + c2 fn + c3 fnm1) / (1 + K2 h2)
// uses om and fnm1 only through q = (1 - K2 h1) om + c3 fnm1, and the next
// stage's weights are known when a stage ends.  With F_Q_OUT a stage stores
// that q for the next stage in place of om (and no fn); with F_Q_IN the stage
// reads q and no fnm1; F_NO_FM_IN skips the fnm1 read of the first stage,
// whose c3 is 0.  The last stage stores om and fn as the reference state.
// QM: the F_Q_* / F_NO_FM_IN flags are honoured (a separate instantiation, so
// that the plain update keeps its register budget).
//
// PLANAR: the tile is ColPlanar's two padded planes instead of the
// interleaved [slot][v] layout; half-warps hold one plane (lane bit 4), so the
// two planes of a butterfly trade operands across lanes 16 apart.
template <typename T, class PL, int NT, bool SMEM_OM, bool PERM, bool HOIST = false, bool QM = false,
          bool PLANAR = false>
__device__ __forceinline__ void col_middle(cplx<T>* sm, const cplx<T>* s_om, const cplx<T>* s_fm,
                                           cplx<T>* __restrict__ om, cplx<T>* __restrict__ fm,
                                           const ModeCoef<T>& cf, int kx, int tid, int flags) {
  const bool q_in = QM && (flags & F_Q_IN) != 0;
  const bool fm_in = !QM || (flags & (F_Q_IN | F_NO_FM_IN)) == 0;
  const bool q_out = QM && (flags & F_Q_OUT) != 0;
  using C = cplx<T>;
  constexpr int M = PL::M;
  constexpr int V = 2;
  constexpr int N = 2 * M / 3, Nh = M / 3;
  constexpr int R = PL::RP;
  constexpr int NB = V * (M / R);
  constexpr int FSTEP = M / R;
  constexpr bool BAND_CT = (R % 3 == 0) && ((R / 3) % 2 == 0);
  const T ax = T(kx);
  constexpr int ES = PLANAR ? 1 : V;           // element stride of a butterfly in the tile
  constexpr int XL = PLANAR ? 16 : 1;          // lane distance between the two planes
  for (int w0i = 0; w0i < NB; w0i += NT) {
    const int w = w0i + tid;
    const bool act = w < NB;
    const int v = PLANAR ? ((w >> 4) & 1) : (w & 1);
    const int b = act ? (PLANAR ? (((w >> 5) << 4) | (w & 15)) : (w >> 1)) : 0;
    C* p;
    if constexpr (PLANAR)
      p = sm + v * ColPlanar<PL>::PB + b * (R + 2);
    else
      p = sm + b * (R + 1) * V + v;
    const int fb = PL::freq(b * R);
    constexpr int NH = HOIST ? R / 2 : 1;
    C h_o[NH], h_f[NH];
    if constexpr (HOIST) {
#pragma unroll
      for (int jj = 0; jj < R / 2; ++jj) {
        const int j = 2 * jj;
        h_o[jj] = h_f[jj] = C{T(0), T(0)};
        if (BAND_CT && j >= R / 3 && j < 2 * R / 3) continue;
        const int f = fb + (j + v) * FSTEP;
        const int z = f < Nh ? f : f - Nh;
        const int zi = PERM ? (j + v) * FSTEP + b : z;
        if (act && (BAND_CT || f < Nh || f >= N)) {
          h_o[jj] = om[zi];
          if (fm_in) h_f[jj] = fm[zi];
        }
      }
    }
    C x[R];
    if constexpr (PLANAR && sizeof(C) == 8) {
      // a planar butterfly is R contiguous, 16-byte aligned slots: pairs by 128-bit loads
#pragma unroll
      for (int j = 0; j < R; j += 2) {
        const float4 t = act ? reinterpret_cast<const float4*>(p)[j / 2] : make_float4(0.f, 0.f, 0.f, 0.f);
        x[j] = C{t.x, t.y};
        x[j + 1] = C{t.z, t.w};
      }
    } else {
#pragma unroll
      for (int j = 0; j < R; ++j) x[j] = act ? p[j * ES] : C{T(0), T(0)};
    }
    Dft<R, -1, C>::run(x);
#pragma unroll
    for (int j = 0; j < R; j += 2) {
      if (BAND_CT && j >= R / 3 && j < 2 * R / 3) {
        x[j] = C{T(0), T(0)};
        x[j + 1] = C{T(0), T(0)};
        continue;
      }
      // lane 0 takes position j, lane 1 position j+1
      const C send = v == 0 ? x[j + 1] : x[j];
      C recv;
      recv.x = __shfl_xor_sync(0xffffffffu, send.x, XL);
      recv.y = __shfl_xor_sync(0xffffffffu, send.y, XL);
      const C Az = v == 0 ? x[j] : recv;
      const C Bz = v == 0 ? recv : x[j + 1];
      const int f = fb + (j + v) * FSTEP;
      const bool inband = act && (BAND_CT || f < Nh || f >= N);
      const int z = f < Nh ? f : f - Nh;
      C uh = {T(0), T(0)}, vh = {T(0), T(0)};
      const int zi = PERM ? (j + v) * FSTEP + b : z;
      if (inband) {
        const C o = SMEM_OM ? s_om[z] : (HOIST ? h_o[j / 2] : om[zi]);
        C fo = {T(0), T(0)};
        if (fm_in) fo = SMEM_OM ? s_fm[z] : (HOIST ? h_f[j / 2] : fm[zi]);
        const T gz = T(z < Nh ? z : z - N);
        const T K2 = ax * ax + gz * gz;
        const T GA = gz * ax;
        const T G2mA2 = gz * gz - ax * ax;
        C fn = {T(0), T(0)};
        if (z != Nh) {
          fn.x = (Az.x * GA + Bz.x * G2mA2) * cf.divxz;
          fn.y = (Az.y * GA + Bz.y * G2mA2) * cf.divxz;
        }
        const T rden = T(1) / (T(1) + K2 * cf.h2);
        C on;
        if (q_in) {
          on.x = (o.x + cf.c2 * fn.x) * rden;
          on.y = (o.y + cf.c2 * fn.y) * rden;
        } else {
          const T c1 = T(1) - K2 * cf.h1;
          on.x = (c1 * o.x + cf.c2 * fn.x + cf.c3 * fo.x) * rden;
          on.y = (c1 * o.y + cf.c2 * fn.y + cf.c3 * fo.y) * rden;
        }
        if (q_out) {
          const T c1n = T(1) - K2 * cf.h1n;
          om[zi] = C{c1n * on.x + cf.c3n * fn.x, c1n * on.y + cf.c3n * fn.y};
        } else {
          om[zi] = on;
          fm[zi] = fn;
        }
        if (kx >= 1) {
          const T ik = T(1) / K2;
          const C t = {on.x * ik, on.y * ik};
          uh = C{t.y * gz, -t.x * gz};
          vh = C{-t.y * ax, t.x * ax};
        } else if (z >= 1) {
          const T ig = T(1) / gz;
          uh = C{on.y * ig, -on.x * ig};
        }
      }
      // lane 0 keeps u^ of position j and receives u^ of j+1; lane 1 the v^ pair
      const C send2 = v == 0 ? vh : uh;
      C recv2;
      recv2.x = __shfl_xor_sync(0xffffffffu, send2.x, XL);
      recv2.y = __shfl_xor_sync(0xffffffffu, send2.y, XL);
      x[j] = v == 0 ? uh : recv2;
      x[j + 1] = v == 0 ? recv2 : vh;
    }
    Dft<R, +1, C>::run(x);
    if (act) {
      if constexpr (PLANAR && sizeof(C) == 8) {
#pragma unroll
        for (int j = 0; j < R; j += 2)
          reinterpret_cast<float4*>(p)[j / 2] = make_float4(x[j].x, x[j].y, x[j + 1].x, x[j + 1].y);
      } else {
#pragma unroll
        for (int j = 0; j < R; ++j) p[j * ES] = x[j];
      }
    }
  }
  __syncthreads();
}

// Last inverse DIT pass of the column straight into the U planes.
template <typename T, class PL, int NT>
__device__ __forceinline__ void col_last_pass(const cplx<T>* sm, cplx<T>* __restrict__ w0, cplx<T>* __restrict__ w1,
                                              const cplx<T>* __restrict__ tw, int kx, int tid) {
  using C = cplx<T>;
  constexpr int M = PL::M;
  constexpr int V = 2;
  constexpr int R = PL::R[0];
  constexpr int S = M / R;
  for (int w = tid; w < V * S; w += NT) {
    const int v = w & 1;
    const int i = w >> 1;
    C* __restrict__ dst = (v == 0 ? w0 : w1) + (size_t)kx * M;
    const C* p = sm + PL::phys(i) * V + v;
    C x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = p[k * PL::pstride(0) * V];
    pass_tw<PL, 0, +1>(x, tw, i);
    Dft<R, +1, C>::run(x);
#pragma unroll
    for (int j = 0; j < R; ++j) dst[i + j * S] = x[j];
  }
}

// Time / cnm1 bookkeeping of the step, done once by the last block to finish.
template <int NT, bool ENS = false>
__device__ __forceinline__ void col_finish(const StepArgs& a, int tid, int nx) {
  if (a.flags & (F_ADVANCE | F_CNM1)) {
    if (last_block(&a.sc->col_counter, tid, nx) && tid == 0) {
      DevScalars* sc = a.sc;
      if constexpr (ENS) {
        if (a.flags & F_DT_FROM_MAX) {  // every block has read the old dt, cn and step_max
          const NextDt nd = nextdt_from_mark(a);
          sc->maxabs = nd.maxabs;
          sc->cflm = nd.cflm;
          sc->dt = nd.dt;
          sc->cn = nd.cn;
          sc->step_max = 0u;
        }
      }
      if (a.flags & F_ADVANCE) {
        sc->t += sc->dt;
        sc->it += 1;
      }
      if (a.flags & F_CNM1) sc->cnm1 = sc->cn;
      sc->col_counter = 0u;
    }
  }
}

// k_col: P-state column -> (om, fnm1 update) -> U-state column.  With PREF == 1
// the column's om and fnm1 are copied into shared memory asynchronously at
// entry, so the update reads them without exposed global latency; PREF == 2
// hoists each lane's om / fnm1 loads above its DFT (col_middle HOIST), PREF == 3
// also overlaps the pass-0 loads of a thread's next butterfly.  With
// PERM the kernel works on om_p / fm_p (butterfly-major columns of M elements).
// QM: the RK3 stage flags F_Q_IN / F_Q_OUT / F_NO_FM_IN are honoured (col_middle).
// ENS: the ensemble's one-launch pass: F_DT_FROM_MAX honoured, and the FP64
// coefficients formed once per block (col_coef_shared), which pays with the
// ensemble's many small column blocks.
template <typename T, class PL, int NT, int PREF, bool PERM, bool QM = true, bool ENS = false>
__device__ __forceinline__ void col_body(const StepArgs& a0, const Blk bk) {
  using C = cplx<T>;
  const StepArgs a = member_args(a0, sizeof(C), bk.y);
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int M = PL::M;
  constexpr int V = 2;
  const int tid = threadIdx.x;
  const int kx = bk.x;
  constexpr int N = 2 * M / 3;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  C* __restrict__ w0 = static_cast<C*>(a.w0);
  C* __restrict__ w1 = static_cast<C*>(a.w1);
  C* __restrict__ om = PERM ? static_cast<C*>(a.om_p) + (size_t)kx * M : static_cast<C*>(a.om) + (size_t)kx * N;
  C* __restrict__ fm = PERM ? static_cast<C*>(a.fm_p) + (size_t)kx * M : static_cast<C*>(a.fnm1) + (size_t)kx * N;
  C* s_om = sm + PL::PADM * V;
  C* s_fm = s_om + N;
  if constexpr (PREF == 1 && !PERM) {
    constexpr int CH = N * (int)sizeof(C) / 16;
    for (int c = tid; c < 2 * CH; c += NT) {
      const bool second = c >= CH;
      const int cc = second ? c - CH : c;
      cp_async16(reinterpret_cast<char*>(second ? s_fm : s_om) + 16 * cc,
                 reinterpret_cast<const char*>(second ? fm : om) + 16 * cc);
    }
    cp_async_commit();
  }
  __shared__ ModeCoef<T> s_cf;
  ModeCoef<T> cf0;
  if constexpr (ENS)
    col_coef_shared<T, true>(a, N, tid, &s_cf);  // read after the barriers of pass 0
  else
    cf0 = col_coef<T>(a, N);

  // pass 0 (forward z-DIF) straight from the P planes.  PREF == 3: the loads
  // of a thread's next butterfly are issued before the current one's DFT.
  if constexpr (PREF == 3 && (V * (M / PL::R[0])) % NT == 0) {
    constexpr int R = PL::R[0];
    constexpr int S = M / R;
    constexpr int IT = V * S / NT;
    C xn[R];
    {
      const C* __restrict__ src = ((tid & 1) == 0 ? w0 : w1) + (size_t)kx * M;
#pragma unroll
      for (int j = 0; j < R; ++j) xn[j] = src[(tid >> 1) + j * S];
    }
#pragma unroll 1
    for (int it = 0; it < IT; ++it) {
      const int w = tid + it * NT;
      const int v = w & 1;
      const int i = w >> 1;
      C x[R];
#pragma unroll
      for (int j = 0; j < R; ++j) x[j] = xn[j];
      if (it + 1 < IT) {
        const int wn = w + NT;
        const C* __restrict__ src = ((wn & 1) == 0 ? w0 : w1) + (size_t)kx * M;
#pragma unroll
        for (int j = 0; j < R; ++j) xn[j] = src[(wn >> 1) + j * S];
      }
      Dft<R, -1, C>::run(x);
      pass_tw<PL, 0, -1>(x, tw, i);
      C* p = sm + PL::phys(i) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) p[k * PL::pstride(0) * V] = x[k];
    }
    __syncthreads();
  } else {
    constexpr int R = PL::R[0];
    constexpr int S = M / R;
    for (int w = tid; w < V * S; w += NT) {
      const int v = w & 1;
      const int i = w >> 1;
      const C* __restrict__ src = (v == 0 ? w0 : w1) + (size_t)kx * M;
      C x[R];
#pragma unroll
      for (int j = 0; j < R; ++j) x[j] = src[i + j * S];
      Dft<R, -1, C>::run(x);
      pass_tw<PL, 0, -1>(x, tw, i);
      C* p = sm + PL::phys(i) * V + v;
#pragma unroll
      for (int k = 0; k < R; ++k) p[k * PL::pstride(0) * V] = x[k];
    }
    __syncthreads();
  }
  dif_range<T, PL, V, NT, -1, 1, PL::NP - 1>(sm, tw, tid);
  if constexpr (PREF == 1 && !PERM) {
    cp_async_wait_all();
    __syncthreads();
  }
  const ModeCoef<T> cf = ENS ? s_cf : cf0;
  col_middle<T, PL, NT, PREF == 1 && !PERM, PERM, PREF == 2 || PREF == 3, QM>(sm, s_om, s_fm, om, fm, cf, kx,
                                                                             tid, a.flags);
  dit_range<T, PL, V, NT, +1, PL::NP - 2, 1>(sm, tw, tid);
  col_last_pass<T, PL, NT>(sm, w0, w1, tw, kx, tid);
  col_finish<NT, ENS>(a, tid, bk.nx);
}
template <typename T, class PL, int NT, int PREF, bool PERM, bool QM = true>
__global__ void __launch_bounds__(NT) k_col(StepArgs a0) {
  col_body<T, PL, NT, PREF, PERM, QM>(a0, hw_blk());
}

// One DIF (DIT = false) or DIT pass over a planar column tile (ColPlanar):
// item w is butterfly ((w >> 5) << 4) | (w & 15) of plane (w >> 4) & 1, so a
// half-warp reads 16 consecutive butterflies of one plane.  The arithmetic is
// dif_pass / dit_pass's; only the addressing differs.
template <typename T, class PL, int NT, int P, int SIGN, bool DIT>
__device__ __forceinline__ void col_pass_planar(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  using C = cplx<T>;
  using CP = ColPlanar<PL>;
  constexpr int R = PL::R[P];
  constexpr int L = PL::span(P);
  constexpr int S = L / R;
  constexpr int SP = CP::pstride(P);
  constexpr int NB = 2 * (PL::M / R);
  static_assert((PL::M / R) % 16 == 0 && NT % 32 == 0, "whole half-warps per plane");
  static_assert(S == 1 || S % CP::RP == 0, "strides other than the last are whole pad groups");
  for (int w = tid; w < NB; w += NT) {
    const int v = (w >> 4) & 1;
    const int b = ((w >> 5) << 4) | (w & 15);
    const int blk = b / S;
    const int i = b - blk * S;
    C* p = sm + v * CP::PB + CP::phys(blk * L + i);
    C x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = p[k * SP];
    if constexpr (DIT) {
      if constexpr (S > 1) pass_tw<PL, P, SIGN>(x, tw, i);
      Dft<R, SIGN, C>::run(x);
    } else {
      Dft<R, SIGN, C>::run(x);
      if constexpr (S > 1) pass_tw<PL, P, SIGN>(x, tw, i);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) p[k * SP] = x[k];
  }
}
// col_pass_planar with a thread's butterflies taken two at a time: both are
// loaded before either is transformed, so the two DFTs and twiddle products
// interleave (the compiler cannot move a later butterfly's shared-memory loads
// above an earlier one's stores, which may alias as far as it can tell).  Same
// arithmetic per butterfly, so the same results bit for bit.
template <typename T, class PL, int NT, int P, int SIGN, bool DIT>
__device__ __forceinline__ void col_pass_planar_dual(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  using C = cplx<T>;
  using CP = ColPlanar<PL>;
  constexpr int R = PL::R[P];
  constexpr int L = PL::span(P);
  constexpr int S = L / R;
  constexpr int SP = CP::pstride(P);
  constexpr int NB = 2 * (PL::M / R);
  static_assert((PL::M / R) % 16 == 0 && NT % 32 == 0, "whole half-warps per plane");
  static_assert(S == 1 || S % CP::RP == 0, "strides other than the last are whole pad groups");
  static_assert(NB % NT == 0, "whole rounds of butterflies");
  constexpr int ROUNDS = NB / NT;
  auto place = [&](int w, int& i) -> C* {
    const int v = (w >> 4) & 1;
    const int b = ((w >> 5) << 4) | (w & 15);
    const int blk = b / S;
    i = b - blk * S;
    return sm + v * CP::PB + CP::phys(blk * L + i);
  };
#pragma unroll
  for (int r = 0; r + 1 < ROUNDS; r += 2) {
    int i1, i2;
    C* p1 = place(tid + r * NT, i1);
    C* p2 = place(tid + (r + 1) * NT, i2);
    C x[R], y[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = p1[k * SP];
#pragma unroll
    for (int k = 0; k < R; ++k) y[k] = p2[k * SP];
    if constexpr (DIT) {
      if constexpr (S > 1) {
        pass_tw<PL, P, SIGN>(x, tw, i1);
        pass_tw<PL, P, SIGN>(y, tw, i2);
      }
      Dft<R, SIGN, C>::run(x);
      Dft<R, SIGN, C>::run(y);
    } else {
      Dft<R, SIGN, C>::run(x);
      Dft<R, SIGN, C>::run(y);
      if constexpr (S > 1) {
        pass_tw<PL, P, SIGN>(x, tw, i1);
        pass_tw<PL, P, SIGN>(y, tw, i2);
      }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) p1[k * SP] = x[k];
#pragma unroll
    for (int k = 0; k < R; ++k) p2[k * SP] = y[k];
  }
  if constexpr (ROUNDS % 2 == 1) {
    int i;
    C* p = place(tid + (ROUNDS - 1) * NT, i);
    C x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = p[k * SP];
    if constexpr (DIT) {
      if constexpr (S > 1) pass_tw<PL, P, SIGN>(x, tw, i);
      Dft<R, SIGN, C>::run(x);
    } else {
      Dft<R, SIGN, C>::run(x);
      if constexpr (S > 1) pass_tw<PL, P, SIGN>(x, tw, i);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) p[k * SP] = x[k];
  }
}

// DIF passes P .. TO-1, DIT passes P down to TO, each followed by a barrier.
template <typename T, class PL, int NT, int SIGN, int P, int TO, bool DUAL = false>
__device__ __forceinline__ void col_dif_planar(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  if constexpr (P < TO) {
    if constexpr (DUAL)
      col_pass_planar_dual<T, PL, NT, P, SIGN, false>(sm, tw, tid);
    else
      col_pass_planar<T, PL, NT, P, SIGN, false>(sm, tw, tid);
    __syncthreads();
    col_dif_planar<T, PL, NT, SIGN, P + 1, TO, DUAL>(sm, tw, tid);
  }
}
template <typename T, class PL, int NT, int SIGN, int P, int TO, bool DUAL = false>
__device__ __forceinline__ void col_dit_planar(cplx<T>* sm, const cplx<T>* __restrict__ tw, int tid) {
  if constexpr (P >= TO) {
    if constexpr (DUAL)
      col_pass_planar_dual<T, PL, NT, P, SIGN, true>(sm, tw, tid);
    else
      col_pass_planar<T, PL, NT, P, SIGN, true>(sm, tw, tid);
    __syncthreads();
    col_dit_planar<T, PL, NT, SIGN, P - 1, TO, DUAL>(sm, tw, tid);
  }
}

// k_col with the column moved by the TMA unit: one elected thread loads both
// P-state planes of column kx (groups of RP complex into ColPlanar's padded
// rows, zero-filled pads) with 3D bulk tensor loads completing on one
// mbarrier, every pass runs in place in shared memory (the first forward DIF
// pass and the last inverse DIT pass included), and the U-state planes leave
// by bulk tensor stores that skip the pads.  om / fnm1 are the butterfly-major
// columns (om_p, fm_p), read and written by the lanes as in k_col.  Same
// arithmetic as k_col, so the same results bit for bit.  FP32.
// MINB > 0 caps the registers so that MINB blocks share an SM.  DUAL: the
// passes around the middle take a thread's butterflies two at a time
// (col_pass_planar_dual).
template <typename T, class PL, int NT, bool QM, int MINB = 0, bool DUAL = false>
__global__ void __launch_bounds__(NT, MINB) k_col_tma(StepArgs a0, const __grid_constant__ TmaMaps maps) {
  using C = cplx<T>;
  using CP = ColPlanar<PL>;
  static_assert(sizeof(C) == 8 && CP::fits, "FP32 planes of whole pad groups and boxes");
  const StepArgs a = member_args(a0, sizeof(C));
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int M = PL::M;
  constexpr int N = 2 * M / 3;
  const int tid = threadIdx.x;
  const int kx = blockIdx.x;
  const int row = (int)blockIdx.y * (N / 2) + kx;  // the plane row of this column in the 3D view
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  C* __restrict__ om = static_cast<C*>(a.om_p) + (size_t)kx * M;
  C* __restrict__ fm = static_cast<C*>(a.fm_p) + (size_t)kx * M;
  __shared__ __align__(8) unsigned long long bar;
  if (tid == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, 2u * CP::G * (2 * CP::RP + 4) * 4u);
#pragma unroll 1
    for (int g = 0; g < CP::G; g += CP::GBOX) {
      tma_load_3d(&maps.w0, sm + g * (CP::RP + 2), &bar, 0, g, row);
      tma_load_3d(&maps.w1, sm + CP::PB + g * (CP::RP + 2), &bar, 0, g, row);
    }
  }
  // every thread forms the coefficients while the bulk copies are in flight
  // (one warp forming them for the block measured 2 % slower here)
  const ModeCoef<T> cf = col_coef<T>(a, N);
  __syncthreads();  // every thread sees the initialised barrier
  if (!mbar_test_wait(&bar, 0, a.dbg_wait0 ? 0 : 1 << 20)) {
    // the copies did not complete in time: report it and wait (bounded) for them
    // before the shared memory is used or released
    if (tid == 0) atomicExch(&a.sc->wait_timeout, 1);
    mbar_test_wait(&bar, 0, 1 << 20);
  }
  col_dif_planar<T, PL, NT, -1, 0, PL::NP - 1, DUAL>(sm, tw, tid);
  col_middle<T, PL, NT, false, true, true, QM, true>(sm, nullptr, nullptr, om, fm, cf, kx, tid, a.flags);
  col_dit_planar<T, PL, NT, +1, PL::NP - 2, 0, DUAL>(sm, tw, tid);
  fence_proxy_async_smem();
  __syncthreads();
  if (tid == 0) {
#pragma unroll 1
    for (int g = 0; g < CP::G; g += CP::GBOX) {
      tma_store_3d(&maps.w0, sm + g * (CP::RP + 2), 0, g, row);
      tma_store_3d(&maps.w1, sm + CP::PB + g * (CP::RP + 2), 0, g, row);
    }
    tma_commit();
    tma_wait_read();  // the shared memory stays the block's until the engine has read it
  }
  col_finish<NT>(a, tid, (int)gridDim.x);
}

// om / fnm1 between the natural [kx][z] columns and the butterfly-major
// columns of the column plan PL (om_p, fm_p; only the N in-band entries of each
// M-element column are written or read).  One block per kx column; the column
// passes through shared memory, so both the natural and the butterfly-major
// side are read and written in consecutive order.
template <typename T, class PL, bool TO_PERM, int NT>
__device__ __forceinline__ void om_perm_body(const StepArgs& a0, const Blk bk) {
  using C = cplx<T>;
  const StepArgs a = member_args(a0, sizeof(C), bk.y);
  constexpr int M = PL::M, N = 2 * M / 3, Nh = M / 3;
  constexpr int RP = PL::RP, FSTEP = PL::FSTEP;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* so = reinterpret_cast<C*>(smraw);
  C* sf = so + N;
  const int kx = bk.x;
  C* __restrict__ no = static_cast<C*>(a.om) + (size_t)kx * N;
  C* __restrict__ nf = static_cast<C*>(a.fnm1) + (size_t)kx * N;
  C* __restrict__ po = static_cast<C*>(a.om_p) + (size_t)kx * M;
  C* __restrict__ pf = static_cast<C*>(a.fm_p) + (size_t)kx * M;
  if constexpr (TO_PERM) {
    for (int z = threadIdx.x; z < N; z += NT) {
      so[z] = no[z];
      sf[z] = nf[z];
    }
    __syncthreads();
  }
  for (int p = threadIdx.x; p < M; p += NT) {
    const int f = PL::freq((p % FSTEP) * RP) + (p / FSTEP) * FSTEP;
    if (f < Nh || f >= N) {
      const int z = f < Nh ? f : f - Nh;
      if constexpr (TO_PERM) {
        po[p] = so[z];
        pf[p] = sf[z];
      } else {
        so[z] = po[p];
        sf[z] = pf[p];
      }
    }
  }
  if constexpr (!TO_PERM) {
    __syncthreads();
    for (int z = threadIdx.x; z < N; z += NT) {
      no[z] = so[z];
      nf[z] = sf[z];
    }
  }
}
template <typename T, class PL, bool TO_PERM>
__global__ void __launch_bounds__(256) k_om_perm(StepArgs a0) {
  om_perm_body<T, PL, TO_PERM, 256>(a0, hw_blk());
}

// k_col_inv: velocity low band -> pad -> inverse z-FFT -> U planes.  The low
// band comes from `src` (reference layout (2, N, N/2), e.g. the generator's
// uc_full) or, when src is null, from the omega -> velocity inversion of om
// (turbo_simulator.py:1555-1585).
template <typename T, class PL, int NT>
__global__ void __launch_bounds__(NT) k_col_inv(StepArgs a0) {
  using C = cplx<T>;
  const StepArgs a = member_args(a0, sizeof(C));
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int M = PL::M;
  constexpr int V = 2;
  const int tid = threadIdx.x;
  const int kx = blockIdx.x;
  const int N = a.N, Nh = N >> 1;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  const C* __restrict__ src = static_cast<const C*>(a.src);
  const C* __restrict__ om = static_cast<const C*>(a.om) + (size_t)kx * N;
  for (int w = tid; w < V * M; w += NT) {
    const int v = w & 1;
    const int pos = w >> 1;
    const int f = PL::freq(pos);
    C val = {T(0), T(0)};
    if (f < Nh || f >= N) {
      const int z = f < Nh ? f : f - Nh;
      if (a.scheme != 0) {
        // scalar band for display (turbo_simulator.py:2639-2709): omega, or the
        // streamfunction omega/(K2 + 1e-30); the kz = -N/2 row is left out
        if (v == 0 && z != Nh) {
          const C o = om[z];
          if (a.scheme == 1) {
            val = o;
          } else {
            const T gz = T(z < Nh ? z : z - N);
            const T ik = T(1) / (T(kx) * T(kx) + gz * gz + T(1.0e-30));
            val = C{o.x * ik, o.y * ik};
          }
        }
      } else if (src != nullptr) {
        val = src[(size_t)v * N * Nh + (size_t)z * Nh + kx];
      } else {
        const C o = om[z];
        const T gz = T(z < Nh ? z : z - N);
        const T ax = T(kx);
        if (kx >= 1) {
          const T ik = T(1) / (ax * ax + gz * gz);
          const C t = {o.x * ik, o.y * ik};
          val = (v == 0) ? C{t.y * gz, -t.x * gz} : C{-t.y * ax, t.x * ax};
        } else if (v == 0 && z >= 1) {
          const T ig = T(1) / gz;
          val = C{o.y * ig, -o.x * ig};
        }
      }
    }
    sm[PL::phys(pos) * V + v] = val;
  }
  __syncthreads();
  dit_range<T, PL, V, NT, +1, PL::NP - 1, 0>(sm, tw, tid);
  C* __restrict__ w0 = static_cast<C*>(a.w0);
  C* __restrict__ w1 = static_cast<C*>(a.w1);
  for (int w = tid; w < V * M; w += NT) {
    const int v = w & 1;
    const int k = w >> 1;
    (v == 0 ? w0 : w1)[(size_t)kx * M + k] = sm[PL::phys(k) * V + v];
  }
}

// --------------------------------------------------------------------------
// Spectral sums over om [kx][z]: E = sum w |om|^2/K2, Lsum = sum w |om|^2/K2^1.5,
// Z = sum w |om|^2 (minus the (0,0) mode), P = sum w K2 |om|^2, with the
// rfft weights w = [1, 2, ..., 2, 1] of turbo_simulator.py:778-781 and
// turbo_main.py:2040-2044.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_spectral(StepArgs a0) {
  using C = cplx<T>;
  const StepArgs a = member_args(a0, sizeof(C));
  const C* __restrict__ om = static_cast<const C*>(a.om);
  const int N = a.N, Nh = N >> 1;
  const long long total = (long long)N * Nh;
  const int tid = threadIdx.x;
  // compensated FP64 sums: E, L numerator, Z (all modes), P, and the (0,0) mode
  double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, c[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  int bad = 0;
  for (long long idx = (long long)blockIdx.x * NT + tid; idx < total; idx += (long long)gridDim.x * NT) {
    const int kx = int(idx / N);
    const int z = int(idx - (long long)kx * N);
    const C o = om[idx];
    const double p = double(o.x) * double(o.x) + double(o.y) * double(o.y);
    if (!isfinite(p)) bad = 1;
    const double gz = double(z < Nh ? z : z - N);
    const double K2 = double(kx) * double(kx) + gz * gz;
    const double wt = (kx == 0 || kx == Nh - 1) ? 1.0 : 2.0;
    if (K2 > 0.0) {
      const double e = wt * p / K2;
      csum_add(s[0], c[0], e);
      csum_add(s[1], c[1], e / sqrt(K2));
    } else {
      csum_add(s[4], c[4], p);  // the (0,0) mode, removed from Z
    }
    csum_add(s[2], c[2], wt * p);
    csum_add(s[3], c[3], wt * K2 * p);
  }
  __shared__ double red[2 * 5 * (NT / 32)];
  block_csum<NT, 5>(s, c, red, tid);
  if (bad) atomicOr(&a.sc->nonfinite, 1);
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < 5; ++q) a.part[5 * blockIdx.x + q] = s[q];
  }
  if (!last_block(&a.sc->diag_counter, tid)) return;
  double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, tc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int q = tid; q < (int)gridDim.x; q += NT) {
#pragma unroll
    for (int r = 0; r < 5; ++r) csum_add(t[r], tc[r], __ldcg(a.part + 5 * q + r));
  }
  block_csum<NT, 5>(t, tc, red, tid);
  if (tid == 0) {
    DevScalars* sc = a.sc;
    sc->E = t[0];
    sc->L = t[1];
    sc->Z = t[2] - t[4];
    sc->P = t[3];
    sc->kmax2 = double(Nh - 1) * double(Nh - 1) + double(Nh) * double(Nh);
    sc->diag_counter = 0u;
  }
}

// Energy spectrum of the compact vorticity band (turbo_simulator.py:2225-2357):
// mode (kx, kz), K2 > 0, goes to bin floor((sqrt(K2)/k_nyq / r_max) nbins)
// (clipped) with p = |om|^2 / K2 * scale2, doubled (and counted twice) for
// kx > 0.  One block per bin: its threads walk the rows kz and only visit the
// kx interval of that bin's annulus (float estimate plus a one-mode margin),
// testing each mode with the reference's double-precision formula, so every
// mode is counted exactly once and the sums are deterministic.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_spectrum(const cplx<T>* __restrict__ om, int N, int nbins, double r_max,
                                                 double k_nyq, double scale2, double* __restrict__ esum,
                                                 int* __restrict__ cnt) {
  const int b = blockIdx.x;
  const int Nh = N >> 1;
  const float c = (float)(k_nyq * r_max / (double)nbins);  // annulus width in k
  const float lo = b * c, hi = (b == nbins - 1) ? 3.0e38f : (b + 1) * c;
  double e = 0.0;
  long long n = 0;
  for (int z = threadIdx.x; z < N; z += NT) {
    const int kz = z < Nh ? z : z - N;
    const float kz2 = (float)kz * (float)kz;
    const float a = lo * lo - kz2;
    int x0 = a > 0.f ? (int)floorf(sqrtf(a)) - 1 : 0;
    const float h = hi * hi - kz2;
    if (h < 0.f) continue;
    int x1 = (hi > 1.0e37f) ? Nh - 1 : (int)ceilf(sqrtf(h)) + 1;
    x0 = max(x0, 0);
    x1 = min(x1, Nh - 1);
    for (int kx = x0; kx <= x1; ++kx) {
      const double k2 = (double)kx * (double)kx + (double)kz * (double)kz;
      if (!(k2 > 0.0)) continue;
      const double r = sqrt(k2) / k_nyq;
      int bin = (int)floor((r / r_max) * (double)nbins);
      bin = bin < 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
      if (bin != b) continue;
      const cplx<T> o = om[(size_t)kx * N + z];
      double p = (((double)o.x * (double)o.x + (double)o.y * (double)o.y) / k2) * scale2;
      const int wgt = kx > 0 ? 2 : 1;
      if (wgt == 2) p *= 2.0;
      e += p;
      n += wgt;
    }
  }
  __shared__ double red[2 * (NT / 32)];
  double v[2] = {e, (double)n};
  block_sum<NT, 2>(v, red, threadIdx.x);
  if (threadIdx.x == 0) {
    esum[b] = v[0];
    cnt[b] = (int)v[1];
  }
}

// Display fields: |u| from the physical planes, then min/max normalisation to
// 8-bit pixels 1..255 (128 for a constant field) as turbo_wrapper.py:317-351.
template <typename T>
__global__ void k_speed(T* __restrict__ ph, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T u = ph[i], v = ph[n + i];
    ph[2 * n + i] = sqrt(u * u + v * v);
  }
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_minmax(const T* __restrict__ f, long long n, double* part, unsigned int* counter,
                                                double* out) {
  double mn = 1e300, mx = -1e300;
  for (long long i = (long long)blockIdx.x * NT + threadIdx.x; i < n; i += (long long)gridDim.x * NT) {
    const double x = (double)f[i];
    mn = fmin(mn, x);
    mx = fmax(mx, x);
  }
  __shared__ double red[NT / 32];
  mx = block_max<NT>(mx, red, threadIdx.x);
  mn = -block_max<NT>(-mn, red, threadIdx.x);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = mn;
    part[2 * blockIdx.x + 1] = mx;
  }
  if (!last_block(counter, threadIdx.x)) return;
  double a = 1e300, b = -1e300;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += NT) {
    a = fmin(a, __ldcg(part + 2 * q));
    b = fmax(b, __ldcg(part + 2 * q + 1));
  }
  b = block_max<NT>(b, red, threadIdx.x);
  a = -block_max<NT>(-a, red, threadIdx.x);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
    *counter = 0u;
  }
}

template <typename T>
__global__ void k_pixels(const T* __restrict__ f, long long n, const double* mm, unsigned char* __restrict__ pix) {
  const double mn = mm[0], rng = mm[1] - mm[0];
  const bool flat = fabs(rng) <= 1.0e-12;
  const T fmn = (T)mn, frng = (T)(flat ? 1.0 : rng);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    T p = T(1) + (f[i] - fmn) / frng * T(254);
    p = p < T(1) ? T(1) : (p > T(255) ? T(255) : p);
    pix[i] = flat ? (unsigned char)128 : (unsigned char)p;
  }
}

// Layout transposes between the reference's (rows, cols) and the device's
// (cols, rows) for complex planes; batch = gridDim.z planes.
template <typename T>
__global__ void k_transpose(const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out, int rows, int cols) {
  __shared__ cplx<T> tile[32][33];
  const size_t plane = (size_t)rows * cols;
  in += plane * blockIdx.z;
  out += plane * blockIdx.z;
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int r = r0 + dy, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[dy][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int c = c0 + dy, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][dy];
  }
}

}  // namespace pal
