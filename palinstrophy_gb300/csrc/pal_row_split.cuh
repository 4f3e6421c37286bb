// Row pass with each row tile split across a cluster of two CTAs.
//
// A row tile of the largest grid (N = 8192, padded lines of M = 12288 points,
// V = 2 lines) is 200 KB of shared memory: one tile per SM, so its loads,
// transforms and stores run one after another.  Split by one radix-2 step
// between the two CTAs of a cluster, each CTA holds a 6144-point half line
// (100 KB) and two halves share an SM, so that one CTA's bulk copies overlap
// the other's transforms, as the N = 4096 tiles do.
//
// The line (Hermitian-packed spectrum Z of the two real rows u, v, as in
// row_first_pass) is transformed as
//   inverse, decimation in frequency:  CTA c forms
//     y_c[k] = (Z[k] + (-1)^c Z[k + M/2]) e^{+2 pi i c k / M},  k < M/2,
//   and its M/2-point inverse transform is x[2n + c], the physical points of
//   parity c;
//   products p = (u^2 - v^2) + i uv of its own points, pointwise;
//   forward, decimation in time:  G_c = M/2-point forward transform of
//     p[2n + c], and P[k] = G_0[k] + w^k G_1[k],
//     P[k + M/2] = G_0[k] - w^k G_1[k]  (w = e^{-2 pi i / M}).
// Only the last step needs both halves: the unpack of output row k < N/2
// reads P[k] and P[M - k] = G_0[M/2 - k] + w^-k G_1[M/2 - k].  CTA 0 writes the
// rows below N/4, CTA 1 the rows N/4 .. N/2, each reading the G values it
// lacks from its peer's shared memory (distributed shared memory), so no
// intermediate line ever goes back to global memory.
//
// Input rows reach the CTAs by TMA bulk tensor loads in eight phases of N/16
// rows over six buffers, in one of three forms (SplitLoad): multicast (each
// row requested once per cluster and delivered to both CTAs), each CTA
// loading every row, or each CTA loading a quarter of the rows and reading the
// other quarter from its peer.  The first DIF pass (radix R = PL::R[0], stride
// S = M / (2R)) accumulates every row's two contributions (Z[k] at position k
// and the mirrored entry conj(u^[k]) + i conj(v^[k]) at position M/2 - k) in
// registers, item by item as in row_first_pass_tma: work item q < S/2 owns
// butterflies q and S - q (0 and S/2 for q = 0).  The plans this supports have
// R divisible by 12, so that N/2 = (2R/3) S and every row k = q + jS (or
// S - q + jS) sits in phase j / (R/12).
//
// Cluster synchronisation is the hardware cluster barrier (barrier.cluster
// arrive / wait), which every thread of both CTAs reaches the same number of
// times on every path; the TMA waits are bounded as in the other row kernels.
// Where a barrier only has to order this CTA's own shared-memory reads, a
// CTA barrier completes them and the cluster arrive is relaxed; where the
// peer must see this CTA's writes, one thread's cluster-scope fence after the
// CTA barrier publishes them (cluster_sync_publish).
#pragma once
#include "pal_kernels.cuh"

namespace pal {

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
// Arrive without release semantics: for the points where the accesses to be
// ordered are this CTA's own shared-memory reads, which the CTA barrier just
// before it has already completed (bar.sync), or mbarrier initialisation,
// which fence.mbarrier_init released.
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
// Cluster barrier after which the peer sees this CTA's shared-memory writes:
// the CTA barrier orders every thread's writes before thread 0's cluster-scope
// fence, so one thread pays the fence instead of all of them.
__device__ __forceinline__ void cluster_sync_publish(int tid) {
  __syncthreads();
  if (tid == 0) asm volatile("fence.acq_rel.cluster;" ::: "memory");
  cluster_arrive_relaxed();
  cluster_wait();
}
// Address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ unsigned peer_smem(const void* p, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float2 ld_peer(unsigned addr) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
  return v;
}

// Bulk tensor load delivered to the same shared-memory offset, and completed
// on the same mbarrier offset, in every CTA of `mask` (this GPU's own memory).
__device__ __forceinline__ void tma_load_3d_mc(const CUtensorMap* map, void* smem, unsigned long long* bar, int x, int y,
                                               int z, unsigned short mask) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
      " [%0], [%1, {%3, %4, %5}], [%2], %6;" ::"r"(d),
      "l"(map), "r"(b), "r"(x), "r"(y), "r"(z), "h"(mask)
      : "memory");
}

// f(std::integral_constant<int, J>) for J = 0 .. n-1, so that the body can use
// J as a template argument (the compile-time twiddles of twc).
template <class F, int... J>
__device__ __forceinline__ void static_for(F&& f, std::integer_sequence<int, J...>) {
  (f(std::integral_constant<int, J>{}), ...);
}

// The same over J = B .. E-1.
template <int B, class F, int... J>
__device__ __forceinline__ void static_for_from(F&& f, std::integer_sequence<int, J...>) {
  (f(std::integral_constant<int, B + J>{}), ...);
}

// Split twiddle e^{-2 pi i (i + jS) / M} of butterfly i, entry j: the loaded
// e^{-2 pi i i / M} times the constant e^{-2 pi i j / (2R)} (S / M = 1 / (2R)).
template <int R2, int J>
__device__ __forceinline__ float2 split_tw(float2 a) {
  return twc<R2, J, -1>(a);
}

// Twiddles of the split: e^{-2 pi i p / M} for p < n (forward convention,
// FP64 angle rounded once).  The kernel keeps one per butterfly of the first
// pass (n = S) and forms the rest with split_tw, so the table stays in L1.
template <typename T>
__global__ void k_split_twiddles(cplx<T>* tw, int n, int mh) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  double sn, cs;
  sincospi((double)p / (double)mh, &sn, &cs);  // 2 p / M = p / (M/2)
  tw[p] = cplx<T>{T(cs), T(-sn)};
}

template <class PL>
struct SplitGeom {
  static constexpr int MH = PL::M;      // half line
  static constexpr int M = 2 * MH;      // padded line
  static constexpr int R = PL::R[0];    // first DIF pass radix
  static constexpr int S = MH / R;      // its stride
  static constexpr int T3 = R / 3;      // S-blocks per N/4 rows
  static constexpr int Nh = M / 3;      // stored rows (N/2)
  static constexpr int NQ = S / 2;      // work items per line
  static constexpr int PHASES = 8;      // input phases of N/16 rows
  static constexpr int NBUF = 6;        // phase buffers in the tile
  static constexpr int JP = 2 * T3 / PHASES;
  static constexpr int ROWS = JP * S;   // rows per input phase
  static constexpr int OUT = T3 * S;    // output rows per CTA (N/4)
  static constexpr int BOX = tma_box_rows(Nh);
  static constexpr int SEND0 = 2 * T3 + 1;  // slots CTA 0 sends (what CTA 1 reads)
  static constexpr int SEND1 = 4 * T3;      // slots CTA 1 sends
  static_assert(R % 12 == 0 && Nh == 2 * T3 * S, "radix of the first pass: a multiple of 12");
  static_assert(ROWS % BOX == 0 && OUT % BOX == 0, "whole TMA boxes per phase");
  static_assert(JP * PHASES == 2 * T3 && 2 * NBUF >= PHASES && NBUF < PHASES, "phases and buffers");
};

// Accumulates the rows of input phase P (j = P JP .. P JP + JP - 1) of work
// item q into its butterflies' inputs x (butterfly q) and y (butterfly i2):
// row k contributes Z[k] at position k and sg times its mirror
// conj(u^[k]) + i conj(v^[k]) at position M/2 - k.  `ld(e)` reads element e of
// the phase's [plane][row][v] staging buffer.
template <class PL, int P, class LD>
__device__ __forceinline__ void split_accumulate(float2 (&x)[SplitGeom<PL>::R], float2 (&y)[SplitGeom<PL>::R], LD&& ld,
                                                 int q, int i2, int v, bool self, float sg) {
  using C = float2;
  using G = SplitGeom<PL>;
  constexpr int R = G::R, S = G::S, ROWS = G::ROWS, JP = G::JP;
  constexpr int V = 2;
#pragma unroll
  for (int jj = 0; jj < JP; ++jj) {
    const int j = P * JP + jj;
    {  // row q + jS: Z at position q + jS, the mirror at M/2 - q - jS
      const int r = q + jj * S;
      const C u = ld(r * V + v), w = ld((ROWS + r) * V + v);
      const C d = (self && j == 0) ? C{u.x, w.x} : C{u.x - w.y, u.y + w.x};
      const C m = C{sg * (u.x + w.y), sg * (w.x - u.y)};
      x[j] = cadd(x[j], d);
      if (self) {
        if (j > 0) x[R - j] = cadd(x[R - j], m);
      } else {
        y[R - 1 - j] = cadd(y[R - 1 - j], m);
      }
    }
    {  // row i2 + jS
      const int r = i2 + jj * S;
      const C u = ld(r * V + v), w = ld((ROWS + r) * V + v);
      const C d = C{u.x - w.y, u.y + w.x};
      const C m = C{sg * (u.x + w.y), sg * (w.x - u.y)};
      y[j] = cadd(y[j], d);
      if (self)
        y[R - 1 - j] = cadd(y[R - 1 - j], m);
      else
        x[R - 1 - j] = cadd(x[R - 1 - j], m);
    }
  }
}

// Bounded wait for a phase's bulk copies; a wait that runs out is reported
// (wait_timeout) and followed by a second bounded wait, so that the buffer is
// not read or reused while copies may still land in it.
__device__ __forceinline__ void split_wait(const StepArgs& a, unsigned long long* bar, unsigned parity, bool first,
                                           int tid) {
  if (!mbar_wait(bar, parity, (first && a.dbg_wait0) ? 0 : 1 << 22)) {
    if (tid == 0) atomicExch(&a.sc->wait_timeout, 1);
    mbar_wait(bar, parity, 1 << 22);
  }
}

// How the input rows reach the two CTAs of a split row tile.
enum SplitLoad {
  SPLIT_LOAD_ALL = 0,   // each CTA TMA-loads every row into its own shared memory
  SPLIT_MULTICAST = 1,  // each CTA fetches one plane by multicast TMA, delivered to both
  SPLIT_HALVES = 2,     // CTA c TMA-loads rows c N/4 .. (c+1) N/4 - 1 and reads the
                        // other half from its peer through distributed shared memory
};

// First pass of the half-line inverse transform of CTA `rank` (see above),
// input rows as LOAD says.
template <class PL, int V, int NT, int LOAD>
__device__ __forceinline__ void split_first_pass(const StepArgs& a, float2* sm, int z0, int tid, const TmaMaps& maps,
                                                 unsigned long long* bars, int member, unsigned rank,
                                                 const float2* __restrict__ sw) {
  using C = float2;
  using G = SplitGeom<PL>;
  constexpr int R = G::R, S = G::S, ROWS = G::ROWS, BOX = G::BOX;
  constexpr int SP = PL::pstride(0);
  static_assert(V == 2 && V * G::NQ == NT, "two lines, one work item per thread");
  constexpr int NBUF = G::NBUF;
  static_assert(size_t(2) * NBUF * ROWS * V <= size_t(PL::PADM) * V, "the phase buffers fit in the tile");
  const int v = tid % V;
  const int q = tid / V;
  const bool self = q == 0;
  const int i2 = self ? S / 2 : S - q;
  const float sg = rank == 0 ? 1.0f : -1.0f;
  C x[R], y[R];
#pragma unroll
  for (int j = 0; j < R; ++j) x[j] = y[j] = C{0.0f, 0.0f};
  if constexpr (LOAD != SPLIT_HALVES) {
    // Phase p's rows of both planes land in buffer p % NBUF ([plane][row][v]).
    // SPLIT_MULTICAST: CTA c fetches plane c's boxes and the TMA unit delivers
    // each to the two CTAs, so every row is requested once per cluster; each
    // CTA's mbarrier counts the bytes of both planes.  SPLIT_LOAD_ALL: each
    // CTA fetches both planes itself.  Phases NBUF.. refill the first buffers
    // once they are consumed: by both CTAs (a cluster barrier) when the peer
    // writes into them too, else by this CTA's threads.
    auto issue = [&](int p) {
      unsigned long long* bar = bars + (p % NBUF);
      C* buf = sm + (size_t)(p % NBUF) * 2 * ROWS * V;
      mbar_expect_tx(bar, 2u * ROWS * V * (unsigned)sizeof(C));
      if constexpr (LOAD == SPLIT_MULTICAST) {
        const CUtensorMap* map = rank == 0 ? &maps.w0 : &maps.w1;
#pragma unroll 1
        for (int bx = 0; bx < ROWS / BOX; ++bx)
          tma_load_3d_mc(map, buf + (size_t)(rank * ROWS + bx * BOX) * V, bar, 2 * z0, p * ROWS + bx * BOX, member,
                         0x3);
      } else {
#pragma unroll 1
        for (int bx = 0; bx < ROWS / BOX; ++bx) {
          tma_load_3d(&maps.w0, buf + (size_t)bx * BOX * V, bar, 2 * z0, p * ROWS + bx * BOX, member);
          tma_load_3d(&maps.w1, buf + (size_t)(ROWS + bx * BOX) * V, bar, 2 * z0, p * ROWS + bx * BOX, member);
        }
      }
    };
    if (tid == 0) {
#pragma unroll 1
      for (int p = 0; p < NBUF; ++p) issue(p);
    }
    static_for(
        [&](auto pc) {
          constexpr int p = decltype(pc)::value;
          split_wait(a, bars + (p % NBUF), (unsigned)(p / NBUF), p == 0, tid);
          const C* stg = sm + (size_t)(p % NBUF) * 2 * ROWS * V;
          split_accumulate<PL, p>(x, y, [&](int e) { return stg[e]; }, q, i2, v, self, sg);
          if (p == G::PHASES - NBUF - 1) {
            // buffers 0 .. p are consumed (by both CTAs, if the peer refills them too)
            __syncthreads();
            if constexpr (LOAD == SPLIT_MULTICAST) {
              cluster_arrive_relaxed();
              cluster_wait();
            }
            if (tid == 0) {
#pragma unroll 1
              for (int pp = NBUF; pp < G::PHASES; ++pp) issue(pp);
            }
          }
        },
        std::make_integer_sequence<int, G::PHASES>{});
  } else {
    constexpr int HALF = G::PHASES / 2;  // phases per CTA: rows rank N/4 ..
    static_assert(HALF <= NBUF, "a CTA's own phases fit in the buffers");
    if (tid == 0) {
#pragma unroll 1
      for (int b = 0; b < HALF; ++b) {
        const int p = (int)rank * HALF + b;
        C* dst = sm + (size_t)b * 2 * ROWS * V;
        mbar_expect_tx(bars + b, 2u * ROWS * V * (unsigned)sizeof(C));
#pragma unroll 1
        for (int bx = 0; bx < ROWS / BOX; ++bx) {
          tma_load_3d(&maps.w0, dst + (size_t)bx * BOX * V, bars + b, 2 * z0, p * ROWS + bx * BOX, member);
          tma_load_3d(&maps.w1, dst + (size_t)(ROWS + bx * BOX) * V, bars + b, 2 * z0, p * ROWS + bx * BOX, member);
        }
      }
    }
    auto own = [&](auto pc) {
      constexpr int p = decltype(pc)::value;
      split_wait(a, bars + p % HALF, 0u, p % HALF == 0, tid);
      const C* stg = sm + (size_t)(p % HALF) * 2 * ROWS * V;
      split_accumulate<PL, p>(x, y, [&](int e) { return stg[e]; }, q, i2, v, self, sg);
    };
    auto peer = [&](auto pc) {
      constexpr int p = decltype(pc)::value;
      const unsigned base = peer_smem(sm + (size_t)(p % HALF) * 2 * ROWS * V, rank ^ 1u);
      split_accumulate<PL, p>(x, y, [&](int e) { return ld_peer(base + (unsigned)e * 8u); }, q, i2, v, self, sg);
    };
    // own rows, then (once both CTAs' rows have landed and are published) the peer's
    if (rank == 0) {
      static_for(own, std::make_integer_sequence<int, HALF>{});
      cluster_sync_publish(tid);
      static_for_from<HALF>(peer, std::make_integer_sequence<int, HALF>{});
    } else {
      static_for_from<HALF>(own, std::make_integer_sequence<int, HALF>{});
      cluster_sync_publish(tid);
      static_for(peer, std::make_integer_sequence<int, HALF>{});
    }
    // the peer has read this CTA's rows before the tile is overwritten
    __syncthreads();
    cluster_arrive_relaxed();
    cluster_wait();
  }
  __syncthreads();  // the tile is free for the DFT outputs
  if (rank == 1) {  // the odd half: y_1[k] = (Z[k] - Z[k + M/2]) e^{+2 pi i k / M}
    const C aq = __ldg(sw + q), ai = __ldg(sw + i2);
    static_for(
        [&](auto jc) {
          constexpr int j = decltype(jc)::value;
          x[j] = twmul<+1>(x[j], split_tw<2 * R, j>(aq));
          y[j] = twmul<+1>(y[j], split_tw<2 * R, j>(ai));
        },
        std::make_integer_sequence<int, R>{});
  }
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
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
  __syncthreads();
}

// Unpack of output row k from P[k] (p) and P[M - k] (c), as row_last_pass_tma.
__device__ __forceinline__ void split_unpack(float2 p, float2 c, float2& A, float2& B) {
  A = float2{0.5f * (p.x + c.x), 0.5f * (p.y - c.y)};
  B = float2{0.5f * (p.y + c.y), -0.5f * (p.x - c.x)};
}
// P[k] and P[M - k] from own / peer G values: g0 = G_0[k], g1 = G_1[k],
// h0 = G_0[M/2 - k], h1 = G_1[M/2 - k], w = e^{-2 pi i k / M}.
__device__ __forceinline__ void split_combine(float2 g0, float2 g1, float2 h0, float2 h1, float2 w, float2& A,
                                              float2& B) {
  const float2 p = cadd(g0, cmul(g1, w));
  const float2 c = cadd(h0, cmulc(h1, w));
  split_unpack(p, c, A, B);
}

// Last forward pass, the exchange and the unpack of this CTA's output rows;
// stores them by TMA.  Returns after the store's shared-memory reads.
template <class PL, int V, int NT>
__device__ __forceinline__ void split_last_pass(const StepArgs& a, float2* sm, int z0, int tid, const TmaMaps& maps,
                                                int member, unsigned rank, const float2* __restrict__ sw) {
  using C = float2;
  using G = SplitGeom<PL>;
  constexpr int R = G::R, S = G::S, T3 = G::T3, OUT = G::OUT, BOX = G::BOX;
  constexpr int SP = PL::pstride(0);
  static_assert(size_t(2) * OUT * V + size_t(G::SEND0) * NT <= size_t(PL::PADM) * V,
                "CTA 0's send slots fit beside its output staging");
  static_assert(size_t(G::SEND1) * NT <= size_t(PL::PADM) * V, "CTA 1's send slots fit in the tile");
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  const int v = tid % V;
  const int q = tid / V;
  const bool self = q == 0;
  const int i2 = self ? S / 2 : S - q;
  C y1[R], y2[R];  // G_rank[q + jS], G_rank[i2 + jS]
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
  __syncthreads();  // every read of the tile is done
  C* stg = sm;      // output staging [plane][row - rank N/4][v]
  // send slots [slot][tid]: CTA 0's beside its staging; CTA 1's at the top of
  // the tile, above its A-plane staging but over part of its B-plane staging
  constexpr size_t SND1 = size_t(PL::PADM) * V - size_t(G::SEND1) * NT;
  static_assert(SND1 >= size_t(OUT) * V, "CTA 1's send slots lie above its A-plane staging");
  C* snd = rank == 0 ? sm + (size_t)2 * OUT * V : sm + SND1;
  if (rank == 0) {  // what CTA 1 reads: y1[T3 .. 2T3], y2[T3 .. 2T3)
#pragma unroll
    for (int s = 0; s < T3; ++s) {
      snd[(size_t)s * NT + tid] = y1[T3 + s];
      snd[(size_t)(T3 + s) * NT + tid] = y2[T3 + s];
    }
    snd[(size_t)(2 * T3) * NT + tid] = y1[2 * T3];
  } else {  // what CTA 0 reads: y1 and y2 at [0, T3) and [2 T3, 3 T3)
#pragma unroll
    for (int s = 0; s < T3; ++s) {
      snd[(size_t)s * NT + tid] = y1[s];
      snd[(size_t)(T3 + s) * NT + tid] = y1[2 * T3 + s];
      snd[(size_t)(2 * T3 + s) * NT + tid] = y2[s];
      snd[(size_t)(3 * T3 + s) * NT + tid] = y2[2 * T3 + s];
    }
  }
  cluster_sync_publish(tid);  // (1) the send slots are written
  const unsigned peer = peer_smem(rank == 0 ? sm + SND1 : sm + (size_t)2 * OUT * V, rank ^ 1u) + (unsigned)tid * 8u;
  // bulk tensor stores of one plane of this CTA's output rows
  auto store_plane = [&](int plane) {
#pragma unroll 1
    for (int bx = 0; bx < OUT / BOX; ++bx)
      tma_store_3d(plane == 0 ? &maps.w0 : &maps.w1, stg + (size_t)(plane * OUT + bx * BOX) * V, 2 * z0,
                   (int)rank * OUT + bx * BOX, member);
  };
  auto slot = [&](int s) { return ld_peer(peer + (unsigned)s * NT * 8u); };
  const C aq = __ldg(sw + q), ai = __ldg(sw + i2);
  if (rank == 0) {
    // rows q + jS and i2 + jS, j < T3: own G_0, peer G_1
    static_for([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      constexpr int e = (R - j) % R;  // butterfly 0 is its own partner
      const int k1 = q + j * S, k2 = i2 + j * S;
      // the four peer values of this j, loaded back to back: G_1 at k1, at
      // M/2 - k1, at k2 and at M/2 - k2 (slot map of the send loop above)
      const C g1 = slot(j);
      const C h1 = slot(self ? (e == 0 ? j : e - T3) : R - 1 - j + T3);
      const C g1b = slot(2 * T3 + j);
      const C h1b = slot(self ? R - 1 - j + T3 : R - 1 - j - T3);
      C A, B;
      split_combine(y1[j], g1, self ? y1[e] : y2[R - 1 - j], h1, split_tw<2 * R, j>(aq), A, B);
      stg[(size_t)k1 * V + v] = A;
      stg[(size_t)(OUT + k1) * V + v] = B;
      split_combine(y2[j], g1b, self ? y2[R - 1 - j] : y1[R - 1 - j], h1b, split_tw<2 * R, j>(ai), A, B);
      stg[(size_t)k2 * V + v] = A;
      stg[(size_t)(OUT + k2) * V + v] = B;
    }, std::make_integer_sequence<int, T3>{});
    __syncthreads();           // every read of the peer's slots has returned
    cluster_arrive_relaxed();  // (2) done with the peer's slots
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      store_plane(0);
      store_plane(1);
      tma_commit();
      tma_wait_read();
    }
    cluster_wait();  // keep the send slots until CTA 1 has read them
  } else {
    // rows q + jS and i2 + jS, T3 <= j < 2T3: peer G_0, own G_1
    C A1[T3], B1[T3], A2[T3], B2[T3];
    static_for([&](auto tc) {
      constexpr int t = decltype(tc)::value;
      constexpr int j = T3 + t;
      constexpr int e = R - j;  // butterfly 0's partner entry, in (T3, 2T3]
      // peer G_0 at k1, at M/2 - k1, at k2 and at M/2 - k2
      const C g0 = slot(t);
      const C h0 = slot(self ? (e == 2 * T3 ? 2 * T3 : e - T3) : R - 1 - j);
      const C g0b = slot(T3 + t);
      const C h0b = slot(self ? R - 1 - j : R - 1 - j - T3);
      split_combine(g0, y1[j], h0, self ? y1[e] : y2[R - 1 - j], split_tw<2 * R, j>(aq), A1[t], B1[t]);
      split_combine(g0b, y2[j], h0b, self ? y2[R - 1 - j] : y1[R - 1 - j], split_tw<2 * R, j>(ai), A2[t], B2[t]);
    }, std::make_integer_sequence<int, T3>{});
    // the A plane's staging lies below the send slots: write and store it now
#pragma unroll
    for (int t = 0; t < T3; ++t) {
      stg[(size_t)(q + t * S) * V + v] = A1[t];  // rows k - N/4
      stg[(size_t)(i2 + t * S) * V + v] = A2[t];
    }
    fence_proxy_async_smem();
    __syncthreads();  // ... and every read of the peer's slots has returned
    if (tid == 0) {
      store_plane(0);
      tma_commit();
    }
    cluster_arrive_relaxed();  // (2) done with the peer's slots
    cluster_wait();            // ... and the peer with ours: the B-plane staging is free
#pragma unroll
    for (int t = 0; t < T3; ++t) {
      stg[(size_t)(OUT + q + t * S) * V + v] = B1[t];
      stg[(size_t)(OUT + i2 + t * S) * V + v] = B2[t];
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      store_plane(1);
      tma_commit();
      tma_wait_read();  // both planes' stores have read the tile
    }
  }
}

// k_row_split: the row pass of one tile (V lines of M = 2 PL::M points) by a
// cluster of two CTAs.  Grid (2 M / V, members); blocks 2t and 2t + 1 are the
// two halves of tile t.  The twiddle table holds the half-line plan's tables,
// then the S split twiddles e^{-2 pi i p / M}, p < S.  LOAD: how the input
// rows arrive (SplitLoad).
template <class PL, int V, int NT, int LOAD>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(NT, 2)
    k_row_split(StepArgs a0, const __grid_constant__ TmaMaps maps) {
  using C = float2;
  const Blk bk = hw_blk();
  const StepArgs a = member_args(a0, sizeof(C), bk.y);
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  __shared__ __align__(8) unsigned long long bars[SplitGeom<PL>::NBUF];
  const int tid = threadIdx.x;
  const unsigned rank = cluster_rank();
  const int z0 = (bk.x >> 1) * V;
  const C* __restrict__ tw = static_cast<const C*>(a.tw);
  const C* __restrict__ sw = tw + PL::TW_TOTAL;
  if (tid == 0) {
#pragma unroll
    for (int b = 0; b < SplitGeom<PL>::NBUF; ++b) mbar_init(&bars[b], 1);
  }
  if constexpr (LOAD == SPLIT_MULTICAST) {
    // both CTAs' mbarriers are initialised before either multicasts into the other
    cluster_arrive_relaxed();
    cluster_wait();
  } else {
    __syncthreads();
  }
  split_first_pass<PL, V, NT, LOAD>(a, sm, z0, tid, maps, bars, bk.y, rank, sw);
  dif_range<float, PL, V, NT, +1, 1, PL::NP - 1>(sm, tw, tid);
  const bool stats = (a.flags & F_STATS) != 0;
  float mx = 0.0f, acc = 0.0f;
  row_products<float, PL, V, NT>(sm, tid, stats, mx, acc);
  dit_range<float, PL, V, NT, -1, PL::NP - 2, 1>(sm, tw, tid);
  split_last_pass<PL, V, NT>(a, sm, z0, tid, maps, bk.y, rank, sw);
  // each CTA's statistics cover its half of the points; the partials of all
  // 2 M / V blocks make the whole field
  if (stats) finish_stats<NT, false>(a, double(mx), double(acc), 0.0, 2 * PL::M, tid, bk);
}

// Row candidate on the split kernel: PL is the half-line plan, PF the
// full-line plan of k_phys (which needs physical rows in natural order).
// Twiddle table: [PL tables | S split twiddles | PF tables].
template <class PL, class PF, int V, int NT, int NTP, int LOAD>
struct RowSplitOf {
  static constexpr int M = 2 * PL::M;
  static_assert(PF::M == M, "the phys plan covers the whole line");
  static constexpr size_t smem = size_t(PL::PADM) * V * sizeof(float2);
  static constexpr size_t smem_phys = size_t(PF::PADM) * V * sizeof(float2);
  static constexpr int TW_SPLIT = PL::TW_TOTAL;
  static constexpr int TW_PHYS = PL::TW_TOTAL + SplitGeom<PL>::S;
  static constexpr int TW_ALL = TW_PHYS + PF::TW_TOTAL;
  static_assert(smem <= kSmemLimit && smem_phys <= kSmemLimit, "tiles fit in shared memory");
  static cudaError_t configure() {
    cudaError_t e = cudaFuncSetAttribute(k_row_split<PL, V, NT, LOAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_row_split<PL, V, NT, LOAD>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_phys<float, PF, V, NTP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_phys);
  }
  static void row(const StepArgs& a, cudaStream_t s) {
    static const TmaMaps none{};
    k_row_split<PL, V, NT, LOAD><<<dim3(2 * M / V, a.members > 1 ? a.members : 1), NT, smem, s>>>(
        a, a.tmaps ? *a.tmaps : none);
  }
  static void phys(const StepArgs& a, cudaStream_t s) {
    StepArgs b = a;
    b.tw = static_cast<const float2*>(a.tw) + TW_PHYS;
    k_phys<float, PF, V, NTP><<<dim3(M / V, a.members > 1 ? a.members : 1), NTP, smem_phys, s>>>(b);
  }
  static void twiddles(void* tw, cudaStream_t s) {
    float2* t = static_cast<float2*>(tw);
    launch_twiddles<float, PL>(t, s);
    k_split_twiddles<float><<<(SplitGeom<PL>::S + 255) / 256, 256, 0, s>>>(t + TW_SPLIT, SplitGeom<PL>::S, PL::M);
    launch_twiddles<float, PF>(t + TW_PHYS, s);
  }
  static int blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_row_split<PL, V, NT, LOAD>, NT, smem) == cudaSuccess) return n;
    (void)cudaGetLastError();  // a refused query must not read as a failed launch later
    return -1;
  }
  static constexpr RowKernels make(const char* name) {
    return RowKernels{name, V, NT, true, smem, TW_ALL, configure, row, phys, twiddles, blocks_per_sm,
                      LOAD == SPLIT_MULTICAST};
  }
};

}  // namespace pal
