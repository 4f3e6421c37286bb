// One kernel launch per pass for an ensemble whose members have several grid
// sizes.  The per-size launches of pal_ensemble.cu run one kernel per size
// group per pass; here one launch covers every group: its blocks are laid out
// group by group and member by member, and each block decodes its (group,
// member, tile or column) from the launch's group table and runs that size's
// kernel body (row_body, col_body, om_perm_body, phys_body of pal_kernels.cuh)
// with that position.  A CNAB2 step of the whole ensemble is then 2 launches
// and an LS-IMEX-RK3 step 6, whatever the number of sizes.
//
// All bodies of one launch share its block size, so each compiled set fixes
// one candidate per size (the twiddle tables depend on the plan alone, so a
// body may run at another block size than the candidate it borrows them from);
// the ensemble builds those candidates' tables and TMA descriptors as for a
// per-size launch.  Blocks of one group come out in order, so the groups run
// mostly one after another and each group's working set stays in L2 as in the
// per-size launches.
#include <cuda_runtime.h>

#include <algorithm>

#include "pal_launch.cuh"

using namespace pal;

namespace {

// One size of a fused set: its row tile (TMA loads and stores, paired first
// pass) and its butterfly-major column pass (lane om / fnm1 loads hoisted).
template <class PLR, int VR, int PFR, class PLC, int PREFC>
struct FusedSize {
  static constexpr int V = VR;
  template <int NT>
  static __device__ __forceinline__ void row(const StepArgs& a, const TmaMaps& m, Blk bk) {
    row_body<float, PLR, VR, NT, PFR, true>(a, m, bk);
  }
  // QM: the flag-aware update of the RK3 stages that carry the combined term,
  // else the plain update (a separate launch, so CNAB2 passes keep the plain
  // body's register budget), as ColOf::col_perm chooses
  template <int NT, bool QM>
  static __device__ __forceinline__ void col(const StepArgs& a, Blk bk) {
    col_body<float, PLC, NT, PREFC, true, QM, true>(a, bk);
  }
  template <int NT>
  static __device__ __forceinline__ void phys(const StepArgs& a, Blk bk) {
    phys_body<float, PLR, VR, NT>(a, bk);
  }
  template <int NT, bool TO>
  static __device__ __forceinline__ void perm(const StepArgs& a, Blk bk) {
    om_perm_body<float, PLC, TO, NT>(a, bk);
  }
  static constexpr size_t smem_row = size_t(PLR::PADM) * VR * sizeof(float2);
  static constexpr size_t smem_col = size_t(PLC::PADM) * 2 * sizeof(float2);
  static constexpr size_t smem_perm = size_t(2) * (2 * PLC::M / 3) * sizeof(float2);
};

// The group of block b and the block's position in it.
__device__ __forceinline__ int fused_place(const FusedArgs& f, Blk& bk) {
  const int b = blockIdx.x;
  int g = 0;
  while (g + 1 < f.ngroups && b >= f.g[g + 1].first) ++g;
  const int local = b - f.g[g].first;
  bk = Blk{local % f.g[g].per_member, local / f.g[g].per_member, f.g[g].per_member};
  return g;
}

enum Pass { P_ROW, P_COL, P_COL_QM, P_PHYS, P_TO, P_FROM };

template <int PASS, int NT, int I, class S0, class... Ss>
__device__ __forceinline__ void fused_run(int slot, const FusedArgs& f, int g, Blk bk) {
  if (slot == I) {
    if constexpr (PASS == P_ROW) S0::template row<NT>(f.g[g].a, f.maps[g], bk);
    if constexpr (PASS == P_COL) S0::template col<NT, false>(f.g[g].a, bk);
    if constexpr (PASS == P_COL_QM) S0::template col<NT, true>(f.g[g].a, bk);
    if constexpr (PASS == P_PHYS) S0::template phys<NT>(f.g[g].a, bk);
    if constexpr (PASS == P_TO) S0::template perm<NT, true>(f.g[g].a, bk);
    if constexpr (PASS == P_FROM) S0::template perm<NT, false>(f.g[g].a, bk);
    return;
  }
  if constexpr (sizeof...(Ss) > 0) fused_run<PASS, NT, I + 1, Ss...>(slot, f, g, bk);
}

template <int PASS, int NT, class... Ss>
__global__ void __launch_bounds__(NT) k_ens_fused(const __grid_constant__ FusedArgs f) {
  Blk bk;
  const int g = fused_place(f, bk);
  fused_run<PASS, NT, 0, Ss...>(f.g[g].slot, f, g, bk);
}

template <int NT, int NTC, class... Ss>
struct FusedOf {
  static constexpr size_t smem_row = std::max({Ss::smem_row...});
  static constexpr size_t smem_col = std::max({Ss::smem_col...});
  static constexpr size_t smem_perm = std::max({Ss::smem_perm...});
  static_assert(smem_row <= kSmemLimit && smem_col <= kSmemLimit, "fused tiles fit in shared memory");
  // row and statistics passes run NT threads per block, the column and layout
  // passes NTC
  template <int PASS>
  static constexpr int threads() {
    return (PASS == P_ROW || PASS == P_PHYS) ? NT : NTC;
  }
  template <int PASS>
  static void launch(const FusedArgs& f, int blocks, size_t smem, cudaStream_t s) {
    k_ens_fused<PASS, threads<PASS>(), Ss...><<<blocks, threads<PASS>(), smem, s>>>(f);
  }
  static void row(const FusedArgs& f, int blocks, cudaStream_t s) { launch<P_ROW>(f, blocks, smem_row, s); }
  static void col(const FusedArgs& f, int blocks, bool qm, cudaStream_t s) {
    if (qm)
      launch<P_COL_QM>(f, blocks, smem_col, s);
    else
      launch<P_COL>(f, blocks, smem_col, s);
  }
  static void phys(const FusedArgs& f, int blocks, cudaStream_t s) { launch<P_PHYS>(f, blocks, smem_row, s); }
  static void to_perm(const FusedArgs& f, int blocks, cudaStream_t s) { launch<P_TO>(f, blocks, smem_perm, s); }
  static void from_perm(const FusedArgs& f, int blocks, cudaStream_t s) { launch<P_FROM>(f, blocks, smem_perm, s); }
  static cudaError_t configure() {
    const struct {
      const void* k;
      size_t smem;
    } ks[] = {{(const void*)k_ens_fused<P_ROW, NT, Ss...>, smem_row},
              {(const void*)k_ens_fused<P_COL, NTC, Ss...>, smem_col},
              {(const void*)k_ens_fused<P_COL_QM, NTC, Ss...>, smem_col},
              {(const void*)k_ens_fused<P_PHYS, NT, Ss...>, smem_row},
              {(const void*)k_ens_fused<P_TO, NTC, Ss...>, smem_perm},
              {(const void*)k_ens_fused<P_FROM, NTC, Ss...>, smem_perm}};
    for (const auto& k : ks) {
      cudaError_t e = cudaFuncSetAttribute(k.k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
};

// The 96-member configuration's sizes: N = 256, 384, 512 (M = 384, 576, 768).
// One block size for all bodies means one register budget (the largest body's):
// the light plans are chosen (the 6.6.16 row plan at N=384 needs ~60 registers
// where the 24.24 plan needs 128).
using P384 = Plan<384, 16, 24>;
using P576 = Plan<576, 24, 24>;
using P576b = Plan<576, 6, 6, 16>;
using P768 = Plan<768, 32, 24>;
using P768b = Plan<768, 16, 2, 24>;
using S256 = FusedSize<Rec<P384>, 4, 14, Rec<P384>, 2>;
using S384 = FusedSize<Rec<P576b>, 2, 14, Rec<P576>, 2>;
using S512 = FusedSize<Rec<P768b>, 4, 14, Rec<P768>, 2>;
// Row tiles of 128 threads, column passes of 64: measured 2620 ensemble steps/s
// for the 96-member configuration, against 2557 with the plain radix-16.24
// column at N=256, 2153 with 128-thread column blocks, and 2505 for per-size
// launches of candidates re-tuned on each group's batched shape.
using F3 = FusedOf<128, 64, S256, S384, S512>;

const FusedSet kSet3 = {3,
                        {256, 384, 512},
                        {"16.24r V4x128 tma-in tma-out", "6.6.16r V2x128 tma-in tma-out",
                         "16.2.24r V4x128 tma-in tma-out"},
                        {"16.24r x128 hoist", "24.24r x128 hoist", "32.24r x128 hoist"},
                        {4, 2, 4},
                        128,
                        F3::smem_row,
                        F3::smem_col,
                        F3::smem_perm,
                        F3::configure,
                        F3::row,
                        F3::col,
                        F3::phys,
                        F3::to_perm,
                        F3::from_perm};

}  // namespace

const pal::FusedSet* pal_fused_set_f32(int n, const int* Ns) {
  if (n <= 0 || n > kFusedMax) return nullptr;
  for (int i = 0; i < n; ++i)
    if (std::find(kSet3.N, kSet3.N + kSet3.nsizes, Ns[i]) == kSet3.N + kSet3.nsizes) return nullptr;
  return &kSet3;
}
