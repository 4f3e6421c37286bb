// Launch wrappers and the autotuning candidates.
//
// For each (precision, N) the library compiles several row-pass and column-pass
// candidates that differ in radix order (the Plan), rows per tile (V, row pass
// only) and threads per block.  The two passes only share the data layout of
// the work planes, so they are chosen independently; each carries its own
// twiddle tables.  pal_create times every candidate on the handle's own state
// and keeps the fastest (pal_autotune in pal_api.cu).
#pragma once
#include <cstdlib>

#include "pal_adjoint.cuh"
#include "pal_kernels.cuh"

namespace pal {

struct RowKernels {
  const char* name;
  int V, NT;
  bool tma;  // stores through TMA: the launch needs StepArgs::tmaps
  size_t smem;
  int tw_elems;
  cudaError_t (*configure)();
  void (*row)(const StepArgs&, cudaStream_t);
  void (*phys)(const StepArgs&, cudaStream_t);
  void (*twiddles)(void* tw, cudaStream_t);
  int (*blocks_per_sm)();  // resident k_row blocks per SM (occupancy calculator)
  bool multicast = false;  // loads by TMA cluster multicast (left out of tuning by PAL_TMA_MULTICAST=0)
};

struct ColKernels {
  const char* name;
  int NT;
  size_t smem;
  int tw_elems;
  cudaError_t (*configure)();
  void (*col)(const StepArgs&, cudaStream_t);
  void (*col_inv)(const StepArgs&, cudaStream_t);
  void (*twiddles)(void* tw, cudaStream_t);
  // the same pass on butterfly-major om / fnm1 (a.om_p, a.fm_p), and the
  // conversions between that order and the natural columns
  void (*col_perm)(const StepArgs&, cudaStream_t);
  void (*to_perm)(const StepArgs&, cudaStream_t);
  void (*from_perm)(const StepArgs&, cudaStream_t);
  int (*blocks_per_sm)();  // resident k_col blocks per SM (occupancy calculator)
  bool tma;                // the butterfly-major pass moves its planes by TMA: the launch needs StepArgs::cmaps
  int rp;                  // last radix of the plan (pad groups of the TMA column tile)
};

// Adjoint of one LS-IMEX-RK3 stage (pal_adjoint.cuh), on fixed plans.
struct AdjKernels {
  int tw_row_elems, tw_col_elems;
  cudaError_t (*configure)();
  void (*col_in)(const StepArgs&, cudaStream_t);
  void (*row)(const StepArgs&, cudaStream_t);
  void (*col_out)(const StepArgs&, cudaStream_t);
  void (*col_vel)(const StepArgs&, cudaStream_t);  // the stage's velocity planes from om_in
  void (*tw_row)(void* tw, cudaStream_t);
  void (*tw_col)(void* tw, cudaStream_t);
  void (*seed)(const void* om, void* lom, void* lf, int N, double* loss_part, int blocks, cudaStream_t);
};

struct KernelSet {
  int N, M, precision;
  const RowKernels* rows;
  int n_rows;
  const ColKernels* cols;
  int n_cols;
  void (*spectral)(const StepArgs&, cudaStream_t, int blocks);
  void (*transpose)(const void* in, void* out, int rows, int cols, int batch, cudaStream_t);
  void (*spectrum)(const void* om, int N, int nbins, double r_max, double k_nyq, double scale2, double* esum, int* cnt,
                   cudaStream_t);
  // display: |u| into plane 2 of `phys`, and min/max -> 8-bit pixels of one plane
  void (*speed)(void* phys, long long plane, cudaStream_t);
  void (*pixels)(const void* plane, long long n, double* part, unsigned int* counter, double* mm, unsigned char* pix,
                 cudaStream_t);
  const AdjKernels* adj;  // nullptr where no adjoint is compiled
};

// Whether the autotuners may pick row candidates that load by TMA cluster
// multicast: yes unless PAL_TMA_MULTICAST=0.
inline bool tma_multicast_allowed() {
  const char* e = std::getenv("PAL_TMA_MULTICAST");
  return !(e && e[0] == '0');
}

constexpr int kSpectralThreads = 256;
constexpr size_t kSmemLimit = 227 * 1024;
constexpr size_t kLargeTile = 64 * 1024;  // tiles from this size on ask for the max shared carveout
// Bytes allocated after each work plane: the column pass's bulk tensor boxes
// reach 16 bytes past the last group of a row (ColPlanar), and this keeps
// every such byte inside the allocation.
constexpr size_t kPlaneSlack = 256;

// TMA descriptors of the planes w0 / w1 (members x N/2 rows x M complex FP32)
// for a row candidate with tile height V; false if the driver call is missing
// or refuses the layout.
bool encode_row_maps(TmaMaps* out, void* w0, void* w1, int N, int V, int members);
// Descriptors of w0 / w1 for k_col_tma: each a 3D view (2 RP floats, M / RP
// groups, N/2 x members rows) with a (2 RP + 4 floats, min(256, M / RP), 1)
// box, so one box row is a padded group of ColPlanar.
bool encode_col_maps(TmaMaps* out, void* w0, void* w1, int N, int RP, int members);

template <typename T, class PL>
void launch_twiddles(void* tw, cudaStream_t s) {
  k_twiddles<T, PL><<<(PL::TW_TOTAL + 255) / 256, 256, 0, s>>>(static_cast<cplx<T>*>(tw));
}

// Blocks of one kernel resident on the whole device at once (one wave).
template <class K>
inline int wave_blocks(K kernel, int nt, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nt, smem) != cudaSuccess) return 0;
  return sms * per_sm;
}

// Column-pass flags of LS-IMEX-RK3 stage s (0..2) on butterfly-major om /
// fnm1: the first stage reads no fnm1, the first two hand the next stage its
// combined q in om (k_col F_Q_OUT / F_Q_IN), the last stores om and fn.
// `beta` is the stage table of beta coefficients.
__host__ __device__ inline void rk3_stage_flags(StepArgs& a, int s, const double* beta) {
  a.flags |= (s == 0 ? F_NO_FM_IN : F_Q_IN) | (s < 2 ? F_Q_OUT : 0);
  a.beta_next = s < 2 ? beta[s + 1] : 0.0;
}

template <typename T, class PL, int V, int NT, int PF = 0>
struct RowOf {
  static constexpr size_t smem = size_t(PL::PADM) * V * sizeof(cplx<T>);
  static_assert(smem <= kSmemLimit, "row tile does not fit in shared memory");
  static_assert(PL::M % V == 0, "row tile must divide M");
  static inline int ahead = 0;
  static cudaError_t configure() {
    cudaError_t e =
        cudaFuncSetAttribute(k_row<T, PL, V, NT, PF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // tiles of 64 KB and more ask for the largest shared-memory carveout, so that
    // two of them are resident per SM whatever ran before; smaller tiles leave
    // the split to the driver (their L1 holds the twiddle tables and planes)
    if (smem >= kLargeTile) {
      e = cudaFuncSetAttribute(k_row<T, PL, V, NT, PF>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
    }
    if (PF & 1) ahead = ((PF & 32) ? 2 : 1) * wave_blocks(k_row<T, PL, V, NT, PF>, NT, smem);
    return cudaFuncSetAttribute(k_phys<T, PL, V, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  static void row(const StepArgs& a, cudaStream_t s) {
    StepArgs b = a;
    b.ahead = ahead;
    static const TmaMaps none{};
    k_row<T, PL, V, NT, PF><<<dim3(PL::M / V, a.members > 1 ? a.members : 1), NT, smem, s>>>(
        b, ((PF & 12) != 0 && a.tmaps) ? *a.tmaps : none);
  }
  static void phys(const StepArgs& a, cudaStream_t s) {
    k_phys<T, PL, V, NT><<<dim3(PL::M / V, a.members > 1 ? a.members : 1), NT, smem, s>>>(a);
  }
  static int blocks_per_sm() {
    int n = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_row<T, PL, V, NT, PF>, NT, smem) == cudaSuccess ? n : -1;
  }
  static constexpr RowKernels make(const char* name) {
    return RowKernels{name, V,   NT, (PF & 12) != 0, smem, PL::TW_TOTAL, configure, row, phys, launch_twiddles<T, PL>,
                      blocks_per_sm};
  }
};

template <typename T, class PL, int NT, int PREF = 0>
struct ColOf {
  // PREF 4: the butterfly-major pass is k_col_tma (planar tile, TMA bulk
  // copies of the planes); the natural-order pass is the plain k_col.
  // PREF 5 / 6: the same with registers capped for three / two blocks per SM.
  // PREF 8: PREF 4 with the passes around the middle taking two butterflies
  // per thread at a time.
  static constexpr bool TMA = PREF == 4 || PREF == 5 || PREF == 6 || PREF == 8;
  static constexpr bool DUAL = PREF == 8;
  static constexpr int BASE = TMA ? 0 : PREF;
  static constexpr size_t smem_inv = size_t(PL::PADM) * 2 * sizeof(cplx<T>);
  static constexpr size_t smem = smem_inv + (BASE == 1 ? size_t(2) * (2 * PL::M / 3) * sizeof(cplx<T>) : 0);
  // the butterfly-major variant has no shared-memory om staging (PREF 1)
  static constexpr int PERM_PREF = BASE == 1 ? 0 : BASE;
  static constexpr size_t smem_tma = TMA ? size_t(2) * ColPlanar<PL>::PB * sizeof(cplx<T>) : 0;
  static constexpr int MINB = PREF == 5 ? 3 : PREF == 6 ? 2 : 0;
  static_assert(MINB * (smem_tma + 1024 + 256) <= size_t(228 * 1024), "the capped block count fits in shared memory");
  static_assert(smem <= kSmemLimit && smem_tma <= kSmemLimit, "column tile does not fit in shared memory");
  static cudaError_t configure() {
    cudaError_t e =
        cudaFuncSetAttribute(k_col<T, PL, NT, BASE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if constexpr (TMA) {
      e = cudaFuncSetAttribute(k_col_tma<T, PL, NT, true, MINB, DUAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_tma);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(k_col_tma<T, PL, NT, false, MINB, DUAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_tma);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(k_col_tma<T, PL, NT, true, MINB, DUAL>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(k_col_tma<T, PL, NT, false, MINB, DUAL>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
    }
    e = cudaFuncSetAttribute(k_col<T, PL, NT, PERM_PREF, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_inv);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_col<T, PL, NT, PERM_PREF, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_inv);
    if (e != cudaSuccess) return e;
    if (smem_inv >= kLargeTile) {
      e = cudaFuncSetAttribute(k_col<T, PL, NT, PERM_PREF, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(k_col<T, PL, NT, PERM_PREF, true, false>,
                               cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
    }
    e = cudaFuncSetAttribute(k_om_perm<T, PL, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_perm);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_om_perm<T, PL, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_perm);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_col_inv<T, PL, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_inv);
  }
  static dim3 grid(const StepArgs& a) { return dim3(a.N / 2, a.members > 1 ? a.members : 1); }
  static void col(const StepArgs& a, cudaStream_t s) { k_col<T, PL, NT, BASE, false><<<grid(a), NT, smem, s>>>(a); }
  // RK3 stages carrying the combined term run the flag-aware instantiation;
  // every other butterfly-major column pass runs the plain update
  static void col_perm(const StepArgs& a, cudaStream_t s) {
    if constexpr (TMA) {
      static const TmaMaps none{};
      const TmaMaps& m = a.cmaps ? *a.cmaps : none;
      if (a.flags & (F_Q_IN | F_Q_OUT | F_NO_FM_IN))
        k_col_tma<T, PL, NT, true, MINB, DUAL><<<grid(a), NT, smem_tma, s>>>(a, m);
      else
        k_col_tma<T, PL, NT, false, MINB, DUAL><<<grid(a), NT, smem_tma, s>>>(a, m);
      return;
    }
    if (a.flags & (F_Q_IN | F_Q_OUT | F_NO_FM_IN))
      k_col<T, PL, NT, PERM_PREF, true, true><<<grid(a), NT, smem_inv, s>>>(a);
    else
      k_col<T, PL, NT, PERM_PREF, true, false><<<grid(a), NT, smem_inv, s>>>(a);
  }
  static constexpr size_t smem_perm = size_t(2) * (2 * PL::M / 3) * sizeof(cplx<T>);  // one om + fnm1 column
  static_assert(smem_perm <= kSmemLimit, "om / fnm1 column does not fit in shared memory");
  static void to_perm(const StepArgs& a, cudaStream_t s) {
    k_om_perm<T, PL, true><<<grid(a), 256, smem_perm, s>>>(a);
  }
  static void from_perm(const StepArgs& a, cudaStream_t s) {
    k_om_perm<T, PL, false><<<grid(a), 256, smem_perm, s>>>(a);
  }
  static void col_inv(const StepArgs& a, cudaStream_t s) {
    k_col_inv<T, PL, NT><<<dim3(a.N / 2, a.members > 1 ? a.members : 1), NT, smem_inv, s>>>(a);
  }
  static int blocks_per_sm() {
    int n = 0;
    cudaError_t e;
    if constexpr (TMA)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_col_tma<T, PL, NT, false, MINB, DUAL>, NT, smem_tma);
    else
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_col<T, PL, NT, PERM_PREF, true, false>, NT, smem_inv);
    return e == cudaSuccess ? n : -1;
  }
  static constexpr ColKernels make(const char* name) {
    return ColKernels{name,    NT,     smem,     PL::TW_TOTAL,          configure, col,
                      col_inv, launch_twiddles<T, PL>, col_perm, to_perm, from_perm, blocks_per_sm, TMA, PL::RP};
  }
};

template <typename T, class PLR, int V, int NTR, class PLC, int NTC>
struct AdjOf {
  static constexpr size_t smem_row = size_t(PLR::PADM) * V * sizeof(cplx<T>) * 2;
  static constexpr size_t smem_col = size_t(PLC::PADM) * 2 * sizeof(cplx<T>);
  static_assert(smem_row <= kSmemLimit && smem_col <= kSmemLimit, "adjoint tiles do not fit");
  static cudaError_t configure() {
    cudaError_t e =
        cudaFuncSetAttribute(k_adj_row<T, PLR, V, NTR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_row);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_adj_col_in<T, PLC, NTC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_col);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_adj_col_out<T, PLC, NTC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_col);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_col_inv<T, PLC, NTC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_col);
    return e;
  }
  static void col_in(const StepArgs& a, cudaStream_t s) { k_adj_col_in<T, PLC, NTC><<<a.N / 2, NTC, smem_col, s>>>(a); }
  static void row(const StepArgs& a, cudaStream_t s) {
    k_adj_row<T, PLR, V, NTR><<<PLR::M / V, NTR, smem_row, s>>>(a);
  }
  static void col_out(const StepArgs& a, cudaStream_t s) {
    k_adj_col_out<T, PLC, NTC><<<a.N / 2, NTC, smem_col, s>>>(a);
  }
  static void col_vel(const StepArgs& a, cudaStream_t s) { k_col_inv<T, PLC, NTC><<<a.N / 2, NTC, smem_col, s>>>(a); }
  static void seed(const void* om, void* lom, void* lf, int N, double* loss_part, int blocks, cudaStream_t s) {
    k_adj_seed<T><<<blocks, 256, 0, s>>>(static_cast<const cplx<T>*>(om), static_cast<cplx<T>*>(lom),
                                         static_cast<cplx<T>*>(lf), N, loss_part);
  }
  static const AdjKernels* get() {
    static const AdjKernels k = {PLR::TW_TOTAL,   PLC::TW_TOTAL, configure, col_in, row, col_out, col_vel,
                                 launch_twiddles<T, PLR>, launch_twiddles<T, PLC>, seed};
    return &k;
  }
};

template <typename T>
void launch_spectral(const StepArgs& a, cudaStream_t s, int blocks) {
  k_spectral<T, kSpectralThreads><<<dim3(blocks, a.members > 1 ? a.members : 1), kSpectralThreads, 0, s>>>(a);
}

template <typename T>
void launch_transpose(const void* in, void* out, int rows, int cols, int batch, cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32, batch);
  k_transpose<T><<<grid, dim3(32, 8), 0, s>>>(static_cast<const cplx<T>*>(in), static_cast<cplx<T>*>(out), rows,
                                              cols);
}

template <typename T>
void launch_spectrum(const void* om, int N, int nbins, double r_max, double k_nyq, double scale2, double* esum,
                     int* cnt, cudaStream_t s) {
  k_spectrum<T, 256><<<nbins, 256, 0, s>>>(static_cast<const cplx<T>*>(om), N, nbins, r_max, k_nyq, scale2, esum,
                                             cnt);
}

template <typename T>
void launch_speed(void* phys, long long plane, cudaStream_t s) {
  k_speed<T><<<1024, 256, 0, s>>>(static_cast<T*>(phys), plane);
}

template <typename T>
void launch_pixels(const void* plane, long long n, double* part, unsigned int* counter, double* mm, unsigned char* pix,
                   cudaStream_t s) {
  k_minmax<T, 256><<<512, 256, 0, s>>>(static_cast<const T*>(plane), n, part, counter, mm);
  k_pixels<T><<<1024, 256, 0, s>>>(static_cast<const T*>(plane), n, mm, pix);
}

#define PAL_KERNEL_SET(T, PREC, N, ROWS, COLS) PAL_KERNEL_SET_ADJ(T, PREC, N, ROWS, COLS, nullptr)
#define PAL_KERNEL_SET_ADJ(T, PREC, N, ROWS, COLS, ADJ)                                                 \
  static const ::pal::KernelSet kSet##N = {N,                                                           \
                                           3 * (N) / 2,                                                 \
                                           PREC,                                                        \
                                           ROWS,                                                        \
                                           (int)(sizeof(ROWS) / sizeof(ROWS[0])),                       \
                                           COLS,                                                        \
                                           (int)(sizeof(COLS) / sizeof(COLS[0])),                       \
                                           ::pal::launch_spectral<T>,                                   \
                                           ::pal::launch_transpose<T>,                                  \
                                           ::pal::launch_spectrum<T>,                                   \
                                           ::pal::launch_speed<T>,                                      \
                                           ::pal::launch_pixels<T>,                                     \
                                           ADJ};

// One launch per pass for an ensemble of several sizes (pal_ens_fused.cu).  The
// blocks of a pass are laid out group by group, member by member: group g's
// blocks start at `first`, `per_member` of them per member; every block
// decodes its (group, member, index) and runs that size's kernel body.
constexpr int kFusedMax = 4;
struct FusedGroupArgs {
  StepArgs a;      // the group's arguments (all of its members)
  int slot;        // which compiled size of the fused set this group is
  int first;       // first block of the group in the launch
  int per_member;  // blocks per member in this pass
};
struct FusedArgs {  // aligned as CUtensorMap
  TmaMaps maps[kFusedMax];  // row-tile TMA descriptors of each group
  FusedGroupArgs g[kFusedMax];
  int ngroups;
};
// A compiled set of sizes with fixed kernel candidates of one block size.
struct FusedSet {
  int nsizes;
  int N[kFusedMax];
  const char* row_name[kFusedMax];  // the KernelSet candidates whose twiddle tables (same plan)
  const char* col_name[kFusedMax];  // and TMA row layout (same tile height) the fused bodies use
  int V[kFusedMax];                 // row tile height of each size
  int NT;  // row-pass block size (the column passes may use another)
  size_t smem_row, smem_col, smem_perm;
  cudaError_t (*configure)();
  void (*row)(const FusedArgs&, int blocks, cudaStream_t);
  void (*col)(const FusedArgs&, int blocks, bool qm, cudaStream_t);  // qm: RK3 stages (ColOf::col_perm)
  void (*phys)(const FusedArgs&, int blocks, cudaStream_t);
  void (*to_perm)(const FusedArgs&, int blocks, cudaStream_t);
  void (*from_perm)(const FusedArgs&, int blocks, cudaStream_t);
};

}  // namespace pal

// The fused set holding every size in Ns (FP32), or nullptr.
const pal::FusedSet* pal_fused_set_f32(int n, const int* Ns);

// Per-precision lookup (pal_inst_f32.cu / pal_inst_f64.cu); nullptr if unsupported.
const pal::KernelSet* pal_kernels_f32(int N);
const pal::KernelSet* pal_kernels_f64(int N);
