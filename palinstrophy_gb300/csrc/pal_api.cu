// C ABI of libpalgpu.so: handle-owned device state, stream-ordered launches of
// the fused row/column kernels, and the reference-shaped entry points.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <string>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "palgpu.h"
#include "pal_launch.cuh"

using pal::ColKernels;
using pal::DevScalars;
using pal::KernelSet;
using pal::RowKernels;
using pal::StepArgs;

namespace {

enum State { ST_EMPTY = 0, ST_VEL_PENDING = 1, ST_U = 2, ST_P = 3 };

// LS-IMEX-RK3 coefficients (turbo_simulator.py:1902-1903)
constexpr double kRkAlpha[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
constexpr double kRkBeta[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};

thread_local std::string g_err;

}  // namespace

struct pal_handle {
  int N = 0, M = 0, Nh = 0, precision = 0;
  size_t esz = 0;  // bytes per complex element
  const KernelSet* ks = nullptr;
  const RowKernels* rk = nullptr;  // selected row-pass candidate
  const ColKernels* ck = nullptr;  // selected column-pass candidate
  int row_idx = 0, col_idx = 0;
  cudaStream_t stream = nullptr;
  void *w0 = nullptr, *w1 = nullptr, *om = nullptr, *fnm1 = nullptr;
  void *om_p = nullptr, *fm_p = nullptr;  // om / fnm1 in butterfly-major order, used inside pal_step
  pal::TmaMaps tmaps{};                   // w0 / w1 descriptors when the row candidate moves rows by TMA
  pal::TmaMaps cmaps{};                   // w0 / w1 descriptors when the column candidate moves planes by TMA
  std::map<std::string, cudaGraphExec_t> step_graphs;  // pal_step sequences of small grids, by NEXTDT pattern
  void *tw_row = nullptr, *tw_col = nullptr;
  void *stage = nullptr, *phys = nullptr;
  void *vis_w = nullptr;      // two scratch work planes for display transforms
  void *vis_phys = nullptr;   // three physical planes (u|scalar, v, |u|)
  DevScalars* sc = nullptr;
  DevScalars* sc_host = nullptr;  // pinned mirror
  double* part = nullptr;
  int state = ST_EMPTY;
  bool vel_uploaded = false;  // ST_VEL_PENDING source: stage buffer (true) or om inversion
  long long it = 0;           // host copy of the iteration counter
  int spectral_blocks = 0;
  int dbg_wait0 = 0;          // pal_set_debug(PAL_DBG_SKIP_FIRST_WAIT)
  std::string err;
};

namespace pal {

bool encode_row_maps(TmaMaps* out, void* w0, void* w1, int N, int V, int members) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return false;
  const int M = 3 * N / 2, Nh = N / 2;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * M, (cuuint64_t)Nh, (cuuint64_t)members};
  const cuuint64_t strides[2] = {(cuuint64_t)M * 8, (cuuint64_t)Nh * M * 8};  // bytes, dims 1 and 2
  const cuuint32_t box[3] = {(cuuint32_t)(2 * V), (cuuint32_t)tma_box_rows(Nh), 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  void* base[2] = {w0, w1};
  CUtensorMap* maps[2] = {&out->w0, &out->w1};
  for (int i = 0; i < 2; ++i) {
    CUresult r = encode(maps[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base[i], dims, strides, box, elem,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
  }
  return true;
}

bool encode_col_maps(TmaMaps* out, void* w0, void* w1, int N, int RP, int members) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return false;
  const int M = 3 * N / 2, Nh = N / 2, G = M / RP;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * RP, (cuuint64_t)G, (cuuint64_t)Nh * members};
  const cuuint64_t strides[2] = {(cuuint64_t)RP * 8, (cuuint64_t)M * 8};  // bytes, dims 1 and 2
  // the box's inner extent (2 RP + 4 floats) runs past the 2 RP floats of a
  // group: loads fill those 4 floats with zeros, stores leave them out
  const cuuint32_t box[3] = {(cuuint32_t)(2 * RP + 4), (cuuint32_t)pal::col_box_groups(G), 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  void* base[2] = {w0, w1};
  CUtensorMap* maps[2] = {&out->w0, &out->w1};
  for (int i = 0; i < 2; ++i) {
    CUresult r = encode(maps[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base[i], dims, strides, box, elem,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
  }
  return true;
}

}  // namespace pal

namespace {

int fail(pal_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  g_err = msg;
  return code;
}

int cuda_fail(pal_handle* h, cudaError_t e, const char* what) {
  return fail(h, e == cudaErrorMemoryAllocation ? PAL_ERR_OOM : PAL_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define PAL_CK(h, expr)                                   \
  do {                                                    \
    cudaError_t e_ = (expr);                              \
    if (e_ != cudaSuccess) return cuda_fail((h), e_, #expr); \
  } while (0)

#define PAL_LAUNCHED(h, what)                                  \
  do {                                                         \
    cudaError_t e_ = cudaGetLastError();                       \
    if (e_ != cudaSuccess) return cuda_fail((h), e_, (what));  \
  } while (0)

StepArgs base_args(pal_handle* h) {
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.w0 = h->w0;
  a.w1 = h->w1;
  a.om = h->om;
  a.fnm1 = h->fnm1;
  a.tw = h->tw_row;
  a.sc = h->sc;
  a.part = h->part;
  a.phys = h->phys;
  a.om_p = h->om_p;
  a.fm_p = h->fm_p;
  a.tmaps = &h->tmaps;
  a.cmaps = &h->cmaps;
  a.N = h->N;
  a.dbg_wait0 = h->dbg_wait0;
  return a;
}

int resolve_velocity(pal_handle* h) {
  if (h->state == ST_EMPTY) return fail(h, PAL_ERR_STATE, "no spectral state set");
  if (h->state != ST_VEL_PENDING) return PAL_OK;
  StepArgs a = base_args(h);
  a.tw = h->tw_col;
  a.src = h->vel_uploaded ? h->stage : nullptr;
  h->ck->col_inv(a, h->stream);
  PAL_LAUNCHED(h, "k_col_inv");
  h->state = ST_U;
  h->vel_uploaded = false;
  return PAL_OK;
}

int launch_row(pal_handle* h, int flags) {
  StepArgs a = base_args(h);
  a.flags = flags;
  h->rk->row(a, h->stream);
  PAL_LAUNCHED(h, "k_row");
  h->state = ST_P;
  return PAL_OK;
}

// `perm`: the column pass on om_p / fm_p (butterfly-major om, fnm1), whose
// update reads and writes om / fnm1 with coalesced accesses; pal_step converts
// to that order on entry and back on exit (om_layout).
int launch_col(pal_handle* h, int scheme, int stage, int flags, bool perm = false) {
  StepArgs a = base_args(h);
  a.tw = h->tw_col;
  a.flags = flags;
  a.scheme = scheme;
  if (scheme == 1) {
    a.alpha = kRkAlpha[stage];
    a.beta = kRkBeta[stage];
    if (perm) pal::rk3_stage_flags(a, stage, kRkBeta);
  }
  if (perm)
    h->ck->col_perm(a, h->stream);
  else
    h->ck->col(a, h->stream);
  PAL_LAUNCHED(h, "k_col");
  h->state = ST_U;
  return PAL_OK;
}

int launch_phys(pal_handle* h, int flags) {
  int rc = resolve_velocity(h);
  if (rc) return rc;
  if (h->state != ST_U) return fail(h, PAL_ERR_STATE, "physical field requested between step2b and step3");
  StepArgs a = base_args(h);
  a.flags = flags | pal::F_STATS;
  h->rk->phys(a, h->stream);
  PAL_LAUNCHED(h, "k_phys");
  return PAL_OK;
}

int read_scalars(pal_handle* h) {
  PAL_CK(h, cudaMemcpyAsync(h->sc_host, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  if (h->sc_host->wait_timeout) {
    // a kernel gave up waiting for its own bulk copies; clear the flag and report
    const int zero = 0;
    cudaMemcpyAsync(reinterpret_cast<char*>(h->sc) + offsetof(DevScalars, wait_timeout), &zero, sizeof(int),
                    cudaMemcpyHostToDevice, h->stream);
    cudaStreamSynchronize(h->stream);
    h->sc_host->wait_timeout = 0;
    return fail(h, PAL_ERR_TIMEOUT, "a device wait for bulk copies timed out; the last steps are not valid");
  }
  return PAL_OK;
}

// om / fnm1 from the natural columns into om_p / fm_p (to_perm) or back.
int om_layout(pal_handle* h, bool to_perm) {
  StepArgs a = base_args(h);
  if (to_perm)
    h->ck->to_perm(a, h->stream);
  else
    h->ck->from_perm(a, h->stream);
  PAL_LAUNCHED(h, "k_om_perm");
  return PAL_OK;
}

// One full step; the first row pass carries a deferred NEXTDT when `dt_update`.
int one_step(pal_handle* h, int method, bool dt_update, bool advance, bool perm = false) {
  const int rflags = dt_update ? (pal::F_STATS | pal::F_UPDATE_DT) : 0;
  int rc;
  if (method == PAL_CNAB2) {
    if ((rc = launch_row(h, rflags))) return rc;
    return launch_col(h, 0, 0, pal::F_CNM1 | (advance ? pal::F_ADVANCE : 0), perm);
  }
  for (int s = 0; s < 3; ++s) {
    if ((rc = launch_row(h, s == 0 ? rflags : 0))) return rc;
    if ((rc = launch_col(h, 1, s, (s == 2 && advance) ? pal::F_ADVANCE : 0, perm))) return rc;
  }
  return PAL_OK;
}

int check(pal_handle* h) {
  if (!h) return fail(nullptr, PAL_ERR_INVALID, "null handle");
  return PAL_OK;
}

// Select candidates and (re)build their twiddle tables.
int select_variant(pal_handle* h, int row, int col) {
  if (row < 0 || row >= h->ks->n_rows || col < 0 || col >= h->ks->n_cols)
    return fail(h, PAL_ERR_INVALID, "variant index out of range");
  h->row_idx = row;
  h->col_idx = col;
  for (auto& kv : h->step_graphs) cudaGraphExecDestroy(kv.second);  // they hold the old kernels
  h->step_graphs.clear();
  h->rk = &h->ks->rows[row];
  h->ck = &h->ks->cols[col];
  if (h->rk->tma && !pal::encode_row_maps(&h->tmaps, h->w0, h->w1, h->N, h->rk->V, 1))
    return fail(h, PAL_ERR_CUDA, "TMA descriptor of the work planes could not be encoded");
  if (h->ck->tma && !pal::encode_col_maps(&h->cmaps, h->w0, h->w1, h->N, h->ck->rp, 1))
    return fail(h, PAL_ERR_CUDA, "TMA descriptor of the work planes (columns) could not be encoded");
  h->rk->twiddles(h->tw_row, h->stream);
  h->ck->twiddles(h->tw_col, h->stream);
  PAL_LAUNCHED(h, "twiddle tables");
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  return PAL_OK;
}

// Process-wide choice per (precision, N), so every handle of a size runs the
// same kernels (and gives bit-identical results).
std::mutex g_tune_mutex;
std::map<std::pair<int, int>, std::pair<int, int>> g_tuned;

// Tuning file (PAL_TUNE_FILE): one line per choice,
//   "<fp32|fp64> <N> <row candidate name>|<column candidate name>"
// A size listed there takes the named candidates without timing; a size that
// is timed is appended, so that later processes run the same kernels and give
// bit-identical results.  Unknown names, other sizes and malformed lines are
// skipped; a row candidate that loads by TMA multicast is skipped under
// PAL_TMA_MULTICAST=0.
const char* tune_file() {
  const char* f = std::getenv("PAL_TUNE_FILE");
  return (f && f[0]) ? f : nullptr;
}
const char* precision_name(int p) { return p == PAL_FP64 ? "fp64" : "fp32"; }

bool tune_file_lookup(const pal_handle* h, int* row, int* col) {
  const char* path = tune_file();
  if (!path) return false;
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    char prec[8] = {0};
    int n = 0, off = 0;
    if (std::sscanf(line, "%7s %d %n", prec, &n, &off) < 2 || off <= 0) continue;
    if (n != h->N || std::strcmp(prec, precision_name(h->precision)) != 0) continue;
    std::string rest(line + off);
    while (!rest.empty() && (rest.back() == '\n' || rest.back() == '\r')) rest.pop_back();
    const size_t bar = rest.find('|');
    if (bar == std::string::npos) continue;
    const std::string rname = rest.substr(0, bar), cname = rest.substr(bar + 1);
    int r = -1, c = -1;
    for (int q = 0; q < h->ks->n_rows; ++q)
      if (rname == h->ks->rows[q].name) r = q;
    for (int q = 0; q < h->ks->n_cols; ++q)
      if (cname == h->ks->cols[q].name) c = q;
    if (r < 0 || c < 0 || (h->ks->rows[r].multicast && !pal::tma_multicast_allowed())) continue;
    *row = r;
    *col = c;
    found = true;  // the last matching line wins
  }
  std::fclose(f);
  return found;
}

void tune_file_append(const pal_handle* h, int row, int col) {
  const char* path = tune_file();
  if (!path) return;
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s %d %s|%s\n", precision_name(h->precision), h->N, h->ks->rows[row].name,
               h->ks->cols[col].name);
  std::fclose(f);
}

// Time every candidate on the handle's (still zero) state and keep the fastest.
// The kernels' cost does not depend on the values they transform.
int autotune(pal_handle* h) {
  const auto key = std::make_pair(h->precision, h->N);
  // held while a size is timed: handles created concurrently wait for the one
  // timing (once per size and process) instead of timing the same candidates
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  {
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) return select_variant(h, it->second.first, it->second.second);
  }
  int best_row = 0, best_col = 0;
  if (tune_file_lookup(h, &best_row, &best_col)) {
    g_tuned[key] = std::make_pair(best_row, best_col);
    return select_variant(h, best_row, best_col);
  }
  const char* env = std::getenv("PAL_AUTOTUNE");
  const bool timed = !(env && env[0] == '0') && (h->ks->n_rows > 1 || h->ks->n_cols > 1);
  if (timed) {
    cudaEvent_t e0, e1;
    PAL_CK(h, cudaEventCreate(&e0));
    PAL_CK(h, cudaEventCreate(&e1));
    // Mean time per launch: one warm-up launch, one timed launch to size the
    // repetitions (about 1 ms of work per trial), then the best of 3 trials,
    // so that clock ramps and one-off stalls do not pick the candidate.
    auto time_launches = [&](auto&& launch, float* out) -> int {
      auto timed = [&](int reps, float* ms) -> int {
        cudaEventRecord(e0, h->stream);
        for (int q = 0; q < reps; ++q) launch();
        cudaEventRecord(e1, h->stream);
        PAL_LAUNCHED(h, "autotune");
        PAL_CK(h, cudaEventSynchronize(e1));
        cudaEventElapsedTime(ms, e0, e1);
        *ms /= (float)reps;
        return PAL_OK;
      };
      launch();
      float one = 0.f;
      if (int rc = timed(1, &one)) return rc;
      const int reps = std::max(2, std::min(50, (int)std::ceil(1.0f / std::max(one, 1e-3f))));
      float best = 1e30f;
      for (int trial = 0; trial < 3; ++trial) {
        float ms = 0.f;
        if (int rc = timed(reps, &ms)) return rc;
        best = std::min(best, ms);
      }
      *out = best;
      return PAL_OK;
    };
    float best = 1e30f;
    const bool mc_ok = pal::tma_multicast_allowed();
    for (int r = 0; r < h->ks->n_rows; ++r) {
      if (h->ks->rows[r].multicast && !mc_ok) continue;
      if (int rc = select_variant(h, r, 0)) return rc;
      const StepArgs a = base_args(h);
      float ms = 0.f;
      if (int rc = time_launches([&] { h->rk->row(a, h->stream); }, &ms)) return rc;
      if (ms < best) {
        best = ms;
        best_row = r;
      }
    }
    best = 1e30f;
    for (int c = 0; c < h->ks->n_cols; ++c) {
      if (int rc = select_variant(h, 0, c)) return rc;
      StepArgs a = base_args(h);
      a.tw = h->tw_col;
      a.scheme = 1;
      pal::rk3_stage_flags(a, 1, kRkBeta);  // the traffic of a middle RK3 stage
      float ms = 0.f;
      if (int rc = time_launches([&] { h->ck->col_perm(a, h->stream); }, &ms)) return rc;
      if (ms < best) {
        best = ms;
        best_col = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // leave the work planes as a fresh handle has them
    const size_t plane_w = (size_t)h->Nh * h->M * h->esz;
    PAL_CK(h, cudaMemsetAsync(h->w0, 0, plane_w, h->stream));
    PAL_CK(h, cudaMemsetAsync(h->w1, 0, plane_w, h->stream));
  }
  g_tuned[key] = std::make_pair(best_row, best_col);
  if (timed) tune_file_append(h, best_row, best_col);
  return select_variant(h, best_row, best_col);
}

}  // namespace

// Device generator (pal_generate.cu).
int pal_generate_device(int N, int precision, double K0, double Re, int seed, int spectrum, void* om_dev,
                        void* uc_dev, cudaStream_t s, double* stats, int* seed_out, std::string* err);

extern "C" {

int pal_supported(int N, int precision) {
  if (precision == PAL_FP32) return pal_kernels_f32(N) != nullptr;
  if (precision == PAL_FP64) return pal_kernels_f64(N) != nullptr;
  return 0;
}

int pal_device_info(int* sm_count, int* smem_optin, char* name, size_t name_len) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDevice");
  cudaDeviceProp p;
  e = cudaGetDeviceProperties(&p, dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDeviceProperties");
  if (sm_count) *sm_count = p.multiProcessorCount;
  if (smem_optin) *smem_optin = (int)p.sharedMemPerBlockOptin;
  if (name && name_len) {
    std::strncpy(name, p.name, name_len - 1);
    name[name_len - 1] = 0;
  }
  return PAL_OK;
}

int pal_create(int N, int precision, double Re, double cfl, pal_handle** out) {
  if (!out) return fail(nullptr, PAL_ERR_INVALID, "out is null");
  *out = nullptr;
  if (precision != PAL_FP32 && precision != PAL_FP64) return fail(nullptr, PAL_ERR_INVALID, "precision must be PAL_FP32 or PAL_FP64");
  const KernelSet* ks = precision == PAL_FP32 ? pal_kernels_f32(N) : pal_kernels_f64(N);
  if (!ks) return fail(nullptr, PAL_ERR_INVALID, "unsupported grid N=" + std::to_string(N) + " for this precision");
  if (!(Re > 0.0) || !(cfl > 0.0)) return fail(nullptr, PAL_ERR_INVALID, "Re and cfl must be positive");
  pal_handle* h = new pal_handle();
  h->N = N;
  h->M = 3 * N / 2;
  h->Nh = N / 2;
  h->precision = precision;
  h->esz = precision == PAL_FP32 ? 8 : 16;
  h->ks = ks;
  auto bail = [&](int code) {
    pal_destroy(h);
    return code;
  };
  cudaError_t e = cudaSuccess;
  size_t tw_max = 0;
  for (int r = 0; r < ks->n_rows && e == cudaSuccess; ++r) {
    e = ks->rows[r].configure();
    tw_max = std::max(tw_max, (size_t)ks->rows[r].tw_elems);
  }
  for (int c = 0; c < ks->n_cols && e == cudaSuccess; ++c) {
    e = ks->cols[c].configure();
    tw_max = std::max(tw_max, (size_t)ks->cols[c].tw_elems);
  }
  if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "kernel configure"));
  e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaStreamCreate"));
  const size_t plane_w = (size_t)h->Nh * h->M * h->esz;
  const size_t plane_om = (size_t)h->Nh * N * h->esz;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  h->spectral_blocks = std::max(1, std::min(4 * sms, (int)(((size_t)N * h->Nh + 255) / 256)));
  const size_t part_n = (size_t)std::max(h->M, std::max(1024, h->spectral_blocks)) * 5;
  void** bufs[] = {&h->w0, &h->w1, &h->om, &h->fnm1, &h->stage, &h->tw_row, &h->tw_col, &h->om_p};
  const size_t sizes[] = {plane_w + pal::kPlaneSlack, plane_w + pal::kPlaneSlack, plane_om, plane_om, 2 * plane_om,
                          tw_max * h->esz, tw_max * h->esz, 2 * plane_w};
  for (int i = 0; i < 8; ++i) {
    e = cudaMalloc(bufs[i], sizes[i]);
    if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaMalloc state"));
    e = cudaMemsetAsync(*bufs[i], 0, sizes[i], h->stream);
    if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaMemset state"));
  }
  h->fm_p = static_cast<char*>(h->om_p) + plane_w;
  e = cudaMalloc(&h->sc, sizeof(DevScalars));
  if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaMalloc scalars"));
  e = cudaMalloc(&h->part, part_n * sizeof(double));
  if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaMalloc partials"));
  e = cudaMallocHost(&h->sc_host, sizeof(DevScalars));
  if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "cudaMallocHost"));
  std::memset(h->sc_host, 0, sizeof(DevScalars));
  h->sc_host->cn = 1.0;
  h->sc_host->visc = (double)(float)(1.0 / (double)(float)Re);
  h->sc_host->cflnum = cfl;
  e = cudaMemcpyAsync(h->sc, h->sc_host, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "upload scalars"));
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return bail(cuda_fail(nullptr, e, "initialise state"));
  if (int rc = autotune(h)) {
    g_err = h->err;
    return bail(rc);
  }
  *out = h;
  return PAL_OK;
}

int pal_destroy(pal_handle* h) {
  if (!h) return PAL_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& kv : h->step_graphs) cudaGraphExecDestroy(kv.second);
  h->step_graphs.clear();
  void* bufs[] = {h->w0,     h->w1,   h->om,   h->fnm1, h->stage, h->tw_row,   h->tw_col,
                  h->phys,   h->sc,   h->part, h->vis_w, h->vis_phys, h->om_p};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (h->sc_host) cudaFreeHost(h->sc_host);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PAL_OK;
}

int pal_set_spectral_state(pal_handle* h, const void* om2, const void* fnm1) {
  if (int rc = check(h)) return rc;
  if (!om2) return fail(h, PAL_ERR_INVALID, "om2 is null");
  const size_t bytes = (size_t)h->N * h->Nh * h->esz;
  // cudaMemcpyDefault: om2 / fnm1 may be host or device memory (unified addressing)
  PAL_CK(h, cudaMemcpyAsync(h->stage, om2, bytes, cudaMemcpyDefault, h->stream));
  h->ks->transpose(h->stage, h->om, h->N, h->Nh, 1, h->stream);
  PAL_LAUNCHED(h, "transpose om2");
  if (fnm1) {
    PAL_CK(h, cudaMemcpyAsync(h->stage, fnm1, bytes, cudaMemcpyDefault, h->stream));
    h->ks->transpose(h->stage, h->fnm1, h->N, h->Nh, 1, h->stream);
    PAL_LAUNCHED(h, "transpose fnm1");
  } else {
    PAL_CK(h, cudaMemsetAsync(h->fnm1, 0, bytes, h->stream));
  }
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  h->state = ST_VEL_PENDING;
  h->vel_uploaded = false;
  return PAL_OK;
}

int pal_generate(pal_handle* h, double K0, double Re, int seed, int spectrum, void* uc_host, double* stats,
                 int* seed_out) {
  if (int rc = check(h)) return rc;
  if (spectrum != PAL_SPEC_KM3 && spectrum != PAL_SPEC_PAO) return fail(h, PAL_ERR_INVALID, "unknown spectrum");
  if (!(K0 > 0.0) || !(Re > 0.0)) return fail(h, PAL_ERR_INVALID, "K0 and Re must be positive");
  std::string err;
  if (int rc = pal_generate_device(h->N, h->precision, K0, Re, seed, spectrum, h->om, h->stage, h->stream, stats,
                                   seed_out, &err))
    return fail(h, rc, err);
  const size_t bytes = (size_t)h->N * h->Nh * h->esz;
  PAL_CK(h, cudaMemsetAsync(h->fnm1, 0, bytes, h->stream));
  if (uc_host) PAL_CK(h, cudaMemcpyAsync(uc_host, h->stage, 2 * bytes, cudaMemcpyDeviceToHost, h->stream));
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  h->state = ST_VEL_PENDING;
  h->vel_uploaded = true;
  return PAL_OK;
}

int pal_set_velocity_spectrum(pal_handle* h, const void* uc_low) {
  if (int rc = check(h)) return rc;
  if (h->state == ST_EMPTY) return fail(h, PAL_ERR_STATE, "set the spectral state first");
  if (!uc_low) {
    h->state = ST_VEL_PENDING;
    h->vel_uploaded = false;
    return PAL_OK;
  }
  const size_t bytes = 2 * (size_t)h->N * h->Nh * h->esz;
  PAL_CK(h, cudaMemcpyAsync(h->stage, uc_low, bytes, cudaMemcpyDefault, h->stream));
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  h->state = ST_VEL_PENDING;
  h->vel_uploaded = true;
  return PAL_OK;
}

int pal_set_scalars(pal_handle* h, double t, double dt, double cn, double cnm1, double visc, double cflnum,
                    long long it) {
  if (int rc = check(h)) return rc;
  PAL_CK(h, cudaMemcpyAsync(h->sc_host, h->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  DevScalars* s = h->sc_host;
  s->t = t;
  s->dt = dt;
  s->cn = cn;
  s->cnm1 = cnm1;
  s->visc = visc;
  s->cflnum = cflnum;
  s->it = it;
  h->it = it;
  PAL_CK(h, cudaMemcpyAsync(h->sc, h->sc_host, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream));
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  return PAL_OK;
}

int pal_set_scalar(pal_handle* h, int which, double value) {
  if (int rc = check(h)) return rc;
  size_t off;
  switch (which) {
    case PAL_SC_T: off = offsetof(DevScalars, t); break;
    case PAL_SC_DT: off = offsetof(DevScalars, dt); break;
    case PAL_SC_CN: off = offsetof(DevScalars, cn); break;
    case PAL_SC_CNM1: off = offsetof(DevScalars, cnm1); break;
    case PAL_SC_VISC: off = offsetof(DevScalars, visc); break;
    case PAL_SC_CFLNUM: off = offsetof(DevScalars, cflnum); break;
    case PAL_SC_IT: {
      const long long it = (long long)value;
      h->it = it;
      PAL_CK(h, cudaMemcpyAsync(reinterpret_cast<char*>(h->sc) + offsetof(DevScalars, it), &it, sizeof(it),
                                cudaMemcpyHostToDevice, h->stream));
      PAL_CK(h, cudaStreamSynchronize(h->stream));
      return PAL_OK;
    }
    default: return fail(h, PAL_ERR_INVALID, "unknown scalar");
  }
  PAL_CK(h, cudaMemcpyAsync(reinterpret_cast<char*>(h->sc) + off, &value, sizeof(double), cudaMemcpyHostToDevice,
                            h->stream));
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  return PAL_OK;
}

int pal_get_scalars(pal_handle* h, double* t, double* dt, double* cn, double* cnm1, double* visc, double* cflnum,
                    long long* it) {
  if (int rc = check(h)) return rc;
  if (int rc = read_scalars(h)) return rc;
  const DevScalars* s = h->sc_host;
  if (t) *t = s->t;
  if (dt) *dt = s->dt;
  if (cn) *cn = s->cn;
  if (cnm1) *cnm1 = s->cnm1;
  if (visc) *visc = s->visc;
  if (cflnum) *cflnum = s->cflnum;
  if (it) *it = s->it;
  return PAL_OK;
}

int pal_step2a(pal_handle* h) {
  if (int rc = check(h)) return rc;
  if (h->state == ST_P) return fail(h, PAL_ERR_STATE, "dns_step2a after dns_step2b without dns_step3");
  return resolve_velocity(h);
}

int pal_step2b(pal_handle* h) {
  if (int rc = check(h)) return rc;
  if (int rc = resolve_velocity(h)) return rc;
  if (h->state != ST_U) return fail(h, PAL_ERR_STATE, "dns_step2b needs the physical velocity (call dns_step2a)");
  return launch_row(h, 0);
}

int pal_step3(pal_handle* h) {
  if (int rc = check(h)) return rc;
  if (h->state != ST_P) return fail(h, PAL_ERR_STATE, "dns_step3 needs the products of dns_step2b");
  return launch_col(h, 0, 0, pal::F_CNM1);
}

int pal_step_rk3(pal_handle* h) {
  if (int rc = check(h)) return rc;
  if (int rc = resolve_velocity(h)) return rc;
  if (h->state != ST_U) return fail(h, PAL_ERR_STATE, "LS-IMEX-RK3 step needs the physical velocity");
  // three column passes: worth the butterfly-major order and its two conversions
  if (int rc = om_layout(h, true)) return rc;
  const int rc = one_step(h, PAL_LS_IMEX_RK3, false, false, true);
  const int rc2 = om_layout(h, false);
  return rc != PAL_OK ? rc : rc2;
}

// Grids up to this size are launch-bound: their step sequences are captured
// once per NEXTDT pattern and replayed as CUDA graphs.
constexpr int kStepGraphMaxN = 1024;
constexpr size_t kStepGraphCache = 16;

int pal_step(pal_handle* h, int method, int nsteps, int update, int final_update) {
  if (int rc = check(h)) return rc;
  if (method != PAL_CNAB2 && method != PAL_LS_IMEX_RK3) return fail(h, PAL_ERR_INVALID, "unknown time stepper");
  if (nsteps < 0) return fail(h, PAL_ERR_INVALID, "nsteps < 0");
  if (int rc = resolve_velocity(h)) return rc;
  if (h->state != ST_U) return fail(h, PAL_ERR_STATE, "pal_step needs the physical velocity");
  bool pending = false;
  if (nsteps > 0) {
    // fused NEXTDT at the start of step j when the previous step ended on the cadence
    std::string key = std::to_string(method) + ":";
    std::vector<char> upd(nsteps);
    const long long it0 = h->it;
    for (int j = 1; j <= nsteps; ++j) {
      upd[j - 1] = pending;
      key += pending ? '1' : '0';
      const long long it = it0 + j;
      pending = update > 0 && (it % update == 0 || it == 1 || (final_update && j == nsteps));
    }
    // The column pass runs on the butterfly-major om order, whose two
    // conversions (~60 us each at N=4096) cost less than one step's three
    // natural-order column passes (~370 us more).
    auto record = [&]() -> int {
      if (int rc = om_layout(h, true)) return rc;
      int rc = PAL_OK;
      for (int j = 0; j < nsteps && rc == PAL_OK; ++j) rc = one_step(h, method, upd[j] != 0, true, true);
      const int rc2 = om_layout(h, false);
      return rc != PAL_OK ? rc : rc2;
    };
    const char* env = std::getenv("PAL_STEP_GRAPHS");
    const bool graphs = h->N <= kStepGraphMaxN && nsteps >= 2 && !(env && env[0] == '0');
    if (!graphs) {
      if (int rc = record()) return rc;
    } else {
      auto found = h->step_graphs.find(key);
      if (found == h->step_graphs.end()) {
        if (h->step_graphs.size() >= kStepGraphCache) {
          for (auto& kv : h->step_graphs) cudaGraphExecDestroy(kv.second);
          h->step_graphs.clear();
        }
        PAL_CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = record();
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
        if (rc != PAL_OK) {
          if (graph) cudaGraphDestroy(graph);
          return rc;
        }
        if (ce != cudaSuccess) return cuda_fail(h, ce, "step graph capture");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_fail(h, ie, "step graph instantiate");
        found = h->step_graphs.emplace(key, exec).first;
      }
      PAL_CK(h, cudaGraphLaunch(found->second, h->stream));
      h->state = ST_U;
    }
    h->it = it0 + nsteps;
  }
  if (pending) return launch_phys(h, pal::F_UPDATE_DT);
  return PAL_OK;
}

int pal_compute_cflm(pal_handle* h, double* cflm) {
  if (int rc = check(h)) return rc;
  if (int rc = launch_phys(h, 0)) return rc;
  if (int rc = read_scalars(h)) return rc;
  if (cflm) *cflm = h->sc_host->cflm;
  return PAL_OK;
}

int pal_next_dt(pal_handle* h, int sync_host, double* cflm) {
  if (int rc = check(h)) return rc;
  if (int rc = launch_phys(h, pal::F_UPDATE_DT)) return rc;
  if (sync_host) {
    if (int rc = read_scalars(h)) return rc;
    if (cflm) *cflm = h->sc_host->cflm;
  }
  return PAL_OK;
}

int pal_diagnostics(pal_handle* h, pal_diag* out) {
  if (int rc = check(h)) return rc;
  if (!out) return fail(h, PAL_ERR_INVALID, "out is null");
  if (int rc = launch_phys(h, pal::F_DIAG)) return rc;
  StepArgs a = base_args(h);
  h->ks->spectral(a, h->stream, h->spectral_blocks);
  PAL_LAUNCHED(h, "k_spectral");
  if (int rc = read_scalars(h)) return rc;
  const DevScalars* s = h->sc_host;
  out->U = std::sqrt(std::max(0.0, s->mean_speed2));
  out->E = s->E;
  out->Z = s->Z;
  out->P = s->P;
  out->kmax2 = s->kmax2;
  out->L = s->E > 0.0 ? 2.0 * pal::kPi * s->L / s->E : NAN;
  out->tau_l = (out->U > 0.0 && s->E > 0.0) ? out->L / out->U : NAN;
  out->pal_over_ens_kmax2 = (s->Z > 0.0 && s->kmax2 > 0.0) ? s->P / (s->Z * s->kmax2) : 0.0;
  out->cflm = s->cflm;
  out->energy_joules = 0.5 * (2.0 * pal::kPi) * (2.0 * pal::kPi) * s->mean_speed2;
  out->nonfinite = s->nonfinite;
  if (s->nonfinite) return fail(h, PAL_ERR_NONFINITE, "NaN/Inf in the field");
  return PAL_OK;
}

int pal_energy_spectrum(pal_handle* h, int nbins, double r_max, double k_nyq, double* esum, int* count) {
  if (int rc = check(h)) return rc;
  if (nbins <= 0 || !(r_max > 0.0) || !(k_nyq > 0.0) || !esum || !count)
    return fail(h, PAL_ERR_INVALID, "bad spectrum arguments");
  if (h->state == ST_EMPTY) return fail(h, PAL_ERR_STATE, "no spectral state set");
  double* d_e = nullptr;
  PAL_CK(h, cudaMallocAsync(reinterpret_cast<void**>(&d_e), (size_t)nbins * (sizeof(double) + sizeof(int)),
                            h->stream));
  int* d_c = reinterpret_cast<int*>(d_e + nbins);
  const double scale = (double)h->M * (double)h->M;
  h->ks->spectrum(h->om, h->N, nbins, r_max, k_nyq, scale * scale, d_e, d_c, h->stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(esum, d_e, nbins * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(count, d_c, nbins * sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  cudaFreeAsync(d_e, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "energy spectrum");
  return PAL_OK;
}

int pal_vis_field(pal_handle* h, int var, void* host_field, unsigned char* host_pixels) {
  if (int rc = check(h)) return rc;
  if (var < PAL_VAR_U || var > PAL_VAR_STREAM) return fail(h, PAL_ERR_INVALID, "unknown display variable");
  if (int rc = resolve_velocity(h)) return rc;
  if (h->state != ST_U) return fail(h, PAL_ERR_STATE, "display between step2b and step3");
  const size_t rsz = h->esz / 2;
  const long long plane = (long long)h->M * h->M;
  // scratch: 3 physical planes, then [DevScalars | min,max | counter | 512 x (min,max) partials | pixels]
  const size_t aux = 256 + 16 + 16 + 512 * 16;
  if (!h->vis_phys) PAL_CK(h, cudaMalloc(&h->vis_phys, 3 * plane * rsz + aux + plane));
  char* auxp = static_cast<char*>(h->vis_phys) + 3 * plane * rsz;
  DevScalars* vsc = reinterpret_cast<DevScalars*>(auxp);
  double* mm = reinterpret_cast<double*>(auxp + 256);
  unsigned int* counter = reinterpret_cast<unsigned int*>(auxp + 256 + 16);
  double* mm_part = reinterpret_cast<double*>(auxp + 256 + 32);
  unsigned char* d_pix = reinterpret_cast<unsigned char*>(auxp + aux);
  PAL_CK(h, cudaMemsetAsync(auxp, 0, 256 + 32, h->stream));
  StepArgs a = base_args(h);
  a.phys = h->vis_phys;
  a.sc = vsc;  // display statistics never touch the state's scalars
  a.flags = pal::F_PHYS | pal::F_STATS;
  if (var == PAL_VAR_OMEGA || var == PAL_VAR_STREAM) {
    if (!h->vis_w) PAL_CK(h, cudaMalloc(&h->vis_w, 2 * (size_t)h->Nh * h->M * h->esz));
    StepArgs b = base_args(h);
    b.w0 = h->vis_w;
    b.w1 = static_cast<char*>(h->vis_w) + (size_t)h->Nh * h->M * h->esz;
    b.tw = h->tw_col;
    b.scheme = var == PAL_VAR_OMEGA ? 1 : 2;
    h->ck->col_inv(b, h->stream);
    PAL_LAUNCHED(h, "k_col_inv (display)");
    a.w0 = b.w0;
    a.w1 = b.w1;
  }
  h->rk->phys(a, h->stream);
  PAL_LAUNCHED(h, "k_phys (display)");
  const char* src = static_cast<const char*>(h->vis_phys);
  if (var == PAL_VAR_V) src += plane * rsz;
  if (var == PAL_VAR_ENERGY) {
    h->ks->speed(h->vis_phys, plane, h->stream);
    PAL_LAUNCHED(h, "k_speed");
    src += 2 * plane * rsz;
  }
  if (host_field) PAL_CK(h, cudaMemcpyAsync(host_field, src, plane * rsz, cudaMemcpyDeviceToHost, h->stream));
  if (host_pixels) {
    h->ks->pixels(src, plane, mm_part, counter, mm, d_pix, h->stream);
    PAL_LAUNCHED(h, "k_pixels");
    PAL_CK(h, cudaMemcpyAsync(host_pixels, d_pix, plane, cudaMemcpyDeviceToHost, h->stream));
  }
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  return PAL_OK;
}

int pal_adjoint_palinstrophy(pal_handle* h, int nsteps, int ckpt_every, double* loss, void* grad_host) {
  if (int rc = check(h)) return rc;
  const pal::AdjKernels* adj = h->ks->adj;
  if (!adj) return fail(h, PAL_ERR_INVALID, "no adjoint kernels compiled for this grid");
  if (nsteps <= 0 || ckpt_every <= 0) return fail(h, PAL_ERR_INVALID, "nsteps and ckpt_every must be positive");
  if (int rc = resolve_velocity(h)) return rc;
  if (h->state != ST_U) return fail(h, PAL_ERR_STATE, "adjoint needs the physical velocity");
  if (adj->configure() != cudaSuccess) return fail(h, PAL_ERR_CUDA, "adjoint configure");
  const size_t plane_om = (size_t)h->Nh * h->N * h->esz, plane_w = (size_t)h->Nh * h->M * h->esz;
  const int n_ck = (nsteps + ckpt_every - 1) / ckpt_every;
  const int stages_max = 3 * ckpt_every;
  // one allocation: checkpoints (om, fnm1) | final state | stage inputs | lam_om, lam_f | Y planes | tables | loss
  const size_t tw_bytes = (size_t)(adj->tw_row_elems + adj->tw_col_elems) * h->esz;
  const int seed_blocks = 256;
  const size_t bytes = 2 * plane_om * (size_t)n_ck + 2 * plane_om + plane_om * (size_t)stages_max + 2 * plane_om +
                       2 * plane_w + tw_bytes + seed_blocks * sizeof(double) + 1024;
  char* buf = nullptr;
  PAL_CK(h, cudaMallocAsync(reinterpret_cast<void**>(&buf), bytes, h->stream));
  char* ck = buf;
  char* fin = ck + 2 * plane_om * (size_t)n_ck;
  char* st = fin + 2 * plane_om;
  char* lom = st + plane_om * (size_t)stages_max;
  char* lf = lom + plane_om;
  char* y0 = lf + plane_om;
  char* y1 = y0 + plane_w;
  char* tw_r = y1 + plane_w;
  char* tw_c = tw_r + (size_t)adj->tw_row_elems * h->esz;
  double* loss_part = reinterpret_cast<double*>(((uintptr_t)(tw_c + (size_t)adj->tw_col_elems * h->esz) + 255) & ~(uintptr_t)255);
  adj->tw_row(tw_r, h->stream);
  adj->tw_col(tw_c, h->stream);
  int rc = PAL_OK;
  auto seg_len = [&](int seg) { return std::min(ckpt_every, nsteps - seg * ckpt_every); };
  // Segments are launch sequences with fixed buffers; full-length segments are
  // captured once as CUDA graphs (forward, and recompute + adjoint sweep) and
  // replayed, the checkpoint copies staying outside the graphs.
  auto forward_body = [&](int ns) -> int {
    int r = PAL_OK;
    for (int j = 0; j < ns && r == PAL_OK; ++j) r = one_step(h, PAL_LS_IMEX_RK3, false, true);
    return r;
  };
  auto backward_body = [&](int ns) -> int {
    h->state = ST_VEL_PENDING;
    h->vel_uploaded = false;
    int r = resolve_velocity(h);
    for (int j = 0; j < ns && r == PAL_OK; ++j) {
      for (int s = 0; s < 3 && r == PAL_OK; ++s) {
        cudaMemcpyAsync(st + plane_om * (size_t)(3 * j + s), h->om, plane_om, cudaMemcpyDeviceToDevice, h->stream);
        if ((r = launch_row(h, 0))) break;
        r = launch_col(h, 1, s, 0);
      }
    }
    for (int q = 3 * ns - 1; q >= 0 && r == PAL_OK; --q) {
      const int s = q % 3;
      StepArgs a = base_args(h);
      a.om = lom;
      a.fnm1 = lf;
      a.alpha = kRkAlpha[s];
      a.beta = kRkBeta[s];
      a.tw = tw_c;
      adj->col_in(a, h->stream);
      StepArgs b = base_args(h);
      b.om = st + plane_om * (size_t)q;
      b.w0 = y0;
      b.w1 = y1;
      b.tw = tw_c;
      b.src = nullptr;
      adj->col_vel(b, h->stream);
      a.y0 = y0;
      a.y1 = y1;
      a.tw = tw_r;
      adj->row(a, h->stream);
      a.tw = tw_c;
      adj->col_out(a, h->stream);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) r = cuda_fail(h, e, "adjoint stage");
    }
    return r;
  };
  auto capture = [&](auto&& body, int ns, cudaGraphExec_t* exec) -> int {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(h, e, "begin capture");
    const int r = body(ns);
    e = cudaStreamEndCapture(h->stream, &g);
    if (r) return r;
    if (e != cudaSuccess) return cuda_fail(h, e, "end capture");
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(h, e, "graph instantiate");
    return PAL_OK;
  };
  const bool use_graphs = !(std::getenv("PAL_ADJOINT_GRAPHS") && std::getenv("PAL_ADJOINT_GRAPHS")[0] == '0');
  cudaGraphExec_t g_fwd = nullptr, g_bwd = nullptr;
  // forward sweep with checkpoints (fixed dt: no NEXTDT)
  for (int seg = 0; seg < n_ck && rc == PAL_OK; ++seg) {
    cudaMemcpyAsync(ck + 2 * plane_om * seg, h->om, plane_om, cudaMemcpyDeviceToDevice, h->stream);
    cudaMemcpyAsync(ck + 2 * plane_om * seg + plane_om, h->fnm1, plane_om, cudaMemcpyDeviceToDevice, h->stream);
    const int ns = seg_len(seg);
    if (use_graphs && ns == ckpt_every) {
      if (!g_fwd) rc = capture(forward_body, ns, &g_fwd);
      if (rc == PAL_OK && cudaGraphLaunch(g_fwd, h->stream) != cudaSuccess) rc = fail(h, PAL_ERR_CUDA, "graph launch");
    } else {
      rc = forward_body(ns);
    }
  }
  if (rc == PAL_OK) {
    cudaMemcpyAsync(fin, h->om, plane_om, cudaMemcpyDeviceToDevice, h->stream);
    cudaMemcpyAsync(fin + plane_om, h->fnm1, plane_om, cudaMemcpyDeviceToDevice, h->stream);
    adj->seed(h->om, lom, lf, h->N, loss_part, seed_blocks, h->stream);
  }
  // backward sweep: per segment, recompute and store the stage inputs, then run
  // the adjoint stages in reverse
  for (int seg = n_ck - 1; seg >= 0 && rc == PAL_OK; --seg) {
    cudaMemcpyAsync(h->om, ck + 2 * plane_om * seg, plane_om, cudaMemcpyDeviceToDevice, h->stream);
    cudaMemcpyAsync(h->fnm1, ck + 2 * plane_om * seg + plane_om, plane_om, cudaMemcpyDeviceToDevice, h->stream);
    const int ns = seg_len(seg);
    if (use_graphs && ns == ckpt_every) {
      if (!g_bwd) rc = capture(backward_body, ns, &g_bwd);
      if (rc == PAL_OK && cudaGraphLaunch(g_bwd, h->stream) != cudaSuccess) rc = fail(h, PAL_ERR_CUDA, "graph launch");
    } else {
      rc = backward_body(ns);
    }
  }
  if (g_fwd) cudaGraphExecDestroy(g_fwd);
  if (g_bwd) cudaGraphExecDestroy(g_bwd);
  // leave the handle at the final forward state
  cudaMemcpyAsync(h->om, fin, plane_om, cudaMemcpyDeviceToDevice, h->stream);
  cudaMemcpyAsync(h->fnm1, fin + plane_om, plane_om, cudaMemcpyDeviceToDevice, h->stream);
  h->state = ST_VEL_PENDING;
  h->vel_uploaded = false;
  if (rc == PAL_OK) rc = resolve_velocity(h);
  if (rc == PAL_OK && grad_host) {
    h->ks->transpose(lom, h->stage, h->Nh, h->N, 1, h->stream);
    cudaError_t e = cudaMemcpyAsync(grad_host, h->stage, plane_om, cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "gradient download");
  }
  std::vector<double> lp(seed_blocks, 0.0);
  if (rc == PAL_OK && loss) {
    cudaError_t e = cudaMemcpyAsync(lp.data(), loss_part, seed_blocks * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "loss download");
  }
  cudaFreeAsync(buf, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (rc == PAL_OK && e != cudaSuccess) rc = cuda_fail(h, e, "adjoint");
  if (rc == PAL_OK && loss) {
    double acc = 0.0;
    for (double v : lp) acc += v;
    *loss = acc;
  }
  return rc;
}

int pal_materialize_physical(pal_handle* h) {
  if (int rc = check(h)) return rc;
  if (!h->phys) {
    const size_t bytes = 2 * (size_t)h->M * h->M * (h->esz / 2);
    PAL_CK(h, cudaMalloc(&h->phys, bytes));
  }
  return launch_phys(h, pal::F_PHYS);
}

int pal_get_field(pal_handle* h, int which, void* host_dst) {
  if (int rc = check(h)) return rc;
  if (!host_dst) return fail(h, PAL_ERR_INVALID, "host_dst is null");
  if (which == PAL_FIELD_OM2 || which == PAL_FIELD_FNM1) {
    // the stage buffer is the transpose's scratch: a velocity band waiting
    // there for STEP2A is turned into the U state first
    if (h->state == ST_VEL_PENDING && h->vel_uploaded)
      if (int rc = resolve_velocity(h)) return rc;
    h->ks->transpose(which == PAL_FIELD_OM2 ? h->om : h->fnm1, h->stage, h->Nh, h->N, 1, h->stream);
    PAL_LAUNCHED(h, "transpose out");
    PAL_CK(h, cudaMemcpyAsync(host_dst, h->stage, (size_t)h->N * h->Nh * h->esz, cudaMemcpyDeviceToHost, h->stream));
    PAL_CK(h, cudaStreamSynchronize(h->stream));
    return PAL_OK;
  }
  if (which == PAL_FIELD_UR_U || which == PAL_FIELD_UR_V) {
    if (int rc = pal_materialize_physical(h)) return rc;
    const size_t plane = (size_t)h->M * h->M * (h->esz / 2);
    const char* src = static_cast<const char*>(h->phys) + (which == PAL_FIELD_UR_V ? plane : 0);
    PAL_CK(h, cudaMemcpyAsync(host_dst, src, plane, cudaMemcpyDeviceToHost, h->stream));
    PAL_CK(h, cudaStreamSynchronize(h->stream));
    return PAL_OK;
  }
  return fail(h, PAL_ERR_INVALID, "unknown field");
}

int pal_field_device_ptr(pal_handle* h, int which, void** ptr) {
  if (int rc = check(h)) return rc;
  if (!ptr) return fail(h, PAL_ERR_INVALID, "ptr is null");
  switch (which) {
    case PAL_FIELD_OM2: *ptr = h->om; return PAL_OK;
    case PAL_FIELD_FNM1: *ptr = h->fnm1; return PAL_OK;
    case PAL_FIELD_UR_U:
    case PAL_FIELD_UR_V:
      if (!h->phys) return fail(h, PAL_ERR_STATE, "physical planes not materialized");
      *ptr = static_cast<char*>(h->phys) + (which == PAL_FIELD_UR_V ? (size_t)h->M * h->M * (h->esz / 2) : 0);
      return PAL_OK;
    default: return fail(h, PAL_ERR_INVALID, "unknown field");
  }
}

int pal_synchronize(pal_handle* h) {
  if (int rc = check(h)) return rc;
  PAL_CK(h, cudaStreamSynchronize(h->stream));
  return PAL_OK;
}

int pal_profile_kernels(pal_handle* h, int method, int nsteps, double* ms_row, double* ms_col, int* launches) {
  if (int rc = check(h)) return rc;
  if (method != PAL_CNAB2 && method != PAL_LS_IMEX_RK3) return fail(h, PAL_ERR_INVALID, "unknown time stepper");
  if (nsteps <= 0) return fail(h, PAL_ERR_INVALID, "nsteps must be positive");
  if (int rc = resolve_velocity(h)) return rc;
  if (h->state != ST_U) return fail(h, PAL_ERR_STATE, "profiling needs the physical velocity");
  const int stages = method == PAL_CNAB2 ? 1 : 3;
  const int n_ev = 2 * stages * nsteps + 1;
  std::vector<cudaEvent_t> ev(n_ev, nullptr);
  int rc = PAL_OK;
  for (auto& e : ev) {
    cudaError_t ce = cudaEventCreate(&e);
    if (ce != cudaSuccess) {
      rc = cuda_fail(h, ce, "cudaEventCreate");
      break;
    }
  }
  int k = 0;
  if (rc == PAL_OK) rc = om_layout(h, true);  // the pass as pal_step runs it
  if (rc == PAL_OK) {
    cudaEventRecord(ev[k++], h->stream);
    for (int j = 0; j < nsteps && rc == PAL_OK; ++j) {
      for (int s = 0; s < stages && rc == PAL_OK; ++s) {
        rc = launch_row(h, 0);
        cudaEventRecord(ev[k++], h->stream);
        if (rc == PAL_OK)
          rc = launch_col(h, method == PAL_CNAB2 ? 0 : 1, s,
                          (method == PAL_CNAB2 ? pal::F_CNM1 : 0) | (s == stages - 1 ? pal::F_ADVANCE : 0), true);
        cudaEventRecord(ev[k++], h->stream);
      }
      if (rc == PAL_OK) h->it += 1;
    }
    const int rc2 = om_layout(h, false);
    if (rc == PAL_OK) rc = rc2;
  }
  double tr = 0.0, tc = 0.0;
  if (rc == PAL_OK) {
    cudaError_t ce = cudaEventSynchronize(ev[k - 1]);
    if (ce != cudaSuccess) rc = cuda_fail(h, ce, "cudaEventSynchronize");
    for (int q = 0; rc == PAL_OK && q + 2 <= k - 1; q += 2) {
      float a = 0.f, b = 0.f;
      cudaEventElapsedTime(&a, ev[q], ev[q + 1]);
      cudaEventElapsedTime(&b, ev[q + 1], ev[q + 2]);
      tr += a;
      tc += b;
    }
  }
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  if (rc != PAL_OK) return rc;
  const int nl = stages * nsteps;
  if (ms_row) *ms_row = tr / nl;
  if (ms_col) *ms_col = tc / nl;
  if (launches) *launches = 2 * nl;
  return PAL_OK;
}

int pal_get_variant(pal_handle* h, int* row, int* col, int* n_rows, int* n_cols, char* desc, size_t desc_len) {
  if (int rc = check(h)) return rc;
  if (row) *row = h->row_idx;
  if (col) *col = h->col_idx;
  if (n_rows) *n_rows = h->ks->n_rows;
  if (n_cols) *n_cols = h->ks->n_cols;
  if (desc && desc_len) {
    std::snprintf(desc, desc_len, "row[%s] col[%s]", h->rk->name, h->ck->name);
  }
  return PAL_OK;
}

int pal_get_occupancy(pal_handle* h, int* row_blocks_per_sm, int* col_blocks_per_sm) {
  if (int rc = check(h)) return rc;
  if (row_blocks_per_sm) *row_blocks_per_sm = h->rk->blocks_per_sm();
  if (col_blocks_per_sm) *col_blocks_per_sm = h->ck->blocks_per_sm();
  return PAL_OK;
}

int pal_set_variant(pal_handle* h, int row, int col) {
  if (int rc = check(h)) return rc;
  if (h->state == ST_P) return fail(h, PAL_ERR_STATE, "change kernels between steps, not between step2b and step3");
  return select_variant(h, row, col);
}

int pal_set_debug(pal_handle* h, int what, int value) {
  if (int rc = check(h)) return rc;
  if (what != PAL_DBG_SKIP_FIRST_WAIT || (value != 0 && value != 1))
    return fail(h, PAL_ERR_INVALID, "unknown debug switch or value");
  h->dbg_wait0 = value;
  for (auto& kv : h->step_graphs) cudaGraphExecDestroy(kv.second);  // they hold the old kernel arguments
  h->step_graphs.clear();
  return PAL_OK;
}

int pal_get_stream(pal_handle* h, void** stream) {
  if (int rc = check(h)) return rc;
  if (!stream) return fail(h, PAL_ERR_INVALID, "stream is null");
  *stream = (void*)h->stream;
  return PAL_OK;
}

int pal_last_error(pal_handle* h, char* buf, size_t n) {
  if (!buf || n == 0) return PAL_ERR_INVALID;
  const std::string& s = h ? h->err : g_err;
  std::strncpy(buf, s.c_str(), n - 1);
  buf[n - 1] = 0;
  return PAL_OK;
}

}  // extern "C"
