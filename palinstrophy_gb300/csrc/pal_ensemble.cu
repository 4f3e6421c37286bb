// Batched ensembles: many independent fields (members) with their own N,
// seed, viscosity, CFL target and adaptive dt, advanced together.
//
// Members of equal N form a group whose state lives in one allocation per
// array, member-major.  Each pass is one launch per group (grid.y = members),
// so a step of the whole ensemble is 2 launches per group (CNAB2) or 6
// (LS-IMEX-RK3) regardless of the member count.  Each member keeps its own
// DevScalars: the fused CFL statistics in the row pass update that member's
// dt, cn from its own CFLM, so per-member adaptive dt costs no extra launch
// (in one-launch passes the row pass marks the member's max |u|+|v| and the
// step's column passes form dt, cn from it: no last-block epilogue per row tile).
// When every group's size belongs to a compiled fused set (pal_ens_fused.cu,
// FP32), each pass is instead ONE launch over all groups -- 2 launches per
// CNAB2 step, 6 per LS-IMEX-RK3 step, whatever the number of sizes -- with the
// set's fixed candidates; pal_ensemble_autotune switches to per-size launches
// of candidates re-tuned on each group's batched shape.
// A sequence of steps can be captured once as a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "palgpu.h"
#include "pal_launch.cuh"

namespace {

using pal::DevScalars;
using pal::StepArgs;

constexpr double kRkAlpha[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
constexpr double kRkBeta[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};

struct Group {
  int N = 0, M = 0, Nh = 0;
  const pal::KernelSet* ks = nullptr;
  const pal::RowKernels* rk = nullptr;
  const pal::ColKernels* ck = nullptr;
  std::vector<int> members;  // global member indices, local order
  std::vector<char> has_vel;  // velocity band uploaded for this member
  void *w0 = nullptr, *w1 = nullptr, *om = nullptr, *fnm1 = nullptr, *vel = nullptr;
  void *om_p = nullptr, *fm_p = nullptr;  // butterfly-major om / fnm1 used during pal_ensemble_step
  pal::TmaMaps tmaps{};                   // w0 / w1 descriptors (member dimension = group size)
  pal::TmaMaps cmaps{};                   // the same for a column candidate that moves planes by TMA
  void *tw_row = nullptr, *tw_col = nullptr, *phys = nullptr;
  DevScalars* sc = nullptr;
  double* part = nullptr;
  long long part_stride = 0;
  int slot = -1;  // size index in the fused set, when the ensemble runs fused passes
};

// dt = cflnum / (CFLM pi), cn = 1, cnm1 = 0, t = 0, it = 0 for every member of a group
// (the NEXTDT INIT of turbo_simulator.py:2814-2823, on the device).
__global__ void k_ens_init_dt(DevScalars* sc, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  DevScalars& s = sc[m];
  s.dt = s.cflm > 0.0 ? s.cflnum / (s.cflm * pal::kPi) : 0.0;
  s.cn = 1.0;
  s.cnm1 = 0.0;
  s.t = 0.0;
  s.it = 0;
}

}  // namespace

struct pal_ensemble {
  int precision = 0;
  size_t esz = 8;
  cudaStream_t stream = nullptr;
  std::vector<Group> groups;
  std::vector<std::pair<int, int>> where;  // member -> (group, local)
  std::vector<DevScalars> host_sc;
  std::map<std::string, cudaGraphExec_t> graphs;
  const pal::FusedSet* fused = nullptr;  // one launch per pass over all groups, or per-size launches
  long long it = 0;
  bool ready = false;  // velocities resolved, dt initialised
  bool has_members = false;  // a member has been set (the buffers hold state)
  std::string err;
};

namespace {

thread_local std::string g_ens_err;

int efail(pal_ensemble* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  g_ens_err = msg;
  return code;
}

#define ENS_CK(e, expr)                                                                             \
  do {                                                                                              \
    cudaError_t c_ = (expr);                                                                        \
    if (c_ != cudaSuccess)                                                                          \
      return efail((e), c_ == cudaErrorMemoryAllocation ? PAL_ERR_OOM : PAL_ERR_CUDA,               \
                   std::string(#expr) + ": " + cudaGetErrorString(c_));                             \
  } while (0)

StepArgs group_args(const pal_ensemble* e, const Group& g) {
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.w0 = g.w0;
  a.w1 = g.w1;
  a.om = g.om;
  a.fnm1 = g.fnm1;
  a.tw = g.tw_row;
  a.sc = g.sc;
  a.part = g.part;
  a.phys = g.phys;
  a.om_p = g.om_p;
  a.fm_p = g.fm_p;
  a.tmaps = &g.tmaps;
  a.cmaps = &g.cmaps;
  a.N = g.N;
  a.members = (int)g.members.size();
  a.ms_w = (long long)g.Nh * g.M;
  a.ms_om = (long long)g.Nh * g.N;
  a.ms_part = g.part_stride;
  a.ms_phys = 2LL * g.M * g.M;
  a.ms_src = 2LL * g.N * g.Nh;
  (void)e;
  return a;
}

// om / fnm1 of every group into butterfly-major order (to_perm) or back.
// The group table of a fused pass: `per_member(g)` blocks per member of group g.
template <class PerMember, class ArgsOf>
int fused_args(const pal_ensemble* e, pal::FusedArgs& f, PerMember per_member, ArgsOf args_of) {
  std::memset(&f, 0, sizeof(f));
  f.ngroups = (int)e->groups.size();
  int blocks = 0;
  for (int gi = 0; gi < f.ngroups; ++gi) {
    const Group& g = e->groups[gi];
    f.g[gi].a = args_of(g);
    f.g[gi].slot = g.slot;
    f.g[gi].first = blocks;
    f.g[gi].per_member = per_member(g);
    f.maps[gi] = g.tmaps;
    blocks += f.g[gi].per_member * (int)g.members.size();
  }
  return blocks;
}

int om_layout(pal_ensemble* e, bool to_perm) {
  if (e->fused) {
    pal::FusedArgs f;
    const int nb = fused_args(e, f, [](const Group& g) { return g.Nh; },
                              [&](const Group& g) { return group_args(e, g); });
    (to_perm ? e->fused->to_perm : e->fused->from_perm)(f, nb, e->stream);
    cudaError_t c = cudaGetLastError();
    if (c != cudaSuccess) return efail(e, PAL_ERR_CUDA, std::string("ensemble om order: ") + cudaGetErrorString(c));
    return PAL_OK;
  }
  for (Group& g : e->groups) {
    StepArgs a = group_args(e, g);
    if (to_perm)
      g.ck->to_perm(a, e->stream);
    else
      g.ck->from_perm(a, e->stream);
  }
  cudaError_t c = cudaGetLastError();
  if (c != cudaSuccess) return efail(e, PAL_ERR_CUDA, std::string("ensemble om order: ") + cudaGetErrorString(c));
  return PAL_OK;
}

// One step of every group; the column pass works on the butterfly-major om / fnm1.
int launch_step(pal_ensemble* e, int method, bool dt_update) {
  const int stages = method == PAL_CNAB2 ? 1 : 3;
  for (int s = 0; s < stages; ++s) {
    // one-launch passes (FP32): NEXTDT as a marked max in the row pass, formed
    // by the step's column passes (F_STATS_MAX / F_DT_FROM_MAX); per-size
    // launches: the row pass's own NEXTDT epilogue
    const bool mark = e->fused != nullptr && dt_update;
    auto row_args = [&](const Group& g) {
      StepArgs a = group_args(e, g);
      a.flags = (s == 0 && dt_update) ? (mark ? pal::F_STATS_MAX : (pal::F_STATS | pal::F_UPDATE_DT)) : 0;
      return a;
    };
    auto col_args = [&](const Group& g) {
      StepArgs a = group_args(e, g);
      a.tw = g.tw_col;
      a.scheme = method == PAL_CNAB2 ? 0 : 1;
      if (method != PAL_CNAB2) {
        a.alpha = kRkAlpha[s];
        a.beta = kRkBeta[s];
      }
      a.flags = (s == stages - 1 ? pal::F_ADVANCE : 0) | (method == PAL_CNAB2 ? pal::F_CNM1 : 0) |
                (mark ? pal::F_DT_FROM_MAX : 0);
      if (method != PAL_CNAB2) pal::rk3_stage_flags(a, s, kRkBeta);
      return a;
    };
    if (e->fused) {
      pal::FusedArgs f;
      int nb = fused_args(e, f, [](const Group& g) { return g.M / g.rk->V; }, row_args);
      e->fused->row(f, nb, e->stream);
      nb = fused_args(e, f, [](const Group& g) { return g.Nh; }, col_args);
      const bool qm = (f.g[0].a.flags & (pal::F_Q_IN | pal::F_Q_OUT | pal::F_NO_FM_IN)) != 0;
      e->fused->col(f, nb, qm, e->stream);
      continue;
    }
    for (Group& g : e->groups) g.rk->row(row_args(g), e->stream);
    for (Group& g : e->groups) g.ck->col_perm(col_args(g), e->stream);
  }
  cudaError_t c = cudaGetLastError();
  if (c != cudaSuccess) return efail(e, PAL_ERR_CUDA, std::string("ensemble step launch: ") + cudaGetErrorString(c));
  return PAL_OK;
}

int launch_stats(pal_ensemble* e, int flags) {
  if (e->fused) {
    pal::FusedArgs f;
    const int nb = fused_args(e, f, [](const Group& g) { return g.M / g.rk->V; }, [&](const Group& g) {
      StepArgs a = group_args(e, g);
      a.flags = flags | pal::F_STATS;
      return a;
    });
    e->fused->phys(f, nb, e->stream);
    cudaError_t c = cudaGetLastError();
    if (c != cudaSuccess) return efail(e, PAL_ERR_CUDA, std::string("ensemble stats: ") + cudaGetErrorString(c));
    return PAL_OK;
  }
  for (Group& g : e->groups) {
    StepArgs a = group_args(e, g);
    a.flags = flags | pal::F_STATS;
    g.rk->phys(a, e->stream);
  }
  cudaError_t c = cudaGetLastError();
  if (c != cudaSuccess) return efail(e, PAL_ERR_CUDA, std::string("ensemble stats: ") + cudaGetErrorString(c));
  return PAL_OK;
}

int check_member(pal_ensemble* e, int member) {
  if (!e) return efail(nullptr, PAL_ERR_INVALID, "null ensemble");
  if (member < 0 || member >= (int)e->where.size()) return efail(e, PAL_ERR_INVALID, "member out of range");
  return PAL_OK;
}

}  // namespace

extern "C" {

int pal_ensemble_create(int n_members, const int* N, int precision, double Re, double cfl, pal_ensemble** out) {
  if (!out || !N || n_members <= 0) return efail(nullptr, PAL_ERR_INVALID, "bad arguments");
  *out = nullptr;
  if (precision != PAL_FP32 && precision != PAL_FP64) return efail(nullptr, PAL_ERR_INVALID, "bad precision");
  if (!(Re > 0.0) || !(cfl > 0.0)) return efail(nullptr, PAL_ERR_INVALID, "Re and cfl must be positive");
  pal_ensemble* e = new pal_ensemble();
  e->precision = precision;
  e->esz = precision == PAL_FP32 ? 8 : 16;
  auto bail = [&](int rc) {
    pal_ensemble_destroy(e);
    return rc;
  };
  std::map<int, int> group_of;
  e->where.resize(n_members);
  for (int m = 0; m < n_members; ++m) {
    const pal::KernelSet* ks = precision == PAL_FP32 ? pal_kernels_f32(N[m]) : pal_kernels_f64(N[m]);
    if (!ks) return bail(efail(nullptr, PAL_ERR_INVALID, "unsupported member grid N=" + std::to_string(N[m])));
    auto it = group_of.find(N[m]);
    if (it == group_of.end()) {
      Group g;
      g.N = N[m];
      g.M = 3 * N[m] / 2;
      g.Nh = N[m] / 2;
      g.ks = ks;
      it = group_of.emplace(N[m], (int)e->groups.size()).first;
      e->groups.push_back(g);
    }
    Group& g = e->groups[it->second];
    e->where[m] = {it->second, (int)g.members.size()};
    g.members.push_back(m);
    g.has_vel.push_back(0);
  }
  cudaError_t c = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (c != cudaSuccess) return bail(efail(nullptr, PAL_ERR_CUDA, "cudaStreamCreate"));
  // one launch per pass when a fused set holds every size (PAL_ENSEMBLE_FUSED=0: per-size launches)
  {
    const char* fenv = std::getenv("PAL_ENSEMBLE_FUSED");
    std::vector<int> gN;
    for (const Group& g : e->groups) gN.push_back(g.N);
    if (precision == PAL_FP32 && !(fenv && fenv[0] == '0'))
      e->fused = pal_fused_set_f32((int)gN.size(), gN.data());
    for (Group& g : e->groups) {
      if (!e->fused) break;
      const pal::FusedSet* fs = e->fused;
      g.slot = (int)(std::find(fs->N, fs->N + fs->nsizes, g.N) - fs->N);
      for (int q = 0; q < g.ks->n_rows; ++q)
        if (std::strcmp(g.ks->rows[q].name, fs->row_name[g.slot]) == 0) g.rk = &g.ks->rows[q];
      for (int q = 0; q < g.ks->n_cols; ++q)
        if (std::strcmp(g.ks->cols[q].name, fs->col_name[g.slot]) == 0) g.ck = &g.ks->cols[q];
      if (!g.rk || !g.ck || g.rk->V != fs->V[g.slot]) e->fused = nullptr;  // candidates not compiled: per-size
    }
    if (e->fused && e->fused->configure() != cudaSuccess) e->fused = nullptr;
    if (!e->fused)
      for (Group& g : e->groups) g.rk = nullptr, g.ck = nullptr, g.slot = -1;
  }
  for (Group& g : e->groups) {
    if (!e->fused) {
      // the autotuned candidates of this size (tuned once per process by pal_create)
      pal_handle* tmp = nullptr;
      if (int rc = pal_create(g.N, precision, Re, cfl, &tmp)) return bail(efail(nullptr, rc, "autotune probe failed"));
      int r = 0, cc = 0;
      pal_get_variant(tmp, &r, &cc, nullptr, nullptr, nullptr, 0);
      pal_destroy(tmp);
      g.rk = &g.ks->rows[r];
      g.ck = &g.ks->cols[cc];
    }
    const size_t nm = g.members.size();
    const size_t plane_w = (size_t)g.Nh * g.M * e->esz, plane_om = (size_t)g.Nh * g.N * e->esz;
    g.part_stride = std::max<long long>(2LL * g.M, 5 * 1024);
    void** bufs[] = {&g.w0, &g.w1, &g.om, &g.fnm1, &g.vel, &g.tw_row, &g.tw_col, &g.om_p};
    size_t tw_row_max = 0, tw_col_max = 0;  // room for any candidate's tables (pal_ensemble_autotune)
    for (int q = 0; q < g.ks->n_rows; ++q) tw_row_max = std::max(tw_row_max, (size_t)g.ks->rows[q].tw_elems);
    for (int q = 0; q < g.ks->n_cols; ++q) tw_col_max = std::max(tw_col_max, (size_t)g.ks->cols[q].tw_elems);
    const size_t sizes[] = {nm * plane_w + pal::kPlaneSlack, nm * plane_w + pal::kPlaneSlack, nm * plane_om, nm * plane_om, 2 * nm * plane_om,
                            tw_row_max * e->esz, tw_col_max * e->esz, 2 * nm * plane_w};
    for (int i = 0; i < 8; ++i) {
      c = cudaMalloc(bufs[i], sizes[i]);
      if (c == cudaSuccess) c = cudaMemsetAsync(*bufs[i], 0, sizes[i], e->stream);
      if (c != cudaSuccess) return bail(efail(nullptr, c == cudaErrorMemoryAllocation ? PAL_ERR_OOM : PAL_ERR_CUDA,
                                              std::string("ensemble alloc: ") + cudaGetErrorString(c)));
    }
    g.fm_p = static_cast<char*>(g.om_p) + nm * plane_w;
    if (g.rk->tma && !pal::encode_row_maps(&g.tmaps, g.w0, g.w1, g.N, g.rk->V, (int)nm))
      return bail(efail(nullptr, PAL_ERR_CUDA, "ensemble TMA descriptors"));
    if (g.ck->tma && !pal::encode_col_maps(&g.cmaps, g.w0, g.w1, g.N, g.ck->rp, (int)nm))
      return bail(efail(nullptr, PAL_ERR_CUDA, "ensemble TMA descriptors (columns)"));
    c = cudaMalloc(&g.sc, nm * sizeof(DevScalars));
    if (c == cudaSuccess) c = cudaMalloc(&g.part, nm * g.part_stride * sizeof(double));
    if (c != cudaSuccess) return bail(efail(nullptr, PAL_ERR_OOM, "ensemble scalars"));
    std::vector<DevScalars> hs(nm);
    for (auto& s : hs) {
      std::memset(&s, 0, sizeof(s));
      s.cn = 1.0;
      s.visc = (double)(float)(1.0 / (double)(float)Re);
      s.cflnum = cfl;
    }
    c = cudaMemcpyAsync(g.sc, hs.data(), nm * sizeof(DevScalars), cudaMemcpyHostToDevice, e->stream);
    if (c == cudaSuccess) {
      if (g.rk->configure() != cudaSuccess || g.ck->configure() != cudaSuccess) c = cudaErrorInvalidValue;
    }
    if (c == cudaSuccess) {
      g.rk->twiddles(g.tw_row, e->stream);
      g.ck->twiddles(g.tw_col, e->stream);
      c = cudaGetLastError();
    }
    if (c != cudaSuccess) return bail(efail(nullptr, PAL_ERR_CUDA, "ensemble setup"));
  }
  c = cudaStreamSynchronize(e->stream);
  if (c != cudaSuccess) return bail(efail(nullptr, PAL_ERR_CUDA, "ensemble setup sync"));
  e->host_sc.resize(n_members);
  *out = e;
  return PAL_OK;
}

int pal_ensemble_destroy(pal_ensemble* e) {
  if (!e) return PAL_OK;
  if (e->stream) cudaStreamSynchronize(e->stream);
  for (auto& kv : e->graphs) cudaGraphExecDestroy(kv.second);
  for (Group& g : e->groups) {
    void* bufs[] = {g.w0, g.w1, g.om, g.fnm1, g.vel, g.tw_row, g.tw_col, g.phys, g.sc, g.part, g.om_p};
    for (void* b : bufs)
      if (b) cudaFree(b);
  }
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return PAL_OK;
}

int pal_ensemble_set_member(pal_ensemble* e, int member, const void* om2, const void* fnm1, const void* uc_low) {
  if (int rc = check_member(e, member)) return rc;
  if (!om2) return efail(e, PAL_ERR_INVALID, "om2 is null");
  Group& g = e->groups[e->where[member].first];
  const int loc = e->where[member].second;
  const size_t plane_om = (size_t)g.Nh * g.N * e->esz;
  char* vel = static_cast<char*>(g.vel) + 2 * plane_om * loc;
  // stage om2 / fnm1 in the velocity slot, transpose into the [kx][z] state
  ENS_CK(e, cudaMemcpyAsync(vel, om2, plane_om, cudaMemcpyHostToDevice, e->stream));
  g.ks->transpose(vel, static_cast<char*>(g.om) + plane_om * loc, g.N, g.Nh, 1, e->stream);
  if (fnm1) {
    ENS_CK(e, cudaMemcpyAsync(vel, fnm1, plane_om, cudaMemcpyHostToDevice, e->stream));
    g.ks->transpose(vel, static_cast<char*>(g.fnm1) + plane_om * loc, g.N, g.Nh, 1, e->stream);
  } else {
    ENS_CK(e, cudaMemsetAsync(static_cast<char*>(g.fnm1) + plane_om * loc, 0, plane_om, e->stream));
  }
  if (uc_low) {
    ENS_CK(e, cudaMemcpyAsync(vel, uc_low, 2 * plane_om, cudaMemcpyHostToDevice, e->stream));
  } else {
    ENS_CK(e, cudaMemsetAsync(vel, 0, 2 * plane_om, e->stream));
  }
  g.has_vel[loc] = uc_low != nullptr;
  ENS_CK(e, cudaStreamSynchronize(e->stream));
  e->ready = false;
  e->has_members = true;
  return PAL_OK;
}

// Time every row and column candidate on each group's batched launch shape
// (grid.y = members) and keep the fastest; the buffers still hold zeros, so
// the timing launches disturb no state.  Without it the groups use the
// candidates pal_create tuned for a single field of the same size, which
// keeps ensemble members bit-identical to single fields.
int pal_ensemble_autotune(pal_ensemble* e) {
  if (!e) return efail(nullptr, PAL_ERR_INVALID, "null ensemble");
  if (e->has_members) return efail(e, PAL_ERR_STATE, "autotune before setting members");
  const char* env = std::getenv("PAL_AUTOTUNE");
  if (env && env[0] == '0') return PAL_OK;
  e->fused = nullptr;  // re-tuned candidates run as per-size launches
  for (Group& g : e->groups) g.slot = -1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ENS_CK(e, cudaEventCreate(&e0));
  ENS_CK(e, cudaEventCreate(&e1));
  auto time_it = [&](auto&& launch) -> float {
    launch();  // warm-up
    cudaEventRecord(e0, e->stream);
    for (int q = 0; q < 3; ++q) launch();
    cudaEventRecord(e1, e->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
  };
  int rc = PAL_OK;
  for (Group& g : e->groups) {
    const int nm = (int)g.members.size();
    float best = 1e30f;
    const pal::RowKernels* best_r = g.rk;
    for (int q = 0; q < g.ks->n_rows && rc == PAL_OK; ++q) {
      const pal::RowKernels* rk = &g.ks->rows[q];
      if (rk->multicast && !pal::tma_multicast_allowed()) continue;
      if (rk->configure() != cudaSuccess) continue;
      if (rk->tma && !pal::encode_row_maps(&g.tmaps, g.w0, g.w1, g.N, rk->V, nm)) continue;
      rk->twiddles(g.tw_row, e->stream);
      StepArgs a = group_args(e, g);
      const float ms = time_it([&]() { rk->row(a, e->stream); });
      if (cudaGetLastError() != cudaSuccess) rc = efail(e, PAL_ERR_CUDA, "ensemble autotune (row)");
      if (ms < best) {
        best = ms;
        best_r = rk;
      }
    }
    best = 1e30f;
    const pal::ColKernels* best_c = g.ck;
    for (int q = 0; q < g.ks->n_cols && rc == PAL_OK; ++q) {
      const pal::ColKernels* ck = &g.ks->cols[q];
      if (ck->configure() != cudaSuccess) continue;
      if (ck->tma && !pal::encode_col_maps(&g.cmaps, g.w0, g.w1, g.N, ck->rp, nm)) continue;
      ck->twiddles(g.tw_col, e->stream);
      StepArgs a = group_args(e, g);
      a.tw = g.tw_col;
      a.scheme = 0;
      const float ms = time_it([&]() { ck->col_perm(a, e->stream); });
      if (cudaGetLastError() != cudaSuccess) rc = efail(e, PAL_ERR_CUDA, "ensemble autotune (column)");
      if (ms < best) {
        best = ms;
        best_c = ck;
      }
    }
    if (rc != PAL_OK) break;
    g.rk = best_r;
    g.ck = best_c;
    if (g.rk->tma && !pal::encode_row_maps(&g.tmaps, g.w0, g.w1, g.N, g.rk->V, nm)) {
      rc = efail(e, PAL_ERR_CUDA, "ensemble TMA descriptors");
      break;
    }
    if (g.ck->tma && !pal::encode_col_maps(&g.cmaps, g.w0, g.w1, g.N, g.ck->rp, nm)) {
      rc = efail(e, PAL_ERR_CUDA, "ensemble TMA descriptors (columns)");
      break;
    }
    g.rk->twiddles(g.tw_row, e->stream);
    g.ck->twiddles(g.tw_col, e->stream);
    const size_t plane_w = (size_t)g.Nh * g.M * e->esz, plane_om = (size_t)g.Nh * g.N * e->esz;
    cudaMemsetAsync(g.w0, 0, nm * plane_w, e->stream);
    cudaMemsetAsync(g.w1, 0, nm * plane_w, e->stream);
    cudaMemsetAsync(g.om, 0, nm * plane_om, e->stream);
    cudaMemsetAsync(g.fnm1, 0, nm * plane_om, e->stream);
    cudaMemsetAsync(g.om_p, 0, 2 * nm * plane_w, e->stream);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (auto& kv : e->graphs) cudaGraphExecDestroy(kv.second);
  e->graphs.clear();
  if (rc != PAL_OK) return rc;
  ENS_CK(e, cudaStreamSynchronize(e->stream));
  return PAL_OK;
}

int pal_ensemble_get_variant(pal_ensemble* e, int group_N, char* desc, size_t desc_len) {
  if (!e || !desc || !desc_len) return efail(e, PAL_ERR_INVALID, "bad arguments");
  for (const Group& g : e->groups) {
    if (g.N == group_N) {
      std::snprintf(desc, desc_len, "%srow[%s] col[%s]", e->fused ? "fused " : "", g.rk->name, g.ck->name);
      return PAL_OK;
    }
  }
  return efail(e, PAL_ERR_INVALID, "no group of that size");
}

int pal_ensemble_set_scalar(pal_ensemble* e, int member, int which, double value) {
  if (!e) return efail(nullptr, PAL_ERR_INVALID, "null ensemble");
  size_t off;
  switch (which) {
    case PAL_SC_T: off = offsetof(DevScalars, t); break;
    case PAL_SC_DT: off = offsetof(DevScalars, dt); break;
    case PAL_SC_CN: off = offsetof(DevScalars, cn); break;
    case PAL_SC_CNM1: off = offsetof(DevScalars, cnm1); break;
    case PAL_SC_VISC: off = offsetof(DevScalars, visc); break;
    case PAL_SC_CFLNUM: off = offsetof(DevScalars, cflnum); break;
    default: return efail(e, PAL_ERR_INVALID, "unknown scalar");
  }
  const int lo = member < 0 ? 0 : member, hi = member < 0 ? (int)e->where.size() : member + 1;
  if (member >= (int)e->where.size()) return efail(e, PAL_ERR_INVALID, "member out of range");
  for (int m = lo; m < hi; ++m) {
    Group& g = e->groups[e->where[m].first];
    char* dst = reinterpret_cast<char*>(g.sc + e->where[m].second) + off;
    ENS_CK(e, cudaMemcpyAsync(dst, &value, sizeof(double), cudaMemcpyHostToDevice, e->stream));
  }
  ENS_CK(e, cudaStreamSynchronize(e->stream));
  return PAL_OK;
}

int pal_ensemble_init_dt(pal_ensemble* e) {
  if (!e) return efail(nullptr, PAL_ERR_INVALID, "null ensemble");
  for (Group& g : e->groups) {
    StepArgs a = group_args(e, g);
    a.tw = g.tw_col;
    // the uploaded velocity bands when every member has one, else the
    // velocity of every member rebuilt from its om2
    const bool all_vel = std::all_of(g.has_vel.begin(), g.has_vel.end(), [](char c) { return c != 0; });
    a.src = all_vel ? g.vel : nullptr;
    g.ck->col_inv(a, e->stream);
  }
  if (int rc = launch_stats(e, 0)) return rc;
  for (Group& g : e->groups) {
    const int n = (int)g.members.size();
    k_ens_init_dt<<<(n + 127) / 128, 128, 0, e->stream>>>(g.sc, n);
  }
  ENS_CK(e, cudaGetLastError());
  ENS_CK(e, cudaStreamSynchronize(e->stream));
  e->it = 0;
  e->ready = true;
  return PAL_OK;
}

int pal_ensemble_step(pal_ensemble* e, int method, int nsteps, int update, int use_graph) {
  if (!e) return efail(nullptr, PAL_ERR_INVALID, "null ensemble");
  if (!e->ready) return efail(e, PAL_ERR_STATE, "call pal_ensemble_init_dt after setting the members");
  if (method != PAL_CNAB2 && method != PAL_LS_IMEX_RK3) return efail(e, PAL_ERR_INVALID, "unknown time stepper");
  if (nsteps <= 0) return PAL_OK;
  // NEXTDT after step `it` when update > 0 and (it % update == 0 || it == 1); it is
  // fused into the next step's row pass, or run at the end of the call.
  std::string key = std::to_string(method) + ":";
  std::vector<bool> upd(nsteps + 1, false);  // upd[j]: fused update at the start of step j
  bool pending = false;
  for (int j = 0; j < nsteps; ++j) {
    upd[j] = pending;
    const long long it = e->it + j + 1;
    pending = update > 0 && (it % update == 0 || it == 1);
  }
  upd[nsteps] = pending;
  for (bool b : upd) key += b ? '1' : '0';
  auto record = [&]() -> int {
    if (int rc = om_layout(e, true)) return rc;
    for (int j = 0; j < nsteps; ++j)
      if (int rc = launch_step(e, method, upd[j])) return rc;
    if (int rc = om_layout(e, false)) return rc;
    if (upd[nsteps])
      if (int rc = launch_stats(e, pal::F_UPDATE_DT)) return rc;
    return PAL_OK;
  };
  if (!use_graph) {
    if (int rc = record()) return rc;
  } else {
    auto it = e->graphs.find(key);
    if (it == e->graphs.end()) {
      cudaGraph_t graph = nullptr;
      ENS_CK(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
      int rc = record();
      cudaError_t c = cudaStreamEndCapture(e->stream, &graph);
      if (rc) return rc;
      if (c != cudaSuccess) return efail(e, PAL_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(c));
      cudaGraphExec_t exec = nullptr;
      c = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (c != cudaSuccess) return efail(e, PAL_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(c));
      it = e->graphs.emplace(key, exec).first;
    }
    ENS_CK(e, cudaGraphLaunch(it->second, e->stream));
  }
  e->it += nsteps;
  return PAL_OK;
}

int pal_ensemble_get_member(pal_ensemble* e, int member, int which, void* host_dst) {
  if (int rc = check_member(e, member)) return rc;
  if (!host_dst) return efail(e, PAL_ERR_INVALID, "host_dst is null");
  if (which != PAL_FIELD_OM2 && which != PAL_FIELD_FNM1) return efail(e, PAL_ERR_INVALID, "om2 or fnm1 only");
  Group& g = e->groups[e->where[member].first];
  const int loc = e->where[member].second;
  const size_t plane_om = (size_t)g.Nh * g.N * e->esz;
  const char* src = static_cast<const char*>(which == PAL_FIELD_OM2 ? g.om : g.fnm1) + plane_om * loc;
  char* stage = static_cast<char*>(g.vel) + 2 * plane_om * loc;  // free after init
  g.ks->transpose(src, stage, g.Nh, g.N, 1, e->stream);
  ENS_CK(e, cudaGetLastError());
  ENS_CK(e, cudaMemcpyAsync(host_dst, stage, plane_om, cudaMemcpyDeviceToHost, e->stream));
  ENS_CK(e, cudaStreamSynchronize(e->stream));
  return PAL_OK;
}

int pal_ensemble_get_scalars(pal_ensemble* e, int member, double* t, double* dt, double* cn, double* cflm,
                             long long* it) {
  if (int rc = check_member(e, member)) return rc;
  Group& g = e->groups[e->where[member].first];
  DevScalars s;
  ENS_CK(e, cudaMemcpyAsync(&s, g.sc + e->where[member].second, sizeof(s), cudaMemcpyDeviceToHost, e->stream));
  ENS_CK(e, cudaStreamSynchronize(e->stream));
  if (t) *t = s.t;
  if (dt) *dt = s.dt;
  if (cn) *cn = s.cn;
  if (cflm) *cflm = s.cflm;
  if (it) *it = s.it;
  return PAL_OK;
}

int pal_ensemble_get_stream(pal_ensemble* e, void** stream) {
  if (!e || !stream) return efail(e, PAL_ERR_INVALID, "bad arguments");
  *stream = (void*)e->stream;
  return PAL_OK;
}

int pal_ensemble_synchronize(pal_ensemble* e) {
  if (!e) return efail(nullptr, PAL_ERR_INVALID, "null ensemble");
  ENS_CK(e, cudaStreamSynchronize(e->stream));
  return PAL_OK;
}

int pal_ensemble_last_error(pal_ensemble* e, char* buf, size_t n) {
  if (!buf || n == 0) return PAL_ERR_INVALID;
  const std::string& s = e ? e->err : g_ens_err;
  std::strncpy(buf, s.c_str(), n - 1);
  buf[n - 1] = 0;
  return PAL_OK;
}

}  // extern "C"
