// pal_step_noalloc: advance a small FP32 field without allocating any memory.
//
// Who needs this: callers that cannot call cudaMalloc at the point where they
// want to step a field -- for example code running inside a host callback or a
// real-time loop that must not block on the allocator, a plugin whose host
// forbids device allocations after start-up, or a tool that budgets device
// memory up front.  The regular entry points allocate their work planes in
// pal_create; this one instead uses a fixed scratch array that is part of the
// library image itself, so the only memory it touches is that array and the
// caller's own om2/fnm1 buffers.
//
// Limits and sharing rules:
//   - FP32 only, N in {32, 64, 128, 256, 384, 512} (the scratch holds at most
//     N = 512: work planes 3 MiB, om2/fnm1 working copies 2 MiB).
//   - The scratch array (kScratchBytes, 6 MiB) exists once per GPU that loads
//     the library and stays resident until the process exits.
//   - Every call reuses the same scratch and leaves its own data in it; two
//     calls whose GPU work overlaps in time (different streams, or different
//     host threads without ordering) race on it and corrupt each other.
//   - The first call on each device looks up the scratch array's device
//     address (cudaGetSymbolAddress, with that device current); make that
//     first call before any stream capture begins.
//   - Calls are asynchronous on `stream` (null = the legacy default stream);
//     om2/fnm1 hold the result once that stream's work has finished.
//   - Launch errors are read with cudaPeekAtLastError, which leaves the
//     thread's pending CUDA error in place: an error raised earlier by the
//     caller's own code is reported here as PAL_ERR_CUDA but not cleared.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "palgpu.h"
#include "pal_launch.cuh"

namespace {

constexpr size_t kScratchBytes = size_t(6) << 20;
constexpr int kMaxN = 512;
constexpr int kMaxDevices = 64;

// The scratch: scalars | reduction partials | twiddles | om, fnm1 | w0, w1.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr size_t kOffScalars = 0;
constexpr size_t kOffPartials = 256;
constexpr size_t kOffTwiddles = kOffPartials + 64 * 1024;
constexpr size_t kOffFields = kOffTwiddles + 16 * 1024;

std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Scalars for this call; the reduction counters must start at zero.
__global__ void k_noalloc_init(pal::DevScalars* sc, double dt, double visc, double cn, double cnm1) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    pal::DevScalars z = {};
    z.dt = dt;
    z.cn = cn;
    z.cnm1 = cnm1;
    z.visc = visc;
    *sc = z;
  }
}

}  // namespace

extern "C" int pal_step_noalloc(int N, int method, int nsteps, double dt, double visc, double cn, double cnm1,
                                void* om2, void* fnm1, void* stream) {
  if (N > kMaxN || N < 32) return PAL_ERR_INVALID;
  const pal::KernelSet* ks = pal_kernels_f32(N);
  if (!ks) return PAL_ERR_INVALID;
  if (method != PAL_CNAB2 && method != PAL_LS_IMEX_RK3) return PAL_ERR_INVALID;
  if (nsteps < 0 || !om2 || !fnm1 || !(dt > 0.0) || !(visc >= 0.0)) return PAL_ERR_INVALID;
  const int M = 3 * N / 2, Nh = N / 2;
  const size_t plane_om = (size_t)Nh * N * sizeof(float2);
  const size_t plane_w = (size_t)Nh * M * sizeof(float2);
  if (kOffFields + 2 * plane_om + 2 * plane_w > kScratchBytes) return PAL_ERR_INVALID;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PAL_ERR_CUDA;
  unsigned char* base;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return PAL_ERR_CUDA;
      g_scratch_ptr[dev] = p;
    }
    base = static_cast<unsigned char*>(g_scratch_ptr[dev]);
  }
  // For N <= 512 every tile fits the default 48 KB of dynamic shared memory,
  // so no kernel attribute needs setting.
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  pal::StepArgs a = {};
  a.sc = reinterpret_cast<pal::DevScalars*>(base + kOffScalars);
  a.part = reinterpret_cast<double*>(base + kOffPartials);
  a.tw = base + kOffTwiddles;  // row-pass table; the column table follows at +8 KB
  a.om = base + kOffFields;
  a.fnm1 = base + kOffFields + plane_om;
  a.w0 = base + kOffFields + 2 * plane_om;
  a.w1 = base + kOffFields + 2 * plane_om + plane_w;
  a.N = N;

  const pal::RowKernels& rk = ks->rows[0];
  const pal::ColKernels& ck = ks->cols[0];
  const size_t tw_half = (kOffFields - kOffTwiddles) / 2;
  if ((size_t)rk.tw_elems * sizeof(float2) > tw_half || (size_t)ck.tw_elems * sizeof(float2) > tw_half)
    return PAL_ERR_INVALID;
  void* tw_row = base + kOffTwiddles;
  void* tw_col = base + kOffTwiddles + tw_half;
  k_noalloc_init<<<1, 32, 0, s>>>(a.sc, dt, visc, cn, cnm1);
  if (cudaPeekAtLastError() != cudaSuccess) return PAL_ERR_CUDA;
  rk.twiddles(tw_row, s);
  ck.twiddles(tw_col, s);
  ks->transpose(om2, a.om, N, Nh, 1, s);      // caller layout (N, N/2) -> [kx][z]
  ks->transpose(fnm1, a.fnm1, N, Nh, 1, s);
  a.src = nullptr;                             // velocity from the om2 inversion
  a.tw = tw_col;
  ck.col_inv(a, s);
  for (int j = 0; j < nsteps; ++j) {
    if (method == PAL_CNAB2) {
      a.flags = 0;
      a.tw = tw_row;
      rk.row(a, s);
      a.flags = pal::F_CNM1 | pal::F_ADVANCE;
      a.scheme = 0;
      a.tw = tw_col;
      ck.col(a, s);
    } else {
      static const double alpha[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
      static const double beta[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
      for (int st = 0; st < 3; ++st) {
        a.flags = 0;
        a.tw = tw_row;
        rk.row(a, s);
        a.flags = st == 2 ? pal::F_ADVANCE : 0;
        a.scheme = 1;
        a.alpha = alpha[st];
        a.beta = beta[st];
        pal::rk3_stage_flags(a, st, beta);  // the same stage arithmetic as pal_step
        a.tw = tw_col;
        ck.col(a, s);
      }
    }
  }
  ks->transpose(a.om, om2, Nh, N, 1, s);      // back to the caller's layout
  ks->transpose(a.fnm1, fnm1, Nh, N, 1, s);
  return cudaPeekAtLastError() == cudaSuccess ? PAL_OK : PAL_ERR_CUDA;
}
