// PAO / KM3 initial condition with the mode arithmetic on the device.
//
// The reference generator (palinstrophy/turbo_simulator.py) draws one number
// per mode from a Fortran-style LCG with a 97-entry shuffle table
// (241-261, 274-286); the table makes the draw order serial, so the host runs
// that loop and hands the per-mode uniforms to the device.  Everything else is
// per mode or per shell and runs here:
//   PAO amplitudes and phases, |u|^2 ~ exp(-(k/K0)^2)/(pi K0^2) ... 287-318
//   zero (0,0), Hermitian kx = 0 column, zero row z = N/2 ......... 320-334
//   KM3 shell energies and weights, rescale with the hash jitter .. 195-204, 336-427
//   moments -> Energy, WiWi ........................................ 432-470
//   om2 = i (gamma u1 - alfa u3) .................................... 1314-1361
// The float32 steps use explicitly rounded operations (no fused multiply-add),
// as NumPy evaluates them; float32 exp/sin/cos and double sin/cos come from
// CUDA's math library, so values can differ from the reference's in the last
// bit, as the host restatement's do.  Shell sums are reduced in a fixed order
// (one block per shell), so the result does not depend on scheduling.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "palgpu.h"
#include "pal_kernels.cuh"

namespace {

constexpr int64_t kImm = 420029, kIt = 2017, kId = 5011;
constexpr int kGenThreads = 256;

__device__ __forceinline__ double hash01(int x, int z, int seed, int salt) {
  double a = __dadd_rn(__dmul_rn((double)x + 1.0, 12.9898), __dmul_rn((double)z + 1.0, 78.233));
  a = __dadd_rn(a, __dmul_rn((double)seed + 1.0, 0.010001));
  a = __dadd_rn(a, __dmul_rn((double)salt + 1.0, 37.719));
  const double s = __dmul_rn(sin(a), 43758.5453123);
  return s - floor(s);
}

__device__ __forceinline__ float2 scale(float a, float2 p) { return make_float2(__fmul_rn(a, p.x), __fmul_rn(a, p.y)); }

// kz of row z as the generator's table holds it: the row z = N/2 is -N/2
// (turbo_simulator.py:1091-1094 writes +N/2 and then overwrites it).
__device__ __forceinline__ float gamma_of(int z, int N) {
  const int nh = N / 2;
  return z < nh ? (float)z : (float)(z - N);
}

// PAO modes from the per-mode uniforms v[z * nh + x]; U planes [c][z][x].
__global__ void k_gen_pao(const float* __restrict__ v, int N, float K0, int km3, float2* __restrict__ U) {
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  const float PI = 3.14159265358979f;
  const float norm = __fmul_rn(__fmul_rn(PI, K0), K0);
  const float floor2 = 1.0e-40f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(i / nh), x = (int)(i % nh);
    const float th = __fmul_rn(__fmul_rn(2.0f, PI), v[i]);
    const float2 ph = make_float2(cosf(th), sinf(th));
    const float ax = (float)x, gz = gamma_of(z, N);
    const float k2 = __fadd_rn(__fmul_rn(ax, ax), __fmul_rn(gz, gz));
    const float k = k2 > 0.0f ? __fsqrt_rn(k2) : 0.0f;
    const float t = __fdiv_rn(k, K0);
    const float g = -__fmul_rn(t, t);
    float2 u0, u1;
    if (x == 0) {
      float e2 = __fdiv_rn(expf(g), norm);
      if (km3 && e2 < floor2) e2 = floor2;
      u1 = make_float2(0.f, 0.f);
      u0 = scale(__fsqrt_rn(e2), ph);
    } else {
      const float den = __fadd_rn(1.0f, __fdiv_rn(__fmul_rn(gz, gz), __fmul_rn(ax, ax)));
      float e2 = __fdiv_rn(expf(g), __fmul_rn(den, norm));
      if (km3 && e2 < floor2) e2 = floor2;
      const float2 w = scale(__fsqrt_rn(e2), ph);
      u1 = w;
      u0 = scale(-__fdiv_rn(gz, ax), w);
    }
    U[i] = u0;
    U[plane + i] = u1;
  }
}

// zero (0,0), mirror the kx = 0 column, zero the row z = N/2.
__global__ void k_gen_fix(int N, float2* __restrict__ U) {
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    U[0] = U[plane] = make_float2(0.f, 0.f);
  }
  if (t >= 1 && t < nh) {
    const float2 a = U[(size_t)t * nh], b = U[plane + (size_t)t * nh];
    U[(size_t)(N - t) * nh] = make_float2(a.x, -a.y);
    U[plane + (size_t)(N - t) * nh] = make_float2(b.x, -b.y);
  }
}
__global__ void k_gen_zero_row(int N, float2* __restrict__ U) {
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x < nh) U[(size_t)nh * nh + x] = U[plane + (size_t)nh * nh + x] = make_float2(0.f, 0.f);
}

// Visit the modes of shell sh (round(k) == sh, 0 < k <= N/2): threads take kx,
// each kx has at most a few |kz| in the shell; both signs of kz.
template <class F>
__device__ __forceinline__ void for_shell(int sh, int N, F&& f) {
  const int nh = N / 2;
  const double knyq = (double)nh;
  const int xmax = min(nh - 1, sh + 1);
  for (int x = threadIdx.x; x <= xmax; x += blockDim.x) {
    const double lo = (sh - 0.5) * (sh - 0.5) - (double)x * x, hi = (sh + 0.5) * (sh + 0.5) - (double)x * x;
    if (hi < 0.0) continue;
    int g0 = lo > 0.0 ? (int)floor(sqrt(lo)) - 1 : 0;
    int g1 = (int)ceil(sqrt(hi)) + 1;
    g0 = max(g0, 0);
    g1 = min(g1, nh);
    for (int g = g0; g <= g1; ++g) {
      for (int sgn = 0; sgn < 2; ++sgn) {
        if (sgn == 1 && (g == 0 || g == nh)) continue;  // kz = -N/2 does not exist; kz = 0 once
        const int z = sgn == 0 ? g : N - g;
        const double gz = sgn == 0 ? (double)g : -(double)g;
        const double k = sqrt((double)x * x + gz * gz);
        const int s = (int)(k + 0.5);
        if (k > 0.0 && k <= knyq && s == sh) f(x, z);
      }
    }
  }
}

// e_shell[sh] = sum m (|u1|^2 + |u3|^2), w_shell[sh] = sum m (0.75 + 0.5 hash), one block per shell.
__global__ void __launch_bounds__(kGenThreads) k_gen_shells(const float2* __restrict__ U, int N, int seed,
                                                             double* __restrict__ e_shell,
                                                             double* __restrict__ w_shell) {
  const int sh = blockIdx.x + 1;
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  double e = 0.0, w = 0.0;
  for_shell(sh, N, [&](int x, int z) {
    const float2 a = U[(size_t)z * nh + x], b = U[plane + (size_t)z * nh + x];
    const double p1 = (double)a.x * a.x + (double)a.y * a.y;
    const double p3 = (double)b.x * b.x + (double)b.y * b.y;
    const double m = x == 0 ? 1.0 : 2.0;
    e += m * (p1 + p3);
    const int zh = (x == 0 && z > nh) ? N - z : z;
    w += m * (0.75 + 0.50 * hash01(x, zh, seed, 17));
  });
  __shared__ double red[2 * (kGenThreads / 32)];
  double vals[2] = {e, w};
  pal::block_sum<kGenThreads, 2>(vals, red, threadIdx.x);
  if (threadIdx.x == 0) {
    e_shell[sh] = vals[0];
    w_shell[sh] = vals[1];
  }
}

// KM3 rescale: every mode of a non-empty shell gets the shell's target energy
// spread with the hash jitter and a hash phase; other modes are zeroed.
__global__ void k_gen_km3(float2* __restrict__ U, int N, int seed, const double* __restrict__ st,
                          const double* __restrict__ w_shell) {
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  const double knyq = (double)nh;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(i / nh), x = (int)(i % nh);
    const double ax = (double)x, ax2 = ax * ax;
    const double gz = (double)gamma_of(z, N), gz2 = gz * gz;
    const double k = sqrt(ax2 + gz2);
    const int sh = (int)(k + 0.5);
    float2 u0 = make_float2(0.f, 0.f), u1 = make_float2(0.f, 0.f);
    if (k > 0.0 && k <= knyq && sh <= nh && w_shell[sh] > 0.0) {
      int zh = z;
      double sign = 1.0;
      if (x == 0 && z > nh) {
        zh = N - z;
        sign = -1.0;
      }
      const double jit = 0.75 + 0.50 * hash01(x, zh, seed, 17);
      const double e_mode = __ddiv_rn(__dmul_rn(st[sh], jit), w_shell[sh]);
      const double th = sign * 2.0 * 3.141592653589793 * hash01(x, zh, seed, 53);
      const float2 ph = make_float2((float)cos(th), (float)sin(th));
      if (x == 0) {
        u0 = scale((float)sqrt(e_mode), ph);
      } else {
        const float2 w = scale((float)sqrt(__ddiv_rn(e_mode, 1.0 + __ddiv_rn(gz2, ax2))), ph);
        u0 = scale((float)(-gz / ax), w);
        u1 = w;
      }
    }
    U[i] = u0;
    U[plane + i] = u1;
  }
}

// Moments A1..A6 per block (fixed tree order); folded on the host in block order.
__global__ void __launch_bounds__(kGenThreads) k_gen_moments(const float2* __restrict__ U, int N,
                                                              double* __restrict__ part) {
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (size_t i = blockIdx.x * (size_t)kGenThreads + threadIdx.x; i < plane; i += (size_t)gridDim.x * kGenThreads) {
    const int z = (int)(i / nh), x = (int)(i % nh);
    const float2 u1 = U[i], u3 = U[plane + i];
    const double p1 = (double)u1.x * u1.x + (double)u1.y * u1.y;
    const double p3 = (double)u3.x * u3.x + (double)u3.y * u3.y;
    const double ax2 = (double)x * x;
    const double g = (double)gamma_of(z, N), gz2 = g * g;
    const double m = x == 0 ? 1.0 : 2.0;
    a[0] += m * p1;
    a[1] += m * p3;
    a[2] += m * p1 * ax2;
    a[3] += m * p1 * gz2;
    a[4] += m * p3 * ax2;
    a[5] += m * p3 * gz2;
  }
  __shared__ double red[6 * (kGenThreads / 32)];
  pal::block_sum<kGenThreads, 6>(a, red, threadIdx.x);
  if (threadIdx.x == 0)
    for (int q = 0; q < 6; ++q) part[(size_t)blockIdx.x * 6 + q] = a[q];
}

// om (device layout [kx][z]) = i (gamma u1 - alfa u3); velocity band (2, N, N/2).
template <typename T>
__global__ void k_gen_out(const float2* __restrict__ U, int N, pal::cplx<T>* __restrict__ om,
                          pal::cplx<T>* __restrict__ uc) {
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
    const int z = (int)(i / nh), x = (int)(i % nh);
    const float2 u1 = U[i], u3 = U[plane + i];
    const float g = gamma_of(z, N), a = (float)x;
    const float dre = __fsub_rn(__fmul_rn(g, u1.x), __fmul_rn(a, u3.x));
    const float dim = __fsub_rn(__fmul_rn(g, u1.y), __fmul_rn(a, u3.y));
    om[(size_t)x * N + z] = pal::cplx<T>{T(-dim), T(dre)};
    uc[i] = pal::cplx<T>{T(u1.x), T(u1.y)};
    uc[plane + i] = pal::cplx<T>{T(u3.x), T(u3.y)};
  }
}

}  // namespace

// Device generator behind pal_generate (pal_api.cu): writes om (device layout)
// and the velocity band (reference layout) of precision T = float / double.
int pal_generate_device(int N, int precision, double K0d, double Re, int seed_init, int spectrum, void* om_dev,
                        void* uc_dev, cudaStream_t s, double* stats, int* seed_out, std::string* err) {
  auto cuda_err = [&](cudaError_t e, const char* what) {
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PAL_ERR_OOM : PAL_ERR_CUDA;
  };
  const bool km3 = spectrum == PAL_SPEC_KM3;
  const int nh = N / 2;
  const size_t plane = (size_t)N * nh;
  // the serial part: LCG draws with the 97-entry shuffle, in the reference's mode order
  std::vector<float> v(plane);
  int64_t sd = seed_init;
  for (int i = 0; i < 97; ++i) sd = (sd * kImm + kIt) % kId;
  float table[97];
  for (int i = 0; i < 97; ++i) {
    sd = (sd * kImm + kIt) % kId;
    table[i] = (float)sd / (float)kId;
  }
  for (size_t i = 0; i < plane; ++i) {
    sd = (sd * kImm + kIt) % kId;
    const float r = (float)sd / (float)kId;
    int idx = (int)((double)r * 97.0);
    idx = idx < 0 ? 0 : (idx > 96 ? 96 : idx);
    v[i] = table[idx];
    table[idx] = r;
  }
  if (seed_out) *seed_out = (int)sd;

  float* d_v = nullptr;
  float2* d_U = nullptr;
  double* d_aux = nullptr;  // e_shell | w_shell | st | moment partials
  const int gen_blocks = 4 * 152;
  const size_t aux_n = 3 * (size_t)(nh + 1) + 6 * (size_t)gen_blocks;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d_v), plane * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&d_U), 2 * plane * sizeof(float2), s);
  if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&d_aux), aux_n * sizeof(double), s);
  auto release = [&]() {
    if (d_v) cudaFreeAsync(d_v, s);
    if (d_U) cudaFreeAsync(d_U, s);
    if (d_aux) cudaFreeAsync(d_aux, s);
  };
  if (e != cudaSuccess) {
    release();
    return cuda_err(e, "generator buffers");
  }
  double* d_e = d_aux;
  double* d_w = d_e + (nh + 1);
  double* d_st = d_w + (nh + 1);
  double* d_part = d_st + (nh + 1);
  e = cudaMemcpyAsync(d_v, v.data(), plane * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_aux, 0, aux_n * sizeof(double), s);
  if (e != cudaSuccess) {
    release();
    return cuda_err(e, "generator upload");
  }
  k_gen_pao<<<gen_blocks, kGenThreads, 0, s>>>(d_v, N, (float)K0d, km3 ? 1 : 0, d_U);
  k_gen_fix<<<(nh + 255) / 256, 256, 0, s>>>(N, d_U);
  k_gen_zero_row<<<(nh + 255) / 256, 256, 0, s>>>(N, d_U);
  if (km3) {
    k_gen_shells<<<nh, kGenThreads, 0, s>>>(d_U, N, seed_init, d_e, d_w);
    std::vector<double> hbuf(2 * (size_t)(nh + 1));
    e = cudaMemcpyAsync(hbuf.data(), d_e, hbuf.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      release();
      return cuda_err(e, "generator shells");
    }
    const double* e_shell = hbuf.data();
    const double* w_shell = hbuf.data() + (nh + 1);
    double k0 = K0d < 1.0 ? 1.0 : K0d;
    std::vector<double> target(nh + 1, 0.0), st(nh + 1, 0.0);
    for (int sh = 1; sh <= nh; ++sh) {
      const double k = (double)sh;
      if (k < k0) {
        const double lo = k / k0;
        target[sh] = (lo * lo * lo * lo) / (k0 * k0 * k0);
      } else {
        target[sh] = 1.0 / (k * k * k);
      }
    }
    double e_orig = 0.0, e_target = 0.0;
    for (int sh = 1; sh <= nh; ++sh) {
      e_orig += e_shell[sh];
      e_target += target[sh];
    }
    if (e_orig > 0.0 && e_target > 0.0) {
      const double scl = e_orig / e_target;
      for (int sh = 1; sh <= nh; ++sh) st[sh] = scl * target[sh];
      e = cudaMemcpyAsync(d_st, st.data(), (nh + 1) * sizeof(double), cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) {
        release();
        return cuda_err(e, "generator targets");
      }
      k_gen_km3<<<gen_blocks, kGenThreads, 0, s>>>(d_U, N, seed_init, d_st, d_w);
    }
  }
  k_gen_moments<<<gen_blocks, kGenThreads, 0, s>>>(d_U, N, d_part);
  if (precision == PAL_FP32)
    k_gen_out<float><<<gen_blocks, kGenThreads, 0, s>>>(d_U, N, static_cast<pal::cplx<float>*>(om_dev),
                                                         static_cast<pal::cplx<float>*>(uc_dev));
  else
    k_gen_out<double><<<gen_blocks, kGenThreads, 0, s>>>(d_U, N, static_cast<pal::cplx<double>*>(om_dev),
                                                          static_cast<pal::cplx<double>*>(uc_dev));
  e = cudaGetLastError();
  std::vector<double> part(6 * (size_t)gen_blocks);
  if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  release();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_err(e, "generator kernels");
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (int b = 0; b < gen_blocks; ++b)
    for (int q = 0; q < 6; ++q) a[q] += part[(size_t)b * 6 + q];
  if (stats) {
    stats[0] = a[0] + a[1];
    stats[1] = a[2] + a[3] + a[4] + a[5];
    stats[2] = (double)(float)(1.0 / (double)(float)Re);
  }
  return PAL_OK;
}
