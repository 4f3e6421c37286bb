// Host-side PAO / KM3 initial condition of the palinstrophy DNS.
//
// Follows the reference generator (palinstrophy/turbo_simulator.py):
//   Fortran LCG + 97-entry shuffle table ............ 241-261, 274-286
//   PAO modes |u|^2 ~ exp(-(k/K0)^2)/(pi K0^2) ....... 287-318
//   zero (0,0), Hermitian kx=0 column, zero z=N/2 ... 320-334
//   KM3 shell rescale with the sin-hash jitter ...... 195-204, 336-427
//   moments A1..A7 -> Energy, WiWi; visc=f32(1/Re) .. 432-470
//   om2 = i (gamma u1 - alfa u3) (dnsCudaCalcom) .... 1314-1361
// The reference evaluates the PAO part with NumPy float32 scalars; it is kept
// in float here (compile with -ffp-contract=off so no multiply-add is fused).
// Its three float32 transcendental values per mode -- cos and sin of the
// random phase 2 pi v and exp(-(k/K0)^2) -- are NumPy's own ufuncs in the
// reference, which the C library's cosf/sinf/expf can miss by an ulp.  So the
// generator is split: pal_pao_draws runs the serial LCG, the caller evaluates
// the three values (palinstrophy_gb300/_lib.py does it with NumPy's float32
// ufuncs, which gives the reference's field bit for bit), and pal_pao_build
// does everything else.  pal_pao_generate is the same pipeline with the C
// library's functions, for C callers.  The KM3 part is double precision with
// the C library's sin/cos/sqrt, as Python's math module uses them.
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

#include "palgpu.h"

namespace {

using cf = std::complex<float>;

constexpr int64_t kImm = 420029, kIt = 2017, kId = 5011;

double hash01(int x, int z, int seed, int salt) {
  double a = (double(x) + 1.0) * 12.9898 + (double(z) + 1.0) * 78.233;
  a = a + (double(seed) + 1.0) * 0.010001;
  a = a + (double(salt) + 1.0) * 37.719;
  const double s = std::sin(a) * 43758.5453123;
  return s - std::floor(s);
}

// complex64(a) * p as NumPy multiplies two complex64 scalars: (a + 0i)(pr + i pi)
inline cf scale(float a, cf p) {
  const float zero = 0.0f;
  return cf(a * p.real() - zero * p.imag(), a * p.imag() + zero * p.real());
}

void wavenumbers(int N, std::vector<float>& alfa, std::vector<float>& gamma) {
  const int nh = N / 2;
  alfa.assign(nh, 0.0f);
  gamma.assign(N, 0.0f);
  for (int x = 0; x < nh; ++x) alfa[x] = (float)x;
  for (int z = 1; z <= nh; ++z) {
    gamma[z] = (float)z;
    gamma[N - z] = -gamma[z];
  }
}

}  // namespace

// Serial LCG draws of the PAO loop (turbo_simulator.py:241-286): v[z * N/2 + x]
// is the shuffled uniform variate of mode (x, z), in the reference's call order.
extern "C" int pal_pao_draws(int N, int seed_init, float* v, int* seed_out) {
  if (N < 8 || N % 4 != 0 || !v) return PAL_ERR_INVALID;
  const int nh = N / 2;
  int64_t s = seed_init;
  for (int i = 0; i < 97; ++i) s = (s * kImm + kIt) % kId;
  float table[97];
  for (int i = 0; i < 97; ++i) {
    s = (s * kImm + kIt) % kId;
    table[i] = (float)s / (float)kId;
  }
  for (int z = 0; z < N; ++z) {
    for (int x = 0; x < nh; ++x) {
      s = (s * kImm + kIt) % kId;
      const float r = (float)s / (float)kId;
      int idx = (int)((double)r * 97.0);
      idx = idx < 0 ? 0 : (idx > 96 ? 96 : idx);
      v[(size_t)z * nh + x] = table[idx];
      table[idx] = r;
    }
  }
  if (seed_out) *seed_out = (int)s;
  return PAL_OK;
}

// Everything after the draws (turbo_simulator.py:287-470, 1314-1361), given the
// per-mode float32 values cos_th = cos(2 pi v), sin_th = sin(2 pi v) and
// exp_g = exp(-(k/K0)^2) in the layout of pal_pao_draws.
extern "C" int pal_pao_build(int N, double K0d, double Re, int seed_init, int spectrum, const float* cos_th,
                             const float* sin_th, const float* exp_g, void* om2_out, void* uc_out,
                             double* stats) {
  if (N < 8 || N % 4 != 0 || !om2_out || !uc_out || !cos_th || !sin_th || !exp_g) return PAL_ERR_INVALID;
  if (spectrum != PAL_SPEC_KM3 && spectrum != PAL_SPEC_PAO) return PAL_ERR_INVALID;
  const bool km3 = spectrum == PAL_SPEC_KM3;
  const int nh = N / 2;
  const float PI = 3.14159265358979f;
  const float K0 = (float)K0d;
  std::vector<float> alfa, gamma;
  wavenumbers(N, alfa, gamma);
  // ur[(x * N + z) * 2 + c]
  std::vector<cf> ur((size_t)nh * N * 2, cf(0.0f, 0.0f));
  auto U = [&](int x, int z, int c) -> cf& { return ur[((size_t)x * N + z) * 2 + c]; };

  const float norm = (PI * K0) * K0;
  const float floor2 = 1.0e-40f;
  for (int z = 0; z < N; ++z) {
    const float gz = gamma[z];
    for (int x = 0; x < nh; ++x) {
      const size_t m = (size_t)z * nh + x;
      const cf phase(cos_th[m], sin_th[m]);
      const float ax = alfa[x];
      if (ax == 0.0f) {
        float e2 = exp_g[m] / norm;
        if (km3 && e2 < floor2) e2 = floor2;
        U(x, z, 1) = cf(0.0f, 0.0f);
        U(x, z, 0) = scale(std::sqrt(e2), phase);
      } else {
        const float den = 1.0f + (gz * gz) / (ax * ax);
        float e2 = exp_g[m] / (den * norm);
        if (km3 && e2 < floor2) e2 = floor2;
        const cf w = scale(std::sqrt(e2), phase);
        U(x, z, 1) = w;
        U(x, z, 0) = scale(-(gz / ax), w);
      }
    }
  }
  U(0, 0, 0) = U(0, 0, 1) = cf(0.0f, 0.0f);
  for (int z = 1; z < nh; ++z) {
    U(0, N - z, 0) = std::conj(U(0, z, 0));
    U(0, N - z, 1) = std::conj(U(0, z, 1));
  }
  for (int x = 0; x < nh; ++x) U(x, nh, 0) = U(x, nh, 1) = cf(0.0f, 0.0f);

  if (km3) {
    const double knyq = (double)nh;
    std::vector<double> e_shell(nh + 1, 0.0), w_shell(nh + 1, 0.0), target(nh + 1, 0.0);
    for (int x = 0; x < nh; ++x) {
      const double m = x == 0 ? 1.0 : 2.0;
      const double ax2 = (double)alfa[x] * (double)alfa[x];
      for (int z = 0; z < N; ++z) {
        const cf u1 = U(x, z, 0), u3 = U(x, z, 1);
        const double p1 = (double)u1.real() * (double)u1.real() + (double)u1.imag() * (double)u1.imag();
        const double p3 = (double)u3.real() * (double)u3.real() + (double)u3.imag() * (double)u3.imag();
        const double k = std::sqrt(ax2 + (double)gamma[z] * (double)gamma[z]);
        const int sh = (int)(k + 0.5);
        if (k > 0.0 && k <= knyq && sh <= nh) {
          e_shell[sh] += m * (p1 + p3);
          const int zh = (x == 0 && z > nh) ? N - z : z;
          w_shell[sh] += m * (0.75 + 0.50 * hash01(x, zh, seed_init, 17));
        }
      }
    }
    double k0 = (double)K0;
    if (k0 < 1.0) k0 = 1.0;
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
      for (int x = 0; x < nh; ++x) {
        const double ax = (double)alfa[x];
        const double ax2 = ax * ax;
        for (int z = 0; z < N; ++z) {
          const double gz = (double)gamma[z];
          const double gz2 = gz * gz;
          const double k = std::sqrt(ax2 + gz2);
          const int sh = (int)(k + 0.5);
          if (k > 0.0 && k <= knyq && sh <= nh && w_shell[sh] > 0.0) {
            int zh = z;
            double sign = 1.0;
            if (x == 0 && z > nh) {
              zh = N - z;
              sign = -1.0;
            }
            const double jit = 0.75 + 0.50 * hash01(x, zh, seed_init, 17);
            const double e_mode = (scl * target[sh]) * jit / w_shell[sh];
            const double th = sign * 2.0 * 3.141592653589793 * hash01(x, zh, seed_init, 53);
            const cf ph((float)std::cos(th), (float)std::sin(th));
            if (ax == 0.0) {
              U(x, z, 0) = scale((float)std::sqrt(e_mode), ph);
              U(x, z, 1) = cf(0.0f, 0.0f);
            } else {
              const cf w = scale((float)std::sqrt(e_mode / (1.0 + gz2 / ax2)), ph);
              U(x, z, 0) = scale((float)(-gz / ax), w);
              U(x, z, 1) = w;
            }
          } else {
            U(x, z, 0) = U(x, z, 1) = cf(0.0f, 0.0f);
          }
        }
      }
    }
  }

  double a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, a6 = 0;
  for (int x = 0; x < nh; ++x) {
    const double ax2 = (double)alfa[x] * (double)alfa[x];
    const double m = x == 0 ? 1.0 : 2.0;
    for (int z = 0; z < N; ++z) {
      const cf u1 = U(x, z, 0), u3 = U(x, z, 1);
      const double p1 = (double)u1.real() * (double)u1.real() + (double)u1.imag() * (double)u1.imag();
      const double p3 = (double)u3.real() * (double)u3.real() + (double)u3.imag() * (double)u3.imag();
      const double gz2 = (double)gamma[z] * (double)gamma[z];
      a1 += m * p1;
      a2 += m * p3;
      a3 += m * p1 * ax2;
      a4 += m * p1 * gz2;
      a5 += m * p3 * ax2;
      a6 += m * p3 * gz2;
    }
  }
  const float visc = (float)(1.0 / (double)(float)Re);
  if (stats) {
    stats[0] = a1 + a2;
    stats[1] = a3 + a4 + a5 + a6;
    stats[2] = (double)visc;
  }

  // outputs: uc_low (2, N, nh) [c][z][x]; om2 (N, nh) = i (gz u1 - ax u3)
  cf* uc = static_cast<cf*>(uc_out);
  cf* om = static_cast<cf*>(om2_out);
  for (int c = 0; c < 2; ++c)
    for (int z = 0; z < N; ++z)
      for (int x = 0; x < nh; ++x) uc[((size_t)c * N + z) * nh + x] = U(x, z, c);
  for (int z = 0; z < N; ++z) {
    for (int x = 0; x < nh; ++x) {
      const cf u1 = U(x, z, 0), u3 = U(x, z, 1);
      const float dre = gamma[z] * u1.real() - alfa[x] * u3.real();
      const float dim = gamma[z] * u1.imag() - alfa[x] * u3.imag();
      om[(size_t)z * nh + x] = cf(-dim, dre);
    }
  }
  return PAL_OK;
}

extern "C" int pal_pao_generate(int N, double K0d, double Re, int seed_init, int spectrum, void* om2_out,
                                void* uc_out, double* stats, int* seed_out) {
  if (N < 8 || N % 4 != 0 || !om2_out || !uc_out) return PAL_ERR_INVALID;
  if (spectrum != PAL_SPEC_KM3 && spectrum != PAL_SPEC_PAO) return PAL_ERR_INVALID;
  const int nh = N / 2;
  const size_t n = (size_t)N * nh;
  std::vector<float> v(n), c(n), sn(n), e(n), alfa, gamma;
  int rc = pal_pao_draws(N, seed_init, v.data(), seed_out);
  if (rc != PAL_OK) return rc;
  wavenumbers(N, alfa, gamma);
  const float PI = 3.14159265358979f;
  const float K0 = (float)K0d;
  for (int z = 0; z < N; ++z) {
    for (int x = 0; x < nh; ++x) {
      const size_t m = (size_t)z * nh + x;
      const float th = (2.0f * PI) * v[m];
      c[m] = std::cos(th);
      sn[m] = std::sin(th);
      const float k2 = alfa[x] * alfa[x] + gamma[z] * gamma[z];
      const float k = k2 > 0.0f ? std::sqrt(k2) : 0.0f;
      const float t = k / K0;
      e[m] = std::exp(-t * t);
    }
  }
  return pal_pao_build(N, K0d, Re, seed_init, spectrum, c.data(), sn.data(), e.data(), om2_out, uc_out, stats);
}
