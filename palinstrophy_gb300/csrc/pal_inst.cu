// Lookup of the per-size candidate sets across the instantiation units.
#include "pal_launch.cuh"

const pal::KernelSet* pal_kernels_f32_a(int N);
const pal::KernelSet* pal_kernels_f32_b(int N);
const pal::KernelSet* pal_kernels_f32_c(int N);
const pal::KernelSet* pal_kernels_f32_d(int N);
const pal::KernelSet* pal_kernels_f32_e(int N);
const pal::KernelSet* pal_kernels_f32_f(int N);
const pal::KernelSet* pal_kernels_f64_a(int N);
const pal::KernelSet* pal_kernels_f64_b(int N);

const pal::KernelSet* pal_kernels_f32(int N) {
  if (auto* k = pal_kernels_f32_a(N)) return k;
  if (auto* k = pal_kernels_f32_e(N)) return k;
  if (auto* k = pal_kernels_f32_f(N)) return k;
  if (auto* k = pal_kernels_f32_b(N)) return k;
  if (auto* k = pal_kernels_f32_c(N)) return k;
  return pal_kernels_f32_d(N);
}

const pal::KernelSet* pal_kernels_f64(int N) {
  if (auto* k = pal_kernels_f64_a(N)) return k;
  return pal_kernels_f64_b(N);
}
