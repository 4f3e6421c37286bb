// Launch wrappers: one KernelSet per (precision, N), built from a radix plan,
// a row-tile height V and the thread counts of the row and column kernels.
#pragma once
#include "pal_kernels.cuh"

namespace pal {

struct KernelSet {
  int N, M, precision;
  int V_row, NT_row, NT_col;
  size_t smem_row, smem_col;
  cudaError_t (*configure)();
  void (*row)(const StepArgs&, cudaStream_t);
  void (*phys)(const StepArgs&, cudaStream_t);
  void (*col)(const StepArgs&, cudaStream_t);
  void (*col_inv)(const StepArgs&, cudaStream_t);
  void (*spectral)(const StepArgs&, cudaStream_t, int blocks);
  void (*transpose)(const void* in, void* out, int rows, int cols, int batch, cudaStream_t);
};

constexpr int kSpectralThreads = 256;

template <typename T, class PL, int VR, int NTR, int NTC>
struct SetOf {
  static constexpr int M = PL::M;
  static constexpr size_t smem_row = size_t(PL::PADM) * VR * sizeof(cplx<T>);
  static constexpr size_t smem_col = size_t(PL::PADM) * 2 * sizeof(cplx<T>);
  static_assert(smem_row <= 227 * 1024 && smem_col <= 227 * 1024, "tile does not fit in shared memory");
  static_assert(M % VR == 0, "row tile must divide M");

  static cudaError_t configure() {
    cudaError_t e;
    e = cudaFuncSetAttribute(k_row<T, PL, VR, NTR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_row);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_phys<T, PL, VR, NTR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_row);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_col<T, PL, NTC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_col);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_col_inv<T, PL, NTC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_col);
  }
  static void row(const StepArgs& a, cudaStream_t s) { k_row<T, PL, VR, NTR><<<M / VR, NTR, smem_row, s>>>(a); }
  static void phys(const StepArgs& a, cudaStream_t s) { k_phys<T, PL, VR, NTR><<<M / VR, NTR, smem_row, s>>>(a); }
  static void col(const StepArgs& a, cudaStream_t s) { k_col<T, PL, NTC><<<a.N / 2, NTC, smem_col, s>>>(a); }
  static void col_inv(const StepArgs& a, cudaStream_t s) { k_col_inv<T, PL, NTC><<<a.N / 2, NTC, smem_col, s>>>(a); }
  static void spectral(const StepArgs& a, cudaStream_t s, int blocks) {
    k_spectral<T, kSpectralThreads><<<blocks, kSpectralThreads, 0, s>>>(a);
  }
  static void transpose(const void* in, void* out, int rows, int cols, int batch, cudaStream_t s) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32, batch);
    k_transpose<T><<<grid, dim3(32, 8), 0, s>>>(static_cast<const cplx<T>*>(in), static_cast<cplx<T>*>(out), rows,
                                                cols);
  }
  static const KernelSet* get(int N, int precision) {
    static const KernelSet ks = {N,        M,          precision, VR,   NTR,     NTC,       smem_row,
                                 smem_col, configure,  row,       phys, col,     col_inv,   spectral,
                                 transpose};
    return &ks;
  }
};

}  // namespace pal

// Per-precision tables, defined in pal_inst_f32.cu / pal_inst_f64.cu.
const pal::KernelSet* pal_kernels_f32(int N);
const pal::KernelSet* pal_kernels_f64(int N);
