// FP64 kernel sets.  FP64 issue rate is the bound on GB300, so the plans keep
// radix-16 butterflies (64 registers of data) and the fused middle pass at 16.
#include "pal_launch.cuh"

using namespace pal;

const KernelSet* pal_kernels_f64(int N) {
  switch (N) {
    case 32: return SetOf<double, Plan<48, 3, 16>, 2, 128, 64>::get(N, 1);
    case 64: return SetOf<double, Plan<96, 6, 16>, 2, 128, 64>::get(N, 1);
    case 128: return SetOf<double, Plan<192, 12, 16>, 2, 128, 64>::get(N, 1);
    case 256: return SetOf<double, Plan<384, 24, 16>, 2, 256, 128>::get(N, 1);
    case 384: return SetOf<double, Plan<576, 6, 6, 16>, 2, 256, 128>::get(N, 1);
    case 512: return SetOf<double, Plan<768, 16, 3, 16>, 2, 256, 128>::get(N, 1);
    case 768: return SetOf<double, Plan<1152, 6, 12, 16>, 2, 256, 256>::get(N, 1);
    case 1024: return SetOf<double, Plan<1536, 16, 6, 16>, 2, 256, 256>::get(N, 1);
    case 1536: return SetOf<double, Plan<2304, 16, 12, 12>, 2, 256, 256>::get(N, 1);
    case 2048: return SetOf<double, Plan<3072, 16, 12, 16>, 2, 256, 256>::get(N, 1);
    case 3072: return SetOf<double, Plan<4608, 12, 24, 16>, 2, 256, 256>::get(N, 1);
    case 4096: return SetOf<double, Plan<6144, 16, 24, 16>, 2, 256, 256>::get(N, 1);
    default: return nullptr;
  }
}
