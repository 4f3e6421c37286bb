// FP32 kernel sets: radix plan, row-tile height V and thread counts per grid N.
// M = 3N/2; the last radix is the fused middle pass.
#include "pal_launch.cuh"

using namespace pal;

const KernelSet* pal_kernels_f32(int N) {
  switch (N) {
    case 32: return SetOf<float, Plan<48, 8, 6>, 4, 128, 64>::get(N, 0);
    case 64: return SetOf<float, Plan<96, 16, 6>, 4, 128, 64>::get(N, 0);
    case 128: return SetOf<float, Plan<192, 16, 12>, 4, 128, 64>::get(N, 0);
    case 256: return SetOf<float, Plan<384, 16, 24>, 4, 256, 128>::get(N, 0);
    case 384: return SetOf<float, Plan<576, 24, 24>, 4, 256, 128>::get(N, 0);
    case 512: return SetOf<float, Plan<768, 32, 24>, 4, 256, 128>::get(N, 0);
    case 768: return SetOf<float, Plan<1152, 8, 6, 24>, 4, 256, 256>::get(N, 0);
    case 1024: return SetOf<float, Plan<1536, 16, 4, 24>, 4, 256, 256>::get(N, 0);
    case 1536: return SetOf<float, Plan<2304, 16, 6, 24>, 4, 512, 256>::get(N, 0);
    case 2048: return SetOf<float, Plan<3072, 16, 8, 24>, 4, 512, 256>::get(N, 0);
    case 3072: return SetOf<float, Plan<4608, 16, 12, 24>, 4, 512, 256>::get(N, 0);
    case 4096: return SetOf<float, Plan<6144, 16, 16, 24>, 4, 512, 256>::get(N, 0);
    case 8192: return SetOf<float, Plan<12288, 16, 32, 24>, 2, 256, 256>::get(N, 0);
    default: return nullptr;
  }
}
