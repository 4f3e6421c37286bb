// FP64 candidates, N = 1536 .. 4096.
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P2304 = Plan<2304, 16, 12, 12>;
using P3072 = Plan<3072, 16, 12, 16>;
using P4608 = Plan<4608, 12, 24, 16>;
using P6144 = Plan<6144, 16, 24, 16>;
using P6144b = Plan<6144, 16, 16, 24>;
using P6144c = Plan<6144, 8, 8, 8, 12>;

const RowKernels r1536[] = {RowOf<double, P2304, 2, 256>::make("16.12.12 V2x256")};
const ColKernels c1536[] = {ColOf<double, P2304, 256>::make("16.12.12 x256")};
const RowKernels r2048[] = {RowOf<double, P3072, 2, 256>::make("16.12.16 V2x256"),
                            RowOf<double, P3072, 1, 256>::make("16.12.16 V1x256")};
const ColKernels c2048[] = {ColOf<double, P3072, 256>::make("16.12.16 x256"), ColOf<double, P3072, 128>::make("16.12.16 x128")};
const RowKernels r3072[] = {RowOf<double, P4608, 2, 256>::make("12.24.16 V2x256")};
const ColKernels c3072[] = {ColOf<double, P4608, 256>::make("12.24.16 x256")};
const RowKernels r4096[] = {RowOf<double, P6144, 2, 256>::make("16.24.16 V2x256"),
                            RowOf<double, P6144, 1, 256>::make("16.24.16 V1x256"),
                            RowOf<double, P6144b, 1, 256>::make("16.16.24 V1x256"),
                            RowOf<double, P6144c, 1, 256>::make("8.8.8.12 V1x256")};
const ColKernels c4096[] = {ColOf<double, P6144, 256>::make("16.24.16 x256"), ColOf<double, P6144, 128>::make("16.24.16 x128"),
                            ColOf<double, P6144b, 256>::make("16.16.24 x256"), ColOf<double, P6144c, 256>::make("8.8.8.12 x256")};

PAL_KERNEL_SET(double, 1, 1536, r1536, c1536)
PAL_KERNEL_SET(double, 1, 2048, r2048, c2048)
PAL_KERNEL_SET(double, 1, 3072, r3072, c3072)
PAL_KERNEL_SET(double, 1, 4096, r4096, c4096)
}  // namespace

const KernelSet* pal_kernels_f64_b(int N) {
  switch (N) {
    case 1536: return &kSet1536;
    case 2048: return &kSet2048;
    case 3072: return &kSet3072;
    case 4096: return &kSet4096;
    default: return nullptr;
  }
}
