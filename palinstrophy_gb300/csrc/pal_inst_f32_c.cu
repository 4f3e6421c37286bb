// FP32 candidates, N = 4096 (M = 6144): radix orders x tile heights x threads.
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P6144 = Plan<6144, 16, 16, 24>;
using P6144b = Plan<6144, 32, 8, 24>;
using P6144c = Plan<6144, 24, 16, 16>;

const RowKernels r4096[] = {RowOf<float, P6144, 4, 512>::make("16.16.24 V4x512"),
                            RowOf<float, Rec<P6144>, 4, 512>::make("16.16.24r V4x512"),
                            RowOf<float, Rec<P6144c>, 4, 512>::make("24.16.16r V4x512"),
                            RowOf<float, P6144, 2, 256>::make("16.16.24 V2x256"),
                            RowOf<float, P6144, 2, 512>::make("16.16.24 V2x512"),
                            RowOf<float, P6144, 1, 256>::make("16.16.24 V1x256"),
                            RowOf<float, P6144b, 2, 256>::make("32.8.24 V2x256"),
                            RowOf<float, P6144c, 2, 256>::make("24.16.16 V2x256")};
const ColKernels c4096[] = {ColOf<float, P6144, 256>::make("16.16.24 x256"), ColOf<float, P6144, 512>::make("16.16.24 x512"),
                            ColOf<float, P6144, 128>::make("16.16.24 x128"), ColOf<float, P6144b, 256>::make("32.8.24 x256"),
                            ColOf<float, P6144c, 256>::make("24.16.16 x256"),
                            ColOf<float, Rec<P6144c>, 256>::make("24.16.16r x256"),
                            ColOf<float, P6144c, 512, true>::make("24.16.16 x512 pref"),
                            ColOf<float, Rec<P6144c>, 512, true>::make("24.16.16r x512 pref"),
                            ColOf<float, Rec<P6144>, 512, true>::make("16.16.24r x512 pref")};

PAL_KERNEL_SET(float, 0, 4096, r4096, c4096)
}  // namespace

const KernelSet* pal_kernels_f32_c(int N) { return N == 4096 ? &kSet4096 : nullptr; }
