// FP32 candidates, N = 4096 (M = 6144): radix orders x tile heights x threads.
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P6144 = Plan<6144, 16, 16, 24>;
using P6144b = Plan<6144, 32, 8, 24>;
using P6144c = Plan<6144, 24, 16, 16>;
using P6144d = Plan<6144, 16, 24, 16>;

const RowKernels r4096[] = {RowOf<float, P6144, 4, 512>::make("16.16.24 V4x512"),
                            RowOf<float, Rec<P6144>, 4, 512>::make("16.16.24r V4x512"),
                            RowOf<float, Rec<P6144>, 4, 512, 3>::make("16.16.24r V4x512 paired l2pf"),
                            RowOf<float, Rec<P6144>, 4, 768, 3>::make("16.16.24r V4x768 paired l2pf"),
                            RowOf<float, Rec<P6144>, 4, 768, 7>::make("16.16.24r V4x768 paired l2pf tma"),
                            RowOf<float, Rec<P6144>, 4, 768, 11>::make("16.16.24r V4x768 tma-in l2pf"),
                            RowOf<float, Rec<P6144>, 4, 768, 15>::make("16.16.24r V4x768 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P6144>, 4, 1024, 3>::make("16.16.24r V4x1024 paired l2pf"),
                            RowOf<float, Rec<P6144b>, 4, 512, 2>::make("32.8.24r V4x512 paired"),
                            RowOf<float, Rec<P6144>, 2, 384, 31>::make("16.16.24r V2x384 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P6144>, 2, 384, 27>::make("16.16.24r V2x384 tma-in l2pf"),
                            RowOf<float, Rec<P6144c>, 2, 256, 31>::make("24.16.16r V2x256 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P6144d>, 2, 384, 31>::make("16.24.16r V2x384 tma-in tma-out l2pf"),
                            RowOf<float, RecT<P6144>, 2, 384, 31>::make("16.16.24t V2x384 tma-in tma-out l2pf"),
                            RowOf<float, RecT<P6144>, 2, 384, 63>::make("16.16.24t V2x384 tma-in tma-out l2pf2"),
                            RowOf<float, RecT<P6144>, 2, 384, 30>::make("16.16.24t V2x384 tma-in tma-out"),
                            RowOf<float, Rec<P6144>, 2, 384, 30>::make("16.16.24r V2x384 tma-in tma-out"),
                            RowOf<float, Rec<P6144c>, 2, 256, 30>::make("24.16.16r V2x256 tma-in tma-out"),
                            RowOf<float, RecT<P6144c>, 2, 256, 30>::make("24.16.16t V2x256 tma-in tma-out"),
                            RowOf<float, Rec<P6144d>, 2, 384, 30>::make("16.24.16r V2x384 tma-in tma-out")};
const ColKernels c4096[] = {ColOf<float, P6144, 256>::make("16.16.24 x256"),
                            ColOf<float, Rec<P6144c>, 256>::make("24.16.16r x256"),
                            ColOf<float, Rec<P6144>, 256>::make("16.16.24r x256"),
                            ColOf<float, Rec<P6144c>, 384>::make("24.16.16r x384"),
                            ColOf<float, Rec<P6144>, 384>::make("16.16.24r x384"),
                            ColOf<float, Rec<P6144>, 256, 2>::make("16.16.24r x256 hoist"),
                            ColOf<float, Rec<P6144c>, 256, 2>::make("24.16.16r x256 hoist"),
                            ColOf<float, Rec<P6144>, 256, 3>::make("16.16.24r x256 hoist pipe0"),
                            ColOf<float, Rec<P6144c>, 256, 3>::make("24.16.16r x256 hoist pipe0"),
                            ColOf<float, RecT<P6144>, 256, 3>::make("16.16.24t x256 hoist pipe0"),
                            ColOf<float, RecT<P6144d>, 256, 3>::make("16.24.16t x256 hoist pipe0"),
                            ColOf<float, Rec<P6144>, 256, 4>::make("16.16.24r x256 tma"),
                            ColOf<float, Rec<P6144>, 256, 8>::make("16.16.24r x256 tma dual")};

PAL_KERNEL_SET(float, 0, 4096, r4096, c4096)
}  // namespace

const KernelSet* pal_kernels_f32_c(int N) { return N == 4096 ? &kSet4096 : nullptr; }
