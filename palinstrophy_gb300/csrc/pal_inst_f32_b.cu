// FP32 candidates, N = 2048 and 3072 (M = 3072, 4608).
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P3072 = Plan<3072, 16, 8, 24>;
using P3072b = Plan<3072, 8, 16, 24>;
using P4608 = Plan<4608, 16, 12, 24>;

const RowKernels r2048[] = {RowOf<float, P3072, 4, 512>::make("16.8.24 V4x512"),
                            RowOf<float, Rec<P3072>, 4, 512>::make("16.8.24r V4x512"),
                            RowOf<float, Rec<P3072>, 4, 512, 1>::make("16.8.24r V4x512 l2pf"),
                            RowOf<float, Rec<P3072>, 4, 512, 3>::make("16.8.24r V4x512 paired l2pf"),
                            RowOf<float, Rec<P3072>, 4, 384, 3>::make("16.8.24r V4x384 paired l2pf"),
                            RowOf<float, P3072, 2, 256>::make("16.8.24 V2x256"),
                            RowOf<float, P3072, 1, 256>::make("16.8.24 V1x256"),
                            RowOf<float, P3072b, 2, 256>::make("8.16.24 V2x256"),
                            RowOf<float, Rec<P3072>, 4, 384, 31>::make("16.8.24r V4x384 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P3072>, 2, 192, 31>::make("16.8.24r V2x192 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P3072>, 4, 384, 30>::make("16.8.24r V4x384 tma-in tma-out")};
const ColKernels c2048[] = {ColOf<float, P3072, 256>::make("16.8.24 x256"), ColOf<float, P3072, 512>::make("16.8.24 x512"),
                            ColOf<float, P3072b, 256>::make("8.16.24 x256"),
                            ColOf<float, Rec<P3072b>, 256>::make("8.16.24r x256"),
                            ColOf<float, Rec<P3072b>, 256, 1>::make("8.16.24r x256 pref"),
                            ColOf<float, Rec<P3072b>, 512, 1>::make("8.16.24r x512 pref"),
                            ColOf<float, Rec<P3072b>, 256, 2>::make("8.16.24r x256 hoist"),
                            ColOf<float, Rec<P3072b>, 256, 3>::make("8.16.24r x256 hoist pipe0"),
                            ColOf<float, Rec<P3072b>, 256, 4>::make("8.16.24r x256 tma"),
                            ColOf<float, Rec<P3072b>, 256, 5>::make("8.16.24r x256 tma occ")};
const RowKernels r3072[] = {RowOf<float, P4608, 4, 512>::make("16.12.24 V4x512"),
                            RowOf<float, Rec<P4608>, 4, 576, 3>::make("16.12.24r V4x576 paired l2pf"),
                            RowOf<float, Rec<P4608>, 4, 512, 3>::make("16.12.24r V4x512 paired l2pf"),
                            RowOf<float, P4608, 2, 256>::make("16.12.24 V2x256"),
                            RowOf<float, Rec<P4608>, 4, 576, 15>::make("16.12.24r V4x576 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P4608>, 2, 288, 31>::make("16.12.24r V2x288 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P4608>, 2, 288, 30>::make("16.12.24r V2x288 tma-in tma-out")};
const ColKernels c3072[] = {ColOf<float, P4608, 256>::make("16.12.24 x256"), ColOf<float, P4608, 512>::make("16.12.24 x512"),
                            ColOf<float, Rec<P4608>, 256>::make("16.12.24r x256"),
                            ColOf<float, Rec<P4608>, 256, 2>::make("16.12.24r x256 hoist"),
                            ColOf<float, Rec<P4608>, 256, 4>::make("16.12.24r x256 tma")};

PAL_KERNEL_SET(float, 0, 2048, r2048, c2048)
PAL_KERNEL_SET(float, 0, 3072, r3072, c3072)
}  // namespace

const KernelSet* pal_kernels_f32_b(int N) {
  switch (N) {
    case 2048: return &kSet2048;
    case 3072: return &kSet3072;
    default: return nullptr;
  }
}
