// FP32 candidates, N = 384 .. 768 (M = 576 .. 1152).  The last radix is the
// fused middle pass and must be even.
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P576 = Plan<576, 24, 24>;
using P576b = Plan<576, 6, 6, 16>;
using P768 = Plan<768, 32, 24>;
using P768b = Plan<768, 16, 2, 24>;
using P1152 = Plan<1152, 8, 6, 24>;
using P1152b = Plan<1152, 12, 4, 24>;

const RowKernels r384[] = {RowOf<float, P576, 4, 256>::make("24.24 V4x256"),
                           RowOf<float, P576, 2, 128>::make("24.24 V2x128"),
                           RowOf<float, P576b, 4, 256>::make("6.6.16 V4x256"),
                           RowOf<float, Rec<P576>, 4, 256, 2>::make("24.24r V4x256 paired"),
                           RowOf<float, Rec<P576>, 4, 128, 15>::make("24.24r V4x128 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P576>, 4, 256, 15>::make("24.24r V4x256 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P576b>, 4, 192, 15>::make("6.6.16r V4x192 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P576b>, 4, 192, 14>::make("6.6.16r V4x192 tma-in tma-out"),
                           RowOf<float, Rec<P576b>, 2, 128, 14>::make("6.6.16r V2x128 tma-in tma-out")};
const ColKernels c384[] = {ColOf<float, P576, 128>::make("24.24 x128"), ColOf<float, P576b, 128>::make("6.6.16 x128"),
                           ColOf<float, Rec<P576>, 128, 2>::make("24.24r x128 hoist")};
const RowKernels r512[] = {RowOf<float, P768, 4, 256>::make("32.24 V4x256"),
                           RowOf<float, P768, 2, 128>::make("32.24 V2x128"),
                           RowOf<float, P768b, 4, 256>::make("16.2.24 V4x256"),
                           RowOf<float, Rec<P768>, 4, 256, 2>::make("32.24r V4x256 paired"),
                           RowOf<float, Rec<P768b>, 4, 256, 2>::make("16.2.24r V4x256 paired"),
                           RowOf<float, Rec<P768b>, 4, 128, 15>::make("16.2.24r V4x128 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P768b>, 4, 256, 15>::make("16.2.24r V4x256 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P768>, 4, 128, 15>::make("32.24r V4x128 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P768b>, 4, 128, 14>::make("16.2.24r V4x128 tma-in tma-out")};
const ColKernels c512[] = {ColOf<float, P768, 128>::make("32.24 x128"), ColOf<float, P768b, 128>::make("16.2.24 x128"),
                           ColOf<float, P768, 256>::make("32.24 x256"),
                           ColOf<float, Rec<P768>, 128, 2>::make("32.24r x128 hoist"),
                           ColOf<float, Rec<P768b>, 128, 2>::make("16.2.24r x128 hoist"),
                           ColOf<float, Rec<P768b>, 128, 4>::make("16.2.24r x128 tma")};
const RowKernels r768[] = {RowOf<float, P1152, 4, 256>::make("8.6.24 V4x256"),
                           RowOf<float, P1152, 2, 256>::make("8.6.24 V2x256"),
                           RowOf<float, P1152b, 4, 256>::make("12.4.24 V4x256"),
                           RowOf<float, Rec<P1152>, 4, 288, 3>::make("8.6.24r V4x288 paired l2pf"),
                           RowOf<float, Rec<P1152>, 4, 288, 15>::make("8.6.24r V4x288 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P1152>, 4, 288, 14>::make("8.6.24r V4x288 tma-in tma-out")};
const ColKernels c768[] = {ColOf<float, P1152, 256>::make("8.6.24 x256"), ColOf<float, P1152, 128>::make("8.6.24 x128"),
                           ColOf<float, P1152b, 256>::make("12.4.24 x256"),
                           ColOf<float, Rec<P1152>, 288, 3>::make("8.6.24r x288 hoist pipe0"),
                           ColOf<float, Rec<P1152>, 256, 2>::make("8.6.24r x256 hoist"),
                           ColOf<float, Rec<P1152>, 256, 4>::make("8.6.24r x256 tma")};

PAL_KERNEL_SET(float, 0, 384, r384, c384)
PAL_KERNEL_SET_ADJ(float, 0, 512, r512, c512, (AdjOf<float, P768, 4, 256, P768, 128>::get()))
PAL_KERNEL_SET(float, 0, 768, r768, c768)
}  // namespace

const KernelSet* pal_kernels_f32_e(int N) {
  switch (N) {
    case 384: return &kSet384;
    case 512: return &kSet512;
    case 768: return &kSet768;
    default: return nullptr;
  }
}
