// FP32 candidates, N = 1024 and 1536 (M = 1536, 2304).
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P1536 = Plan<1536, 16, 4, 24>;
using P1536b = Plan<1536, 8, 8, 24>;
using P2304 = Plan<2304, 16, 6, 24>;

const RowKernels r1024[] = {RowOf<float, P1536, 4, 256>::make("16.4.24 V4x256"),
                            RowOf<float, Rec<P1536>, 4, 256>::make("16.4.24r V4x256"),
                            RowOf<float, P1536, 2, 256>::make("16.4.24 V2x256"),
                            RowOf<float, P1536, 1, 128>::make("16.4.24 V1x128"),
                            RowOf<float, P1536b, 4, 256>::make("8.8.24 V4x256"),
                            RowOf<float, Rec<P1536>, 4, 192, 3>::make("16.4.24r V4x192 paired l2pf"),
                            RowOf<float, Rec<P1536>, 4, 256, 3>::make("16.4.24r V4x256 paired l2pf"),
                            RowOf<float, Rec<P1536>, 4, 192, 31>::make("16.4.24r V4x192 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P1536>, 4, 192, 30>::make("16.4.24r V4x192 tma-in tma-out")};
const ColKernels c1024[] = {ColOf<float, P1536, 256>::make("16.4.24 x256"), ColOf<float, P1536, 128>::make("16.4.24 x128"),
                            ColOf<float, P1536b, 256>::make("8.8.24 x256"),
                            ColOf<float, Rec<P1536>, 128, 1>::make("16.4.24r x128 pref"),
                            ColOf<float, Rec<P1536>, 256, 1>::make("16.4.24r x256 pref"),
                            ColOf<float, Rec<P1536>, 192, 3>::make("16.4.24r x192 hoist pipe0"),
                            ColOf<float, Rec<P1536>, 256, 2>::make("16.4.24r x256 hoist"),
                            ColOf<float, Rec<P1536>, 128, 4>::make("16.4.24r x128 tma")};
const RowKernels r1536[] = {RowOf<float, P2304, 4, 512>::make("16.6.24 V4x512"),
                            RowOf<float, P2304, 2, 256>::make("16.6.24 V2x256"),
                            RowOf<float, Rec<P2304>, 4, 288, 3>::make("16.6.24r V4x288 paired l2pf"),
                            RowOf<float, Rec<P2304>, 4, 576, 3>::make("16.6.24r V4x576 paired l2pf"),
                            RowOf<float, Rec<P2304>, 4, 288, 31>::make("16.6.24r V4x288 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P2304>, 4, 288, 30>::make("16.6.24r V4x288 tma-in tma-out")};
const ColKernels c1536[] = {ColOf<float, P2304, 256>::make("16.6.24 x256"), ColOf<float, P2304, 128>::make("16.6.24 x128"),
                            ColOf<float, Rec<P2304>, 288, 3>::make("16.6.24r x288 hoist pipe0"),
                            ColOf<float, Rec<P2304>, 256, 2>::make("16.6.24r x256 hoist"),
                            ColOf<float, Rec<P2304>, 256, 4>::make("16.6.24r x256 tma"),
                            ColOf<float, Rec<P2304>, 256, 5>::make("16.6.24r x256 tma occ")};
PAL_KERNEL_SET(float, 0, 1024, r1024, c1024)
PAL_KERNEL_SET(float, 0, 1536, r1536, c1536)
}  // namespace

const KernelSet* pal_kernels_f32_f(int N) {
  switch (N) {
    case 1024: return &kSet1024;
    case 1536: return &kSet1536;
    default: return nullptr;
  }
}
