// FP32 candidates, N = 1024 .. 3072 (M = 1536 .. 4608).
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P1536 = Plan<1536, 16, 4, 24>;
using P1536b = Plan<1536, 8, 8, 24>;
using P2304 = Plan<2304, 16, 6, 24>;
using P3072 = Plan<3072, 16, 8, 24>;
using P3072b = Plan<3072, 8, 16, 24>;
using P4608 = Plan<4608, 16, 12, 24>;

const RowKernels r1024[] = {RowOf<float, P1536, 4, 256>::make("16.4.24 V4x256"),
                            RowOf<float, Rec<P1536>, 4, 256>::make("16.4.24r V4x256"),
                            RowOf<float, P1536, 2, 256>::make("16.4.24 V2x256"),
                            RowOf<float, P1536, 1, 128>::make("16.4.24 V1x128"),
                            RowOf<float, P1536b, 4, 256>::make("8.8.24 V4x256")};
const ColKernels c1024[] = {ColOf<float, P1536, 256>::make("16.4.24 x256"), ColOf<float, P1536, 128>::make("16.4.24 x128"),
                            ColOf<float, P1536b, 256>::make("8.8.24 x256"),
                            ColOf<float, Rec<P1536>, 128, 1>::make("16.4.24r x128 pref"),
                            ColOf<float, Rec<P1536>, 256, 1>::make("16.4.24r x256 pref")};
const RowKernels r1536[] = {RowOf<float, P2304, 4, 512>::make("16.6.24 V4x512"),
                            RowOf<float, P2304, 2, 256>::make("16.6.24 V2x256")};
const ColKernels c1536[] = {ColOf<float, P2304, 256>::make("16.6.24 x256"), ColOf<float, P2304, 128>::make("16.6.24 x128")};
const RowKernels r2048[] = {RowOf<float, P3072, 4, 512>::make("16.8.24 V4x512"),
                            RowOf<float, Rec<P3072>, 4, 512>::make("16.8.24r V4x512"),
                            RowOf<float, Rec<P3072>, 4, 512, 1>::make("16.8.24r V4x512 l2pf"),
                            RowOf<float, Rec<P3072>, 4, 512, 3>::make("16.8.24r V4x512 paired l2pf"),
                            RowOf<float, Rec<P3072>, 4, 384, 3>::make("16.8.24r V4x384 paired l2pf"),
                            RowOf<float, P3072, 2, 256>::make("16.8.24 V2x256"),
                            RowOf<float, P3072, 1, 256>::make("16.8.24 V1x256"),
                            RowOf<float, P3072b, 2, 256>::make("8.16.24 V2x256")};
const ColKernels c2048[] = {ColOf<float, P3072, 256>::make("16.8.24 x256"), ColOf<float, P3072, 512>::make("16.8.24 x512"),
                            ColOf<float, P3072b, 256>::make("8.16.24 x256"),
                            ColOf<float, Rec<P3072b>, 256>::make("8.16.24r x256"),
                            ColOf<float, Rec<P3072b>, 256, 1>::make("8.16.24r x256 pref"),
                            ColOf<float, Rec<P3072b>, 512, 1>::make("8.16.24r x512 pref"),
                            ColOf<float, Rec<P3072b>, 256, 2>::make("8.16.24r x256 hoist")};
const RowKernels r3072[] = {RowOf<float, P4608, 4, 512>::make("16.12.24 V4x512"),
                            RowOf<float, Rec<P4608>, 4, 576, 3>::make("16.12.24r V4x576 paired l2pf"),
                            RowOf<float, Rec<P4608>, 4, 512, 3>::make("16.12.24r V4x512 paired l2pf"),
                            RowOf<float, P4608, 2, 256>::make("16.12.24 V2x256")};
const ColKernels c3072[] = {ColOf<float, P4608, 256>::make("16.12.24 x256"), ColOf<float, P4608, 512>::make("16.12.24 x512"),
                            ColOf<float, Rec<P4608>, 256>::make("16.12.24r x256"),
                            ColOf<float, Rec<P4608>, 256, 2>::make("16.12.24r x256 hoist")};

PAL_KERNEL_SET(float, 0, 1024, r1024, c1024)
PAL_KERNEL_SET(float, 0, 1536, r1536, c1536)
PAL_KERNEL_SET(float, 0, 2048, r2048, c2048)
PAL_KERNEL_SET(float, 0, 3072, r3072, c3072)
}  // namespace

const KernelSet* pal_kernels_f32_b(int N) {
  switch (N) {
    case 1024: return &kSet1024;
    case 1536: return &kSet1536;
    case 2048: return &kSet2048;
    case 3072: return &kSet3072;
    default: return nullptr;
  }
}
