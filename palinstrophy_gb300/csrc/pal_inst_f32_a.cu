// FP32 candidates, N = 32 .. 256 (M = 48 .. 384).  The last radix is the
// fused middle pass and must be even.
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P48 = Plan<48, 8, 6>;
using P96 = Plan<96, 16, 6>;
using P192 = Plan<192, 16, 12>;
using P384 = Plan<384, 16, 24>;
using P384b = Plan<384, 24, 16>;

const RowKernels r32[] = {RowOf<float, P48, 4, 64>::make("8.6 V4x64"), RowOf<float, P48, 2, 64>::make("8.6 V2x64")};
const ColKernels c32[] = {ColOf<float, P48, 64>::make("8.6 x64")};
const RowKernels r64[] = {RowOf<float, P96, 4, 128>::make("16.6 V4x128"), RowOf<float, P96, 2, 64>::make("16.6 V2x64")};
const ColKernels c64[] = {ColOf<float, P96, 64>::make("16.6 x64")};
const RowKernels r128[] = {RowOf<float, P192, 4, 128>::make("16.12 V4x128"),
                           RowOf<float, P192, 2, 128>::make("16.12 V2x128")};
const ColKernels c128[] = {ColOf<float, P192, 64>::make("16.12 x64"), ColOf<float, P192, 128>::make("16.12 x128")};
const RowKernels r256[] = {RowOf<float, P384, 4, 256>::make("16.24 V4x256"),
                           RowOf<float, P384, 2, 128>::make("16.24 V2x128"),
                           RowOf<float, P384b, 4, 256>::make("24.16 V4x256"),
                           RowOf<float, Rec<P384>, 4, 256, 2>::make("16.24r V4x256 paired"),
                           RowOf<float, Rec<P384b>, 4, 256, 2>::make("24.16r V4x256 paired"),
                           RowOf<float, Rec<P384>, 4, 128, 15>::make("16.24r V4x128 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P384>, 4, 256, 15>::make("16.24r V4x256 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P384b>, 4, 128, 15>::make("24.16r V4x128 tma-in tma-out l2pf"),
                           RowOf<float, Rec<P384>, 4, 128, 14>::make("16.24r V4x128 tma-in tma-out")};
const ColKernels c256[] = {ColOf<float, P384, 128>::make("16.24 x128"), ColOf<float, P384, 64>::make("16.24 x64"),
                           ColOf<float, P384b, 128>::make("24.16 x128"),
                           ColOf<float, Rec<P384>, 128, 2>::make("16.24r x128 hoist"),
                           ColOf<float, Rec<P384b>, 128, 2>::make("24.16r x128 hoist")};
PAL_KERNEL_SET_ADJ(float, 0, 32, r32, c32, (AdjOf<float, P48, 4, 64, P48, 64>::get()))
PAL_KERNEL_SET_ADJ(float, 0, 64, r64, c64, (AdjOf<float, P96, 4, 128, P96, 64>::get()))
PAL_KERNEL_SET_ADJ(float, 0, 128, r128, c128, (AdjOf<float, P192, 4, 128, P192, 64>::get()))
PAL_KERNEL_SET_ADJ(float, 0, 256, r256, c256, (AdjOf<float, P384, 4, 256, P384, 128>::get()))
}  // namespace

const KernelSet* pal_kernels_f32_a(int N) {
  switch (N) {
    case 32: return &kSet32;
    case 64: return &kSet64;
    case 128: return &kSet128;
    case 256: return &kSet256;
    default: return nullptr;
  }
}
