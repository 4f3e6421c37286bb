// FP64 candidates, N = 32 .. 1024.  FP64 issue rate bounds these kernels on
// GB300, so plans keep radix-16 butterflies and a radix-16 middle pass.
#include "pal_launch.cuh"

using namespace pal;

namespace {
using P48 = Plan<48, 3, 16>;
using P96 = Plan<96, 6, 16>;
using P192 = Plan<192, 12, 16>;
using P384 = Plan<384, 24, 16>;
using P576 = Plan<576, 6, 6, 16>;
using P768 = Plan<768, 16, 3, 16>;
using P1152 = Plan<1152, 6, 12, 16>;
using P1536 = Plan<1536, 16, 6, 16>;

const RowKernels r32[] = {RowOf<double, P48, 2, 64>::make("3.16 V2x64")};
const ColKernels c32[] = {ColOf<double, P48, 64>::make("3.16 x64")};
const RowKernels r64[] = {RowOf<double, P96, 2, 64>::make("6.16 V2x64")};
const ColKernels c64[] = {ColOf<double, P96, 64>::make("6.16 x64")};
const RowKernels r128[] = {RowOf<double, P192, 2, 128>::make("12.16 V2x128")};
const ColKernels c128[] = {ColOf<double, P192, 64>::make("12.16 x64")};
const RowKernels r256[] = {RowOf<double, P384, 2, 256>::make("24.16 V2x256")};
const ColKernels c256[] = {ColOf<double, P384, 128>::make("24.16 x128")};
const RowKernels r384[] = {RowOf<double, P576, 2, 256>::make("6.6.16 V2x256")};
const ColKernels c384[] = {ColOf<double, P576, 128>::make("6.6.16 x128")};
const RowKernels r512[] = {RowOf<double, P768, 2, 256>::make("16.3.16 V2x256")};
const ColKernels c512[] = {ColOf<double, P768, 128>::make("16.3.16 x128")};
const RowKernels r768[] = {RowOf<double, P1152, 2, 256>::make("6.12.16 V2x256")};
const ColKernels c768[] = {ColOf<double, P1152, 256>::make("6.12.16 x256")};
const RowKernels r1024[] = {RowOf<double, P1536, 2, 256>::make("16.6.16 V2x256"),
                            RowOf<double, P1536, 1, 128>::make("16.6.16 V1x128")};
const ColKernels c1024[] = {ColOf<double, P1536, 256>::make("16.6.16 x256"), ColOf<double, P1536, 128>::make("16.6.16 x128")};

PAL_KERNEL_SET_ADJ(double, 1, 32, r32, c32, (AdjOf<double, P48, 2, 64, P48, 64>::get()))
PAL_KERNEL_SET_ADJ(double, 1, 64, r64, c64, (AdjOf<double, P96, 2, 64, P96, 64>::get()))
PAL_KERNEL_SET_ADJ(double, 1, 128, r128, c128, (AdjOf<double, P192, 2, 128, P192, 64>::get()))
PAL_KERNEL_SET_ADJ(double, 1, 256, r256, c256, (AdjOf<double, P384, 2, 256, P384, 128>::get()))
PAL_KERNEL_SET(double, 1, 384, r384, c384)
PAL_KERNEL_SET_ADJ(double, 1, 512, r512, c512, (AdjOf<double, P768, 2, 256, P768, 128>::get()))
PAL_KERNEL_SET(double, 1, 768, r768, c768)
PAL_KERNEL_SET(double, 1, 1024, r1024, c1024)
}  // namespace

const KernelSet* pal_kernels_f64_a(int N) {
  switch (N) {
    case 32: return &kSet32;
    case 64: return &kSet64;
    case 128: return &kSet128;
    case 256: return &kSet256;
    case 384: return &kSet384;
    case 512: return &kSet512;
    case 768: return &kSet768;
    case 1024: return &kSet1024;
    default: return nullptr;
  }
}
