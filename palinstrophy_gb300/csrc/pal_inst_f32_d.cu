// FP32 candidates, N = 8192 (M = 12288).
#include "pal_launch.cuh"
#include "pal_row_split.cuh"

using namespace pal;

namespace {
using P12288 = Plan<12288, 16, 32, 24>;
using P6144c = Plan<6144, 24, 16, 16>;  // half lines of the cluster-split row pass

const RowKernels r8192[] = {RowOf<float, P12288, 2, 256>::make("16.32.24 V2x256"),
                            RowOf<float, Rec<P12288>, 2, 512>::make("16.32.24r V2x512"),
                            RowOf<float, Rec<P12288>, 2, 512, 1>::make("16.32.24r V2x512 l2pf"),
                            RowOf<float, Rec<P12288>, 2, 512, 2>::make("16.32.24r V2x512 paired"),
                            RowOf<float, Rec<P12288>, 2, 512, 3>::make("16.32.24r V2x512 paired l2pf"),
                            RowOf<float, Rec<P12288>, 2, 768, 7>::make("16.32.24r V2x768 paired l2pf tma"),
                            RowOf<float, Rec<P12288>, 2, 768, 15>::make("16.32.24r V2x768 tma-in tma-out l2pf"),
                            RowOf<float, Rec<P12288>, 2, 768, 11>::make("16.32.24r V2x768 tma-in l2pf"),
                            RowOf<float, RecT<P12288>, 2, 768, 15>::make("16.32.24t V2x768 tma-in tma-out l2pf"),
                            RowOf<float, RecT<P12288>, 2, 768, 14>::make("16.32.24t V2x768 tma-in tma-out"),
                            RowSplitOf<RecT<P6144c>, Rec<P12288>, 2, 256, 512, SPLIT_MULTICAST>::make(
                                "2x24.16.16t V2x256 cluster tma-in mc tma-out"),
                            RowSplitOf<RecT<P6144c>, Rec<P12288>, 2, 256, 512, SPLIT_HALVES>::make(
                                "2x24.16.16t V2x256 cluster tma-in dsmem tma-out"),
                            RowSplitOf<RecT<P6144c>, Rec<P12288>, 2, 256, 512, SPLIT_LOAD_ALL>::make(
                                "2x24.16.16t V2x256 cluster tma-in tma-out")};
const ColKernels c8192[] = {ColOf<float, P12288, 512>::make("16.32.24 x512"),
                            ColOf<float, Rec<P12288>, 512>::make("16.32.24r x512"),
                            ColOf<float, Rec<P12288>, 512, 2>::make("16.32.24r x512 hoist"),
                            ColOf<float, Rec<P12288>, 512, 3>::make("16.32.24r x512 hoist pipe0"),
                            ColOf<float, RecT<P12288>, 512, 3>::make("16.32.24t x512 hoist pipe0"),
                            ColOf<float, Rec<P12288>, 512, 4>::make("16.32.24r x512 tma")};

PAL_KERNEL_SET(float, 0, 8192, r8192, c8192)
}  // namespace

const KernelSet* pal_kernels_f32_d(int N) { return N == 8192 ? &kSet8192 : nullptr; }
