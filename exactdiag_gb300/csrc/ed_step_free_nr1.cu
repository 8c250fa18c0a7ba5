// ed_step_free_nr1.cu -- fused step kernel for rows of blocks with a trivial stabiliser (the bulk of
// every doped sector): the segment kernel of ed_seg.cuh when rung and leg J agree, a lane's two rows
// one after the other, in three register budgets (2, 3 or 4 resident CTAs per SM).
#include "ed_seg.cuh"

namespace ed {

namespace {

template <typename R, bool CPLX, int MINB>
int launch_seg(const StepArgs& a, cudaStream_t st) {
    if (a.count <= 0) return ED_OK;
    auto* kern = seg_step_kernel<R, CPLX, MINB, true, 1>;
    const int grid = a.grid < a.count ? a.grid : a.count;
    kern<<<grid, kSegThreads, 0, st>>>(a.views, a.offs, a.chunks, a.idx, a.count, a.w, a.v, a.vprev, a.other, a.first,
                                       a.scal, a.stride, a.k, a.partials, a.xfull);
    ED_CHECK_LAUNCH("seg_step_kernel");
    return ED_OK;
}

template <int MINB>
int seg_dtype(int dtype, const StepArgs& a, cudaStream_t st) {
    switch (dtype) {
    case ED_F64: return launch_seg<double, false, MINB>(a, st);
    case ED_C128: return launch_seg<double, true, MINB>(a, st);
    case ED_F32: return launch_seg<float, false, MINB>(a, st);
    default: return launch_seg<float, true, MINB>(a, st);
    }
}

}  // namespace

int step_hv_free_nr1(int dtype, int minb, const StepArgs& a, cudaStream_t st) {
    if (minb == 2) return seg_dtype<2>(dtype, a, st);
    if (minb == 4) return seg_dtype<4>(dtype, a, st);
    return seg_dtype<3>(dtype, a, st);
}

}  // namespace ed
