// ed_step_free_nr1.cu -- fused step kernel for rows of blocks with a trivial stabiliser (the bulk of
// every doped sector): the segment kernel of ed_seg.cuh when rung and leg J agree, a lane's two rows
// one after the other, in three register budgets (2, 3 or 4 resident CTAs per SM) and both window
// layouts (PAIR).
#include "ed_seg.cuh"

namespace ed {

namespace {

template <typename R, bool CPLX, int MINB, bool PAIR>
int launch_seg(const StepArgs& a, cudaStream_t st) {
    if (a.count <= 0) return ED_OK;
    auto* kern = seg_step_kernel<R, CPLX, MINB, true, 1, false, PAIR>;
    const int grid = a.grid < a.count ? a.grid : a.count;
    kern<<<grid, kSegThreads, 0, st>>>(a.views, a.offs, a.chunks, a.idx, a.count, a.w, a.v, a.vprev, a.other, a.first,
                                       a.scal, a.stride, a.k, a.partials, a.xfull);
    ED_CHECK_LAUNCH("seg_step_kernel");
    return ED_OK;
}

template <int MINB, bool PAIR>
int seg_dtype(int dtype, const StepArgs& a, cudaStream_t st) {
    switch (dtype) {
    case ED_F64: return launch_seg<double, false, MINB, PAIR>(a, st);
    case ED_C128: return launch_seg<double, true, MINB, PAIR>(a, st);
    case ED_F32: return launch_seg<float, false, MINB, PAIR>(a, st);
    default: return launch_seg<float, true, MINB, PAIR>(a, st);
    }
}

template <bool PAIR>
int seg_minb(int dtype, int minb, const StepArgs& a, cudaStream_t st) {
    if (minb == 2) return seg_dtype<2, PAIR>(dtype, a, st);
    if (minb == 4) return seg_dtype<4, PAIR>(dtype, a, st);
    return seg_dtype<3, PAIR>(dtype, a, st);
}

}  // namespace

int step_hv_free_nr1(int dtype, int minb, int pair, const StepArgs& a, cudaStream_t st) {
    return pair ? seg_minb<true>(dtype, minb, a, st) : seg_minb<false>(dtype, minb, a, st);
}

}  // namespace ed
