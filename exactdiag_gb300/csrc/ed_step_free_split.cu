// ed_step_free_split.cu -- the segment kernel of ed_seg.cuh for unequal rung and leg J (each
// exchange element picks its coefficient), one register budget (2 resident CTAs per SM), one or two
// rows per lane worked on together, both window layouts (PAIR).
#include "ed_seg.cuh"

namespace ed {

namespace {

template <typename R, bool CPLX, int NR, bool PAIR>
int launch_split(const StepArgs& a, cudaStream_t st) {
    if (a.count <= 0) return ED_OK;
    auto* kern = seg_step_kernel<R, CPLX, 2, false, NR, false, PAIR>;
    const int grid = a.grid < a.count ? a.grid : a.count;
    kern<<<grid, kSegThreads, 0, st>>>(a.views, a.offs, a.chunks, a.idx, a.count, a.w, a.v, a.vprev, a.other, a.first,
                                       a.scal, a.stride, a.k, a.partials, a.xfull);
    ED_CHECK_LAUNCH("seg_step_kernel");
    return ED_OK;
}

template <int NR, bool PAIR>
int split_dtype(int dtype, const StepArgs& a, cudaStream_t st) {
    switch (dtype) {
    case ED_F64: return launch_split<double, false, NR, PAIR>(a, st);
    case ED_C128: return launch_split<double, true, NR, PAIR>(a, st);
    case ED_F32: return launch_split<float, false, NR, PAIR>(a, st);
    default: return launch_split<float, true, NR, PAIR>(a, st);
    }
}

}  // namespace

int step_hv_free_split(int dtype, int nr, int pair, const StepArgs& a, cudaStream_t st) {
    if (pair) return nr == 1 ? split_dtype<1, true>(dtype, a, st) : split_dtype<2, true>(dtype, a, st);
    return nr == 1 ? split_dtype<1, false>(dtype, a, st) : split_dtype<2, false>(dtype, a, st);
}

}  // namespace ed
