// ed_step_free_split.cu -- the segment kernel of ed_seg.cuh for unequal rung and leg J (each
// exchange element picks its coefficient), one register budget (2 resident CTAs per SM).
#include "ed_seg.cuh"

namespace ed {

namespace {

template <typename R, bool CPLX>
int launch_split(const StepArgs& a, cudaStream_t st) {
    if (a.count <= 0) return ED_OK;
    auto* kern = seg_step_kernel<R, CPLX, 2, false, sizeof(R) == 4 ? 2 : 1>;
    const int grid = a.grid < a.count ? a.grid : a.count;
    kern<<<grid, kSegThreads, 0, st>>>(a.views, a.offs, a.chunks, a.idx, a.count, a.w, a.v, a.vprev, a.other, a.first,
                                       a.scal, a.stride, a.k, a.partials, a.xfull);
    ED_CHECK_LAUNCH("seg_step_kernel");
    return ED_OK;
}

}  // namespace

int step_hv_free_split(int dtype, const StepArgs& a, cudaStream_t st) {
    switch (dtype) {
    case ED_F64: return launch_split<double, false>(a, st);
    case ED_C128: return launch_split<double, true>(a, st);
    case ED_F32: return launch_split<float, false>(a, st);
    default: return launch_split<float, true>(a, st);
    }
}

}  // namespace ed
