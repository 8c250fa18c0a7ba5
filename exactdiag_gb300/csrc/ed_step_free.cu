// ed_step_free.cu -- fused step kernel for rows of blocks with a trivial stabiliser (the bulk of
// every doped sector): the segment kernel of ed_seg.cuh when rung and leg J agree, a lane's two rows
// worked on together, in three register budgets (2, 3 or 4 resident CTAs per SM) and both window
// layouts (PAIR).  One row at a time: ed_step_free_nr1.cu; unequal rung and leg J:
// ed_step_free_split.cu.
#include "ed_seg.cuh"

namespace ed {

namespace {

template <typename R, bool CPLX, int MINB, bool PAIR>
int launch_seg(const StepArgs& a, cudaStream_t st) {
    if (a.count <= 0) return ED_OK;
    auto* kern = seg_step_kernel<R, CPLX, MINB, true, 2, false, PAIR>;
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

template <int MINB>
int seg_occupancy() {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, seg_step_kernel<float, false, MINB, true, 2, false, true>,
                                                      kSegThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return per_sm > 0 ? per_sm : 1;
}

}  // namespace

int step_hv_free(int dtype, int minb, int nr, int staged, int pair, const StepArgs& a, cudaStream_t st) {
    nr = seg_rows_for(dtype, nr);
    // staged gathers exist for 32-offset windows only; the unstaged kernel gives the same bits
    if (staged && pair) return step_hv_free_staged(dtype, nr, a, st);
    // one exchange coefficient when J_rung = J_leg (the sums need no per-element choice)
    if (a.w.w[2] != a.w.w[3]) return step_hv_free_split(dtype, nr, pair, a, st);
    if (nr == 1) return step_hv_free_nr1(dtype, minb, pair, a, st);
    return pair ? seg_minb<true>(dtype, minb, a, st) : seg_minb<false>(dtype, minb, a, st);
}

int step_free_occupancy(int minb, size_t /*smem*/) {
    if (minb == 2) return seg_occupancy<2>();
    if (minb == 4) return seg_occupancy<4>();
    return seg_occupancy<3>();
}

}  // namespace ed
