// ed_step_free_staged.cu -- the segment kernel of ed_seg.cuh with its gathers staged through shared
// memory (cp.async: every gather of a segment's rows in flight at once, one wait per pass), one or two
// rows per lane, both exchange modes; 80 KB of dynamic shared memory per CTA (kSegStageBytes per
// warp), so at most two CTAs per SM (register budget of 128).
#include "ed_seg.cuh"

namespace ed {

namespace {

template <typename R, bool CPLX, bool MERGED, int NR>
int launch_staged(const StepArgs& a, cudaStream_t st) {
    if (a.count <= 0) return ED_OK;
    auto* kern = seg_step_kernel<R, CPLX, 2, MERGED, NR, true>;
    const size_t dyn = (size_t)(kSegThreads / 32) * kSegStageBytes;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return set_error(ED_ERR_INVALID, "seg_step_kernel (staged): device ordinal");
    // CTAs per SM with this dynamic shared memory, per device (the attribute is set once per device)
    static int per_sm_of[64] = {};
    int& per_sm = per_sm_of[dev];
    if (per_sm < 1) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSegThreads, dyn) != cudaSuccess ||
            per_sm < 1) {
            cudaGetLastError();
            per_sm = 0;
            return set_error(ED_ERR_CUDA, "seg_step_kernel (staged): shared memory configuration");
        }
    }
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = a.grid < sms * per_sm ? a.grid : sms * per_sm;
    if (grid > a.count) grid = a.count;
    kern<<<grid, kSegThreads, dyn, st>>>(a.views, a.offs, a.chunks, a.idx, a.count, a.w, a.v, a.vprev, a.other,
                                         a.first, a.scal, a.stride, a.k, a.partials, a.xfull);
    ED_CHECK_LAUNCH("seg_step_kernel (staged)");
    return ED_OK;
}

template <bool MERGED, int NR>
int staged_dtype(int dtype, const StepArgs& a, cudaStream_t st) {
    switch (dtype) {
    case ED_F64: return launch_staged<double, false, MERGED, NR>(a, st);
    case ED_C128: return launch_staged<double, true, MERGED, NR>(a, st);
    case ED_F32: return launch_staged<float, false, MERGED, NR>(a, st);
    default: return launch_staged<float, true, MERGED, NR>(a, st);
    }
}

}  // namespace

int step_hv_free_staged(int dtype, int nr, const StepArgs& a, cudaStream_t st) {
    const bool merged = a.w.w[2] == a.w.w[3];
    if (merged) return nr == 1 ? staged_dtype<true, 1>(dtype, a, st) : staged_dtype<true, 2>(dtype, a, st);
    return nr == 1 ? staged_dtype<false, 1>(dtype, a, st) : staged_dtype<false, 2>(dtype, a, st);
}

}  // namespace ed
