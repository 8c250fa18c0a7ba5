// ed_step.cuh -- the fused Lanczos step kernel (H.v + the step's partial sums), one instantiation
// per row kind.
//
// One pass over a list of chunks computes, for each row i of a chunk,
//   y_i = (H v)_i - b_k v_{k-1,i}                    (general/cython_lanczos_diagonalization.pyx:68-77)
// stores y_i, and accumulates the chunk's partial sums <v,Hv>, |y|^2, <v,y>, |v|^2 (per thread
// exactly, see Accum; per chunk in FP64).  Every row of a chunk lies in one block, so the CTA
// stages that block's descriptor once per chunk and builds from it what all its rows share: the
// hop records (BlockHop) and, for a two-element stabiliser, the images of the bond flips
// (PairStab).  Instantiations by row kind keep each kernel's register budget to the code its rows
// need: free blocks never touch the coset or bitmap code of the others.
#pragma once

#include "ed_device.cuh"

namespace ed {

__device__ __forceinline__ void chunk_reduce(double v[kReduceSlots], double* __restrict__ out) {
    __shared__ double red[kReduceSlots][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < kReduceSlots; ++k) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) red[k][wid] = t;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < kReduceSlots; ++k) {
            double t = lane < nw ? red[k][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) out[k] = t;
        }
    }
    __syncthreads();
}

// Float-float variant for FP32 vectors: the CTA-wide sums stay in FP32 pairs (TwoSum), one
// thread converts the chunk's results to FP64.
__device__ __forceinline__ void chunk_reduce(Accum<float> (&v)[kReduceSlots], double* __restrict__ out) {
    __shared__ float2 red[kReduceSlots][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < kReduceSlots; ++k) {
        Accum<float> t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_down_sync(0xffffffffu, t.hi, o);
            const float ol = __shfl_down_sync(0xffffffffu, t.lo, o);
            t.add(oh, ol);
        }
        if (lane == 0) red[k][wid] = make_float2(t.hi, t.lo);
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < kReduceSlots; ++k) {
            Accum<float> t;
            if (lane < nw) {
                t.hi = red[k][lane].x;
                t.lo = red[k][lane].y;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_down_sync(0xffffffffu, t.hi, o);
                const float ol = __shfl_down_sync(0xffffffffu, t.lo, o);
                t.add(oh, ol);
            }
            if (lane == 0) out[k] = t.value();
        }
    }
    __syncthreads();
}

template <typename R, bool CPLX>
__device__ __forceinline__ void* vec_at(void* base, int64_t off) {
    return reinterpret_cast<typename Vec<R, CPLX>::T*>(base) + off;
}

template <typename R, bool CPLX, int MINB, int KIND>
__global__ void __launch_bounds__(kHvThreads, MINB)
    lanczos_hv_kernel(const SectorView* __restrict__ views, const int64_t* __restrict__ offs,
                      const BatchChunk* __restrict__ chunks, const int* __restrict__ idx, int count, HvWeights W,
                      void* v, void* vprev, void* other, int first, const double* __restrict__ scal, int stride,
                      int k, double* __restrict__ partials) {
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<R> tb = load_tables<R>(views[0], smem);
    const R w[4] = {(R)W.w[0], (R)W.w[1], (R)W.w[2], (R)W.w[3]};
    __shared__ __align__(16) BlockDesc sdesc;
    __shared__ BlockHop<R> shop[KIND == kRowsGeneric ? 1 : kMaxHops];
    __shared__ PairStab pstab;
    for (int c = blockIdx.x; c < count; c += gridDim.x) {
        const int cid = idx[c];
        const BatchChunk ch = chunks[cid];
        const SectorView S = views[ch.sec];
        if constexpr (KIND != kRowsGeneric) {
            // stage_block's first barrier also ends the previous chunk's reads of shop and pstab
            stage_block(S.desc + ch.block, &sdesc);
            build_block_hops<R, CPLX>(sdesc, tb, w, S.Ns, S.N, KIND == kRowsFree, shop);
            if (KIND == kRowsCand && sdesc.ncand == 2) build_pair_stab(sdesc, S.Ns, pstab);
            __syncthreads();
        }
        const void* x = vec_at<R, CPLX>(v, offs[ch.sec]);
        void* y = vec_at<R, CPLX>(other, offs[ch.sec]);
        const void* yp = first ? nullptr : vec_at<R, CPLX>(vprev, offs[ch.sec]);
        const R beta = first ? R(0) : (R)scal[(int64_t)ch.sec * stride + 2 * k];
        Accum<R> acc[kReduceSlots];
        auto finish_row = [&](int64_t i, R hr, R hi, R xr, R xi, R pr, R pi) {
            R yr = hr - beta * pr, yi = hi;
            if constexpr (CPLX) yi -= beta * pi;
            st<R, CPLX>(y, i, yr, yi);
            acc[0].add_prod(xr, hr);
            acc[1].add_prod(yr, yr);
            acc[2].add_prod(xr, yr);
            acc[3].add_prod(xr, xr);
            if constexpr (CPLX) {
                acc[0].add_prod(xi, hi);
                acc[1].add_prod(yi, yi);
                acc[2].add_prod(xi, yi);
                acc[3].add_prod(xi, xi);
            }
        };
        if constexpr (KIND == kRowsGeneric) {
            for (int64_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
                R hr, hi, xr, xi, pr = R(0), pi = R(0);
                hv_row<R, CPLX>(S, tb, w, i, x, hr, hi, xr, xi);
                if (!first) ld<R, CPLX>(yp, i, pr, pi);  // v_{k-1}; may be the same buffer as y (read before written)
                finish_row(i, hr, hi, xr, xi, pr, pi);
            }
        } else {
            // the next row's key, x_i and v_{k-1,i} are loaded one row ahead, so their DRAM latency
            // overlaps this row's gathers (v_{k-1} may share y's buffer: each entry is read before
            // its row writes it)
            int64_t i = ch.begin + threadIdx.x;
            uint64_t key = 0;
            R xr = R(0), xi = R(0), pr = R(0), pi = R(0);
            if (i < ch.end) {
                key = S.keys[i];
                ld<R, CPLX>(x, i, xr, xi);
                if (!first) ld<R, CPLX>(yp, i, pr, pi);
            }
            for (; i < ch.end; i += blockDim.x) {
                const int64_t in = i + blockDim.x;
                uint64_t key_n = 0;
                R xr_n = R(0), xi_n = R(0), pr_n = R(0), pi_n = R(0);
                if (in < ch.end) {
                    key_n = S.keys[in];
                    ld<R, CPLX>(x, in, xr_n, xi_n);
                    if (!first) ld<R, CPLX>(yp, in, pr_n, pi_n);
                }
                R hr, hi;
                hv_row_fast<R, CPLX, KIND, true>(S, tb, w, i, key, &sdesc, x, hr, hi, xr, xi, shop, &pstab);
                finish_row(i, hr, hi, xr, xi, pr, pi);
                key = key_n;
                xr = xr_n;
                xi = xi_n;
                pr = pr_n;
                pi = pi_n;
            }
        }
        if constexpr (sizeof(R) == 4) {
            chunk_reduce(acc, partials + (int64_t)cid * kReduceSlots);
        } else {
            double tot[kReduceSlots] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value()};
            chunk_reduce(tot, partials + (int64_t)cid * kReduceSlots);
        }
    }
}

// Launch one instantiation over the chunk list in `a`.
template <typename R, bool CPLX, int MINB, int KIND>
inline int launch_step_kind(const StepArgs& a, cudaStream_t st) {
    if (a.count <= 0) return ED_OK;
    auto* kern = lanczos_hv_kernel<R, CPLX, MINB, KIND>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a.smem);
    const int grid = a.grid < a.count ? a.grid : a.count;
    kern<<<grid, kHvThreads, a.smem, st>>>(a.views, a.offs, a.chunks, a.idx, a.count, a.w, a.v, a.vprev, a.other,
                                           a.first, a.scal, a.stride, a.k, a.partials);
    ED_CHECK_LAUNCH("lanczos_hv_kernel");
    return ED_OK;
}

template <int MINB, int KIND>
inline int step_kind_dtype(int dtype, const StepArgs& a, cudaStream_t st) {
    switch (dtype) {
    case ED_F64: return launch_step_kind<double, false, MINB, KIND>(a, st);
    case ED_C128: return launch_step_kind<double, true, MINB, KIND>(a, st);
    case ED_F32: return launch_step_kind<float, false, MINB, KIND>(a, st);
    default: return launch_step_kind<float, true, MINB, KIND>(a, st);
    }
}

template <int MINB, int KIND>
inline int step_kind_occupancy(size_t smem) {
    auto* kern = lanczos_hv_kernel<float, false, MINB, KIND>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kHvThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return per_sm > 0 ? per_sm : 1;
}

}  // namespace ed
