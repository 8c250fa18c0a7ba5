// ed_step.cuh -- the fused Lanczos step kernel (H.v + the step's partial sums), one instantiation
// per row kind.
//
// One pass over a list of chunks computes, for each row i of a chunk,
//   y_i = (H v)_i - b_k v_{k-1,i}                    (general/cython_lanczos_diagonalization.pyx:68-77)
// stores y_i, and accumulates the chunk's partial sums <v,Hv>, |y|^2, <v,y>, |v|^2 (per thread
// exactly, see Accum; per chunk in FP64).  Every row of a chunk lies in one block, so the CTA
// stages that block's descriptor once per chunk and builds from it the hop records all its rows
// share (BlockHop).  Rows of stabiliser blocks read their exchange targets from the block's
// expanded copy (expand_cand_kernel, run first in the step).  Instantiations by row kind keep each
// kernel's register budget to the code its rows need.
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
                      int k, double* __restrict__ partials, void* xfull) {
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<R> tb = load_tables<R>(views[0], smem);
    const R w[4] = {(R)W.w[0], (R)W.w[1], (R)W.w[2], (R)W.w[3]};
    __shared__ __align__(16) BlockDesc sdesc;
    __shared__ BlockHop<R> shop[KIND == kRowsGeneric ? 1 : kMaxHops];
    for (int c = blockIdx.x; c < count; c += gridDim.x) {
        const int cid = idx[c];
        const BatchChunk ch = chunks[cid];
        const SectorView S = views[ch.sec];
        if constexpr (KIND != kRowsGeneric) {
            // stage_block's first barrier also ends the previous chunk's reads of shop
            stage_block(S.desc + ch.block, &sdesc);
            build_block_hops<R, CPLX>(sdesc, tb, w, S.Ns, S.N, KIND == kRowsFree, shop);
            __syncthreads();
        }
        const void* x = vec_at<R, CPLX>(v, offs[ch.sec]);
        const void* xfull_b = KIND == kRowsCand ? vec_at<R, CPLX>(xfull, ch.xoff) : nullptr;
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
                hv_row_fast<R, CPLX, KIND, true>(S, tb, w, i, key, &sdesc, x, hr, hi, xr, xi, shop, xfull_b);
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
                                           a.first, a.scal, a.stride, a.k, a.partials, a.xfull);
    ED_CHECK_LAUNCH("lanczos_hv_kernel");
    return ED_OK;
}

// ------------------------------------------------------------ stabiliser blocks' expanded copies

constexpr int kExpandRun = 16;  // consecutive colex ranks per thread: one unrank, then next-combination steps
constexpr int kExpandBatch = 4;  // configurations of a run resolved together (loads in flight)
constexpr int kExpandThreads = 256;

// out[r] = conj(u^e) x[rep] / sqrt(orbit) for every spin configuration r of each task's block, as
// the stabiliser rows' exchange terms read it (resolve_cand, bitmap_row and the phase rule of
// gather_add, applied once per configuration instead of once per row and bond); 0 where the
// sector's phases exclude the configuration.
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kExpandThreads)
    expand_cand_kernel(const SectorView* __restrict__ views, const int64_t* __restrict__ offs,
                       const ExpandTask* __restrict__ tasks, int ntasks, int64_t n_spin, void* v, void* xfull) {
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<R> tb = load_tables<R>(views[0], smem);
    const int64_t runs = (n_spin + kExpandRun - 1) / kExpandRun;
    const int64_t total = runs * ntasks;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        const int t = (int)(u / runs);
        const int64_t r0 = (u - (int64_t)t * runs) * kExpandRun;
        const int64_t r1 = r0 + kExpandRun < n_spin ? r0 + kExpandRun : n_spin;
        const ExpandTask T = tasks[t];
        const SectorView& S = views[T.sec];
        const BlockDesc* D = S.desc + T.block;
        const int ncand = D->ncand;
        const int64_t word_off = D->word_off;
        const void* x = vec_at<R, CPLX>(v, offs[T.sec]);
        void* out = vec_at<R, CPLX>(xfull, T.out_off);
        uint32_t cfg = colex_unrank(r0, S.Ns, S.Nd, tb.comb);
        // kExpandBatch configurations at a time: their bitmap words, then their x, are in flight together
        for (int64_t r = r0; r < r1; r += kExpandBatch) {
            CandResult c[kExpandBatch];
            uint32_t rk[kExpandBatch];
            bool live[kExpandBatch];
#pragma unroll
            for (int u = 0; u < kExpandBatch; ++u) {
                live[u] = false;
                rk[u] = 0;
                c[u] = CandResult{0u, 1, 0, false};
                if (r + u < r1) {
                    c[u] = resolve_cand<true>(D->cand, ncand, cfg, S.Ns);
                    live[u] = c[u].valid;
                    if (live[u]) rk[u] = spin_rank(c[u].best, tb.rank, S.Nd);
                    if (r + u + 1 < r1) cfg = next_combination(cfg);
                }
            }
            ulonglong2 bp[kExpandBatch];
#pragma unroll
            for (int u = 0; u < kExpandBatch; ++u)
                if (live[u]) bp[u] = S.bitpref[word_off + (rk[u] >> 6)];
            R xr[kExpandBatch], xi[kExpandBatch];
#pragma unroll
            for (int u = 0; u < kExpandBatch; ++u) {
                xr[u] = xi[u] = R(0);
                if (live[u]) {
                    const uint64_t bit = 1ull << (rk[u] & 63u);
                    if (bp[u].x & bit) {
                        const int64_t j = (int64_t)bp[u].y + __popcll(bp[u].x & (bit - 1ull));
                        ld<R, CPLX>(x, j, xr[u], xi[u]);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kExpandBatch; ++u) {
                if (r + u >= r1) continue;
                const R f = tb.rsqrtv[orbit_of_count(S.N, c[u].count)];
                R vr, vi = R(0);
                if constexpr (CPLX) {
                    const R pr = f * tb.cosv[c[u].e], pi = f * tb.sinv[c[u].e];
                    vr = pr * xr[u] - pi * xi[u];
                    vi = pr * xi[u] + pi * xr[u];
                } else {
                    vr = (c[u].e == 0 ? f : -f) * xr[u];
                }
                st<R, CPLX>(out, r + u, vr, vi);
            }
        }
    }
}

template <typename R, bool CPLX>
inline int launch_expand(const StepArgs& a, cudaStream_t st, int num_sms) {
    auto* kern = expand_cand_kernel<R, CPLX>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a.smem);
    const int64_t work = ((a.n_spin + kExpandRun - 1) / kExpandRun) * a.ntasks;
    const int grid = grid_for(work, kExpandThreads, num_sms, 4);
    kern<<<grid, kExpandThreads, a.smem, st>>>(a.views, a.offs, a.tasks, a.ntasks, a.n_spin, a.v, a.xfull);
    ED_CHECK_LAUNCH("expand_cand_kernel");
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
