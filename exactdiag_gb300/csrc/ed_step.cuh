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
// sector's phases exclude the configuration.  A warp takes 32 runs of kExpandRun consecutive ranks
// (one per lane: one unrank, then next-combination steps); for vectors of at most 8 bytes the
// values go through shared memory so that the warp's stores are contiguous (the runs of a task
// follow one another), else each lane stores its own run.
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kExpandThreads)
    expand_cand_kernel(const SectorView* __restrict__ views, const int64_t* __restrict__ offs,
                       const ExpandTask* __restrict__ tasks, int ntasks, int64_t n_spin, void* v, void* xfull) {
    using T = typename Vec<R, CPLX>::T;
    constexpr bool kStage = sizeof(T) <= 8;
    constexpr int kW = kExpandThreads / 32;
    // [warp][position in the run][lane, padded]: a lane's writes and the warp's reads stay within
    // two-way bank conflicts
    __shared__ T s_stage[kStage ? kW : 1][kExpandRun][kStage ? 33 : 1];
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<R> tb = load_tables<R>(views[0], smem);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t runs = (n_spin + kExpandRun - 1) / kExpandRun;
    const int64_t total = runs * ntasks;
    const int64_t nwarps = (int64_t)gridDim.x * kW;
    for (int64_t wi = (int64_t)blockIdx.x * kW + warp; wi * 32 < total; wi += nwarps) {
        const int64_t u = wi * 32 + lane;
        T* dst = nullptr;  // this lane's run in the output
        int len = 0;
        if (u < total) {
            const int t = (int)(u / runs);
            const int64_t r0 = (u - (int64_t)t * runs) * kExpandRun;
            const int64_t r1 = r0 + kExpandRun < n_spin ? r0 + kExpandRun : n_spin;
            const ExpandTask T_ = tasks[t];
            const SectorView& S = views[T_.sec];
            const BlockDesc* D = S.desc + T_.block;
            const int ncand = D->ncand;
            const int64_t word_off = D->word_off;
            const void* x = vec_at<R, CPLX>(v, offs[T_.sec]);
            dst = reinterpret_cast<T*>(xfull) + T_.out_off + r0;
            len = (int)(r1 - r0);
            uint32_t cfg = colex_unrank(r0, S.Ns, S.Nd, tb.comb);
            if (len == kExpandRun) {
                // a full run (all but a block's last): the same resolution and values without per-entry
                // branches -- every bitmap word and x load is issued (a configuration that is not a
                // row reads x[0] and takes zero), the candidates are held in registers
                CandParams cp[kMaxCand];
#pragma unroll
                for (int k = 0; k < kMaxCand; ++k) cp[k] = k < ncand ? D->cand[k] : D->cand[0];
                const ulonglong2* __restrict__ bw = S.bitpref + word_off;
#pragma unroll 1
                for (int q0 = 0; q0 < kExpandRun; q0 += kExpandBatch) {
                    CandResult c[kExpandBatch];
                    uint32_t rk[kExpandBatch];
#pragma unroll
                    for (int q = 0; q < kExpandBatch; ++q) {
                        c[q] = resolve_cand_held(cp, ncand, cfg, S.Ns);
                        rk[q] = spin_rank(c[q].best, tb.rank, S.Nd);
                        cfg = next_combination(cfg);  // past the run's last entry: unused
                    }
                    ulonglong2 bp[kExpandBatch];
#pragma unroll
                    for (int q = 0; q < kExpandBatch; ++q) bp[q] = bw[rk[q] >> 6];
                    R xr[kExpandBatch], xi[kExpandBatch];
                    bool hit[kExpandBatch];
#pragma unroll
                    for (int q = 0; q < kExpandBatch; ++q) {
                        const uint64_t bit = 1ull << (rk[q] & 63u);
                        hit[q] = c[q].valid && (bp[q].x & bit) != 0ull;
                        const int64_t j = hit[q] ? (int64_t)bp[q].y + __popcll(bp[q].x & (bit - 1ull)) : 0;
                        ld<R, CPLX>(x, j, xr[q], xi[q]);
                        if (!hit[q]) xr[q] = xi[q] = R(0);  // as the general path: the product of zero
                    }
#pragma unroll
                    for (int q = 0; q < kExpandBatch; ++q) {
                        const R f = tb.rsqrtv[orbit_of_count(S.N, c[q].count)];
                        R vr, vi = R(0);
                        if constexpr (CPLX) {
                            const R pr = f * tb.cosv[c[q].e], pi = f * tb.sinv[c[q].e];
                            vr = pr * xr[q] - pi * xi[q];
                            vi = pr * xi[q] + pi * xr[q];
                        } else {
                            vr = (c[q].e == 0 ? f : -f) * xr[q];
                        }
                        if constexpr (kStage) {
                            if constexpr (CPLX) s_stage[warp][q0 + q][lane] = T{vr, vi};
                            else s_stage[warp][q0 + q][lane] = vr;
                        } else {
                            st<R, CPLX>(dst, q0 + q, vr, vi);
                        }
                    }
                }
            } else
            // kExpandBatch configurations at a time: their bitmap words, then their x, are in flight together
            for (int64_t r = r0; r < r1; r += kExpandBatch) {
                CandResult c[kExpandBatch];
                uint32_t rk[kExpandBatch];
                bool live[kExpandBatch];
#pragma unroll
                for (int q = 0; q < kExpandBatch; ++q) {
                    live[q] = false;
                    rk[q] = 0;
                    c[q] = CandResult{0u, 1, 0, false};
                    if (r + q < r1) {
                        c[q] = resolve_cand<true>(D->cand, ncand, cfg, S.Ns);
                        live[q] = c[q].valid;
                        if (live[q]) rk[q] = spin_rank(c[q].best, tb.rank, S.Nd);
                        if (r + q + 1 < r1) cfg = next_combination(cfg);
                    }
                }
                ulonglong2 bp[kExpandBatch];
#pragma unroll
                for (int q = 0; q < kExpandBatch; ++q)
                    if (live[q]) bp[q] = S.bitpref[word_off + (rk[q] >> 6)];
                R xr[kExpandBatch], xi[kExpandBatch];
#pragma unroll
                for (int q = 0; q < kExpandBatch; ++q) {
                    xr[q] = xi[q] = R(0);
                    if (live[q]) {
                        const uint64_t bit = 1ull << (rk[q] & 63u);
                        if (bp[q].x & bit) {
                            const int64_t j = (int64_t)bp[q].y + __popcll(bp[q].x & (bit - 1ull));
                            ld<R, CPLX>(x, j, xr[q], xi[q]);
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < kExpandBatch; ++q) {
                    if (r + q >= r1) continue;
                    const R f = tb.rsqrtv[orbit_of_count(S.N, c[q].count)];
                    R vr, vi = R(0);
                    if constexpr (CPLX) {
                        const R pr = f * tb.cosv[c[q].e], pi = f * tb.sinv[c[q].e];
                        vr = pr * xr[q] - pi * xi[q];
                        vi = pr * xi[q] + pi * xr[q];
                    } else {
                        vr = (c[q].e == 0 ? f : -f) * xr[q];
                    }
                    if constexpr (kStage) {
                        if constexpr (CPLX) s_stage[warp][r + q - r0][lane] = T{vr, vi};
                        else s_stage[warp][r + q - r0][lane] = vr;
                    } else {
                        st<R, CPLX>(dst, r + q - r0, vr, vi);
                    }
                }
            }
        }
        if constexpr (kStage) {
            // element e of the warp's 32 runs: run e / kExpandRun, position e % kExpandRun
            __syncwarp();
#pragma unroll 4
            for (int j = 0; j < kExpandRun; ++j) {
                const int e = j * 32 + lane, src = e / kExpandRun, pos = e % kExpandRun;
                T* const d = reinterpret_cast<T*>(__shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(dst), src));
                const int n = __shfl_sync(0xffffffffu, len, src);
                if (pos < n) d[pos] = s_stage[warp][pos][src];
            }
            __syncwarp();  // the stage is read before the warp's next runs write it
        }
    }
}

template <typename R, bool CPLX>
inline int launch_expand(const StepArgs& a, cudaStream_t st, int num_sms) {
    auto* kern = expand_cand_kernel<R, CPLX>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a.smem);
    const int64_t work = ((a.n_spin + kExpandRun - 1) / kExpandRun) * a.ntasks;
    // every CTA loops over the work: launch no more than fit at once (a second, partial wave would
    // leave most SMs idle)
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kExpandThreads, a.smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int grid = grid_for(work, kExpandThreads, num_sms, per_sm < 4 ? per_sm : 4);
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
