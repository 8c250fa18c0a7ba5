// ed_batch.cu -- several Lanczos recursions at once, and Gram-Schmidt projection.
//
// Batched recursion: the target sectors of a dynamical spectrum (all momenta q
// and rung parities, uneven dimensions; tJ_spin_half_ladder/api.py:116-161
// loops over them one at a time, each through
// general/cython_lanczos_diagonalization.pyx:50-77) run together.  The rows of
// all sectors are cut into chunks; each phase of a step is one launch over all
// chunks (fused H.v with per-chunk FP64 partial sums, per-sector scalars, the
// in-place update), and the m steps are captured once into a CUDA graph.  The
// workspace and the instantiated graph are kept for the next call of the same
// batch shape, which only copies its start vectors in and replays the graph.
// The sectors of one batch share L, Nh and Nd (one set of shared-memory
// tables); they differ in momentum and dimension.
//
// Projection (full reorthogonalisation for the lowest-eigenpair solver):
// w <- w - sum_j <v_j, w> v_j with FP64 dot products.
#include <mutex>
#include <vector>

#include "ed_step.cuh"

namespace ed {

// Step flag (scal[2k+3] until a_{k+1} overwrites it): how the update pass finishes v_{k+1}.
constexpr double kFlagOk = 0.0;            // v_{k+1} = (y - a v) / b
constexpr double kFlagBreakdown = 1.0;     // b < kBreakdown: v_{k+1} = y - a v, the recursion has ended
constexpr double kFlagExactPending = 2.0;  // v_{k+1} = y - a v and its exact norm, then b, then the scaling
constexpr double kFlagScale = 3.0;         // exact b known: v_{k+1} /= b
constexpr double kBreakdown = 1e-8;        // cython_lanczos_diagonalization.pyx:68-77 stops below this b
constexpr double kCancel = 1e-6;

// One CTA of kScalarThreads per sector: a_k, b_{k+1} from the sector's chunk partials.  Each thread
// sums a fixed strided subset of chunks in four independent partial sums (loads stay in flight);
// the order depends only on the chunk count, so every launch configuration gives the same bits.
constexpr int kScalarThreads = 512;

__global__ void __launch_bounds__(kScalarThreads)
    lanczos_scalars_kernel(const double* __restrict__ partials, const int* __restrict__ cfirst,
                           const int* __restrict__ ccount, double* __restrict__ scal, int stride, int k,
                           int norm_mode, int norm_off) {
    __shared__ double red[kReduceSlots][32];
    const int s = blockIdx.x;
    double* X = scal + (int64_t)s * stride;
    // norm_mode 2 runs only for sectors whose step left the exact norm pending (uniform per CTA)
    if (norm_mode == 2 && X[2 * k + 3] != kFlagExactPending) return;
    const int cnt = ccount[s];
    const double2* P = reinterpret_cast<const double2*>(partials + (int64_t)cfirst[s] * kReduceSlots);
    double t[4][kReduceSlots] = {};
    int c = threadIdx.x;
    for (; c + 3 * kScalarThreads < cnt; c += 4 * kScalarThreads) {
        double2 q[4][2];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            q[u][0] = P[2 * (c + u * kScalarThreads)];
            q[u][1] = P[2 * (c + u * kScalarThreads) + 1];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            t[u][0] += q[u][0].x;
            t[u][1] += q[u][0].y;
            t[u][2] += q[u][1].x;
            t[u][3] += q[u][1].y;
        }
    }
#pragma unroll
    for (int u = 0; u < 3; ++u) {
        const int cc = c + u * kScalarThreads;
        if (cc < cnt) {
            const double2 q0 = P[2 * cc], q1 = P[2 * cc + 1];
            t[u][0] += q0.x;
            t[u][1] += q0.y;
            t[u][2] += q1.x;
            t[u][3] += q1.y;
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < kReduceSlots; ++q) {
        double v = (t[0][q] + t[1][q]) + (t[2][q] + t[3][q]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[q][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot[kReduceSlots];
        for (int q = 0; q < kReduceSlots; ++q) {
            tot[q] = 0.0;
            for (int i = 0; i < nw; ++i) tot[q] += red[q][i];
        }
        if (norm_mode == 1) {
            X[norm_off] = sqrt(tot[3]);  // |v0|
            return;
        }
        if (norm_mode == 2) {  // b = |y - a v| summed by the update pass
            const double b = sqrt(tot[3]);
            X[2 * k + 2] = b;
            X[2 * k + 3] = (b < kBreakdown) ? kFlagBreakdown : kFlagScale;
            return;
        }
        // b^2 = |y - a v|^2 = |y|^2 - 2a<v,y> + a^2|v|^2 from the one-pass sums; when the terms cancel
        // to fewer than about 10 significant digits (y close to a v: a start vector near an
        // eigenvector) the exact norm is taken by a second pass instead
        const double a = tot[0];
        const double nn = tot[1] - 2.0 * a * tot[2] + a * a * tot[3];
        const double size = tot[1] + a * a * tot[3];
        X[2 * k + 1] = a;
        if (nn <= kCancel * size) {
            X[2 * k + 2] = sqrt(nn > 0.0 ? nn : 0.0);
            X[2 * k + 3] = kFlagExactPending;
            return;
        }
        const double b = sqrt(nn);
        X[2 * k + 2] = b;
        X[2 * k + 3] = (b < kBreakdown) ? kFlagBreakdown : kFlagOk;
    }
}

template <typename R, bool CPLX>
__global__ void norm_partials_kernel(const int64_t* __restrict__ offs, const BatchChunk* __restrict__ chunks,
                                           int nchunks, const void* v, double* __restrict__ partials) {
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const BatchChunk ch = chunks[c];
        const void* x = vec_at<R, CPLX>(const_cast<void*>(v), offs[ch.sec]);
        double acc[kReduceSlots] = {0.0, 0.0, 0.0, 0.0};
        for (int64_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
            R xr, xi;
            ld<R, CPLX>(x, i, xr, xi);
            acc[3] = fma((double)xr, (double)xr, fma((double)xi, (double)xi, acc[3]));
        }
        chunk_reduce(acc, partials + (int64_t)c * kReduceSlots);
    }
}

// The update v_{k+1} = (y - a v) / b.  Every real component (real and imaginary parts alike) is
// updated the same way, so rows from the first 16-byte boundary on move as 16-byte vectors, a
// thread's loads all issued before its stores; rows before the boundary and the tail go one by one.
constexpr int kUpdThreads = 256;

template <typename R>
__device__ __forceinline__ R recip_r(double b) {
    if constexpr (sizeof(R) == 4) return __frcp_rn((float)b);  // FP32 vectors: no FP64 division
    else return 1.0 / b;
}

// y[i] = (y[i] - a x[i]) * inv for i in [0, rows), by one CTA; EXACT also sums |y[i]|^2 (FP64).
// Called once per chunk: kept out of line so each caller's register budget stays its own.
template <typename R, bool CPLX, bool EXACT>
__device__ __noinline__ void update_rows(const typename Vec<R, CPLX>::T* x, typename Vec<R, CPLX>::T* y,
                                            int rows, R a, R inv, double& nrm) {
    using T = typename Vec<R, CPLX>::T;
    constexpr int kComp = 16 / sizeof(R);                        // real components per 16-byte vector
    constexpr int kRowsPerVec = 16 / sizeof(T);                  // rows per 16-byte vector
    auto row = [&](int i) {
        R vr, vi, yr, yi;
        ld<R, CPLX>(x, i, vr, vi);
        ld<R, CPLX>(y, i, yr, yi);
        const R nr = (yr - a * vr) * inv, ni = (yi - a * vi) * inv;
        st<R, CPLX>(y, i, nr, ni);
        if constexpr (EXACT) nrm += (double)nr * (double)nr + (CPLX ? (double)ni * (double)ni : 0.0);
    };
    const uintptr_t ax = reinterpret_cast<uintptr_t>(x), ay = reinterpret_cast<uintptr_t>(y);
    int head = rows;
    if (((ax ^ ay) & 15u) == 0 && (ax % sizeof(T)) == 0) {
        head = (int)(((16u - (ax & 15u)) & 15u) / sizeof(T));
        if (head > rows) head = rows;
    }
    for (int i = threadIdx.x; i < head; i += kUpdThreads) row(i);
    int done = head;
    if (head < rows) {
        const int nvec = (rows - head) / kRowsPerVec;
        const uint4* xs = reinterpret_cast<const uint4*>(x + head);
        uint4* ys = reinterpret_cast<uint4*>(y + head);
        for (int q0 = threadIdx.x; q0 < nvec; q0 += 4 * kUpdThreads) {
            uint4 xa[4], ya[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int q = q0 + u * kUpdThreads;
                if (q < nvec) {
                    xa[u] = __ldcs(xs + q);
                    ya[u] = __ldcs(ys + q);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int q = q0 + u * kUpdThreads;
                if (q < nvec) {
                    const R* xv = reinterpret_cast<const R*>(&xa[u]);
                    R* yv = reinterpret_cast<R*>(&ya[u]);
#pragma unroll
                    for (int e = 0; e < kComp; ++e) {
                        yv[e] = (yv[e] - a * xv[e]) * inv;
                        if constexpr (EXACT) nrm += (double)yv[e] * (double)yv[e];
                    }
                    __stcs(ys + q, ya[u]);
                }
            }
        }
        done = head + nvec * kRowsPerVec;
    }
    for (int i = done + threadIdx.x; i < rows; i += kUpdThreads) row(i);
}

// Chunked update over every chunk (batched recursions and start vectors): mode 0 the step update
// (sectors whose exact norm is pending are left to lanczos_exact_kernel), mode 1 v *= 1/|v0|.
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kUpdThreads, 4)
    lanczos_update_kernel(const int64_t* __restrict__ offs, const BatchChunk* __restrict__ chunks, int nchunks,
                          void* v, void* other, const double* __restrict__ scal, int stride, int k, int mode,
                          int norm_off) {
    using T = typename Vec<R, CPLX>::T;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const BatchChunk ch = chunks[c];
        const double* X = scal + (int64_t)ch.sec * stride;
        T* x = reinterpret_cast<T*>(vec_at<R, CPLX>(v, offs[ch.sec])) + ch.begin;
        double nrm = 0.0;
        if (mode == 1) {
            const double nv = X[norm_off];
            update_rows<R, CPLX, false>(x, x, (int)(ch.end - ch.begin), R(0), nv > 0.0 ? recip_r<R>(nv) : R(0),
                                        nrm);
            continue;
        }
        const double flag = X[2 * k + 3];
        if (flag == kFlagExactPending) continue;
        T* y = reinterpret_cast<T*>(vec_at<R, CPLX>(other, offs[ch.sec])) + ch.begin;
        update_rows<R, CPLX, false>(x, y, (int)(ch.end - ch.begin), (R)X[2 * k + 1],
                                    flag != kFlagOk ? R(1) : recip_r<R>(X[2 * k + 2]), nrm);
    }
}

// Single-sector step update as one flat stream over the vector (no chunk table): every thread
// handles whole 16-byte vectors, four per array in flight.  Left to lanczos_exact_kernel when the
// step's exact norm is pending.
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kUpdThreads, 4)
    lanczos_update_flat_kernel(int64_t n, const void* __restrict__ v, void* __restrict__ other,
                               const double* __restrict__ X) {
    using T = typename Vec<R, CPLX>::T;
    constexpr int kComp = 16 / sizeof(R);
    constexpr int kRowsPerVec = 16 / sizeof(T);
    const double flag = X[3];
    if (flag == kFlagExactPending) return;
    const R a = (R)X[1];
    const R inv = flag != kFlagOk ? R(1) : recip_r<R>(X[2]);
    const T* x = reinterpret_cast<const T*>(v);
    T* y = reinterpret_cast<T*>(other);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
    const uintptr_t ax = reinterpret_cast<uintptr_t>(x), ay = reinterpret_cast<uintptr_t>(y);
    int64_t head = n;
    if (((ax ^ ay) & 15u) == 0 && (ax % sizeof(T)) == 0) {
        head = (int64_t)(((16u - (ax & 15u)) & 15u) / sizeof(T));
        if (head > n) head = n;
    }
    auto row = [&](int64_t i) {
        R vr, vi, yr, yi;
        ld<R, CPLX>(x, i, vr, vi);
        ld<R, CPLX>(y, i, yr, yi);
        st<R, CPLX>(y, i, (yr - a * vr) * inv, (yi - a * vi) * inv);
    };
    for (int64_t i = tid; i < head; i += nth) row(i);
    if (head >= n) return;
    const int64_t nvec = (n - head) / kRowsPerVec;
    const uint4* xs = reinterpret_cast<const uint4*>(x + head);
    uint4* ys = reinterpret_cast<uint4*>(y + head);
    for (int64_t q0 = tid; q0 < nvec; q0 += 4 * nth) {
        uint4 xa[4], ya[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t q = q0 + u * nth;
            if (q < nvec) {
                xa[u] = __ldcs(xs + q);
                ya[u] = __ldcs(ys + q);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t q = q0 + u * nth;
            if (q < nvec) {
                const R* xv = reinterpret_cast<const R*>(&xa[u]);
                R* yv = reinterpret_cast<R*>(&ya[u]);
#pragma unroll
                for (int e = 0; e < kComp; ++e) yv[e] = (yv[e] - a * xv[e]) * inv;
                __stcs(ys + q, ya[u]);
            }
        }
    }
    for (int64_t i = head + nvec * kRowsPerVec + tid; i < n; i += nth) row(i);
}

// Sectors whose step left the exact norm pending (rare: a start vector near an eigenvector):
// v_{k+1} = y - a v and its per-chunk |v_{k+1}|^2 partial sums.  The flag is read per sector,
// so CTAs skip the other sectors' chunk ranges at once.
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kUpdThreads, 4)
    lanczos_exact_kernel(const int64_t* __restrict__ offs, const BatchChunk* __restrict__ chunks,
                         const int* __restrict__ cfirst, const int* __restrict__ ccount, int nsec, void* v,
                         void* other, const double* __restrict__ scal, int stride, int k,
                         double* __restrict__ partials) {
    using T = typename Vec<R, CPLX>::T;
    for (int s = 0; s < nsec; ++s) {
        const double* X = scal + (int64_t)s * stride;
        if (X[2 * k + 3] != kFlagExactPending) continue;
        const R a = (R)X[2 * k + 1];
        for (int c = cfirst[s] + blockIdx.x; c < cfirst[s] + ccount[s]; c += gridDim.x) {
            const BatchChunk ch = chunks[c];
            const T* x = reinterpret_cast<const T*>(vec_at<R, CPLX>(v, offs[s])) + ch.begin;
            T* y = reinterpret_cast<T*>(vec_at<R, CPLX>(other, offs[s])) + ch.begin;
            double nrm = 0.0;
            update_rows<R, CPLX, true>(x, y, (int)(ch.end - ch.begin), a, R(1), nrm);
            double tot[kReduceSlots] = {0.0, 0.0, 0.0, nrm};
            chunk_reduce(tot, partials + (int64_t)c * kReduceSlots);
        }
    }
}

// After the exact b is known: v_{k+1} /= b for the sectors flagged kFlagScale.
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kUpdThreads, 4)
    lanczos_scale_kernel(const int64_t* __restrict__ offs, const BatchChunk* __restrict__ chunks,
                         const int* __restrict__ cfirst, const int* __restrict__ ccount, int nsec, void* other,
                         const double* __restrict__ scal, int stride, int k) {
    using T = typename Vec<R, CPLX>::T;
    for (int s = 0; s < nsec; ++s) {
        const double* X = scal + (int64_t)s * stride;
        if (X[2 * k + 3] != kFlagScale) continue;
        const R inv = recip_r<R>(X[2 * k + 2]);
        for (int c = cfirst[s] + blockIdx.x; c < cfirst[s] + ccount[s]; c += gridDim.x) {
            const BatchChunk ch = chunks[c];
            T* y = reinterpret_cast<T*>(vec_at<R, CPLX>(other, offs[s])) + ch.begin;
            double nrm = 0.0;
            update_rows<R, CPLX, false>(y, y, (int)(ch.end - ch.begin), R(0), inv, nrm);
        }
    }
}

// Chunks of every sector.  Row chunks: each block's rows cut every chunk_rows[kind] (a chunk never
// straddles two blocks), sector-major in row order; a kind's chunks are kChunkRows long, halved (down
// to kChunkRows / 8) while the sector's rows of that kind would make fewer chunks than four per SM.
// H.v chunks: for a free block, its segments class by class (kl = 0 .. P), seg_chunk_rows / seg_win
// segments per range (whole rounds of the CTA's warps: two segments per warp with 32-offset windows,
// one with 64), each range window by window (seg_win offsets of every segment; listed as kRowsFree
// or, with 64-offset windows, kRowsFree64); for the other blocks, their row chunks.
// Both depend on the sector alone: a sector is cut the same way alone and in a batch, so its
// per-chunk sums, and with them its recursion, are the same bits either way.  Expanded copies: one
// per block of Sector::copy_blocks, sector by sector.
void plan_chunks(const std::vector<const Sector*>& secs, ChunkPlan& P) {
    const int nsec = (int)secs.size();
    P.chunks.clear();
    P.hv.clear();
    P.kind_idx.clear();
    P.cfirst.assign(nsec, 0);
    P.ccount.assign(nsec, 0);
    P.hv_first.assign(nsec, 0);
    P.hv_count.assign(nsec, 0);
    P.tasks.clear();
    P.n_full = 0;
    std::vector<int> by_kind[4];
    for (int s = 0; s < nsec; ++s) {
        const Sector& S = *secs[s];
        P.cfirst[s] = (int)P.chunks.size();
        P.hv_first[s] = (int)P.hv.size();
        const int64_t copy_base = P.n_full;
        std::vector<int64_t> copy_off(S.view.n_blocks > 0 ? S.view.n_blocks : 1, -1);
        for (int b : S.copy_blocks) {
            copy_off[b] = P.n_full;
            P.tasks.push_back(ExpandTask{s, b, P.n_full});
            P.n_full += (int64_t)S.n_spin;
        }
        int64_t kind_rows[4] = {0, 0, 0, 0};
        if (S.spans.empty()) kind_rows[kRowsGeneric] += S.view.n;
        for (const BlockSpan& sp : S.spans) kind_rows[sp.kind] += sp.count;
        const int64_t want = 4 * (int64_t)(S.num_sms > 0 ? S.num_sms : 1);
        int64_t chunk_rows[4];
        for (int kind = 0; kind < 4; ++kind) {
            chunk_rows[kind] = kChunkRows;
            while (chunk_rows[kind] > kChunkRows / 8 && kind_rows[kind] / chunk_rows[kind] < want) chunk_rows[kind] /= 2;
        }
        auto add_span = [&](int64_t start, int64_t count, int block, int kind) {
            const int64_t cr = chunk_rows[kind];
            const int64_t xoff = kind == kRowsCand ? copy_off[block] : -1;
            for (int64_t b = 0; b < count; b += cr) {
                BatchChunk c{};
                c.sec = s;
                c.block = block;
                c.begin = start + b;
                c.end = start + std::min<int64_t>(count, b + cr);
                c.xoff = xoff;
                c.kl = -1;
                P.chunks.push_back(c);
                if (kind != kRowsFree) {
                    by_kind[kind].push_back((int)P.hv.size());
                    P.hv.push_back(c);
                }
            }
            if (kind != kRowsFree) return;
            // segment chunks of a free block: per class, per range of segments (whole rounds of the CTA's
            // warps, two segments each), per window of kSegWin offsets -- the windows of one range next to
            // each other, so that the CTAs working at the same time share the range's records and values
            const int Pb = S.view.seg_p;
            const int64_t warps = kSegThreads / 32;
            for (int kl = 0; kl <= Pb; ++kl) {
                const int64_t nseg = (int64_t)S.host_seg_off[kl + 1] - (int64_t)S.host_seg_off[kl];
                if (nseg <= 0) continue;
                int64_t nA = 1;  // C(Pb, kl)
                for (int j = 1; j <= kl; ++j) nA = nA * (Pb - kl + j) / j;
                const int64_t sw = S.seg_win, spw = sw == 32 ? 2 : 1;  // offsets per window, segments per warp
                const int64_t windows = (nA + sw - 1) / sw;
                const int64_t per = spw * warps * std::max<int64_t>(1, S.seg_chunk_rows / (spw * warps * sw));
                for (int64_t g = 0; g < nseg; g += per)
                    for (int64_t pc = 0; pc < windows; ++pc) {
                        BatchChunk c{};
                        c.sec = s;
                        c.block = block;
                        c.begin = g;
                        c.end = std::min<int64_t>(nseg, g + per);
                        c.xoff = copy_base;
                        c.kl = kl;
                        c.piece = (int32_t)pc;
                        by_kind[S.seg_win == 32 ? kRowsFree : kRowsFree64].push_back((int)P.hv.size());
                        P.hv.push_back(c);
                    }
            }
        };
        if (S.spans.empty()) add_span(0, S.view.n, -1, kRowsGeneric);
        for (const BlockSpan& sp : S.spans)
            if (sp.count > 0) add_span(sp.start, sp.count, sp.block, sp.kind);
        P.ccount[s] = (int)P.chunks.size() - P.cfirst[s];
        P.hv_count[s] = (int)P.hv.size() - P.hv_first[s];
    }
    for (int kind = kRowsFree64; kind <= kRowsGeneric; ++kind) {
        P.kind_first[kind] = (int)P.kind_idx.size();
        P.kind_count[kind] = (int)by_kind[kind].size();
        P.kind_idx.insert(P.kind_idx.end(), by_kind[kind].begin(), by_kind[kind].end());
    }
}

// The fused H.v pass of one step over every row kind of a plan (device tables in `a`, whose idx
// points at the whole kind-ordered id list), one launch per kind present.
static int step_hv_all(int dtype, int minb, int nr, int staged, int free_grid, int other_grid, int cand_grid_f32,
                       const int kind_first[4], const int kind_count[4], StepArgs a, cudaStream_t st) {
    const int* idx0 = a.idx;
    // the expanded copies first: hops out of free blocks and the stabiliser rows read them
    if (a.ntasks > 0) {
        if (int rc = step_expand(dtype, a, st)) return rc;
    }
    a.idx = idx0 + kind_first[kRowsFree];
    a.count = kind_count[kRowsFree];
    a.grid = free_grid;
    if (int rc = step_hv_free(dtype, minb, nr, staged, 1, a, st)) return rc;
    a.idx = idx0 + kind_first[kRowsFree64];
    a.count = kind_count[kRowsFree64];
    if (int rc = step_hv_free(dtype, minb, nr, 0, 0, a, st)) return rc;
    a.idx = idx0 + kind_first[kRowsCand];
    a.count = kind_count[kRowsCand];
    a.grid = dtype == ED_F32 ? cand_grid_f32 : other_grid;
    if (int rc = step_hv_cand(dtype, a, st)) return rc;
    a.grid = other_grid;
    a.idx = idx0 + kind_first[kRowsGeneric];
    a.count = kind_count[kRowsGeneric];
    return step_hv_generic(dtype, a, st);
}

static int dtype_code(bool dbl, bool cplx) { return dbl ? (cplx ? ED_C128 : ED_F64) : (cplx ? ED_C64 : ED_F32); }

static int update_grid(const Sector& s, int nchunks) { return std::max(1, std::min(nchunks, s.num_sms * 8)); }

namespace {

// A batch's device workspace (tables, both vector buffers of every sector, reduction scratch, the
// expanded copies, the step scalars) and its instantiated step graph, kept for the next call of the
// same shape: the same sectors in the same order on the same device, dtype, m, weights, graph use
// and launch shape.  Repeated recursions of one batch (one per degenerate ground state, or a sweep
// of start vectors) then plan, allocate and capture once.  One workspace is kept: a call of another
// shape replaces it, and destroying one of its sectors frees it (batch_forget).
struct BatchWorkspace {
    std::vector<uint64_t> serials;
    std::vector<int> chunk_rows;  // each sector's segment chunk length (its plan)
    std::vector<int> wins;        // each sector's segment window (its plan)
    int device = -1, dtype = -1, m = 0, use_graph = 0, nr = 0, staged = 0;
    HvWeights w{};
    int minb = 0, hv_grid = 0, other_grid = 0, cand_grid = 0;
    int nsec = 0, nchunks = 0, nhv = 0, ntasks = 0, stride = 0, grid = 0;
    size_t smem = 0;
    int64_t total = 0;
    int kind_first[4] = {0, 0, 0, 0}, kind_count[4] = {0, 0, 0, 0};
    std::vector<int64_t> hoffs, hn;
    DevBuf<SectorView> dviews;
    DevBuf<int64_t> doffs;
    DevBuf<BatchChunk> dchunks, dhv;
    DevBuf<int> dkidx, dcfirst, dccount, dhfirst, dhcount;
    DevBuf<double> partials, coef;
    DevBuf<uint8_t> buf0, buf1, xfull;
    DevBuf<ExpandTask> dtasks;
    cudaStream_t priv = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~BatchWorkspace() {
        if (exec) cudaGraphExecDestroy(exec);
        if (priv) cudaStreamDestroy(priv);
    }
    bool matches(const std::vector<const Sector*>& secs, int dev, int dt, int mm, const HvWeights& ww,
                 int graph) const {
        if (dev != device || dt != dtype || mm != m || graph != use_graph || secs.size() != serials.size())
            return false;
        for (size_t i = 0; i < secs.size(); ++i)
            if (secs[i]->serial != serials[i] || secs[i]->seg_chunk_rows != chunk_rows[i] || secs[i]->seg_win != wins[i])
                return false;
        for (int t = 0; t < 4; ++t)
            if (ww.w[t] != w.w[t]) return false;
        const Sector& s0 = *secs[0];
        return ww.faithful == w.faithful && s0.hv_minb == minb && s0.seg_nr == nr && s0.seg_staged == staged &&
               s0.hv_grid == hv_grid &&
               s0.other_grid == other_grid && s0.cand_grid_f32 == cand_grid;
    }
};

std::mutex g_batch_mu;
BatchWorkspace* g_batch = nullptr;  // left to the driver at process exit (no CUDA calls from static destructors)

void drop_batch_workspace() {
    if (!g_batch) return;
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != g_batch->device) cudaSetDevice(g_batch->device);
    delete g_batch;
    g_batch = nullptr;
    cudaSetDevice(cur);
}

}  // namespace

void batch_forget(const Sector& s) {
    std::lock_guard<std::mutex> lock(g_batch_mu);
    if (!g_batch) return;
    for (uint64_t id : g_batch->serials)
        if (id == s.serial) {
            drop_batch_workspace();
            return;
        }
}

// Plans the batch, allocates its workspace and uploads the tables (no vector data yet).
template <typename R, bool CPLX>
static int batch_prepare(BatchWorkspace& W, const std::vector<const Sector*>& secs, int m, cudaStream_t st) {
    const int nsec = (int)secs.size();
    const size_t esz = sizeof(typename Vec<R, CPLX>::T);
    std::vector<SectorView> hviews(nsec);
    ChunkPlan plan;
    plan_chunks(secs, plan);
    W.nsec = nsec;
    W.hoffs.assign(nsec, 0);
    W.hn.assign(nsec, 0);
    W.total = 0;
    for (int s = 0; s < nsec; ++s) {
        hviews[s] = secs[s]->view;
        W.hoffs[s] = W.total;
        W.hn[s] = hviews[s].n;
        W.total += hviews[s].n;
    }
    W.nchunks = (int)plan.chunks.size();
    W.nhv = (int)plan.hv.size();
    W.ntasks = (int)plan.tasks.size();
    W.stride = 2 * m + 4;
    for (int kind = 0; kind < 4; ++kind) {
        W.kind_first[kind] = plan.kind_first[kind];
        W.kind_count[kind] = plan.kind_count[kind];
    }
    const Sector& s0 = *secs[0];
    W.grid = update_grid(s0, W.nchunks);
    W.smem = hv_smem_bytes(hviews[0], sizeof(R));
    if (!W.dviews.alloc(nsec) || !W.doffs.alloc(nsec) || !W.dchunks.alloc(W.nchunks) || !W.dhv.alloc(W.nhv) ||
        !W.dkidx.alloc(W.nhv) || !W.dcfirst.alloc(nsec) || !W.dccount.alloc(nsec) || !W.dhfirst.alloc(nsec) ||
        !W.dhcount.alloc(nsec) || !W.partials.alloc((int64_t)std::max(W.nchunks, W.nhv) * kReduceSlots) ||
        !W.coef.alloc((int64_t)nsec * W.stride) || !W.buf0.alloc((int64_t)(W.total * esz)) ||
        !W.buf1.alloc((int64_t)(W.total * esz)) || !W.dtasks.alloc(W.ntasks) ||
        !W.xfull.alloc((int64_t)(plan.n_full * (int64_t)esz)))
        return set_error(ED_ERR_NOMEM, "ed_batch_lanczos: workspace");
    if (W.ntasks)
        cudaMemcpyAsync(W.dtasks.p, plan.tasks.data(), W.ntasks * sizeof(ExpandTask), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(W.dviews.p, hviews.data(), nsec * sizeof(SectorView), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(W.doffs.p, W.hoffs.data(), nsec * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(W.dchunks.p, plan.chunks.data(), W.nchunks * sizeof(BatchChunk), cudaMemcpyHostToDevice, st);
    if (W.nhv) {
        cudaMemcpyAsync(W.dhv.p, plan.hv.data(), W.nhv * sizeof(BatchChunk), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(W.dkidx.p, plan.kind_idx.data(), W.nhv * sizeof(int), cudaMemcpyHostToDevice, st);
    }
    cudaMemcpyAsync(W.dcfirst.p, plan.cfirst.data(), nsec * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(W.dccount.p, plan.ccount.data(), nsec * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(W.dhfirst.p, plan.hv_first.data(), nsec * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(W.dhcount.p, plan.hv_count.data(), nsec * sizeof(int), cudaMemcpyHostToDevice, st);
    // the host vectors above are freed on return: the uploads must have finished
    if (cudaStreamSynchronize(st) != cudaSuccess) return set_error(ED_ERR_CUDA, "ed_batch_lanczos: table upload");
    return ED_OK;
}

// The m steps of the recursion on stream `st` (recorded into the graph when `st` is capturing).
// Per step: the fused H.v of every kind, the per-sector scalars and the update; the exact-norm
// launches return at once unless a sector's step flagged cancellation.
template <typename R, bool CPLX>
static int batch_steps(BatchWorkspace& W, const Sector& s0, const HvWeights& w, cudaStream_t st) {
    uint8_t* b[2] = {W.buf0.p, W.buf1.p};
    for (int k = 0; k < W.m; ++k) {
        void* v = b[k % 2];
        void* other = b[(k + 1) % 2];
        StepArgs a{W.dviews.p, W.doffs.p, W.dhv.p, W.dkidx.p, 0, 0, W.smem, w, v, other, other, k == 0, W.coef.p,
                   W.stride, k, W.partials.p, W.dtasks.p, W.ntasks, (int64_t)s0.n_spin, W.xfull.p};
        if (int rc = step_hv_all(dtype_code(sizeof(R) == 8, CPLX), s0.hv_minb, s0.seg_nr, s0.seg_staged,
                                 s0.hv_grid, s0.other_grid, s0.cand_grid_f32, W.kind_first, W.kind_count, a, st))
            return rc;
        lanczos_scalars_kernel<<<W.nsec, kScalarThreads, 0, st>>>(W.partials.p, W.dhfirst.p, W.dhcount.p, W.coef.p,
                                                                  W.stride, k, 0, 0);
        lanczos_update_kernel<R, CPLX><<<W.grid, kUpdThreads, 0, st>>>(W.doffs.p, W.dchunks.p, W.nchunks, v, other,
                                                                       W.coef.p, W.stride, k, 0, 0);
        // sectors whose b needs the exact norm: y - a v and its norm, b, then v_{k+1} /= b
        lanczos_exact_kernel<R, CPLX><<<W.grid, kUpdThreads, 0, st>>>(W.doffs.p, W.dchunks.p, W.dcfirst.p,
                                                                      W.dccount.p, W.nsec, v, other, W.coef.p,
                                                                      W.stride, k, W.partials.p);
        lanczos_scalars_kernel<<<W.nsec, kScalarThreads, 0, st>>>(W.partials.p, W.dcfirst.p, W.dccount.p, W.coef.p,
                                                                  W.stride, k, 2, 0);
        lanczos_scale_kernel<R, CPLX><<<W.grid, kUpdThreads, 0, st>>>(W.doffs.p, W.dchunks.p, W.dcfirst.p,
                                                                      W.dccount.p, W.nsec, other, W.coef.p, W.stride, k);
    }
    return ED_OK;
}

template <typename R, bool CPLX>
static int batch_typed(const std::vector<const Sector*>& secs, const HvWeights& w, const void* const* v0, int m,
                       double* coef, int use_graph, cudaStream_t st) {
    std::lock_guard<std::mutex> lock(g_batch_mu);
    int dev = 0;
    cudaGetDevice(&dev);
    const int dtype = dtype_code(sizeof(R) == 8, CPLX);
    const Sector& s0 = *secs[0];
    if (!g_batch || !g_batch->matches(secs, dev, dtype, m, w, use_graph)) {
        drop_batch_workspace();  // the old workspace's memory first
        auto* W = new (std::nothrow) BatchWorkspace();
        if (!W) return set_error(ED_ERR_NOMEM, "ed_batch_lanczos: host allocation");
        W->device = dev;
        W->dtype = dtype;
        W->m = m;
        W->use_graph = use_graph;
        W->w = w;
        W->minb = s0.hv_minb;
        W->nr = s0.seg_nr;
        W->staged = s0.seg_staged;
        W->hv_grid = s0.hv_grid;
        W->other_grid = s0.other_grid;
        W->cand_grid = s0.cand_grid_f32;
        for (const Sector* s : secs) {
            W->serials.push_back(s->serial);
            W->chunk_rows.push_back(s->seg_chunk_rows);
            W->wins.push_back(s->seg_win);
        }
        int rc = batch_prepare<R, CPLX>(*W, secs, m, st);
        if (rc == ED_OK && use_graph) {
            // capture the m steps once on a private stream; later calls of this shape replay them
            cudaGraph_t graph = nullptr;
            if (cudaStreamCreateWithFlags(&W->priv, cudaStreamNonBlocking) != cudaSuccess)
                rc = set_error(ED_ERR_CUDA, "ed_batch_lanczos: stream");
            else if (cudaStreamBeginCapture(W->priv, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                rc = set_error(ED_ERR_CUDA, "ed_batch_lanczos: begin capture");
            else {
                rc = batch_steps<R, CPLX>(*W, s0, w, W->priv);
                cudaError_t e = cudaStreamEndCapture(W->priv, &graph);
                if (rc == ED_OK && e == cudaSuccess) e = cudaGraphInstantiate(&W->exec, graph, 0);
                if (graph) cudaGraphDestroy(graph);
                if (rc == ED_OK && e != cudaSuccess) rc = set_cuda_error(e, "ed_batch_lanczos: graph");
            }
        }
        if (rc != ED_OK) {
            delete W;
            return rc;
        }
        g_batch = W;
    }
    BatchWorkspace& W = *g_batch;
    const size_t esz = sizeof(typename Vec<R, CPLX>::T);
    cudaMemsetAsync(W.coef.p, 0, (size_t)W.nsec * W.stride * sizeof(double), st);
    for (int s = 0; s < W.nsec; ++s)
        if (W.hn[s]) cudaMemcpyAsync(W.buf0.p + W.hoffs[s] * esz, v0[s], W.hn[s] * esz, cudaMemcpyDeviceToDevice, st);
    // start vectors: |v0| and normalisation
    norm_partials_kernel<R, CPLX><<<W.grid, 256, 0, st>>>(W.doffs.p, W.dchunks.p, W.nchunks, W.buf0.p, W.partials.p);
    lanczos_scalars_kernel<<<W.nsec, kScalarThreads, 0, st>>>(W.partials.p, W.dcfirst.p, W.dccount.p, W.coef.p,
                                                              W.stride, 0, 1, W.stride - 1);
    lanczos_update_kernel<R, CPLX><<<W.grid, kUpdThreads, 0, st>>>(W.doffs.p, W.dchunks.p, W.nchunks, W.buf0.p,
                                                                   nullptr, W.coef.p, W.stride, 0, 1, W.stride - 1);
    ED_CHECK_LAUNCH("batch start vectors");
    if (use_graph) {
        const cudaError_t e = cudaGraphLaunch(W.exec, st);
        if (e != cudaSuccess) return set_cuda_error(e, "ed_batch_lanczos: graph launch");
    } else {
        if (int rc = batch_steps<R, CPLX>(W, s0, w, st)) return rc;
        ED_CHECK_LAUNCH("batch steps");
    }
    cudaMemcpyAsync(coef, W.coef.p, (size_t)W.nsec * W.stride * sizeof(double), cudaMemcpyDeviceToDevice, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error(e, "ed_batch_lanczos: steps");
    return ED_OK;
}

int batch_lanczos_launch(const std::vector<const Sector*>& secs, const HvWeights& w, int dtype, const void* const* v0,
                         int m, double* coef, int use_graph, cudaStream_t st) {
    if (secs.empty() || m <= 0) return set_error(ED_ERR_INVALID, "ed_batch_lanczos: empty batch or m <= 0");
    const SectorView& a = secs[0]->view;
    for (const Sector* s : secs) {
        if (!s->built) return set_error(ED_ERR_NOT_BUILT, "ed_batch_lanczos: basis not built");
        if (s->view.L != a.L || s->view.Nh != a.Nh || s->view.Nd != a.Nd)
            return set_error(ED_ERR_INVALID, "ed_batch_lanczos: sectors must share L, Nh and Nd");
        if ((dtype == ED_F64 || dtype == ED_F32) && !s->real)
            return set_error(ED_ERR_INVALID, "ed_batch_lanczos: real dtype with a complex sector");
    }
    switch (dtype) {
    case ED_F64: return batch_typed<double, false>(secs, w, v0, m, coef, use_graph, st);
    case ED_C128: return batch_typed<double, true>(secs, w, v0, m, coef, use_graph, st);
    case ED_F32: return batch_typed<float, false>(secs, w, v0, m, coef, use_graph, st);
    case ED_C64: return batch_typed<float, true>(secs, w, v0, m, coef, use_graph, st);
    default: return set_error(ED_ERR_INVALID, "ed_batch_lanczos: dtype");
    }
}

// ------------------------------------------------------------ single sector
//
// A single sector runs through the same kernels as a batch of one (same chunks,
// same reduction order), so sequential and batched recursions agree bit for bit.

int single_setup(Sector& s) {
    ChunkPlan plan;
    plan_chunks({&s}, plan);
    const int64_t zero = 0;
    const int count = (int)plan.chunks.size();
    const int nhv = (int)plan.hv.size();
    s.n_chunks = count;
    s.n_hv_chunks = nhv;
    for (int kind = 0; kind < 4; ++kind) {
        s.kind_first[kind] = plan.kind_first[kind];
        s.kind_count[kind] = plan.kind_count[kind];
    }
    if (!s.d_self.alloc(1) || !s.d_offs.alloc(1) || !s.d_chunks.alloc(count > 0 ? count : 1) ||
        !s.d_hv_chunks.alloc(nhv > 0 ? nhv : 1) || !s.d_kidx.alloc(nhv > 0 ? nhv : 1) || !s.d_cfirst.alloc(1) ||
        !s.d_ccount.alloc(1) || !s.d_hv_first.alloc(1) || !s.d_hv_count.alloc(1))
        return set_error(ED_ERR_NOMEM, "sector step tables");
    cudaMemcpy(s.d_self.p, &s.view, sizeof(SectorView), cudaMemcpyHostToDevice);
    cudaMemcpy(s.d_offs.p, &zero, sizeof(int64_t), cudaMemcpyHostToDevice);
    if (count) cudaMemcpy(s.d_chunks.p, plan.chunks.data(), count * sizeof(BatchChunk), cudaMemcpyHostToDevice);
    if (nhv) {
        cudaMemcpy(s.d_hv_chunks.p, plan.hv.data(), nhv * sizeof(BatchChunk), cudaMemcpyHostToDevice);
        cudaMemcpy(s.d_kidx.p, plan.kind_idx.data(), nhv * sizeof(int), cudaMemcpyHostToDevice);
    }
    cudaMemcpy(s.d_cfirst.p, plan.cfirst.data(), sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(s.d_ccount.p, plan.ccount.data(), sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(s.d_hv_first.p, plan.hv_first.data(), sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(s.d_hv_count.p, plan.hv_count.data(), sizeof(int), cudaMemcpyHostToDevice);
    const int slots = std::max(std::max(count, nhv), 1);
    if (!s.d_partials.alloc((int64_t)slots * kReduceSlots) || !s.d_hv_scal.alloc(8))
        return set_error(ED_ERR_NOMEM, "sector reduction scratch");
    // stabiliser blocks' expanded copies: allocated here, once, for the widest element (complex
    // double, which a real sector also accepts), so that no step allocates (steps may be captured
    // in a CUDA graph)
    s.n_tasks = (int)plan.tasks.size();
    s.n_full = plan.n_full;
    if (s.n_tasks > 0) {
        if (!s.d_tasks.alloc(s.n_tasks) || !s.d_xfull.alloc(s.n_full * 16))
            return set_error(ED_ERR_NOMEM, "sector expansion scratch");
        cudaMemcpy(s.d_tasks.p, plan.tasks.data(), s.n_tasks * sizeof(ExpandTask), cudaMemcpyHostToDevice);
    }
    return ED_OK;
}

static bool dtype_fits(const Sector& s, int dtype) {
    if (dtype == ED_C128 || dtype == ED_C64) return true;
    if (dtype == ED_F64 || dtype == ED_F32) return s.real;
    return false;
}

static int step_grid(const Sector& s) { return update_grid(s, s.n_chunks); }

template <typename R, bool CPLX>
static int single_hv_typed(const Sector& s, const HvWeights& w, const void* v, const void* vprev, void* vnext,
                           double* scal, cudaStream_t st) {
    StepArgs a{s.d_self.p, s.d_offs.p, s.d_hv_chunks.p, s.d_kidx.p, 0, 0, hv_smem_bytes(s.view, sizeof(R)), w,
               const_cast<void*>(v), const_cast<void*>(vprev), vnext, vprev == nullptr, scal, 0, 0, s.d_partials.p,
               s.d_tasks.p, s.n_tasks, (int64_t)s.n_spin, s.d_xfull.p};
    if (int rc = step_hv_all(dtype_code(sizeof(R) == 8, CPLX), s.hv_minb, s.seg_nr, s.seg_staged, s.hv_grid,
                             s.other_grid, s.cand_grid_f32, s.kind_first, s.kind_count, a, st))
        return rc;
    lanczos_scalars_kernel<<<1, kScalarThreads, 0, st>>>(s.d_partials.p, s.d_hv_first.p, s.d_hv_count.p, scal, 0, 0, 0,
                                                         0);
    ED_CHECK_LAUNCH("lanczos_scalars_kernel");
    return ED_OK;
}

// Launch shape of the step kernels: the free-row kernel's register variant (3 or 4 resident CTAs
// per SM) and CTAs per SM (0 = as many as fit); the other kinds run as many CTAs as fit.
int set_launch(Sector& s, int minb, int ctas_per_sm) {
    if (minb < 2 || minb > 4) return set_error(ED_ERR_INVALID, "ed_sector_set_launch: variant must be 2, 3 or 4");
    if (ctas_per_sm < 0 || ctas_per_sm > 8) return set_error(ED_ERR_INVALID, "ed_sector_set_launch: ctas_per_sm");
    const size_t smem = hv_smem_bytes(s.view, sizeof(float));
    const int occ = step_free_occupancy(minb, smem);
    const int per_sm = (ctas_per_sm == 0 || ctas_per_sm > occ) ? occ : ctas_per_sm;
    s.hv_minb = minb;
    s.hv_grid = s.num_sms * per_sm;
    s.other_grid = s.num_sms * step_rest_occupancy(smem, false);
    s.cand_grid_f32 = s.num_sms * step_rest_occupancy(smem, true);
    return ED_OK;
}

// Rows per lane of the free-row kernel (1, 2, or 0 = by dtype), the rows of a segment chunk (a power of
// two from 1024 to 65536) and whether its gathers go through shared memory.  A new chunk length re-plans the sector's steps: its per-chunk sums,
// and with them the last bits of its recursions, follow the plan (the same alone and in a batch).
int set_step_shape(Sector& s, int rows_per_lane, int chunk_rows, int staged) {
    if (rows_per_lane < 0 || rows_per_lane > 2) return set_error(ED_ERR_INVALID, "ed_sector_set_step_shape: rows per lane");
    if (staged != 0 && staged != 1) return set_error(ED_ERR_INVALID, "ed_sector_set_step_shape: staged must be 0 or 1");
    if (staged && s.seg_win != 32)
        return set_error(ED_ERR_INVALID, "ed_sector_set_step_shape: staged gathers need 32-offset segment windows");
    if (chunk_rows < 1024 || chunk_rows > 65536 || (chunk_rows & (chunk_rows - 1)))
        return set_error(ED_ERR_INVALID, "ed_sector_set_step_shape: chunk rows must be a power of two in [1024, 65536]");
    s.seg_nr = rows_per_lane;
    s.seg_staged = staged;
    if (chunk_rows == s.seg_chunk_rows) return ED_OK;
    s.seg_chunk_rows = chunk_rows;
    return s.built ? single_setup(s) : ED_OK;
}

// The offsets of a segment chunk's window, 32 or 64 (a new value re-plans the sector, like a new chunk
// length).  64 cannot go with staged gathers.
int set_segment_window(Sector& s, int offsets) {
    if (offsets != 32 && offsets != 64)
        return set_error(ED_ERR_INVALID, "ed_sector_set_segment_window: offsets must be 32 or 64");
    if (offsets == 64 && s.seg_staged)
        return set_error(ED_ERR_INVALID, "ed_sector_set_segment_window: staged gathers need 32-offset windows");
    if (offsets == s.seg_win) return ED_OK;
    s.seg_win = offsets;
    return s.built ? single_setup(s) : ED_OK;
}

int lanczos_hv_launch(const Sector& s, const HvWeights& w, int dtype, const void* v, const void* vprev, void* vnext,
                      double* scal, double* /*partials*/, cudaStream_t st) {
    if (!dtype_fits(s, dtype)) return set_error(ED_ERR_INVALID, "ed_lanczos_step: dtype does not match the sector");
    if (s.view.n == 0) return set_error(ED_ERR_INVALID, "ed_lanczos_step: empty sector");
    switch (dtype) {
    case ED_F64: return single_hv_typed<double, false>(s, w, v, vprev, vnext, scal, st);
    case ED_C128: return single_hv_typed<double, true>(s, w, v, vprev, vnext, scal, st);
    case ED_F32: return single_hv_typed<float, false>(s, w, v, vprev, vnext, scal, st);
    default: return single_hv_typed<float, true>(s, w, v, vprev, vnext, scal, st);
    }
}

template <typename R, bool CPLX>
static void single_update_typed(const Sector& s, const void* v, void* vnext, const double* scal, cudaStream_t st) {
    const int flat_grid = s.num_sms * 8;
    lanczos_update_flat_kernel<R, CPLX><<<flat_grid, kUpdThreads, 0, st>>>(s.view.n, v, vnext, scal);
    // when the step left the exact norm pending: y - a v and its norm, b, then v_{k+1} /= b
    lanczos_exact_kernel<R, CPLX><<<step_grid(s), kUpdThreads, 0, st>>>(
        s.d_offs.p, s.d_chunks.p, s.d_cfirst.p, s.d_ccount.p, 1, const_cast<void*>(v), vnext, scal, 0, 0,
        s.d_partials.p);
    lanczos_scalars_kernel<<<1, kScalarThreads, 0, st>>>(s.d_partials.p, s.d_cfirst.p, s.d_ccount.p,
                                                         const_cast<double*>(scal), 0, 0, 2, 0);
    lanczos_scale_kernel<R, CPLX><<<step_grid(s), kUpdThreads, 0, st>>>(s.d_offs.p, s.d_chunks.p, s.d_cfirst.p,
                                                                        s.d_ccount.p, 1, vnext, scal, 0, 0);
}

int lanczos_update_launch(const Sector& s, int dtype, const void* v, void* vnext, const double* scal, cudaStream_t st) {
    if (!dtype_fits(s, dtype)) return set_error(ED_ERR_INVALID, "ed_lanczos_update: dtype does not match the sector");
    if (s.view.n == 0) return ED_OK;
    switch (dtype) {
    case ED_F64: single_update_typed<double, false>(s, v, vnext, scal, st); break;
    case ED_C128: single_update_typed<double, true>(s, v, vnext, scal, st); break;
    case ED_F32: single_update_typed<float, false>(s, v, vnext, scal, st); break;
    default: single_update_typed<float, true>(s, v, vnext, scal, st); break;
    }
    ED_CHECK_LAUNCH("lanczos_update_kernel");
    return ED_OK;
}

// y = H x through the step kernels (the step's first pass: no previous vector; its scalars go to a
// per-sector scratch nobody reads).
int hv_step_launch(const Sector& s, const HvWeights& w, int dtype, const void* x, void* y, cudaStream_t st) {
    if (s.view.n == 0) return ED_OK;
    return lanczos_hv_launch(s, w, dtype, x, nullptr, y, s.d_hv_scal.p, nullptr, st);
}

int lanczos_step_launch(const Sector& s, const HvWeights& w, int dtype, const void* v, const void* vprev, void* vnext,
                        double* scal, double* partials, cudaStream_t st) {
    const int rc = lanczos_hv_launch(s, w, dtype, v, vprev, vnext, scal, partials, st);
    if (rc != ED_OK) return rc;
    return lanczos_update_launch(s, dtype, v, vnext, scal, st);
}

template <typename R, bool CPLX>
static void single_norm_typed(const Sector& s, void* x, double* norm, cudaStream_t st) {
    norm_partials_kernel<R, CPLX><<<step_grid(s), 256, 0, st>>>(s.d_offs.p, s.d_chunks.p, s.n_chunks, x,
                                                                s.d_partials.p);
    lanczos_scalars_kernel<<<1, kScalarThreads, 0, st>>>(s.d_partials.p, s.d_cfirst.p, s.d_ccount.p, norm, 0, 0, 1, 0);
    lanczos_update_kernel<R, CPLX><<<step_grid(s), kUpdThreads, 0, st>>>(s.d_offs.p, s.d_chunks.p, s.n_chunks, x, nullptr,
                                                                 norm, 0, 0, 1, 0);
}

int normalize_launch(const Sector& s, int dtype, void* x, double* norm, double* /*partials*/, cudaStream_t st) {
    if (!dtype_fits(s, dtype)) return set_error(ED_ERR_INVALID, "ed_normalize: dtype does not match the sector");
    if (s.view.n == 0) return ED_OK;
    switch (dtype) {
    case ED_F64: single_norm_typed<double, false>(s, x, norm, st); break;
    case ED_C128: single_norm_typed<double, true>(s, x, norm, st); break;
    case ED_F32: single_norm_typed<float, false>(s, x, norm, st); break;
    default: single_norm_typed<float, true>(s, x, norm, st); break;
    }
    ED_CHECK_LAUNCH("normalize kernels");
    return ED_OK;
}

// ------------------------------------------------------------ projection

template <typename R, bool CPLX>
__global__ void proj_dots_kernel(int64_t n, const void* __restrict__ V, const void* __restrict__ w, int nchunks,
                                 double* __restrict__ partials) {
    const int j = blockIdx.y;
    const int64_t per = (n + nchunks - 1) / nchunks;
    const int64_t b = (int64_t)blockIdx.x * per, e = min(n, b + per);
    double acc[kReduceSlots] = {0.0, 0.0, 0.0, 0.0};
    const typename Vec<R, CPLX>::T* vj = reinterpret_cast<const typename Vec<R, CPLX>::T*>(V) + (int64_t)j * n;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        R vr, vi, wr, wi;
        ld<R, CPLX>(vj, i, vr, vi);
        ld<R, CPLX>(w, i, wr, wi);
        // conj(v) * w
        acc[0] = fma((double)vr, (double)wr, fma((double)vi, (double)wi, acc[0]));
        acc[1] = fma((double)vr, (double)wi, fma(-(double)vi, (double)wr, acc[1]));
    }
    chunk_reduce(acc, partials + ((int64_t)j * nchunks + blockIdx.x) * kReduceSlots);
}

__global__ void proj_coef_kernel(const double* __restrict__ partials, int nchunks, double* __restrict__ coef) {
    const int j = blockIdx.x;
    if (threadIdx.x == 0) {
        double re = 0.0, im = 0.0;
        for (int c = 0; c < nchunks; ++c) {
            re += partials[((int64_t)j * nchunks + c) * kReduceSlots];
            im += partials[((int64_t)j * nchunks + c) * kReduceSlots + 1];
        }
        coef[2 * j] = re;
        coef[2 * j + 1] = im;
    }
}

template <typename R, bool CPLX>
__global__ void proj_sub_kernel(int64_t n, const void* __restrict__ V, int k, const double* __restrict__ coef,
                                void* __restrict__ w) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R wr0, wi0;
        ld<R, CPLX>(w, i, wr0, wi0);
        double wr = wr0, wi = wi0;
        for (int j = 0; j < k; ++j) {
            R vr, vi;
            ld<R, CPLX>(reinterpret_cast<const typename Vec<R, CPLX>::T*>(V) + (int64_t)j * n, i, vr, vi);
            const double cr = coef[2 * j], ci = coef[2 * j + 1];
            wr -= cr * (double)vr - ci * (double)vi;
            wi -= cr * (double)vi + ci * (double)vr;
        }
        st<R, CPLX>(w, i, (R)wr, (R)wi);
    }
}

template <typename R, bool CPLX>
static int project_typed(const Sector& s, const void* V, int k, void* w, double* coef, double* partials,
                         int nchunks, cudaStream_t st) {
    const int64_t n = s.view.n;
    dim3 g(nchunks, k);
    proj_dots_kernel<R, CPLX><<<g, 256, 0, st>>>(n, V, w, nchunks, partials);
    proj_coef_kernel<<<k, 32, 0, st>>>(partials, nchunks, coef);
    proj_sub_kernel<R, CPLX><<<grid_for(n, 256, s.num_sms, 16), 256, 0, st>>>(n, V, k, coef, w);
    ED_CHECK_LAUNCH("projection kernels");
    return ED_OK;
}

int project_launch(const Sector& s, int dtype, const void* V, int k, void* w, double* coef, double* scratch,
                   int64_t scratch_len, cudaStream_t st) {
    if (k <= 0 || s.view.n == 0) return ED_OK;
    int nchunks = (int)std::min<int64_t>(2 * s.num_sms, (s.view.n + 1023) / 1024);
    if (nchunks < 1) nchunks = 1;
    if ((int64_t)k * nchunks * kReduceSlots > scratch_len) nchunks = (int)(scratch_len / ((int64_t)k * kReduceSlots));
    if (nchunks < 1) return set_error(ED_ERR_TOO_LARGE, "ed_project_out: scratch too small for k vectors");
    if (k > 65535) return set_error(ED_ERR_TOO_LARGE, "ed_project_out: k too large");
    switch (dtype) {
    case ED_F64: return project_typed<double, false>(s, V, k, w, coef, scratch, nchunks, st);
    case ED_C128: return project_typed<double, true>(s, V, k, w, coef, scratch, nchunks, st);
    case ED_F32: return project_typed<float, false>(s, V, k, w, coef, scratch, nchunks, st);
    case ED_C64: return project_typed<float, true>(s, V, k, w, coef, scratch, nchunks, st);
    default: return set_error(ED_ERR_INVALID, "ed_project_out: dtype");
    }
}

// ------------------------------------------------------------ projection without allocation
//
// ed_project_out_noalloc: the projection with its scratch (the per-chunk partial dot products and
// the coefficients) in one fixed device array instead of the per-sector buffer that ed_project_out
// grows with cudaMalloc.  Every GPU that loads the library holds the array until the process ends.
// All calls share it, so calls that overlap on the GPU (different streams, or threads) race; the
// kernels write every partial and coefficient they later read, so nothing needs clearing between
// calls.

constexpr int kNoAllocMaxVectors = 256;  // largest k accepted
constexpr int kNoAllocMaxChunks = 256;   // partial sums per vector
constexpr int64_t kNoAllocScratchDoubles =
    (int64_t)kNoAllocMaxVectors * kNoAllocMaxChunks * kReduceSlots + 2 * kNoAllocMaxVectors;  // 2.1 MB

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Device address of the array in the current device's context.  Looked up on every call (a cheap
// host-side query, not a stream operation): a cached address would dangle once a context is torn down
// and the module reloaded elsewhere (host code may not use the symbol itself: on the host it names a
// stand-in, not device memory).
static int noalloc_scratch_address(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return set_cuda_error(e, "ed_project_out_noalloc: cudaGetSymbolAddress");
    *out = static_cast<double*>(p);
    return ED_OK;
}

int project_noalloc_launch(const Sector& s, int dtype, const void* V, int k, void* w, double* coef_out,
                           cudaStream_t st) {
    if (k < 0) return set_error(ED_ERR_INVALID, "ed_project_out_noalloc: k < 0");
    if (k > kNoAllocMaxVectors)
        return set_error(ED_ERR_TOO_LARGE, "ed_project_out_noalloc: k exceeds the fixed scratch (at most 256 vectors)");
    if (k == 0 || s.view.n == 0) return ED_OK;
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error(e, "ed_project_out_noalloc: cudaGetDevice");
    if (dev != s.device)
        return set_error(ED_ERR_INVALID, "ed_project_out_noalloc: the current device is not the sector's device");
    double* scratch = nullptr;
    if (int rc = noalloc_scratch_address(&scratch)) return rc;
    int nchunks = (int)std::min<int64_t>(kNoAllocMaxChunks, (s.view.n + 1023) / 1024);
    if (nchunks < 1) nchunks = 1;
    double* partials = scratch;
    double* coef = coef_out ? coef_out : scratch + (int64_t)kNoAllocMaxVectors * kNoAllocMaxChunks * kReduceSlots;
    switch (dtype) {
    case ED_F64: return project_typed<double, false>(s, V, k, w, coef, partials, nchunks, st);
    case ED_C128: return project_typed<double, true>(s, V, k, w, coef, partials, nchunks, st);
    case ED_F32: return project_typed<float, false>(s, V, k, w, coef, partials, nchunks, st);
    case ED_C64: return project_typed<float, true>(s, V, k, w, coef, partials, nchunks, st);
    default: return set_error(ED_ERR_INVALID, "ed_project_out_noalloc: dtype");
    }
}

}  // namespace ed
