// ed_hv.cu -- matrix-free, pull-style H.v and the fused Lanczos step.
//
// Replaces the stored triangle matrices of the reference
// (general/cython_sparse_matrices.pyx:186-241, built column by column by
// general/column_functions.h:99-207 with the rules of
// tJ_spin_half_ladder/matrix_setup.pyx:80-110) and their SpMV
// (general/cpp_sparse_dot.h:59-138 via general/cython_sparse_dot.pyx:40-80).
//
// Every term matrix M_t is Hermitian, so row i of H is the conjugate of the
// column that the reference generates from representative i:
//     y_i = sum_t w_t * [ diag_t(i) x_i + sum_{bond b valid in i} conj(M_t[j(b), i]) x_{j(b)} ]
//     M_t[j, i] = c_t * sign_F * sqrt(N_i) * u^{e} / sqrt(N_j)
// with c_t = -1 for hopping (tl, tr) and +1/2 for exchange (jl, jr), diag = -1/2
// per antiparallel bond, sign_F = (-1)^{electrons strictly between the hop
// sites} (column_functions.h:317-346), u = exp(-i pi / L) and e the phase
// exponent of the lowest image of the new state (general/symmetry.h:97-126).
// One thread owns one row and writes y_i once: no atomics, deterministic.
//
// Bonds are generated bit-parallel from the row's masks.  For L = 2 the
// reference lists every leg bond twice ((x+1) and (x-1) coincide); iterating
// the two hop directions and all N leg-exchange start sites reproduces that.
//
// Lookup of the new state's dense row:
//   * hole-mask table (per hole mask): canonical block, the group element that
//     reaches it and its phase;
//   * free block (trivial stabiliser): every spin configuration is a
//     representative, orbit size 2L, dense row = block start + colex spin rank
//     (4 shared-memory table reads);
//   * other blocks: the reference's orbit walk on the packed key, then the
//     block's candidate bitmap + word prefix give the dense row (or "absent").
#include "ed_device.cuh"

namespace ed {

template <typename R, bool CPLX>
__global__ void __launch_bounds__(kHvThreads) hv_kernel(const SectorView S, HvWeights W, const void* __restrict__ x,
                                                        void* __restrict__ y) {
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<R> tb = load_tables<R>(S, smem);
    const R w[4] = {(R)W.w[0], (R)W.w[1], (R)W.w[2], (R)W.w[3]};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n; i += (int64_t)gridDim.x * blockDim.x) {
        R yr, yi, xr, xi;
        hv_row<R, CPLX>(S, tb, w, i, x, yr, yi, xr, xi);
        st<R, CPLX>(y, i, yr, yi);
    }
}

// Block reduction of kReduceSlots doubles into partials[blockIdx.x * kReduceSlots + k].
__device__ __forceinline__ void block_reduce_store(double v[kReduceSlots], double* __restrict__ partials) {
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
            if (lane == 0) partials[blockIdx.x * kReduceSlots + k] = t;
        }
    }
}

// Fused step, part 1: w = H v (kept implicit), y = w - b_k v_prev written to
// `y`; FP64 partial sums of <v, w>, |y|^2, <v, y>, |v|^2.
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kHvThreads)
    lanczos_hv_kernel(const SectorView S, HvWeights W, const void* __restrict__ v, const void* __restrict__ vprev,
                      void* __restrict__ y, const double* __restrict__ scal, double* __restrict__ partials) {
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<R> tb = load_tables<R>(S, smem);
    const R w[4] = {(R)W.w[0], (R)W.w[1], (R)W.w[2], (R)W.w[3]};
    const R beta = vprev ? (R)scal[0] : R(0);
    double acc[kReduceSlots] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n; i += (int64_t)gridDim.x * blockDim.x) {
        R hr, hi, xr, xi;
        hv_row<R, CPLX>(S, tb, w, i, v, hr, hi, xr, xi);
        R yr = hr, yi = hi;
        if (vprev) {
            R pr, pi;
            ld<R, CPLX>(vprev, i, pr, pi);
            yr -= beta * pr;
            yi -= beta * pi;
        }
        st<R, CPLX>(y, i, yr, yi);
        const double dxr = xr, dxi = xi, dyr = yr, dyi = yi;
        acc[0] = fma(dxr, (double)hr, fma(dxi, (double)hi, acc[0]));
        acc[1] = fma(dyr, dyr, fma(dyi, dyi, acc[1]));
        acc[2] = fma(dxr, dyr, fma(dxi, dyi, acc[2]));
        acc[3] = fma(dxr, dxr, fma(dxi, dxi, acc[3]));
    }
    block_reduce_store(acc, partials);
}

// Fused step, part 2 (one CTA): deterministic sum of the partials, a_k and b_{k+1}.
__global__ void lanczos_scalars_kernel(const double* __restrict__ partials, int nblocks, double* __restrict__ scal) {
    __shared__ double red[kReduceSlots][32];
    double s[kReduceSlots] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < kReduceSlots; ++k) s[k] += partials[b * kReduceSlots + k];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < kReduceSlots; ++k) {
        double t = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) red[k][wid] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot[kReduceSlots];
        for (int k = 0; k < kReduceSlots; ++k) {
            tot[k] = 0.0;
            for (int q = 0; q < nw; ++q) tot[k] += red[k][q];
        }
        const double a = tot[0];
        // |y - a v|^2 = |y|^2 - 2 a <v, y> + a^2 |v|^2
        const double nn = tot[1] - 2.0 * a * tot[2] + a * a * tot[3];
        const double b = sqrt(nn > 0.0 ? nn : 0.0);
        scal[1] = a;
        scal[2] = b;
        scal[3] = (b < 1e-8) ? 1.0 : 0.0;
    }
}

// Fused step, part 3: v_next = (y - a_k v) / b_{k+1}, elementwise.
template <typename R, bool CPLX>
__global__ void lanczos_update_kernel(int64_t n, const void* __restrict__ v, void* __restrict__ y_next,
                                      const double* __restrict__ scal) {
    const R a = (R)scal[1];
    const bool brk = scal[3] != 0.0;
    const R inv = brk ? R(1) : (R)(1.0 / scal[2]);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R vr, vi, yr, yi;
        ld<R, CPLX>(v, i, vr, vi);
        ld<R, CPLX>(y_next, i, yr, yi);
        st<R, CPLX>(y_next, i, (yr - a * vr) * inv, (yi - a * vi) * inv);
    }
}

template <typename R, bool CPLX>
__global__ void norm_partials_kernel(int64_t n, const void* __restrict__ x, double* __restrict__ partials) {
    double acc[kReduceSlots] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R xr, xi;
        ld<R, CPLX>(x, i, xr, xi);
        acc[0] = fma((double)xr, (double)xr, fma((double)xi, (double)xi, acc[0]));
    }
    block_reduce_store(acc, partials);
}

__global__ void norm_finish_kernel(const double* __restrict__ partials, int nblocks, double* __restrict__ norm) {
    __shared__ double red[32];
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[b * kReduceSlots];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < nw; ++q) t += red[q];
        norm[0] = sqrt(t);
    }
}

template <typename R, bool CPLX>
__global__ void scale_kernel(int64_t n, void* __restrict__ x, const double* __restrict__ norm) {
    const double nv = norm[0];
    const R inv = nv > 0.0 ? (R)(1.0 / nv) : R(0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R xr, xi;
        ld<R, CPLX>(x, i, xr, xi);
        st<R, CPLX>(x, i, xr * inv, xi * inv);
    }
}

// Continued fraction over the omega grid, one thread per omega, FP64 complex,
// bottom-up exactly as general/cython_lanczos_diagonalization.pyx:42-48.
__global__ void cf_kernel(const double* __restrict__ a, const double* __restrict__ b, int m,
                          const double* __restrict__ omega, int W, double e0, double eta, double factor,
                          double* __restrict__ out) {
    extern __shared__ double s_ab[];
    double* sa = s_ab;
    double* sb2 = s_ab + m;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        sa[i] = a[i];
        sb2[i] = b[i] * b[i];
    }
    __syncthreads();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < W; k += gridDim.x * blockDim.x) {
        const double zr = omega[k] + e0, zi = eta;
        double dr = zr - sa[m - 1], di = zi;
        for (int i = 1; i < m; ++i) {
            // det = z - a[m-1-i] - b[m-i]^2 / det
            const double den = dr * dr + di * di;
            const double qr = sb2[m - i] * dr / den, qi = -sb2[m - i] * di / den;
            dr = zr - sa[m - 1 - i] - qr;
            di = zi - qi;
        }
        const double den = dr * dr + di * di;
        out[k] = factor * (-di / den);
    }
}

// ------------------------------------------------------------------ launchers

// Resident CTAs per SM of the fused step kernel (the largest shared-memory user).
int hv_blocks_per_sm(const SectorView& S) {
    const size_t smem = hv_smem_bytes(S, sizeof(double));
    cudaFuncSetAttribute(lanczos_hv_kernel<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lanczos_hv_kernel<double, true>, kHvThreads, smem) !=
        cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return per_sm;
}

static bool dtype_ok(const Sector& s, int dtype) {
    if (dtype == ED_C128 || dtype == ED_C64) return true;
    if (dtype == ED_F64 || dtype == ED_F32) return s.real;
    return false;
}

template <typename R, bool CPLX>
static int hv_typed(const Sector& s, const HvWeights& w, const void* x, void* y, cudaStream_t st) {
    const size_t smem = hv_smem_bytes(s.view, sizeof(R));
    cudaFuncSetAttribute(hv_kernel<R, CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    hv_kernel<R, CPLX><<<s.hv_grid, kHvThreads, smem, st>>>(s.view, w, x, y);
    ED_CHECK_LAUNCH("hv_kernel");
    return ED_OK;
}

int hv_launch(const Sector& s, const HvWeights& w, int dtype, const void* x, void* y, cudaStream_t st) {
    if (!dtype_ok(s, dtype)) return set_error(ED_ERR_INVALID, "ed_hv: dtype does not match the sector");
    if (s.view.n == 0) return ED_OK;
    switch (dtype) {
    case ED_F64: return hv_typed<double, false>(s, w, x, y, st);
    case ED_C128: return hv_typed<double, true>(s, w, x, y, st);
    case ED_F32: return hv_typed<float, false>(s, w, x, y, st);
    default: return hv_typed<float, true>(s, w, x, y, st);
    }
}

template <typename R, bool CPLX>
static int step_hv_typed(const Sector& s, const HvWeights& w, const void* v, const void* vprev, void* vnext,
                         double* scal, double* partials, cudaStream_t st) {
    const size_t smem = hv_smem_bytes(s.view, sizeof(R));
    cudaFuncSetAttribute(lanczos_hv_kernel<R, CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    lanczos_hv_kernel<R, CPLX><<<s.hv_grid, kHvThreads, smem, st>>>(s.view, w, v, vprev, vnext, scal, partials);
    ED_CHECK_LAUNCH("lanczos_hv_kernel");
    lanczos_scalars_kernel<<<1, 256, 0, st>>>(partials, s.hv_grid, scal);
    ED_CHECK_LAUNCH("lanczos_scalars_kernel");
    return ED_OK;
}

template <typename R, bool CPLX>
static int step_update_typed(const Sector& s, const void* v, void* vnext, const double* scal, cudaStream_t st) {
    lanczos_update_kernel<R, CPLX><<<grid_for(s.view.n, 256, s.num_sms, 16), 256, 0, st>>>(s.view.n, v, vnext, scal);
    ED_CHECK_LAUNCH("lanczos_update_kernel");
    return ED_OK;
}

int lanczos_hv_launch(const Sector& s, const HvWeights& w, int dtype, const void* v, const void* vprev, void* vnext,
                      double* scal, double* partials, cudaStream_t st) {
    if (!dtype_ok(s, dtype)) return set_error(ED_ERR_INVALID, "ed_lanczos_step: dtype does not match the sector");
    if (s.view.n == 0) return set_error(ED_ERR_INVALID, "ed_lanczos_step: empty sector");
    switch (dtype) {
    case ED_F64: return step_hv_typed<double, false>(s, w, v, vprev, vnext, scal, partials, st);
    case ED_C128: return step_hv_typed<double, true>(s, w, v, vprev, vnext, scal, partials, st);
    case ED_F32: return step_hv_typed<float, false>(s, w, v, vprev, vnext, scal, partials, st);
    default: return step_hv_typed<float, true>(s, w, v, vprev, vnext, scal, partials, st);
    }
}

int lanczos_update_launch(const Sector& s, int dtype, const void* v, void* vnext, const double* scal, cudaStream_t st) {
    if (!dtype_ok(s, dtype)) return set_error(ED_ERR_INVALID, "ed_lanczos_update: dtype does not match the sector");
    if (s.view.n == 0) return ED_OK;
    switch (dtype) {
    case ED_F64: return step_update_typed<double, false>(s, v, vnext, scal, st);
    case ED_C128: return step_update_typed<double, true>(s, v, vnext, scal, st);
    case ED_F32: return step_update_typed<float, false>(s, v, vnext, scal, st);
    default: return step_update_typed<float, true>(s, v, vnext, scal, st);
    }
}

int lanczos_step_launch(const Sector& s, const HvWeights& w, int dtype, const void* v, const void* vprev, void* vnext,
                        double* scal, double* partials, cudaStream_t st) {
    int rc = lanczos_hv_launch(s, w, dtype, v, vprev, vnext, scal, partials, st);
    if (rc != ED_OK) return rc;
    return lanczos_update_launch(s, dtype, v, vnext, scal, st);
}

template <typename R, bool CPLX>
__global__ void accumulate_kernel(int64_t n, const void* __restrict__ x, double cr, double ci, void* __restrict__ acc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R xr, xi;
        ld<R, CPLX>(x, i, xr, xi);
        if constexpr (CPLX) {
            double2* a = reinterpret_cast<double2*>(acc) + i;
            double2 t = *a;
            t.x += cr * (double)xr - ci * (double)xi;
            t.y += cr * (double)xi + ci * (double)xr;
            *a = t;
        } else {
            reinterpret_cast<double*>(acc)[i] += cr * (double)xr;
        }
    }
}

int accumulate_launch(const Sector& s, int dtype, const void* x, double cr, double ci, void* acc, cudaStream_t st) {
    if (!dtype_ok(s, dtype)) return set_error(ED_ERR_INVALID, "ed_accumulate: dtype does not match the sector");
    if (s.view.n == 0) return ED_OK;
    const int g = grid_for(s.view.n, 256, s.num_sms, 16);
    switch (dtype) {
    case ED_F64: accumulate_kernel<double, false><<<g, 256, 0, st>>>(s.view.n, x, cr, ci, acc); break;
    case ED_C128: accumulate_kernel<double, true><<<g, 256, 0, st>>>(s.view.n, x, cr, ci, acc); break;
    case ED_F32: accumulate_kernel<float, false><<<g, 256, 0, st>>>(s.view.n, x, cr, ci, acc); break;
    default: accumulate_kernel<float, true><<<g, 256, 0, st>>>(s.view.n, x, cr, ci, acc); break;
    }
    ED_CHECK_LAUNCH("accumulate_kernel");
    return ED_OK;
}

template <typename R, bool CPLX>
static int norm_typed(const Sector& s, void* x, double* norm, double* partials, cudaStream_t st) {
    norm_partials_kernel<R, CPLX><<<s.hv_grid, kHvThreads, 0, st>>>(s.view.n, x, partials);
    ED_CHECK_LAUNCH("norm_partials_kernel");
    norm_finish_kernel<<<1, 256, 0, st>>>(partials, s.hv_grid, norm);
    ED_CHECK_LAUNCH("norm_finish_kernel");
    scale_kernel<R, CPLX><<<grid_for(s.view.n, 256, s.num_sms, 16), 256, 0, st>>>(s.view.n, x, norm);
    ED_CHECK_LAUNCH("scale_kernel");
    return ED_OK;
}

int normalize_launch(const Sector& s, int dtype, void* x, double* norm, double* partials, cudaStream_t st) {
    if (!dtype_ok(s, dtype)) return set_error(ED_ERR_INVALID, "ed_normalize: dtype does not match the sector");
    if (s.view.n == 0) return ED_OK;
    switch (dtype) {
    case ED_F64: return norm_typed<double, false>(s, x, norm, partials, st);
    case ED_C128: return norm_typed<double, true>(s, x, norm, partials, st);
    case ED_F32: return norm_typed<float, false>(s, x, norm, partials, st);
    default: return norm_typed<float, true>(s, x, norm, partials, st);
    }
}

int cf_launch(const double* a, const double* b, int m, const double* omega, int W, double e0, double eta, double norm2,
              double* out, cudaStream_t st) {
    if (m <= 0 || W < 0) return set_error(ED_ERR_INVALID, "ed_continued_fraction: bad sizes");
    if (W == 0) return ED_OK;
    const size_t smem = 2 * (size_t)m * sizeof(double);
    if (smem > 200 * 1024) return set_error(ED_ERR_TOO_LARGE, "ed_continued_fraction: too many coefficients");
    cudaFuncSetAttribute(cf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const double factor = -1.0 / 3.14159265358979323846 * norm2;
    cf_kernel<<<(W + 127) / 128, 128, smem, st>>>(a, b, m, omega, W, e0, eta, factor, out);
    ED_CHECK_LAUNCH("cf_kernel");
    return ED_OK;
}

}  // namespace ed
