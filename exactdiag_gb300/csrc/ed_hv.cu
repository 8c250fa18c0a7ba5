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
        hv_row_any<R, CPLX>(S, tb, w, W.faithful, i, x, yr, yi, xr, xi);
        st<R, CPLX>(y, i, yr, yi);
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

// Resident CTAs per SM of the plain H.v kernel (the largest shared-memory user).
int hv_blocks_per_sm(const SectorView& S) {
    const size_t smem = hv_smem_bytes(S, sizeof(double));
    cudaFuncSetAttribute(hv_kernel<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hv_kernel<double, true>, kHvThreads, smem) !=
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

// acc_i += c x_i as explicit fused multiply-adds in a fixed order, so that one vector at a time
// (accumulate_kernel) and several in one pass (accumulate_many_kernel) give the same bits.
template <typename R, bool CPLX>
__device__ __forceinline__ void acc_term(double& ar, double& ai, double cr, double ci, R xr, R xi) {
    ar = __fma_rn(cr, (double)xr, ar);
    if constexpr (CPLX) {
        ar = __fma_rn(-ci, (double)xi, ar);
        ai = __fma_rn(ci, (double)xr, __fma_rn(cr, (double)xi, ai));
    }
}

template <typename R, bool CPLX>
__global__ void accumulate_kernel(int64_t n, const void* __restrict__ x, double cr, double ci, void* __restrict__ acc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R xr, xi;
        ld<R, CPLX>(x, i, xr, xi);
        if constexpr (CPLX) {
            double2* a = reinterpret_cast<double2*>(acc) + i;
            double2 t = *a;
            acc_term<R, CPLX>(t.x, t.y, cr, ci, xr, xi);
            *a = t;
        } else {
            double* a = reinterpret_cast<double*>(acc) + i;
            double t = *a, unused = 0.0;
            acc_term<R, CPLX>(t, unused, cr, ci, xr, xi);
            *a = t;
        }
    }
}

// Up to kAccumMany vectors and their coefficients, passed by value.
struct AccumMany {
    const void* x[kAccumMany];
    double cr[kAccumMany], ci[kAccumMany];
    int k;
};

// acc_i += sum_j c_j x_{j,i}, the terms added in order j = 0, 1, ... exactly as k calls of
// accumulate_kernel would, reading and writing acc once.
template <typename R, bool CPLX>
__global__ void accumulate_many_kernel(int64_t n, const AccumMany m, void* __restrict__ acc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double ar, ai = 0.0;
        if constexpr (CPLX) {
            const double2 t = reinterpret_cast<const double2*>(acc)[i];
            ar = t.x;
            ai = t.y;
        } else {
            ar = reinterpret_cast<const double*>(acc)[i];
        }
        for (int j = 0; j < m.k; ++j) {
            R xr, xi;
            ld<R, CPLX>(m.x[j], i, xr, xi);
            acc_term<R, CPLX>(ar, ai, m.cr[j], m.ci[j], xr, xi);
        }
        if constexpr (CPLX) reinterpret_cast<double2*>(acc)[i] = make_double2(ar, ai);
        else reinterpret_cast<double*>(acc)[i] = ar;
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

int accumulate_many_launch(const Sector& s, int dtype, int k, const void* const* xs, const double* coefs, void* acc,
                           cudaStream_t st) {
    if (!dtype_ok(s, dtype)) return set_error(ED_ERR_INVALID, "ed_accumulate_many: dtype does not match the sector");
    if (s.view.n == 0 || k == 0) return ED_OK;
    const int g = grid_for(s.view.n, 256, s.num_sms, 16);
    for (int j0 = 0; j0 < k; j0 += kAccumMany) {
        AccumMany m{};
        m.k = std::min(kAccumMany, k - j0);
        for (int j = 0; j < m.k; ++j) {
            m.x[j] = xs[j0 + j];
            m.cr[j] = coefs[2 * (j0 + j)];
            m.ci[j] = coefs[2 * (j0 + j) + 1];
        }
        switch (dtype) {
        case ED_F64: accumulate_many_kernel<double, false><<<g, 256, 0, st>>>(s.view.n, m, acc); break;
        case ED_C128: accumulate_many_kernel<double, true><<<g, 256, 0, st>>>(s.view.n, m, acc); break;
        case ED_F32: accumulate_many_kernel<float, false><<<g, 256, 0, st>>>(s.view.n, m, acc); break;
        default: accumulate_many_kernel<float, true><<<g, 256, 0, st>>>(s.view.n, m, acc); break;
        }
        ED_CHECK_LAUNCH("accumulate_many_kernel");
    }
    return ED_OK;
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
