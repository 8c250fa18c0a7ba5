// ed_excite.cu -- excitation operators applied pull-style from the target sector.
//
// Replaces the column-major operator matrices of
// tJ_spin_half_ladder/matrix_setup.pyx:195-374 (built by
// general/column_functions.h:150-207 and applied through
// general/sparse_matrices.py:83-105):
//   op 0  Szq:                     O = sum_r w_r S^z_r                  (matrix_setup.pyx:235-246)
//   op 1  spectral_function_minus: O = sum_r w_r c_{r,sigma}            (matrix_setup.pyx:302-325)
//   op 2  spectral_function_plus:  O = sum_r w_r c^+_{r,sigma}          (matrix_setup.pyx:281-300)
//   op 3  current_rung:            O = sum_r w_r c^+_{r'} c_r, r' the rung partner   (:248-263)
//   op 4  current_leg:             O = sum_r w_r (c^+_{r+x} c_r - c^+_{r-x} c_r)    (:265-279)
// with w_r = base * exp(-i q.r), base = 1/(2 sqrt(N)), 1/sqrt(N), 1/sqrt(N), i, i, q_y raised by
// one for current_rung (:251), and q.r evaluated per axis in single precision like get_q_dot_r
// (general/group/symmetry_generator.h:87-102).
//
// Row j of O is the conjugate of column j of the adjoint O^+, which the
// reference's column rule computes from the target representative t_j:
//   O[j, i] = sum_{r} w_r * sqrt(N_j) * conj(u^{e}/sqrt(N_i)) * s_r
// where the sum runs over the sites r at which O^+ acts on t_j (every occupied
// site for Szq, with s_r = +1 up / -1 down; every hole site for c_minus, with
// s_r = (-1)^{electrons of t_j above r} and the removed spin sigma re-added;
// every electron of spin sigma for c_plus, removed; for the currents every
// bond whose one end is a hole of t_j and whose other end holds the electron
// that hopped, moved back, with s_r = (-1)^{electrons strictly between} on the
// leg), and (i, N_i, e) is the representative of the resulting configuration in
// the source sector.  One thread per target row, no atomics.
#include "ed_device.cuh"

namespace ed {

struct ExciteParams {
    int op;
    int add_down;      // c_minus: the removed (pull: re-added) spin is down; c_plus: the added one is
    int qx, qy;
    double wr[kMaxN];  // w_r
    double wi[kMaxN];
};

template <typename R>
__global__ void __launch_bounds__(kHvThreads)
    excite_kernel(const SectorView T, const SectorView S, const ExciteParams P, const void* __restrict__ x,
                  void* __restrict__ y) {
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<R> tb = load_tables<R>(S, smem);  // source-sector rank tables
    const int N = T.N;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < T.n; j += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = T.keys[j];
        const uint32_t h = (uint32_t)(key >> 32), d = (uint32_t)key;
        const uint32_t occ = ~h & T.mask;
        const double sqNj = sqrt((double)T.orbit[j]);
        double accr = 0.0, acci = 0.0;
        if (P.op == 0) {
            const Resolved rv = resolve(S, tb.rank, tb.comb, h, d);
            if (rv.j >= 0) {
                double cr = 0.0, ci = 0.0;
                for (int r = 0; r < N; ++r) {
                    if (!((occ >> r) & 1u)) continue;
                    const double sgn = ((d >> r) & 1u) ? -1.0 : 1.0;
                    cr += sgn * P.wr[r];
                    ci += sgn * P.wi[r];
                }
                // conj(u^e / sqrt(N_i)) with u = exp(-i pi / L): exp(+i pi e / L)
                double sp, cp;
                sincospi((double)rv.e / (double)S.L, &sp, &cp);
                const double f = sqNj / sqrt((double)rv.nj);
                const double vr = f * (cr * cp - ci * sp), vi = f * (cr * sp + ci * cp);
                R xr, xi;
                ld<R, true>(x, rv.j, xr, xi);
                accr += vr * (double)xr - vi * (double)xi;
                acci += vr * (double)xi + vi * (double)xr;
            }
        } else {
            // one source configuration (h2, d2) reached by O^+ at site r (the operator's site in the
            // target frame, the startpoint for the currents), with its sign and endpoint weight
            auto add_term = [&](uint32_t h2, uint32_t d2, int r, double sgn) {
                const Resolved rv = resolve(S, tb.rank, tb.comb, h2, d2);
                if (rv.j < 0) return;
                // The reference evaluates this term from the source representative, at the site
                // rs = g(r) where g maps the new configuration to its lowest image, with w_rs rounded
                // in single precision; w_r = w_rs * exp(+i q.(rs - r)) exactly.
                const int shift = rv.p >> 1, mir = rv.p & 1;
                int rs = (mir ? (r ^ 1) : r) + 2 * shift;
                if (rs >= N) rs -= N;
                double sq, cq;
                sincospi(2.0 * (double)P.qx * (double)shift / (double)S.L + (double)(P.qy * mir), &sq, &cq);
                const double wr = P.wr[rs] * cq - P.wi[rs] * sq, wi = P.wr[rs] * sq + P.wi[rs] * cq;
                double sp, cp;
                sincospi((double)rv.e / (double)S.L, &sp, &cp);
                const double f = sgn * sqNj / sqrt((double)rv.nj);
                const double vr = f * (wr * cp - wi * sp), vi = f * (wr * sp + wi * cp);
                R xr, xi;
                ld<R, true>(x, rv.j, xr, xi);
                accr += vr * (double)xr - vi * (double)xi;
                acci += vr * (double)xi + vi * (double)xr;
            };
            auto above = [](int r) -> uint32_t { return (r == 31) ? 0u : (~0u << (r + 1)); };
            if (P.op == 1) {  // c_minus: re-add the removed electron at each hole
                for (uint32_t holes = h; holes; holes &= holes - 1u) {
                    const int r = __ffs(holes) - 1;
                    const uint32_t bit = 1u << r;
                    add_term(h ^ bit, P.add_down ? (d | bit) : d, r, (__popc(occ & above(r)) & 1) ? -1.0 : 1.0);
                }
            } else if (P.op == 2) {  // c_plus: remove the added electron at each site holding that spin
                for (uint32_t el = occ & (P.add_down ? d : ~d); el; el &= el - 1u) {
                    const int r = __ffs(el) - 1;
                    const uint32_t bit = 1u << r;
                    add_term(h | bit, d & ~bit, r, (__popc(occ & above(r)) & 1) ? -1.0 : 1.0);
                }
            } else {  // currents: the electron at `end` came from the hole `start`
                for (uint32_t holes = h; holes; holes &= holes - 1u) {
                    const int start = __ffs(holes) - 1;
                    const int nshift = P.op == 3 ? 1 : 2;
                    for (int k = 0; k < nshift; ++k) {
                        const int end = P.op == 3 ? (start ^ 1) : ((start + (k == 0 ? 2 : N - 2)) % N);
                        if (!((occ >> end) & 1u)) continue;
                        const uint32_t bs = 1u << start, be = 1u << end;
                        const uint32_t d2 = ((d >> end) & 1u) ? (d ^ be ^ bs) : d;
                        double sgn = k == 0 ? 1.0 : -1.0;  // endpoint weights (0, 1), (0, -1)
                        if (P.op == 4) {
                            const int lo = start < end ? start : end, hi = start < end ? end : start;
                            const uint32_t between = ((1u << hi) - 1u) & ~((2u << lo) - 1u);
                            if (__popc(occ & between) & 1) sgn = -sgn;
                        }
                        add_term(h ^ bs ^ be, d2, start, sgn);
                    }
                }
            }
        }
        st<R, true>(y, j, (R)accr, (R)acci);
    }
}

// general/group/symmetry_generator.h:87-102 get_q_dot_r: per-axis terms in
// single precision (int * int / float), summed in double, times 2 pi.
static double q_dot_r(int site, int qx, int qy, int L) {
    const int sx = site / 2, sy = site % 2;
    double acc = 0.0;
    acc += (double)((float)(qx * sx) / (float)L);
    acc += (double)((float)(qy * sy) / 2.0f);
    return acc * 2.0 * 3.14159265358979323846;
}

int excite_launch(const Sector& src, const Sector& dst, int op, int qx, int qy, int initial_sz2, int dtype,
                  const void* x, void* y, cudaStream_t st) {
    const SectorView& S = src.view;
    const SectorView& T = dst.view;
    if (S.L != T.L) return set_error(ED_ERR_INVALID, "ed_excitation_apply: sectors of different ladders");
    const int L = S.L;
    const int qye = op == 3 ? qy + 1 : qy;
    const int kx2 = (((src.kx_raw + qx + (L - 1) / 2) % L) + L) % L - (L - 1) / 2;
    const int ky2 = (((S.ky + qye) % 2) + 2) % 2;
    if (((kx2 % L) + L) % L != T.kx || ky2 != T.ky)
        return set_error(ED_ERR_INVALID, "ed_excitation_apply: target sector momentum does not match k + q");
    ExciteParams P{};
    P.op = op;
    P.qx = qx;
    P.qy = op == 3 ? qy + 1 : qy;  // current_rung (matrix_setup.pyx:251)
    double base;
    if (op == 0) {
        if (T.Nh != S.Nh || T.Nd != S.Nd) return set_error(ED_ERR_INVALID, "ed_excitation_apply: Szq keeps Nh, Nd");
        base = 0.5 / std::sqrt((double)S.N);
    } else if (op == 1) {
        P.add_down = initial_sz2 <= 0;
        if (T.Nh != S.Nh + 1 || T.Nd != S.Nd - (P.add_down ? 1 : 0))
            return set_error(ED_ERR_INVALID, "ed_excitation_apply: spectral_function_minus target must have one more "
                                             "hole and the removed spin");
        base = 1.0 / std::sqrt((double)S.N);
    } else if (op == 2) {
        P.add_down = initial_sz2 > 0;
        if (S.Nh < 1 || T.Nh != S.Nh - 1 || T.Nd != S.Nd + (P.add_down ? 1 : 0))
            return set_error(ED_ERR_INVALID, "ed_excitation_apply: spectral_function_plus target must have one hole "
                                             "less and the added spin");
        base = 1.0 / std::sqrt((double)S.N);
    } else if (op == 3 || op == 4) {
        if (T.Nh != S.Nh || T.Nd != S.Nd)
            return set_error(ED_ERR_INVALID, "ed_excitation_apply: currents keep Nh, Nd");
        base = 1.0;
    } else {
        return set_error(ED_ERR_INVALID, "ed_excitation_apply: unknown operator");
    }
    for (int r = 0; r < S.N; ++r) {
        const double qr = q_dot_r(r, qx, P.qy, L);
        if (op == 3 || op == 4) {  // i exp(-i q.r)
            P.wr[r] = std::sin(qr);
            P.wi[r] = std::cos(qr);
        } else {
            P.wr[r] = base * std::cos(qr);
            P.wi[r] = -base * std::sin(qr);
        }
    }
    if (T.n == 0) return ED_OK;
    if (dtype != ED_C128 && dtype != ED_C64)
        return set_error(ED_ERR_INVALID, "ed_excitation_apply: vectors must be complex (ED_C128 or ED_C64)");
    const int grid = grid_for(T.n, kHvThreads, dst.num_sms, 4);
    if (dtype == ED_C128) {
        const size_t smem = hv_smem_bytes(S, sizeof(double));
        cudaFuncSetAttribute(excite_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        excite_kernel<double><<<grid, kHvThreads, smem, st>>>(T, S, P, x, y);
    } else {
        const size_t smem = hv_smem_bytes(S, sizeof(float));
        cudaFuncSetAttribute(excite_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        excite_kernel<float><<<grid, kHvThreads, smem, st>>>(T, S, P, x, y);
    }
    ED_CHECK_LAUNCH("excite_kernel");
    return ED_OK;
}

}  // namespace ed
