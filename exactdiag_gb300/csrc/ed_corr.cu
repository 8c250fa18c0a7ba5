// ed_corr.cu -- hole and S^z position correlations of a state, one pass over the basis.
//
// Replaces tJ_spin_half_ladder/position_correlations.pyx:83-118
// (calculate_hole_spin_projection_correlations) and :174-195 (calculate_position_correlations):
//   corr[dist] = sum_i |psi_i|^2 sum_r value(state_i; r, rel(r, dist), shift_1(r), ...)
// over the representatives i (their own configurations, as the reference takes them) and every
// reference site r, with rel(r, dist) = get_index_by_relative_index (symmetry_ladder.h:88-95) and
// shift_k(r) = get_index_by_relative_shift(r, fixed_k) (:96-101).  value is 1 when every listed
// site holds a hole (get_holes_present_value, :200-207), or the product of the spin signs when
// none does (get_spin_projection_value, :188-198).
//
// Every listed position is "mirror the legs (b = 1) after translating by m rungs" of r, so the
// sum over r is a popcount: with P(x) the mask whose bit r is x's bit at that position,
//   holes: popc(h & P_dist(h) & P_1(h) & ...)
//   S^z:   popc(A) - 2 popc(A & (d ^ P_dist(d) ^ P_1(d) ^ ...)),  A = occ & P_dist(occ) & ...
// One thread per row, FP64 sums per thread and distance, a fixed-order block reduction and a
// fixed-order sum over blocks: the same bits on every run.  Singlet-singlet correlations
// (singlet_kernel below) evaluate <psi|O|psi> with O's columns from the reference's column rule.
#include <vector>

#include "ed_device.cuh"

namespace ed {

namespace {

constexpr int kCorrThreads = 256;
constexpr int kMaxFixed = 4;

struct CorrParams {
    int kind;  // 0 holes, 1 S^z
    int nfixed;
    int fm[kMaxFixed], fb[kMaxFixed];  // fixed positions: rungs to translate, leg mirror
};

// Bit r of the result is bit (translate r by m rungs, then mirror if b) of x.
__device__ __forceinline__ uint32_t permute(uint32_t x, int m, int b, int N, uint32_t mask) {
    const int s = 2 * m;
    uint32_t y = s ? (((x >> s) | (x << (N - s))) & mask) : x;
    if (b) y = ((y & 0x55555555u) << 1) | ((y >> 1) & 0x55555555u);
    return y & mask;
}

template <typename R, bool CPLX>
__global__ void __launch_bounds__(kCorrThreads)
    corr_kernel(const SectorView S, const CorrParams P, const void* __restrict__ psi, double* __restrict__ partials) {
    const int N = S.N;
    const uint32_t mask = S.mask;
    double acc[kMaxN];
#pragma unroll
    for (int t = 0; t < kMaxN; ++t) acc[t] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n; i += (int64_t)gridDim.x * blockDim.x) {
        R pr, pi;
        ld<R, CPLX>(psi, i, pr, pi);
        const double w = (double)pr * (double)pr + (CPLX ? (double)pi * (double)pi : 0.0);
        const uint64_t key = S.keys[i];
        const uint32_t h = (uint32_t)(key >> 32) & mask, d = (uint32_t)key & mask, occ = ~h & mask;
        const uint32_t base = P.kind == 0 ? h : occ;
        uint32_t fa = base, fd = d;
        for (int k = 0; k < P.nfixed; ++k) {
            fa &= permute(base, P.fm[k], P.fb[k], N, mask);
            fd ^= permute(d, P.fm[k], P.fb[k], N, mask);
        }
#pragma unroll
        for (int t = 0; t < kMaxN; ++t) {
            if (t >= N) break;
            const uint32_t a = fa & permute(base, t >> 1, t & 1, N, mask);
            int c = __popc(a);
            if (P.kind == 1) c -= 2 * __popc(a & (fd ^ permute(d, t >> 1, t & 1, N, mask)));
            if (c) acc[t] += w * (double)c;
        }
    }
    __shared__ double red[kCorrThreads / 32][kMaxN];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < kMaxN; ++t) {
        double v = acc[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wid][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < kMaxN) {
        double v = 0.0;
        for (int q = 0; q < kCorrThreads / 32; ++q) v += red[q][threadIdx.x];
        partials[(int64_t)blockIdx.x * kMaxN + threadIdx.x] = v;
    }
}

// get_index_by_relative_shift (symmetry_ladder.h:96-101): C++ remainder of the rung shift, then a
// positive modulo of the site.
__device__ __forceinline__ int rel_shift(int first, int sx, int sy, int N) {
    const int leg = first / 2 + sx;
    int rung = (first + (sy % 2)) % 2;
    if (rung < 0) rung += 2;
    int site = (2 * leg + rung) % N;
    return site < 0 ? site + N : site;
}

// Singlet-singlet correlations (tJ_spin_half_ladder/position_correlations.pyx:112-124 with the
// operator of matrix_setup.pyx:434-469): corr[t] = Re <psi| O(free_t) |psi>, O's column i by the
// reference's column rule (general/column_functions.h:99-207) from representative i, so
// <psi|O|psi> = sum_i psi_i sum_combos conj(psi_j) O[j, i].
template <typename R, bool CPLX>
__global__ void __launch_bounds__(kCorrThreads)
    singlet_kernel(const SectorView S, int f0x, int f0y, int f1x, int f1y, const void* __restrict__ psi,
                   double* __restrict__ partials) {
    extern __shared__ __align__(16) uint8_t smem[];
    const HvTables<double> tb = load_tables<double>(S, smem);
    const int N = S.N;
    const uint32_t mask = S.mask;
    const double w0 = 0.5 / (double)N;
    double acc[kMaxN];
#pragma unroll
    for (int t = 0; t < kMaxN; ++t) acc[t] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n; i += (int64_t)gridDim.x * blockDim.x) {
        R pr, pi;
        ld<R, CPLX>(psi, i, pr, pi);
        const uint64_t key = S.keys[i];
        const uint32_t h = (uint32_t)(key >> 32) & mask, d = (uint32_t)key & mask, occ = ~h & mask;
        const double sqNi = sqrt((double)S.orbit[i]);
#pragma unroll
        for (int t = 0; t < kMaxN; ++t) {
            if (t >= N) break;
            const int fsx = t >> 1, fsy = t & 1;
            double cr = 0.0, ci = 0.0;  // sum over combinations of conj(psi_j) O[j, i]
            for (int first = 0; first < N; ++first) {
                for (int e = 0; e < 2; ++e) {
                    // endpoint shift sets (f0, fs, f1 + fs) and (-f0, fs - f0, f1 + fs - f0)
                    const int sg = e ? -1 : 1;
                    int ind[4];
                    ind[0] = first;
                    ind[1] = rel_shift(first, sg * f0x, sg * f0y, N);
                    ind[2] = rel_shift(first, fsx - (e ? f0x : 0), fsy - (e ? f0y : 0), N);
                    ind[3] = rel_shift(first, f1x + fsx - (e ? f0x : 0), f1y + fsy - (e ? f0y : 0), N);
                    // is_valid_state_unequal_spins_2holes (matrix_element_functions.pyx:53-62)
                    if (ind[0] == ind[1]) continue;
                    if (!((occ >> ind[2]) & 1u) || !((occ >> ind[3]) & 1u)) continue;
                    if (((d >> ind[2]) & 1u) == ((d >> ind[3]) & 1u)) continue;
                    const bool h0 = ind[0] == ind[2] || ind[0] == ind[3] || ((h >> ind[0]) & 1u);
                    const bool h1 = ind[1] == ind[2] || ind[1] == ind[3] || ((h >> ind[1]) & 1u);
                    if (!h0 || !h1) continue;
                    // get_weights_annihilation_part_singlet_singlet (:84-95)
                    double wgt = ((d >> ind[2]) & 1u) ? -w0 : w0;
                    // count_commutations (column_functions.h:317-346): the last index acts first
                    int cnt = 0;
                    for (int k = 3; k >= 0; --k) {
                        const int r = ind[k];
                        cnt += __popc(occ & ((r == 31) ? 0u : (~0u << (r + 1))));
                        for (int k2 = k + 1; k2 < 4; ++k2) cnt += ind[k2] > r;
                    }
                    if (cnt & 1) wgt = -wgt;
                    // remove_two_add_up_down (:120-130): holes at 3 and 2, up at 1, down at 0
                    uint32_t h2 = h | (1u << ind[3]) | (1u << ind[2]);
                    uint32_t d2 = d & ~((1u << ind[3]) | (1u << ind[2]));
                    h2 &= ~(1u << ind[1]);
                    d2 &= ~(1u << ind[1]);
                    h2 &= ~(1u << ind[0]);
                    d2 |= 1u << ind[0];
                    const Resolved rv = resolve(S, tb.rank, tb.comb, h2, d2);
                    if (rv.j < 0) continue;
                    // O[j, i] = w sqrt(N_i) u^e / sqrt(N_j), u = exp(-i pi / L)
                    const double c = wgt * sqNi / sqrt((double)rv.nj);
                    double sp, cp;
                    sincospi((double)rv.e / (double)S.L, &sp, &cp);
                    R qr, qi;
                    ld<R, CPLX>(psi, rv.j, qr, qi);
                    // conj(psi_j) * c (cos - i sin)
                    const double ar = c * cp, ai = -c * sp;
                    cr += (double)qr * ar + (double)qi * ai;
                    ci += (double)qr * ai - (double)qi * ar;
                }
            }
            acc[t] += (double)pr * cr - (double)pi * ci;  // Re(psi_i * (cr + i ci))
        }
    }
    __shared__ double red[kCorrThreads / 32][kMaxN];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < kMaxN; ++t) {
        double v = acc[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wid][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < kMaxN) {
        double v = 0.0;
        for (int q = 0; q < kCorrThreads / 32; ++q) v += red[q][threadIdx.x];
        partials[(int64_t)blockIdx.x * kMaxN + threadIdx.x] = v;
    }
}

}  // namespace

int singlet_corr_launch(const Sector& s, int dtype, const void* psi, const int* fixed, double* out, cudaStream_t st) {
    const SectorView& V = s.view;
    if (!fixed) return set_error(ED_ERR_INVALID, "ed_singlet_correlations: NULL fixed distances");
    if (!V.holes) return set_error(ED_ERR_INVALID, "ed_singlet_correlations: the sector has no hole table");
    const int grid = 2 * s.num_sms;
    DevBuf<double> part((int64_t)grid * kMaxN);
    if (!part.ok()) return set_error(ED_ERR_NOMEM, "ed_singlet_correlations: scratch");
    const size_t smem = hv_smem_bytes(V, sizeof(double));
    switch (dtype) {
    case ED_F64:
        cudaFuncSetAttribute(singlet_kernel<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        singlet_kernel<double, false><<<grid, kCorrThreads, smem, st>>>(V, fixed[0], fixed[1], fixed[2], fixed[3], psi,
                                                                       part.p);
        break;
    case ED_C128:
        cudaFuncSetAttribute(singlet_kernel<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        singlet_kernel<double, true><<<grid, kCorrThreads, smem, st>>>(V, fixed[0], fixed[1], fixed[2], fixed[3], psi,
                                                                      part.p);
        break;
    default: return set_error(ED_ERR_INVALID, "ed_singlet_correlations: dtype must be ED_F64 or ED_C128");
    }
    ED_CHECK_LAUNCH("singlet_kernel");
    std::vector<double> h((size_t)grid * kMaxN);
    if (cudaMemcpyAsync(h.data(), part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return set_error(ED_ERR_CUDA, "ed_singlet_correlations: reading the sums");
    for (int t = 0; t < V.N; ++t) {
        double v = 0.0;
        for (int b = 0; b < grid; ++b) v += h[(size_t)b * kMaxN + t];
        out[t] = v;
    }
    return ED_OK;
}

int corr_launch(const Sector& s, int dtype, const void* psi, int kind, int nfixed, const int* fixed, double* out,
                cudaStream_t st) {
    const SectorView& V = s.view;
    if (kind != 0 && kind != 1) return set_error(ED_ERR_INVALID, "ed_position_correlations: kind must be 0 or 1");
    if (nfixed < 0 || nfixed > kMaxFixed || (nfixed && !fixed))
        return set_error(ED_ERR_INVALID, "ed_position_correlations: at most 4 fixed shifts");
    CorrParams P{};
    P.kind = kind;
    P.nfixed = nfixed;
    for (int k = 0; k < nfixed; ++k) {  // get_index_by_relative_shift: python_mod of the leg and rung shifts
        P.fm[k] = ((fixed[2 * k] % V.L) + V.L) % V.L;
        P.fb[k] = ((fixed[2 * k + 1] % 2) + 2) % 2;
    }
    const int grid = 2 * s.num_sms;
    DevBuf<double> part((int64_t)grid * kMaxN);
    if (!part.ok()) return set_error(ED_ERR_NOMEM, "ed_position_correlations: scratch");
    switch (dtype) {
    case ED_F64: corr_kernel<double, false><<<grid, kCorrThreads, 0, st>>>(V, P, psi, part.p); break;
    case ED_C128: corr_kernel<double, true><<<grid, kCorrThreads, 0, st>>>(V, P, psi, part.p); break;
    case ED_F32: corr_kernel<float, false><<<grid, kCorrThreads, 0, st>>>(V, P, psi, part.p); break;
    case ED_C64: corr_kernel<float, true><<<grid, kCorrThreads, 0, st>>>(V, P, psi, part.p); break;
    default: return set_error(ED_ERR_INVALID, "ed_position_correlations: dtype");
    }
    ED_CHECK_LAUNCH("corr_kernel");
    std::vector<double> h((size_t)grid * kMaxN);
    if (cudaMemcpyAsync(h.data(), part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return set_error(ED_ERR_CUDA, "ed_position_correlations: reading the sums");
    for (int t = 0; t < V.N; ++t) {
        double v = 0.0;
        for (int b = 0; b < grid; ++b) v += h[(size_t)b * kMaxN + t];
        out[t] = v;
    }
    return ED_OK;
}

}  // namespace ed
