// ed_device.cuh -- device-side pieces shared by the row kernels: shared-memory
// tables, typed vector access, the representative lookup and the H.v row.
#pragma once
#include "ed_internal.cuh"

namespace ed {

// Per-thread sums of products for the Lanczos dot products.  FP64 vectors: FP64 fused
// multiply-adds.  FP32 vectors: each product is split exactly into a float pair (fma gives the
// rounding error) and added with Knuth's TwoSum into a float-float sum, so a thread's partial
// sum carries about 48 bits.  The CTA reduction of a chunk stays in float-float (only its result
// is converted), and the reduction over chunks runs in FP64.  This keeps the FP64 units (a small
// fraction of the FP32 rate on this part) off the per-row and per-chunk paths.
template <typename R>
struct Accum;

template <>
struct Accum<double> {
    double s = 0.0;
    __device__ __forceinline__ void add_prod(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};

template <>
struct Accum<float> {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add_prod(float a, float b) {
        // explicit round-to-nearest operations: no contraction may merge the product into the sum
        const float p = __fmul_rn(a, b);
        const float pe = __fmaf_rn(a, b, -p);
        const float t = __fadd_rn(hi, p);
        const float bv = __fsub_rn(t, hi);
        const float te = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bv)), __fsub_rn(p, bv));
        lo = __fadd_rn(lo, __fadd_rn(te, pe));
        hi = t;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
    // this += o, both float-float (TwoSum of the high parts, low parts added to the error term)
    __device__ __forceinline__ void add(float ohi, float olo) {
        const float t = __fadd_rn(hi, ohi);
        const float bv = __fsub_rn(t, hi);
        const float te = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bv)), __fsub_rn(ohi, bv));
        const float e = __fadd_rn(te, __fadd_rn(lo, olo));
        hi = __fadd_rn(t, e);
        lo = __fsub_rn(e, __fsub_rn(hi, t));
    }
};

template <typename R>
struct HvTables {
    RankTab rank;          // shared
    const uint32_t* comb;  // shared
    const uint32_t* d2;    // shared: [(k * 32 + a) * 2 + mid] = C(a, k) + C(a + 1, k + mid), k <= Nd
    const R* cosv;         // cos(pi e / L), e in [0, 2L)
    const R* sinv;         // +sin(pi e / L): conj(u^e) = cos + i sin
    const R* sqrtv;        // sqrt(k), k in [0, 32]
    const R* rsqrtv;       // 1/sqrt(k)
};

template <typename R, bool CPLX>
struct Vec;
template <>
struct Vec<float, false> {
    using T = float;
};
template <>
struct Vec<float, true> {
    using T = float2;
};
template <>
struct Vec<double, false> {
    using T = double;
};
template <>
struct Vec<double, true> {
    using T = double2;
};

template <typename R, bool CPLX>
__device__ __forceinline__ void ld(const void* v, int64_t j, R& re, R& im) {
    using T = typename Vec<R, CPLX>::T;
    const T t = __ldg(reinterpret_cast<const T*>(v) + j);
    if constexpr (CPLX) {
        re = t.x;
        im = t.y;
    } else {
        re = t;
        im = R(0);
    }
}

template <typename R, bool CPLX>
__device__ __forceinline__ void st(void* v, int64_t j, R re, R im) {
    using T = typename Vec<R, CPLX>::T;
    if constexpr (CPLX) {
        T t;
        t.x = re;
        t.y = im;
        reinterpret_cast<T*>(v)[j] = t;
    } else {
        reinterpret_cast<T*>(v)[j] = re;
    }
}

// Dense row of representative spin mask `dr` in block B, or -1 when the
// configuration is not a representative of the sector.
__device__ __forceinline__ int64_t dense_in_block(const SectorView& S, const BlockInfo& B, uint32_t dr,
                                                  const RankTab& rank_tab) {
    const uint32_t r = spin_rank(compress_spins(dr, B.hmask), rank_tab, S.Nd);
    if (B.flags & kBlockFree) return B.start + (int64_t)r;
    const ulonglong2 bp = S.bitpref[B.word_off + (r >> 6)];
    const uint64_t bit = 1ull << (r & 63u);
    if (!(bp.x & bit)) return -1;
    return (int64_t)bp.y + __popcll(bp.x & (bit - 1ull));
}

struct Resolved {
    int64_t j;  // dense row of the representative, -1 if absent or incompatible
    int nj;     // orbit size of the new state
    int e;      // phase exponent (units of pi/L) of its lowest image
    int p;      // product index of the group element that gives the lowest image
};

// Representative of the configuration (h2, d2) in sector S: dense row, orbit
// size and phase exponent of the lowest image
// (general/symmetry.h:97-126 then general/basis_indexing.h:152-168).
__device__ __forceinline__ Resolved resolve(const SectorView& S, const RankTab& rank_tab, const uint32_t* comb,
                                            uint32_t h2, uint32_t d2) {
    const HoleEntry he = S.holes[hole_rank(h2, comb)];
    if (he.block < 0) return {-1, 0, 0, 0};
    const BlockInfo B = S.blocks[he.block];
    int nj, e, p;
    uint32_t dr;
    if (he.free_) {
        uint32_t hh = h2;
        dr = d2;
        apply_p(he.p_star, hh, dr, S.N, S.mask);
        nj = S.N;
        e = he.e_star;
        p = he.p_star;
    } else {
        const OrbitResult o = orbit_walk(S.L, S.kx, S.ky, S.ne_even, S.mask, h2, d2, false);
        if (o.found == 0) return {-1, 0, 0, 0};
        dr = (uint32_t)o.low;
        nj = o.found;
        e = o.e;
        p = o.p;
    }
    return {dense_in_block(S, B, dr, rank_tab), nj, e, p};
}

// Accumulate conj(M[j,i]) x_j for the new state (h2, d2); `coef` already holds
// w_t * c_t * sign_F * sqrt(N_i).
template <typename R, bool CPLX>
__device__ __forceinline__ void add_target(const SectorView& S, const HvTables<R>& tb, uint32_t h2, uint32_t d2, R coef,
                                           const void* __restrict__ x, R& accr, R& acci) {
    const Resolved rv = resolve(S, tb.rank, tb.comb, h2, d2);
    const int64_t j = rv.j;
    if (j < 0) return;
    const int nj = rv.nj, e = rv.e;
    const R c = coef * tb.rsqrtv[nj];
    R xr, xi;
    ld<R, CPLX>(x, j, xr, xi);
    if constexpr (CPLX) {
        const R pr = c * tb.cosv[e], pi = c * tb.sinv[e];
        accr += pr * xr - pi * xi;
        acci += pr * xi + pi * xr;
    } else {
        accr += (e == 0 ? c : -c) * xr;
    }
}

// Row i of H applied to x.  Returns (re, im) of (Hx)_i.
template <typename R, bool CPLX>
__device__ __forceinline__ void hv_row(const SectorView& S, const HvTables<R>& tb, const R w[4], int64_t i,
                                       const void* __restrict__ x, R& outr, R& outi, R& xir, R& xii) {
    const uint64_t key = S.keys[i];
    const uint32_t h = (uint32_t)(key >> 32), d = (uint32_t)key;
    const int N = S.N;
    const uint32_t mask = S.mask;
    const uint32_t occ = ~h & mask;
    const R sqNi = tb.sqrtv[S.orbit[i]];
    const HoleEntry hrow = S.holes[hole_rank(h, tb.comb)];
    const BlockInfo Brow = S.blocks[hrow.block];
    const bool row_free = hrow.free_;
    R accr = R(0), acci = R(0), diag = R(0);
    ld<R, CPLX>(x, i, xir, xii);

    // exchange: jl (leg bonds a -- a+2), jr (rung bonds 2x -- 2x+1)
#pragma unroll
    for (int t = 2; t < 4; ++t) {
        const R wt = w[t];
        if (wt == R(0)) continue;
        uint32_t m;
        int step;
        if (t == 2) {
            const uint32_t occ2 = rotl_n(occ, N - 2, N, mask), d2r = rotl_n(d, N - 2, N, mask);
            m = occ & occ2 & (d ^ d2r);
            step = 2;
        } else {
            m = occ & (occ >> 1) & (d ^ (d >> 1)) & 0x55555555u & mask;
            step = 1;
        }
        diag += R(-0.5) * wt * (R)__popc(m);
        const R coef = R(0.5) * wt * sqNi;
        while (m) {
            const int a = __ffs(m) - 1;
            m &= m - 1u;
            int b = a + step;
            if (b >= N) b -= N;
            const uint32_t d2 = d ^ (1u << a) ^ (1u << b);
            if (row_free) {
                // the row's hole mask is canonical with a trivial stabiliser: the new
                // state is its own representative, orbit 2L, phase 1.
                const int64_t j = Brow.start + (int64_t)spin_rank(compress_spins(d2, h), tb.rank, S.Nd);
                R xr, xi;
                ld<R, CPLX>(x, j, xr, xi);
                const R c = coef * tb.rsqrtv[N];
                accr += c * xr;
                if constexpr (CPLX) acci += c * xi;
            } else {
                add_target<R, CPLX>(S, tb, h, d2, coef, x, accr, acci);
            }
        }
    }
    // hopping: tl (a -> a +- 2 along the leg), tr (across the rung)
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const R wt = w[t];
        if (wt == R(0)) continue;
        const R coef = -wt * sqNi;
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
            uint32_t m;
            if (t == 0) {
                // electron at a, hole at a+2 (dir 0) or a-2 (dir 1)
                m = occ & (dir == 0 ? rotl_n(h, N - 2, N, mask) : rotl_n(h, 2 % N, N, mask));
            } else {
                m = dir == 0 ? (occ & (h >> 1) & 0x55555555u) : (occ & (h << 1) & 0xAAAAAAAAu & mask);
            }
            while (m) {
                const int a = __ffs(m) - 1;
                m &= m - 1u;
                int b;
                if (t == 0) {
                    b = dir == 0 ? a + 2 : a - 2;
                    if (b >= N) b -= N;
                    if (b < 0) b += N;
                } else {
                    b = dir == 0 ? a + 1 : a - 1;
                }
                const int lo = min(a, b), hi = max(a, b);
                const uint32_t between = ((1u << hi) - 1u) & ~((2u << lo) - 1u);
                const int sgn = (__popc(occ & between) & 1) ? -1 : 1;
                const uint32_t h2 = h ^ (1u << a) ^ (1u << b);
                const uint32_t d2 = ((d >> a) & 1u) ? (d ^ (1u << a) ^ (1u << b)) : d;
                add_target<R, CPLX>(S, tb, h2, d2, sgn > 0 ? coef : -coef, x, accr, acci);
            }
        }
    }
    outr = accr + diag * xir;
    outi = acci + diag * xii;
}


// ------------------------------------------------------------------ fast row (descriptors)

// Left rotation of an Ns-bit mask (0 <= r < Ns, 1 <= Ns <= 32): bits pushed above Ns by the
// left shift are the ones the right shift brings back in at the bottom, so both run in 32 bits.
__device__ __forceinline__ uint32_t rot_ns(uint32_t x, int r, int Ns) {
    const uint32_t m = 0xffffffffu >> (32 - Ns);
    return ((x << r) | (x >> ((Ns - r) & 31))) & m;
}

__device__ __forceinline__ uint32_t swap_pairs(uint32_t x, uint32_t m) {
    const uint32_t t = (x ^ (x >> 1)) & m;
    return x ^ t ^ (t << 1);
}

__device__ __forceinline__ uint32_t cand_image(const CandParams& c, uint32_t x, int Ns) {
    return rot_ns(swap_pairs(x, c.swap), c.rot, Ns);
}

// Lowest image among the coset candidates: its compressed mask, the number of candidates
// reaching it (the state's stabiliser order: orbit = 2L / count) and its phase; the state is
// incompatible with the sector when those candidates disagree in phase (the reference's
// amplitude tests, symmetry_ladder.h:196-224).
// Orbit size 2L / count of a state whose lowest image `count` coset candidates reach (count <= 4):
// shifts and a multiply in place of an integer division.
__device__ __forceinline__ int orbit_of_count(int N, int count) {
    return count == 1 ? N : (count == 2 ? (N >> 1) : (count == 4 ? (N >> 2) : ((N * 21846) >> 16)));
}

struct CandResult {
    uint32_t best;
    int count, e;
    bool valid;
};

// FIRST_IDENTITY: c[0] is the identity (a block's own stabiliser lists it first), so its image is x.
template <bool FIRST_IDENTITY = false>
__device__ __forceinline__ CandResult resolve_cand(const CandParams* c, int nc, uint32_t x, int Ns) {
    CandResult r{FIRST_IDENTITY ? x : cand_image(c[0], x, Ns), 1, c[0].e, true};
    for (int k = 1; k < nc; ++k) {
        const uint32_t img = cand_image(c[k], x, Ns);
        if (img < r.best) {
            r = {img, 1, c[k].e, true};
        } else if (img == r.best) {
            ++r.count;
            if (c[k].e != r.e) r.valid = false;
        }
    }
    return r;
}

// resolve_cand<true> over candidates held in registers (nc <= kMaxCand): the same rule, the same result.
__device__ __forceinline__ CandResult resolve_cand_held(const CandParams (&c)[kMaxCand], int nc, uint32_t x, int Ns) {
    CandResult r{x, 1, c[0].e, true};
#pragma unroll
    for (int k = 1; k < kMaxCand; ++k) {
        if (k >= nc) break;
        const uint32_t img = cand_image(c[k], x, Ns);
        if (img < r.best) {
            r = {img, 1, c[k].e, true};
        } else if (img == r.best) {
            ++r.count;
            if (c[k].e != r.e) r.valid = false;
        }
    }
    return r;
}

__device__ __forceinline__ int64_t bitmap_row(const SectorView& S, int64_t word_off, uint32_t r) {
    const ulonglong2 bp = S.bitpref[word_off + (r >> 6)];
    const uint64_t bit = 1ull << (r & 63u);
    if (!(bp.x & bit)) return -1;
    return (int64_t)bp.y + __popcll(bp.x & (bit - 1ull));
}

template <typename R, bool CPLX>
__device__ __forceinline__ void gather_add(const void* __restrict__ x, int64_t j, R c, int e, const HvTables<R>& tb,
                                           R& accr, R& acci) {
    R xr, xi;
    ld<R, CPLX>(x, j, xr, xi);
    if constexpr (CPLX) {
        const R pr = c * tb.cosv[e], pi = c * tb.sinv[e];
        accr += pr * xr - pi * xi;
        acci += pr * xi + pi * xr;
    } else {
        accr += (e == 0 ? c : -c) * xr;
    }
}

// Gathers of up to four targets issued together: the addresses first, then the loads, then the
// products, so a thread keeps several loads in flight (targets with j < 0 contribute nothing).
template <typename R, bool CPLX>
__device__ __forceinline__ void gather4(const void* __restrict__ x, const int64_t (&j)[4], const R (&c)[4],
                                        const int (&e)[4], const HvTables<R>& tb, R& accr, R& acci) {
    R xr[4], xi[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        if (j[u] >= 0) ld<R, CPLX>(x, j[u], xr[u], xi[u]);
        else xr[u] = xi[u] = R(0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        if constexpr (CPLX) {
            const R pr = c[u] * tb.cosv[e[u]], pi = c[u] * tb.sinv[e[u]];
            accr += pr * xr[u] - pi * xi[u];
            acci += pr * xi[u] + pi * xr[u];
        } else {
            accr += (e[u] == 0 ? c[u] : -c[u]) * xr[u];
        }
    }
}

// K gathers from one block: x_blk points at the block's first row, offsets are 32-bit rows
// inside it; slots whose bit in `live` is clear contribute nothing.
template <typename R, bool CPLX, int K>
__device__ __forceinline__ void gather_block(const typename Vec<R, CPLX>::T* __restrict__ xb,
                                             const uint32_t (&off)[K], unsigned live, const R (&c)[K],
                                             R& accr, R& acci) {
    R xr[K], xi[K];
#pragma unroll
    for (int u = 0; u < K; ++u) {
        if ((live >> u) & 1u) ld<R, CPLX>(xb, off[u], xr[u], xi[u]);
        else xr[u] = xi[u] = R(0);
    }
#pragma unroll
    for (int u = 0; u < K; ++u) {
        accr += c[u] * xr[u];
        if constexpr (CPLX) acci += c[u] * xi[u];
    }
}

// Exchange terms of a row whose neighbours are read from xb at the row's colex rank ri +- delta,
// delta the colex rank change of the swap: a free block's rows (every neighbour is a
// representative of the same block, orbit 2L, phase 1, at that row offset), or a stabiliser
// block's rows reading the block's expanded copy (ExpandTask).  Bonds are taken from the highest
// bit down, one find-leading-one each, in counted loops unrolled by four (FP32) or two (FP64):
// independent gathers in flight per thread.  UNI (rung and leg exchange weights equal): the x_j
// are summed with coefficient 1 and the sum scaled once; acc must be zero on entry.
template <typename R, bool CPLX, bool UNI>
__device__ __forceinline__ void free_exchange(const HvTables<R>& tb, const typename Vec<R, CPLX>::T* __restrict__ xb,
                                              uint32_t ri, uint32_t dc, uint32_t mr, uint32_t ma, uint32_t m2,
                                              uint32_t wrap_anti, const int (&wlo)[2], const int (&whi)[2], R cr,
                                              R cl, int Nd, R& accr, R& acci) {
    // unroll factor: four FP32 gathers in flight; two for FP64 (measured: fewer registers win there)
    constexpr int kUnroll = sizeof(R) == 4 ? 4 : 2;
    uint32_t m1 = (cr != R(0) ? mr : 0u) | (cl != R(0) ? ma : 0u);
    const int n1 = __popc(m1);
#pragma unroll kUnroll
    for (int q = 0; q < n1; ++q) {
        const int a = 31 - __clz(m1);
        const uint32_t bit = 1u << a;
        m1 ^= bit;
        const int k = __popc(dc & (bit - 1u));
        const uint32_t delta = tb.comb[k * kCombStride + a];
        const uint32_t o = (dc & bit) ? ri + delta : ri - delta;
        R xr, xi;
        ld<R, CPLX>(xb, o, xr, xi);
        if constexpr (UNI) {
            accr += xr;
            if constexpr (CPLX) acci += xi;
        } else {
            const R c = (mr & bit) ? cr : cl;
            accr += c * xr;
            if constexpr (CPLX) acci += c * xi;
        }
    }
    uint32_t mm = cl != R(0) ? m2 : 0u;
    const int n2 = __popc(mm);
#pragma unroll kUnroll
    for (int q = 0; q < n2; ++q) {
        const int a = 31 - __clz(mm);
        const uint32_t bit = 1u << a;
        mm ^= bit;
        const int k = __popc(dc & (bit - 1u));
        const int mid = (dc >> (a + 1)) & 1u;
        const uint32_t delta = tb.d2[(k * 32 + a) * 2 + mid];
        const uint32_t o = (dc & bit) ? ri + delta : ri - delta;
        R xr, xi;
        ld<R, CPLX>(xb, o, xr, xi);
        const R c = UNI ? R(1) : cl;
        accr += c * xr;
        if constexpr (CPLX) acci += c * xi;
    }
    if (cl != R(0) && wrap_anti) {
        uint32_t offw[2];
        R cw[2];
        unsigned live = 0;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            offw[u] = ri;
            cw[u] = UNI ? R(1) : R(0);
            if ((wrap_anti >> u) & 1u) {
                offw[u] = spin_rank(dc ^ (1u << wlo[u]) ^ (1u << whi[u]), tb.rank, Nd);
                if constexpr (!UNI) cw[u] = cl;
                live |= 1u << u;
            }
        }
        gather_block<R, CPLX, 2>(xb, offw, live, cw, accr, acci);
    }
    if constexpr (UNI) {
        accr *= cl;
        if constexpr (CPLX) acci *= cl;
    }
}

// A hop of the rows of one block with everything that is the same for all of them folded in,
// built once per chunk from the block's HopDesc and the weights (build_block_hops): the move of
// the electron in compressed coordinates, the coset permutation of a free target, and the
// coefficient w * sign (times sqrt(2L) for rows of a free block, whose orbit is 2L; rows of a
// stabiliser block multiply by sqrt of their own orbit).  For a free target the coefficient also
// holds 1 / sqrt(2L) and the target's phase; for a stabiliser target the orbit and phase of the
// target are resolved per row (coset candidates and bitmap word).
// Every field is a full word, read as four 16-byte words without unpacking.
template <typename R>
struct alignas(16) BlockHop {
    uint32_t keep;    // bits of the compressed mask that stay in place: ~(band | 1 << p)
    uint32_t band;    // bits that shift by one position toward p
    uint32_t sl, sr;  // moved = ((dc & band) << sl) >> sr
    uint32_t p, q;    // the electron's compressed position before and after
    uint32_t swap;    // target coset permutation (free targets): mirror pairs
    uint32_t rot;     // and left rotation by rot ...
    uint32_t nsr;     // ... as (x << rot | x >> nsr) & mask, nsr = (Ns - rot) % 32
    uint32_t mode;    // kModeFree / kModeCand / kModeAbsent (weight zero)
    int64_t start;    // target block's first row (free targets)
    R cr, ci;         // coefficient, real and imaginary parts
};
static_assert(sizeof(BlockHop<float>) == 64 && sizeof(BlockHop<double>) == 64, "BlockHop is four 16-byte words");

// BlockHop mode of a free target reached without a coset permutation (rot = 0, no mirror pairs)
// by a move of at most one compressed position, from a row of a free block: the target's spin
// rank is the row's own rank (its offset in the block) plus the rank change of one adjacent swap.
constexpr uint32_t kHopDelta = 4;

template <typename R, bool CPLX>
__device__ __forceinline__ void build_block_hop(const HopDesc& H, const HvTables<R>& tb, const R w[4], int Ns, int N,
                                                bool row_free, BlockHop<R>& F) {
    const R wt = H.term ? w[1] : w[0];
    uint32_t mode = wt == R(0) ? (uint32_t)kModeAbsent : (uint32_t)H.mode;
    const int dpq = (int)H.p - (int)H.q;
    if (row_free && mode == kModeFree && H.rot == 0 && H.swap == 0 && dpq >= -1 && dpq <= 1 &&
        H.band == (dpq == 0 ? 0u : (1u << H.q)))
        mode = kHopDelta;
    const uint32_t sl = H.q > H.p ? 0u : 1u;
    F.keep = ~(H.band | (1u << H.p));
    F.band = H.band;
    F.sl = sl;
    F.sr = 1u - sl;
    F.p = H.p;
    F.q = H.q;
    F.swap = H.swap;
    F.rot = H.rot;
    F.nsr = (uint32_t)((Ns - H.rot) & 31);
    F.mode = mode;
    F.start = H.start;
    const R sw = (uint8_t)H.sign == 1u ? -wt : wt;
    const R base = row_free ? sw * tb.sqrtv[N] : sw;
    if (mode == kModeFree || mode == kHopDelta) {
        const R c = base * tb.rsqrtv[N];
        if constexpr (CPLX) {
            F.cr = c * tb.cosv[H.e];
            F.ci = c * tb.sinv[H.e];
        } else {
            F.cr = H.e == 0 ? c : -c;
            F.ci = R(0);
        }
    } else {
        F.cr = base;
        F.ci = R(0);
    }
}

// The hops of a chunk's block (threads 0 .. nhop-1 build one each; the caller synchronises).
template <typename R, bool CPLX>
__device__ __forceinline__ void build_block_hops(const BlockDesc& D, const HvTables<R>& tb, const R w[4], int Ns, int N,
                                                 bool row_free, BlockHop<R>* shop) {
    if (threadIdx.x < D.nhop) build_block_hop<R, CPLX>(D.hop[threadIdx.x], tb, w, Ns, N, row_free, shop[threadIdx.x]);
}

// Gathers of up to K targets with their coefficients already multiplied by the phase.
template <typename R, bool CPLX, int K>
__device__ __forceinline__ void gather_kc(const void* __restrict__ x, const int64_t (&j)[K], const R (&cr)[K],
                                          const R (&ci)[K], R& accr, R& acci) {
    R xr[K], xi[K];
#pragma unroll
    for (int u = 0; u < K; ++u) {
        if (j[u] >= 0) ld<R, CPLX>(x, j[u], xr[u], xi[u]);
        else xr[u] = xi[u] = R(0);
    }
#pragma unroll
    for (int u = 0; u < K; ++u) {
        if constexpr (CPLX) {
            accr += cr[u] * xr[u] - ci[u] * xi[u];
            acci += cr[u] * xi[u] + ci[u] * xr[u];
        } else {
            accr += cr[u] * xr[u];
        }
    }
}

// Hops of a row, four (FP32) or two (FP64) at a time, from the pre-built BlockHop records.
// ROW_FREE: the row's orbit (2L) is folded into the records; otherwise every coefficient is scaled
// by sqNi = sqrt(orbit).
// ri: the row's offset in its block (= its spin rank), used by kHopDelta records (free rows only).
template <typename R, bool CPLX, bool ROW_FREE>
__device__ __forceinline__ void block_hops(const SectorView& S, const HvTables<R>& tb, const BlockDesc* __restrict__ D,
                                           const BlockHop<R>* __restrict__ shop, int nhop, uint32_t dc, uint32_t ri,
                                           int Ns, R sqNi, const void* __restrict__ x, R& accr, R& acci) {
    const uint32_t nsmask = 0xffffffffu >> (32 - Ns);
    constexpr int kB = sizeof(R) == 4 ? 4 : 2;  // targets in flight: four FP32, two FP64
#pragma unroll 1
    for (int t0 = 0; t0 < nhop; t0 += kB) {
        int64_t jj[kB];
        R cr[kB], ci[kB];
#pragma unroll
        for (int u = 0; u < kB; ++u) {
            jj[u] = -1;
            cr[u] = ci[u] = R(0);
            const int t = t0 + u;
            if (t >= nhop) continue;
            const BlockHop<R>& F = shop[t];
            const uint4 f0 = reinterpret_cast<const uint4*>(&F)[0];  // keep, band, sl, sr
            const uint4 f1 = reinterpret_cast<const uint4*>(&F)[1];  // p, q, swap, rot
            const uint4 f2 = reinterpret_cast<const uint4*>(&F)[2];  // nsr, mode, start
            if (f2.y == kModeAbsent) continue;
            if (ROW_FREE && f2.y == kHopDelta) {
                // adjacent swap of compressed positions p, q (or none when p == q)
                const uint32_t lo = min(f1.x, f1.y);
                const uint32_t bit = 1u << lo;
                uint32_t r = ri;
                if (((dc >> f1.x) ^ (dc >> f1.y)) & 1u) {
                    const uint32_t delta = tb.comb[__popc(dc & (bit - 1u)) * kCombStride + lo];
                    r = (dc & bit) ? ri + delta : ri - delta;
                }
                jj[u] = (int64_t)(((uint64_t)f2.w << 32) | f2.z) + (int64_t)r;
                cr[u] = F.cr;
                ci[u] = F.ci;
                continue;
            }
            const uint32_t moved = ((dc & f0.y) << f0.z) >> f0.w;
            const uint32_t dcm = (dc & f0.x) | moved | (((dc >> f1.x) & 1u) << f1.y);
            if (f2.y == kModeFree) {
                const uint32_t sw = swap_pairs(dcm, f1.z);
                const uint32_t dct = ((sw << f1.w) | (sw >> f2.x)) & nsmask;
                jj[u] = (int64_t)(((uint64_t)f2.w << 32) | f2.z) + (int64_t)spin_rank(dct, tb.rank, S.Nd);
                cr[u] = ROW_FREE ? F.cr : F.cr * sqNi;
                ci[u] = ROW_FREE ? F.ci : F.ci * sqNi;
            } else {
                // stabiliser target: lowest coset image, its orbit and phase, then the bitmap
                const HopDesc& H = D->hop[t];
                const CandResult c2 = resolve_cand(H.cand, H.ncand, dcm, Ns);
                if (!c2.valid) continue;
                const int64_t j = bitmap_row(S, H.word_off, spin_rank(c2.best, tb.rank, S.Nd));
                if (j < 0) continue;
                R c = F.cr * tb.rsqrtv[orbit_of_count(S.N, c2.count)];
                if constexpr (!ROW_FREE) c *= sqNi;
                jj[u] = j;
                if constexpr (CPLX) {
                    cr[u] = c * tb.cosv[c2.e];
                    ci[u] = c * tb.sinv[c2.e];
                } else {
                    cr[u] = c2.e == 0 ? c : -c;
                }
            }
        }
        gather_kc<R, CPLX, kB>(x, jj, cr, ci, accr, acci);
    }
}

// Row i of H via the block descriptor D (the row's own block): free blocks move in dense-row
// space directly (colex rank deltas), hops and non-free blocks go through the precomputed coset
// permutations.  Rows of blocks marked generic take hv_row.
// XIN: the caller has already loaded x_i into (xir, xii).
// shop: the block's pre-built hops (kind-specialised rows, ROWS != 0); xfull: the block's expanded
// copy (ExpandTask), read by the stabiliser-row kernel (ROWS == kRowsCand).
template <typename R, bool CPLX, int ROWS = 0, bool XIN = false>
__device__ __forceinline__ void hv_row_fast(const SectorView& S, const HvTables<R>& tb, const R w[4], int64_t i,
                                            uint64_t key, const BlockDesc* __restrict__ D,
                                            const void* __restrict__ x, R& outr, R& outi, R& xir, R& xii,
                                            const BlockHop<R>* __restrict__ shop = nullptr,
                                            const void* __restrict__ xfull = nullptr) {
    const uint32_t h = (uint32_t)(key >> 32), d = (uint32_t)key;
    const int Ns = S.Ns, N = S.N;
    if constexpr (!XIN) ld<R, CPLX>(x, i, xir, xii);
    const uint32_t dc = compress_spins(d, h);
    // hot words of the descriptor: {hmask, m_rung, m_legadj, m_legd2}, {mode|nhop|ncand|nwrap, wrap, start}
    const uint4 dw0 = reinterpret_cast<const uint4*>(D)[0];
    const uint4 dw1 = reinterpret_cast<const uint4*>(D)[1];
    // ROWS: 0 decides per row from the descriptor; kRowsFree / kRowsCand fix the block kind at compile time
    const bool row_free = ROWS == 0 ? ((dw1.x & 255u) == kModeFree) : (ROWS == kRowsFree);
    const int nhop = (dw1.x >> 8) & 255u, nwrap = dw1.x >> 24;
    const int wlo[2] = {(int)(dw1.y & 255u), (int)((dw1.y >> 16) & 255u)};
    const int whi[2] = {(int)((dw1.y >> 8) & 255u), (int)(dw1.y >> 24)};
    const int64_t dstart = (int64_t)(((uint64_t)dw1.w << 32) | dw1.z);
    const int Ni = row_free ? N : (int)S.orbit[i];
    const R sqNi = tb.sqrtv[Ni];
    R accr = R(0), acci = R(0);
    // exchange bonds (jl, jr)
    const uint32_t dif1 = dc ^ (dc >> 1), dif2 = dc ^ (dc >> 2);
    const uint32_t mr = dw0.y & dif1, ma = dw0.z & dif1, m2 = dw0.w & dif2;
    uint32_t wrap_anti = 0;
#pragma unroll
    for (int t = 0; t < 2; ++t)
        if (t < nwrap) wrap_anti |= (((dc >> wlo[t]) ^ (dc >> whi[t])) & 1u) << t;
    const R wl = w[2], wr = w[3];
    const R diag = R(-0.5) * (wr * (R)__popc(mr) + wl * (R)(__popc(ma) + __popc(m2) + __popc(wrap_anti)));
    int64_t jj[4];
    R cc[4];
    int ee[4] = {0, 0, 0, 0};
    if (row_free) {
        // every neighbour in the block is a representative with orbit 2L and phase 1: y += w/2 x_j,
        // at row i + delta of the same block (32-bit offsets from the block's first row)
        const R cr = R(0.5) * wr, cl = R(0.5) * wl;
        const typename Vec<R, CPLX>::T* xb = reinterpret_cast<const typename Vec<R, CPLX>::T*>(x) + dstart;
        const uint32_t ri = (uint32_t)(i - dstart);
        if (cr == cl) free_exchange<R, CPLX, true>(tb, xb, ri, dc, mr, ma, m2, wrap_anti, wlo, whi, cr, cl, S.Nd, accr, acci);
        else free_exchange<R, CPLX, false>(tb, xb, ri, dc, mr, ma, m2, wrap_anti, wlo, whi, cr, cl, S.Nd, accr, acci);
    } else {
        // non-free block: each exchange target is resolved through the block's stabiliser (lowest
        // image, orbit, phase agreement), then its bitmap word
        const int ncand = (dw1.x >> 16) & 255u;
        const int64_t word_off = D->word_off;
        const R cr = R(0.5) * wr * sqNi, cl = R(0.5) * wl * sqNi;
        if constexpr (ROWS == kRowsCand) {
            // the block's expanded copy holds every spin configuration's resolved value: its rows
            // read exchange targets like a free block's, at the row's own colex rank +- delta
            const typename Vec<R, CPLX>::T* xb = reinterpret_cast<const typename Vec<R, CPLX>::T*>(xfull);
            const uint32_t rr = spin_rank(dc, tb.rank, S.Nd);
            if (cr == cl) free_exchange<R, CPLX, true>(tb, xb, rr, dc, mr, ma, m2, wrap_anti, wlo, whi, cr, cl, S.Nd, accr, acci);
            else free_exchange<R, CPLX, false>(tb, xb, rr, dc, mr, ma, m2, wrap_anti, wlo, whi, cr, cl, S.Nd, accr, acci);
        }
#pragma unroll 1
        for (int kind = 0; kind < (ROWS == kRowsCand ? 0 : 4); ++kind) {
            uint32_t m;
            int dist;
            R coef;
            if (kind == 0) { m = mr; dist = 1; coef = cr; }
            else if (kind == 1) { m = ma; dist = 1; coef = cl; }
            else if (kind == 2) { m = m2; dist = 2; coef = cl; }
            else { m = wrap_anti; dist = 0; coef = cl; }
            if (coef == R(0)) continue;
            while (m) {
                const int a = __ffs(m) - 1;
                m &= m - 1u;
                const uint32_t flip = dist ? ((1u << a) | (1u << (a + dist)))
                                           : ((1u << (a ? wlo[1] : wlo[0])) | (1u << (a ? whi[1] : whi[0])));
                const CandResult cr2 = resolve_cand<true>(D->cand, ncand, dc ^ flip, Ns);
                if (!cr2.valid) continue;
                const int64_t j = bitmap_row(S, word_off, spin_rank(cr2.best, tb.rank, S.Nd));
                if (j < 0) continue;
                gather_add<R, CPLX>(x, j, coef * tb.rsqrtv[orbit_of_count(N, cr2.count)], cr2.e, tb, accr, acci);
            }
        }
    }
    if constexpr (ROWS != 0) {
        block_hops<R, CPLX, ROWS == kRowsFree>(S, tb, D, shop, nhop, dc, (uint32_t)(i - dstart), Ns, sqNi, x, accr,
                                               acci);
    } else {
        // hops (tl, tr), four at a time
#pragma unroll 1
        for (int t0 = 0; t0 < nhop; t0 += 4) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                jj[u] = -1;
                cc[u] = R(0);
                ee[u] = 0;
                const int t = t0 + u;
                if (t >= nhop) continue;
                const HopDesc& H = D->hop[t];
                // hot words: {band, swap, p|q|rot|e, term|mode|ncand|sign}, {start, word_off}
                const uint4 hw = reinterpret_cast<const uint4*>(&H)[0];
                const uint32_t hmode = (hw.w >> 8) & 255u;
                const R wt = (hw.w & 255u) ? w[1] : w[0];
                if (wt == R(0) || hmode == kModeAbsent) continue;
                const R coef = ((hw.w >> 24) == 1u ? -wt : wt) * sqNi;
                // (blocks with such hops are orbit-walk blocks: the kind-specialised kernels never see one)
                if (ROWS == 0 && hmode == kModeGeneric) {
                    const uint32_t h2 = h ^ (1u << H.a) ^ (1u << H.b);
                    const uint32_t d2 = ((d >> H.a) & 1u) ? (d ^ (1u << H.a) ^ (1u << H.b)) : d;
                    add_target<R, CPLX>(S, tb, h2, d2, coef, x, accr, acci);
                    continue;
                }
                const uint4 hw1 = reinterpret_cast<const uint4*>(&H)[1];
                const int p = hw.z & 255u, q = (hw.z >> 8) & 255u;
                const uint32_t band = hw.x;
                const uint32_t moved = (q > p) ? ((dc & band) >> 1) : ((dc & band) << 1);
                const uint32_t dcm = (dc & ~(band | (1u << p))) | moved | (((dc >> p) & 1u) << q);
                if (hmode == kModeFree) {
                    const uint32_t dct = rot_ns(swap_pairs(dcm, hw.y), (hw.z >> 16) & 255u, Ns);
                    jj[u] = (int64_t)(((uint64_t)hw1.y << 32) | hw1.x) + (int64_t)spin_rank(dct, tb.rank, S.Nd);
                    cc[u] = coef * tb.rsqrtv[N];
                    ee[u] = hw.z >> 24;
                } else {
                    const CandResult cr2 = resolve_cand(H.cand, (hw.w >> 16) & 255u, dcm, Ns);
                    if (!cr2.valid) continue;
                    const int64_t j =
                        bitmap_row(S, (int64_t)(((uint64_t)hw1.w << 32) | hw1.z), spin_rank(cr2.best, tb.rank, S.Nd));
                    if (j < 0) continue;
                    jj[u] = j;
                    cc[u] = coef * tb.rsqrtv[orbit_of_count(N, cr2.count)];
                    ee[u] = cr2.e;
                }
            }
            gather4<R, CPLX>(x, jj, cc, ee, tb, accr, acci);
        }
    }
    outr = accr + diag * xir;
    outi = acci + diag * xii;
}

// Descriptor of the row's block: the chunk's staged copy when the hole masks agree, else the table.
__device__ __forceinline__ const BlockDesc* row_desc(const SectorView& S, const uint32_t* comb, uint32_t h,
                                                     const BlockDesc* staged) {
    if (staged && staged->hmask == h) return staged;
    return S.desc + S.holes[hole_rank(h, comb)].block;
}

template <typename R, bool CPLX>
__device__ __forceinline__ void hv_row_any(const SectorView& S, const HvTables<R>& tb, const R w[4], int faithful,
                                           int64_t i, const void* __restrict__ x, R& outr, R& outi, R& xir, R& xii,
                                           const BlockDesc* staged = nullptr) {
    if (faithful || S.desc == nullptr) {
        hv_row<R, CPLX>(S, tb, w, i, x, outr, outi, xir, xii);
        return;
    }
    const uint64_t key = S.keys[i];
    const BlockDesc* D = row_desc(S, tb.comb, (uint32_t)(key >> 32), staged);
    if (D->mode == kModeGeneric) hv_row<R, CPLX>(S, tb, w, i, x, outr, outi, xir, xii);
    else hv_row_fast<R, CPLX>(S, tb, w, i, key, D, x, outr, outi, xir, xii);
}

// Stage one block descriptor in shared memory (all threads of the CTA call this).
__device__ __forceinline__ void stage_block(const BlockDesc* __restrict__ src, BlockDesc* sdesc) {
    __syncthreads();  // the previous chunk's rows are done with sdesc
    const int words = (int)(sizeof(BlockDesc) / sizeof(uint4));
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(sdesc);
    for (int t = threadIdx.x; t < words; t += blockDim.x) d4[t] = s4[t];
    __syncthreads();
}

template <typename R>
__device__ HvTables<R> load_tables(const SectorView& S, uint8_t* smem) {
    uint32_t* s_rank = reinterpret_cast<uint32_t*>(smem);
    const int tab_words = S.rank_words;
    uint32_t* s_comb = s_rank + ((tab_words + 1) & ~1);
    uint32_t* s_d2 = s_comb + kCombStride * kCombStride + 1;  // 8-byte aligned (odd count + 1)
    const int d2_words = (S.Nd + 1) * 64;
    R* s_f = reinterpret_cast<R*>(s_d2 + d2_words);
    R* s_cos = s_f;
    R* s_sin = s_f + 64;
    R* s_sqrt = s_f + 128;
    R* s_rsqrt = s_f + 161;
    for (int i = threadIdx.x; i < tab_words; i += blockDim.x) s_rank[i] = S.rank_tab[i];
    for (int i = threadIdx.x; i < kCombStride * kCombStride; i += blockDim.x) s_comb[i] = S.comb[i];
    for (int i = threadIdx.x; i < d2_words; i += blockDim.x) {
        const int k = i >> 6, a = (i >> 1) & 31, mid = i & 1;
        s_d2[i] = S.comb[k * kCombStride + a] + (k + mid <= kMaxN ? S.comb[(k + mid) * kCombStride + a + 1] : 0u);
    }
    for (int i = threadIdx.x; i < 2 * S.L; i += blockDim.x) {
        double c, s;
        sincospi((double)i / (double)S.L, &s, &c);
        s_cos[i] = (R)c;
        s_sin[i] = (R)s;
    }
    for (int i = threadIdx.x; i <= kMaxN; i += blockDim.x) {
        s_sqrt[i] = (R)sqrt((double)i);
        s_rsqrt[i] = i ? (R)(1.0 / sqrt((double)i)) : R(0);
    }
    __syncthreads();
    return HvTables<R>{rank_tab_of(S, s_rank), s_comb, s_d2, s_cos, s_sin, s_sqrt, s_rsqrt};
}

inline size_t hv_smem_bytes(const SectorView& S, size_t real_size) {
    return (((S.rank_words + 1) & ~1) + kCombStride * kCombStride + 1 + (S.Nd + 1) * 64) * sizeof(uint32_t) +
           (64 + 64 + 33 + 33) * real_size;
}

}  // namespace ed
