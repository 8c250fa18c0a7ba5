// ed_seg.cuh -- the fused Lanczos step over the rows of free blocks, organised by segments.
//
// A free block (canonical hole mask with a trivial stabiliser) holds every spin configuration of its
// hole mask: the row of compressed down mask dc is  block start + colex rank(dc).  Split dc at
// compressed position P into a low part Lo (bits [0, P), kl down spins) and a high part H (bits
// [P, Ns)).  Colex rank is a sum over the set bits, so
//     rank(dc) = base(H) + rank_P(Lo),     base(H) = rank((H << P) | (2^kl - 1)),
// and the rows sharing H form a contiguous *segment* of C(P, kl) rows, ordered by rank_P(Lo).  The
// row order is the reference's (dense index = colex rank, general/basis_indexing.h:188-242); only
// the work is regrouped.  Each term of H.v (the rules of tJ_spin_half_ladder/matrix_setup.pyx:80-110
// as the row kernel in ed_device.cuh applies them) splits into a part that depends on Lo alone --
// computed once per thread for all segments of a chunk -- and a part that depends on H alone -- read
// from the segment's record (built once per sector, ed_segrec.cu):
//   * exchange bonds below P: the partner row is in the same segment at rank_P(Lo ^ f);
//   * exchange bonds at or above P: the partner is segment H ^ f at the same offset -- one coalesced
//     read per antiparallel bond, whose partner bases the record lists;
//   * bonds across P: the partner is base(H ^ f_H) + rank_P(Lo ^ f_L), in the class kl -+ 1;
//   * hops: the target is a fixed bit permutation pi of dc (the electron's move, then the target's
//     coset permutation) ranked in the target block.  With U = pi(H << P) and V = pi(Lo), at most
//     two bits of V land at or above P (and as many of U below P) for the hops of the ladder's
//     blocks, so the target row is  sb[vbi] + rank_P(ua | va):  ua and the sb per segment, vbi (V's
//     bits above P) and va per thread; otherwise the full rank of U | V is taken per row.
//     Stabiliser targets read the expanded copy of the target block (expand_cand_kernel) at the same
//     rank, with the coset's first phase folded in.
// A chunk covers a 32-offset window of a range of segments (lane = offset in the window); a warp takes
// two segments at a time (a lane's two rows share the offset, so the per-offset terms are read once
// for both) and walks the range with the CTA's other warps; warps never wait on one another inside a
// chunk, and every per-segment loop bound is the same for all lanes of a warp.  32-offset windows
// keep the lanes busy on the classes whose C(P, kl) is not a multiple of 64 (210 rows: 94 % against
// 82 % with 64-offset windows) and the low lists, padded to the window's longest, shorter.  The
// per-lane terms of a chunk live in shared memory (every warp maps its lanes to the same offsets).
// While a warp works on one pair, the next pair's records are copied into shared memory (cp.async)
// and its row values loaded, so a row's gathers wait on one round trip per group (low bonds, high
// bonds four at a time, cross bonds, hops) rather than on chains of dependent loads.
// The key table is not read: a free row's configuration follows from its index.
//
// Per-row sums of the step (ed_step.cuh) are kept per thread in plain FP32 (FP64) over four rows and
// then added into a float-float (FP64) sum; per chunk they are reduced in a fixed order, so a sector
// gives the same bits alone and in a batch.
#pragma once

#include "ed_step.cuh"

namespace ed {

constexpr int kSegLow = 1 << kSegA;  // P-bit masks

// Permutation of a hop applied to a compressed mask (a bit permutation: it maps disjoint parts of a
// mask independently, which the split into U and V relies on).
__host__ __device__ __forceinline__ uint32_t seg_perm(uint32_t x, uint32_t keep, uint32_t band, uint32_t sl,
                                                      uint32_t sr, uint32_t p, uint32_t q, uint32_t swap,
                                                      uint32_t rot, uint32_t nsr, uint32_t nsmask) {
    const uint32_t xm = (x & keep) | (((x & band) << sl) >> sr) | (((x >> p) & 1u) << q);
    const uint32_t t = (xm ^ (xm >> 1)) & swap;
    const uint32_t sw = xm ^ t ^ (t << 1);
    return ((sw << rot) | (sw >> nsr)) & nsmask;
}

// ---- the index arithmetic of segments, shared by the kernels and the host checks ---------------
// (Hs = H << P: the high part in place; kl = down spins below P; rt = rank_P table; R = rank tables)

// Position of antiparallel high bond (a, .) of list index i among the segment's antiparallel high
// bonds (rung, leg at distance one, leg at distance two, each by ascending a).
__host__ __device__ __forceinline__ int seg_high_pos(uint32_t Hs, int i, uint32_t a, int nBr, int nBa, uint32_t mr,
                                                     uint32_t ma, uint32_t m2) {
    const uint32_t d1 = Hs ^ (Hs >> 1), below = (1u << a) - 1u;
    const uint32_t ar = d1 & mr, aa = d1 & ma, a2 = (Hs ^ (Hs >> 2)) & m2;
    if (i < nBr) return popc32(ar & below);
    if (i < nBr + nBa) return popc32(ar) + popc32(aa & below);
    return popc32(ar) + popc32(aa) + popc32(a2 & below);
}

// First row of the segment H ^ (bits a, b), same class (both ends at or above P).
__host__ __device__ __forceinline__ uint32_t seg_high_partner(uint32_t Hs, uint32_t a, uint32_t b, int kl,
                                                              const RankTab& R, int Nd) {
    return spin_rank((Hs ^ (1u << a) ^ (1u << b)) | ((1u << kl) - 1u), R, Nd);
}

// Cross bond with its high end at b: first row of segment H ^ b in class kl -+ 1 (0 when that class
// is empty: no row then has the bond antiparallel).
__host__ __device__ __forceinline__ uint32_t seg_cross_partner(uint32_t Hs, uint32_t b, int kl, int P,
                                                               const RankTab& R, int Nd) {
    const int klp = ((Hs >> b) & 1u) ? kl + 1 : kl - 1;
    if (klp < 0 || klp > P) return 0u;
    return spin_rank((Hs ^ (1u << b)) | ((1u << klp) - 1u), R, Nd);
}

// Hop with nb <= 2: rank of the target's high part for U = pi(H << P) and the low positions' bits vbi
// (bit 0 at bp0, bit 1 at bp1) that land at or above P.
__host__ __device__ __forceinline__ uint32_t seg_hop_base(uint32_t U, uint32_t amask, int vbi, uint32_t bp0,
                                                          uint32_t bp1, int P, const RankTab& R, int Nd) {
    uint32_t mB = U & ~amask;
    if (vbi & 1) mB |= 1u << bp0;
    if (vbi & 2) mB |= 1u << bp1;
    const int klt = Nd - popc32(mB);
    if (klt < 0 || klt > P) return 0u;
    return spin_rank(mB | ((1u << klt) - 1u), R, Nd);
}

// Per-lane part of a hop (nb <= 2): V's low bits and, above them (bits kSegA, kSegA + 1), vbi.
__host__ __device__ __forceinline__ uint32_t seg_hop_thread(uint32_t V, uint32_t amask, uint32_t nb, uint32_t bp0,
                                                            uint32_t bp1) {
    const uint32_t vbi = nb == 0 ? 0u : (((V >> bp0) & 1u) | (nb == 2 ? ((V >> bp1) & 1u) << 1 : 0u));
    return (V & amask) | (vbi << kSegA);
}

// Target rank of a hop (nb <= 2) from its per-segment (ua, sb) and per-lane (hc) parts.
__host__ __device__ __forceinline__ uint32_t seg_hop_rank(const uint32_t* sb, uint32_t ua, uint32_t hc,
                                                          const uint8_t* rt) {
    return sb[hc >> kSegA] + rt[ua | (hc & (kSegLow - 1u))];
}

// A hop of the chunk's block as the rows use it (built per chunk from SegHopDesc and the weights).
template <typename R, bool CPLX>
struct alignas(16) SegHop {
    const typename Vec<R, CPLX>::T* tp;  // target block's values: x at its first row, or its expanded copy
    R cr, ci;                            // weight * fermion sign * phase (* sqrt(2L) for stabiliser targets)
    uint32_t keep, band, sl, sr, p, q, swap, rot, nsr;
    uint32_t nb, bp0, bp1;               // low positions landing at or above P (nb = 3: more than two)
    uint32_t kind;                       // 0 / 1 present, 3 absent (no target, or weight 0)
};

template <typename R, bool CPLX>
__device__ __forceinline__ void seg_ld(const typename Vec<R, CPLX>::T* p, R& re, R& im) {
    const typename Vec<R, CPLX>::T t = __ldg(p);
    if constexpr (CPLX) {
        re = t.x;
        im = t.y;
    } else {
        re = t;
        im = R(0);
    }
}

// Fused multiply-add in the vectors' own precision (FP32 stays FP32).
__device__ __forceinline__ float fma_r(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return __fma_rn(a, b, c); }

// Adds a hop's term c * v to a row's hop sum (c, v complex when CPLX), by explicit fused
// multiply-adds so that every path of the kernel rounds it the same way.
template <typename R, bool CPLX>
__device__ __forceinline__ void seg_hop_acc(R& hr, R& hi, R cr, R ci, R vr, R vi) {
    hr = fma_r(cr, vr, hr);
    if constexpr (CPLX) {
        hr = fma_r(-ci, vi, hr);
        hi = fma_r(ci, vr, fma_r(cr, vi, hi));
    }
}

template <typename R, bool CPLX>
__device__ __forceinline__ void seg_ld_shared(const typename Vec<R, CPLX>::T* p, R& re, R& im) {
    const typename Vec<R, CPLX>::T t = *p;
    if constexpr (CPLX) {
        re = t.x;
        im = t.y;
    } else {
        re = t;
        im = R(0);
    }
}


// A thread's running sum kept in shared memory: two words for FP32 ([0] high, [1] low part), one for FP64.
constexpr int seg_acc_words(int real_size) { return real_size == 4 ? 2 : 1; }
template <typename R>
__device__ __forceinline__ Accum<R> seg_acc_load(const R (&s)[seg_acc_words(sizeof(R))][kSegThreads], int i) {
    Accum<R> a;
    if constexpr (sizeof(R) == 4) {
        a.hi = s[0][i];
        a.lo = s[1][i];
    } else {
        a.s = s[0][i];
    }
    return a;
}
template <typename R>
__device__ __forceinline__ void seg_acc_store(R (&s)[seg_acc_words(sizeof(R))][kSegThreads], int i, const Accum<R>& a) {
    if constexpr (sizeof(R) == 4) {
        s[0][i] = a.hi;
        s[1][i] = a.lo;
    } else {
        s[0][i] = a.s;
    }
}

template <typename R>
__device__ __forceinline__ void fold(Accum<R>& a, R p);
template <>
__device__ __forceinline__ void fold(Accum<double>& a, double p) {
    a.s += p;
}
template <>
__device__ __forceinline__ void fold(Accum<float>& a, float p) {
    a.add(p, 0.0f);
}

constexpr int kSegRecMax = 128;  // words of a staged segment record (one 16-byte copy per lane)
constexpr int kSegHopSlots = 24; // hops of a block padded to groups of four per kind (at most 12 + 12)

__device__ __forceinline__ void seg_cp_async16(void* smem_dst, const void* gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void seg_cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void seg_cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Adds a partner's value to a row's exchange sum: the one sum when rung and leg J agree, else the
// rung or the leg sum.
template <typename R, bool CPLX, bool MERGED>
__device__ __forceinline__ void seg_add(R& er, R& ei, R& lr, R& li, bool rung, R vr, R vi) {
    if (MERGED || rung) {
        er += vr;
        if constexpr (CPLX) ei += vi;
    } else {
        lr += vr;
        if constexpr (CPLX) li += vi;
    }
}

// Copies one vector element global -> shared asynchronously (cp.async; 4, 8 or 16 bytes).
template <typename T>
__device__ __forceinline__ void seg_cp_async_elem(T* smem_dst, const T* gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    if constexpr (sizeof(T) == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(gsrc), "n"((int)sizeof(T)) : "memory");
}

constexpr int kSegStageBytes = 10240;  // staged gathers: shared memory per warp

constexpr int kSegLowMax = 16;  // antiparallel bonds below P of one row (at most kSegMaxA), padded to fours

// A hop slot of a chunk as every row reads it: the target values, the coefficient, the slot's first
// record word.  Staged in shared memory; one 16-byte load for real FP32 vectors.
template <typename R, bool CPLX>
struct alignas(16) SegSlot {
    const typename Vec<R, CPLX>::T* tp;
    R cr;
    uint32_t off;
};
template <typename R>
struct alignas(16) SegSlot<R, true> {
    const typename Vec<R, true>::T* tp;
    R cr, ci;
    uint32_t off;
};

template <typename R, bool CPLX>
__device__ __forceinline__ R seg_slot_ci(const SegSlot<R, CPLX>& S) {
    if constexpr (CPLX) return S.ci;
    else return R(0);
}

// The fused step over segment chunks: a chunk is (free block, class kl, 32-offset window, range of
// segments); warp w of the CTA takes the segment pairs (begin + 2w, begin + 2w + 1), then 16 segments
// further, ... and, in both segments of a pair, the row at offset t = window + lane.  The per-offset
// tables (low-bond partners, cross and hop parts) are read once for the two rows; each row reads its
// own segment's record.  NR = 2 works on the two rows together (their gathers in flight at once);
// NR = 1 takes them one after the other.  MERGED: rung and leg exchanges share one coefficient
// (J_rung = J_leg), so each row keeps one exchange sum over one list per bond class; otherwise every
// element picks its coefficient.  PAIR = false: 64-offset windows, warp w taking segments begin + w,
// + 8, ... and in each the rows at offsets t and t + 32 (one record for both rows, two table
// columns); the sector's plan says which (Sector::seg_win), and the autotuner picks per sector shape.
template <typename R, bool CPLX, int MINB, bool MERGED, int NR, bool STAGED = false, bool PAIR = true>
__global__ void __launch_bounds__(kSegThreads, MINB)
    seg_step_kernel(const SectorView* __restrict__ views, const int64_t* __restrict__ offs,
                    const BatchChunk* __restrict__ chunks, const int* __restrict__ idx, int count, HvWeights W,
                    void* v, void* vprev, void* other, int first, const double* __restrict__ scal, int stride, int k,
                    double* __restrict__ partials, void* xfull) {
    using T = typename Vec<R, CPLX>::T;
    constexpr int kWarps = kSegThreads / 32;
    constexpr int kWin = PAIR ? 32 : 64;     // offsets of a chunk's window (columns of the tables)
    constexpr int kHalves = kWin / 32;       // table columns per lane
    constexpr int kSegStep = PAIR ? 2 : 1;   // segments a warp takes at a time
    static_assert(PAIR || !STAGED, "staged gathers use 32-offset windows");
    constexpr int kCols = 32 * NR;  // staged gathers: columns of a slot (the rows worked on together)
    constexpr int kScap = kSegStageBytes / (kCols * (int)sizeof(T));  // staged slots per pass
    extern __shared__ __align__(16) uint8_t seg_stage_smem[];  // STAGED: kWarps * kSegStageBytes
    __shared__ uint8_t s_rt[kSegLow];           // rank_P of each P-bit mask within its popcount class
    __shared__ uint16_t s_ut[kSegLow];          // the masks by (popcount, rank_P)
    __shared__ uint32_t s_utoff[kSegA + 2];
    __shared__ __align__(16) SegDesc s_desc;
    __shared__ __align__(16) SegHop<R, CPLX> s_hop[kMaxHops];
    // hop slots of the chunk: the kind-0 hops then dummies up to a multiple of four, the same for kind 1
    // (nb 1 or 2); a dummy reads the block's first element with coefficient 0
    __shared__ __align__(16) SegSlot<R, CPLX> s_slot[kSegHopSlots];
    // per-offset terms of the chunk's window (column = offset - window, lane + 32 h): a column past
    // the class's rows repeats one that is a row (its own half's first, else the window's first), so
    // its reads stay valid
    __shared__ uint8_t s_al[kSegLowMax][kWin];      // partners of the antiparallel bonds below P (rung
                                                    // first), padded with the offset itself
    __shared__ uint8_t s_xo[kSegMaxX][kWin];        // cross bond c: rank_P(Lo ^ low end) (0 past nX)
    __shared__ uint16_t s_hc[kSegHopSlots][kWin];   // hop slot: rank_P(V) (kind 0) or va | vbi << kSegA
    __shared__ uint32_t s_lane[kWin];               // Lo | lob << 16 (cross-bond low-end spins)
    __shared__ uint32_t s_cnt[kWin];                // nr | nlow << 8 (antiparallel bonds below P)
    __shared__ int s_maxw;                          // longest low list of the window, in fours
    // per warp: this and the next iteration's records (a pair's two, or one segment's)
    __shared__ __align__(16) uint32_t s_rec[kWarps][2][kSegStep][kSegRecMax];
    __shared__ R s_acc[kReduceSlots][seg_acc_words(sizeof(R))][kSegThreads];  // per thread: the step's sums
    const int P = views[0].seg_p;
    const uint32_t amask = (1u << P) - 1u;
    const uint32_t* __restrict__ comb = views[0].comb;
    for (int m = threadIdx.x; m < (1 << P); m += blockDim.x) {
        uint32_t r = 0, mm = (uint32_t)m;
        int j = 0;
        while (mm) {
            const int b = __ffs(mm) - 1;
            mm &= mm - 1u;
            ++j;
            r += comb[j * kCombStride + b];
        }
        s_rt[m] = (uint8_t)r;
    }
    if (threadIdx.x <= P + 1) {
        uint32_t o = 0;
        for (int kk = 0; kk < (int)threadIdx.x; ++kk) o += comb[kk * kCombStride + P];
        s_utoff[threadIdx.x] = o;
    }
    __syncthreads();
    for (int m = threadIdx.x; m < (1 << P); m += blockDim.x) s_ut[s_utoff[__popc(m)] + s_rt[m]] = (uint16_t)m;
    const R wr = R(0.5) * (R)W.w[3], wl = R(0.5) * (R)W.w[2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    for (int c = blockIdx.x; c < count; c += gridDim.x) {
        const int cid = idx[c];
        const BatchChunk ch = chunks[cid];
        const SectorView* Sp = views + ch.sec;
        const int kl = ch.kl, Ns = Sp->Ns, Nd = Sp->Nd, N = Sp->N, L = Sp->L;
        const uint32_t nsmask = 0xffffffffu >> (32 - Ns);
        const int nA = (int)comb[kl * kCombStride + P];
        const int win = kWin * ch.piece;
        const int nact = min(32, nA - win);  // lanes with rows
        __syncthreads();  // the previous chunk's rows are done with the shared tables
        {
            const uint4* src = reinterpret_cast<const uint4*>(Sp->seg + ch.block);
            uint4* dst = reinterpret_cast<uint4*>(&s_desc);
            for (int i = threadIdx.x; i < (int)(sizeof(SegDesc) / 16); i += blockDim.x) dst[i] = src[i];
        }
        __syncthreads();
        const int nhop = s_desc.nhop, n0 = s_desc.n0, n12 = s_desc.n12, nX = s_desc.nX, nXr = s_desc.nXr;
        const int64_t bstart = s_desc.start;
        T* const x = reinterpret_cast<T*>(v) + offs[ch.sec];
        const T* const xb = x + bstart;
        const int n04 = (n0 + 3) & ~3, n124 = (n12 + 3) & ~3;
        {  // the chunk's tables: hop records, per-offset terms, hop slots
            // the offset whose terms column lane + 32 h holds: its own, or (past the class's rows) the
            // first half's, or the window's first
            auto tsrc_of = [&](int h) {
                const int j = win + lane + 32 * h;
                return j < nA ? j : (win + lane < nA ? win + lane : win);
            };
            if (warp == 2 && lane < kMaxHops) {
                // every hop gets a record: absent hops (and those past nhop) read a valid element with
                // coefficient 0
                const int h = lane;
                SegHop<R, CPLX>& F = s_hop[h];
                const SegHopDesc& G = s_desc.hop[h];
                const bool live = h < nhop && G.kind != 3 && W.w[G.term] != 0.0;
                F.keep = G.keep;
                F.band = G.band;
                F.sl = G.sl;
                F.sr = G.sr;
                F.p = G.p;
                F.q = G.q;
                F.swap = G.swap;
                F.rot = G.rot;
                F.nsr = G.nsr;
                F.nb = h < nhop ? G.nb : 0u;
                F.bp0 = G.bpos[0];
                F.bp1 = G.bpos[1];
                F.kind = live ? (uint32_t)G.kind : 3u;
                F.tp = xb;
                F.cr = F.ci = R(0);
                if (live) {
                    const R w = (R)W.w[G.term];
                    const R sw = G.sign ? -w : w;
                    R cf = sw;
                    if (G.kind == 1) {
                        cf = sw * (R)sqrt((double)N);
                        F.tp = reinterpret_cast<const T*>(xfull) + ch.xoff +
                               G.tstart * (int64_t)comb[Nd * kCombStride + Ns];
                    } else {
                        F.tp = x + G.tstart;
                    }
                    double sn, cs;
                    sincospi((double)G.e / (double)L, &sn, &cs);
                    if constexpr (CPLX) {
                        F.cr = cf * (R)cs;
                        F.ci = cf * (R)sn;
                    } else {
                        F.cr = G.e == 0 ? cf : -cf;
                    }
                }
            } else if (warp == 0) {
                // bonds below P: the antiparallel ones' partners, rung bonds first, padded with the offset
                // itself up to the table's length (read in fours, the padding taken back out after the sums)
                int mx = 0;
                for (int hh = 0; hh < kHalves; ++hh) {
                    const int col = lane + 32 * hh, tsrc = tsrc_of(hh);
                    const uint32_t lo_c = s_ut[s_utoff[kl] + tsrc];
                    int nr = 0, nlow = 0;
                    const int nAb = s_desc.nA, nAr = s_desc.nAr;
                    for (int i = 0; i < nAb; ++i) {
                        const uint32_t f = s_desc.fA[i], sb = lo_c & f;
                        if (sb != 0u && sb != f) {
                            s_al[nlow++][col] = s_rt[lo_c ^ f];
                            if (i < nAr) ++nr;
                        }
                    }
                    for (int q = nlow; q < kSegLowMax; ++q) s_al[q][col] = (uint8_t)tsrc;
                    mx = max(mx, (int)__reduce_max_sync(0xffffffffu, (unsigned)nlow));
                    s_cnt[col] = (uint32_t)nr | ((uint32_t)nlow << 8);
                }
                if (lane == 0) s_maxw = (mx + 3) & ~3;
            } else if (warp == 1) {
                // bonds across P: the partner's low part and this offset's spin at the low end
                for (int hh = 0; hh < kHalves; ++hh) {
                    const int col = lane + 32 * hh;
                    const uint32_t lo_c = s_ut[s_utoff[kl] + tsrc_of(hh)];
                    uint32_t lob = 0;
                    for (int cc = 0; cc < kSegMaxX; ++cc) {
                        const uint32_t a = s_desc.cX[cc][0];
                        if (cc < nX) lob |= ((lo_c >> a) & 1u) << cc;
                        s_xo[cc][col] = cc < nX ? s_rt[lo_c ^ (1u << a)] : (uint8_t)0;
                    }
                    s_lane[col] = lo_c | (lob << 16);
                }
            }
            __syncthreads();
            if (warp != 2) {
                // hop slots, spread over the other warps
                for (int sl = warp < 2 ? warp : warp - 1; sl < n04 + n124; sl += kWarps - 1) {
                    const int h = sl < n04 ? (sl < n0 ? sl : -1) : (sl - n04 < n12 ? n0 + sl - n04 : -1);
                    for (int hh = 0; hh < kHalves; ++hh) {
                        const uint32_t lo_c = s_ut[s_utoff[kl] + tsrc_of(hh)];
                        uint32_t hc = 0;
                        if (h >= 0 && s_hop[h].kind != 3) {
                            const SegHop<R, CPLX>& F = s_hop[h];
                            const uint32_t V = seg_perm(lo_c, F.keep, F.band, F.sl, F.sr, F.p, F.q, F.swap, F.rot, F.nsr, nsmask);
                            hc = F.nb == 0 ? s_rt[V] : seg_hop_thread(V, amask, F.nb, F.bp0, F.bp1);
                        }
                        s_hc[sl][lane + 32 * hh] = (uint16_t)hc;
                    }
                }
            } else if (lane < n04 + n124) {
                const int sl = lane;
                const int h = sl < n04 ? (sl < n0 ? sl : -1) : (sl - n04 < n12 ? n0 + sl - n04 : -1);
                SegSlot<R, CPLX>& S = s_slot[sl];
                S.tp = h >= 0 ? s_hop[h].tp : xb;
                S.cr = h >= 0 ? s_hop[h].cr : R(0);
                if constexpr (CPLX) S.ci = h >= 0 ? s_hop[h].ci : R(0);
                S.off = h >= 0 ? s_desc.hop_off[h] : s_desc.zero_w;
            }
            __syncthreads();
        }

        const int smax = s_maxw;  // low lists read, in fours
        const uint32_t rec_len = s_desc.rec_len, xo = s_desc.xo;
        const uint32_t* __restrict__ rec0 = Sp->seg_rec + s_desc.rec + (int64_t)Sp->seg_off[kl] * rec_len;
        const uint32_t* __restrict__ segb = Sp->seg_base + Sp->seg_off[kl];
        const int nX4 = (nX + 3) & ~3;  // cross bonds read in groups of four (the padding is never antiparallel)
        const uint32_t xall = (1u << nX) - 1u, xrmask = (1u << nXr) - 1u, x4mask = (1u << nX4) - 1u;
        T* const y = reinterpret_cast<T*>(other) + offs[ch.sec] + bstart;
        const T* const yp = first ? nullptr : reinterpret_cast<const T*>(vprev) + offs[ch.sec] + bstart;
        const R beta = first ? R(0) : (R)scal[(int64_t)ch.sec * stride + 2 * k];
        // per row r of an iteration: its column of the tables, its offset (read for every lane: a
        // valid offset), whether it is a row (PAIR: the pair's second segment decides per iteration)
        const int t = win + lane;
        int col[2], tt[2];
        bool act[2];
        uint32_t lnw[2];
        int nlow[2], nrl[2];
        const T* xt[2];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            col[r] = PAIR ? lane : lane + 32 * r;
            const int to = PAIR ? t : t + 32 * r;
            act[r] = to < nA;
            tt[r] = act[r] ? to : t;
            lnw[r] = s_lane[col[r]];
            const uint32_t cn = s_cnt[col[r]];
            nlow[r] = (int)(cn >> 8);
            nrl[r] = (int)(cn & 255u);
            xt[r] = xb + tt[r];
        }

        // the step's running sums (float-float for FP32) wait in shared memory between folds: eight
        // registers fewer in the row loop, which lets the 4-CTA variant run without spills
        R pend[kReduceSlots] = {R(0), R(0), R(0), R(0)};
        int npend = 0;
#pragma unroll
        for (int q = 0; q < kReduceSlots; ++q) seg_acc_store<R>(s_acc[q], threadIdx.x, Accum<R>{});

        // the next pair's records are copied into shared memory, and its rows' values and v_{k-1}
        // loaded, while this pair is worked on; the active lanes together copy every word of a record
        // (segment indices of a class fit 32 bits: SectorView::seg_off)
        const int gend = (int)ch.end;
        int g = lane < nact ? (int)ch.begin + kSegStep * warp : gend;  // lanes without rows skip to the reduction
        auto copy_pair = [&](int gg, uint32_t* dst) {
#pragma unroll
            for (int r = 0; r < kSegStep; ++r)
                if (gg + r < gend)
                    for (int w4 = 4 * lane; w4 < (int)rec_len; w4 += 4 * nact)
                        seg_cp_async16(dst + r * kSegRecMax + w4, rec0 + (uint32_t)(gg + r) * rec_len + w4);
        };
        uint32_t base[2] = {0u, 0u};
        R xr[2] = {R(0), R(0)}, xi[2] = {R(0), R(0)}, pr[2] = {R(0), R(0)}, pi[2] = {R(0), R(0)};
        if (g < gend) {
            copy_pair(g, s_rec[warp][0][0]);
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                base[r] = (PAIR || r == 0) ? __ldg(segb + (PAIR && g + r < gend ? g + r : g)) : base[0];
                seg_ld<R, CPLX>(xt[r] + base[r], xr[r], xi[r]);
                if (!first) seg_ld<R, CPLX>(yp + base[r] + tt[r], pr[r], pi[r]);
            }
        }
        seg_cp_commit();
        for (int it = 0; g < gend; ++it, g += kSegStep * kWarps) {
            const bool act1 = PAIR && g + 1 < gend;  // PAIR: the pair's second segment exists (warp-uniform)
            const uint32_t* const sw[2] = {s_rec[warp][it & 1][0], s_rec[warp][it & 1][act1 ? kSegStep - 1 : 0]};
            const int gn = g + kSegStep * kWarps;
            if (gn < gend) copy_pair(gn, s_rec[warp][(it + 1) & 1][0]);
            seg_cp_commit();
            uint32_t nbase[2] = {0u, 0u};
            R nxr[2] = {R(0), R(0)}, nxi[2] = {R(0), R(0)}, npr[2] = {R(0), R(0)}, npi[2] = {R(0), R(0)};
            if (gn < gend) {
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    nbase[r] = (PAIR || r == 0) ? __ldg(segb + (PAIR && gn + r < gend ? gn + r : gn)) : nbase[0];
                    seg_ld<R, CPLX>(xt[r] + nbase[r], nxr[r], nxi[r]);
                    if (!first) seg_ld<R, CPLX>(yp + nbase[r] + tt[r], npr[r], npi[r]);
                }
            }
            seg_cp_wait<1>();  // this pair's records have arrived (the next pair's may be in flight)
            __syncwarp(__activemask());

            int zb[2], zbr[2], zb4[2];
            uint32_t xm[2];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const uint32_t w1 = sw[r][1];
                zb[r] = (int)(w1 & 255u);
                zbr[r] = (int)((w1 >> 8) & 255u);
                zb4[r] = (zb[r] + 3) & ~3;
                xm[r] = ((lnw[r] >> 16) ^ (w1 >> 16)) & xall;  // cross bonds antiparallel in row r
            }
#pragma unroll
            for (int r0 = 0; r0 < 2; r0 += NR) {
                if (PAIR && NR == 1 && r0 == 1 && !act1) break;
                // ---- the rows at offset t of segments g + r0 (+ 1): y = H x - beta v_{k-1}
                const T* xs[NR];
                R er[NR], ei[NR], lr[NR], li[NR], hr[NR], hi[NR];
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    xs[r] = xb + base[r0 + r];
                    er[r] = ei[r] = lr[r] = li[r] = hr[r] = hi[r] = R(0);
                }
                if constexpr (!STAGED) {
                    // exchange bonds below P: partners in the row's own segment, one table read for the rows
                    for (int q0 = 0; q0 < smax; q0 += 4) {
                        R vr[NR][4], vi[NR][4];
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int r = 0; r < NR; ++r)
                                seg_ld<R, CPLX>(xs[r] + (uint32_t)s_al[q0 + u][col[r0 + r]], vr[r][u], vi[r][u]);
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int r = 0; r < NR; ++r) seg_add<R, CPLX, MERGED>(er[r], ei[r], lr[r], li[r], q0 + u < nrl[r0 + r], vr[r][u], vi[r][u]);
                    }
                    // exchange bonds at or above P: the partner segments at the same offset, four at a
                    // time; the rows together up to the shorter list, then each row's rest
                    auto high4 = [&](int r, int q0, R (&vr)[4], R (&vi)[4]) {
                        const uint4 pw = *reinterpret_cast<const uint4*>(sw[r0 + r] + 4 + q0);  // 16-byte aligned
                        seg_ld<R, CPLX>(xt[r0 + r] + pw.x, vr[0], vi[0]);
                        seg_ld<R, CPLX>(xt[r0 + r] + pw.y, vr[1], vi[1]);
                        seg_ld<R, CPLX>(xt[r0 + r] + pw.z, vr[2], vi[2]);
                        seg_ld<R, CPLX>(xt[r0 + r] + pw.w, vr[3], vi[3]);
                    };
                    const int zc = NR == 2 ? min(zb4[r0], zb4[r0 + NR - 1]) : zb4[r0];
                    for (int q0 = 0; q0 < zc; q0 += 4) {
                        R vr[NR][4], vi[NR][4];
#pragma unroll
                        for (int r = 0; r < NR; ++r) high4(r, q0, vr[r], vi[r]);
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int r = 0; r < NR; ++r)
                                seg_add<R, CPLX, MERGED>(er[r], ei[r], lr[r], li[r], q0 + u < zbr[r0 + r], vr[r][u], vi[r][u]);
                    }
#pragma unroll
                    for (int r = 0; r < NR; ++r)
                        for (int q0 = zc; q0 < zb4[r0 + r]; q0 += 4) {
                            R vr[4], vi[4];
                            high4(r, q0, vr, vi);
#pragma unroll
                            for (int u = 0; u < 4; ++u)
                                seg_add<R, CPLX, MERGED>(er[r], ei[r], lr[r], li[r], q0 + u < zbr[r0 + r], vr[u], vi[u]);
                        }
                    // bonds across P, antiparallel when the two ends' spins differ (otherwise the row itself is read)
                    for (int c0 = 0; c0 < nX4; c0 += 4) {
                        R vr[NR][4], vi[NR][4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int cc = c0 + u;
#pragma unroll
                            for (int r = 0; r < NR; ++r) {
                                const uint32_t xoc = s_xo[cc][col[r0 + r]];
                                const uint32_t pw = sw[r0 + r][xo + cc];
                                const uint32_t on = 0u - ((xm[r0 + r] >> cc) & 1u);  // all ones when antiparallel
                                const uint32_t o = (on & (pw + xoc)) | (~on & (base[r0 + r] + (uint32_t)tt[r0 + r]));
                                seg_ld<R, CPLX>(xb + o, vr[r][u], vi[r][u]);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int r = 0; r < NR; ++r) seg_add<R, CPLX, MERGED>(er[r], ei[r], lr[r], li[r], c0 + u < nXr, vr[r][u], vi[r][u]);
                    }
                    // hops, four at a time: kind 0 (r = sb + rank_P(V)), then kind 1 (r = sb[vbi] + rank_P(ua | va))
                    for (int h4 = 0; h4 < n04; h4 += 4) {
                        R vr[NR][4], vi[NR][4];
                        SegSlot<R, CPLX> S[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            S[u] = s_slot[h4 + u];
#pragma unroll
                            for (int r = 0; r < NR; ++r)
                                seg_ld<R, CPLX>(S[u].tp + (sw[r0 + r][S[u].off] + s_hc[h4 + u][col[r0 + r]]), vr[r][u], vi[r][u]);
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int r = 0; r < NR; ++r)
                                seg_hop_acc<R, CPLX>(hr[r], hi[r], S[u].cr, seg_slot_ci(S[u]), vr[r][u], vi[r][u]);
                    }
                    for (int h4 = n04; h4 < n04 + n124; h4 += 4) {
                        R vr[NR][4], vi[NR][4];
                        SegSlot<R, CPLX> S[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            S[u] = s_slot[h4 + u];
#pragma unroll
                            for (int r = 0; r < NR; ++r) {
                                const uint32_t hc = s_hc[h4 + u][col[r0 + r]];
                                const uint32_t wv = S[u].off + 1u + (hc >> kSegA), va = hc & (kSegLow - 1u);
                                const uint32_t rr = sw[r0 + r][wv] + s_rt[sw[r0 + r][S[u].off] | va];
                                seg_ld<R, CPLX>(S[u].tp + rr, vr[r][u], vi[r][u]);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int r = 0; r < NR; ++r)
                                seg_hop_acc<R, CPLX>(hr[r], hi[r], S[u].cr, seg_slot_ci(S[u]), vr[r][u], vi[r][u]);
                    }
                } else {
                    // every gather of the rows goes to shared memory by cp.async, up to kScap slots per
                    // pass: all in flight together, one wait, then the sums read them back.  Slots:
                    // low bonds [0, e0), high [e0, e1) (the pair's longer list: the shorter row skips
                    // the slots past its own, so each row adds the terms of the unstaged kernel in its
                    // order), cross [e1, e2), hop slots [e2, e3)
                    T* const stg = reinterpret_cast<T*>(seg_stage_smem) + (size_t)warp * kScap * kCols;
                    const int zs = NR == 2 ? max(zb4[r0], zb4[r0 + NR - 1]) : zb4[r0];
                    const int e0 = smax, e1 = e0 + zs, e2 = e1 + nX4, e3 = e2 + n04 + n124;
                    for (int p0 = 0; p0 < e3; p0 += kScap) {
                        const int p1 = min(e3, p0 + kScap);
                        for (int sl = p0; sl < min(p1, e0); ++sl)
#pragma unroll
                            for (int r = 0; r < NR; ++r)
                                seg_cp_async_elem<T>(stg + (sl - p0) * kCols + lane + 32 * r,
                                                     xs[r] + (uint32_t)s_al[sl][col[r0 + r]]);
                        for (int sl = max(p0, e0); sl < min(p1, e1); ++sl)
#pragma unroll
                            for (int r = 0; r < NR; ++r)
                                if (sl - e0 < zb4[r0 + r])
                                    seg_cp_async_elem<T>(stg + (sl - p0) * kCols + lane + 32 * r, xt[r0 + r] + sw[r0 + r][4 + sl - e0]);
                        for (int sl = max(p0, e1); sl < min(p1, e2); ++sl) {
                            const int cc = sl - e1;
#pragma unroll
                            for (int r = 0; r < NR; ++r) {
                                const uint32_t xoc = s_xo[cc][col[r0 + r]];
                                const uint32_t pw = sw[r0 + r][xo + cc];
                                const uint32_t on = 0u - ((xm[r0 + r] >> cc) & 1u);  // all ones when antiparallel
                                const uint32_t o = (on & (pw + xoc)) | (~on & (base[r0 + r] + (uint32_t)tt[r0 + r]));
                                seg_cp_async_elem<T>(stg + (sl - p0) * kCols + lane + 32 * r, xb + o);
                            }
                        }
                        for (int sl = max(p0, e2); sl < p1; ++sl) {
                            const int hs = sl - e2;  // hop slot: kind 0 below n04, kind 1 from n04
                            const SegSlot<R, CPLX>& S = s_slot[hs];
#pragma unroll
                            for (int r = 0; r < NR; ++r) {
                                const uint32_t hc = s_hc[hs][col[r0 + r]];
                                const uint32_t w0 = sw[r0 + r][S.off];
                                const uint32_t rr = hs < n04 ? w0 + hc
                                                             : sw[r0 + r][S.off + 1u + (hc >> kSegA)] +
                                                                   s_rt[w0 | (hc & (kSegLow - 1u))];
                                seg_cp_async_elem<T>(stg + (sl - p0) * kCols + lane + 32 * r, S.tp + rr);
                            }
                        }
                        seg_cp_commit();
                        seg_cp_wait<0>();
                        __syncwarp(__activemask());
                        for (int sl = p0; sl < min(p1, e2); ++sl)
#pragma unroll
                            for (int r = 0; r < NR; ++r) {
                                if (sl >= e0 && sl < e1 && sl - e0 >= zb4[r0 + r]) continue;  // past the row's high list
                                R vr, vi;
                                seg_ld_shared<R, CPLX>(stg + (sl - p0) * kCols + lane + 32 * r, vr, vi);
                                const bool rung = sl < e0 ? sl < nrl[r0 + r]
                                                          : (sl < e1 ? sl - e0 < zbr[r0 + r] : sl - e1 < nXr);
                                seg_add<R, CPLX, MERGED>(er[r], ei[r], lr[r], li[r], rung, vr, vi);
                            }
                        for (int sl = max(p0, e2); sl < p1; ++sl) {
                            const SegSlot<R, CPLX>& S = s_slot[sl - e2];
#pragma unroll
                            for (int r = 0; r < NR; ++r) {
                                R vr, vi;
                                seg_ld_shared<R, CPLX>(stg + (sl - p0) * kCols + lane + 32 * r, vr, vi);
                                seg_hop_acc<R, CPLX>(hr[r], hi[r], S.cr, seg_slot_ci(S), vr, vi);
                            }
                        }
                        __syncwarp(__activemask());  // the pass's slots are read before the next pass writes them
                    }
                }
                if (n0 + n12 < nhop) {
                    // hops that move more than two low positions above P: the full rank of U | V
                    const RankTab RT = rank_tab_of(*Sp, Sp->rank_tab);
#pragma unroll 1
                    for (int hh = n0 + n12; hh < nhop; ++hh) {
                        const SegHop<R, CPLX>& F = s_hop[hh];
#pragma unroll
                        for (int r = 0; r < NR; ++r) {
                            const uint32_t V = seg_perm(lnw[r0 + r] & 0xffffu, F.keep, F.band, F.sl, F.sr, F.p, F.q, F.swap,
                                                        F.rot, F.nsr, nsmask);
                            const uint32_t rr = spin_rank(sw[r0 + r][s_desc.hop_off[hh]] | V, RT, Nd);
                            R vr, vi;
                            seg_ld<R, CPLX>(F.tp + rr, vr, vi);
                            seg_hop_acc<R, CPLX>(hr[r], hi[r], F.cr, F.ci, vr, vi);
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    const int rr = r0 + r;
                    // the padding read the row itself (in split mode into the leg sum; a parallel cross
                    // bond into its own kind's sum): take it back out; then the diagonal, -J/2 per
                    // antiparallel bond
                    const int pads = (smax - nlow[rr]) + (zb4[rr] - zb[rr]) + __popc(~xm[rr] & x4mask & ~(MERGED ? 0u : xrmask));
                    R h_r, h_i;
                    if constexpr (MERGED) {
                        const R e_r = er[r] - (R)pads * xr[rr];
                        const R e_i = CPLX ? ei[r] - (R)pads * xi[rr] : R(0);
                        const R diag = -wr * (R)(nlow[rr] + zb[rr] + __popc(xm[rr]));
                        h_r = wr * e_r + hr[r] + diag * xr[rr];
                        h_i = CPLX ? wr * e_i + hi[r] + diag * xi[rr] : R(0);
                    } else {
                        const R rpad = (R)__popc(~xm[rr] & xrmask);
                        const R a_r = er[r] - rpad * xr[rr], a_i = CPLX ? ei[r] - rpad * xi[rr] : R(0);
                        const R l_r = lr[r] - (R)pads * xr[rr], l_i = CPLX ? li[r] - (R)pads * xi[rr] : R(0);
                        const int anr = nrl[rr] + zbr[rr] + __popc(xm[rr] & xrmask);
                        const int anl = (nlow[rr] - nrl[rr]) + (zb[rr] - zbr[rr]) + __popc(xm[rr] & ~xrmask);
                        const R diag = -(wr * (R)anr + wl * (R)anl);
                        h_r = wr * a_r + wl * l_r + hr[r] + diag * xr[rr];
                        h_i = CPLX ? wr * a_i + wl * l_i + hi[r] + diag * xi[rr] : R(0);
                    }
                    if (PAIR ? (rr == 0 || act1) : act[rr]) {
                        const R y_r = h_r - beta * pr[rr];
                        const R y_i = CPLX ? h_i - beta * pi[rr] : R(0);
                        st<R, CPLX>(y, (int64_t)base[rr] + tt[rr], y_r, y_i);
                        pend[0] = fma_r(xr[rr], h_r, pend[0]);
                        pend[1] = fma_r(y_r, y_r, pend[1]);
                        pend[2] = fma_r(xr[rr], y_r, pend[2]);
                        pend[3] = fma_r(xr[rr], xr[rr], pend[3]);
                        if constexpr (CPLX) {
                            pend[0] = fma_r(xi[rr], h_i, pend[0]);
                            pend[1] = fma_r(y_i, y_i, pend[1]);
                            pend[2] = fma_r(xi[rr], y_i, pend[2]);
                            pend[3] = fma_r(xi[rr], xi[rr], pend[3]);
                        }
                    }
                }
            }
            npend += 2;
            if (npend >= 4) {
#pragma unroll
                for (int q = 0; q < kReduceSlots; ++q) {
                    Accum<R> a = seg_acc_load<R>(s_acc[q], threadIdx.x);
                    fold<R>(a, pend[q]);
                    seg_acc_store<R>(s_acc[q], threadIdx.x, a);
                    pend[q] = R(0);
                }
                npend = 0;
            }
            __syncwarp(__activemask());  // every lane is done with this pair's buffer before it is refilled
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                base[r] = nbase[r];
                xr[r] = nxr[r];
                xi[r] = nxi[r];
                pr[r] = npr[r];
                pi[r] = npi[r];
            }
        }
        seg_cp_wait<0>();
        Accum<R> acc[kReduceSlots];
#pragma unroll
        for (int q = 0; q < kReduceSlots; ++q) {
            acc[q] = seg_acc_load<R>(s_acc[q], threadIdx.x);
            fold<R>(acc[q], pend[q]);
        }
        if constexpr (sizeof(R) == 4) {
            chunk_reduce(acc, partials + (int64_t)cid * kReduceSlots);
        } else {
            double tot[kReduceSlots] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value()};
            chunk_reduce(tot, partials + (int64_t)cid * kReduceSlots);
        }
    }
}

}  // namespace ed
