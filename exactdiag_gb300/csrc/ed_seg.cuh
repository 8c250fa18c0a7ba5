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
// A thread owns one offset t of every segment in its slot (segments g = begin + slot, + slots, ...);
// threads never wait on one another inside a chunk.  Each row issues its gathers in groups (low and
// high bonds eight at a time, cross bonds all at once, hops six at a time) before it adds them up.
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

// Per-thread part of a hop: rank_P(V) when nb = 0, else V's low bits and vbi (bits 9, 10).
__host__ __device__ __forceinline__ uint32_t seg_hop_thread(uint32_t V, uint32_t amask, uint32_t nb, uint32_t bp0,
                                                            uint32_t bp1, const uint8_t* rt) {
    if (nb == 0) return rt[V];
    return (V & amask) | ((((V >> bp0) & 1u) | (nb == 2 ? ((V >> bp1) & 1u) << 1 : 0u)) << 9);
}

// Target rank of a hop (nb <= 2) from its per-segment (sb, ua) and per-thread (hc) parts.
__host__ __device__ __forceinline__ uint32_t seg_hop_rank(uint32_t nb, const uint32_t* sb, uint32_t ua, uint32_t hc,
                                                          const uint8_t* rt) {
    if (nb == 0) return sb[0] + hc;
    return sb[hc >> 9] + rt[ua | (hc & 511u)];
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

template <typename R, bool CPLX, int MINB>
__global__ void __launch_bounds__(kSegThreads, MINB)
    seg_step_kernel(const SectorView* __restrict__ views, const int64_t* __restrict__ offs,
                    const BatchChunk* __restrict__ chunks, const int* __restrict__ idx, int count, HvWeights W,
                    void* v, void* vprev, void* other, int first, const double* __restrict__ scal, int stride, int k,
                    double* __restrict__ partials, void* xfull) {
    using T = typename Vec<R, CPLX>::T;
    __shared__ uint8_t s_rt[kSegLow];           // rank_P of each P-bit mask within its popcount class
    __shared__ uint16_t s_ut[kSegLow];          // the masks by (popcount, rank_P)
    __shared__ uint32_t s_utoff[kSegA + 2];
    __shared__ __align__(16) SegDesc s_desc;
    __shared__ __align__(16) SegHop<R, CPLX> s_hop[kMaxHops];
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

    for (int c = blockIdx.x; c < count; c += gridDim.x) {
        const int cid = idx[c];
        const BatchChunk ch = chunks[cid];
        const SectorView* Sp = views + ch.sec;
        const int kl = ch.kl, Ns = Sp->Ns, Nd = Sp->Nd, N = Sp->N, L = Sp->L;
        const uint32_t nsmask = 0xffffffffu >> (32 - Ns);
        const int nA = (int)comb[kl * kCombStride + P];
        const int nslots = min(kSegSlots, (kSegThreads - 1) / nA);
        const int slot = (int)threadIdx.x / nA, t = (int)threadIdx.x - slot * nA;
        const bool act = slot < nslots;
        __syncthreads();  // the previous chunk's rows are done with the shared descriptor and hops
        {
            const uint4* src = reinterpret_cast<const uint4*>(Sp->seg + ch.block);
            uint4* dst = reinterpret_cast<uint4*>(&s_desc);
            for (int i = threadIdx.x; i < (int)(sizeof(SegDesc) / 16); i += blockDim.x) dst[i] = src[i];
        }
        __syncthreads();
        const int nhop = s_desc.nhop, nX = s_desc.nX, nXr = s_desc.nXr;
        const int64_t bstart = s_desc.start;
        T* const x = reinterpret_cast<T*>(v) + offs[ch.sec];
        const T* const xb = x + bstart;
        if ((int)threadIdx.x < kMaxHops) {
            // every hop slot gets a record: absent hops (and slots past nhop) read a valid element with
            // coefficient 0
            const int h = threadIdx.x;
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
        }
        __syncthreads();

        // ---- per-thread terms of Lo (fixed for every segment of the chunk)
        uint64_t aw0 = 0, aw1 = 0;   // rank_P of the antiparallel low-bond partners (bytes; 0 past na)
        uint64_t xw = 0;             // cross bond c: rank_P(Lo ^ low end) (byte c)
        uint32_t hw[kMaxHops / 2] = {0, 0, 0, 0, 0, 0};  // hop: 16-bit rank_P(V) (nb 0) or va | vbi << 9
        uint32_t lo = 0, lob = 0;
        int na = 0, nar = 0;
        if (act) {
            lo = s_ut[s_utoff[kl] + t];
            const int nAb = s_desc.nA, nAr = s_desc.nAr;
            for (int i = 0; i < nAb; ++i) {
                const uint32_t f = s_desc.fA[i], sb = lo & f;
                if (sb != 0u && sb != f) {
                    const uint64_t o = (uint64_t)s_rt[lo ^ f];
                    if (na < 8) aw0 |= o << (8 * na);
                    else aw1 |= o << (8 * (na - 8));
                    ++na;
                    if (i < nAr) ++nar;
                }
            }
#pragma unroll
            for (int cc = 0; cc < kSegMaxX; ++cc) {
                if (cc < nX) {
                    const uint32_t a = s_desc.cX[cc][0];
                    lob |= ((lo >> a) & 1u) << cc;
                    xw |= (uint64_t)s_rt[lo ^ (1u << a)] << (8 * cc);
                }
            }
#pragma unroll
            for (int h = 0; h < kMaxHops; ++h) {
                const SegHop<R, CPLX>& F = s_hop[h];
                if (h < nhop && F.kind != 3 && F.nb < 3) {
                    const uint32_t V = seg_perm(lo, F.keep, F.band, F.sl, F.sr, F.p, F.q, F.swap, F.rot, F.nsr, nsmask);
                    hw[h >> 1] |= seg_hop_thread(V, amask, F.nb, F.bp0, F.bp1, s_rt) << (16 * (h & 1));
                }
            }
        }
        const int namax = (int)__reduce_max_sync(0xffffffffu, (unsigned)na);
        bool ngen = false;  // the block has hops that take the full rank per row
        for (int h = 0; h < nhop; ++h) ngen = ngen || (s_hop[h].nb >= 3 && s_hop[h].kind != 3);
        const uint32_t rec_len = s_desc.rec_len;
        const uint32_t* __restrict__ rec0 = Sp->seg_rec + s_desc.rec + (int64_t)Sp->seg_off[kl] * rec_len;
        const uint32_t xoff_w = 2u + s_desc.nB;  // first cross-partner word
        T* const y = reinterpret_cast<T*>(other) + offs[ch.sec] + bstart;
        const T* const yp = first ? nullptr : reinterpret_cast<const T*>(vprev) + offs[ch.sec] + bstart;
        const R beta = first ? R(0) : (R)scal[(int64_t)ch.sec * stride + 2 * k];

        Accum<R> acc[kReduceSlots];
        R pend[kReduceSlots] = {R(0), R(0), R(0), R(0)};
        int npend = 0;
        for (int64_t g = ch.begin + slot; act && g < ch.end; g += nslots) {
            const uint32_t* __restrict__ rec = rec0 + g * (int64_t)rec_len;
            const uint32_t base = __ldg(rec), w1 = __ldg(rec + 1);
            const int zb = (int)(w1 & 255u), zbr = (int)((w1 >> 8) & 255u);
            const uint32_t hib = w1 >> 16;
            const T* const xs = xb + base;  // the segment
            const T* const xt = xb + t;     // this row's offset in every segment of the block
            R xr, xi, pr = R(0), pi = R(0);
            seg_ld<R, CPLX>(xs + t, xr, xi);
            if (!first) seg_ld<R, CPLX>(yp + base + t, pr, pi);  // v_{k-1}; may share y's buffer (read first)
            R arr = R(0), ari = R(0), alr = R(0), ali = R(0), hr = R(0), hi = R(0);
            // exchange bonds below P: partners in the same segment (L1), eight loads in flight
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                if (half * 8 < namax) {
                    const uint64_t aw = half ? aw1 : aw0;
                    R vr[8], vi[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) seg_ld<R, CPLX>(xs + (uint32_t)((aw >> (8 * u)) & 255u), vr[u], vi[u]);
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int q = half * 8 + u;
                        if (q >= na) continue;
                        if (q < nar) {
                            arr += vr[u];
                            if constexpr (CPLX) ari += vi[u];
                        } else {
                            alr += vr[u];
                            if constexpr (CPLX) ali += vi[u];
                        }
                    }
                }
            }
            // exchange bonds at or above P: the partner segments at the same offset, eight loads in flight
            for (int q0 = 0; q0 < zb; q0 += 8) {
                R vr[8], vi[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int q = q0 + u;
                    const uint32_t o = q < zb ? __ldg(rec + 2 + q) : 0u;
                    seg_ld<R, CPLX>(xt + o, vr[u], vi[u]);
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int q = q0 + u;
                    if (q >= zb) continue;
                    if (q < zbr) {
                        arr += vr[u];
                        if constexpr (CPLX) ari += vi[u];
                    } else {
                        alr += vr[u];
                        if constexpr (CPLX) ali += vi[u];
                    }
                }
            }
            // bonds across P (antiparallel when the two ends' spins differ)
            const uint32_t xm = (lob ^ hib) & ((1u << nX) - 1u);
            {
                R vr[kSegMaxX], vi[kSegMaxX];
#pragma unroll
                for (int cc = 0; cc < kSegMaxX; ++cc) {
                    vr[cc] = vi[cc] = R(0);
                    if (cc < nX) {
                        const bool on = (xm >> cc) & 1u;
                        const uint32_t o = on ? __ldg(rec + xoff_w + cc) + (uint32_t)((xw >> (8 * cc)) & 255u) : 0u;
                        seg_ld<R, CPLX>(xb + o, vr[cc], vi[cc]);
                        if (!on) vr[cc] = vi[cc] = R(0);
                    }
                }
#pragma unroll
                for (int cc = 0; cc < kSegMaxX; ++cc) {
                    if (cc < nXr) {
                        arr += vr[cc];
                        if constexpr (CPLX) ari += vi[cc];
                    } else {
                        alr += vr[cc];
                        if constexpr (CPLX) ali += vi[cc];
                    }
                }
            }
            // hops: six target addresses, then their loads, then the products
#pragma unroll
            for (int h0 = 0; h0 < kMaxHops; h0 += 6) {
                if (h0 < nhop) {
                    R vr[6], vi[6];
#pragma unroll
                    for (int u = 0; u < 6; ++u) {
                        const int h = h0 + u;
                        vr[u] = vi[u] = R(0);
                        if (h < nhop && s_hop[h].nb < 3) {
                            const SegHop<R, CPLX>& F = s_hop[h];
                            const uint32_t* hr_ = rec + s_desc.hop_off[h];
                            const uint32_t hc = (hw[h >> 1] >> (16 * (h & 1))) & 0xffffu;
                            const uint32_t r = F.nb == 0 ? __ldg(hr_) + hc
                                                         : __ldg(hr_ + 1 + (hc >> 9)) + s_rt[__ldg(hr_) | (hc & 511u)];
                            seg_ld<R, CPLX>(F.tp + r, vr[u], vi[u]);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 6; ++u) {
                        const int h = h0 + u;
                        if (h < nhop) {
                            const R cr = s_hop[h].cr, ci = s_hop[h].ci;
                            hr += cr * vr[u];
                            if constexpr (CPLX) {
                                hr -= ci * vi[u];
                                hi += cr * vi[u] + ci * vr[u];
                            }
                        }
                    }
                }
            }
            if (ngen) {
                // hops that move more than two low positions above P: the full rank of U | V
                const RankTab RT = rank_tab_of(*Sp, Sp->rank_tab);
#pragma unroll 1
                for (int h = 0; h < nhop; ++h) {
                    const SegHop<R, CPLX>& F = s_hop[h];
                    if (F.nb < 3 || F.kind == 3) continue;
                    const uint32_t V = seg_perm(lo, F.keep, F.band, F.sl, F.sr, F.p, F.q, F.swap, F.rot, F.nsr, nsmask);
                    const uint32_t r = spin_rank(__ldg(rec + s_desc.hop_off[h]) | V, RT, Nd);
                    R vr, vi;
                    seg_ld<R, CPLX>(F.tp + r, vr, vi);
                    hr += F.cr * vr;
                    if constexpr (CPLX) {
                        hr -= F.ci * vi;
                        hi += F.cr * vi + F.ci * vr;
                    }
                }
            }
            // diagonal: -J/2 per antiparallel bond
            const uint32_t rmask = (1u << nXr) - 1u;
            const R diag = -(wr * (R)(nar + zbr + __popc(xm & rmask)) +
                             wl * (R)((na - nar) + (zb - zbr) + __popc(xm & ~rmask)));
            const R h_r = wr * arr + wl * alr + hr + diag * xr;
            const R h_i = CPLX ? (wr * ari + wl * ali + hi + diag * xi) : R(0);
            const R yr = h_r - beta * pr;
            const R yi = CPLX ? h_i - beta * pi : R(0);
            st<R, CPLX>(y, (int64_t)base + t, yr, yi);
            pend[0] = fma(xr, h_r, pend[0]);
            pend[1] = fma(yr, yr, pend[1]);
            pend[2] = fma(xr, yr, pend[2]);
            pend[3] = fma(xr, xr, pend[3]);
            if constexpr (CPLX) {
                pend[0] = fma(xi, h_i, pend[0]);
                pend[1] = fma(yi, yi, pend[1]);
                pend[2] = fma(xi, yi, pend[2]);
                pend[3] = fma(xi, xi, pend[3]);
            }
            if (++npend == 4) {
#pragma unroll
                for (int q = 0; q < kReduceSlots; ++q) {
                    fold<R>(acc[q], pend[q]);
                    pend[q] = R(0);
                }
                npend = 0;
            }
        }
#pragma unroll
        for (int q = 0; q < kReduceSlots; ++q) fold<R>(acc[q], pend[q]);
        if constexpr (sizeof(R) == 4) {
            chunk_reduce(acc, partials + (int64_t)cid * kReduceSlots);
        } else {
            double tot[kReduceSlots] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value()};
            chunk_reduce(tot, partials + (int64_t)cid * kReduceSlots);
        }
    }
}

}  // namespace ed
