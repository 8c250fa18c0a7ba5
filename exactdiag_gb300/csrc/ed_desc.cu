// ed_desc.cu -- per-block descriptors of the fast H.v row, built once per sector.
//
// For each eligible hole mask (block) of a built basis this precomputes everything of the
// reference's matrix-element rule (tJ_spin_half_ladder/matrix_setup.pyx:80-110,
// general/column_functions.h:99-148) that depends on the holes only:
//   * the exchange bonds in compressed-spin coordinates (rung, leg with a hole in the middle,
//     leg with an electron in the middle, leg across the periodic boundary);
//   * for each hop (hole b, electron a at a leg or rung neighbour): the fermion sign
//     (electrons strictly between a and b, column_functions.h:317-346), how the electron moves
//     in the compressed string, and the target: its block and the group elements that map the
//     new hole mask to the canonical one, each with its compressed-string permutation and its
//     phase exponent (the cumulative rule of symmetry_ladder.h:157-175);
//   * the block's own stabiliser (for resolving exchange targets of non-free blocks).
// A hop or block whose canonical mask has more than kMaxCand such elements (e.g. the undoped
// sector) keeps the reference-faithful orbit walk.
#include <algorithm>
#include <vector>

#include "ed_internal.cuh"

namespace ed {

namespace {

struct HostSector {
    int L, N, Nh, Ns, kx, ky, ne_even;
    uint32_t mask;
};

int cpos(const HostSector& S, uint32_t h, int site) {
    return popc32(~h & S.mask & ((1u << site) - 1u));
}

// Phase exponent of product index p applied to a state with hole mask h (orbit_walk's rule).
int phase_exponent(const HostSector& S, uint32_t h, int p) {
    const int L = S.L, twoL = 2 * L;
    const uint32_t single = (h ^ (h >> 1)) & 0x55555555u & S.mask;
    const uint32_t any_hole = (h | (h >> 1)) & 0x55555555u & S.mask;
    const int P = L - popc32(any_hole);
    const int e_mirror = (L * S.ky + L * (P & 1)) % twoL;
    int eT = 0;
    for (int s = 1; s <= (p >> 1); ++s) {
        eT += 2 * S.kx;
        if (S.ne_even && ((single >> (2 * (L - s))) & 1u)) eT += L;
        eT %= twoL;
    }
    return (p & 1) ? (eT + e_mirror) % twoL : eT;
}

uint32_t image_holes(const HostSector& S, uint32_t h, int p) {
    uint32_t d = 0;
    apply_p(p, h, d, S.N, S.mask);
    return h;
}

// The permutation of compressed masks that product index p induces on states with hole mask h.
CandParams cand_params(const HostSector& S, uint32_t h, int p, int e) {
    CandParams c{};
    c.p = (uint8_t)p;
    c.e = (uint8_t)e;
    if (p & 1) {
        for (int x = 0; x < S.L; ++x)
            if (!((h >> (2 * x)) & 3u)) c.swap |= 1u << cpos(S, h, 2 * x);
    }
    const int s = p >> 1;
    if (s > 0) {
        const uint32_t hm = (p & 1) ? mirror_legs(h) : h;
        const uint32_t high = S.mask & ~((1u << (S.N - 2 * s)) - 1u);
        c.rot = (uint8_t)popc32(~hm & high);
    }
    return c;
}

// Group elements mapping h to hc (all p with image_p(h) == hc), up to kMaxCand of them.
int coset(const HostSector& S, uint32_t h, uint32_t hc, CandParams* out) {
    int n = 0;
    for (int p = 0; p < S.N; ++p) {
        if (image_holes(S, h, p) != hc) continue;
        if (n < kMaxCand) out[n] = cand_params(S, h, p, phase_exponent(S, h, p));
        ++n;
    }
    return n;
}

// Host copy of the hop permutation (ed_seg.cuh: seg_perm).
uint32_t host_perm(const SegHopDesc& G, uint32_t x, uint32_t nsmask) {
    const uint32_t xm = (x & G.keep) | (((x & G.band) << G.sl) >> G.sr) | (((x >> G.p) & 1u) << G.q);
    const uint32_t t = (xm ^ (xm >> 1)) & G.swap;
    const uint32_t sw = xm ^ t ^ (t << 1);
    return ((sw << G.rot) | (sw >> G.nsr)) & nsmask;
}

// Segment descriptor of a free block from its row descriptor: the exchange bonds sorted by where
// their ends lie relative to P, each hop as a compressed-mask permutation with its target, and the
// layout of the block's segment records.  copy_index[b]: index of block b's expanded copy among the
// sector's copies (-1: none).
SegDesc make_seg_desc(const BlockDesc& D, int Ns, int P, const std::vector<int>& copy_index) {
    SegDesc G{};
    G.start = D.start;
    G.ok = 1;
    const uint32_t nsmask = 0xffffffffu >> (32 - Ns);
    const uint32_t amask = (1u << P) - 1u;
    struct Bond {
        int a, b, kind;  // kind 0 rung, 1 leg at distance one, 2 leg at distance two, 3 leg across the boundary
    };
    std::vector<Bond> bonds;
    for (uint32_t m = D.m_rung; m; m &= m - 1u) bonds.push_back({ctz32(m), ctz32(m) + 1, 0});
    for (uint32_t m = D.m_legadj; m; m &= m - 1u) bonds.push_back({ctz32(m), ctz32(m) + 1, 1});
    for (uint32_t m = D.m_legd2; m; m &= m - 1u) bonds.push_back({ctz32(m), ctz32(m) + 2, 2});
    for (int u = 0; u < D.nwrap; ++u) bonds.push_back({D.wrap[u][0], D.wrap[u][1], 3});
    // low and cross bonds: rung bonds first
    for (int pass = 0; pass < 2; ++pass)
        for (const Bond& bd : bonds) {
            if ((bd.kind == 0) != (pass == 0)) continue;
            const bool rung = bd.kind == 0;
            if (bd.b < P) {
                if (G.nA >= kSegMaxA) {
                    G.ok = 0;
                    continue;
                }
                G.fA[G.nA++] = (1u << bd.a) | (1u << bd.b);
                if (rung) ++G.nAr;
            } else if (bd.a >= P) {
                // high bonds are ranked by kind (rung, leg-1, leg-2) in the kernel: no boundary bonds here
                if (bd.kind == 3) G.ok = 0;
            } else {
                if (G.nX >= kSegMaxX) {
                    G.ok = 0;
                    continue;
                }
                G.cX[G.nX][0] = (uint8_t)bd.a;
                G.cX[G.nX][1] = (uint8_t)bd.b;
                ++G.nX;
                if (rung) ++G.nXr;
            }
        }
    for (int kind = 0; kind < 3; ++kind)
        for (const Bond& bd : bonds) {
            if (bd.kind != kind || bd.a < P) continue;
            if (G.nB >= kSegMaxB) {
                G.ok = 0;
                continue;
            }
            G.bB[G.nB][0] = (uint8_t)bd.a;
            G.bB[G.nB][1] = (uint8_t)bd.b;
            ++G.nB;
            if (kind == 0) {
                ++G.nBr;
                G.mr |= 1u << bd.a;
            }
            if (kind == 1) {
                ++G.nBa;
                G.ma |= 1u << bd.a;
            }
            if (kind == 2) G.m2 |= 1u << bd.a;
        }
    G.nhop = D.nhop;
    for (int t = 0; t < D.nhop; ++t) {
        const HopDesc& H = D.hop[t];
        SegHopDesc& S = G.hop[t];
        S.p = H.p;
        S.q = H.q;
        S.band = H.band;
        S.sl = H.q > H.p ? 0 : 1;
        S.sr = (uint8_t)(1 - S.sl);
        S.keep = ~(H.band | (1u << H.p));
        S.swap = H.swap;
        S.rot = H.rot;
        S.nsr = (uint8_t)((Ns - H.rot) & 31);
        S.term = H.term;
        S.sign = H.sign > 0 ? 1 : 0;  // 1: coefficient -w (the hopping term's -t times a positive fermion sign)
        S.e = H.e;
        S.tblock = H.block;
        if (H.mode == kModeFree) {
            S.kind = 0;
            S.tstart = H.start;
        } else if (H.mode == kModeCand && H.block >= 0 && copy_index[H.block] >= 0) {
            S.kind = 1;
            S.tstart = copy_index[H.block];
        } else {
            S.kind = 3;  // no target block, or a stabiliser target without representatives
        }
        const uint32_t above = host_perm(S, amask, nsmask) & ~amask;
        const int nb = popc32(above);
        S.nb = (uint8_t)(nb > 2 ? 3 : nb);
        if (nb >= 1 && nb <= 2) {
            S.bpos[0] = (uint8_t)ctz32(above);
            S.bpos[1] = nb == 2 ? (uint8_t)hibit32(above) : 0;
        }
        if (S.kind == 3) S.nb = 0;  // an absent hop keeps one zero record word and contributes nothing
    }
    // hops by kind: nb = 0 (and absent), nb 1 or 2, nb 3 (stable within a kind)
    {
        SegHopDesc sorted[kMaxHops];
        int n = 0;
        for (int cls = 0; cls < 3; ++cls)
            for (int t = 0; t < D.nhop; ++t) {
                const int nb = G.hop[t].nb;
                if ((cls == 0 && nb == 0) || (cls == 1 && (nb == 1 || nb == 2)) || (cls == 2 && nb == 3)) {
                    sorted[n++] = G.hop[t];
                    if (cls == 0) ++G.n0;
                    if (cls == 1) ++G.n12;
                }
            }
        for (int t = 0; t < D.nhop; ++t) G.hop[t] = sorted[t];
    }
    // record layout: header, high-bond partners (rung then leg, padded to a multiple of four), cross
    // partners, then each hop's words
    G.HB = (uint8_t)((G.nB + 3) & ~3);
    uint32_t w = 4u + G.HB;
    G.xo = (uint8_t)w;
    w += G.nX;
    for (int t = 0; t < D.nhop; ++t) {
        G.hop_off[t] = (uint8_t)w;
        const int nb = G.hop[t].nb;
        w += nb == 0 ? 1u : (nb <= 2 ? 1u + (1u << nb) : 1u);
    }
    G.zero_w = (uint8_t)w;
    w += 2u;
    G.rec_len = (w + 3u) & ~3u;
    if (G.rec_len > 128u) G.ok = 0;  // a record is staged in one 16-byte copy per lane of a warp
    return G;
}

}  // namespace

// Per class kl = 0 .. P of down spins below P: the high parts H (Ns - P bits, Nd - kl set) in colex
// order and each segment's first row in a block, the colex rank of (H << P) | (2^kl - 1); off[kl] is
// the first segment of class kl (off[P + 1] = all segments).
void seg_tables(int Ns, int Nd, int P, const uint32_t (&comb)[kCombStride][kCombStride], uint32_t* off,
                std::vector<uint32_t>& hs, std::vector<uint32_t>& bases) {
    const int B = Ns - P;
    hs.clear();
    bases.clear();
    for (int kl = 0; kl <= P + 1; ++kl) {
        off[kl] = (uint32_t)hs.size();
        if (kl > P) break;
        const int kh = Nd - kl;  // down spins of the high part
        if (kh < 0 || kh > B) continue;
        const uint64_t count = comb[kh][B];
        uint32_t H = kh == 0 ? 0u : ((1u << kh) - 1u);
        for (uint64_t g = 0; g < count; ++g) {
            uint32_t r = 0;
            int j = kl;
            for (uint32_t m = H; m; m &= m - 1u) {
                ++j;
                r += comb[j][P + ctz32(m)];
            }
            hs.push_back(H);
            bases.push_back(r);
            if (g + 1 < count) H = next_combination(H);
        }
    }
}

// The sector's expanded copies (Sector::copy_blocks) and the segment layout of its free blocks: the
// segment tables, the segment descriptors and the segment records.
int build_segments(Sector& s, const std::vector<BlockDesc>& desc, const uint32_t (&comb)[kCombStride][kCombStride]) {
    SectorView& V = s.view;
    V.seg = nullptr;
    V.seg_h = V.seg_base = V.seg_rec = nullptr;
    const int Ns = V.Ns, Nd = V.Nd;
    const int P = std::min(kSegA, Ns);
    V.seg_p = P;
    // blocks whose values are expanded every step (ExpandTask), in block order: the stabiliser blocks
    // with rows, and the blocks with a stabiliser that hops out of free blocks reach (whatever kernel
    // their own rows take); copy_index[b] is b's place in that list
    std::vector<int> copy_index(V.n_blocks, -1);
    {
        std::vector<char> need(V.n_blocks, 0);
        for (const BlockSpan& sp : s.spans) {
            if (sp.count <= 0) continue;
            if (sp.kind == kRowsCand) need[sp.block] = 1;
            if (sp.kind != kRowsFree) continue;
            const BlockDesc& D = desc[sp.block];
            for (int t = 0; t < D.nhop; ++t)
                if (D.hop[t].mode == kModeCand && D.hop[t].block >= 0 && s.spans[D.hop[t].block].count > 0)
                    need[D.hop[t].block] = 1;
        }
        s.copy_blocks.clear();
        for (int b = 0; b < V.n_blocks; ++b)
            if (need[b]) {
                copy_index[b] = (int)s.copy_blocks.size();
                s.copy_blocks.push_back(b);
            }
    }
    bool any = false;
    for (const BlockSpan& sp : s.spans) any = any || sp.kind == kRowsFree;
    if (!any) return ED_OK;
    std::vector<uint32_t> hs, bases;
    seg_tables(Ns, Nd, P, comb, V.seg_off, hs, bases);
    std::vector<SegDesc> seg(V.n_blocks);
    std::vector<int> free_blocks;
    int64_t rec_words = 0;
    const int64_t nseg = (int64_t)hs.size();
    for (const BlockSpan& sp : s.spans) {
        if (sp.kind != kRowsFree) continue;
        SegDesc& G = seg[sp.block];
        G = make_seg_desc(desc[sp.block], Ns, P, copy_index);
        if (!G.ok) return set_error(ED_ERR_INTERNAL, "segments: a free block's terms exceed the segment limits");
        G.rec = rec_words;
        rec_words += nseg * (int64_t)G.rec_len;
        free_blocks.push_back(sp.block);
    }
    if (!s.d_seg_h.alloc((int64_t)hs.size()) || !s.d_seg_base.alloc((int64_t)bases.size()) ||
        !s.d_seg.alloc(V.n_blocks) || !s.d_seg_rec.alloc(rec_words))
        return set_error(ED_ERR_NOMEM, "segments: device allocation");
    if (cudaMemcpy(s.d_seg_h.p, hs.data(), hs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s.d_seg_base.p, bases.data(), bases.size() * sizeof(uint32_t), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(s.d_seg.p, seg.data(), seg.size() * sizeof(SegDesc), cudaMemcpyHostToDevice) != cudaSuccess)
        return set_error(ED_ERR_CUDA, "segments: upload");
    V.seg_h = s.d_seg_h.p;
    V.seg_base = s.d_seg_base.p;
    V.seg = s.d_seg.p;
    V.seg_rec = s.d_seg_rec.p;
    s.host_seg_off.assign(V.seg_off, V.seg_off + P + 2);
    return seg_records_build(s, free_blocks, nseg);
}

int build_descriptors(Sector& s) {
    SectorView& V = s.view;
    V.desc = nullptr;
    s.spans.clear();
    if (V.n_blocks == 0 || !V.holes) return ED_OK;
    const HostSector S{V.L, V.N, V.Nh, V.Ns, V.kx, V.ky, V.ne_even, V.mask};
    std::vector<BlockInfo> blocks(V.n_blocks);
    std::vector<HoleEntry> holes(s.n_hole_masks);
    if (cudaMemcpy(blocks.data(), V.blocks, blocks.size() * sizeof(BlockInfo), cudaMemcpyDeviceToHost) !=
            cudaSuccess ||
        cudaMemcpy(holes.data(), V.holes, holes.size() * sizeof(HoleEntry), cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error(ED_ERR_CUDA, "descriptors: copying block tables");
    uint32_t comb[kCombStride][kCombStride];
    if (cudaMemcpy(comb, V.comb, sizeof(comb), cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error(ED_ERR_CUDA, "descriptors: copying combinatorics");
    std::vector<BlockDesc> desc(V.n_blocks);
    const int N = S.N;
    for (int b = 0; b < V.n_blocks; ++b) {
        BlockDesc D{};
        const uint32_t h = blocks[b].hmask;
        D.hmask = h;
        D.start = blocks[b].start;
        D.word_off = blocks[b].word_off;
        const uint32_t occ = ~h & S.mask;
        // own stabiliser
        const int nst = coset(S, h, h, D.cand);
        D.ncand = (uint8_t)std::min(nst, kMaxCand);
        D.mode = (nst == 1) ? kModeFree : (nst <= kMaxCand ? kModeCand : kModeGeneric);
        if (S.Nh > 4) D.mode = kModeGeneric;
        // the fast rows take the first stabiliser candidate to be the identity (its image is the state)
        if (D.mode == kModeCand && (D.cand[0].p != 0 || D.cand[0].swap != 0 || D.cand[0].rot != 0))
            D.mode = kModeGeneric;
        if (D.mode == kModeGeneric) {
            desc[b] = D;
            continue;
        }
        // exchange bonds in compressed coordinates
        for (int x = 0; x < S.L; ++x)
            if (((occ >> (2 * x)) & 3u) == 3u) D.m_rung |= 1u << cpos(S, h, 2 * x);
        for (int a = 0; a + 2 < N; ++a) {
            if (!((occ >> a) & 1u) || !((occ >> (a + 2)) & 1u)) continue;
            if ((occ >> (a + 1)) & 1u) D.m_legd2 |= 1u << cpos(S, h, a);
            else D.m_legadj |= 1u << cpos(S, h, a);
        }
        for (int a = N - 2; a < N; ++a) {
            const int partner = a + 2 - N;
            if (!((occ >> a) & 1u) || !((occ >> partner) & 1u)) continue;
            D.wrap[D.nwrap][0] = (uint8_t)cpos(S, h, partner);
            D.wrap[D.nwrap][1] = (uint8_t)cpos(S, h, a);
            ++D.nwrap;
        }
        // hops: hole b, electron a at b+2, b-2 (leg) and b^1 (rung)
        int nh = 0;
        for (uint32_t hs = h; hs; hs &= hs - 1u) {
            const int hb = ctz32(hs);
            const int nbr[3] = {(hb + 2) % N, (hb - 2 + N) % N, hb ^ 1};
            for (int t = 0; t < 3; ++t) {
                const int a = nbr[t];
                if (!((occ >> a) & 1u) || a == hb) continue;
                HopDesc H{};
                H.term = (t < 2) ? 0 : 1;
                H.a = (uint8_t)a;
                H.b = (uint8_t)hb;
                const int lo = std::min(a, hb), hi = std::max(a, hb);
                const uint32_t between = ((1u << hi) - 1u) & ~((2u << lo) - 1u);
                H.sign = (popc32(occ & between) & 1) ? -1 : 1;
                const uint32_t h2 = h ^ (1u << a) ^ (1u << hb);
                H.p = (uint8_t)cpos(S, h, a);
                H.q = (uint8_t)cpos(S, h2, hb);
                uint32_t band = 0;
                if (H.q > H.p)
                    for (int c = H.p + 1; c <= H.q; ++c) band |= 1u << c;
                else
                    for (int c = H.q; c < H.p; ++c) band |= 1u << c;
                H.band = band;
                const HoleEntry he = holes[hole_rank(h2, &comb[0][0])];
                H.block = he.block;
                if (he.block < 0) {
                    H.mode = kModeAbsent;
                } else {
                    const BlockInfo& T = blocks[he.block];
                    H.start = T.start;
                    H.word_off = T.word_off;
                    const int nc = coset(S, h2, T.hmask, H.cand);
                    H.ncand = (uint8_t)std::min(nc, kMaxCand);
                    H.mode = (nc == 1) ? kModeFree : (nc <= kMaxCand ? kModeCand : kModeGeneric);
                    H.swap = H.cand[0].swap;
                    H.rot = H.cand[0].rot;
                    H.e = H.cand[0].e;
                }
                if (nh < kMaxHops) D.hop[nh++] = H;
            }
        }
        D.nhop = (uint8_t)nh;
        // a block with a hop whose target needs the orbit walk takes the orbit walk for all its rows:
        // the fast-row kernels then never carry that code
        for (int t = 0; t < nh; ++t)
            if (D.hop[t].mode == kModeGeneric) D.mode = kModeGeneric;
        desc[b] = D;
    }
    // row ranges of the blocks by kind; they tile [0, n) in block order
    int64_t next = 0;
    for (int b = 0; b < V.n_blocks; ++b) {
        const int mode = desc[b].mode;
        const int kind = mode == kModeFree ? kRowsFree : (mode == kModeCand ? kRowsCand : kRowsGeneric);
        if (blocks[b].start != next) return set_error(ED_ERR_INTERNAL, "descriptors: block rows are not contiguous");
        s.spans.push_back(BlockSpan{blocks[b].start, blocks[b].count, b, kind});
        next += blocks[b].count;
    }
    if (next != V.n) return set_error(ED_ERR_INTERNAL, "descriptors: block rows do not cover the sector");
    if (!s.d_desc.alloc(V.n_blocks)) return set_error(ED_ERR_NOMEM, "descriptors: device allocation");
    if (cudaMemcpy(s.d_desc.p, desc.data(), desc.size() * sizeof(BlockDesc), cudaMemcpyHostToDevice) != cudaSuccess)
        return set_error(ED_ERR_CUDA, "descriptors: upload");
    V.desc = s.d_desc.p;
    return build_segments(s, desc, comb);
}

}  // namespace ed
