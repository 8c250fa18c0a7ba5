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

}  // namespace

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
    return ED_OK;
}

}  // namespace ed
