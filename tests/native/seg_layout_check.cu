// Host check of the segment layout of free blocks (ed_desc.cu: seg_tables; ed_seg.cuh: the index
// helpers the segment kernels call).  For many (Ns, Nd):
//   * segments tile the C(Ns, Nd) configurations: the row of (H << P) | Lo is the segment's first
//     row plus rank_P(Lo), which is the configuration's colex rank;
//   * every exchange pair (a, b) -- below P, at or above P, across P -- reaches the colex rank of the
//     flipped configuration through its per-thread and per-segment parts, and the antiparallel high
//     bonds of a segment are listed in the order seg_high_pos gives;
//   * every hop permutation (an electron moved over a band of positions, mirror pairs, a rotation)
//     reaches the colex rank of the permuted configuration, as sb[vbi] + rank_P(ua | va) when at most
//     two low positions land above P, else by the full rank.
// Built with nvcc as host code and run by tests/test_native_host.py; exits non-zero on any difference.
#include <cstdio>
#include <cstring>
#include <random>

#include "ed_desc.cu"
#include "ed_seg.cuh"

namespace ed {
int set_error(int code, const char*) { return code; }
int set_cuda_error(cudaError_t, const char*) { return ED_ERR_CUDA; }
int seg_records_build(Sector&, const std::vector<int>&, int64_t) { return ED_OK; }
}  // namespace ed

using namespace ed;

namespace {

uint32_t C[kCombStride][kCombStride];
long bad = 0, checks = 0;

void expect(bool ok, const char* what, int Ns, int Nd, uint32_t dc) {
    ++checks;
    if (!ok && bad++ < 20) std::printf("FAIL %s Ns=%d Nd=%d dc=%x\n", what, Ns, Nd, dc);
}

uint32_t colex(uint32_t m) {
    uint32_t r = 0;
    int j = 0;
    for (int b = 0; b < 32; ++b)
        if ((m >> b) & 1u) r += C[++j][b];
    return r;
}

uint32_t random_config(std::mt19937_64& rng, int Ns, int Nd) {
    uint32_t m = 0;
    for (int placed = 0; placed < Nd;) {
        const int b = (int)(rng() % (uint64_t)Ns);
        if (!((m >> b) & 1u)) {
            m |= 1u << b;
            ++placed;
        }
    }
    return m;
}

void check_sector(int Ns, int Nd, std::mt19937_64& rng, long hop_counts[4]) {
    const int P = std::min(kSegA, Ns);
    const uint32_t amask = (1u << P) - 1u, nsmask = 0xffffffffu >> (32 - Ns);
    SectorView V{};
    std::vector<uint32_t> tab;
    rank_tables_build(Ns, Nd, C, V, tab);
    const RankTab R = rank_tab_of(V, tab.data());
    // rank_P and its inverse, as the kernel builds them
    uint8_t rt[kSegLow];
    uint16_t ut[kSegLow];
    uint32_t utoff[kSegA + 2] = {};
    for (int kk = 0; kk <= P + 1; ++kk)
        for (int j = 0; j < kk; ++j) utoff[kk] += C[j][P];
    for (uint32_t m = 0; m < (1u << P); ++m) {
        uint32_t r = 0;
        int j = 0;
        for (int b = 0; b < P; ++b)
            if ((m >> b) & 1u) r += C[++j][b];
        rt[m] = (uint8_t)r;
    }
    for (uint32_t m = 0; m < (1u << P); ++m) ut[utoff[popc32(m)] + rt[m]] = (uint16_t)m;
    uint32_t off[kSegA + 2];
    std::vector<uint32_t> hs, bases;
    seg_tables(Ns, Nd, P, C, off, hs, bases);
    // tiling: every class's segments times C(P, kl) rows add up to C(Ns, Nd); sampled segments map
    // every offset to the configuration's rank
    uint64_t rows = 0;
    for (int kl = 0; kl <= P; ++kl) {
        const uint32_t nA = C[kl][P];
        const uint32_t nseg = off[kl + 1] - off[kl];
        rows += (uint64_t)nA * nseg;
        for (uint32_t s = 0; s < nseg && s < 64; ++s) {
            const uint32_t g = s < 32 ? s : nseg - 1 - (uint32_t)(rng() % nseg);
            const uint32_t H = hs[off[kl] + g];
            for (uint32_t t = 0; t < nA; ++t) {
                const uint32_t lo = ut[utoff[kl] + t];
                const uint32_t dc = (H << P) | lo;
                expect(popc32(dc) == Nd && colex(dc) == bases[off[kl] + g] + t, "segment row", Ns, Nd, dc);
            }
        }
    }
    expect(rows == C[Nd][Ns], "segments tile the block", Ns, Nd, 0);
    // exchange pairs and hop permutations on random configurations
    std::vector<SegHopDesc> hops;
    for (int h = 0; h < 64; ++h) {
        SegHopDesc G{};
        const int p = (int)(rng() % Ns);
        int q = p;
        const int r = (int)(rng() % 4);
        if (r == 1 && p + 1 < Ns) q = p + 1;
        if (r == 2 && p > 0) q = p - 1;
        if (r == 3) q = (int)(rng() % Ns);  // a move over a longer band (the periodic leg hops)
        uint32_t band = 0;
        if (q > p)
            for (int c = p + 1; c <= q; ++c) band |= 1u << c;
        else
            for (int c = q; c < p; ++c) band |= 1u << c;
        G.p = (uint8_t)p;
        G.q = (uint8_t)q;
        G.band = band;
        G.sl = q > p ? 0 : 1;
        G.sr = (uint8_t)(1 - G.sl);
        G.keep = ~(band | (1u << p));
        if (rng() % 2)
            for (int c = (int)(rng() % 2); c + 1 < Ns; c += 2 + (int)(rng() % 2)) G.swap |= 1u << c;
        G.rot = (uint8_t)((rng() % 3 == 0) ? 0 : rng() % Ns);
        if (rng() % 2) G.rot = (uint8_t)((rng() % 3 == 0 ? (Ns - 1 - rng() % 2) : rng() % 3) % Ns);
        G.nsr = (uint8_t)((Ns - G.rot) & 31);
        const uint32_t above = host_perm(G, amask, nsmask) & ~amask;
        const int nb = popc32(above);
        G.nb = (uint8_t)(nb > 2 ? 3 : nb);
        if (nb >= 1 && nb <= 2) {
            G.bpos[0] = (uint8_t)ctz32(above);
            G.bpos[1] = nb == 2 ? (uint8_t)hibit32(above) : 0;
        }
        hops.push_back(G);
    }
    // a random list of high bonds (rung / leg-1 / leg-2 masks) for the ordering check
    uint32_t mr = 0, ma = 0, m2 = 0;
    for (int a = P; a + 1 < Ns; ++a) {
        const int kind = (int)(rng() % 4);
        if (kind == 0) mr |= 1u << a;
        if (kind == 1) ma |= 1u << a;
        if (kind == 2 && a + 2 < Ns) m2 |= 1u << a;
    }
    std::vector<std::pair<int, int>> hb;  // (a, b) in list order
    for (uint32_t m = mr; m; m &= m - 1u) hb.push_back({ctz32(m), ctz32(m) + 1});
    const int nBr = (int)hb.size();
    for (uint32_t m = ma; m; m &= m - 1u) hb.push_back({ctz32(m), ctz32(m) + 1});
    const int nBa = (int)hb.size() - nBr;
    for (uint32_t m = m2; m; m &= m - 1u) hb.push_back({ctz32(m), ctz32(m) + 2});
    for (int trial = 0; trial < 300; ++trial) {
        const uint32_t dc = random_config(rng, Ns, Nd);
        const uint32_t lo = dc & amask, Hs = dc & ~amask;
        const int kl = popc32(lo);
        const uint32_t base = colex(Hs | ((1u << kl) - 1u));
        const uint32_t t = rt[lo];
        expect(base + t == colex(dc), "split rank", Ns, Nd, dc);
        for (int a = 0; a < Ns; ++a)
            for (int b = a + 1; b < Ns; ++b) {
                if (!(((dc >> a) ^ (dc >> b)) & 1u)) continue;
                const uint32_t f = (1u << a) | (1u << b);
                const uint32_t want = colex(dc ^ f);
                uint32_t got;
                if (b < P) got = base + rt[lo ^ f];
                else if (a >= P) got = seg_high_partner(Hs, a, b, kl, R, Nd) + t;
                else got = seg_cross_partner(Hs, b, kl, P, R, Nd) + rt[lo ^ (1u << a)];
                expect(got == want, "exchange partner", Ns, Nd, dc);
            }
        int pos = 0;
        for (int i = 0; i < (int)hb.size(); ++i) {
            const int a = hb[i].first, b = hb[i].second;
            if (!(((Hs >> a) ^ (Hs >> b)) & 1u)) continue;
            expect(seg_high_pos(Hs, i, (uint32_t)a, nBr, nBa, mr, ma, m2) == pos++, "high bond order", Ns, Nd, dc);
        }
        for (const SegHopDesc& G : hops) {
            const uint32_t want = colex(host_perm(G, dc, nsmask));
            const uint32_t U = host_perm(G, Hs, nsmask), Vp = host_perm(G, lo, nsmask);
            uint32_t got;
            if (G.nb >= 3) {
                got = spin_rank(U | Vp, R, Nd);
            } else {
                uint32_t sb[4] = {0, 0, 0, 0};
                for (int vbi = 0; vbi < (1 << G.nb); ++vbi)
                    sb[vbi] = seg_hop_base(U, amask, vbi, G.bpos[0], G.bpos[1], P, R, Nd);
                const uint32_t hc = seg_hop_thread(Vp, amask, G.nb, G.bpos[0], G.bpos[1]);
                got = seg_hop_rank(sb, U & amask, hc, rt);
            }
            ++hop_counts[G.nb];
            expect(got == want, "hop target", Ns, Nd, dc);
        }
    }
}

}  // namespace

int main() {
    std::memset(C, 0, sizeof(C));
    for (int n = 0; n <= kMaxN; ++n) {
        C[0][n] = 1;
        for (int k = 1; k <= n; ++k) C[k][n] = C[k - 1][n - 1] + (k <= n - 1 ? C[k][n - 1] : 0);
    }
    std::mt19937_64 rng(11);
    long hop_counts[4] = {0, 0, 0, 0};
    const int cases[][2] = {{3, 1},   {6, 3},   {8, 2},   {9, 4},   {10, 5},  {11, 3},  {12, 6},  {14, 7},
                            {14, 5},  {16, 8},  {18, 9},  {20, 10}, {22, 11}, {24, 12}, {26, 13}, {26, 12},
                            {27, 13}, {27, 14}, {28, 14}, {30, 15}, {31, 15}, {22, 2},  {22, 20}, {30, 1}};
    for (const auto& c : cases) check_sector(c[0], c[1], rng, hop_counts);
    std::printf("hops by nb: %ld %ld %ld %ld\n", hop_counts[0], hop_counts[1], hop_counts[2], hop_counts[3]);
    std::printf("checks %ld differences %ld\n", checks, bad);
    return bad != 0;
}
