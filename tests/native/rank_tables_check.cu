// Host check of the colex spin-rank tables and of the configuration enumeration used by the
// stabiliser blocks' expansion: for every spin count Ns <= 32 and down count Nd (with C(Ns, Nd) <
// 2^32), spin_rank over the tables of rank_tables_build equals the direct colex rank
// sum_j C(p_j, j) of random masks; colex_unrank inverts it; next_combination steps to rank + 1.
// Built with nvcc as host code and run by tests/test_native_host.py; exits non-zero on any
// difference.
#include <cstdio>
#include <random>
#include <vector>

#include "ed_internal.cuh"

using namespace ed;

namespace {

uint64_t direct_rank(uint32_t m, int Ns, const uint64_t (&C)[33][33]) {
    uint64_t r = 0;
    int j = 0;
    for (int b = 0; b < Ns; ++b)
        if ((m >> b) & 1u) r += C[++j][b];
    return r;
}

}  // namespace

int main() {
    uint64_t C[33][33] = {};
    for (int n = 0; n <= 32; ++n) {
        C[0][n] = 1;
        for (int k = 1; k <= n; ++k) C[k][n] = C[k - 1][n - 1] + (k <= n - 1 ? C[k][n - 1] : 0);
    }
    uint32_t comb[kCombStride][kCombStride];
    for (int k = 0; k < kCombStride; ++k)
        for (int n = 0; n < kCombStride; ++n) comb[k][n] = (uint32_t)C[k][n];
    std::mt19937_64 rng(11);
    long checks = 0, bad = 0;
    for (int Ns = 1; Ns <= 32; ++Ns)
        for (int Nd = 0; Nd <= Ns; ++Nd) {
            const uint64_t total = C[Nd][Ns];
            if (total >= (1ull << 32)) continue;
            SectorView V{};
            std::vector<uint32_t> tab;
            rank_tables_build(Ns, Nd, comb, V, tab);
            if (V.rank_words != (int)tab.size()) ++bad;
            const RankTab rt = rank_tab_of(V, tab.data());
            for (int t = 0; t < 500; ++t) {
                uint32_t m = 0;
                for (int placed = 0; placed < Nd;) {
                    const int b = (int)(rng() % (uint64_t)Ns);
                    if (!((m >> b) & 1u)) {
                        m |= 1u << b;
                        ++placed;
                    }
                }
                const uint64_t want = direct_rank(m, Ns, C);
                const uint32_t got = spin_rank(m, rt, Nd);
                const uint32_t back = colex_unrank((int64_t)want, Ns, Nd, &comb[0][0]);
                bool ok = got == want && back == m;
                if (want + 1 < total) ok = ok && direct_rank(next_combination(m), Ns, C) == want + 1;
                ++checks;
                if (!ok && bad++ < 10)
                    std::printf("Ns=%d Nd=%d m=%x: rank %llu table %u unrank %x\n", Ns, Nd, m,
                                (unsigned long long)want, got, back);
            }
        }
    std::printf("checks %ld differences %ld\n", checks, bad);
    return bad != 0;
}
