// Host check of the descriptor builder's group phases (ed_desc.cu: coset, phase_exponent).
// Resolving a spin configuration through the coset {g : g(h) = hc} of a hole mask h must agree
// with taking it to the canonical mask hc by the coset's first element g0 and resolving there with
// hc's stabiliser: same lowest image, count and validity, phase e(g0) + e_stab (mod 2L) -- the
// cocycle property of the symmetry amplitudes.  Built with nvcc as host code and run by
// tests/test_native_host.py; exits non-zero on any difference.
#include <cstdio>
#include <random>

#include "ed_desc.cu"

namespace ed {
int set_error(int code, const char*) { return code; }
int set_cuda_error(cudaError_t, const char*) { return ED_ERR_CUDA; }
int seg_records_build(Sector&, const std::vector<int>&, int64_t) { return ED_OK; }
}  // namespace ed

using namespace ed;

namespace {

uint32_t rot_ns_host(uint32_t x, int r, int Ns) {
    const uint32_t m = 0xffffffffu >> (32 - Ns);
    return ((x << r) | (x >> ((Ns - r) & 31))) & m;
}

uint32_t swap_pairs_host(uint32_t x, uint32_t m) {
    const uint32_t t = (x ^ (x >> 1)) & m;
    return x ^ t ^ (t << 1);
}

uint32_t image(const CandParams& c, uint32_t x, int Ns) { return rot_ns_host(swap_pairs_host(x, c.swap), c.rot, Ns); }

struct Res {
    uint32_t best;
    int count, e;
    bool valid;
};

// The rule of resolve_cand (ed_device.cuh) on the host.
Res resolve(const CandParams* c, int nc, uint32_t x, int Ns) {
    Res r{image(c[0], x, Ns), 1, c[0].e, true};
    for (int k = 1; k < nc; ++k) {
        const uint32_t im = image(c[k], x, Ns);
        if (im < r.best) {
            r = {im, 1, c[k].e, true};
        } else if (im == r.best) {
            ++r.count;
            if (c[k].e != r.e) r.valid = false;
        }
    }
    return r;
}

uint64_t colex_rank(uint32_t h, int N) {
    uint64_t C[33][33] = {};
    for (int n = 0; n <= 32; ++n) {
        C[0][n] = 1;
        for (int k = 1; k <= n; ++k) C[k][n] = C[k - 1][n - 1] + (k <= n - 1 ? C[k][n - 1] : 0);
    }
    uint64_t r = 0;
    int j = 0;
    for (int b = 0; b < N; ++b)
        if ((h >> b) & 1u) r += C[++j][b];
    return r;
}

}  // namespace

int main() {
    std::mt19937_64 rng(7);
    long cases = 0, checks = 0, bad = 0;
    for (int L = 4; L <= 8; ++L)
        for (int Nh = 1; Nh <= 4; ++Nh)
            for (int kx = 0; kx < L; ++kx)
                for (int ky = 0; ky < 2; ++ky) {
                    const int N = 2 * L, Ns = N - Nh;
                    const uint32_t mask = (1u << N) - 1u;
                    const HostSector S{L, N, Nh, Ns, kx, ky, (Ns % 2) == 0 ? 1 : 0, mask};
                    for (uint32_t h = 0; h <= mask; ++h) {
                        if (popc32(h) != Nh) continue;
                        uint32_t hc = h;
                        uint64_t low = colex_rank(h, N);
                        for (int p = 0; p < N; ++p) {
                            const uint32_t t = image_holes(S, h, p);
                            const uint64_t r = colex_rank(t, N);
                            if (r < low) {
                                low = r;
                                hc = t;
                            }
                        }
                        CandParams A[kMaxCand], B[kMaxCand];
                        const int na = coset(S, h, hc, A), nb = coset(S, hc, hc, B);
                        if (nb < 2 || nb > kMaxCand || na > kMaxCand) continue;
                        if (B[0].p != 0 || B[0].swap || B[0].rot) continue;
                        ++cases;
                        for (int Nd = 0; Nd <= Ns; Nd += (Ns > 6 ? 2 : 1))
                            for (int t = 0; t < 40; ++t) {
                                uint32_t dcm = 0;
                                for (int placed = 0; placed < Nd;) {
                                    const int b = (int)(rng() % (uint64_t)Ns);
                                    if (!((dcm >> b) & 1u)) {
                                        dcm |= 1u << b;
                                        ++placed;
                                    }
                                }
                                const Res ra = resolve(A, na, dcm, Ns);
                                const Res rb = resolve(B, nb, image(A[0], dcm, Ns), Ns);
                                const int e = (A[0].e + rb.e) % (2 * L);
                                ++checks;
                                const bool ok = ra.best == rb.best && ra.count == rb.count && ra.valid == rb.valid &&
                                                (!ra.valid || ra.e == e);
                                if (!ok && bad++ < 10)
                                    std::printf("L=%d Nh=%d k=(%d,%d) h=%x hc=%x dcm=%x: coset %x/%d/%d/%d, composed %x/%d/%d/%d\n",
                                                L, Nh, kx, ky, h, hc, dcm, ra.best, ra.count, ra.e, (int)ra.valid, rb.best,
                                                rb.count, e, (int)rb.valid);
                            }
                    }
                }
    std::printf("cases %ld checks %ld differences %ld\n", cases, checks, bad);
    return bad != 0 || cases == 0;
}
