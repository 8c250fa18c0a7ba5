// ed_common.cuh -- bit-level state model of the spin-1/2 t-J two-leg ladder
// shared by the basis, H.v, Lanczos and excitation kernels.
//
// A configuration of N = 2L sites (site i = 2x + y, rung x, leg y) is two
// N-bit masks: h (holes) and d (down spins); every other site is an up spin.
// The packed key (h << 32) | d orders configurations exactly like the
// reference's sparse index (hole rank * C(Ns,Nd) + spin rank,
// tJ_spin_half_ladder/symmetry_ladder.h:346-361): colex rank is monotone in the
// mask value, holes are compared first, and for equal hole masks the raw down
// mask orders like its compressed form.  State_Hierarchy::check_lower_state
// (general/group/commutation_counter.h:45-69) therefore becomes a 64-bit compare.
//
// Symmetry group (2L elements, product index p = 1..N-1 in the reference's
// order, general/cpp_classes.h:14-105): translation by s = p/2 rungs is a
// rotation of both masks by 2s bits; odd p first swaps the two legs (even and
// odd bits).  Amplitudes are powers of u = exp(-i*pi/L); an amplitude is held
// as its exponent e mod 2L, which makes the reference's |amp - 1| > 1e-8 tests
// (symmetry_ladder.h:196-224) exact integer tests.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace ed {

constexpr int kMaxN = 32;
constexpr int kCombStride = 33;

enum : uint32_t { kBlockFree = 1u };

// One eligible (canonical) hole mask: a contiguous range of dense rows.
struct BlockInfo {
    uint32_t hmask;     // canonical hole mask of the block
    uint32_t flags;     // kBlockFree: trivial stabiliser -> every spin rank is a representative
    int64_t start;      // first dense row of the block
    int64_t count;      // rows in the block
    int64_t word_off;   // first word of the block's candidate bitmap (non-free blocks), else -1
};

// One hole mask (any, indexed by its colex rank): how it maps to its canonical block.
struct HoleEntry {
    int32_t block;      // block of the canonical mask, -1 if the canonical mask has no block
    uint8_t p_star;     // product index whose image carries the canonical mask (free masks)
    uint8_t e_star;     // phase exponent of that image (free masks)
    uint8_t free_;      // 1 if the canonical mask has a trivial stabiliser
    uint8_t pad_;
};

// ---- per-block descriptors of the fast H.v row (built once per sector) ----------------------
//
// Spin configurations are handled as compressed down masks: the down spins of the non-hole
// sites, packed in increasing site order (bit c = c-th electron).  A group element maps the
// compressed mask of a state with hole mask h to the compressed mask of its image by swapping
// the two spins of every doubly occupied rung (mirror, odd product index) and rotating the
// Ns-bit string left by the number of electrons that wrap around (translation).

constexpr int kMaxCand = 4;    // stabiliser-coset candidates resolved without the orbit walk
constexpr int kMaxHops = 12;   // 3 hops per hole, up to 4 holes

enum : uint8_t { kModeFree = 0, kModeCand = 1, kModeGeneric = 2, kModeAbsent = 3 };

struct CandParams {
    uint32_t swap;  // compressed positions c whose spins (c, c+1) the mirror exchanges
    uint8_t rot;    // left rotation of the Ns-bit compressed mask
    uint8_t e;      // phase exponent of this group element for the transformed hole mask
    uint8_t p;      // product index
    uint8_t pad;
};

// A hop of the fast row.  The first 32 bytes are what the row kernel reads for every row (as two
// 16-byte words in hv_row_fast); keep their order.
struct alignas(16) HopDesc {
    uint32_t band;   // compressed bits that shift by one position
    uint32_t swap;   // cand[0].swap
    uint8_t p, q;    // electron's compressed position before (row mask) and after (new mask) the hop
    uint8_t rot, e;  // cand[0].rot, cand[0].e
    uint8_t term;    // 0 tl (leg), 1 tr (rung)
    uint8_t mode;    // kModeFree / kModeCand / kModeGeneric / kModeAbsent
    uint8_t ncand;
    int8_t sign;     // fermion sign (electrons strictly between a and b)
    int64_t start, word_off;  // target block rows and bitmap
    // read by the candidate and generic modes only
    uint8_t a, b;    // electron site, hole site
    uint8_t pad[2];
    int32_t block;   // target block
    CandParams cand[kMaxCand];
};

// Descriptor of one block.  The first 32 bytes are read per row as two 16-byte words; keep
// their order.
struct alignas(16) BlockDesc {
    uint32_t hmask;
    uint32_t m_rung;     // rung bonds, at the lower compressed position (partner one above)
    uint32_t m_legadj;   // leg bonds whose middle site is a hole (partner one above)
    uint32_t m_legd2;    // leg bonds whose middle site is occupied (partner two above)
    uint8_t mode;        // kModeFree / kModeCand / kModeGeneric
    uint8_t nhop;
    uint8_t ncand;
    uint8_t nwrap;
    uint8_t wrap[2][2];  // leg bonds across the periodic boundary: compressed positions (lo, hi)
    int64_t start;
    int64_t word_off;
    uint8_t pad[8];
    CandParams cand[kMaxCand];  // stabiliser of hmask (exchange targets in kModeCand blocks)
    HopDesc hop[kMaxHops];
};

static_assert(offsetof(HopDesc, start) == 16 && offsetof(HopDesc, a) == 32, "HopDesc hot words");
static_assert(offsetof(BlockDesc, mode) == 16 && offsetof(BlockDesc, start) == 24, "BlockDesc hot words");

// ---- segment layout of free blocks (ed_seg.cuh) ------------------------------------------------
//
// The compressed down mask dc of a free block's row splits at position P = min(kSegA, Ns) into a
// low part (bits [0, P)) and a high part H (bits [P, Ns)); the rows sharing H are contiguous (a
// segment).  SegDesc lists a free block's terms by where their bits lie relative to P.

constexpr int kSegA = 10;     // low compressed bits resolved per lane: C(10, k) <= 252 rows per segment
constexpr int kSegMaxA = 16;  // exchange bonds with both ends below P
constexpr int kSegMaxB = 48;  // exchange bonds with both ends at or above P
constexpr int kSegMaxX = 8;   // exchange bonds across P

// A hop as a permutation pi of compressed masks (move of the electron, then the target's coset
// permutation: mirror pairs and rotation), classified by how it maps [0, P): nb of the P low
// positions land at or above P (at bpos[0] < bpos[1]), and as many high positions land below P;
// nb = 3 stands for "more than two" (the target rank is then taken per row).
struct SegHopDesc {
    uint32_t keep, band, swap;     // bits kept in place, bits shifted by one toward p, mirror pairs
    uint8_t sl, sr, p, q;          // moved = ((x & band) << sl) >> sr; the electron goes from p to q
    uint8_t rot, nsr, term, sign;  // left rotation by rot (nsr = (Ns - rot) % 32); 0 tl / 1 tr; 1: coefficient -w
    uint8_t e, kind, nb, pad;      // phase exponent; 0 free target, 1 stabiliser target, 3 absent
    uint8_t bpos[2], pad2[2];
    int32_t tblock;                // target block
    int64_t tstart;                // free target: its first row; stabiliser target: the index of its
                                   // expanded copy among the sector's copies
};

// Per segment of a free block, a record of rec_len 32-bit words (built once per sector by
// seg_records_kernel; the values depend on the segment's high part only, never on a vector):
//   [0] the segment's first row in the block;  [1] zb | zbr << 8 | hib << 16 (antiparallel high
//   bonds, the rung bonds among them, the spins at the high ends of the cross bonds); [2, 4) zero;
//   [4, 4 + zb) the first rows of the partner segments of its antiparallel high bonds, rung bonds
//   first, then the segment's own first row up to a multiple of four (HB words are reserved; the
//   list starts on a 16-byte boundary and is read four words at a time);
//   [xo, xo + nX) cross bond c: first row of the partner segment; hop h from word hop_off[h]: the
//   first n0 hops (nb = 0, and absent hops) the target's high-part rank; the next n12 (nb 1 or 2) ua,
//   then the 2^nb high-part ranks by vbi; the rest (nb = 3) pi(H << P); then two zero words
//   (zero_w), which the kernel's padding hops read.
struct alignas(16) SegDesc {
    int64_t start;              // the block's first row
    int64_t rec;                // first word of the block's segment records
    uint32_t fA[kSegMaxA];      // bonds below P as two-bit flip masks, rung bonds first
    uint8_t bB[kSegMaxB][2];    // bonds at or above P (a < b): rung, then leg at distance one, then two
    uint8_t cX[kSegMaxX][2];    // bonds across P: (end below P, end at or above P), rung bonds first
    uint32_t mr, ma, m2;        // lower ends of the rung / leg-1 / leg-2 bonds at or above P
    uint8_t nA, nAr, nB, nBr, nBa, nX, nXr, nhop;
    uint8_t ok, HB, xo, pad1;   // ok: every term fits the limits; record layout (above)
    uint32_t rec_len;           // words per segment record, a multiple of 4
    uint8_t hop_off[kMaxHops];  // first word of hop h in a record
    uint8_t n0, n12, zero_w, pad2;  // hops by kind (record layout above); two zero words from zero_w
    SegHopDesc hop[kMaxHops];
};
static_assert(sizeof(SegDesc) % 16 == 0, "SegDesc is staged as 16-byte words");

// Read-only view of a built sector, passed to kernels by value.
struct SectorView {
    int L, N, Nh, Nd, Ns;
    int kx;                 // leg momentum mod L
    int ky;                 // rung parity
    int ne_even;            // number of electrons even
    uint32_t mask;          // low N bits
    int64_t n;              // number of representatives
    int64_t n_hole_masks;   // C(N, Nh) (size of `holes`, 0 when no table)
    int n_blocks;
    const BlockInfo* blocks;
    const HoleEntry* holes;        // may be null: generic mode (block found by binary search)
    const uint64_t* keys;          // [n] packed representative keys, ascending
    const uint8_t* orbit;          // [n] orbit size (num_sparse_states_in_dense)
    const uint64_t* bitmap;        // candidate bitmaps of every block (basis construction only)
    const int64_t* word_prefix;    // dense row of the first set bit of each bitmap word (construction only)
    const ulonglong2* bitpref;     // {bitmap word, its prefix} side by side: one 16-byte load per lookup
    const uint32_t* rank_tab;      // tables of the colex spin rank (layout: see RankTab)
    uint32_t rk_off[4];            // first word of chunk c's table
    uint32_t rk_pos[4];            // first compressed bit of chunk c (c >= 1)
    uint32_t rk_m0;                // bits of chunk 0
    uint32_t rk_nch;               // number of chunks, 3 or 4
    int rank_words;                // words of rank_tab
    const uint32_t* comb;          // [33][33] comb[k*33+n] = C(n,k)
    const BlockDesc* desc;         // [n_blocks] fast-row descriptors (null: the orbit-walk row only)
    // segment layout of free blocks (ed_seg.cuh)
    int seg_p;                     // P = min(kSegA, Ns)
    uint32_t seg_off[kSegA + 2];   // first segment of class kl (kl low down spins), kl = 0 .. P + 1
    const uint32_t* seg_h;         // per segment: its high part H (bits [P, Ns) of dc, shifted down by P)
    const uint32_t* seg_base;      // per segment: its first row in a block, rank((H << P) | (2^kl - 1))
    const SegDesc* seg;            // [n_blocks] segment descriptors (free blocks)
    const uint32_t* seg_rec;       // segment records of every free block (SegDesc::rec, rec_len)
};

// ---------------------------------------------------------------- bit helpers

__host__ __device__ __forceinline__ uint32_t rotl_n(uint32_t x, int r, int N, uint32_t mask) {
    uint64_t xx = x;
    return (uint32_t)(((xx << r) | (xx >> (N - r))) & mask);
}

__host__ __device__ __forceinline__ uint32_t mirror_legs(uint32_t x) {
    return ((x & 0x55555555u) << 1) | ((x >> 1) & 0x55555555u);
}

// Image of (h, d) under product index p (0 = identity).
__host__ __device__ __forceinline__ void apply_p(int p, uint32_t& h, uint32_t& d, int N, uint32_t mask) {
    if (p & 1) {
        h = mirror_legs(h);
        d = mirror_legs(d);
    }
    const int r = 2 * (p >> 1);
    h = rotl_n(h, r, N, mask);
    d = rotl_n(d, r, N, mask);
}

__host__ __device__ __forceinline__ int ctz32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __ffs(x) - 1;
#else
    return __builtin_ctz(x);
#endif
}
__host__ __device__ __forceinline__ int popc32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}
__host__ __device__ __forceinline__ int hibit32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return 31 - __clz(x);
#else
    return 31 - __builtin_clz(x);
#endif
}

// Remove the bits at hole positions (parallel bit extract over ~h).
__host__ __device__ __forceinline__ uint32_t compress_spins(uint32_t d, uint32_t h) {
    while (h) {
        const int p = hibit32(h);
        h &= ~(1u << p);
        const uint32_t low = (1u << p) - 1u;
        d = (d & low) | ((d >> 1) & ~low);
    }
    return d;
}

// Colex rank of a compressed down mask from tables, three lookups for Ns <= 28.  Chunk 0 covers
// compressed bits [0, w0) (m0 = 2^w0 - 1), which have no set bits below them: T[dc & m0] is the
// sum over its set bits (j-th from the bottom, at position b) of C(b, j).  Chunks c = 1 .. nch-1
// cover the eight bits from pos[c]; with k set bits below the chunk, T[off[c] + (k << 8) + byte]
// is the sum over the byte's set bits of C(pos[c] + b, k + j).  nch = 3 and w0 = max(0, Ns - 16)
// for Ns <= 28, else nch = 4 and w0 = Ns - 24.  The mask must hold exactly Nd set bits (every
// configuration of the sector does), so k stays within the Nd + 1 rows of each chunk.
struct RankTab {
    const uint32_t* T;
    uint32_t m0;
    uint32_t nch;
    uint32_t off[4];
    uint32_t pos[4];
};

__host__ __device__ __forceinline__ uint32_t spin_rank(uint32_t dc, const RankTab& R, int Nd) {
    (void)Nd;
    uint32_t r = R.T[dc & R.m0];
    uint32_t k = (uint32_t)popc32(dc & R.m0);
#pragma unroll
    for (int c = 1; c < 4; ++c) {
        if (c == 3 && R.nch < 4) break;
        const uint32_t byte = (dc >> R.pos[c]) & 255u;
        r += R.T[R.off[c] + (k << 8) + byte];
        k += (uint32_t)popc32(byte);
    }
    return r;
}

// The Nd-bit mask of colex rank r among Ns bits (comb[k * kCombStride + n] = C(n, k)): the j-th set
// bit from the top is the largest p with C(p, k) <= what remains of r, k counting down from Nd.
__host__ __device__ __forceinline__ uint32_t colex_unrank(int64_t r, int Ns, int Nd, const uint32_t* comb) {
    uint32_t m = 0;
    int p = Ns - 1;
    for (int k = Nd; k >= 1; --k) {
        while ((int64_t)comb[k * kCombStride + p] > r) --p;
        m |= 1u << p;
        r -= comb[k * kCombStride + p];
        --p;
    }
    return m;
}

// The next mask with the same number of set bits (next colex rank); v must be non-zero and not the
// last such mask below 2^32.
__host__ __device__ __forceinline__ uint32_t next_combination(uint32_t v) {
    const uint32_t t = v | (v - 1u);
    return (t + 1u) | (((~t & (0u - ~t)) - 1u) >> (ctz32(v) + 1));
}

// RankTab over a copy T of the sector's rank tables.
__host__ __device__ __forceinline__ RankTab rank_tab_of(const SectorView& S, const uint32_t* T) {
    RankTab rt;
    rt.T = T;
    rt.m0 = S.rk_m0;
    rt.nch = S.rk_nch;
    for (int c = 0; c < 4; ++c) {
        rt.off[c] = S.rk_off[c];
        rt.pos[c] = S.rk_pos[c];
    }
    return rt;
}

// Colex rank of a hole mask (general/symmetry_ladder.h:346-361, hole part).
__host__ __device__ __forceinline__ uint32_t hole_rank(uint32_t h, const uint32_t* comb) {
    uint32_t r = 0;
    int j = 0;
    while (h) {
        const int p = ctz32(h);
        h &= h - 1u;
        ++j;
        r += comb[j * kCombStride + p];
    }
    return r;
}

// --------------------------------------------------------------- orbit walk

struct OrbitResult {
    int found;      // orbit size as the reference counts it, 0 = not lowest / incompatible
    uint64_t low;   // lowest image (first strictly-lowest in the reference's list order)
    int e;          // phase exponent of the lowest image, mod 2L
    int p;          // product index of the lowest image (0 = the state itself)
};

// Restatement of Symmetries_Single_Spin_Half_2leg_Ladder::get_symmetry_states_from_state
// (tJ_spin_half_ladder/symmetry_ladder.h:113-235) on packed keys, followed by
// the lowest-image pick of get_lowest_sparse_amplitude_from_state
// (general/symmetry.h:97-126).  Same iteration order, same early exits, same
// orbit-closure rule (only while s < L/2 + 1).
__host__ __device__ __forceinline__ OrbitResult orbit_walk(int L, int kx, int ky, int ne_even, uint32_t mask, uint32_t h,
                                                           uint32_t d, bool check_lowest) {
    const int N = 2 * L, twoL = 2 * L;
    const uint64_t key = ((uint64_t)h << 32) | d;
    const uint32_t any_hole = (h | (h >> 1)) & 0x55555555u & mask;
    const uint32_t single = (h ^ (h >> 1)) & 0x55555555u & mask;
    const int P = L - popc32(any_hole);
    const int e_mirror = (L * ky + L * (P & 1)) % twoL;
    const uint32_t hm = mirror_legs(h), dm = mirror_legs(d);
    int eT = 0, found = 1, e1 = 0, elow = 0, plow = 0;
    bool msym = false;
    uint64_t img1 = 0, low = key;
    for (int p = 1; p < N; ++p) {
        const int s = p >> 1;
        uint64_t img;
        int e;
        if (p & 1) {
            if (msym) continue;
            img = ((uint64_t)rotl_n(hm, 2 * s, N, mask) << 32) | rotl_n(dm, 2 * s, N, mask);
            e = eT + e_mirror;
            if (e >= twoL) e -= twoL;
        } else {
            img = ((uint64_t)rotl_n(h, 2 * s, N, mask) << 32) | rotl_n(d, 2 * s, N, mask);
            eT += 2 * kx;
            if (ne_even && ((single >> (2 * (L - s))) & 1u)) eT += L;
            eT %= twoL;
            e = eT;
        }
        if (check_lowest && img < key) return {0, 0, 0, 0};
        if (s < L / 2 + 1) {
            if (img == key) {
                if (e != 0) return {0, 0, 0, 0};
                if (p == 1) {
                    msym = true;
                    continue;
                }
                break;
            }
            if (found != 1 && img == img1) {
                if (e != e1) return {0, 0, 0, 0};
                break;
            }
        }
        if (found == 1) {
            img1 = img;
            e1 = e;
        }
        ++found;
        if (img < low) {
            low = img;
            elow = e;
            plow = p;
        }
    }
    return {found, low, elow, plow};
}

}  // namespace ed
