// ed_basis.cu -- GPU enumeration of the symmetry-reduced basis.
//
// Replaces general/basis_indexing.h:188-242 calc_basis_map with its two loops
// (check_major_index_supports_lowest_states over hole ranks,
// symmetry_ladder.h:363-388; get_lowest_sparse_indices_from_major_index over
// spin ranks, general/symmetry.h:56-81) and the serial concatenation.
//
//   1. hole_classify_kernel: one thread per hole mask.  Eligibility probe of
//      the reference, the hole mask's canonical image (lowest mask over the
//      2L group elements), the product index and phase exponent of that image,
//      and whether the canonical mask has a trivial stabiliser ("free").
//   2. candidate_bitmap_kernel: one thread per 64 consecutive spin ranks of one
//      eligible hole mask (one bitmap word).  Colex-unranks the first spin
//      rank, walks the next 63 with Gosper's next-combination step, runs the
//      reference's lowest/compatibility test on each and sets the word's bits.
//   3. a deterministic exclusive scan of the word popcounts gives every word's
//      first dense row (the dense order is ascending sparse index, exactly the
//      reference's order).
//   4. fill_rows_kernel: writes the packed keys and orbit sizes of the set bits.
#include "ed_internal.cuh"

namespace ed {

__device__ __forceinline__ uint32_t unrank_colex(uint64_t r, int k, int n, const uint32_t* comb) {
    // k ones among n positions, colex rank r (symmetry_ladder.h:314-344 per part).
    uint32_t m = 0;
    for (int j = n - 1; j >= 0 && k > 0; --j) {
        const uint64_t c = comb[k * kCombStride + j];
        if (r >= c) {
            m |= 1u << j;
            r -= c;
            --k;
        }
    }
    return m;
}

// Deposit the compressed spin bits into the non-hole positions.
__device__ __forceinline__ uint32_t expand_spins(uint32_t dc, uint32_t h) {
    while (h) {
        const int p = __ffs(h) - 1;
        h &= h - 1u;
        const uint32_t low = (1u << p) - 1u;
        dc = (dc & low) | ((dc & ~low) << 1);
    }
    return dc;
}

__global__ void hole_classify_kernel(int L, int Nh, int kx, int ky, int ne_even, uint32_t mask, int64_t n_masks,
                                     const uint32_t* __restrict__ comb, uint8_t* __restrict__ elig,
                                     uint32_t* __restrict__ canon_rank, uint8_t* __restrict__ p_star,
                                     uint8_t* __restrict__ e_star, uint8_t* __restrict__ is_free,
                                     uint32_t* __restrict__ hmask_of_rank) {
    const int N = 2 * L, twoL = 2 * L;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_masks;
         r += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t h = unrank_colex((uint64_t)r, Nh, N, comb);
        hmask_of_rank[r] = h;
        // eligibility probe: symmetry_ladder.h:363-388
        uint8_t ok;
        if (Nh <= 1 || Nh >= N - 1) {
            ok = (r == 0);
        } else {
            const uint32_t free_sites = ~h & mask;
            const uint32_t d = free_sites & (0u - free_sites);  // first non-hole site flipped down
            ok = orbit_walk(L, kx, ky, ne_even, mask, h, d, true).found > 0;
        }
        elig[r] = ok;
        // canonical image of the hole mask and the phase exponent of the reaching image,
        // accumulated exactly like the orbit walk (translation phases are cumulative).
        const uint32_t single = (h ^ (h >> 1)) & 0x55555555u & mask;
        const uint32_t any_hole = (h | (h >> 1)) & 0x55555555u & mask;
        const int P = L - __popc(any_hole);
        const int e_mirror = (L * ky + L * (P & 1)) % twoL;
        uint32_t best = h;
        int best_p = 0, best_e = 0, nbest = 1, eT = 0;
        const uint32_t hm = mirror_legs(h);
        for (int p = 1; p < N; ++p) {
            const int s = p >> 1;
            uint32_t img;
            int e;
            if (p & 1) {
                img = rotl_n(hm, 2 * s, N, mask);
                e = (eT + e_mirror) % twoL;
            } else {
                img = rotl_n(h, 2 * s, N, mask);
                eT += 2 * kx;
                if (ne_even && ((single >> (2 * (L - s))) & 1u)) eT += L;
                eT %= twoL;
                e = eT;
            }
            if (img < best) {
                best = img;
                best_p = p;
                best_e = e;
                nbest = 1;
            } else if (img == best) {
                ++nbest;
            }
        }
        canon_rank[r] = hole_rank(best, comb);
        p_star[r] = (uint8_t)best_p;
        e_star[r] = (uint8_t)best_e;
        is_free[r] = (nbest == 1);
    }
}

__global__ void hole_entries_kernel(int64_t n_masks, const uint8_t* __restrict__ elig,
                                    const int64_t* __restrict__ elig_scan, const uint32_t* __restrict__ canon_rank,
                                    const uint8_t* __restrict__ p_star, const uint8_t* __restrict__ e_star,
                                    const uint8_t* __restrict__ is_free, const uint32_t* __restrict__ hmask_of_rank,
                                    int64_t spin_words, HoleEntry* __restrict__ holes, BlockInfo* __restrict__ blocks) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_masks;
         r += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = canon_rank[r];
        HoleEntry e;
        e.block = elig[c] ? (int32_t)elig_scan[c] : -1;
        e.p_star = p_star[r];
        e.e_star = e_star[r];
        e.free_ = is_free[r];
        e.pad_ = 0;
        holes[r] = e;
        if (elig[r]) {
            const int64_t b = elig_scan[r];
            BlockInfo bi;
            bi.hmask = hmask_of_rank[r];
            bi.flags = is_free[r] ? kBlockFree : 0u;
            bi.start = 0;
            bi.count = 0;
            bi.word_off = b * spin_words;
            blocks[b] = bi;
        }
    }
}

__global__ void candidate_bitmap_kernel(SectorView S, int64_t spin_words, uint64_t n_spin,
                                        uint64_t* __restrict__ bitmap) {
    extern __shared__ uint32_t s_comb[];
    for (int i = threadIdx.x; i < kCombStride * kCombStride; i += blockDim.x) s_comb[i] = S.comb[i];
    __syncthreads();
    const int64_t total = (int64_t)S.n_blocks * spin_words;
    for (int64_t gw = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gw < total;
         gw += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = gw / spin_words, w = gw - b * spin_words;
        const uint32_t h = S.blocks[b].hmask;
        const uint64_t r0 = (uint64_t)w * 64u;
        const int cnt = (n_spin - r0 < 64u) ? (int)(n_spin - r0) : 64;
        uint64_t x = unrank_colex(r0, S.Nd, S.Ns, s_comb);
        uint64_t word = 0;
        for (int k = 0; k < cnt; ++k) {
            const uint32_t d = expand_spins((uint32_t)x, h);
            if (orbit_walk(S.L, S.kx, S.ky, S.ne_even, S.mask, h, d, true).found > 0) word |= 1ull << k;
            if (x != 0) {  // Gosper's hack: next combination with the same popcount
                const uint64_t c = x & (0 - x), rr = x + c;
                x = (((rr ^ x) >> 2) / c) | rr;
            }
        }
        bitmap[gw] = word;
    }
}

// Block-level exclusive scan of popcount(bitmap) in three kernels; deterministic.
constexpr int kScanThreads = 256, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* sh, int64_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) sh[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int64_t s = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
        int64_t si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        if (lane < (int)(blockDim.x >> 5)) sh[lane] = si - s;
        if (lane == (int)(blockDim.x >> 5) - 1) sh[32] = si;
    }
    __syncthreads();
    const int64_t r = sh[wid] + incl - v;
    *total = sh[32];
    __syncthreads();
    return r;
}

__global__ void scan_tiles_kernel(const uint64_t* __restrict__ words, int64_t m, int64_t* __restrict__ tile_sums) {
    __shared__ int64_t sh[33];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < m) v += __popcll(words[base + k]);
    int64_t total;
    block_exclusive_scan(v, sh, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void scan_tile_sums_kernel(int64_t* __restrict__ tile_sums, int64_t ntiles, int64_t* __restrict__ grand) {
    __shared__ int64_t sh[33];
    int64_t carry = 0;
    for (int64_t base = 0; base < ntiles; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const int64_t v = (i < ntiles) ? tile_sums[i] : 0;
        int64_t total;
        const int64_t ex = block_exclusive_scan(v, sh, &total);
        if (i < ntiles) tile_sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void scan_apply_kernel(const uint64_t* __restrict__ words, int64_t m, const int64_t* __restrict__ tile_sums,
                                  int64_t* __restrict__ prefix) {
    __shared__ int64_t sh[33];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t c[kScanItems];
    int64_t v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        c[k] = (base + k < m) ? __popcll(words[base + k]) : 0;
        v += c[k];
    }
    int64_t total;
    int64_t ex = block_exclusive_scan(v, sh, &total) + tile_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < m) prefix[base + k] = ex;
        ex += c[k];
    }
}

__global__ void block_ranges_kernel(int n_blocks, int64_t spin_words, const uint64_t* __restrict__ bitmap,
                                    const int64_t* __restrict__ prefix, int64_t n_total, uint64_t n_spin,
                                    BlockInfo* __restrict__ blocks, int* __restrict__ err) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n_blocks; b += gridDim.x * blockDim.x) {
        const int64_t w0 = (int64_t)b * spin_words;
        const int64_t start = prefix[w0];
        const int64_t end = (b + 1 < n_blocks) ? prefix[w0 + spin_words] : n_total;
        blocks[b].start = start;
        blocks[b].count = end - start;
        // a free canonical mask admits every spin configuration as a representative
        if ((blocks[b].flags & kBlockFree) && (uint64_t)(end - start) != n_spin) atomicExch(err, 1);
    }
}

__global__ void fill_rows_kernel(SectorView S, int64_t spin_words, uint64_t n_spin, const int64_t* __restrict__ prefix,
                                 uint64_t* __restrict__ keys, uint8_t* __restrict__ orbit) {
    extern __shared__ uint32_t s_comb[];
    for (int i = threadIdx.x; i < kCombStride * kCombStride; i += blockDim.x) s_comb[i] = S.comb[i];
    __syncthreads();
    const int64_t total = (int64_t)S.n_blocks * spin_words;
    for (int64_t gw = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gw < total;
         gw += (int64_t)gridDim.x * blockDim.x) {
        uint64_t word = S.bitmap[gw];
        if (!word) continue;
        const int64_t b = gw / spin_words, w = gw - b * spin_words;
        const uint32_t h = S.blocks[b].hmask;
        const bool is_free = S.blocks[b].flags & kBlockFree;
        uint64_t x = unrank_colex((uint64_t)w * 64u, S.Nd, S.Ns, s_comb);
        int64_t pos = prefix[gw];
        for (int k = 0; k < 64 && word; ++k) {
            if (word & 1ull) {
                const uint32_t d = expand_spins((uint32_t)x, h);
                const int nf = is_free ? S.N : orbit_walk(S.L, S.kx, S.ky, S.ne_even, S.mask, h, d, true).found;
                keys[pos] = ((uint64_t)h << 32) | d;
                orbit[pos] = (uint8_t)nf;
                ++pos;
            }
            word >>= 1;
            if (x != 0) {
                const uint64_t c = x & (0 - x), rr = x + c;
                x = (((rr ^ x) >> 2) / c) | rr;
            }
        }
    }
}

__global__ void interleave_bitmap_kernel(int64_t words, const uint64_t* __restrict__ bitmap,
                                         const int64_t* __restrict__ prefix, ulonglong2* __restrict__ out) {
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x)
        out[w] = make_ulonglong2(bitmap[w], (unsigned long long)prefix[w]);
}

__global__ void export_sparse_kernel(SectorView S, uint64_t n_spin, int64_t* __restrict__ sparse,
                                     int32_t* __restrict__ orbit_out) {
    extern __shared__ uint32_t s_tab[];
    uint32_t* s_comb = s_tab;
    uint32_t* s_rank = s_tab + kCombStride * kCombStride;
    const int tab_words = S.rank_words;
    for (int i = threadIdx.x; i < kCombStride * kCombStride; i += blockDim.x) s_comb[i] = S.comb[i];
    for (int i = threadIdx.x; i < tab_words; i += blockDim.x) s_rank[i] = S.rank_tab[i];
    __syncthreads();
    const RankTab rt = rank_tab_of(S, s_rank);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = S.keys[i];
        const uint32_t h = (uint32_t)(key >> 32), d = (uint32_t)key;
        sparse[i] = (int64_t)hole_rank(h, s_comb) * (int64_t)n_spin + spin_rank(compress_spins(d, h), rt, S.Nd);
        orbit_out[i] = S.orbit[i];
    }
}

// ------------------------------------------------------------------ host side

int basis_build(Sector& s, cudaStream_t st) {
    SectorView& V = s.view;
    const int N = V.N;
    const int64_t n_masks = s.n_hole_masks;
    // hole masks: classification and canonical map
    DevBuf<uint8_t> elig(n_masks), pstar(n_masks), estar(n_masks), isfree(n_masks);
    DevBuf<uint32_t> canon(n_masks), hmr(n_masks);
    DevBuf<int64_t> elig_scan(n_masks + 1);
    if (!elig.ok() || !pstar.ok() || !estar.ok() || !isfree.ok() || !canon.ok() || !hmr.ok() || !elig_scan.ok())
        return set_error(ED_ERR_NOMEM, "basis: allocating hole-mask tables");
    const int grid = grid_for(n_masks, 256, s.num_sms);
    hole_classify_kernel<<<grid, 256, 0, st>>>(V.L, V.Nh, V.kx, V.ky, V.ne_even, V.mask, n_masks, s.d_comb.p, elig.p,
                                               canon.p, pstar.p, estar.p, isfree.p, hmr.p);
    ED_CHECK_LAUNCH("hole_classify_kernel");
    // eligible masks -> block ids: reuse the word scan on a byte->bit packing is overkill; masks are few
    // (C(N,Nh) <= 2^24 when a table exists), so scan them with the same tile scan over packed words.
    const int64_t n_mwords = (n_masks + 63) / 64;
    DevBuf<uint64_t> ebits(n_mwords);
    DevBuf<int64_t> eword_prefix(n_mwords + 1);
    if (!ebits.ok() || !eword_prefix.ok()) return set_error(ED_ERR_NOMEM, "basis: allocating scan buffers");
    pack_flags(elig.p, n_masks, ebits.p, st, s.num_sms);
    int64_t n_blocks = 0;
    if (int rc = scan_popcounts(ebits.p, n_mwords, eword_prefix.p, &n_blocks, st)) return rc;
    expand_flag_scan(elig.p, n_masks, ebits.p, eword_prefix.p, elig_scan.p, st, s.num_sms);
    if (n_blocks <= 0) {
        // empty sector: no representative
        V.n = 0;
        V.n_blocks = 0;
        s.built = true;
        return ED_OK;
    }
    if (n_blocks > INT32_MAX) return set_error(ED_ERR_TOO_LARGE, "basis: too many hole blocks");
    s.d_blocks.alloc(n_blocks);
    s.d_holes.alloc(n_masks);
    if (!s.d_blocks.ok() || !s.d_holes.ok()) return set_error(ED_ERR_NOMEM, "basis: allocating block tables");
    const uint64_t n_spin = s.n_spin;
    const int64_t spin_words = (int64_t)((n_spin + 63) / 64);
    hole_entries_kernel<<<grid, 256, 0, st>>>(n_masks, elig.p, elig_scan.p, canon.p, pstar.p, estar.p, isfree.p,
                                              hmr.p, spin_words, s.d_holes.p, s.d_blocks.p);
    ED_CHECK_LAUNCH("hole_entries_kernel");
    V.n_blocks = (int)n_blocks;
    V.blocks = s.d_blocks.p;
    V.holes = s.d_holes.p;
    V.n_hole_masks = n_masks;
    // candidate bitmaps of every eligible hole mask
    const int64_t total_words = n_blocks * spin_words;
    if (total_words / spin_words != n_blocks) return set_error(ED_ERR_TOO_LARGE, "basis: bitmap size overflow");
    s.d_bitmap.alloc(total_words);
    s.d_prefix.alloc(total_words + 1);
    if (!s.d_bitmap.ok() || !s.d_prefix.ok()) return set_error(ED_ERR_NOMEM, "basis: allocating candidate bitmaps");
    V.bitmap = s.d_bitmap.p;
    V.word_prefix = s.d_prefix.p;
    const size_t comb_smem = kCombStride * kCombStride * sizeof(uint32_t);
    candidate_bitmap_kernel<<<grid_for(total_words, 256, s.num_sms), 256, comb_smem, st>>>(V, spin_words, n_spin,
                                                                                            s.d_bitmap.p);
    ED_CHECK_LAUNCH("candidate_bitmap_kernel");
    int64_t n_total = 0;
    if (int rc = scan_popcounts(s.d_bitmap.p, total_words, s.d_prefix.p, &n_total, st)) return rc;
    DevBuf<int> err(1);
    cudaMemsetAsync(err.p, 0, sizeof(int), st);
    block_ranges_kernel<<<grid_for(n_blocks, 128, s.num_sms), 128, 0, st>>>((int)n_blocks, spin_words, s.d_bitmap.p,
                                                                            s.d_prefix.p, n_total, n_spin,
                                                                            s.d_blocks.p, err.p);
    ED_CHECK_LAUNCH("block_ranges_kernel");
    int herr = 0;
    cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return set_error(ED_ERR_CUDA, "basis: block ranges");
    if (herr) return set_error(ED_ERR_INTERNAL, "basis: a trivially-stabilised hole block is not full");
    V.n = n_total;
    s.d_keys.alloc(n_total > 0 ? n_total : 1);
    s.d_orbit.alloc(n_total > 0 ? n_total : 1);
    if (!s.d_keys.ok() || !s.d_orbit.ok()) return set_error(ED_ERR_NOMEM, "basis: allocating the representative table");
    V.keys = s.d_keys.p;
    V.orbit = s.d_orbit.p;
    fill_rows_kernel<<<grid_for(total_words, 256, s.num_sms), 256, comb_smem, st>>>(V, spin_words, n_spin,
                                                                                     s.d_prefix.p, s.d_keys.p,
                                                                                     s.d_orbit.p);
    ED_CHECK_LAUNCH("fill_rows_kernel");
    if (!s.d_bitpref.alloc(total_words)) return set_error(ED_ERR_NOMEM, "basis: allocating the bitmap index");
    interleave_bitmap_kernel<<<grid_for(total_words, 256, s.num_sms), 256, 0, st>>>(total_words, s.d_bitmap.p,
                                                                                     s.d_prefix.p, s.d_bitpref.p);
    ED_CHECK_LAUNCH("interleave_bitmap_kernel");
    if (cudaStreamSynchronize(st) != cudaSuccess) return set_error(ED_ERR_CUDA, "basis: fill rows");
    V.bitpref = s.d_bitpref.p;
    s.d_bitmap.reset();
    s.d_prefix.reset();
    V.bitmap = nullptr;
    V.word_prefix = nullptr;
    (void)N;
    s.built = true;
    return ED_OK;
}

int basis_export(Sector& s, int64_t* sparse_dev, int32_t* orbit_dev, cudaStream_t st) {
    const SectorView& V = s.view;
    if (V.n == 0) return ED_OK;
    const size_t smem = (kCombStride * kCombStride + V.rank_words) * sizeof(uint32_t);
    export_sparse_kernel<<<grid_for(V.n, 256, s.num_sms), 256, smem, st>>>(V, s.n_spin, sparse_dev, orbit_dev);
    ED_CHECK_LAUNCH("export_sparse_kernel");
    return ED_OK;
}

// ---- small scan helpers (also used by the hole-mask stage) ----

__global__ void pack_flags_kernel(const uint8_t* __restrict__ f, int64_t n, uint64_t* __restrict__ words) {
    const int64_t nw = (n + 63) / 64;
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
        uint64_t v = 0;
        for (int k = 0; k < 64; ++k) {
            const int64_t i = w * 64 + k;
            if (i < n && f[i]) v |= 1ull << k;
        }
        words[w] = v;
    }
}

__global__ void expand_flag_scan_kernel(const uint8_t* __restrict__ f, int64_t n, const uint64_t* __restrict__ words,
                                        const int64_t* __restrict__ wprefix, int64_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t w = i >> 6;
        const uint64_t below = words[w] & ((1ull << (i & 63)) - 1ull);
        out[i] = wprefix[w] + __popcll(below);
    }
}

void pack_flags(const uint8_t* f, int64_t n, uint64_t* words, cudaStream_t st, int sms) {
    pack_flags_kernel<<<grid_for((n + 63) / 64, 256, sms), 256, 0, st>>>(f, n, words);
}

void expand_flag_scan(const uint8_t* f, int64_t n, const uint64_t* words, const int64_t* wprefix, int64_t* out,
                      cudaStream_t st, int sms) {
    expand_flag_scan_kernel<<<grid_for(n, 256, sms), 256, 0, st>>>(f, n, words, wprefix, out);
}

int scan_popcounts(const uint64_t* words, int64_t m, int64_t* prefix, int64_t* total_host, cudaStream_t st) {
    const int64_t ntiles = (m + kScanTile - 1) / kScanTile;
    DevBuf<int64_t> tiles(ntiles > 0 ? ntiles : 1), grand(1);
    if (!tiles.ok() || !grand.ok()) return set_error(ED_ERR_NOMEM, "scan: allocating tile sums");
    if (ntiles > 0) {
        scan_tiles_kernel<<<(unsigned)ntiles, kScanThreads, 0, st>>>(words, m, tiles.p);
        ED_CHECK_LAUNCH("scan_tiles_kernel");
    }
    scan_tile_sums_kernel<<<1, 1024, 0, st>>>(tiles.p, ntiles, grand.p);
    ED_CHECK_LAUNCH("scan_tile_sums_kernel");
    if (ntiles > 0) {
        scan_apply_kernel<<<(unsigned)ntiles, kScanThreads, 0, st>>>(words, m, tiles.p, prefix);
        ED_CHECK_LAUNCH("scan_apply_kernel");
    }
    cudaMemcpyAsync(prefix + m, grand.p, sizeof(int64_t), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(total_host, grand.p, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return set_error(ED_ERR_CUDA, "scan: synchronize");
    return ED_OK;
}

}  // namespace ed
