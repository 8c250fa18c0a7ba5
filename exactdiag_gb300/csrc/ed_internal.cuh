// ed_internal.cuh -- host-side sector object, device buffers and error plumbing
// shared by the translation units of libexactdiag_gb300.so.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/exactdiag_gb300.h"
#include "ed_common.cuh"

namespace ed {

// Thread-local error text behind ed_last_error_string().
int set_error(int code, const char* what);
int set_cuda_error(cudaError_t e, const char* what);

#define ED_CHECK_LAUNCH(name)                                           \
    do {                                                                \
        cudaError_t e_ = cudaGetLastError();                            \
        if (e_ != cudaSuccess) return ::ed::set_cuda_error(e_, name);   \
    } while (0)

// Owning device buffer; frees on destruction.  Allocation failure leaves p null.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    int64_t n = 0;
    DevBuf() = default;
    explicit DevBuf(int64_t count) { alloc(count); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { reset(); }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    bool alloc(int64_t count) {
        reset();
        if (count <= 0) count = 1;
        // 64-bit size check before cudaMalloc
        if ((uint64_t)count > UINT64_MAX / sizeof(T)) return false;
        if (cudaMalloc((void**)&p, (size_t)count * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return false;
        }
        n = count;
        return true;
    }
    bool ok() const { return p != nullptr; }
};

inline int grid_for(int64_t work, int threads, int sms, int per_sm = 8) {
    int64_t g = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)sms * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

constexpr int kHvThreads = 256;
constexpr int kReduceSlots = 4;  // FP64 partial sums per chunk in the fused Lanczos step
// Rows per chunk (at most; plan_chunks halves it for row kinds with few rows): small enough that the
// CTAs running at one time cover a narrow window of rows (the gathered x_j of neighbouring rows
// stay in L2), large enough to amortise the per-chunk reduction and descriptor staging.
constexpr int kChunkRows = 8192;
// The segment kernel of free blocks (ed_seg.cuh): threads per CTA, and about how many rows one H.v
// chunk of it holds.
constexpr int kSegThreads = 256;
constexpr int kSegChunkRows = 16384;
constexpr int kSegWin = 32;  // default offsets of a segment a segment chunk covers (Sector::seg_win: 32 or 64)

// Row kinds of the fused step: each kind has its own kernel (and register budget).
enum RowKind : int {
    kRowsFree64 = 0,   // blocks with a trivial stabiliser, planned with 64-offset windows (Sector::seg_win)
    kRowsFree = 1,     // blocks with a trivial stabiliser: colex deltas, no orbit lookups
    kRowsCand = 2,     // blocks with a small stabiliser: coset candidates and bitmap lookups
    kRowsGeneric = 3,  // everything else (and sectors without descriptors): the orbit walk
};

// Rows [start, start + count) of one block (block = descriptor index, -1 without descriptors).
struct BlockSpan {
    int64_t start, count;
    int32_t block;
    int32_t kind;
};

struct BatchChunk {
    int32_t sec;
    int32_t block;       // descriptor of the chunk's block (every row of a chunk is in one block), or -1
    int64_t begin, end;  // rows of sector `sec`; segment chunks: segments [begin, end) of class kl
    int64_t xoff;        // stabiliser blocks: first element of the block's expanded copy (ExpandTask);
                         // segment chunks: first element of the sector's copies; else -1
    int32_t kl;          // segment chunks (free blocks, ed_seg.cuh): down spins below P; row chunks: -1
    int32_t piece;       // segment chunks: the window of offsets [kSegWin piece, kSegWin piece + kSegWin)
};

// One stabiliser block of a step layout whose vector entries are expanded, every step, to all
// C(Ns, Nd) spin configurations of its hole mask: out[r] for the configuration of colex rank r is
// conj(u^e) x[rep] / sqrt(orbit) (0 for a configuration the sector's phases exclude), so that its
// rows' exchange targets are read like a free block's (row rank +- delta).
struct ExpandTask {
    int32_t sec;
    int32_t block;
    int64_t out_off;  // first element of the block's copy in the step layout's expansion scratch
};

// Chunk tables of a step layout (one sector, or a batch of sectors).  Row chunks cut every sector's
// rows in order (the update, normalisation and exact-norm passes); H.v chunks are the segment
// chunks of free blocks and the row chunks of the other blocks, sector-major (the step's partial
// sums are indexed by H.v chunk), with their ids grouped by row kind.
struct ChunkPlan {
    std::vector<BatchChunk> chunks;   // row chunks
    std::vector<int> cfirst, ccount;  // per sector, into chunks
    std::vector<BatchChunk> hv;       // H.v chunks
    std::vector<int> hv_first, hv_count;  // per sector, into hv
    std::vector<int> kind_idx;        // hv ids by kind
    int kind_first[4] = {0, 0, 0, 0};
    int kind_count[4] = {0, 0, 0, 0};
    std::vector<ExpandTask> tasks;    // expanded copies (Sector::copy_blocks of every sector, in order)
    int64_t n_full = 0;               // elements of the expansion scratch
};

struct Sector {
    SectorView view{};
    uint64_t serial = 0;         // unique per created sector in this process (batch workspace key)
    int64_t n_hole_masks = 0;
    uint64_t n_spin = 0;
    int kx_raw = 0;
    bool real = false;
    bool built = false;
    int device = 0;
    int num_sms = 152;
    int hv_grid = 0;             // persistent grid of the H.v kernels (free-row step kernel)
    int hv_minb = 3;             // launch variant of the free-row step kernel (minimum resident CTAs per SM)
    int seg_nr = 0;              // rows per lane the free-row kernel works on together (0: by dtype)
    int seg_staged = 0;          // 1: the free-row kernel gathers through shared memory (cp.async)
    int seg_chunk_rows = kSegChunkRows;  // rows of a segment chunk (the plan's unit of work and of partial sums)
    // offsets of a segment chunk's window: 32 (a lane's two rows in two segments at the same offset)
    // or 64 (a lane's two rows 32 offsets apart in one segment); part of the plan, like the chunk rows
    int seg_win = kSegWin;
    int other_grid = 0;          // grid of the other row kinds' step kernels
    int cand_grid_f32 = 0;       // grid of the stabiliser-row kernel for real FP32 vectors
    std::vector<BlockSpan> spans;  // host copy of the blocks' row ranges and kinds
    DevBuf<uint32_t> d_comb;     // [33][33]
    DevBuf<uint32_t> d_rank_tab; // colex spin-rank tables (layout: RankTab)
    DevBuf<BlockInfo> d_blocks;
    DevBuf<HoleEntry> d_holes;
    DevBuf<uint64_t> d_bitmap;
    DevBuf<int64_t> d_prefix;
    DevBuf<ulonglong2> d_bitpref;
    DevBuf<uint64_t> d_keys;
    DevBuf<uint8_t> d_orbit;
    DevBuf<double> d_partials;   // [hv_grid][kReduceSlots] scratch of the fused Lanczos step
    DevBuf<double> d_hv_scal;    // step scalars written by ed_hv's pass through the step kernels (unused)
    DevBuf<double> d_proj;       // projection scratch: partial dots and coefficients
    // the sector as a batch of one (step kernels): device view, offsets and chunk table
    int n_chunks = 0;
    DevBuf<SectorView> d_self;
    DevBuf<int64_t> d_offs;
    DevBuf<BatchChunk> d_chunks;
    DevBuf<int> d_kidx;
    int kind_first[4] = {0, 0, 0, 0};
    int kind_count[4] = {0, 0, 0, 0};
    DevBuf<int> d_cfirst, d_ccount;
    DevBuf<BlockDesc> d_desc;    // fast-row descriptors
    // stabiliser blocks' expanded copies (single-sector steps): tasks and scratch for the widest
    // element (16 bytes)
    int n_tasks = 0;
    int64_t n_full = 0;
    DevBuf<ExpandTask> d_tasks;
    DevBuf<uint8_t> d_xfull;
    std::vector<int> copy_blocks;  // blocks with an expanded copy, in block order (build_segments)
    // segment layout of free blocks (build_segments)
    DevBuf<SegDesc> d_seg;
    DevBuf<uint32_t> d_seg_h, d_seg_base, d_seg_rec;
    std::vector<uint32_t> host_seg_off;  // seg_off of the view, kl = 0 .. P + 1
    // H.v chunks of single-sector steps (ChunkPlan::hv)
    int n_hv_chunks = 0;
    DevBuf<BatchChunk> d_hv_chunks;
    DevBuf<int> d_hv_first, d_hv_count;
};

// Colex spin-rank tables of Ns spins with Nd down (layout: RankTab): fills V's rk_* fields and
// rank_words and the table words.  comb[k][n] = C(n, k).  Host code, shared by ed_sector_create
// and the host checks of the tables.
inline void rank_tables_build(int Ns, int Nd, const uint32_t (&comb)[kCombStride][kCombStride], SectorView& V,
                              std::vector<uint32_t>& tab) {
    // chunk 0 of w0 bits (2^w0 entries, no set bits below it), then 8-bit chunks of Nd + 1 rows
    const int nch = Ns <= 28 ? 3 : 4;
    int w0 = Ns - 8 * (nch - 1);
    if (w0 < 0) w0 = 0;
    V.rk_nch = (uint32_t)nch;
    V.rk_m0 = (1u << w0) - 1u;
    uint32_t words = 1u << w0;
    for (int c = 0; c < 4; ++c) {
        V.rk_pos[c] = c == 0 ? 0u : (uint32_t)(w0 + 8 * (c - 1));
        V.rk_off[c] = c == 0 ? 0u : words;
        if (c > 0 && c < nch) words += (uint32_t)(Nd + 1) << 8;
    }
    V.rank_words = (int)words;
    tab.assign(words, 0u);
    auto chunk_sum = [&](uint32_t bits, int pos, int k) {
        // sum over the set bits of `bits` (j-th from the bottom, at pos + b) of C(pos + b, k + j)
        uint32_t r = 0;
        int j = 0;
        for (int b = 0; b < 16; ++b)
            if (bits & (1u << b)) {
                ++j;
                const int nn = pos + b, kk = k + j;
                if (nn <= kMaxN && kk <= kMaxN) r += comb[kk][nn];
            }
        return r;
    };
    for (uint32_t bits = 0; bits < (1u << w0); ++bits) tab[bits] = chunk_sum(bits, 0, 0);
    for (int c = 1; c < nch; ++c)
        for (int k = 0; k <= Nd; ++k)
            for (uint32_t byte = 0; byte < 256u; ++byte)
                tab[V.rk_off[c] + ((uint32_t)k << 8) + byte] = chunk_sum(byte, (int)V.rk_pos[c], k);
}

// ed_basis.cu
int basis_build(Sector& s, cudaStream_t st);
int basis_export(Sector& s, int64_t* sparse_dev, int32_t* orbit_dev, cudaStream_t st);
void pack_flags(const uint8_t* f, int64_t n, uint64_t* words, cudaStream_t st, int sms);
void expand_flag_scan(const uint8_t* f, int64_t n, const uint64_t* words, const int64_t* wprefix, int64_t* out,
                      cudaStream_t st, int sms);
int scan_popcounts(const uint64_t* words, int64_t m, int64_t* prefix, int64_t* total_host, cudaStream_t st);

// ed_hv.cu
struct HvWeights {
    double w[4];   // tl, tr, jl, jr; 0 disables a term
    int faithful;  // 1: every term through the reference-faithful orbit walk (self-check path)
};
int hv_launch(const Sector& s, const HvWeights& w, int dtype, const void* x, void* y, cudaStream_t st);
int hv_step_launch(const Sector& s, const HvWeights& w, int dtype, const void* x, void* y, cudaStream_t st);
int lanczos_step_launch(const Sector& s, const HvWeights& w, int dtype, const void* v, const void* vprev,
                        void* vnext, double* scal, double* partials, cudaStream_t st);
int lanczos_hv_launch(const Sector& s, const HvWeights& w, int dtype, const void* v, const void* vprev, void* vnext,
                      double* scal, double* partials, cudaStream_t st);
int lanczos_update_launch(const Sector& s, int dtype, const void* v, void* vnext, const double* scal, cudaStream_t st);
int accumulate_launch(const Sector& s, int dtype, const void* x, double cr, double ci, void* acc, cudaStream_t st);
constexpr int kAccumMany = 32;  // vectors one accumulate_many_kernel launch takes (the rest in further launches)
int accumulate_many_launch(const Sector& s, int dtype, int k, const void* const* xs, const double* coefs, void* acc,
                           cudaStream_t st);
int normalize_launch(const Sector& s, int dtype, void* x, double* norm, double* partials, cudaStream_t st);
int single_setup(Sector& s);
int build_descriptors(Sector& s);
int seg_records_build(Sector& s, const std::vector<int>& free_blocks, int64_t nseg);  // ed_segrec.cu
int set_launch(Sector& s, int minb, int ctas_per_sm);
int set_step_shape(Sector& s, int rows_per_lane, int chunk_rows, int staged);  // re-plans when chunk_rows changes
int set_segment_window(Sector& s, int offsets);  // 32 or 64; re-plans when it changes
void plan_chunks(const std::vector<const Sector*>& secs, ChunkPlan& plan);

// ed_step_free.cu / ed_step_rest.cu: the fused step kernel of one row kind over a list of chunks
struct StepArgs {
    const SectorView* views;
    const int64_t* offs;
    const BatchChunk* chunks;
    const int* idx;  // chunk ids of this kind
    int count;
    int grid;
    size_t smem;
    HvWeights w;
    void* v;
    void* vprev;
    void* other;
    int first;
    const double* scal;
    int stride;
    int k;
    double* partials;
    // stabiliser blocks' expansion: tasks, their count, C(Ns, Nd), the scratch
    const ExpandTask* tasks;
    int ntasks;
    int64_t n_spin;
    void* xfull;
};
// pair: 1 for chunks planned with 32-offset windows (a lane's rows in two segments), 0 for 64-offset
// windows (kRowsFree64)
int step_hv_free(int dtype, int minb, int nr, int staged, int pair, const StepArgs& a, cudaStream_t st);
int step_hv_free_staged(int dtype, int nr, const StepArgs& a, cudaStream_t st);
int step_hv_free_nr1(int dtype, int minb, int pair, const StepArgs& a, cudaStream_t st);
int step_hv_free_split(int dtype, int nr, int pair, const StepArgs& a, cudaStream_t st);
// rows per lane of the free-row kernel for a dtype when the sector leaves it open (seg_nr = 0)
inline int seg_rows_for(int dtype, int nr) { return nr ? nr : ((dtype == ED_F32 || dtype == ED_C64) ? 2 : 1); }
int step_expand(int dtype, const StepArgs& a, cudaStream_t st);
int step_hv_cand(int dtype, const StepArgs& a, cudaStream_t st);
int step_hv_generic(int dtype, const StepArgs& a, cudaStream_t st);
int step_free_occupancy(int minb, size_t smem);
int step_rest_occupancy(size_t smem, bool f32);
int singlet_corr_launch(const Sector& s, int dtype, const void* psi, const int* fixed, double* out, cudaStream_t st);
int corr_launch(const Sector& s, int dtype, const void* psi, int kind, int nfixed, const int* fixed, double* out,
                cudaStream_t st);
int excite_launch(const Sector& src, const Sector& dst, int op, int qx, int qy, int initial_sz2, int dtype,
                  const void* x, void* y, cudaStream_t st);
void batch_forget(const Sector& s);  // frees the kept batch workspace if it holds s
int batch_lanczos_launch(const std::vector<const Sector*>& secs, const HvWeights& w, int dtype, const void* const* v0,
                         int m, double* coef, int use_graph, cudaStream_t st);
int project_launch(const Sector& s, int dtype, const void* V, int k, void* w, double* coef, double* scratch,
                   int64_t scratch_len, cudaStream_t st);
int project_noalloc_launch(const Sector& s, int dtype, const void* V, int k, void* w, double* coef_out,
                           cudaStream_t st);
int cf_launch(const double* a, const double* b, int m, const double* omega, int W, double e0, double eta,
              double norm2, double* out, cudaStream_t st);

}  // namespace ed
