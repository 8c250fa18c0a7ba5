// Host check of the step layout (ed_batch.cu: plan_chunks) on synthetic sectors: row chunks tile
// every sector's rows, never straddle two blocks and follow the per-kind length rule (pinned on two
// hand-built sectors as well); segment chunks tile every class and offset window of every free block
// in whole rounds of the CTA's warps, for 32- and 64-offset windows; a sector is cut the same way alone and inside a batch (what keeps batched
// and sequential recursions bit-identical); every listed block gets one expanded copy, and
// stabiliser chunks point at their block's copy.  Built with nvcc (the file's kernels are compiled
// but never launched) and run by tests/test_native_host.py; exits non-zero on any difference.
#include <cstdio>
#include <random>

#include "ed_batch.cu"
#include "ed_desc.cu"

namespace ed {
// the other translation units of the library, not exercised here
int set_error(int code, const char*) { return code; }
int set_cuda_error(cudaError_t, const char*) { return ED_ERR_CUDA; }
int step_hv_free(int, int, int, int, int, const StepArgs&, cudaStream_t) { return 0; }
int step_expand(int, const StepArgs&, cudaStream_t) { return 0; }
int step_hv_cand(int, const StepArgs&, cudaStream_t) { return 0; }
int step_hv_generic(int, const StepArgs&, cudaStream_t) { return 0; }
int step_free_occupancy(int, size_t) { return 4; }
int step_rest_occupancy(size_t, bool) { return 3; }
int seg_records_build(Sector&, const std::vector<int>&, int64_t) { return ED_OK; }
}  // namespace ed

using namespace ed;

namespace {

long bad = 0;

void expect(bool ok, const char* what, int a = 0, int b = 0) {
    if (!ok && bad++ < 10) std::printf("FAIL %s (%d, %d)\n", what, a, b);
}

// A synthetic built sector: blocks of random sizes and kinds tiling [0, n); free blocks hold all
// C(Ns, Nd) configurations (segment tables from seg_tables); the blocks with an expanded copy are
// the stabiliser blocks with rows plus a few others (as hop targets of free blocks can add).
void make_sector(Sector& s, std::mt19937_64& rng, int nblocks, int Ns, int Nd) {
    uint32_t comb[kCombStride][kCombStride] = {};
    for (int n = 0; n <= kMaxN; ++n) {
        comb[0][n] = 1;
        for (int k = 1; k <= n; ++k) comb[k][n] = comb[k - 1][n - 1] + (k <= n - 1 ? comb[k][n - 1] : 0);
    }
    const uint64_t n_spin = comb[Nd][Ns];
    s.num_sms = 152;
    s.n_spin = n_spin;
    s.seg_win = rng() % 2 ? 32 : 64;
    s.view.Ns = Ns;
    s.view.Nd = Nd;
    s.view.n_blocks = nblocks;
    s.view.seg_p = std::min(kSegA, Ns);
    std::vector<uint32_t> hs, bases;
    seg_tables(Ns, Nd, s.view.seg_p, comb, s.view.seg_off, hs, bases);
    s.host_seg_off.assign(s.view.seg_off, s.view.seg_off + s.view.seg_p + 2);
    s.spans.clear();
    s.copy_blocks.clear();
    int64_t next = 0;
    for (int b = 0; b < nblocks; ++b) {
        const int kind = 1 + (int)(rng() % 3);
        const int64_t count = kind == kRowsFree ? (int64_t)n_spin : (int64_t)(rng() % n_spin);
        s.spans.push_back(BlockSpan{next, count, b, kind});
        if (count > 0 && (kind == kRowsCand || (kind == kRowsGeneric && rng() % 3 == 0))) s.copy_blocks.push_back(b);
        next += count;
    }
    s.view.n = next;
}

int64_t expected_chunk_rows(const Sector& s, int kind) {
    int64_t rows = 0;
    for (const BlockSpan& sp : s.spans)
        if (sp.kind == kind) rows += sp.count;
    int64_t c = kChunkRows;
    while (c > kChunkRows / 8 && rows / c < 4 * (int64_t)s.num_sms) c /= 2;
    return c;
}

int64_t binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    int64_t r = 1;
    for (int j = 1; j <= k; ++j) r = r * (n - k + j) / j;
    return r;
}

}  // namespace

int main() {
    std::mt19937_64 rng(5);
    // the chunk-length rule on hand-built sectors: kChunkRows / 8 below 4 * SMs * kChunkRows / 8 rows of
    // a kind, kChunkRows from 4 * SMs * kChunkRows rows on
    {
        Sector a, b;
        for (Sector* x : {&a, &b}) {
            x->num_sms = 152;
            x->view.Ns = 10;
            x->view.Nd = 5;
            x->view.seg_p = 9;
        }
        a.spans = {BlockSpan{0, 100, 0, kRowsCand}};
        a.view.n = 100;
        b.spans = {BlockSpan{0, 4 * 152 * (int64_t)kChunkRows, 0, kRowsGeneric}};
        b.view.n = b.spans[0].count;
        ChunkPlan pa, pb;
        plan_chunks({&a}, pa);
        plan_chunks({&b}, pb);
        expect(pa.chunks.size() == 1 && pa.chunks[0].end - pa.chunks[0].begin == 100, "a 100-row kind is one chunk");
        expect(expected_chunk_rows(a, kRowsCand) == kChunkRows / 8, "small kinds use the shortest chunks");
        expect((int64_t)pb.chunks.size() == 4 * 152 && pb.chunks[0].end - pb.chunks[0].begin == kChunkRows,
               "large kinds use kChunkRows");
    }
    for (int trial = 0; trial < 40; ++trial) {
        const int nsec = 1 + (int)(rng() % 5);
        const int Ns = 10 + (int)(rng() % 9);
        const int Nd = 1 + (int)(rng() % (Ns - 1));
        std::vector<Sector> secs(nsec);
        for (int s = 0; s < nsec; ++s) make_sector(secs[s], rng, 1 + (int)(rng() % 12), Ns, Nd);
        const int64_t n_spin = (int64_t)secs[0].n_spin;
        std::vector<const Sector*> ptrs;
        for (const Sector& s : secs) ptrs.push_back(&s);
        ChunkPlan batch;
        plan_chunks(ptrs, batch);
        int64_t task_elems = 0;
        size_t ti = 0;
        std::vector<int64_t> sec_base(nsec, 0);
        for (int s = 0; s < nsec; ++s) {
            sec_base[s] = task_elems;
            for (int b : secs[s].copy_blocks) {
                expect(ti < batch.tasks.size() && batch.tasks[ti].sec == s && batch.tasks[ti].block == b &&
                           batch.tasks[ti].out_off == task_elems,
                       "one copy per listed block, consecutive", trial, (int)ti);
                ++ti;
                task_elems += n_spin;
            }
        }
        expect(ti == batch.tasks.size() && batch.n_full == task_elems, "expansion scratch size", trial);
        for (int s = 0; s < nsec; ++s) {
            ChunkPlan alone;
            plan_chunks({&secs[s]}, alone);
            // row chunks
            expect(alone.ccount[0] == batch.ccount[s], "row chunk count alone and in a batch", trial, s);
            int64_t covered = 0;
            for (int c = 0; c < alone.ccount[0]; ++c) {
                const BatchChunk& a = alone.chunks[c];
                const BatchChunk& b = batch.chunks[batch.cfirst[s] + c];
                expect(a.begin == b.begin && a.end == b.end && a.block == b.block, "same cut alone and in a batch",
                       trial, c);
                expect(b.sec == s && a.kl == -1, "row chunk sector and class", trial, c);
                expect(a.begin == covered, "chunks tile the rows", trial, c);
                covered = a.end;
                const BlockSpan& sp = secs[s].spans[a.block];
                expect(a.begin >= sp.start && a.end <= sp.start + sp.count, "chunk inside its block", trial, c);
                expect(a.end - a.begin <= expected_chunk_rows(secs[s], sp.kind), "chunk length", trial, c);
                if (sp.kind == kRowsCand) {
                    size_t task = 0;
                    while (task < alone.tasks.size() && alone.tasks[task].block != a.block) ++task;
                    expect(task < alone.tasks.size() && alone.tasks[task].out_off == a.xoff &&
                               b.xoff - sec_base[s] == a.xoff,
                           "stabiliser chunk points at its block's copy", trial, c);
                } else {
                    expect(a.xoff == -1, "only stabiliser row chunks point at a copy", trial, c);
                }
            }
            expect(covered == secs[s].view.n, "every row in a chunk", trial, s);
            // H.v chunks: the same alone and in a batch; segment chunks tile every class of every free block
            expect(alone.hv_count[0] == batch.hv_count[s], "H.v chunk count alone and in a batch", trial, s);
            const int P = secs[s].view.seg_p;
            // per (block, class, window): the next segment the chunks must start at
            std::vector<std::vector<int64_t>> seg_next(secs[s].spans.size(), std::vector<int64_t>((P + 1) * 8, 0));
            for (int c = 0; c < alone.hv_count[0]; ++c) {
                const BatchChunk& a = alone.hv[c];
                const BatchChunk& b = batch.hv[batch.hv_first[s] + c];
                expect(a.begin == b.begin && a.end == b.end && a.block == b.block && a.kl == b.kl &&
                           a.piece == b.piece && b.xoff - (a.kl >= 0 || a.xoff >= 0 ? sec_base[s] : 0) == a.xoff &&
                           b.sec == s,
                       "same H.v chunk alone and in a batch", trial, c);
                const BlockSpan& sp = secs[s].spans[a.block];
                if (sp.kind != kRowsFree) {
                    expect(a.kl == -1, "row chunks of other blocks", trial, c);
                    continue;
                }
                expect(a.kl >= 0 && a.kl <= P && a.xoff == 0, "segment chunk class and copies", trial, c);
                const int64_t nseg = (int64_t)secs[s].host_seg_off[a.kl + 1] - secs[s].host_seg_off[a.kl];
                const int64_t nA = binom(P, a.kl);
                const int64_t sw = secs[s].seg_win;
                const int64_t pieces = (nA + sw - 1) / sw;
                const int64_t round = (sw == 32 ? 2 : 1) * (kSegThreads / 32);  // segments per round of the warps
                expect(a.piece >= 0 && a.piece < pieces, "window inside the segment", trial, c);
                int64_t& next = seg_next[a.block][a.kl * 8 + a.piece];
                expect(a.begin == next && a.end > a.begin && a.end <= nseg, "segment chunks tile their class", trial, c);
                expect(a.end == nseg || (a.end - a.begin) % round == 0, "whole rounds of the CTA's warps", trial, c);
                next = a.end;
            }
            for (const BlockSpan& sp : secs[s].spans)
                if (sp.kind == kRowsFree && sp.count > 0)
                    for (int kl = 0; kl <= P; ++kl) {
                        const int64_t nA = binom(P, kl);
                        const int64_t pieces = (nA + secs[s].seg_win - 1) / secs[s].seg_win;
                        for (int64_t pc = 0; pc < pieces; ++pc)
                            expect(seg_next[sp.block][kl * 8 + pc] ==
                                       (int64_t)secs[s].host_seg_off[kl + 1] - secs[s].host_seg_off[kl],
                                   "every segment window in a chunk", trial, kl);
                    }
        }
        // kind lists: every H.v chunk id once, grouped by kind
        std::vector<int> seen(batch.hv.size(), 0);
        for (int kind = kRowsFree64; kind <= kRowsGeneric; ++kind)
            for (int i = 0; i < batch.kind_count[kind]; ++i) {
                const int id = batch.kind_idx[batch.kind_first[kind] + i];
                ++seen[id];
                const BatchChunk& c = batch.hv[id];
                const int bk = ptrs[c.sec]->spans[c.block].kind;
                const int want = bk == kRowsFree && ptrs[c.sec]->seg_win == 64 ? kRowsFree64 : bk;
                expect(want == kind, "chunk listed under its kind", trial, id);
            }
        for (int v : seen) expect(v == 1, "every chunk listed once", trial, v);
    }
    std::printf("differences %ld\n", bad);
    return bad != 0;
}
