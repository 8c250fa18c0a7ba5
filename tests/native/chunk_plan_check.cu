// Host check of the step layout (ed_batch.cu: plan_chunks) on synthetic sectors: chunks tile every
// sector's rows, never straddle two blocks and follow the per-kind length rule; a sector is cut the
// same way alone and inside a batch (what keeps batched and sequential recursions bit-identical);
// every stabiliser block gets one expansion task whose copy the block's chunks point at.  Built with
// nvcc (the file's kernels are compiled but never launched) and run by tests/test_native_host.py;
// exits non-zero on any difference.
#include <cstdio>
#include <random>

#include "ed_batch.cu"

namespace ed {
// the other translation units of the library, not exercised here
int set_error(int code, const char*) { return code; }
int set_cuda_error(cudaError_t, const char*) { return ED_ERR_CUDA; }
int step_hv_free(int, int, const StepArgs&, cudaStream_t) { return 0; }
int step_expand(int, const StepArgs&, cudaStream_t) { return 0; }
int step_hv_cand(int, const StepArgs&, cudaStream_t) { return 0; }
int step_hv_generic(int, const StepArgs&, cudaStream_t) { return 0; }
int step_free_occupancy(int, size_t) { return 4; }
int step_rest_occupancy(size_t, bool) { return 3; }
}  // namespace ed

using namespace ed;

namespace {

long bad = 0;

void expect(bool ok, const char* what, int a = 0, int b = 0) {
    if (!ok && bad++ < 10) std::printf("FAIL %s (%d, %d)\n", what, a, b);
}

// A synthetic built sector: blocks of random sizes and kinds tiling [0, n).
void make_sector(Sector& s, std::mt19937_64& rng, int nblocks, uint64_t n_spin) {
    s.num_sms = 152;
    s.n_spin = n_spin;
    s.spans.clear();
    int64_t next = 0;
    for (int b = 0; b < nblocks; ++b) {
        const int kind = 1 + (int)(rng() % 3);
        const int64_t count = kind == kRowsFree ? (int64_t)n_spin : 1 + (int64_t)(rng() % n_spin);
        s.spans.push_back(BlockSpan{next, count, b, kind});
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

}  // namespace

int main() {
    std::mt19937_64 rng(5);
    for (int trial = 0; trial < 40; ++trial) {
        const int nsec = 1 + (int)(rng() % 5);
        std::vector<Sector> secs(nsec);
        const uint64_t n_spin = 1000 + rng() % 400000;
        for (int s = 0; s < nsec; ++s) make_sector(secs[s], rng, 1 + (int)(rng() % 12), n_spin);
        std::vector<const Sector*> ptrs;
        for (const Sector& s : secs) ptrs.push_back(&s);
        ChunkPlan batch;
        plan_chunks(ptrs, batch);
        int64_t task_elems = 0;
        for (const ExpandTask& t : batch.tasks) {
            expect(t.out_off == task_elems, "expansion copies are consecutive", trial);
            task_elems += (int64_t)n_spin;
        }
        expect(batch.n_full == task_elems, "expansion scratch size", trial);
        for (int s = 0; s < nsec; ++s) {
            ChunkPlan alone;
            plan_chunks({&secs[s]}, alone);
            expect(alone.ccount[0] == batch.ccount[s], "chunk count alone and in a batch", trial, s);
            int64_t covered = 0;
            size_t task = 0;
            for (int c = 0; c < alone.ccount[0]; ++c) {
                const BatchChunk& a = alone.chunks[c];
                const BatchChunk& b = batch.chunks[batch.cfirst[s] + c];
                expect(a.begin == b.begin && a.end == b.end && a.block == b.block, "same cut alone and in a batch",
                       trial, c);
                expect(b.sec == s, "chunk sector", trial, c);
                expect(a.begin == covered, "chunks tile the rows", trial, c);
                covered = a.end;
                const BlockSpan& sp = secs[s].spans[a.block];
                expect(a.begin >= sp.start && a.end <= sp.start + sp.count, "chunk inside its block", trial, c);
                expect(a.end - a.begin <= expected_chunk_rows(secs[s], sp.kind), "chunk length", trial, c);
                if (sp.kind == kRowsCand) {
                    expect(a.xoff >= 0 && b.xoff >= 0, "stabiliser chunk points at a copy", trial, c);
                    // the batch's task of this block
                    while (task < alone.tasks.size() && alone.tasks[task].block != a.block) ++task;
                    expect(task < alone.tasks.size() && alone.tasks[task].out_off == a.xoff, "copy of the block",
                           trial, c);
                } else {
                    expect(a.xoff == -1, "only stabiliser chunks point at a copy", trial, c);
                }
            }
            expect(covered == secs[s].view.n, "every row in a chunk", trial, s);
        }
        // kind lists: every chunk id once, grouped by kind
        std::vector<int> seen(batch.chunks.size(), 0);
        for (int kind = kRowsFree; kind <= kRowsGeneric; ++kind)
            for (int i = 0; i < batch.kind_count[kind]; ++i) {
                const int id = batch.kind_idx[batch.kind_first[kind] + i];
                ++seen[id];
                const BatchChunk& c = batch.chunks[id];
                expect(ptrs[c.sec]->spans[c.block].kind == kind, "chunk listed under its kind", trial, id);
            }
        for (int v : seen) expect(v == 1, "every chunk listed once", trial, v);
    }
    std::printf("differences %ld\n", bad);
    return bad != 0;
}
