// ed_segrec.cu -- the segment records of free blocks, built once per sector.
//
// What the rows of one segment share (the partner segments of its antiparallel high bonds and of its
// cross bonds, the target bases of its hops; layout in ed_common.cuh above SegDesc) depends only on
// the segment's high part H and the block's terms, never on a vector.  One thread per (free block,
// segment) writes the record with the same index helpers the step kernel's rows use (ed_seg.cuh);
// the step kernel then reads records instead of recomputing them every step.
#include "ed_seg.cuh"

namespace ed {

__global__ void seg_records_kernel(const SectorView S, const int* __restrict__ free_blocks, int nfree, int64_t nseg,
                                   uint32_t* __restrict__ rec) {
    const int P = S.seg_p, Nd = S.Nd, Ns = S.Ns;
    const uint32_t amask = (1u << P) - 1u, nsmask = 0xffffffffu >> (32 - Ns);
    const RankTab R = rank_tab_of(S, S.rank_tab);
    const int64_t total = (int64_t)nfree * nseg;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        const int fb = (int)(u / nseg);
        const int64_t g = u - (int64_t)fb * nseg;
        const SegDesc& D = S.seg[free_blocks[fb]];
        int kl = 0;
        while ((int64_t)S.seg_off[kl + 1] <= g) ++kl;
        const uint32_t Hs = S.seg_h[g] << P;
        uint32_t* out = rec + D.rec + g * (int64_t)D.rec_len;
        for (uint32_t w = 0; w < D.rec_len; ++w) out[w] = 0u;
        const uint32_t base = S.seg_base[g];
        out[0] = base;
        const uint32_t d1 = Hs ^ (Hs >> 1);
        const uint32_t zbr = (uint32_t)popc32(d1 & D.mr);
        const uint32_t zbl = (uint32_t)popc32(d1 & D.ma) + (uint32_t)popc32((Hs ^ (Hs >> 2)) & D.m2);
        uint32_t hib = 0;
        for (int c = 0; c < D.nX; ++c) hib |= ((Hs >> D.cX[c][1]) & 1u) << c;
        const uint32_t zb = zbr + zbl;
        out[1] = zb | (zbr << 8) | (hib << 16);
        // padding of the high-bond list: the segment itself (the kernel takes it back out)
        for (uint32_t q = zb; q < ((zb + 3u) & ~3u); ++q) out[4 + q] = base;
        for (int i = 0; i < D.nB; ++i) {
            const uint32_t a = D.bB[i][0], b = D.bB[i][1];
            if (((Hs >> a) ^ (Hs >> b)) & 1u)
                out[4 + seg_high_pos(Hs, i, a, D.nBr, D.nBa, D.mr, D.ma, D.m2)] = seg_high_partner(Hs, a, b, kl, R, Nd);
        }
        for (int c = 0; c < D.nX; ++c) out[D.xo + c] = seg_cross_partner(Hs, D.cX[c][1], kl, P, R, Nd);
        for (int h = 0; h < D.nhop; ++h) {
            const SegHopDesc& G = D.hop[h];
            uint32_t* o = out + D.hop_off[h];
            if (G.kind == 3) continue;  // the record word stays 0
            const uint32_t U = seg_perm(Hs, G.keep, G.band, G.sl, G.sr, G.p, G.q, G.swap, G.rot, G.nsr, nsmask);
            if (G.nb >= 3) {
                o[0] = U;
            } else if (G.nb == 0) {
                o[0] = seg_hop_base(U, amask, 0, 0, 0, P, R, Nd);
            } else {
                o[0] = U & amask;
                for (int vbi = 0; vbi < (1 << G.nb); ++vbi)
                    o[1 + vbi] = seg_hop_base(U, amask, vbi, G.bpos[0], G.bpos[1], P, R, Nd);
            }
        }
    }
}

int seg_records_build(Sector& s, const std::vector<int>& free_blocks, int64_t nseg) {
    const int nfree = (int)free_blocks.size();
    if (nfree == 0 || nseg == 0) return ED_OK;
    DevBuf<int> d_free(nfree);
    if (!d_free.ok()) return set_error(ED_ERR_NOMEM, "segment records: device allocation");
    if (cudaMemcpy(d_free.p, free_blocks.data(), nfree * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return set_error(ED_ERR_CUDA, "segment records: upload");
    const int threads = 256;
    const int grid = grid_for((int64_t)nfree * nseg, threads, s.num_sms, 16);
    seg_records_kernel<<<grid, threads>>>(s.view, d_free.p, nfree, nseg, s.d_seg_rec.p);
    ED_CHECK_LAUNCH("seg_records_kernel");
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return set_cuda_error(e, "segment records");
    return ED_OK;
}

}  // namespace ed
