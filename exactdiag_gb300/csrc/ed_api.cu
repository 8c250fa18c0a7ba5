// ed_api.cu -- the extern "C" boundary of libexactdiag_gb300.so.
// Every entry point validates its arguments, returns an int status and never
// lets a C++ exception or CUDA error escape; the text of the last failure is
// kept per thread for ed_last_error_string().
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "ed_internal.cuh"

namespace ed {

namespace {
thread_local std::string g_last_error;
}

int set_error(int code, const char* what) {
    g_last_error = what ? what : "";
    return code;
}

int set_cuda_error(cudaError_t e, const char* what) {
    g_last_error = std::string(what ? what : "") + ": " + cudaGetErrorString(e);
    return ED_ERR_CUDA;
}

size_t hv_smem_bytes_host(const SectorView& S, size_t real_size);
int hv_blocks_per_sm(const SectorView& S);

static void host_comb(uint32_t c[kCombStride][kCombStride]) {
    // c[k][n] = C(n, k) for n <= 32 (all values < 2^32)
    uint64_t t[kCombStride][kCombStride];
    std::memset(t, 0, sizeof(t));
    for (int n = 0; n <= kMaxN; ++n) {
        t[0][n] = 1;
        for (int k = 1; k <= n; ++k) t[k][n] = t[k - 1][n - 1] + (k <= n - 1 ? t[k][n - 1] : 0);
    }
    for (int k = 0; k < kCombStride; ++k)
        for (int n = 0; n < kCombStride; ++n) c[k][n] = (uint32_t)t[k][n];
}

}  // namespace ed

using namespace ed;

struct ed_sector {
    Sector s;
};

extern "C" {

const char* ed_last_error_string(void) { return ed::g_last_error.c_str(); }

int ed_sector_create(int L, int Nh, int Nd, int kx, int ky, ed_sector** out) {
    if (!out) return set_error(ED_ERR_INVALID, "ed_sector_create: out is NULL");
    *out = nullptr;
    if (L < 2 || 2 * L > kMaxN) return set_error(ED_ERR_INVALID, "ed_sector_create: L must be in [2, 16]");
    const int N = 2 * L;
    if (Nh < 0 || Nh > N) return set_error(ED_ERR_INVALID, "ed_sector_create: Nh out of range");
    if (Nd < 0 || Nd > N - Nh) return set_error(ED_ERR_INVALID, "ed_sector_create: Nd out of range");
    if (ky != 0 && ky != 1) return set_error(ED_ERR_INVALID, "ed_sector_create: ky must be 0 or 1");
    ed_sector* h = new (std::nothrow) ed_sector();
    if (!h) return set_error(ED_ERR_NOMEM, "ed_sector_create: host allocation");
    Sector& s = h->s;
    static std::atomic<uint64_t> next_serial{1};
    s.serial = next_serial.fetch_add(1);
    uint32_t comb[kCombStride][kCombStride];
    host_comb(comb);
    SectorView& V = s.view;
    V.L = L;
    V.N = N;
    V.Nh = Nh;
    V.Nd = Nd;
    V.Ns = N - Nh;
    V.kx = ((kx % L) + L) % L;
    V.ky = ky;
    V.ne_even = ((N - Nh) % 2) == 0;
    V.mask = (N == 32) ? 0xffffffffu : ((1u << N) - 1u);
    s.kx_raw = kx;
    s.real = ((2 * V.kx) % L) == 0;
    s.n_spin = comb[Nd][N - Nh];
    s.n_hole_masks = comb[Nh][N];
    if (s.n_hole_masks > (int64_t(1) << 26)) {
        delete h;
        return set_error(ED_ERR_TOO_LARGE, "ed_sector_create: more than 2^26 hole masks");
    }
    cudaGetDevice(&s.device);
    cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, s.device);
    // colex spin-rank tables (layout: RankTab)
    std::vector<uint32_t> tab;
    rank_tables_build(N - Nh, Nd, comb, V, tab);
    if (!s.d_comb.alloc(kCombStride * kCombStride) || !s.d_rank_tab.alloc((int64_t)tab.size())) {
        delete h;
        return set_error(ED_ERR_NOMEM, "ed_sector_create: device tables");
    }
    cudaError_t e1 = cudaMemcpy(s.d_comb.p, comb, sizeof(comb), cudaMemcpyHostToDevice);
    cudaError_t e2 = cudaMemcpy(s.d_rank_tab.p, tab.data(), tab.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        delete h;
        return set_cuda_error(e1 != cudaSuccess ? e1 : e2, "ed_sector_create: table upload");
    }
    V.comb = s.d_comb.p;
    V.rank_tab = s.d_rank_tab.p;
    *out = h;
    return ED_OK;
}

int ed_sector_destroy(ed_sector* h) {
    if (h) batch_forget(h->s);
    delete h;
    return ED_OK;
}

int ed_basis_build(ed_sector* h, void* stream) {
    if (!h) return set_error(ED_ERR_INVALID, "ed_basis_build: NULL sector");
    Sector& s = h->s;
    if (s.built) return ED_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int rc;
    try {
        rc = basis_build(s, st);
    } catch (...) {
        return set_error(ED_ERR_INTERNAL, "ed_basis_build: exception");
    }
    if (rc != ED_OK) return rc;
    // persistent grid for the row kernels: SM count x resident CTAs per SM
    int per_sm = hv_blocks_per_sm(s.view);
    if (per_sm <= 0) per_sm = 1;
    if (per_sm > 8) per_sm = 8;
    s.hv_grid = s.num_sms * per_sm;
    if (int rc2 = build_descriptors(s)) return rc2;
    if (int rc3 = single_setup(s)) return rc3;
    return set_launch(s, 2, 0);
}

int ed_sector_set_launch(ed_sector* h, int min_ctas_per_sm, int ctas_per_sm) {
    if (!h) return set_error(ED_ERR_INVALID, "ed_sector_set_launch: NULL sector");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_sector_set_launch: basis not built");
    return set_launch(h->s, min_ctas_per_sm, ctas_per_sm);
}

int ed_sector_get_launch(const ed_sector* h, int* min_ctas_per_sm, int* grid) {
    if (!h || !min_ctas_per_sm || !grid) return set_error(ED_ERR_INVALID, "ed_sector_get_launch: NULL argument");
    *min_ctas_per_sm = h->s.hv_minb;
    *grid = h->s.hv_grid;
    return ED_OK;
}

int ed_sector_set_step_shape(ed_sector* h, int rows_per_lane, int chunk_rows, int staged_gathers) {
    if (!h) return set_error(ED_ERR_INVALID, "ed_sector_set_step_shape: NULL sector");
    return set_step_shape(h->s, rows_per_lane, chunk_rows, staged_gathers);
}

int ed_sector_set_segment_window(ed_sector* h, int offsets) {
    if (!h) return set_error(ED_ERR_INVALID, "ed_sector_set_segment_window: NULL sector");
    return set_segment_window(h->s, offsets);
}

int ed_sector_get_segment_window(const ed_sector* h, int* offsets) {
    if (!h || !offsets) return set_error(ED_ERR_INVALID, "ed_sector_get_segment_window: NULL argument");
    *offsets = h->s.seg_win;
    return ED_OK;
}

int ed_sector_get_step_shape(const ed_sector* h, int* rows_per_lane, int* chunk_rows, int* staged_gathers) {
    if (!h || !rows_per_lane || !chunk_rows || !staged_gathers)
        return set_error(ED_ERR_INVALID, "ed_sector_get_step_shape: NULL argument");
    *rows_per_lane = h->s.seg_nr;
    *chunk_rows = h->s.seg_chunk_rows;
    *staged_gathers = h->s.seg_staged;
    return ED_OK;
}

int ed_position_correlations(const ed_sector* h, int dtype, const void* psi_dev, int kind, int nfixed,
                             const int* fixed_shifts, double* out_host, void* stream) {
    if (!h || !psi_dev || !out_host) return set_error(ED_ERR_INVALID, "ed_position_correlations: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_position_correlations: basis not built");
    if ((dtype == ED_F64 || dtype == ED_F32) && !h->s.real)
        return set_error(ED_ERR_INVALID, "ed_position_correlations: real dtype with a complex sector");
    try {
        return corr_launch(h->s, dtype, psi_dev, kind, nfixed, fixed_shifts, out_host, (cudaStream_t)stream);
    } catch (...) {
        return set_error(ED_ERR_INTERNAL, "ed_position_correlations: exception");
    }
}

int ed_singlet_correlations(const ed_sector* h, int dtype, const void* psi_dev, const int fixed_shifts[4],
                            double* out_host, void* stream) {
    if (!h || !psi_dev || !out_host || !fixed_shifts)
        return set_error(ED_ERR_INVALID, "ed_singlet_correlations: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_singlet_correlations: basis not built");
    if (dtype == ED_F64 && !h->s.real)
        return set_error(ED_ERR_INVALID, "ed_singlet_correlations: real dtype with a complex sector");
    try {
        return singlet_corr_launch(h->s, dtype, psi_dev, fixed_shifts, out_host, (cudaStream_t)stream);
    } catch (...) {
        return set_error(ED_ERR_INTERNAL, "ed_singlet_correlations: exception");
    }
}

int ed_sector_row_kinds(const ed_sector* h, int counts[3]) {
    if (!h || !counts) return set_error(ED_ERR_INVALID, "ed_sector_row_kinds: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_sector_row_kinds: basis not built");
    counts[0] = h->s.kind_count[kRowsFree] + h->s.kind_count[kRowsFree64];
    counts[1] = h->s.kind_count[kRowsCand];
    counts[2] = h->s.kind_count[kRowsGeneric];
    return ED_OK;
}

int ed_sector_step_launches(const ed_sector* h, int* launches) {
    if (!h || !launches) return set_error(ED_ERR_INVALID, "ed_sector_step_launches: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_sector_step_launches: basis not built");
    const Sector& s = h->s;
    int n = s.n_tasks > 0 ? 1 : 0;  // expanded copies
    for (int kind = kRowsFree64; kind <= kRowsGeneric; ++kind) n += s.kind_count[kind] > 0 ? 1 : 0;
    *launches = n + 1 + 4;  // + scalars; update: flat pass, exact-norm pass, exact b, scaling pass
    return ED_OK;
}

int ed_sector_kind_rows(const ed_sector* h, int64_t rows[3]) {
    if (!h || !rows) return set_error(ED_ERR_INVALID, "ed_sector_kind_rows: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_sector_kind_rows: basis not built");
    rows[0] = rows[1] = rows[2] = 0;
    for (const BlockSpan& b : h->s.spans) {
        if (b.kind == kRowsFree) rows[0] += b.count;
        else if (b.kind == kRowsCand) rows[1] += b.count;
        else rows[2] += b.count;
    }
    return ED_OK;
}

int ed_basis_size(const ed_sector* h, int64_t* n) {
    if (!h || !n) return set_error(ED_ERR_INVALID, "ed_basis_size: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_basis_size: basis not built");
    *n = h->s.view.n;
    return ED_OK;
}

int ed_sector_is_real(const ed_sector* h, int* is_real) {
    if (!h || !is_real) return set_error(ED_ERR_INVALID, "ed_sector_is_real: NULL argument");
    *is_real = h->s.real ? 1 : 0;
    return ED_OK;
}

int ed_basis_export(const ed_sector* h, int64_t* sparse_dev, int32_t* orbit_dev, void* stream) {
    if (!h || !sparse_dev || !orbit_dev) return set_error(ED_ERR_INVALID, "ed_basis_export: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_basis_export: basis not built");
    return basis_export(const_cast<Sector&>(h->s), sparse_dev, orbit_dev, (cudaStream_t)stream);
}

static bool weights_ok(const double* w, HvWeights& out) {
    if (!w) return false;
    for (int t = 0; t < 4; ++t) {
        if (!std::isfinite(w[t])) return false;
        // matrix_setup.pyx:120-127 keeps terms with weight != 0 and
        // sparse_matrices.py:89 skips |weight| < 1e-6
        out.w[t] = (std::fabs(w[t]) < 1e-6) ? 0.0 : w[t];
    }
    out.faithful = 0;
    return true;
}

int ed_hv(const ed_sector* h, const double weights[4], int dtype, const void* x_dev, void* y_dev, void* stream) {
    if (!h) return set_error(ED_ERR_INVALID, "ed_hv: NULL sector");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_hv: basis not built");
    HvWeights w;
    if (!weights_ok(weights, w)) return set_error(ED_ERR_INVALID, "ed_hv: weights");
    if (h->s.view.n == 0) return ED_OK;  // empty sector: nothing to read or write (the vectors may be NULL)
    if (!x_dev || !y_dev) return set_error(ED_ERR_INVALID, "ed_hv: NULL argument");
    if (x_dev == y_dev) return set_error(ED_ERR_INVALID, "ed_hv: x and y must not alias");
    return hv_step_launch(h->s, w, dtype, x_dev, y_dev, (cudaStream_t)stream);
}

int ed_hv_mode(const ed_sector* h, const double weights[4], int dtype, const void* x_dev, void* y_dev, int mode,
               void* stream) {
    if (!h) return set_error(ED_ERR_INVALID, "ed_hv_mode: NULL sector");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_hv_mode: basis not built");
    if (mode != 0 && mode != 1) return set_error(ED_ERR_INVALID, "ed_hv_mode: mode must be 0 or 1");
    HvWeights w;
    if (!weights_ok(weights, w)) return set_error(ED_ERR_INVALID, "ed_hv_mode: weights");
    if (h->s.view.n == 0) return ED_OK;
    if (!x_dev || !y_dev) return set_error(ED_ERR_INVALID, "ed_hv_mode: NULL argument");
    if (x_dev == y_dev) return set_error(ED_ERR_INVALID, "ed_hv_mode: x and y must not alias");
    w.faithful = mode;
    return hv_launch(h->s, w, dtype, x_dev, y_dev, (cudaStream_t)stream);
}

int ed_lanczos_step(const ed_sector* h, const double weights[4], int dtype, const void* v_dev, const void* v_prev_dev,
                    void* v_next_dev, double* scal_dev, void* stream) {
    if (h && h->s.built && h->s.view.n == 0) return set_error(ED_ERR_INVALID, "ed_lanczos_step: empty sector");
    if (!h || !v_dev || !v_next_dev || !scal_dev) return set_error(ED_ERR_INVALID, "ed_lanczos_step: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_lanczos_step: basis not built");
    HvWeights w;
    if (!weights_ok(weights, w)) return set_error(ED_ERR_INVALID, "ed_lanczos_step: weights");
    if (v_dev == v_next_dev) return set_error(ED_ERR_INVALID, "ed_lanczos_step: v and v_next must not alias");
    return lanczos_step_launch(h->s, w, dtype, v_dev, v_prev_dev, v_next_dev, scal_dev, h->s.d_partials.p,
                               (cudaStream_t)stream);
}

int ed_lanczos_hv(const ed_sector* h, const double weights[4], int dtype, const void* v_dev, const void* v_prev_dev,
                  void* v_next_dev, double* scal_dev, void* stream) {
    if (h && h->s.built && h->s.view.n == 0) return set_error(ED_ERR_INVALID, "ed_lanczos_hv: empty sector");
    if (!h || !v_dev || !v_next_dev || !scal_dev) return set_error(ED_ERR_INVALID, "ed_lanczos_hv: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_lanczos_hv: basis not built");
    HvWeights w;
    if (!weights_ok(weights, w)) return set_error(ED_ERR_INVALID, "ed_lanczos_hv: weights");
    if (v_dev == v_next_dev) return set_error(ED_ERR_INVALID, "ed_lanczos_hv: v and v_next must not alias");
    return lanczos_hv_launch(h->s, w, dtype, v_dev, v_prev_dev, v_next_dev, scal_dev, h->s.d_partials.p,
                             (cudaStream_t)stream);
}

int ed_lanczos_update(const ed_sector* h, int dtype, const void* v_dev, void* v_next_dev, const double* scal_dev,
                      void* stream) {
    if (h && h->s.built && h->s.view.n == 0) return set_error(ED_ERR_INVALID, "ed_lanczos_update: empty sector");
    if (!h || !v_dev || !v_next_dev || !scal_dev) return set_error(ED_ERR_INVALID, "ed_lanczos_update: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_lanczos_update: basis not built");
    return lanczos_update_launch(h->s, dtype, v_dev, v_next_dev, scal_dev, (cudaStream_t)stream);
}

int ed_accumulate(const ed_sector* h, int dtype, const void* x_dev, double coef_re, double coef_im, void* acc_dev,
                  void* stream) {
    if (h && h->s.built && h->s.view.n == 0) return ED_OK;
    if (!h || !x_dev || !acc_dev) return set_error(ED_ERR_INVALID, "ed_accumulate: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_accumulate: basis not built");
    if (!std::isfinite(coef_re) || !std::isfinite(coef_im)) return set_error(ED_ERR_INVALID, "ed_accumulate: coef");
    return accumulate_launch(h->s, dtype, x_dev, coef_re, coef_im, acc_dev, (cudaStream_t)stream);
}

int ed_accumulate_many(const ed_sector* h, int dtype, int k, const void* const* x_devs, const double* coefs,
                       void* acc_dev, void* stream) {
    if (h && h->s.built && h->s.view.n == 0) return ED_OK;
    if (!h || !acc_dev || k < 0 || (k > 0 && (!x_devs || !coefs)))
        return set_error(ED_ERR_INVALID, "ed_accumulate_many: NULL argument or k < 0");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_accumulate_many: basis not built");
    for (int j = 0; j < k; ++j) {
        if (!x_devs[j]) return set_error(ED_ERR_INVALID, "ed_accumulate_many: NULL vector");
        if (!std::isfinite(coefs[2 * j]) || !std::isfinite(coefs[2 * j + 1]))
            return set_error(ED_ERR_INVALID, "ed_accumulate_many: coef");
    }
    return accumulate_many_launch(h->s, dtype, k, x_devs, coefs, acc_dev, (cudaStream_t)stream);
}

int ed_normalize(const ed_sector* h, int dtype, void* x_dev, double* norm_dev, void* stream) {
    if (h && h->s.built && h->s.view.n == 0) return set_error(ED_ERR_INVALID, "ed_normalize: empty sector");
    if (!h || !x_dev || !norm_dev) return set_error(ED_ERR_INVALID, "ed_normalize: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_normalize: basis not built");
    return normalize_launch(h->s, dtype, x_dev, norm_dev, h->s.d_partials.p, (cudaStream_t)stream);
}

int ed_excitation_apply(const ed_sector* src, const ed_sector* dst, int op, int qx, int qy, int initial_sz2, int dtype,
                        const void* x_src_dev, void* y_dst_dev, void* stream) {
    if (!src || !dst || !x_src_dev || !y_dst_dev) return set_error(ED_ERR_INVALID, "ed_excitation_apply: NULL");
    if (!src->s.built || !dst->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_excitation_apply: basis not built");
    return excite_launch(src->s, dst->s, op, qx, qy, initial_sz2, dtype, x_src_dev, y_dst_dev, (cudaStream_t)stream);
}

int ed_batch_lanczos(const ed_sector* const* sectors, int nsec, const double weights[4], int dtype,
                     const void* const* v0_dev, int m, double* coef_dev, int use_graph, void* stream) {
    if (!sectors || nsec <= 0 || !v0_dev || !coef_dev) return set_error(ED_ERR_INVALID, "ed_batch_lanczos: NULL");
    HvWeights w;
    if (!weights_ok(weights, w)) return set_error(ED_ERR_INVALID, "ed_batch_lanczos: weights");
    std::vector<const Sector*> secs;
    for (int i = 0; i < nsec; ++i) {
        if (!sectors[i] || !v0_dev[i]) return set_error(ED_ERR_INVALID, "ed_batch_lanczos: NULL sector or vector");
        secs.push_back(&sectors[i]->s);
    }
    try {
        return batch_lanczos_launch(secs, w, dtype, v0_dev, m, coef_dev, use_graph, (cudaStream_t)stream);
    } catch (...) {
        return set_error(ED_ERR_INTERNAL, "ed_batch_lanczos: exception");
    }
}

int ed_project_out(ed_sector* h, int dtype, const void* basis_dev, int k, void* w_dev, double* coef_dev,
                   void* stream) {
    if (!h || !basis_dev || !w_dev || k < 0) return set_error(ED_ERR_INVALID, "ed_project_out: bad argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_project_out: basis not built");
    if ((dtype == ED_F64 || dtype == ED_F32) && !h->s.real)
        return set_error(ED_ERR_INVALID, "ed_project_out: real dtype with a complex sector");
    if (k == 0) return ED_OK;
    Sector& s = h->s;
    const int64_t need = (int64_t)k * 2 * s.num_sms * kReduceSlots + 2 * (int64_t)k;
    if (s.d_proj.n < need) {
        cudaStreamSynchronize((cudaStream_t)stream);
        if (!s.d_proj.alloc(need)) return set_error(ED_ERR_NOMEM, "ed_project_out: scratch");
    }
    return project_launch(s, dtype, basis_dev, k, w_dev, coef_dev ? coef_dev : s.d_proj.p, s.d_proj.p + 2 * k,
                          s.d_proj.n - 2 * k, (cudaStream_t)stream);
}

int ed_project_out_noalloc(const ed_sector* h, int dtype, const void* basis_dev, int k, void* w_dev, double* coef_dev,
                           void* stream) {
    if (!h || !basis_dev || !w_dev) return set_error(ED_ERR_INVALID, "ed_project_out_noalloc: NULL argument");
    if (!h->s.built) return set_error(ED_ERR_NOT_BUILT, "ed_project_out_noalloc: basis not built");
    if ((dtype == ED_F64 || dtype == ED_F32) && !h->s.real)
        return set_error(ED_ERR_INVALID, "ed_project_out_noalloc: real dtype with a complex sector");
    return project_noalloc_launch(h->s, dtype, basis_dev, k, w_dev, coef_dev, (cudaStream_t)stream);
}

int ed_continued_fraction(const double* a_dev, const double* b_dev, int m, const double* omega_dev, int W, double e0,
                          double eta, double norm2, double* out_dev, void* stream) {
    if (!a_dev || !b_dev || !omega_dev || !out_dev) return set_error(ED_ERR_INVALID, "ed_continued_fraction: NULL");
    return cf_launch(a_dev, b_dev, m, omega_dev, W, e0, eta, norm2, out_dev, (cudaStream_t)stream);
}

}  // extern "C"
