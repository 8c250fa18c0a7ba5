/*
 * exactdiag_gb300.h -- C ABI of the GB300 t-J ladder engine (libexactdiag_gb300.so).
 *
 * The engine replaces four native pieces of exactdiag's hot path; each entry
 * point below names the reference interface it stands in for (paths inside
 * the reference project).  Conventions:
 *   - every function returns an int status: ED_OK (0) or a negative ED_ERR_*;
 *     ed_last_error_string() gives a thread-local description;
 *   - no exception, C++ type or torch type crosses this boundary;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream);
 *   - pointers named *_dev are device memory owned by the caller; *_host are host memory;
 *   - vectors are indexed by the dense basis index, i.e. in the reference's
 *     own order (ascending sparse index, general/basis_indexing.h:188-242).
 */
#ifndef EXACTDIAG_GB300_H
#define EXACTDIAG_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ED_OK 0
#define ED_ERR_INVALID (-1)   /* bad argument */
#define ED_ERR_NOMEM (-2)     /* device allocation failed */
#define ED_ERR_CUDA (-3)      /* CUDA runtime error */
#define ED_ERR_NOT_BUILT (-4) /* ed_basis_build has not run */
#define ED_ERR_TOO_LARGE (-5) /* sector exceeds a supported table size */
#define ED_ERR_INTERNAL (-6)  /* an internal consistency check failed */
#define ED_ERR_TIMEOUT (-7)   /* a bounded device-side wait gave up */

/* Arithmetic types of the vectors passed to the operator entry points. */
#define ED_F64 0 /* double, real sectors (k_x in {0, L/2}) */
#define ED_C128 1 /* interleaved complex double */
#define ED_F32 2 /* float, real sectors */
#define ED_C64 3 /* interleaved complex float */

typedef struct ed_sector ed_sector;

/* Sector of the periodic two-leg ladder: L rungs (2..16), Nh holes, Nd down
 * spins, leg momentum kx (any integer, taken mod L) and rung parity ky (0/1).
 * L = 1 is refused with ED_ERR_INVALID: its periodic leg bond would join a
 * site to itself.  A sector without representatives is valid (n = 0).
 * Stands in for Hamiltonian_Config.get_translators()
 * (tJ_spin_half_ladder/matrix_setup.pyx:377-406), which builds
 * State_Index_Amplitude_Translator (symmetry_ladder.h:271-406) and
 * Symmetries_Single_Spin_Half_2leg_Ladder (symmetry_ladder.h:55-269). */
int ed_sector_create(int L, int Nh, int Nd, int kx, int ky, ed_sector** out);
/* Frees the sector (and the kept ed_batch_lanczos workspace when it holds this sector). */
int ed_sector_destroy(ed_sector* s);

/* Enumerates the representatives on the device.  Replaces get_basis_map /
 * calc_basis_map (general/basis_indexing.h:188-261). Synchronises `stream`. */
int ed_basis_build(ed_sector* s, void* stream);

/* Launch configuration of the fused Lanczos step (tuning; no reference counterpart):
 * min_ctas_per_sm selects the compiled variant of the free-row kernel (2, 3 or 4 resident CTAs per
 * SM, i.e. a register budget of 128, 80 or 64 per thread) and ctas_per_sm the persistent grid (0 =
 * as many as fit).  exactdiag_gb300.autotune times the candidates and caches the fastest per sector
 * shape.  Results do not depend on these two. */
int ed_sector_set_launch(ed_sector* s, int min_ctas_per_sm, int ctas_per_sm);
int ed_sector_get_launch(const ed_sector* s, int* min_ctas_per_sm, int* grid);

/* Work shape of the free-row kernel (tuning; no reference counterpart): rows_per_lane, the rows of
 * a segment each lane works on together (1 or 2; 0 = two for FP32 vectors, one for FP64), and
 * chunk_rows, the rows of one chunk of work (a power of two in [1024, 65536]; default 16384).  The
 * rows per lane do not change results; a new chunk length re-plans the sector, and since the step's
 * partial sums are kept per chunk, its recursions then differ in the last bits (a sector still gives
 * the same bits alone and in a batch).  staged_gathers = 1 sends the free-row kernel's gathers through
 * shared memory (cp.async; results unchanged, at most two CTAs per SM; 32-offset segment windows
 * only).  ED_ERR_INVALID for values out of range.  Call it between steps: a new chunk length replaces
 * the sector's step tables. */
int ed_sector_set_step_shape(ed_sector* s, int rows_per_lane, int chunk_rows, int staged_gathers);
int ed_sector_get_step_shape(const ed_sector* s, int* rows_per_lane, int* chunk_rows, int* staged_gathers);

/* Offsets of a segment chunk's window (tuning; no reference counterpart): 32 (default; a lane's two
 * rows lie in two segments at the same offset, which keeps the lanes busier on segments whose length
 * is not a multiple of 64) or 64 (a lane's two rows lie 32 offsets apart in one segment).  Like a new
 * chunk length, a new window re-plans the sector and changes the last bits of its recursions (the
 * same alone and in a batch).  ED_ERR_INVALID for other values, and for 64 while staged gathers are
 * set.  Call it between steps. */
int ed_sector_set_segment_window(ed_sector* s, int offsets);
int ed_sector_get_segment_window(const ed_sector* s, int* offsets);

/* Chunks of the sector's fused step per row kind: counts[0] chunks of rows of blocks with a
 * trivial stabiliser (colex-delta rows), counts[1] chunks of rows of blocks with a small
 * stabiliser (coset candidates + bitmap), counts[2] chunks of rows taking the orbit walk.  Each non-zero count is one
 * kernel launch per step.  No reference counterpart (a property of this engine's layout). */
int ed_sector_row_kinds(const ed_sector* sector, int counts[3]);

/* Rows of the sector per row kind, in the order of ed_sector_row_kinds. */
int ed_sector_kind_rows(const ed_sector* sector, int64_t rows[3]);

/* Kernel launches of one ed_lanczos_step on this sector: the expanded copies (when the sector has
 * any), one fused H.v kernel per row kind present, the scalar reduction and the four launches of the
 * update.  No reference counterpart (a property of this engine's step). */
int ed_sector_step_launches(const ed_sector* sector, int* launches);

/* Number of representatives (Basis_Index_Map::get_num_states, basis_indexing.h:180-182). */
int ed_basis_size(const ed_sector* s, int64_t* n);

/* 1 if the sector's matrix elements are real (k_x*2 = 0 mod L), else 0. */
int ed_sector_is_real(const ed_sector* s, int* is_real);

/* Writes the basis in the reference's format: dense_to_sparse (int64 sparse
 * index) and num_sparse_states_in_dense (int32 orbit size), device arrays of
 * length n (Basis_Index_Map fields, basis_indexing.h:31-46, saved layout :128-146). */
int ed_basis_export(const ed_sector* s, int64_t* sparse_dev, int32_t* orbit_dev, void* stream);

/* y = H x with H = sum_t weights[t] * term_t, t in (tl, tr, jl, jr), applied
 * matrix-free and pull-style (no atomics, deterministic).  Replaces
 * Added_Sparse_Matrices.dot (general/sparse_matrices.py:233-237) ->
 * sparse_matrix_dot (general/cython_sparse_dot.pyx:40-80) over the terms built
 * by setup_hamiltonian (tJ_spin_half_ladder/matrix_setup.pyx:41-129).
 * dtype is ED_F64/ED_C128/ED_F32/ED_C64; real dtypes require a real sector. */
int ed_hv(const ed_sector* s, const double weights[4], int dtype, const void* x_dev, void* y_dev, void* stream);

/* H x by one of two independent row algorithms, as self-checks of ed_hv (which runs the fused
 * step kernels: segments of free blocks, expanded copies of stabiliser blocks): mode 0 one thread
 * per row with per-block descriptors (colex-rank deltas inside blocks whose hole pattern has a
 * trivial stabiliser, precomputed coset permutations elsewhere); mode 1 every term through the
 * reference-faithful orbit walk (get_symmetry_states_from_state, symmetry_ladder.h:113-235).  All
 * three give the same operator; mode 1 checks the others at sizes the CPU oracle cannot reach. */
int ed_hv_mode(const ed_sector* s, const double weights[4], int dtype, const void* x_dev, void* y_dev, int mode,
               void* stream);

/* One Lanczos step of the spectrum recursion
 * (general/cython_lanczos_diagonalization.pyx:68-77 _lanczos_vec_iteration):
 *   w = H v_k,  a_k = Re<v_k, w>,  v' = w - a_k v_k - b_k v_{k-1},
 *   b_{k+1} = |v'|,  v_{k+1} = v' / b_{k+1}.
 * scal_dev is a device double array: scal_dev[0] = b_k (read), on return
 * scal_dev[1] = a_k and scal_dev[2] = b_{k+1} (written on the device; nothing is
 * copied to the host, so the call can be captured in a CUDA graph).  v_prev may
 * be NULL (b_k ignored).  v_next receives v_{k+1}; it may alias v_prev.  The
 * products are accumulated in FP64 whatever dtype is.  When b_{k+1} < 1e-8
 * (the reference's breakdown test, :63-64) v_next is left as v' unnormalised
 * and scal_dev[3] is set to 1.  ed_lanczos_step, ed_lanczos_hv,
 * ed_lanczos_update and ed_normalize refuse an empty sector (n = 0) with
 * ED_ERR_INVALID; ed_hv, ed_hv_mode and ed_accumulate do nothing on one. */
int ed_lanczos_step(const ed_sector* s, const double weights[4], int dtype, const void* v_dev, const void* v_prev_dev,
                    void* v_next_dev, double* scal_dev, void* stream);

/* The two halves of ed_lanczos_step, for callers that time or interleave them:
 * ed_lanczos_hv writes y = H v - b_k v_prev into v_next_dev and a_k, b_{k+1} into
 * scal_dev[1..3]; ed_lanczos_update then forms v_{k+1} = (y - a_k v) / b_{k+1} in place. */
int ed_lanczos_hv(const ed_sector* s, const double weights[4], int dtype, const void* v_dev, const void* v_prev_dev,
                  void* v_next_dev, double* scal_dev, void* stream);
int ed_lanczos_update(const ed_sector* s, int dtype, const void* v_dev, void* v_next_dev, const double* scal_dev,
                      void* stream);

/* acc += (coef_re + i coef_im) * x, with acc in FP64 (double for real dtypes,
 * interleaved complex double otherwise) and x of the given dtype.  Builds Ritz
 * vectors sum_k s_k v_k of a Lanczos run in FP64 (the refinement input). */
int ed_accumulate(const ed_sector* s, int dtype, const void* x_dev, double coef_re, double coef_im, void* acc_dev,
                  void* stream);

/* acc += sum_j (coefs[2j] + i coefs[2j+1]) * x_devs[j] for j < k in one pass over acc (x_devs and
 * coefs are host arrays of k device pointers and 2k doubles): the same bits as k calls of
 * ed_accumulate in that order, with acc read and written once per 32 vectors instead of once per
 * vector.  ED_ERR_INVALID for k < 0, a NULL vector or a non-finite coefficient. */
int ed_accumulate_many(const ed_sector* s, int dtype, int k, const void* const* x_devs, const double* coefs,
                       void* acc_dev, void* stream);

/* Scales x in place to unit norm (FP64 accumulation); norm written to norm_dev[0]. */
int ed_normalize(const ed_sector* s, int dtype, void* x_dev, double* norm_dev, void* stream);

/* Continued fraction S(w) = -(1/pi) * norm2 * Im[1 / (z - a_0 - b_1^2/(z - a_1 - ...))],
 * z = omega + e0 + i*eta, evaluated bottom-up for every omega
 * (general/cython_lanczos_diagonalization.pyx:42-48, :36-39 and
 * general/lanczos_diagonalization.py:158-175).  a_dev[m], b_dev[m] (b[0]
 * unused), omega_dev[W], out_dev[W]: device doubles. */
int ed_continued_fraction(const double* a_dev, const double* b_dev, int m, const double* omega_dev, int W, double e0,
                          double eta, double norm2, double* out_dev, void* stream);

/* Applies an excitation operator from sector src (initial, e.g. the ground
 * state's) into sector dst: y = O x, pull-style over the rows of dst.
 *   op 0: Szq = sum_r (1/2sqrt(N)) e^{-iq.r} S^z_r
 *         (tJ_spin_half_ladder/matrix_setup.pyx:235-246; dst has the same Nh, Nd)
 *   op 1: spectral_function_minus = sum_r (1/sqrt(N)) e^{-iq.r} c_{r,sigma},
 *         sigma = down if initial_sz2 <= 0 else up (matrix_setup.pyx:302-325;
 *         dst has Nh+1 holes and the removed spin)
 *   op 2: spectral_function_plus = sum_r (1/sqrt(N)) e^{-iq.r} c^+_{r,sigma},
 *         sigma = down if initial_sz2 > 0 else up (matrix_setup.pyx:281-300;
 *         dst has Nh-1 holes and the added spin)
 *   op 3: current_rung = sum_r i e^{-iq'.r} c^+_{r'} c_r, r' the rung partner,
 *         q' = (qx, qy+1) (matrix_setup.pyx:248-263; dst has the same Nh, Nd)
 *   op 4: current_leg = sum_r i e^{-iq.r} (c^+_{r+x} c_r - c^+_{r-x} c_r)
 *         (matrix_setup.pyx:265-279; dst has the same Nh, Nd)
 * (qx, qy) are the operator quantum numbers as the matrix setup receives them;
 * dst must be the sector the reference's target rule gives (matrix_setup.pyx:329-330,
 * with q_y raised by one for current_rung).
 * Vectors are complex: dtype ED_C128 or ED_C64, x of length n(src), y of n(dst).
 * Replaces setup_excitation_operator's stored matrix and its .dot. */
int ed_excitation_apply(const ed_sector* src, const ed_sector* dst, int op, int qx, int qy, int initial_sz2, int dtype,
                        const void* x_src_dev, void* y_dst_dev, void* stream);

/* Position correlations of a state psi of the sector (device vector of n entries, dtype as for
 * ed_hv), distances 0..N-1 written to out_host[N] (host memory; the call synchronises `stream`):
 *   kind 0, hole correlations: sum_i |psi_i|^2 sum_r [holes at r, rel(r, dist) and every fixed shift of r]
 *   kind 1, S^z correlations:  the same with the product of the spin signs (0 if any site is a hole)
 * fixed_shifts holds nfixed (leg, rung) pairs (at most 4), the fixed_distances of the config.
 * Replaces tJ_spin_half_ladder/position_correlations.pyx:83-118 and :174-207 for one state. */
int ed_position_correlations(const ed_sector* sector, int dtype, const void* psi_dev, int kind, int nfixed,
                             const int* fixed_shifts, double* out_host, void* stream);

/* Singlet-singlet correlations of a state psi (dtype ED_F64 or ED_C128): out_host[t] =
 * Re <psi| O(t) |psi> for t = 0..N-1, O(t) the singlet-pair operator of
 * tJ_spin_half_ladder/matrix_setup.pyx:434-469 with fixed distances
 * fixed_shifts = {y leg, y rung, x leg, x rung} and free shift (t / 2, t % 2), columns by the
 * reference's column rule.  Replaces position_correlations.pyx:112-124 for one state. */
int ed_singlet_correlations(const ed_sector* sector, int dtype, const void* psi_dev, const int fixed_shifts[4],
                            double* out_host, void* stream);

/* Runs the spectrum Lanczos recursion (general/cython_lanczos_diagonalization.pyx:50-77)
 * for nsec sectors together: m steps each from the start vectors v0_dev[s]
 * (device pointers, dtype, any norm), all sectors' rows handled by one launch per
 * phase and the m steps captured in one CUDA graph (use_graph != 0).  The
 * sectors must share L, Nh and Nd.  coef_dev holds nsec * (2m+4) doubles
 * (device); sector s's block X: X[2k+1] = a_k, X[2k+2] = b_{k+1}, X[2m+3] = |v0|.
 * The caller truncates after the first b_{k+1} < 1e-8.  Synchronises `stream`.
 * The workspace (two vectors per sector, chunk tables, scratch) and the captured
 * graph are kept after the call for the next call with the same sectors in the
 * same order, dtype, m, weights, use_graph and launch shape; one such workspace
 * is kept per process, replaced by a call of another shape and freed when one of
 * its sectors is destroyed.  Calls are serialised by a lock.
 * Replaces the per-q loop of tJ_spin_half_ladder/api.py:116-161 over
 * general/lanczos_diagonalization.py:124-175. */
int ed_batch_lanczos(const ed_sector* const* sectors, int nsec, const double weights[4], int dtype,
                     const void* const* v0_dev, int m, double* coef_dev, int use_graph, void* stream);

/* w <- w - sum_{j<k} <v_j, w> v_j for k vectors stored contiguously in basis_dev
 * (k x n, dtype), dot products in FP64 (classical Gram-Schmidt; call twice for
 * full reorthogonalisation).  coef_dev (device, 2k doubles, may be NULL)
 * receives the coefficients <v_j, w> as (re, im) pairs.  The first call with a
 * larger k grows a per-sector scratch buffer (a device allocation). */
int ed_project_out(ed_sector* s, int dtype, const void* basis_dev, int k, void* w_dev, double* coef_dev, void* stream);

/* The same projection as ed_project_out, allocating nothing.  No counterpart in the
 * reference.  ed_project_out grows a per-sector scratch buffer with cudaMalloc on its first
 * call with a larger k, which some callers cannot allow: services that run under a fixed
 * device-memory budget or hand all device memory to their own allocator, and callers that may
 * not synchronise the device in the middle of their work (cudaMalloc can).  This variant keeps
 * its scratch (per-chunk partial dot products and the coefficients) in one fixed device array
 * of 2.1 MB that every GPU loading the library holds until the process exits; k is limited to
 * 256 vectors (ED_ERR_TOO_LARGE above).  Each call looks up the array's address in the current
 * device's context (a host-side query) and must be made with the sector's device current
 * (ED_ERR_INVALID otherwise).  All calls share the array: calls that overlap on the GPU (other
 * streams or threads) race.  coef_dev as in ed_project_out. */
int ed_project_out_noalloc(const ed_sector* s, int dtype, const void* basis_dev, int k, void* w_dev, double* coef_dev,
                           void* stream);

/* Thread-local description of the last error. */
const char* ed_last_error_string(void);

#ifdef __cplusplus
}
#endif

#endif /* EXACTDIAG_GB300_H */
