/*
 * ed_oracle.c -- CPU oracle for the t-J ladder path
 *     basis enumeration -> matrix elements of H and of the excitation operators.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The
 * GPU product path (exactdiag_gb300/csrc) does not link or call it.
 *
 * It restates, in plain C and one function per reference function, the
 * algorithm of exactdiag's C++ headers and Cython rule tables.  It keeps the
 * reference's own data representation (one int16 value per site, per-site
 * loops, complex<double> cumulative phases, bsearch over the sorted basis) so
 * that it is an independent check of the bit-level GPU kernels.
 *
 * Citations are paths inside the reference project (src/exactdiag/...).
 * Parity of this file is pinned against (a) the reference's 68 basis-size and
 * 51 eigenvalue fixtures and (b) the reference's own C++ headers compiled
 * unmodified into oracle/_ref (see oracle/Makefile, oracle/ref_driver.cpp).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAXN 32

typedef int16_t st_t; /* general/types_and_constants.h:10 (state_int = short) */
enum { HOLE = 0, DOWN = 1, UP = 2 }; /* general/types_and_constants.h:14-16 */

typedef struct {
    int L, N, Nh, Nd, Ns;
    int kx, ky;
    int64_t comb[OR_MAXN + 1][OR_MAXN + 1]; /* comb[k][n] = C(n, k) */
    int64_t n_spin;                         /* C(Ns, Nd) = num_spin_states */
    double complex rung_exp, mirror_exp;
} ors_t;

/* Error codes shared with the Python wrapper. */
#define OR_OK 0
#define OR_EINVAL (-1)
#define OR_ECAP (-2)
#define OR_ENOMEM (-3)

/* general/symmetry_utils.h:60-67 python_mod (divisor > 0 here). */
static int pmod(int a, int b) {
    int r = a % b;
    return r < 0 ? r + b : r;
}

/* general/matrix_rules_utils.pyx:122-134 set_combinatorics: comb[j,i] = C(i,j).
 * The reference builds it through float products and np.around, which is exact
 * for N <= 32; exact integer recursion gives the same table. */
static void fill_comb(ors_t *s) {
    memset(s->comb, 0, sizeof(s->comb));
    for (int n = 0; n <= OR_MAXN; ++n) {
        s->comb[0][n] = 1;
        for (int k = 1; k <= n; ++k)
            s->comb[k][n] = s->comb[k - 1][n - 1] + (k <= n - 1 ? s->comb[k][n - 1] : 0);
    }
}

static int sector_init(ors_t *s, int L, int Nh, int Nd, int kx, int ky) {
    if (L < 1 || 2 * L > OR_MAXN || Nh < 0 || Nh > 2 * L || Nd < 0 || Nd > 2 * L - Nh || ky < 0 || ky > 1)
        return OR_EINVAL;
    s->L = L;
    s->N = 2 * L;
    s->Nh = Nh;
    s->Nd = Nd;
    s->Ns = s->N - Nh;
    s->kx = kx;
    s->ky = ky;
    fill_comb(s);
    s->n_spin = s->comb[Nd][s->Ns];
    /* tJ_spin_half_ladder/symmetry_ladder.h:134-138 */
    const double two_pi = 2.0 * 3.14159265358979323846;
    s->mirror_exp = cexp(-I * two_pi * ((double)ky / 2.0));
    s->rung_exp = cexp(-I * two_pi * ((double)kx / (double)L));
    return OR_OK;
}

/* general/group/commutation_counter.h:45-69 State_Hierarchy::check_lower_state
 * with hierarchy {HOLE, DOWN, UP}: 0 equal, 1 state1 lower, 2 state2 lower. */
static int check_lower_state(const st_t *s1, const st_t *s2, int n) {
    static const st_t hier[2] = {HOLE, DOWN};
    for (int k = 0; k < 2; ++k) {
        for (int j = 0; j < n; ++j) {
            int i = n - 1 - j;
            int a = (s2[i] == hier[k]), b = (s1[i] == hier[k]);
            if (a && !b) return 1;
            if (!a && b) return 2;
        }
    }
    return 0;
}

static int states_equal(const st_t *a, const st_t *b, int n) { return memcmp(a, b, (size_t)n * sizeof(st_t)) == 0; }

/* tJ_spin_half_ladder/symmetry_ladder.h:113-235
 * Symmetries_Single_Spin_Half_2leg_Ladder::get_symmetry_states_from_state.
 * Writes up to N images into imgs/amps; returns the number found or 0. */
static int orbit(const ors_t *s, const st_t *state, int check_lowest, st_t imgs[][OR_MAXN], double complex *amps) {
    const int N = s->N, L = s->L;
    st_t rep[2 * OR_MAXN], mrep[2 * OR_MAXN];
    int ne_even = 1; /* num_spins_less_one_odd */
    int paired = 0;
    for (int i = 0; i < N; ++i) {
        st_t v = state[i];
        paired += (i % 2 == 0) && (v != HOLE) && (state[i + 1] != HOLE);
        ne_even ^= (v != HOLE);
    }
    double complex mirror_fac = s->mirror_exp * (double complex)(paired % 2 == 0 ? 1 : -1);
    double complex rung_amp = 1.0;
    int mirror_symmetric = 0;

    memcpy(imgs[0], state, (size_t)N * sizeof(st_t));
    amps[0] = 1.0;
    memcpy(rep, state, (size_t)N * sizeof(st_t));
    memcpy(rep + N, state, (size_t)N * sizeof(st_t));
    for (int i = 0; i < N; i += 2) {
        mrep[i] = state[i + 1];
        mrep[i + 1] = state[i];
    }
    memcpy(mrep + N, mrep, (size_t)N * sizeof(st_t));

    int found = 1;
    /* general/cpp_classes.h:14-105 Product_Generator over periodicities {L, 2}
     * starting at iteration 1: symmetry_indices = {p/2 % L, p % 2}. */
    for (int p = 1; p < N; ++p) {
        int sx = (p / 2) % L;
        const st_t *tr;
        double complex amp;
        if (p % 2 == 1) {
            if (mirror_symmetric) continue;
            tr = &mrep[N - 2 * sx];
            amp = rung_amp * mirror_fac;
        } else {
            tr = &rep[N - 2 * sx];
            rung_amp *= s->rung_exp;
            if (ne_even && ((tr[0] == HOLE) ^ (tr[1] == HOLE))) rung_amp *= -1.0;
            amp = rung_amp;
        }
        if (check_lowest && check_lower_state(state, tr, N) == 2) return 0;
        const double eps = 1e-8;
        if (sx < L / 2 + 1) {
            if (states_equal(imgs[0], tr, N)) {
                if (cabs(amp - 1.0) > eps) return 0;
                if (p == 1) {
                    mirror_symmetric = 1;
                    continue;
                }
                break;
            }
            if (found != 1 && states_equal(imgs[1], tr, N)) {
                if (cabs(amp - amps[1]) > eps) return 0;
                break;
            }
        }
        memcpy(imgs[found], tr, (size_t)N * sizeof(st_t));
        amps[found] = amp;
        found += 1;
    }
    double norm = sqrt((double)found);
    for (int i = 0; i < found; ++i) amps[i] /= norm;
    return found;
}

/* tJ_spin_half_ladder/symmetry_ladder.h:314-344 sparse_index_to_state. */
static void sparse_index_to_state(const ors_t *s, int64_t sparse, st_t *state) {
    int rh = s->Nh, rs = s->Nd;
    int64_t hole_ind = sparse / s->n_spin;
    int64_t spin_ind = sparse - hole_ind * s->n_spin;
    for (int j = s->N - 1; j >= 0; --j) {
        if (rh > 0) {
            int64_t cost = s->comb[rh][j];
            if (hole_ind >= cost) {
                state[j] = HOLE;
                rh -= 1;
                hole_ind -= cost;
                continue;
            }
        }
        if (rs > 0) {
            int64_t cost = (j - rh >= 0) ? s->comb[rs][j - rh] : 0;
            if (spin_ind >= cost) {
                state[j] = DOWN;
                rs -= 1;
                spin_ind -= cost;
                continue;
            }
        }
        state[j] = UP;
    }
}

/* tJ_spin_half_ladder/symmetry_ladder.h:346-361 state_to_sparse_index. */
static int64_t state_to_sparse_index(const ors_t *s, const st_t *state) {
    int64_t hole_index = 0, spin_index = 0;
    int ah = (state[0] == HOLE), ad = (state[0] == DOWN);
    for (int i = 1; i < s->N; ++i) {
        if (state[i] == HOLE) {
            ah += 1;
            hole_index += s->comb[ah][i];
        } else if (state[i] == DOWN) {
            ad += 1;
            spin_index += s->comb[ad][i - ah];
        }
    }
    return spin_index + hole_index * s->n_spin;
}

/* tJ_spin_half_ladder/symmetry_ladder.h:363-405
 * check_major_index_supports_lowest_states + find_hole_positions. */
static int64_t check_major_index(const ors_t *s, int64_t hole_index) {
    const int N = s->N;
    if (s->Nh <= 1 || s->Nh >= N - 1) return hole_index == 0 ? 0 : -1;
    st_t state[OR_MAXN];
    for (int i = 0; i < N; ++i) state[i] = UP;
    int rh = s->Nh;
    int64_t t = hole_index;
    for (int j = N - 1; j >= 0 && rh > 0; --j) {
        int64_t cost = s->comb[rh][j];
        if (t >= cost) {
            state[j] = HOLE;
            rh -= 1;
            t -= cost;
        }
    }
    for (int i = 0; i < N; ++i) {
        if (state[i] == UP) {
            state[i] = DOWN;
            break;
        }
    }
    st_t imgs[OR_MAXN][OR_MAXN];
    double complex amps[OR_MAXN];
    return orbit(s, state, 1, imgs, amps) > 0 ? hole_index : -1;
}

/* general/symmetry.h:97-126 get_lowest_sparse_amplitude_from_state. */
static void lowest_sparse_amplitude(const ors_t *s, const st_t *state, int64_t *ind, double complex *amp) {
    st_t imgs[OR_MAXN][OR_MAXN];
    double complex amps[OR_MAXN];
    int n = orbit(s, state, 0, imgs, amps);
    if (n == 0) {
        *ind = -1;
        *amp = 0;
        return;
    }
    int low = 0;
    for (int i = 1; i < n; ++i)
        if (check_lower_state(imgs[low], imgs[i], s->N) == 2) low = i;
    *ind = state_to_sparse_index(s, imgs[low]);
    *amp = amps[low];
}

/* general/basis_indexing.h:152-168 Basis_Index_Map::get_dense (bsearch). */
static int64_t get_dense(const int64_t *d2s, int64_t n, int64_t sparse) {
    if (sparse < 0) return -1;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (d2s[mid] < sparse) lo = mid + 1;
        else hi = mid;
    }
    return (lo < n && d2s[lo] == sparse) ? lo : -1;
}

/* ------------------------------------------------------------------------ */
/* Basis: general/basis_indexing.h:188-242 calc_basis_map and
 * general/symmetry.h:56-81 get_lowest_sparse_indices_from_major_index.      */

typedef struct {
    int64_t *idx;
    int32_t *cnt;
    int64_t n;
} hole_chunk_t;

int or_basis_build(int L, int Nh, int Nd, int kx, int ky, int64_t *out_sparse, int32_t *out_orbit, int64_t cap,
                   int64_t *n_out) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, kx, ky) != OR_OK) return OR_EINVAL;
    int64_t n_major = s.comb[Nh][s.N];
    int64_t *elig = (int64_t *)malloc((size_t)n_major * sizeof(int64_t));
    if (!elig) return OR_ENOMEM;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t h = 0; h < n_major; ++h) elig[h] = check_major_index(&s, h);
    int64_t ne = 0;
    for (int64_t h = 0; h < n_major; ++h)
        if (elig[h] != -1) elig[ne++] = elig[h];
    hole_chunk_t *ch = (hole_chunk_t *)calloc((size_t)(ne > 0 ? ne : 1), sizeof(hole_chunk_t));
    int failed = 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t e = 0; e < ne; ++e) {
        int64_t start = elig[e] * s.n_spin, end = start + s.n_spin;
        int64_t *idx = (int64_t *)malloc((size_t)(s.n_spin > 0 ? s.n_spin : 1) * sizeof(int64_t));
        int32_t *cnt = (int32_t *)malloc((size_t)(s.n_spin > 0 ? s.n_spin : 1) * sizeof(int32_t));
        if (!idx || !cnt) {
            failed = 1;
            free(idx);
            free(cnt);
            continue;
        }
        int64_t k = 0;
        st_t state[OR_MAXN];
        st_t imgs[OR_MAXN][OR_MAXN];
        double complex amps[OR_MAXN];
        for (int64_t i = start; i < end; ++i) {
            sparse_index_to_state(&s, i, state);
            int nf = orbit(&s, state, 1, imgs, amps);
            if (nf != 0) {
                idx[k] = i;
                cnt[k] = nf;
                k += 1;
            }
        }
        ch[e].idx = idx;
        ch[e].cnt = cnt;
        ch[e].n = k;
    }
    int64_t total = 0;
    for (int64_t e = 0; e < ne; ++e) total += ch[e].n;
    int rc = OR_OK;
    if (failed) rc = OR_ENOMEM;
    else if (out_sparse && total > cap) rc = OR_ECAP;
    else if (out_sparse) {
        int64_t off = 0;
        for (int64_t e = 0; e < ne; ++e) {
            memcpy(out_sparse + off, ch[e].idx, (size_t)ch[e].n * sizeof(int64_t));
            if (out_orbit) memcpy(out_orbit + off, ch[e].cnt, (size_t)ch[e].n * sizeof(int32_t));
            off += ch[e].n;
        }
    }
    for (int64_t e = 0; e < ne; ++e) {
        free(ch[e].idx);
        free(ch[e].cnt);
    }
    free(ch);
    free(elig);
    *n_out = total;
    return rc;
}

/* Eligible hole ranks (loop 1 of calc_basis_map); returns count. */
int or_eligible_hole_ranks(int L, int Nh, int Nd, int kx, int ky, int64_t *out, int64_t cap, int64_t *n_out) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, kx, ky) != OR_OK) return OR_EINVAL;
    int64_t n_major = s.comb[Nh][s.N], k = 0;
    for (int64_t h = 0; h < n_major; ++h) {
        if (check_major_index(&s, h) != -1) {
            if (out && k < cap) out[k] = h;
            k++;
        }
    }
    *n_out = k;
    return (out && k > cap) ? OR_ECAP : OR_OK;
}

/* sparse index <-> per-site state (exported for tests). */
int or_sparse_to_state(int L, int Nh, int Nd, int64_t sparse, int16_t *state) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, 0, 0) != OR_OK) return OR_EINVAL;
    sparse_index_to_state(&s, sparse, state);
    return OR_OK;
}

int64_t or_state_to_sparse(int L, int Nh, int Nd, const int16_t *state) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, 0, 0) != OR_OK) return OR_EINVAL;
    return state_to_sparse_index(&s, state);
}

/* Orbit of one state (exported for tests): returns num_found, fills the
 * lowest image's sparse index and amplitude. */
int or_orbit_lowest(int L, int Nh, int Nd, int kx, int ky, const int16_t *state, int64_t *ind, double *amp_re,
                    double *amp_im) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, kx, ky) != OR_OK) return OR_EINVAL;
    st_t imgs[OR_MAXN][OR_MAXN];
    double complex amps[OR_MAXN];
    int n = orbit(&s, state, 0, imgs, amps);
    double complex a;
    lowest_sparse_amplitude(&s, state, ind, &a);
    *amp_re = creal(a);
    *amp_im = cimag(a);
    return n;
}

/* ------------------------------------------------------------------------ */
/* Matrix-element rules.                                                     */

typedef struct {
    int n;                   /* number of operator index combinations */
    int len;                 /* indices per combination (1 or 2) */
    int16_t idx[2 * OR_MAXN][4];
    double complex wd[2 * OR_MAXN], wo[2 * OR_MAXN];
} combos_t;

/* tJ_spin_half_ladder/symmetry_ladder.h:96-101 get_index_by_relative_shift. */
static int index_by_relative_shift(int N, int initial, int sx, int sy) {
    initial = pmod(initial, N);
    int leg = initial / 2 + sx;
    int rung = pmod(initial + (sy % 2), 2);
    return pmod(2 * leg + rung, N);
}

/* general/matrix_rules_utils.pyx:15-87 combinations_from_start_end_points
 * with startpoints = all sites, one shift per endpoint set, reverse=True;
 * general/matrix_rules_utils.pyx:136-148 Validator_Unique_Pairs.
 * validator: 0 none, 1 ordered unique, 2 unordered unique. */
static void make_pair_combos(int N, const int (*shifts)[2], int nshift, int validator, double wd, double wo,
                             combos_t *c) {
    c->n = 0;
    c->len = 2;
    int seen[4 * OR_MAXN][2];
    int nseen = 0;
    for (int first = 0; first < N; ++first) {
        for (int k = 0; k < nshift; ++k) {
            int end = index_by_relative_shift(N, first, shifts[k][0], shifts[k][1]);
            int pair[2] = {first, end};
            if (validator) {
                int dup = 0;
                for (int q = 0; q < nseen; ++q) {
                    if (seen[q][0] == pair[0] && seen[q][1] == pair[1]) dup = 1;
                    if (validator == 2 && seen[q][0] == pair[1] && seen[q][1] == pair[0]) dup = 1;
                }
                if (dup) continue;
                seen[nseen][0] = pair[0];
                seen[nseen][1] = pair[1];
                nseen++;
            }
            c->idx[c->n][0] = (int16_t)end; /* reversed: [end, start] */
            c->idx[c->n][1] = (int16_t)first;
            c->wd[c->n] = wd;
            c->wo[c->n] = wo;
            c->n++;
        }
    }
}

/* tJ_spin_half_ladder/matrix_setup.pyx:80-110 term table. term: 0 tl, 1 tr, 2 jl, 3 jr */
static void term_combos(int N, int term, combos_t *c) {
    static const int tl[2][2] = {{1, 0}, {-1, 0}};
    static const int tr[2][2] = {{0, 1}, {0, -1}};
    static const int jl[1][2] = {{1, 0}};
    static const int jr[1][2] = {{0, 1}};
    switch (term) {
    case 0: make_pair_combos(N, tl, 2, 0, 0.0, -1.0, c); break;
    case 1: make_pair_combos(N, tr, 2, 1, 0.0, -1.0, c); break;
    case 2: make_pair_combos(N, jl, 1, 0, -0.5, 0.5, c); break;
    default: make_pair_combos(N, jr, 1, 2, -0.5, 0.5, c); break;
    }
}

/* general/column_functions.h:317-346 count_commutations with counted_value
 * HOLE and compare_equals false, as used by
 * tJ_spin_half_ladder/matrix_element_functions.pyx:66-69 get_anticommutation_sign. */
static int anticommutation_sign(const st_t *state, int N, const int16_t *ind, int nind) {
    int op[OR_MAXN] = {0};
    for (int i = 0; i < N; ++i)
        if (state[i] != HOLE)
            for (int j = 0; j < i; ++j) op[j] += 1;
    int count = 0;
    for (int i = nind - 1; i >= 0; --i) {
        int index = ind[i];
        count += op[index];
        for (int j = 0; j < index; ++j) op[j] += 1;
    }
    return (count % 2) == 0 ? 1 : -1;
}

/* general/column_functions.h:48-60 add_matrix_element_to_results. */
static void add_elem(double complex v, int64_t index, double complex *vals, int64_t *inds, int *n) {
    for (int i = 0; i < *n; ++i)
        if (inds[i] == index) {
            vals[i] += v;
            return;
        }
    vals[*n] = v;
    inds[*n] = index;
    *n += 1;
}

/* general/column_functions.h:79-97 order_nonzero_value_index_pairs. */
static void order_nonzero(double complex *vals, int64_t *inds, int *n) {
    int m = 0;
    for (int i = 0; i < *n; ++i)
        if (cabs(vals[i]) >= 1e-8) {
            vals[m] = vals[i];
            inds[m] = inds[i];
            m++;
        }
    for (int i = 1; i < m; ++i) { /* insertion sort: indices are unique */
        int64_t ki = inds[i];
        double complex vi = vals[i];
        int j = i - 1;
        while (j >= 0 && inds[j] > ki) {
            inds[j + 1] = inds[j];
            vals[j + 1] = vals[j];
            j--;
        }
        inds[j + 1] = ki;
        vals[j + 1] = vi;
    }
    *n = m;
}

typedef enum {
    VAL_HOLE_HOP = 0,  /* matrix_element_functions.pyx:16-17 */
    VAL_SPIN_SWAP = 1, /* matrix_element_functions.pyx:19-22 */
    VAL_NO_HOLES = 2,  /* :25-30 */
    VAL_ALL_DOWN = 3,  /* :39-44 */
    VAL_ALL_UP = 4,    /* :32-37 */
    VAL_ALL_HOLES = 5, /* :46-51 */
    VAL_UNEQUAL_SPINS_2HOLES = 6, /* :53-62 */
} validator_t;

/* tJ_spin_half_ladder/matrix_element_functions.pyx: swap, dont_change, add_hole (:112-118),
 * add_spin_down (:98-103), add_spin_up (:105-110) */
typedef enum {
    NEW_SWAP = 0,
    NEW_KEEP = 1,
    NEW_ADD_HOLE = 2,
    NEW_ADD_DOWN = 3,
    NEW_ADD_UP = 4,
    NEW_REMOVE_TWO_ADD_UP_DOWN = 5, /* :120-130 */
} newstate_t;

typedef struct {
    const combos_t *c;
    validator_t valid;
    newstate_t gen;
    int use_sign;        /* get_anticommutation_sign */
    int spin_weights;    /* 1: get_weights_spin_projection (matrix_element_functions.pyx:71-82);
                          * 2: get_weights_annihilation_part_singlet_singlet (:84-95) */
    int triangle;        /* is_valid_indices_triangular (column_functions.h:71-73) */
    const ors_t *fin;    /* final-sector translator */
    const int64_t *fin_d2s;
    int64_t fin_n;
} rule_t;

static int is_valid(validator_t v, const st_t *st, const int16_t *ind, int len) {
    switch (v) {
    case VAL_HOLE_HOP: return st[ind[0]] == HOLE && st[ind[1]] != HOLE;
    case VAL_SPIN_SWAP: return st[ind[0]] != st[ind[1]] && st[ind[0]] != HOLE && st[ind[1]] != HOLE;
    case VAL_NO_HOLES:
        for (int i = 0; i < len; ++i)
            if (st[ind[i]] == HOLE) return 0;
        return 1;
    case VAL_ALL_DOWN:
        for (int i = 0; i < len; ++i)
            if (st[ind[i]] != DOWN) return 0;
        return 1;
    case VAL_ALL_HOLES:
        for (int i = 0; i < len; ++i)
            if (st[ind[i]] != HOLE) return 0;
        return 1;
    case VAL_UNEQUAL_SPINS_2HOLES: {
        if (ind[0] == ind[1]) return 0;
        const int h0 = ind[0] == ind[2] || ind[0] == ind[3] || st[ind[0]] == HOLE;
        const int h1 = ind[1] == ind[2] || ind[1] == ind[3] || st[ind[1]] == HOLE;
        const int sp = st[ind[2]] != st[ind[3]] && st[ind[2]] != HOLE && st[ind[3]] != HOLE;
        return h0 && h1 && sp;
    }
    default:
        for (int i = 0; i < len; ++i)
            if (st[ind[i]] != UP) return 0;
        return 1;
    }
}

/* general/column_functions.h:150-207 calc_column_matrix_elements with
 * commutes_with_symmetries = true and general/column_functions.h:99-148
 * add_generic_matrix_element for every combination (Lambda_Matrix_Elements, :271-285). */
static int column(const ors_t *ini, int64_t col, int64_t sparse, int orbit_size, const rule_t *r,
                  double complex *vals, int64_t *inds) {
    st_t st[OR_MAXN], ns[OR_MAXN];
    sparse_index_to_state(ini, sparse, st);
    int n = 0;
    double complex diag_w = 1.0, off_w = sqrt((double)orbit_size);
    const int N = ini->N;
    for (int k = 0; k < r->c->n; ++k) {
        const int16_t *ind = r->c->idx[k];
        double complex ed = diag_w * r->c->wd[k], eo = off_w * r->c->wo[k];
        if (!is_valid(r->valid, st, ind, r->c->len)) continue;
        if (r->spin_weights == 1) {
            double f = 1.0;
            for (int i = 0; i < r->c->len; ++i)
                if (st[ind[i]] == DOWN) f *= -1.0;
            ed *= f;
            eo *= f;
        } else if (r->spin_weights == 2 && st[ind[2]] == DOWN) {
            ed *= -1.0;
            eo *= -1.0;
        }
        if (cabs(ed) > 1e-8) add_elem(ed, col, vals, inds, &n);
        if (cabs(eo) < 1e-8) continue;
        memcpy(ns, st, (size_t)N * sizeof(st_t));
        if (r->gen == NEW_SWAP) {
            ns[ind[0]] = st[ind[1]];
            ns[ind[1]] = st[ind[0]];
        } else if (r->gen == NEW_ADD_HOLE || r->gen == NEW_ADD_DOWN || r->gen == NEW_ADD_UP) {
            const st_t v = r->gen == NEW_ADD_HOLE ? HOLE : (r->gen == NEW_ADD_DOWN ? DOWN : UP);
            for (int i = 0; i < r->c->len; ++i) ns[ind[i]] = v;
        } else if (r->gen == NEW_REMOVE_TWO_ADD_UP_DOWN) {
            /* the last index acts first: holes at 3 and 2, then up at 1, down at 0 (repeating) */
            static const st_t changes[4] = {HOLE, HOLE, UP, DOWN};
            for (int i = 0; i < r->c->len; ++i) ns[ind[r->c->len - 1 - i]] = changes[i % 4];
        }
        int64_t fs;
        double complex amp;
        lowest_sparse_amplitude(r->fin, ns, &fs, &amp);
        int64_t fd = get_dense(r->fin_d2s, r->fin_n, fs);
        if (fd < 0 || (r->triangle && !(col <= fd))) continue;
        double complex v = eo * amp;
        if (r->use_sign) v *= (double)anticommutation_sign(st, N, ind, r->c->len);
        add_elem(v, fd, vals, inds, &n);
    }
    order_nonzero(vals, inds, &n);
    return n;
}

/* Column-major sparse matrix of one rule over all columns: two passes
 * (count, then fill) so the result needs no per-column capacity guess. */
static int rule_columns(const ors_t *ini, const int64_t *d2s, const int32_t *orb, int64_t n, const rule_t *r,
                        int64_t *colptr, int64_t *rows, double *vre, double *vim, int64_t cap, int64_t *nnz_out) {
    int64_t *cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    if (!cnt) return OR_ENOMEM;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        double complex vals[4 * OR_MAXN + 2];
        int64_t inds[4 * OR_MAXN + 2];
        cnt[i + 1] = column(ini, i, d2s[i], orb[i], r, vals, inds);
    }
    for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    *nnz_out = cnt[n];
    if (colptr) memcpy(colptr, cnt, ((size_t)n + 1) * sizeof(int64_t));
    if (!rows) {
        free(cnt);
        return OR_OK;
    }
    if (cnt[n] > cap) {
        free(cnt);
        return OR_ECAP;
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        double complex vals[4 * OR_MAXN + 2];
        int64_t inds[4 * OR_MAXN + 2];
        int m = column(ini, i, d2s[i], orb[i], r, vals, inds);
        for (int k = 0; k < m; ++k) {
            rows[cnt[i] + k] = inds[k];
            vre[cnt[i] + k] = creal(vals[k]);
            vim[cnt[i] + k] = cimag(vals[k]);
        }
    }
    free(cnt);
    return OR_OK;
}

/* One Hamiltonian term (tl/tr/jl/jr) as the column-major matrix the
 * reference computes (tJ_spin_half_ladder/matrix_setup.pyx:132-192,
 * general/cython_sparse_matrices.pyx:186-241 before value deduplication).
 * triangle != 0 keeps only final >= initial, as the reference's default
 * triangle_only storage does.  Call with rows == NULL to get nnz. */
int or_term_columns(int L, int Nh, int Nd, int kx, int ky, int term, int triangle, const int64_t *d2s,
                    const int32_t *orb, int64_t n, int64_t *colptr, int64_t *rows, double *vre, double *vim,
                    int64_t cap, int64_t *nnz_out) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, kx, ky) != OR_OK || term < 0 || term > 3) return OR_EINVAL;
    combos_t c;
    term_combos(s.N, term, &c);
    rule_t r = {&c, term < 2 ? VAL_HOLE_HOP : VAL_SPIN_SWAP, NEW_SWAP, term < 2, 0, triangle, &s, d2s, n};
    return rule_columns(&s, d2s, orb, n, &r, colptr, rows, vre, vim, cap, nnz_out);
}

/* general/group/symmetry_generator.h:87-102 get_q_dot_r: the per-axis terms
 * are evaluated in single precision (int * int / float) before the sum. */
static double q_dot_r(int site, int qx, int qy, int L) {
    int sx = site / 2, sy = site % 2;
    double acc = 0.0;
    acc += (double)((float)(qx * sx) / (float)L);
    acc += (double)((float)(qy * sy) / 2.0f);
    return acc * 2.0 * 3.14159265358979323846;
}

/* Excitation operators (tJ_spin_half_ladder/matrix_setup.pyx:195-374):
 *   op 0: Szq (:235-246), op 1: spectral_function_minus (:302-325),
 *   op 2: spectral_function_plus (:281-300), op 3: current_rung (:248-263),
 *   op 4: current_leg (:265-279).
 * (qx, qy) are operator_symmetry_qs as the matrix setup receives them.
 * The final sector (L, Nh2, Nd2, kx2, ky2) and its basis are given by the
 * caller (the target-sector rule is in the Python wrapper). */
int or_excitation_columns(int op, int L, int Nh, int Nd, int kx, int ky, int Sz2, const int64_t *d2s,
                          const int32_t *orb, int64_t n, int Nh2, int Nd2, int kx2, int ky2, const int64_t *fd2s,
                          int64_t fn, int qx, int qy, int64_t *colptr, int64_t *rows, double *vre, double *vim,
                          int64_t cap, int64_t *nnz_out) {
    ors_t s, f;
    if (sector_init(&s, L, Nh, Nd, kx, ky) != OR_OK) return OR_EINVAL;
    if (sector_init(&f, L, Nh2, Nd2, kx2, ky2) != OR_OK) return OR_EINVAL;
    combos_t c;
    if (op == 3 || op == 4) {
        /* matrix_rules_utils.pyx:15-87 with startpoints = all sites, reverse=True: [end, start];
         * startpoint weights (0, i) exp(-i q.r_start) (:90-119), endpoint weights (0, 1) and, for the
         * leg's second shift, (0, -1).  current_rung raises q_y by one first (matrix_setup.pyx:251). */
        const int qye = op == 3 ? qy + 1 : qy;
        static const int rung[1][2] = {{0, 1}};
        static const int leg[2][2] = {{1, 0}, {-1, 0}};
        const int (*sh)[2] = op == 3 ? rung : leg;
        const int nsh = op == 3 ? 1 : 2;
        c.n = 0;
        c.len = 2;
        for (int first = 0; first < s.N; ++first) {
            const double complex sw = I * cexp(-I * q_dot_r(first, qx, qye, L));
            for (int k = 0; k < nsh; ++k) {
                const int end = index_by_relative_shift(s.N, first, sh[k][0], sh[k][1]);
                c.idx[c.n][0] = (int16_t)end;
                c.idx[c.n][1] = (int16_t)first;
                c.wd[c.n] = 0.0 * sw;
                c.wo[c.n] = (k == 0 ? 1.0 : -1.0) * sw;
                c.n++;
            }
        }
    } else {
        c.n = s.N;
        c.len = 1;
        double base = (op == 0) ? 0.5 / sqrt((double)s.N) : 1.0 / sqrt((double)s.N);
        for (int i = 0; i < s.N; ++i) {
            c.idx[i][0] = (int16_t)i;
            double complex ph = cexp(-I * q_dot_r(i, qx, qy, L)); /* matrix_rules_utils.pyx:90-119 */
            c.wd[i] = 0.0 * ph;
            c.wo[i] = base * ph;
        }
    }
    rule_t r;
    r.c = &c;
    r.fin = &f;
    r.fin_d2s = fd2s;
    r.fin_n = fn;
    r.triangle = 0;
    if (op == 0) {
        r.valid = VAL_NO_HOLES;
        r.gen = NEW_KEEP;
        r.use_sign = 0;
        r.spin_weights = 1;
    } else if (op == 1) {
        r.valid = (Sz2 <= 0) ? VAL_ALL_DOWN : VAL_ALL_UP;
        r.gen = NEW_ADD_HOLE;
        r.use_sign = 1;
        r.spin_weights = 0;
    } else if (op == 2) {
        r.valid = VAL_ALL_HOLES;
        r.gen = (Sz2 > 0) ? NEW_ADD_DOWN : NEW_ADD_UP;
        r.use_sign = 1;
        r.spin_weights = 0;
    } else if (op == 3 || op == 4) {
        r.valid = VAL_HOLE_HOP;
        r.gen = NEW_SWAP;
        r.use_sign = op == 4;
        r.spin_weights = 0;
    } else {
        return OR_EINVAL;
    }
    return rule_columns(&s, d2s, orb, n, &r, colptr, rows, vre, vim, cap, nnz_out);
}

/* Singlet-singlet position-correlation operator (tJ_spin_half_ladder/matrix_setup.pyx:434-469):
 * startpoints i, endpoint shift sets (f0, fs, f1 + fs) and (-f0, fs - f0, f1 + fs - f0) with
 * f0, f1 the fixed distances and fs the free shift (each (leg, rung)), reverse=False; weights
 * (0, 0.5/N); validator is_valid_state_unequal_spins_2holes, remove_two_add_up_down,
 * get_weights_annihilation_part_singlet_singlet and the anticommutation sign.  Same sector in and
 * out.  shifts = {f0 leg, f0 rung, f1 leg, f1 rung, fs leg, fs rung}. */
int or_singlet_columns(int L, int Nh, int Nd, int kx, int ky, const int64_t *d2s, const int32_t *orb, int64_t n,
                       const int *shifts, int64_t *colptr, int64_t *rows, double *vre, double *vim, int64_t cap,
                       int64_t *nnz_out) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, kx, ky) != OR_OK || !shifts) return OR_EINVAL;
    const int f0[2] = {shifts[0], shifts[1]}, f1[2] = {shifts[2], shifts[3]}, fs[2] = {shifts[4], shifts[5]};
    const int sets[2][3][2] = {
        {{f0[0], f0[1]}, {fs[0], fs[1]}, {f1[0] + fs[0], f1[1] + fs[1]}},
        {{-f0[0], -f0[1]}, {fs[0] - f0[0], fs[1] - f0[1]}, {f1[0] + fs[0] - f0[0], f1[1] + fs[1] - f0[1]}},
    };
    combos_t c;
    c.n = 0;
    c.len = 4;
    for (int first = 0; first < s.N; ++first)
        for (int e = 0; e < 2; ++e) {
            c.idx[c.n][0] = (int16_t)first;
            for (int k = 0; k < 3; ++k)
                c.idx[c.n][k + 1] = (int16_t)index_by_relative_shift(s.N, first, sets[e][k][0], sets[e][k][1]);
            c.wd[c.n] = 0.0;
            c.wo[c.n] = 0.5 / (double)s.N;
            c.n++;
        }
    rule_t r = {&c, VAL_UNEQUAL_SPINS_2HOLES, NEW_REMOVE_TWO_ADD_UP_DOWN, 1, 2, 0, &s, d2s, n};
    return rule_columns(&s, d2s, orb, n, &r, colptr, rows, vre, vim, cap, nnz_out);
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Full columns (both triangles) of one term for a subset of column indices:
 * the sample used by the timed CPU baseline.  Same rule as or_term_columns. */
int or_term_columns_subset(int L, int Nh, int Nd, int kx, int ky, int term, int triangle, const int64_t *d2s,
                           const int32_t *orb, int64_t n, const int64_t *cols, int64_t ncols, int64_t *colptr,
                           int64_t *rows, double *vre, double *vim, int64_t cap, int64_t *nnz_out) {
    ors_t s;
    if (sector_init(&s, L, Nh, Nd, kx, ky) != OR_OK || term < 0 || term > 3) return OR_EINVAL;
    combos_t c;
    term_combos(s.N, term, &c);
    rule_t r = {&c, term < 2 ? VAL_HOLE_HOP : VAL_SPIN_SWAP, NEW_SWAP, term < 2, 0, triangle, &s, d2s, n};
    int64_t *cnt = (int64_t *)calloc((size_t)ncols + 1, sizeof(int64_t));
    if (!cnt) return OR_ENOMEM;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < ncols; ++k) {
        double complex vals[4 * OR_MAXN + 2];
        int64_t inds[4 * OR_MAXN + 2];
        int64_t i = cols[k];
        cnt[k + 1] = column(&s, i, d2s[i], orb[i], &r, vals, inds);
    }
    for (int64_t k = 0; k < ncols; ++k) cnt[k + 1] += cnt[k];
    *nnz_out = cnt[ncols];
    if (colptr) memcpy(colptr, cnt, ((size_t)ncols + 1) * sizeof(int64_t));
    if (!rows) {
        free(cnt);
        return OR_OK;
    }
    if (cnt[ncols] > cap) {
        free(cnt);
        return OR_ECAP;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < ncols; ++k) {
        double complex vals[4 * OR_MAXN + 2];
        int64_t inds[4 * OR_MAXN + 2];
        int64_t i = cols[k];
        int m = column(&s, i, d2s[i], orb[i], &r, vals, inds);
        for (int q = 0; q < m; ++q) {
            rows[cnt[k] + q] = inds[q];
            vre[cnt[k] + q] = creal(vals[q]);
            vim[cnt[k] + q] = cimag(vals[q]);
        }
    }
    free(cnt);
    return OR_OK;
}

/* The reference's SpMV over its row-major Hermitian-triangle storage, for a
 * set of stored rows (general/cpp_sparse_dot.h:59-71 explicit pass and
 * :104-138 Hermitian-conjugate pass, driven as in
 * general/cython_sparse_dot.pyx:65-79 with num_threads = 1): row r holds the
 * entries (col >= r, value index) of U; y[r] += w * sum U[r,c] x[c] and
 * y[c] += w * x[r] * conj(U[r,c]) for c != r.  Single-threaded like the
 * reference's only race-free setting. */
void or_spmv_triangle_rows(int64_t nrows, const int64_t *row_ids, const int64_t *ptr, const int64_t *cols,
                           const int16_t *vidx, const double complex *vals, const double complex *x,
                           double complex *y, double w_re, double w_im) {
    const double complex w = w_re + I * w_im;
    for (int64_t k = 0; k < nrows; ++k) {
        double complex acc = 0;
        for (int64_t j = ptr[k]; j < ptr[k + 1]; ++j) acc += x[cols[j]] * vals[vidx[j]];
        y[row_ids[k]] += w * acc;
    }
    for (int64_t k = 0; k < nrows; ++k) {
        const int64_t r = row_ids[k];
        for (int64_t j = ptr[k]; j < ptr[k + 1]; ++j) {
            const int64_t c = cols[j];
            if (c == r) continue;
            y[c] += x[r] * conj(vals[vidx[j]]) * w;
        }
    }
}
