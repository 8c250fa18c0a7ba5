"""CPU oracle for the t-J ladder path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module, and only as the checker.  The GPU product
(``exactdiag_gb300``) never imports it.

Two CPU implementations sit behind it:

* ``oracle/ed_oracle.c`` (always available): a plain-C restatement of the
  reference's basis enumeration and matrix-element rules;
* ``oracle/_ref/libedref.so`` (only where the reference tree is present): the
  reference's own C++ headers compiled in place by ``oracle/Makefile``.

On top of them this module restates, in numpy, the reference's Python/Cython
numerics: the Hermitian triangle storage as ``.dot`` applies it
(general/cpp_sparse_dot.h:59-138, general/cython_sparse_dot.pyx:40-80,
general/sparse_matrices.py:83-105, 210-243), the spectrum Lanczos recursion
(general/cython_lanczos_diagonalization.pyx:50-77), the continued fraction
(:42-48) and the spectrum driver (general/lanczos_diagonalization.py:158-175).
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libedoracle.so"
REF_PATH = HERE / "_ref" / "libedref.so"
# the reference's src/exactdiag directory, when a checkout is at hand (oracle/_ref and the tests that
# compare with the reference's own code need it; nothing else does)
REF_SRC = pathlib.Path(os.environ["EXACTDIAG_REF_SRC"]) if os.environ.get("EXACTDIAG_REF_SRC") else None

TERMS = ("tl", "tr", "jl", "jr")
OPS = {"Szq": 0, "spectral_function_minus": 1, "spectral_function_plus": 2, "current_rung": 3, "current_leg": 4}

_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i16p = ctypes.POINTER(ctypes.c_int16)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(ref: bool | None = None) -> None:
    """Compile the C restatement and, when the reference tree exists, oracle/_ref."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if ref is None:
        ref = REF_SRC is not None and REF_SRC.is_dir()
    if ref:
        if REF_SRC is None:
            raise RuntimeError("set EXACTDIAG_REF_SRC to the reference's src/exactdiag directory")
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_SRC={REF_SRC}"], check=True)


_LIB = None
_REF = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            build(ref=False)
        _LIB = ctypes.CDLL(str(LIB_PATH))
        _LIB.or_state_to_sparse.restype = ctypes.c_int64
    return _LIB


def ref_lib() -> ctypes.CDLL | None:
    """The reference's own C++ compiled into oracle/_ref, or None when absent."""
    global _REF
    if _REF is None and REF_PATH.exists():
        _REF = ctypes.CDLL(str(REF_PATH))
    return _REF


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


@dataclass(frozen=True)
class Sector:
    """A symmetry sector of the ladder: L rungs, Nh holes, Nd down spins, k = (kx, ky)."""

    L: int
    Nh: int
    Nd: int
    kx: int
    ky: int

    @property
    def N(self) -> int:
        return 2 * self.L

    @property
    def Sz2(self) -> int:
        """total_spin_projection (tJ_spin_half_ladder/configs.py:107-109)."""
        return self.N - self.Nh - 2 * self.Nd

    def args(self):
        return (self.L, self.Nh, self.Nd, self.kx, self.ky)


def basis(sec: Sector, impl: str = "oracle", threads: int = 0):
    """Return (dense_to_sparse int64[n], num_sparse_in_dense int32[n]) (basis_indexing.h:188-242)."""
    n = ctypes.c_int64(0)
    if impl == "ref":
        r = ref_lib()
        if r is None:
            raise RuntimeError("oracle/_ref is not built")
        _check(r.ref_basis(*sec.args(), None, None, ctypes.c_int64(0), ctypes.byref(n), threads or 1), "ref_basis")
        sp = np.empty(n.value, np.int64)
        orb = np.empty(n.value, np.int32)
        _check(r.ref_basis(*sec.args(), _p(sp, _i64p), _p(orb, _i32p), ctypes.c_int64(n.value), ctypes.byref(n),
                           threads or 1), "ref_basis")
        return sp, orb
    L = lib()
    _check(L.or_basis_build(*sec.args(), None, None, ctypes.c_int64(0), ctypes.byref(n)), "or_basis_build")
    sp = np.empty(n.value, np.int64)
    orb = np.empty(n.value, np.int32)
    _check(L.or_basis_build(*sec.args(), _p(sp, _i64p), _p(orb, _i32p), ctypes.c_int64(n.value), ctypes.byref(n)),
           "or_basis_build")
    return sp, orb


def eligible_hole_ranks(sec: Sector) -> np.ndarray:
    n = ctypes.c_int64(0)
    _check(lib().or_eligible_hole_ranks(*sec.args(), None, ctypes.c_int64(0), ctypes.byref(n)), "eligible")
    out = np.empty(n.value, np.int64)
    _check(lib().or_eligible_hole_ranks(*sec.args(), _p(out, _i64p), ctypes.c_int64(n.value), ctypes.byref(n)),
           "eligible")
    return out


def sparse_to_state(sec: Sector, sparse: int) -> np.ndarray:
    st = np.empty(sec.N, np.int16)
    _check(lib().or_sparse_to_state(sec.L, sec.Nh, sec.Nd, ctypes.c_int64(int(sparse)), _p(st, _i16p)), "unrank")
    return st


def state_to_sparse(sec: Sector, state) -> int:
    st = np.ascontiguousarray(state, np.int16)
    return int(lib().or_state_to_sparse(sec.L, sec.Nh, sec.Nd, _p(st, _i16p)))


def _columns(fn, args, n_cols, what):
    nnz = ctypes.c_int64(0)
    colptr = np.empty(n_cols + 1, np.int64)
    _check(fn(*args, _p(colptr, _i64p), None, None, None, ctypes.c_int64(0), ctypes.byref(nnz)), what)
    rows = np.empty(nnz.value, np.int64)
    vre = np.empty(nnz.value, np.float64)
    vim = np.empty(nnz.value, np.float64)
    _check(fn(*args, _p(colptr, _i64p), _p(rows, _i64p), _p(vre, _f64p), _p(vim, _f64p), ctypes.c_int64(nnz.value),
              ctypes.byref(nnz)), what)
    return colptr, rows, vre + 1j * vim


def term_columns(sec: Sector, term: str, bas, triangle: bool = True, impl: str = "oracle"):
    """Column-major (colptr, rows, values) of one Hamiltonian term as the reference computes it."""
    sp, orb = bas
    t = TERMS.index(term)
    if impl == "ref":
        r = ref_lib()
        if r is None:
            raise RuntimeError("oracle/_ref is not built")
        fn = r.ref_term_columns
    else:
        fn = lib().or_term_columns
    args = (*sec.args(), t, int(triangle), _p(sp, _i64p), _p(orb, _i32p), ctypes.c_int64(len(sp)))
    return _columns(fn, args, len(sp), f"{impl} term {term}")


def target_sector(sec: Sector, name: str, qx: int, qy: int) -> Sector:
    """Final sector of an excitation (tJ_spin_half_ladder/matrix_setup.pyx:263-330); (qx, qy) as the setup sees them."""
    L = sec.L
    if name == "current_rung":
        qy += 1  # matrix_setup.pyx:251
    kx2 = (sec.kx + qx + (L - 1) // 2) % L - (L - 1) // 2
    ky2 = (sec.ky + qy) % 2
    if name in ("Szq", "current_rung", "current_leg"):
        return Sector(L, sec.Nh, sec.Nd, kx2, ky2)
    if name == "spectral_function_minus":
        if sec.Sz2 <= 0:
            return Sector(L, sec.Nh + 1, sec.Nd - 1, kx2, ky2)
        return Sector(L, sec.Nh + 1, sec.Nd, kx2, ky2)
    if name == "spectral_function_plus":  # matrix_setup.pyx:281-300: a down spin when Sz > 0, else an up spin
        if sec.Sz2 > 0:
            return Sector(L, sec.Nh - 1, sec.Nd + 1, kx2, ky2)
        return Sector(L, sec.Nh - 1, sec.Nd, kx2, ky2)
    raise ValueError(name)


def excitation_columns(sec: Sector, bas, name: str, qx: int, qy: int, fsec: Sector, fbas, impl: str = "oracle"):
    """Column-major operator from sector `sec` into `fsec` (matrix_setup.pyx:195-374)."""
    sp, orb = bas
    fsp, forb = fbas
    op = OPS[name]
    if impl == "ref":
        r = ref_lib()
        if r is None:
            raise RuntimeError("oracle/_ref is not built")
        args = (op, *sec.args(), sec.Sz2, _p(sp, _i64p), _p(orb, _i32p), ctypes.c_int64(len(sp)), fsec.Nh, fsec.Nd,
                fsec.kx, fsec.ky, _p(fsp, _i64p), _p(forb, _i32p), ctypes.c_int64(len(fsp)), qx, qy)
        return _columns(r.ref_excitation_columns, args, len(sp), "ref excitation")
    args = (op, *sec.args(), sec.Sz2, _p(sp, _i64p), _p(orb, _i32p), ctypes.c_int64(len(sp)), fsec.Nh, fsec.Nd,
            fsec.kx, fsec.ky, _p(fsp, _i64p), ctypes.c_int64(len(fsp)), qx, qy)
    return _columns(lib().or_excitation_columns, args, len(sp), "oracle excitation")


def _csc(colptr, rows, vals, shape):
    import scipy.sparse as sps

    return sps.csc_matrix((vals, rows, colptr), shape=shape)


def term_matrix(sec: Sector, term: str, bas, impl: str = "oracle"):
    """The matrix one term's `.dot` applies with triangle_only storage.

    Storage is the column lower triangle M (row >= column); the row-major
    Hermitian pass applies U + U^H - diag(U) with U = M^H
    (cython_sparse_matrices.pyx:149-155, cpp_sparse_dot.h:59-138), i.e.
    M^H + M - diag(M).
    """
    import scipy.sparse as sps

    colptr, rows, vals = term_columns(sec, term, bas, triangle=True, impl=impl)
    n = len(bas[0])
    m = _csc(colptr, rows, vals, (n, n)).tocsr()
    d = m.diagonal()
    return (m.conj().T + m - sps.diags(d)).tocsr()


def hamiltonian(sec: Sector, weights: dict, bas, impl: str = "oracle"):
    """H = sum_t w_t * term_t over terms with w_t != 0 (matrix_setup.pyx:118-129, sparse_matrices.py:233-237)."""
    import scipy.sparse as sps

    n = len(bas[0])
    h = sps.csr_matrix((n, n), dtype=np.complex128)
    for t in TERMS:
        w = weights.get(t, 0)
        if w != 0 and abs(w) >= 1e-6:
            h = h + w * term_matrix(sec, t, bas, impl)
    return h.tocsr()


def excitation_matrix(sec: Sector, bas, name: str, qx: int, qy: int, fsec: Sector, fbas, impl: str = "oracle"):
    colptr, rows, vals = excitation_columns(sec, bas, name, qx, qy, fsec, fbas, impl)
    return _csc(colptr, rows, vals, (len(fbas[0]), len(bas[0]))).tocsr()


def _start_vector(n: int, dtype) -> np.ndarray:
    """Seeded random start vector for eigsh.  A uniform one is not safe: it can lie in a subspace
    of a residual symmetry of the sector and miss the ground state there (2x8, two holes,
    k = (3, 1): all ones finds -9.7705, the second level, not the ground state -9.8664)."""
    rng = np.random.default_rng(1234)
    v = rng.uniform(-1, 1, n)
    if np.iscomplexobj(np.zeros(0, dtype)):
        v = v + 1j * rng.uniform(-1, 1, n)
    return (v / np.linalg.norm(v)).astype(dtype)


def lowest_eigvals(h, k: int, tol: float = 1e-14):
    """Tight FP64 eigen-oracle: dense eigh for small n, eigsh otherwise."""
    n = h.shape[0]
    if n == 0:
        return np.zeros(0)
    if n <= 600:
        return np.sort(np.linalg.eigvalsh(h.toarray()))[:k]
    import scipy.sparse.linalg as spl

    vals = spl.eigsh(h, k=min(k, n - 2), which="SA", tol=tol, v0=_start_vector(n, h.dtype),
                     return_eigenvectors=False)
    return np.sort(vals)


def lowest_eigpairs(h, k: int, tol: float = 1e-14):
    n = h.shape[0]
    if n <= 600:
        w, v = np.linalg.eigh(h.toarray())
        return w[:k], v[:, :k]
    import scipy.sparse.linalg as spl

    w, v = spl.eigsh(h, k=min(k, n - 2), which="SA", tol=tol, v0=_start_vector(n, h.dtype))
    o = np.argsort(w)
    return w[o], v[:, o]


# --- numpy restatement of general/cython_lanczos_diagonalization.pyx -------------------------

def lanczos_get_anbn(v0, num_lanczos_vecs: int, apply_h):
    """_lanczos_get_anbn (:50-66) with _lanczos_vec_iteration (:68-77)."""
    vn = v0 / np.linalg.norm(v0)
    ans = np.zeros(num_lanczos_vecs)
    bns = np.zeros(num_lanczos_vecs + 1)
    vnm = np.zeros(len(vn), np.complex128)
    k = 0
    for i in range(num_lanczos_vecs):
        hvn = apply_h(vn)
        an = np.real(np.vdot(vn, hvn))
        vnp = hvn - an * vn - bns[i] * vnm
        bnp = np.linalg.norm(vnp)
        vnp = vnp / bnp if bnp != 0 else vnp
        ans[i], bns[i + 1] = an, bnp
        k += 1
        if bns[i + 1] < 1e-8:
            break
        vnm = vn
        vn = vnp
    return ans[:k], bns[:k]


def spectral_value_at_z(ans, bns, z):
    """_spectral_value_at_z (:42-48): bottom-up continued fraction, returns Im(1/det)."""
    m = len(ans)
    det = z - ans[m - 1]
    for i in range(1, m):
        det = z - ans[m - 1 - i] - bns[m - i] ** 2 / det
    return (1.0 / det).imag


def continued_fraction(ans, bns, zs, norm2):
    """-1/pi * |phi|^2 * Im(1/det(z)) for every z, vectorised over z (lanczos_dynamical_response :36-39)."""
    zs = np.asarray(zs, np.complex128)
    m = len(ans)
    det = zs - ans[m - 1]
    for i in range(1, m):
        det = zs - ans[m - 1 - i] - bns[m - i] ** 2 / det
    return -1.0 / np.pi * norm2 * (1.0 / det).imag


def lanczos_dynamical_response(gs, op_apply, h_apply, zs, num_lanczos_vecs):
    """lanczos_dynamical_response (:18-40)."""
    phi = op_apply(gs)
    norm = np.linalg.norm(phi)
    if norm < 1e-8:
        return np.zeros(len(zs)), np.zeros(0), np.zeros(0), 0.0
    ans, bns = lanczos_get_anbn(phi / norm, num_lanczos_vecs, h_apply)
    return continued_fraction(ans, bns, zs, norm ** 2), ans, bns, norm


def num_threads() -> int:
    return int(lib().or_num_threads())


def _relative_index(N: int, initial: int, relative: int) -> int:
    """tJ_spin_half_ladder/symmetry_ladder.h:88-95 get_index_by_relative_index."""
    initial %= N
    relative %= N
    leg = initial // 2 + relative // 2
    rung = (initial + relative) % 2
    return (2 * leg + rung) % N


def _relative_shift(N: int, initial: int, shift) -> int:
    """tJ_spin_half_ladder/symmetry_ladder.h:96-101 get_index_by_relative_shift (C++ % on the rung
    shift, then a positive modulo)."""
    initial %= N
    leg = initial // 2 + int(shift[0])
    r1 = int(shift[1])
    r1 = r1 - 2 * int(r1 / 2)  # C++ truncating remainder
    rung = (initial + r1) % 2
    return (2 * leg + rung) % N


def position_correlations(sec: Sector, bas, psi: np.ndarray, name: str, fixed=()) -> np.ndarray:
    """Hole / S^z correlations of one state over distances 0..N-1
    (tJ_spin_half_ladder/position_correlations.pyx:83-118, :174-207): every representative's own
    configuration, weighted by |psi_i|^2, summed over reference sites."""
    N = sec.N
    states = np.array([sparse_to_state(sec, s) for s in bas[0]], dtype=np.int16).reshape(-1, N)
    w = np.abs(np.asarray(psi)) ** 2
    spin = np.where(states == 1, -1, 1) * (states != 0)  # 0 hole, 1 down, 2 up
    out = np.zeros(N)
    for dist in range(N):
        for r in range(N):
            pos = [r, _relative_index(N, r, dist)] + [_relative_shift(N, r, f) for f in fixed]
            if name == "hole_correlations":
                val = np.all(states[:, pos] == 0, axis=1).astype(float)
            else:
                val = np.prod(spin[:, pos], axis=1).astype(float)
            out[dist] += float(np.dot(w, val))
    return out


def singlet_columns(sec: Sector, bas, shifts, impl: str = "oracle"):
    """Column-major singlet-singlet correlation operator for one free shift
    (tJ_spin_half_ladder/matrix_setup.pyx:434-469); shifts = (f0, f1, free), each (leg, rung)."""
    sp, orb = bas
    sh = np.ascontiguousarray(np.asarray(shifts, dtype=np.int32).reshape(6))
    shp = sh.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    if impl == "ref":
        r = ref_lib()
        if r is None:
            raise RuntimeError("oracle/_ref is not built")
        args = (*sec.args(), _p(sp, _i64p), _p(orb, _i32p), ctypes.c_int64(len(sp)), shp)
        return _columns(r.ref_singlet_columns, args, len(sp), "ref singlet")
    args = (*sec.args(), _p(sp, _i64p), _p(orb, _i32p), ctypes.c_int64(len(sp)), shp)
    return _columns(lib().or_singlet_columns, args, len(sp), "oracle singlet")


def singlet_correlations(sec: Sector, bas, gs: np.ndarray, fixed) -> np.ndarray:
    """Re <gs| O(free) |gs> for the free shifts of every distance index, free = (d // 2, d % 2)
    (tJ_spin_half_ladder/position_correlations.pyx:112-124)."""
    n = len(bas[0])
    out = np.zeros(sec.N)
    for d in range(sec.N):
        colptr, rows, vals = singlet_columns(sec, bas, [fixed[0], fixed[1], (d // 2, d % 2)])
        op = _csc(colptr, rows, vals, (n, n))
        out[d] = float(np.real(np.vdot(gs, op @ gs)))
    return out
