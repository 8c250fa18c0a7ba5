"""Lowest eigenpairs of a sector on the GPU.

Replaces general/lanczos_diagonalization.py:53-121 (calculate_eigenpairs:
dense eigh below 250 rows, otherwise scipy ARPACK's implicitly restarted
Arnoldi on H.dot).  Here:

* n < 250 or n < 2 (k + 4): the dense matrix is assembled column by column with
  the GPU operator and diagonalised with numpy's eigh, like the reference;
* otherwise: Lanczos on the device with full reorthogonalisation (classical
  Gram-Schmidt applied twice, FP64 dot products, ed_project_out) and explicit
  deflation: converged eigenvectors are locked and the next run starts in their
  orthogonal complement, which also finds the second copy of a degenerate
  eigenvalue that a single Krylov space cannot hold.  A final run in the
  complement of all locked vectors confirms that no lower eigenvalue was missed.

Ritz values and residuals come from the small tridiagonal matrices on the host;
every vector operation runs through libexactdiag_gb300.so.
"""

from __future__ import annotations

import numpy as np
import torch

from exactdiag_gb300.engine import DeviceSector


def dense_matrix(sector: DeviceSector, weights, dtype: torch.dtype) -> np.ndarray:
    """H as a dense host matrix, one GPU H.v per column (small sectors only)."""
    n = sector.n
    cdt = dtype if dtype.is_complex else dtype
    e = torch.zeros(n, dtype=cdt, device=sector.device)
    y = torch.empty_like(e)
    cols = []
    for j in range(n):
        e.zero_()
        e[j] = 1
        sector.hv(e, weights, out=y)
        cols.append(y.cpu().numpy().copy())
    return np.stack(cols, axis=1).astype(np.complex128)


class _Krylov:
    def __init__(self, sector: DeviceSector, weights, dtype: torch.dtype, m_max: int):
        self.s = sector
        self.w = weights
        self.dt = dtype
        self.m_max = m_max
        n = sector.n
        self.V = torch.empty(m_max + 1, n, dtype=dtype, device=sector.device)
        self.coefs = torch.zeros(m_max + 1, 2 * (m_max + 1), dtype=torch.float64, device=sector.device)
        self.betas = torch.zeros(m_max + 2, dtype=torch.float64, device=sector.device)
        self.tmp = torch.empty(n, dtype=dtype, device=sector.device)

    def run(self, start: torch.Tensor, locked: torch.Tensor | None, n_locked: int, need: int, tol: float,
            check_every: int = 10):
        s, V = self.s, self.V
        v = V[0]
        v.copy_(start)
        for _ in range(2):
            if n_locked:
                s.project_out(locked, n_locked, v)
        s.normalize(v, self.betas[0:1])
        m = 0
        theta = vecs = None
        for j in range(self.m_max):
            w = V[j + 1]
            s.hv(V[j], self.w, out=w)
            if n_locked:
                s.project_out(locked, n_locked, w)
            s.project_out(V, j + 1, w, self.coefs[j])
            s.project_out(V, j + 1, w)
            if n_locked:
                s.project_out(locked, n_locked, w)
            s.normalize(w, self.betas[j + 1: j + 2])
            m = j + 1
            if m % check_every == 0 or m == self.m_max or m >= s.n - n_locked:
                theta, vecs, done, breakdown = self._ritz(m, need, tol)
                if done or breakdown:
                    break
        if theta is None:
            theta, vecs, _, _ = self._ritz(m, need, tol)
        return m, theta, vecs

    def _ritz(self, m: int, need: int, tol: float):
        from scipy.linalg import eigh_tridiagonal

        c = self.coefs[:m].cpu().numpy()
        a = np.array([c[j, 2 * j] for j in range(m)])
        b = self.betas[1: m + 1].cpu().numpy()
        if m == 1:
            theta, vecs = np.array([a[0]]), np.ones((1, 1))
        else:
            theta, vecs = eigh_tridiagonal(a, b[: m - 1])
        breakdown = b[m - 1] < 1e-10
        resid = np.abs(b[m - 1] * vecs[m - 1, :need])
        done = bool(np.all(resid < tol * np.maximum(1.0, np.abs(theta[:need])))) and m >= need
        return theta, vecs, done, breakdown

    def ritz_vectors(self, m: int, vecs: np.ndarray, cols: list[int]) -> torch.Tensor:
        s = self.s
        acc_dt = torch.float64 if s.is_real else torch.complex128
        out = torch.zeros(len(cols), s.n, dtype=acc_dt, device=s.device)
        for q, i in enumerate(cols):
            for j in range(m):
                s.accumulate(self.V[j], float(vecs[j, i]), out[q])
        return out


def _lowest(sector: DeviceSector, weights, k: int, dt: torch.dtype, tol: float, max_krylov: int, seed: int,
            memory_fraction: float):
    """Deflated Lanczos rounds until k eigenpairs are locked and a confirmation run finds nothing lower:
    (eigenvalues in the order found, the locked vectors (k + 1, n) of dtype dt)."""
    n = sector.n
    elem = torch.empty(0, dtype=dt).element_size()
    free, _ = torch.cuda.mem_get_info(sector.device)
    m_cap = int(memory_fraction * free / (n * elem)) - k - 2
    m_max = max(8, min(max_krylov, n - 1, m_cap))
    kry = _Krylov(sector, weights, dt, m_max)
    locked = torch.zeros(k + 1, n, dtype=dt, device=sector.device)
    vals: list[float] = []
    rng = np.random.default_rng(seed)
    rounds = 0
    while True:
        rounds += 1
        need = max(1, k - len(vals))
        x = rng.uniform(-1, 1, n)
        start = torch.as_tensor(x, device=sector.device).to(dt)
        m, theta, vecs = kry.run(start, locked, len(vals), need, tol)
        if len(vals) >= k:
            # confirmation run: the lowest eigenvalue left in the complement must not undercut the k-th found one
            kth = sorted(vals)[k - 1]
            if theta[0] >= kth - 10 * tol * max(1.0, abs(kth)) or len(vals) >= n:
                break
            take = 1
        else:
            take = min(need, m)
        ys = kry.ritz_vectors(m, vecs, list(range(take)))
        norm = torch.zeros(1, dtype=torch.float64, device=sector.device)
        for q in range(take):
            if len(vals) >= locked.shape[0]:
                locked = torch.cat([locked, torch.zeros(1, n, dtype=dt, device=sector.device)])
            row = locked[len(vals)]
            row.copy_(ys[q].to(dt))
            for _ in range(2):
                if len(vals):
                    sector.project_out(locked, len(vals), row)
            sector.normalize(row, norm)
            vals.append(float(theta[q]))
        if rounds > 4 * k + 4:
            break
    return vals, locked


def lowest_eigenpairs(sector: DeviceSector, weights, k: int, precision: str = "fp64", tol: float = 1e-10,
                      max_krylov: int = 300, seed: int = 0, memory_fraction: float = 0.5, fp32_tol: float = 1e-6,
                      refine_krylov: int = 120):
    """(eigenvalues[k], eigenvectors (n, k) complex128 on the host) of the sector's H.

    precision "fp64": FP64 (complex128) Krylov vectors throughout.
    precision "mixed": the eigenpairs are first found with FP32 (complex64) Krylov vectors and FP64
    dot products to `fp32_tol`; each is then refined by an FP64 Lanczos run started from its FP32
    vector, in the complement of the eigenvectors already refined, to `tol`.
    """
    n = sector.n
    if n == 0:
        return np.zeros(0), np.zeros((0, 0), np.complex128)
    if n < 250 or n < 2 * (k + 4):
        h = dense_matrix(sector, weights, sector.dtype("fp64"))
        vals, vecs = np.linalg.eigh(h)
        return vals[:k], vecs[:, :k]
    k = min(k, n)
    if precision != "mixed":
        vals, locked = _lowest(sector, weights, k, sector.dtype("fp64"), tol, max_krylov, seed, memory_fraction)
    else:
        vals32, locked32 = _lowest(sector, weights, k, sector.dtype("fp32"), fp32_tol, max_krylov, seed,
                                   memory_fraction)
        dt = sector.dtype("fp64")
        order32 = np.argsort(vals32)[:k]
        free, _ = torch.cuda.mem_get_info(sector.device)
        elem = torch.empty(0, dtype=dt).element_size()
        m_cap = int(memory_fraction * free / (n * elem)) - k - 2
        kry = _Krylov(sector, weights, dt, max(8, min(refine_krylov, n - 1, m_cap)))
        locked = torch.zeros(k + 1, n, dtype=dt, device=sector.device)
        norm = torch.zeros(1, dtype=torch.float64, device=sector.device)
        vals = []
        for j, i in enumerate(order32):
            m, theta, vecs = kry.run(locked32[int(i)].to(dt), locked, j, 1, tol, check_every=4)
            row = locked[j]
            row.copy_(kry.ritz_vectors(m, vecs, [0])[0].to(dt))
            for _ in range(2):
                if j:
                    sector.project_out(locked, j, row)
            sector.normalize(row, norm)
            vals.append(float(theta[0]))
        del locked32
    order = np.argsort(vals)[:k]
    out_vals = np.array(vals)[order]
    out_vecs = locked[torch.as_tensor(order, device=sector.device)].to(torch.complex128).cpu().numpy().T
    return out_vals, out_vecs
