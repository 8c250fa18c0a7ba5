"""Device-resident Lanczos recursions on a DeviceSector.

`lanczos_coefficients` is the GPU form of the reference's spectrum recursion
(general/cython_lanczos_diagonalization.pyx:50-77): v_0 = v/|v|, then per step
w = H v_k, a_k = Re<v_k, w>, v' = w - a_k v_k - b_k v_{k-1}, b_{k+1} = |v'|,
stopping after the first b_{k+1} < 1e-8.  Each step is one ed_lanczos_step
call (fused H.v + FP64 reductions, scalars kept on the device), so the whole
recursion can be captured once in a CUDA graph and replayed without a host
round trip; the host reads the coefficients once at the end.

Scalar layout: step k reads b_k from X[2k] and writes a_k to X[2k+1] and
b_{k+1} to X[2k+2], which is where step k+1 reads its b.  Vectors rotate over
two buffers because v_{k+1} overwrites v_{k-1} in place.
"""

from __future__ import annotations

import numpy as np
import torch

from exactdiag_gb300.engine import DeviceSector, weights_tuple


class LanczosRun:
    """Buffers of one recursion; reusable for repeated runs of the same length (graph replay)."""

    def __init__(self, sector: DeviceSector, weights, num_lanczos_vecs: int, dtype: torch.dtype):
        self.sector = sector
        self.weights = weights_tuple(weights)
        self.m = int(num_lanczos_vecs)
        self.dtype = dtype
        dev = sector.device
        self.buf = [torch.zeros(sector.n, dtype=dtype, device=dev), torch.zeros(sector.n, dtype=dtype, device=dev)]
        self.scal = torch.zeros(2 * self.m + 4, dtype=torch.float64, device=dev)
        self.norm = torch.zeros(1, dtype=torch.float64, device=dev)
        self.graph = None
        from exactdiag_gb300 import autotune

        autotune.ensure(sector, self.weights, dtype)

    def _record(self, ritz=None, acc=None, steps: int | None = None) -> None:
        s = self.sector
        s.normalize(self.buf[0], self.norm)
        self.scal.zero_()
        for k in range(self.m if steps is None else min(steps, self.m)):
            v = self.buf[k % 2]
            other = self.buf[(k + 1) % 2]
            if ritz is not None and k < len(ritz):
                s.accumulate(v, ritz[k], acc)
            s.lanczos_step(self.weights, v, other if k > 0 else None, other, self.scal[2 * k: 2 * k + 4])

    def run(self, v0: torch.Tensor, use_graph: bool = True) -> None:
        """Run the recursion from v0 (copied in); results stay on the device."""
        self.buf[0].copy_(v0)
        if not use_graph:
            self._record()
            return
        if self.graph is None:
            # warm up outside capture with two steps (every kernel of the recursion launches once
            # and sets its attributes), then capture the whole recursion
            self._record(steps=2)
            self.buf[0].copy_(v0)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._record()
            self.graph = g
        self.graph.replay()

    def coefficients(self) -> tuple[np.ndarray, np.ndarray, float]:
        """(a[:k], b[:k]) truncated like _lanczos_get_anbn (b[0] = 0) and |v0|."""
        x = self.scal.cpu().numpy()
        a = x[1: 2 * self.m: 2].copy()
        b_next = x[2: 2 * self.m + 1: 2].copy()
        k = self.m
        small = np.nonzero(b_next < 1e-8)[0]
        if len(small):
            k = int(small[0]) + 1
        b = np.concatenate([[0.0], b_next[: k - 1]])
        return a[:k], b[:k], float(self.norm.item())

    def last_vectors(self) -> tuple[torch.Tensor, torch.Tensor]:
        """(v_m, v_{m-1}) after a run of m steps (v_m normalised unless breakdown)."""
        return self.buf[self.m % 2], self.buf[(self.m + 1) % 2]


def ritz_vector(run: LanczosRun, v0: torch.Tensor, coeffs: np.ndarray) -> torch.Tensor:
    """sum_k coeffs[k] v_k in FP64, regenerating v_k by a second, bitwise-identical run from v0."""
    sec = run.sector
    acc = torch.zeros(sec.n, dtype=torch.float64 if sec.is_real else torch.complex128, device=sec.device)
    run.buf[0].copy_(v0)
    run._record(ritz=[complex(c) for c in coeffs], acc=acc)
    return acc


def ground_state(sector: DeviceSector, weights, num_steps: int, precision: str = "mixed", seed: int = 0,
                 refine_steps: int = 32, v0: torch.Tensor | None = None, use_graph: bool = True) -> dict:
    """Ground energy of a sector.

    precision "fp64": plain FP64 Lanczos; E0 = lowest Ritz value.
    precision "mixed": FP32 (complex64) Lanczos vectors with FP64 reductions;
    the lowest Ritz vector is rebuilt in FP64 on a second pass and refined by
    `refine_steps` FP64 Lanczos steps started from it (Rayleigh quotient and
    residual come from that refinement run).
    """
    from scipy.linalg import eigh_tridiagonal

    dt = sector.dtype("fp64" if precision == "fp64" else "fp32")
    if v0 is None:
        x = np.random.default_rng(seed).uniform(-1, 1, sector.n)
        v0 = torch.as_tensor(x, device=sector.device).to(dt)
    else:
        v0 = v0.to(device=sector.device, dtype=dt)
    run = LanczosRun(sector, weights, num_steps, dt)
    run.run(v0, use_graph=use_graph)
    a, b, _ = run.coefficients()
    if len(a) == 1:
        theta, vecs = np.array([a[0]]), np.ones((1, 1))
    else:
        theta, vecs = eigh_tridiagonal(a, b[1:])
    out = {"theta": float(theta[0]), "a": a, "b": b, "steps": len(a), "E0": float(theta[0])}
    if precision == "fp64":
        return out
    psi = ritz_vector(run, v0, vecs[:, 0])
    ref = LanczosRun(sector, weights, refine_steps, psi.dtype)
    ref.run(psi, use_graph=False)
    ra, rb, _ = ref.coefficients()
    rq = float(ra[0])
    resid = float(rb[1]) if len(rb) > 1 else 0.0
    e_ref = float(tridiagonal_eigvals(ra, rb)[0])
    out.update({"E0": e_ref, "rayleigh": rq, "residual": resid, "refine_steps": len(ra)})
    return out


def lanczos_coefficients(sector: DeviceSector, weights, v0: torch.Tensor, num_lanczos_vecs: int,
                         use_graph: bool = False):
    """(a, b, |v0|) of the spectrum recursion started from v0 (any norm)."""
    run = LanczosRun(sector, weights, num_lanczos_vecs, v0.dtype)
    run.run(v0, use_graph=use_graph)
    return run.coefficients()


def tridiagonal_eigvals(a: np.ndarray, b: np.ndarray, k: int | None = None) -> np.ndarray:
    """Eigenvalues of the Lanczos tridiagonal matrix T (diagonal a, off-diagonal b[1:])."""
    from scipy.linalg import eigh_tridiagonal

    if len(a) == 1:
        return np.array([a[0]])
    w = eigh_tridiagonal(a, b[1:], eigvals_only=True)
    return w if k is None else w[:k]
