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


def _lowest_ritz(a: np.ndarray, b_next: np.ndarray):
    """Lowest eigenpair of the tridiagonal matrix (diagonal a, off-diagonal b_next[:-1])."""
    from scipy.linalg import eigh_tridiagonal

    if len(a) == 1:
        return float(a[0]), np.ones(1)
    w, s = eigh_tridiagonal(a, b_next[: len(a) - 1], select="i", select_range=(0, 0))
    return float(w[0]), s[:, 0]


class CheckedLanczos:
    """A ground-state Lanczos recursion that reads its coefficients every `check_every` steps and
    stops once the lowest Ritz value changes by at most `tol` (relative) over a window, on breakdown,
    or after `max_steps`.  The first `keep` Lanczos vectors are kept (one vector of the run's dtype
    each) and the later ones rotate over two buffers; the Ritz vector then takes the kept vectors as
    they are and regenerates only the others, by continuing the recursion from the last two kept ones
    (the fused step is deterministic, so the regenerated vectors are the same bits)."""

    def __init__(self, sector: DeviceSector, weights, dtype: torch.dtype, max_steps: int, keep: int = 0):
        from exactdiag_gb300 import autotune

        self.sector, self.weights, self.dtype = sector, weights_tuple(weights), dtype
        self.max_steps = int(max_steps)
        self.keep = max(0, min(int(keep), self.max_steps + 1))
        dev = sector.device
        # kept vectors are allocated as the recursion reaches them
        self.V: list[torch.Tensor] = []
        self.R = [torch.zeros(sector.n, dtype=dtype, device=dev) for _ in range(2)]
        self.scal = torch.zeros(2 * self.max_steps + 4, dtype=torch.float64, device=dev)
        self.norm = torch.zeros(1, dtype=torch.float64, device=dev)
        autotune.ensure(sector, self.weights, dtype)

    def _buf(self, k: int) -> torch.Tensor:
        if k < self.keep:
            while len(self.V) <= k:
                self.V.append(torch.empty_like(self.R[0]))
            return self.V[k]
        return self.R[(k - self.keep) % 2]

    def _step(self, k: int, scal: torch.Tensor) -> None:
        # v_{k+1} overwrites v_{k-1} in place once both rotate; before that they are distinct buffers
        self.sector.lanczos_step(self.weights, self._buf(k), self._buf(k - 1) if k > 0 else None,
                                 self._buf(k + 1), scal[2 * k: 2 * k + 4])

    def run(self, v0: torch.Tensor, tol: float, check_every: int = 10, min_steps: int = 2) -> dict:
        s = self.sector
        self._buf(0).copy_(v0)
        s.normalize(self._buf(0), self.norm)
        self.scal.zero_()
        theta_prev, steps = None, self.max_steps
        for k in range(self.max_steps):
            self._step(k, self.scal)
            m = k + 1
            if m % check_every and m != self.max_steps:
                continue
            x = self.scal[: 2 * m + 2].cpu().numpy()
            a, b_next = x[1: 2 * m: 2], x[2: 2 * m + 1: 2]
            small = np.nonzero(b_next < 1e-8)[0]
            if len(small):
                steps = int(small[0]) + 1
                break
            theta, _ = _lowest_ritz(a, b_next)
            if m >= min_steps and theta_prev is not None and abs(theta - theta_prev) <= tol * abs(theta):
                steps = m
                break
            theta_prev = theta
        x = self.scal[: 2 * steps + 2].cpu().numpy()
        self.a, self.b_next = x[1: 2 * steps: 2].copy(), x[2: 2 * steps + 1: 2].copy()
        self.steps = steps
        self.theta, self.s = _lowest_ritz(self.a, self.b_next)
        self.residual = abs(float(self.b_next[steps - 1]) * float(self.s[-1]))
        return {"theta": self.theta, "steps": steps, "residual": self.residual}

    def ritz_vector(self, v0: torch.Tensor) -> torch.Tensor:
        """The lowest Ritz vector in FP64 (complex128 for complex sectors): the kept vectors as they
        are, the others regenerated (from v0 when none is kept)."""
        s = self.sector
        acc = torch.zeros(s.n, dtype=torch.float64 if s.is_real else torch.complex128, device=s.device)
        kept = min(self.keep, self.steps)
        if kept < 2 and kept < self.steps:
            kept = 0  # too few kept to continue from: regenerate from v0
        # the kept vectors in one pass over acc (the same bits as one accumulate per vector)
        s.accumulate_many(self.V[:kept], [complex(self.s[k]) for k in range(kept)], acc)
        if kept == self.steps:
            return acc
        if kept >= 2:
            # continue from v_{kept-2}, v_{kept-1}: step kept-1 writes v_kept again, and so on; the
            # scalars it reads (b_k) are the first pass's, the ones it writes the same bits
            start = kept - 1
        else:
            self.keep = 0
            self.V.clear()
            self._buf(0).copy_(v0)
            s.normalize(self._buf(0), self.norm)
            s.accumulate(self._buf(0), complex(self.s[0]), acc)
            start = 0
        for k in range(start, self.steps - 1):
            self._step(k, self.scal)
            s.accumulate(self._buf(k + 1), complex(self.s[k + 1]), acc)
        return acc


def _vectors_that_fit(sector: DeviceSector, dtype: torch.dtype, fraction: float = 0.6) -> int:
    """How many vectors of dtype fit in `fraction` of the device memory that is free (blocks that
    torch holds in its cache but does not use count as free)."""
    elem = torch.empty(0, dtype=dtype).element_size()
    free, _ = torch.cuda.mem_get_info(sector.device)
    cached = torch.cuda.memory_reserved(sector.device) - torch.cuda.memory_allocated(sector.device)
    return int(fraction * (free + cached) / max(1, sector.n * elem))


def ground_state(sector: DeviceSector, weights, max_steps: int = 240, precision: str = "mixed", seed: int = 0,
                 v0: torch.Tensor | None = None, tol: float = 1e-13, fp32_tol: float = 1e-7,
                 refine_max: int = 160, check_every: int = 10, keep_vectors: int | None = None) -> dict:
    """Ground energy of a sector, each form run until its lowest Ritz value has converged.

    precision "fp64": plain FP64 Lanczos until the lowest Ritz value changes by at most `tol`
    (relative) over `check_every` steps.
    precision "mixed": FP32 (complex64) Lanczos with FP64 reductions until the Ritz value changes by
    at most `fp32_tol` (the FP32 vectors' resolution); the Ritz vector is accumulated in FP64 from the
    FP32 Lanczos vectors -- those kept in device memory as they are (`keep_vectors`, by default as many
    as fit), the others regenerated by a second pass from the last two kept -- and refined by FP64
    Lanczos started from it, until its Ritz value changes by at most `tol`.  E0 is the refined
    value; the result also carries the step counts and the wall time of each phase.
    """
    import time

    dt = sector.dtype("fp64" if precision == "fp64" else "fp32")
    if v0 is None:
        x = np.random.default_rng(seed).uniform(-1, 1, sector.n)
        v0 = torch.as_tensor(x, device=sector.device).to(dt)
    else:
        v0 = v0.to(device=sector.device, dtype=dt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if precision == "fp64":
        run = CheckedLanczos(sector, weights, dt, max_steps)
        r = run.run(v0, tol, check_every)
        torch.cuda.synchronize()
        return {"E0": r["theta"], "theta": r["theta"], "steps": r["steps"], "residual": r["residual"],
                "a": run.a, "time_s": time.perf_counter() - t0}
    steps32 = max_steps
    cap = _vectors_that_fit(sector, dt) - 2  # two more buffers rotate beside the kept vectors
    if keep_vectors is None:
        # keep every FP32 vector when at least 100 fit (the FP32 stage then stops where they run out
        # at the latest; the refinement takes the rest of the convergence); else keep as many as fit
        # and regenerate the others for the Ritz vector
        if cap >= 100:
            steps32 = min(max_steps, cap)
            keep = steps32 + 1
        else:
            keep = max(0, cap)
    else:
        keep = int(keep_vectors)
    run = CheckedLanczos(sector, weights, dt, steps32, keep=keep)
    r = run.run(v0, fp32_tol, check_every)
    psi = run.ritz_vector(v0)
    del run
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ref = CheckedLanczos(sector, weights, psi.dtype, refine_max)
    rr = ref.run(psi, tol, check_every=4)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"E0": rr["theta"], "theta": r["theta"], "steps": r["steps"], "refine_steps": rr["steps"],
            "residual": rr["residual"], "rayleigh": float(ref.a[0]), "kept_vectors": min(keep, r["steps"]),
            "time_s": t2 - t0, "time_fp32_s": t1 - t0, "time_refine_s": t2 - t1}


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
