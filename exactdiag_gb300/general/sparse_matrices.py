"""Operator objects with the reference's .dot / .shape / .toarray protocol.

The reference hands ARPACK and its spectrum Lanczos an Added_Sparse_Matrices
(general/sparse_matrices.py:210-243) whose .dot(vec) runs the stored SpMV.  The
objects here expose the same protocol over the matrix-free GPU operator: .dot
takes and returns host complex128 vectors (one host->device and one
device->host copy per call), and .device_dot keeps everything on the GPU.
"""

from __future__ import annotations

import numpy as np
import torch

from exactdiag_gb300.engine import DeviceSector, weights_tuple

VALUE_TYPE = np.complex128


class Device_Hamiltonian:
    """H = sum_t w_t term_t of one sector, applied matrix-free on the GPU."""

    def __init__(self, sector: DeviceSector, weights, num_threads: int = 1, precision: str = "fp64"):
        self.sector = sector
        self.weights_tuple = weights_tuple(weights)
        self.shape = [sector.n, sector.n]
        self.num_threads = num_threads
        self.precision = precision
        self.num_matrices = sum(1 for w in self.weights_tuple if w != 0)
        self.weights = np.array([w for w in self.weights_tuple if w != 0], dtype=VALUE_TYPE)

    def device_dot(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """H x for a CUDA tensor x (any of the four vector dtypes)."""
        return self.sector.hv(x, self.weights_tuple, out=out)

    def dot(self, vec) -> np.ndarray:
        """H vec for a host vector; returns complex128 like Added_Sparse_Matrices.dot."""
        v = np.asarray(vec, dtype=VALUE_TYPE)
        if v.shape != (self.shape[1],):
            raise ValueError(f"expected a vector of length {self.shape[1]}")
        if self.shape[0] == 0:
            return np.zeros(0, VALUE_TYPE)
        dt = torch.complex128 if self.precision == "fp64" else torch.complex64
        x = torch.as_tensor(v).to(device=self.sector.device, dtype=dt)
        return self.device_dot(x).cpu().numpy().astype(VALUE_TYPE)

    def toarray(self) -> np.ndarray:
        """Dense matrix (small sectors only), assembled from GPU H.v on unit vectors."""
        from exactdiag_gb300.eigensolver import dense_matrix

        return dense_matrix(self.sector, self.weights_tuple, torch.complex128)


class Device_Operator:
    """An excitation operator from one sector into another (general/sparse_matrices.py:27-139 protocol)."""

    def __init__(self, name: str, src: DeviceSector, dst: DeviceSector, qx: int, qy: int, initial_sz2: int,
                 num_threads: int = 1, precision: str = "fp64"):
        self.name = name
        self.src, self.dst = src, dst
        self.qx, self.qy, self.initial_sz2 = int(qx), int(qy), int(initial_sz2)
        self.shape = [dst.n, src.n]
        self.num_threads = num_threads
        self.precision = precision

    def device_dot(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        if not x.dtype.is_complex:
            x = x.to(torch.complex128 if x.dtype == torch.float64 else torch.complex64)
        return self.src.excite_into(self.dst, self.name, self.qx, self.qy, self.initial_sz2, x, out=out)

    def dot(self, vec) -> np.ndarray:
        v = np.asarray(vec, dtype=VALUE_TYPE)
        if v.shape != (self.shape[1],):
            raise ValueError(f"expected a vector of length {self.shape[1]}")
        if self.shape[0] == 0:
            return np.zeros(0, VALUE_TYPE)
        dt = torch.complex128 if self.precision == "fp64" else torch.complex64
        x = torch.as_tensor(v).to(device=self.src.device, dtype=dt)
        return self.device_dot(x).cpu().numpy().astype(VALUE_TYPE)


TERMS = ("tl", "tr", "jl", "jr")


class Sparse_Matrix:
    """One Hamiltonian term of a sector (general/sparse_matrices.py:27-139), applied matrix-free.

    The reference loads the term's stored matrix from the sector's calculation folder; here
    from_name gives the same `.dot(vec, weight=1, matvec=None)` / `.shape` / `.toarray` protocol
    over the GPU operator with that term's weight set to one.
    """

    def __init__(self, sector: DeviceSector, name: str, num_threads: int = 1, precision: str = "fp64"):
        if name not in TERMS:
            raise ValueError(f"unknown Hamiltonian term {name!r}; expected one of {TERMS}")
        self.name = name
        self.num_threads = num_threads
        self._op = Device_Hamiltonian(sector, {t: (1.0 if t == name else 0.0) for t in TERMS}, num_threads,
                                      precision)
        self.shape = self._op.shape

    @classmethod
    def from_name(cls, name: str, config, num_threads: int | None = None) -> "Sparse_Matrix":
        """The term `name` of the sector `config` (a Hamiltonian config) describes (:127-139)."""
        from exactdiag_gb300.tJ_spin_half_ladder.matrix_setup import sector_of

        num_threads = config.num_threads if num_threads is None else num_threads
        return cls(sector_of(config), name, num_threads, getattr(config, "precision", "fp64"))

    def dot(self, vec, weight=1, matvec=None) -> np.ndarray:
        """matvec + weight * (term @ vec) (the reference's accumulate-into convention)."""
        out = complex(weight) * self._op.dot(vec)
        return out if matvec is None else matvec + out

    def toarray(self) -> np.ndarray:
        return self._op.toarray()


class Added_Sparse_Matrices:
    """Weighted sum of operators with a common shape (general/sparse_matrices.py:210-243)."""

    def __init__(self, mats, weights=None):
        self.refs = list(mats)
        if any(m.shape != self.refs[0].shape for m in self.refs[1:]):
            raise ValueError("incompatible shapes")
        self.shape = self.refs[0].shape
        self.num_matrices = len(self.refs)
        if weights is None:
            weights = [1] * self.num_matrices
        elif len(weights) != self.num_matrices:
            raise ValueError("wrong weights supplied")
        self.weights = np.array(list(weights), dtype=VALUE_TYPE)
        self.num_threads = max(getattr(m, "num_threads", 1) for m in self.refs)

    def add_matrix(self, matrix, weight) -> None:
        if self.shape != matrix.shape:
            raise ValueError(f"Nonmatching shapes {self.shape} and {matrix.shape}.")
        self.refs.append(matrix)
        self.weights = np.append(self.weights, VALUE_TYPE(weight))
        self.num_matrices += 1

    def dot(self, vec) -> np.ndarray:
        matvec = None
        for m, w in zip(self.refs, self.weights):
            matvec = m.dot(vec, w, matvec)
        return matvec

    def toarray(self) -> np.ndarray:
        mat = np.zeros(self.shape, dtype=VALUE_TYPE)
        for m, w in zip(self.refs, self.weights):
            mat += w * m.toarray()
        return mat
