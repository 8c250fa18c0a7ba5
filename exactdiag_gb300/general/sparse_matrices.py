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
