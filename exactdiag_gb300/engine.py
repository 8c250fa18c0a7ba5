"""Device sectors: the Python face of the C ABI (include/exactdiag_gb300.h).

PyTorch provides device memory and the current CUDA stream; every operation on
the path is a call into libexactdiag_gb300.so.  Vectors are torch tensors on the
sector's device, indexed by dense basis index (the reference's own order).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from exactdiag_gb300 import _native as nat

TERMS = ("tl", "tr", "jl", "jr")

# (dtype code, torch dtype) per precision and sector kind
_DTYPES = {
    ("fp64", True): (nat.ED_F64, torch.float64),
    ("fp64", False): (nat.ED_C128, torch.complex128),
    ("fp32", True): (nat.ED_F32, torch.float32),
    ("fp32", False): (nat.ED_C64, torch.complex64),
}
_CODE_OF_TORCH = {torch.float64: nat.ED_F64, torch.complex128: nat.ED_C128, torch.float32: nat.ED_F32,
                  torch.complex64: nat.ED_C64}


def _stream_ptr() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


def weights_tuple(weights) -> tuple[float, float, float, float]:
    """(tl, tr, jl, jr) from a mapping, an object with those attributes, or a 4-sequence."""
    if isinstance(weights, dict):
        return tuple(float(weights.get(t, 0.0)) for t in TERMS)
    if hasattr(weights, "tl"):
        return tuple(float(getattr(weights, t)) for t in TERMS)
    w = tuple(float(v) for v in weights)
    if len(w) != 4:
        raise ValueError("weights must have 4 entries (tl, tr, jl, jr)")
    return w


# ed_excitation_apply operator codes (tJ_spin_half_ladder/matrix_setup.pyx:235-325)
EXCITATION_OPS = {"Szq": 0, "spectral_function_minus": 1, "spectral_function_plus": 2, "current_rung": 3,
                  "current_leg": 4}


@dataclass(frozen=True)
class SectorKey:
    num_rungs: int
    num_holes: int
    num_down_spins: int
    kx: int
    ky: int


class DeviceSector:
    """A symmetry sector whose basis lives on the GPU (ed_sector_create + ed_basis_build)."""

    def __init__(self, num_rungs: int, num_holes: int, num_down_spins: int, kx: int, ky: int):
        if not torch.cuda.is_available():
            raise RuntimeError("exactdiag_gb300 needs a CUDA device; there is no CPU path")
        self._lib = nat.load()
        self.key = SectorKey(int(num_rungs), int(num_holes), int(num_down_spins), int(kx), int(ky))
        h = ctypes.c_void_p()
        nat.check("ed_sector_create",
                  self._lib.ed_sector_create(self.key.num_rungs, self.key.num_holes, self.key.num_down_spins,
                                             self.key.kx, self.key.ky, ctypes.byref(h)))
        self._h = h
        nat.check("ed_basis_build", self._lib.ed_basis_build(h, _stream_ptr()))
        n = ctypes.c_int64()
        nat.check("ed_basis_size", self._lib.ed_basis_size(h, ctypes.byref(n)))
        self.n = int(n.value)
        r = ctypes.c_int()
        nat.check("ed_sector_is_real", self._lib.ed_sector_is_real(h, ctypes.byref(r)))
        self.is_real = bool(r.value)
        self.device = torch.device("cuda", torch.cuda.current_device())

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.ed_sector_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def dtype(self, precision: str = "fp64") -> torch.dtype:
        return _DTYPES[(precision, self.is_real)][1]

    def export_basis(self) -> tuple[np.ndarray, np.ndarray]:
        """(dense_to_sparse int64, num_sparse_in_dense int32) in the reference's format."""
        sp = torch.empty(max(self.n, 1), dtype=torch.int64, device=self.device)
        orb = torch.empty(max(self.n, 1), dtype=torch.int32, device=self.device)
        nat.check("ed_basis_export", self._lib.ed_basis_export(self._h, _ptr(sp), _ptr(orb), _stream_ptr()))
        return sp[: self.n].cpu().numpy(), orb[: self.n].cpu().numpy()

    def _code(self, t: torch.Tensor) -> int:
        code = _CODE_OF_TORCH.get(t.dtype)
        if code is None:
            raise TypeError(f"unsupported vector dtype {t.dtype}")
        if not t.is_cuda or not t.is_contiguous() or t.numel() != self.n:
            raise ValueError("vectors must be contiguous CUDA tensors of length n")
        return code

    def hv(self, x: torch.Tensor, weights, out: torch.Tensor | None = None) -> torch.Tensor:
        """y = H x (ed_hv)."""
        code = self._code(x)
        y = torch.empty_like(x) if out is None else out
        self._code(y)
        w = nat.weights_array(weights_tuple(weights))
        nat.check("ed_hv", self._lib.ed_hv(self._h, w, code, _ptr(x), _ptr(y), _stream_ptr()))
        return y

    def hv_mode(self, x: torch.Tensor, weights, mode: int, out: torch.Tensor | None = None) -> torch.Tensor:
        """y = H x with the row algorithm chosen (ed_hv_mode): 0 fast, 1 reference-faithful orbit walk."""
        code = self._code(x)
        y = torch.empty_like(x) if out is None else out
        self._code(y)
        w = nat.weights_array(weights_tuple(weights))
        nat.check("ed_hv_mode", self._lib.ed_hv_mode(self._h, w, code, _ptr(x), _ptr(y), int(mode), _stream_ptr()))
        return y

    def lanczos_step(self, weights, v: torch.Tensor, v_prev: torch.Tensor | None, v_next: torch.Tensor,
                     scal: torch.Tensor) -> None:
        """One fused step (ed_lanczos_step); scal is a float64 CUDA tensor of length >= 4."""
        code = self._code(v)
        self._code(v_next)
        if v_prev is not None:
            self._code(v_prev)
        if scal.dtype != torch.float64 or not scal.is_cuda or scal.numel() < 4:
            raise ValueError("scal must be a float64 CUDA tensor with 4 entries")
        w = nat.weights_array(weights_tuple(weights))
        nat.check("ed_lanczos_step",
                  self._lib.ed_lanczos_step(self._h, w, code, _ptr(v), _ptr(v_prev), _ptr(v_next),
                                            _ptr(scal), _stream_ptr()))

    def lanczos_hv(self, weights, v: torch.Tensor, v_prev: torch.Tensor | None, v_next: torch.Tensor,
                   scal: torch.Tensor) -> None:
        """First half of a step (ed_lanczos_hv): v_next <- H v - b v_prev, scalars on the device."""
        code = self._code(v)
        w = nat.weights_array(weights_tuple(weights))
        nat.check("ed_lanczos_hv",
                  self._lib.ed_lanczos_hv(self._h, w, code, _ptr(v), _ptr(v_prev), _ptr(v_next), _ptr(scal),
                                          _stream_ptr()))

    def lanczos_update(self, v: torch.Tensor, v_next: torch.Tensor, scal: torch.Tensor) -> None:
        """Second half of a step (ed_lanczos_update): v_next <- (v_next - a v) / b."""
        code = self._code(v)
        nat.check("ed_lanczos_update",
                  self._lib.ed_lanczos_update(self._h, code, _ptr(v), _ptr(v_next), _ptr(scal), _stream_ptr()))

    def accumulate(self, x: torch.Tensor, coef: complex, acc: torch.Tensor) -> None:
        """acc += coef * x with acc float64 (real sectors) or complex128 (ed_accumulate)."""
        code = self._code(x)
        want = torch.float64 if self.is_real else torch.complex128
        if acc.dtype != want or not acc.is_cuda or acc.numel() != self.n:
            raise ValueError(f"acc must be a {want} CUDA tensor of length n")
        c = complex(coef)
        nat.check("ed_accumulate",
                  self._lib.ed_accumulate(self._h, code, _ptr(x), c.real, c.imag, _ptr(acc), _stream_ptr()))

    def accumulate_many(self, xs: list, coefs: list, acc: torch.Tensor) -> None:
        """acc += sum_j coefs[j] * xs[j] in one pass over acc (ed_accumulate_many): the same bits as
        accumulate() called for each j in order."""
        if len(xs) != len(coefs):
            raise ValueError("one coefficient per vector")
        if not xs:
            return
        code = self._code(xs[0])
        want = torch.float64 if self.is_real else torch.complex128
        if acc.dtype != want or not acc.is_cuda or acc.numel() != self.n:
            raise ValueError(f"acc must be a {want} CUDA tensor of length n")
        for x in xs:
            if x.dtype != xs[0].dtype or not x.is_cuda or not x.is_contiguous() or x.numel() != self.n:
                raise ValueError("the vectors must be contiguous CUDA tensors of one dtype and length n")
        k = len(xs)
        ptrs = (ctypes.c_void_p * k)(*[x.data_ptr() for x in xs])
        cf = (ctypes.c_double * (2 * k))()
        for j, c in enumerate(coefs):
            c = complex(c)
            cf[2 * j], cf[2 * j + 1] = c.real, c.imag
        nat.check("ed_accumulate_many",
                  self._lib.ed_accumulate_many(self._h, code, k, ptrs, cf, _ptr(acc), _stream_ptr()))

    def project_out(self, basis: torch.Tensor, k: int, w: torch.Tensor, coef_out: torch.Tensor | None = None) -> None:
        """w <- w - sum_{j<k} <basis[j], w> basis[j] (ed_project_out); coef_out float64 (2k,) gets the dots."""
        code = self._code(w)
        if basis.dtype != w.dtype or not basis.is_contiguous() or basis.shape[-1] != self.n or basis.shape[0] < k:
            raise ValueError("basis must be a contiguous (>=k, n) tensor of the vector dtype")
        if coef_out is not None and (coef_out.dtype != torch.float64 or coef_out.numel() < 2 * k):
            raise ValueError("coef_out must be float64 with 2k entries")
        nat.check("ed_project_out", self._lib.ed_project_out(self._h, code, _ptr(basis), int(k), _ptr(w),
                                                             _ptr(coef_out), _stream_ptr()))

    def excite_into(self, dst: "DeviceSector", name: str, qx: int, qy: int, initial_sz2: int, x: torch.Tensor,
                    out: torch.Tensor | None = None) -> torch.Tensor:
        """y = O x into sector dst (ed_excitation_apply); x, y complex."""
        op = EXCITATION_OPS[str(name)]
        if x.dtype not in (torch.complex128, torch.complex64) or x.numel() != self.n or not x.is_cuda:
            raise ValueError("x must be a complex CUDA tensor of the source sector's length")
        code = _CODE_OF_TORCH[x.dtype]
        y = torch.empty(dst.n, dtype=x.dtype, device=dst.device) if out is None else out
        nat.check("ed_excitation_apply",
                  self._lib.ed_excitation_apply(self._h, dst._h, op, int(qx), int(qy), int(initial_sz2), code,
                                                _ptr(x), _ptr(y), _stream_ptr()))
        return y

    def position_correlations(self, psi: torch.Tensor, kind: str, fixed_shifts=()) -> np.ndarray:
        """Hole ("hole_correlations") or S^z ("Sz_correlations") correlations of psi over the
        distances 0..N-1 (ed_position_correlations); fixed_shifts: (leg, rung) pairs."""
        code = self._code(psi)
        k = {"hole_correlations": 0, "Sz_correlations": 1}[str(kind)]
        fixed = np.ascontiguousarray(np.asarray(fixed_shifts, dtype=np.int32).reshape(-1, 2))
        out = np.zeros(2 * self.key.num_rungs, dtype=np.float64)
        nat.check("ed_position_correlations",
                  self._lib.ed_position_correlations(
                      self._h, code, _ptr(psi), k, len(fixed),
                      fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if len(fixed) else None,
                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _stream_ptr()))
        return out

    def singlet_correlations(self, psi: torch.Tensor, fixed_shifts) -> np.ndarray:
        """Re <psi|O(t)|psi> of the singlet-pair operator for the free shifts t = 0..N-1
        (ed_singlet_correlations); fixed_shifts: the two (leg, rung) fixed distances."""
        code = self._code(psi)
        fixed = np.ascontiguousarray(np.asarray(fixed_shifts, dtype=np.int32).reshape(4))
        out = np.zeros(2 * self.key.num_rungs, dtype=np.float64)
        nat.check("ed_singlet_correlations",
                  self._lib.ed_singlet_correlations(self._h, code, _ptr(psi),
                                                    fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                    _stream_ptr()))
        return out

    def normalize(self, x: torch.Tensor, norm_out: torch.Tensor) -> None:
        code = self._code(x)
        nat.check("ed_normalize", self._lib.ed_normalize(self._h, code, _ptr(x), _ptr(norm_out), _stream_ptr()))


def batch_lanczos(sectors: list, weights, v0s: list, num_lanczos_vecs: int, use_graph: bool = True):
    """Spectrum recursions of several sectors at once (ed_batch_lanczos).

    Returns one (a, b, |v0|) per sector, truncated like _lanczos_get_anbn.
    """
    from exactdiag_gb300 import autotune

    lib = nat.load()
    m = int(num_lanczos_vecs)
    nsec = len(sectors)
    stride = 2 * m + 4
    # every sector gets its tuned work shape (its plan, as when it runs alone); the batch launches with
    # the first sector's launch
    for s in sectors[::-1]:
        autotune.ensure(s, weights, v0s[0].dtype)
    dev = sectors[0].device
    coef = torch.zeros(nsec * stride, dtype=torch.float64, device=dev)
    code = _CODE_OF_TORCH[v0s[0].dtype]
    for s, v in zip(sectors, v0s):
        s._code(v)
        if v.dtype != v0s[0].dtype:
            raise TypeError("all start vectors must share a dtype")
    harr = (ctypes.c_void_p * nsec)(*[s._h.value for s in sectors])
    varr = (ctypes.c_void_p * nsec)(*[v.data_ptr() for v in v0s])
    w = nat.weights_array(weights_tuple(weights))
    nat.check("ed_batch_lanczos", lib.ed_batch_lanczos(harr, nsec, w, code, varr, m, _ptr(coef), int(bool(use_graph)),
                                                       _stream_ptr()))
    x = coef.view(nsec, stride).cpu().numpy()
    out = []
    for s in range(nsec):
        a = x[s, 1: 2 * m: 2].copy()
        b_next = x[s, 2: 2 * m + 1: 2].copy()
        k = m
        small = np.nonzero(b_next < 1e-8)[0]
        if len(small):
            k = int(small[0]) + 1
        b = np.concatenate([[0.0], b_next[: k - 1]])
        out.append((a[:k], b[:k], float(x[s, stride - 1])))
    return out


def continued_fraction(a: torch.Tensor, b: torch.Tensor, omegas: torch.Tensor, e0: float, eta: float,
                       norm2: float) -> torch.Tensor:
    """S(omega) on the device (ed_continued_fraction); a, b, omegas float64 CUDA tensors."""
    lib = nat.load()
    out = torch.empty_like(omegas)
    m = int(a.numel())
    nat.check("ed_continued_fraction",
              lib.ed_continued_fraction(_ptr(a), _ptr(b), m, _ptr(omegas), int(omegas.numel()), float(e0),
                                        float(eta), float(norm2), _ptr(out), _stream_ptr()))
    return out
