"""GPU: the allocation-free projection entry point against the allocating one.

ed_project_out_noalloc exists for callers that cannot let the library call cudaMalloc during a
call: services running under a fixed device-memory budget or their own allocator, and callers that
may not synchronise the device mid-work.  It keeps its scratch in a fixed device array (k <= 256
vectors).
This file is collected last so that a failing run has already run every other test; it also
passes on its own in a fresh process.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vectors(torch, sec, k, seed, dtype):
    rng = np.random.default_rng(seed)
    re = rng.uniform(-1, 1, (k, sec.n))
    if dtype.is_complex:
        return torch.as_tensor(re + 1j * rng.uniform(-1, 1, (k, sec.n)), device=sec.device).to(dtype)
    return torch.as_tensor(re, device=sec.device).to(dtype)


@pytest.mark.parametrize("key", [(8, 2, 7, 0, 0), (7, 2, 6, 2, 1)])
def test_noalloc_projection_matches_allocating_entry_point(cuda, key):
    torch = cuda
    from exactdiag_gb300 import _native as nat
    from exactdiag_gb300.engine import DeviceSector, _stream_ptr

    lib = nat.load()
    sec = DeviceSector(*key)
    dt = sec.dtype("fp64")
    code = nat.ED_F64 if not dt.is_complex else nat.ED_C128
    # two calls in a row with different inputs: the shared scratch keeps the previous call's data
    for call, k in enumerate((7, 23)):
        V = _vectors(torch, sec, k, 100 + call, dt)
        w = _vectors(torch, sec, 1, 200 + call, dt)[0]
        w_ref, w_new = w.clone(), w.clone()
        c_ref = torch.zeros(2 * k, dtype=torch.float64, device=sec.device)
        c_new = torch.full((2 * k,), float("nan"), dtype=torch.float64, device=sec.device)
        nat.check("ed_project_out", lib.ed_project_out(sec.handle, code, ctypes.c_void_p(V.data_ptr()), k,
                                                       ctypes.c_void_p(w_ref.data_ptr()),
                                                       ctypes.c_void_p(c_ref.data_ptr()), _stream_ptr()))
        nat.check("ed_project_out_noalloc",
                  lib.ed_project_out_noalloc(sec.handle, code, ctypes.c_void_p(V.data_ptr()), k,
                                             ctypes.c_void_p(w_new.data_ptr()), ctypes.c_void_p(c_new.data_ptr()),
                                             _stream_ptr()))
        torch.cuda.synchronize()
        scale = float(torch.max(torch.abs(w_ref)).item())
        assert float(torch.max(torch.abs(w_new - w_ref)).item()) <= 1e-12 * max(1.0, scale)
        assert float(torch.max(torch.abs(c_new - c_ref)).item()) <= 1e-12 * max(1.0, float(torch.max(torch.abs(c_ref))))


def test_noalloc_projection_rejects_too_many_vectors(cuda):
    torch = cuda
    from exactdiag_gb300 import _native as nat
    from exactdiag_gb300.engine import DeviceSector, _stream_ptr

    lib = nat.load()
    sec = DeviceSector(4, 2, 3, 0, 0)
    V = torch.zeros(257, sec.n, dtype=torch.float64, device=sec.device)
    w = torch.zeros(sec.n, dtype=torch.float64, device=sec.device)
    rc = lib.ed_project_out_noalloc(sec.handle, nat.ED_F64, ctypes.c_void_p(V.data_ptr()), 257,
                                    ctypes.c_void_p(w.data_ptr()), None, _stream_ptr())
    assert rc == -5
    assert b"at most 256" in lib.ed_last_error_string()
