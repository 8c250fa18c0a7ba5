"""GPU: the fused Lanczos step kernels (one per block kind) against the one-thread-per-row H.v kernel.

ed_lanczos_hv with no previous vector writes y = H v and the step's partial sums; y must equal
ed_hv_mode(..., 0)'s H v (an independent row algorithm, pinned by the core tests to the oracle and
to the reference-faithful orbit walk), and <v, Hv> must equal the FP64 dot product of the two
vectors.
"""

import numpy as np
import pytest

from conftest import seeded_vector

pytestmark = pytest.mark.gpu

W = {"tl": 1.0, "tr": 1.0, "jl": 0.5, "jr": 0.5}
# weight sets that take the step kernels' other branches: rung and leg exchange weights that differ
# (per-bond coefficients), terms switched off (absent hops, one exchange kind off), negative hopping
WEIGHTS = [W, {"tl": 1.0, "tr": 0.7, "jl": 0.5, "jr": 0.3}, {"tl": 1.0, "tr": 0.0, "jl": 0.5, "jr": 0.5},
           {"tl": 0.0, "tr": -1.3, "jl": 0.0, "jr": 0.4}, {"tl": 0.6, "tr": 1.0, "jl": 0.35, "jr": 0.0}]
SMALL = [(6, 2, 5, kx, ky) for kx in range(6) for ky in (0, 1)] + [(7, 3, 5, 2, 1), (8, 4, 6, 3, 0), (6, 0, 6, 1, 1),
                                                                   (8, 1, 7, 5, 1), (5, 5, 0, 0, 0)]
FULL = [(12, 2, 11, kx, ky) for kx in range(12) for ky in (0, 1)]


def _check(torch, key, precision, tol, w=W):
    from exactdiag_gb300.engine import DeviceSector

    sec = DeviceSector(*key)
    dt = sec.dtype(precision)
    x = seeded_vector(sec.n, 17, not sec.is_real)
    v = torch.as_tensor(x if not sec.is_real else x.real, device=sec.device).to(dt)
    ref = sec.hv_mode(v, w, 0)
    y = torch.zeros_like(v)
    scal = torch.zeros(8, dtype=torch.float64, device=sec.device)
    sec.lanczos_hv(w, v, None, y, scal[0:4])
    torch.cuda.synchronize()
    scale = max(1.0, float(torch.max(torch.abs(ref)).item()))
    err = float(torch.max(torch.abs(y - ref)).item())
    assert err <= tol * scale, (key, precision, err)
    a = float(scal[1].item())
    a_ref = float(torch.vdot(v.to(torch.complex128 if v.is_complex() else torch.float64),
                             ref.to(torch.complex128 if v.is_complex() else torch.float64)).real.item())
    assert abs(a - a_ref) <= 1e-9 * max(1.0, abs(a_ref)) * (1 if precision == "fp64" else 1e3), (key, a, a_ref)


@pytest.mark.parametrize("key", SMALL)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("w", range(len(WEIGHTS)))
def test_step_kernel_equals_hv_small(cuda, key, precision, w):
    _check(cuda, key, precision, 1e-12 if precision == "fp64" else 1e-6, WEIGHTS[w])


@pytest.mark.parametrize("key", [(6, 2, 5, 1, 1), (7, 3, 5, 2, 1), (5, 2, 4, 0, 0)])
@pytest.mark.parametrize("w", range(1, len(WEIGHTS)))
def test_step_kernel_vs_oracle_weights(cuda, oracle, key, w):
    """The step kernel's y = H v against the oracle's matrix directly, for the weight sets that
    take the per-bond coefficient, absent-hop and exchange-off branches."""
    torch = cuda
    from exactdiag_gb300.engine import DeviceSector

    weights = WEIGHTS[w]
    sec = DeviceSector(*key)
    osec = oracle.Sector(*key)
    h = oracle.hamiltonian(osec, weights, oracle.basis(osec))
    x = seeded_vector(sec.n, 29, not sec.is_real)
    if sec.is_real:
        x = x.real
    v = torch.as_tensor(x, device=sec.device)
    y = torch.zeros_like(v)
    scal = torch.zeros(8, dtype=torch.float64, device=sec.device)
    sec.lanczos_hv(weights, v, None, y, scal[0:4])
    assert np.max(np.abs(y.cpu().numpy() - h @ x)) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_step_kernel_equals_hv_2x12_all_sectors(cuda, precision):
    for key in FULL:
        _check(cuda, key, precision, 1e-12 if precision == "fp64" else 1e-6)


@pytest.mark.parametrize("key", [(12, 2, 11, 0, 0), (12, 2, 11, 5, 1)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_step_shapes(cuda, key, precision):
    """Every launch variant and rows-per-lane choice gives the same bits; every chunk length gives
    the step kernel's y = H v (the one-thread-per-row H v, to the form's tolerance), and a sector
    re-planned back to its first chunk length gives its first bits again."""
    torch = cuda
    from exactdiag_gb300 import _native as nat
    from exactdiag_gb300 import autotune
    from exactdiag_gb300.engine import DeviceSector

    sec = DeviceSector(*key)
    dt = sec.dtype(precision)
    x = seeded_vector(sec.n, 23, not sec.is_real)
    v = torch.as_tensor(x if not sec.is_real else x.real, device=sec.device).to(dt)
    ref = sec.hv_mode(v, W, 0)
    tol = 1e-12 if precision == "fp64" else 1e-6
    scale = max(1.0, float(torch.max(torch.abs(ref)).item()))

    def step():
        y = torch.zeros_like(v)
        scal = torch.zeros(8, dtype=torch.float64, device=sec.device)
        sec.lanczos_hv(W, v, None, y, scal[0:4])
        torch.cuda.synchronize()
        return y, scal[:4].cpu().numpy()

    first_y, first_s = step()
    shapes = [(minb, ctas, nr, 0) for minb, ctas in autotune.CANDIDATES for nr in (1, 2)]
    shapes += [(minb, ctas, nr, 1) for minb, ctas, nr in autotune.STAGED_CANDIDATES]
    for minb, ctas, nr, staged in shapes:
        autotune.set_launch(sec, minb, ctas)
        autotune.set_step_shape(sec, nr, autotune.DEFAULT_CHUNK_ROWS, staged)
        y, s = step()
        assert torch.equal(y, first_y) and np.array_equal(s, first_s), (minb, ctas, nr, staged)
    autotune.set_step_shape(sec, 0, autotune.DEFAULT_CHUNK_ROWS, 0)
    for rows in (1024, 4096, 8192, 32768, 65536):
        autotune.set_step_shape(sec, 0, rows)
        assert autotune.get_step_shape(sec) == (0, rows, 0)
        y, s = step()
        assert float(torch.max(torch.abs(y - ref)).item()) <= tol * scale, rows
        assert abs(s[1] - first_s[1]) <= 1e-9 * max(1.0, abs(first_s[1])) * (1 if precision == "fp64" else 1e3)
    autotune.set_step_shape(sec, 0, autotune.DEFAULT_CHUNK_ROWS)
    y, s = step()
    assert torch.equal(y, first_y) and np.array_equal(s, first_s)
    for bad in ((3, 16384, 0), (-1, 16384, 0), (1, 12288, 0), (1, 512, 0), (2, 131072, 0), (1, 16384, 2)):
        with pytest.raises(nat.EngineError):
            autotune.set_step_shape(sec, *bad)


@pytest.mark.parametrize("key", [(12, 2, 11, 0, 0), (12, 2, 11, 5, 1)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("weights", ["merged", "split"])
def test_segment_windows(cuda, key, precision, weights):
    """64-offset segment windows (a lane's two rows in one segment): every launch variant gives the
    same bits, y = H v to the form's tolerance, staged gathers refused with them, and a sector
    re-planned back to 32-offset windows gives its first bits again."""
    torch = cuda
    from exactdiag_gb300 import _native as nat
    from exactdiag_gb300 import autotune
    from exactdiag_gb300.engine import DeviceSector

    w = W if weights == "merged" else {"tl": 1.0, "tr": 0.7, "jl": 0.5, "jr": 0.3}
    sec = DeviceSector(*key)
    dt = sec.dtype(precision)
    x = seeded_vector(sec.n, 29, not sec.is_real)
    v = torch.as_tensor(x if not sec.is_real else x.real, device=sec.device).to(dt)
    ref = sec.hv_mode(v, w, 0)
    tol = 1e-12 if precision == "fp64" else 1e-6
    scale = max(1.0, float(torch.max(torch.abs(ref)).item()))

    def step():
        y = torch.zeros_like(v)
        scal = torch.zeros(8, dtype=torch.float64, device=sec.device)
        sec.lanczos_hv(w, v, None, y, scal[0:4])
        torch.cuda.synchronize()
        return y, scal[:4].cpu().numpy()

    first_y, first_s = step()
    assert autotune.get_window(sec) == 32
    autotune.set_window(sec, 64)
    assert autotune.get_window(sec) == 64
    y64, s64 = step()
    assert float(torch.max(torch.abs(y64 - ref)).item()) <= tol * scale
    assert abs(s64[1] - first_s[1]) <= 1e-9 * max(1.0, abs(first_s[1])) * (1 if precision == "fp64" else 1e3)
    for minb, ctas in autotune.CANDIDATES:
        for nr in (1, 2):
            autotune.set_launch(sec, minb, ctas)
            autotune.set_step_shape(sec, nr, autotune.DEFAULT_CHUNK_ROWS, 0)
            y, s = step()
            assert torch.equal(y, y64) and np.array_equal(s, s64), (minb, ctas, nr)
    with pytest.raises(nat.EngineError):
        autotune.set_step_shape(sec, 0, autotune.DEFAULT_CHUNK_ROWS, 1)
    for bad in (0, 16, 48, 128):
        with pytest.raises(nat.EngineError):
            autotune.set_window(sec, bad)
    autotune.set_window(sec, 32)
    autotune.set_launch(sec, 3, 0)
    autotune.set_step_shape(sec, 0, autotune.DEFAULT_CHUNK_ROWS, 1)
    with pytest.raises(nat.EngineError):
        autotune.set_window(sec, 64)
    autotune.set_step_shape(sec, 0, autotune.DEFAULT_CHUNK_ROWS, 0)
    y, s = step()
    assert torch.equal(y, first_y) and np.array_equal(s, first_s)
