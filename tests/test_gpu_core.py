"""GPU parity: basis, H.v, Lanczos step and continued fraction against the oracle and golden fixtures.

All calls go through the C ABI (libexactdiag_gb300.so via exactdiag_gb300.engine).
Tolerances: integer/index work bit-exact; FP64 H.v 1e-12 absolute (entries are
O(10)); FP32/complex64 H.v 2e-5 relative to max|y|.
"""

import numpy as np
import pytest
import scipy.special

from conftest import fixture_sector, seeded_vector

pytestmark = pytest.mark.gpu

W = {"tl": 1.0, "tr": 1.0, "jl": 0.5, "jr": 0.5}
SECTORS = [
    (3, 0, 3, 0, 0), (3, 1, 2, 1, 1), (4, 2, 3, 0, 0), (4, 2, 3, 1, 0), (4, 1, 3, 2, 1), (4, 3, 2, 1, 1),
    (5, 2, 4, 1, 1), (5, 3, 3, 2, 0), (5, 0, 5, 2, 1), (6, 0, 6, 0, 0), (6, 0, 6, 3, 1), (6, 1, 5, 2, 1),
    (6, 2, 5, 3, 0), (6, 4, 4, 1, 1), (6, 2, 4, -2, 1), (6, 2, 4, 8, 0), (7, 2, 6, 2, 1), (7, 1, 6, 0, 0),
    (8, 2, 7, 0, 0), (8, 2, 7, 3, 1), (8, 0, 8, 4, 0), (8, 4, 5, 1, 0),
]


def _real(key):
    return (2 * (key[3] % key[0])) % key[0] == 0


@pytest.fixture(scope="module")
def torch(cuda):
    return cuda


def _sector(key):
    from exactdiag_gb300.engine import DeviceSector

    return DeviceSector(*key)


@pytest.mark.parametrize("key", SECTORS)
def test_basis_bit_exact_vs_oracle(torch, oracle, key):
    sec = _sector(key)
    sp, orb = sec.export_basis()
    osp, oorb = oracle.basis(oracle.Sector(*key))
    assert sec.n == len(osp)
    assert np.array_equal(sp, osp)
    assert np.array_equal(orb, oorb)


def test_basis_sizes_vs_reference_fixtures(torch, reference_fixtures):
    for d in reference_fixtures:
        sec = _sector(fixture_sector(d))
        assert sec.n == d["basis_size"], d["file"]


def test_basis_vs_golden(torch, golden_sectors):
    for key in golden_sectors["sectors"]:
        key = tuple(int(v) for v in key)
        tag = "s%d_%d_%d_%d_%d" % key
        sp, orb = _sector(key).export_basis()
        assert np.array_equal(sp, golden_sectors[f"{tag}_sparse"])
        assert np.array_equal(orb, golden_sectors[f"{tag}_orbit"].astype(np.int32))


def _to_dev(torch, x, sec, precision):
    dt = sec.dtype(precision)
    arr = x.real if sec.is_real else x
    return torch.as_tensor(np.ascontiguousarray(arr)).to(device=sec.device, dtype=dt)


@pytest.mark.parametrize("key", SECTORS)
def test_hv_fp64_vs_oracle(torch, oracle, key):
    sec = _sector(key)
    osec = oracle.Sector(*key)
    h = oracle.hamiltonian(osec, W, oracle.basis(osec))
    x = seeded_vector(sec.n, 7, not sec.is_real)
    if sec.is_real:
        x = x.real.astype(np.complex128)
    y_ref = h @ x
    y = sec.hv(_to_dev(torch, x, sec, "fp64"), W).cpu().numpy()
    assert np.max(np.abs(y - y_ref)) < 1e-12


def test_hv_vs_golden(torch, golden_sectors):
    w = dict(zip(("tl", "tr", "jl", "jr"), golden_sectors["weights"]))
    for key in golden_sectors["sectors"]:
        key = tuple(int(v) for v in key)
        tag = "s%d_%d_%d_%d_%d" % key
        sec = _sector(key)
        x = seeded_vector(sec.n, int(golden_sectors[f"{tag}_seed"][0]), not _real(key))
        y = sec.hv(_to_dev(torch, x, sec, "fp64"), w).cpu().numpy()
        assert np.max(np.abs(y - golden_sectors[f"{tag}_y"])) < 1e-12


@pytest.mark.parametrize("key", [(6, 2, 5, 3, 0), (7, 2, 6, 2, 1), (8, 2, 7, 0, 0), (8, 2, 7, 3, 1)])
def test_hv_fp32_vs_fp64(torch, key):
    sec = _sector(key)
    x = seeded_vector(sec.n, 11, not sec.is_real)
    y64 = sec.hv(_to_dev(torch, x, sec, "fp64"), W).cpu().numpy()
    y32 = sec.hv(_to_dev(torch, x, sec, "fp32"), W).cpu().numpy()
    assert np.max(np.abs(y32 - y64)) <= 2e-5 * np.max(np.abs(y64))


@pytest.mark.parametrize("weights", [{"tl": 0.7, "tr": 0, "jl": 0, "jr": 0}, {"tl": 0, "tr": -1.3, "jl": 0, "jr": 0},
                                     {"tl": 0, "tr": 0, "jl": 0.25, "jr": 0}, {"tl": 0, "tr": 0, "jl": 0, "jr": 2.0},
                                     {"tl": 1, "tr": 0.3, "jl": 0.4, "jr": 1e-7}])
def test_hv_single_terms(torch, oracle, weights):
    key = (6, 2, 5, 1, 1)
    sec = _sector(key)
    osec = oracle.Sector(*key)
    h = oracle.hamiltonian(osec, weights, oracle.basis(osec))
    x = seeded_vector(sec.n, 3, True)
    y = sec.hv(_to_dev(torch, x, sec, "fp64"), weights).cpu().numpy()
    assert np.max(np.abs(y - h @ x)) < 1e-12


def test_hv_deterministic(torch):
    sec = _sector((8, 2, 7, 3, 1))
    x = _to_dev(torch, seeded_vector(sec.n, 5, True), sec, "fp32")
    y1 = sec.hv(x, W)
    y2 = sec.hv(x, W)
    assert torch.equal(y1, y2)


def test_lanczos_coefficients_vs_golden(torch, golden_sectors):
    from exactdiag_gb300.lanczos import lanczos_coefficients, tridiagonal_eigvals

    w = dict(zip(("tl", "tr", "jl", "jr"), golden_sectors["weights"]))
    for key in golden_sectors["sectors"]:
        key = tuple(int(v) for v in key)
        tag = "s%d_%d_%d_%d_%d" % key
        sec = _sector(key)
        v0 = seeded_vector(sec.n, int(golden_sectors[f"{tag}_seed"][1]), False)
        for graph in (False, True):
            a, b, nrm = lanczos_coefficients(sec, w, _to_dev(torch, v0, sec, "fp64"), 30, use_graph=graph)
            ga, gb = golden_sectors[f"{tag}_a"], golden_sectors[f"{tag}_b"]
            assert len(a) == len(ga)
            # the recursion amplifies rounding differences late in long runs; compare the first steps tightly
            k = min(len(a), 12)
            assert np.max(np.abs(a[:k] - ga[:k])) < 1e-9
            assert np.max(np.abs(b[:k] - gb[:k])) < 1e-9
            assert abs(nrm - np.linalg.norm(v0)) < 1e-10
            # past step 12 the coefficients themselves drift apart (two FP64 runs that differ in the last
            # bit of a dot product diverge roughly threefold per step once Ritz values converge), but what
            # the whole recursion computes is pinned: the extremal eigenvalues of the 30-step tridiagonal
            # matrix, which converge to eigenvalues of H in both runs
            ritz, gritz = tridiagonal_eigvals(a, b), tridiagonal_eigvals(ga, gb)
            scale = max(1.0, float(np.max(np.abs(gritz))))
            assert abs(ritz[0] - gritz[0]) <= 1e-10 * scale, (tag, ritz[0], gritz[0])
            assert abs(ritz[-1] - gritz[-1]) <= 1e-10 * scale, (tag, ritz[-1], gritz[-1])


def test_continued_fraction_vs_oracle(torch, oracle):
    from exactdiag_gb300.engine import continued_fraction

    rng = np.random.default_rng(5)
    a = rng.uniform(-2, 2, 150)
    b = np.concatenate([[0.0], rng.uniform(0.1, 1.0, 149)])
    om = np.linspace(0, 6, 2000)
    e0, eta, n2 = -3.2, 0.05, 1.7
    dev = lambda v: torch.as_tensor(v, dtype=torch.float64, device="cuda")
    s = continued_fraction(dev(a), dev(b), dev(om), e0, eta, n2).cpu().numpy()
    ref = oracle.continued_fraction(a, b, om + e0 + 1j * eta, n2)
    assert np.max(np.abs(s - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))


def test_sum_over_k_full_size(torch):
    # size-independent invariant at a configuration far beyond the oracle's reach: 2x12, 2 holes
    L, Nh, Nd = 12, 2, 11
    total = 0
    for kx in range(L):
        for ky in (0, 1):
            total += _sector((L, Nh, Nd, kx, ky)).n
    assert total == scipy.special.comb(2 * L, Nh, exact=True) * scipy.special.comb(2 * L - Nh, Nd, exact=True)


@pytest.mark.parametrize("key", [(10, 2, 9, 0, 0), (10, 2, 9, 3, 1)])
def test_hv_hermitian_full_size(torch, key):
    sec = _sector(key)
    x = _to_dev(torch, seeded_vector(sec.n, 21, not sec.is_real), sec, "fp64")
    z = _to_dev(torch, seeded_vector(sec.n, 22, not sec.is_real), sec, "fp64")
    hx = sec.hv(x, W)
    hz = sec.hv(z, W)
    lhs = torch.vdot(z, hx).item()
    rhs = torch.vdot(hz, x).item()
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


@pytest.mark.parametrize("key", [(8, 2, 7, 3, 1), (9, 3, 7, 2, 0), (8, 4, 6, 4, 1), (10, 2, 9, 0, 0), (10, 2, 9, 5, 1),
                                 (10, 1, 9, 3, 0), (8, 0, 8, 2, 1), (12, 2, 11, 0, 0), (12, 2, 11, 6, 1),
                                 (12, 2, 11, 5, 0), (11, 3, 9, 2, 1)])
def test_fast_rows_equal_faithful_orbit_walk(torch, key):
    """The descriptor-driven rows (colex deltas, coset permutations) and the fused step kernels
    (ed_hv: segments, expanded copies) against the reference-faithful walk."""
    sec = _sector(key)
    x = _to_dev(torch, seeded_vector(sec.n, 41, not sec.is_real), sec, "fp64")
    y_fast = sec.hv_mode(x, W, 0)
    y_step = sec.hv(x, W)
    y_walk = sec.hv_mode(x, W, 1)
    scale = float(torch.max(torch.abs(y_walk)).item())
    assert float(torch.max(torch.abs(y_fast - y_walk)).item()) < 1e-12 * max(1.0, scale)
    assert float(torch.max(torch.abs(y_step - y_walk)).item()) < 1e-12 * max(1.0, scale)


def test_fast_rows_equal_faithful_orbit_walk_2x14(torch):
    """Full-size check of the fast rows and of the fused step kernels on the 2x14 two-hole sector
    (1.4e8 rows), FP64; and of the FP32 step kernels against the FP64 walk at FP32 resolution."""
    sec = _sector((14, 2, 13, 0, 0))
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.rand(sec.n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    y_walk = sec.hv_mode(x, W, 1)
    scale = float(torch.max(torch.abs(y_walk)).item())
    y = sec.hv_mode(x, W, 0)
    assert float(torch.max(torch.abs(y - y_walk)).item()) < 1e-12 * scale
    y = sec.hv(x, W)
    assert float(torch.max(torch.abs(y - y_walk)).item()) < 1e-12 * scale
    y = sec.hv(x.float(), W)
    assert float(torch.max(torch.abs(y.double() - y_walk)).item()) < 2e-5 * scale
