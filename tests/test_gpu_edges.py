"""GPU: degenerate sectors -- two-rung ladders, all holes, no down spins, empty sectors -- and the
one-rung ladder, which the engine refuses (its leg bonds would join a site to itself)."""

import numpy as np
import pytest

from conftest import seeded_vector

pytestmark = pytest.mark.gpu

W = {"tl": 1.0, "tr": 0.7, "jl": 0.5, "jr": 0.3}
NONEMPTY = [(2, 0, 2, 0, 0), (2, 0, 2, 1, 1), (2, 1, 1, 0, 0), (2, 2, 1, 1, 0), (3, 6, 0, 0, 0), (5, 2, 0, 2, 1),
            (4, 0, 4, 2, 1), (6, 12, 0, 0, 0), (3, 0, 0, 0, 1)]
EMPTY = [(3, 6, 0, 1, 1), (3, 0, 0, 0, 0), (4, 8, 0, 1, 0)]


@pytest.mark.parametrize("key", NONEMPTY + EMPTY)
def test_edge_basis_vs_oracle(cuda, oracle, key):
    from exactdiag_gb300.engine import DeviceSector

    sec = DeviceSector(*key)
    sp, orb = sec.export_basis()
    osp, oorb = oracle.basis(oracle.Sector(*key))
    assert sec.n == len(osp) and np.array_equal(sp, osp) and np.array_equal(orb, oorb)


@pytest.mark.parametrize("key", [(1, 0, 1, 0, 0), (1, 1, 0, 0, 1), (17, 2, 15, 0, 0)])
def test_rung_count_out_of_range_is_refused(cuda, key):
    from exactdiag_gb300 import _native as nat
    from exactdiag_gb300.engine import DeviceSector

    with pytest.raises(nat.EngineError, match="L must be in"):
        DeviceSector(*key)


@pytest.mark.parametrize("key", NONEMPTY)
def test_edge_hv_and_eigenvalues_vs_oracle(cuda, oracle, key):
    torch = cuda
    from exactdiag_gb300.eigensolver import lowest_eigenpairs
    from exactdiag_gb300.engine import DeviceSector, weights_tuple

    sec = DeviceSector(*key)
    osec = oracle.Sector(*key)
    bas = oracle.basis(osec)
    h = oracle.hamiltonian(osec, W, bas)
    x = seeded_vector(sec.n, 5, not sec.is_real)
    if sec.is_real:
        x = x.real
    y = sec.hv(torch.as_tensor(x, device=sec.device), W).cpu().numpy()
    assert np.max(np.abs(y - h @ x)) < 1e-12
    k = min(2, sec.n)
    vals, _ = lowest_eigenpairs(sec, weights_tuple(W), k)
    want = np.sort(np.linalg.eigvalsh(h.toarray()))[:k]
    assert np.max(np.abs(np.real(vals) - want)) < 1e-10


@pytest.mark.parametrize("key", EMPTY)
def test_empty_sector_calls(cuda, in_tmp, key):
    """An empty sector: H.v of an empty vector is empty, a Lanczos step is refused with a status,
    and the eigen problem is skipped like the reference's (lanczos_diagonalization.py:53-78)."""
    torch = cuda
    from exactdiag_gb300 import _native as nat
    from exactdiag_gb300.engine import DeviceSector
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    sec = DeviceSector(*key)
    assert sec.n == 0
    x = torch.zeros(0, dtype=sec.dtype("fp64"), device=sec.device)
    assert sec.hv(x, W).numel() == 0
    scal = torch.zeros(8, dtype=torch.float64, device=sec.device)
    with pytest.raises(nat.EngineError):
        sec.lanczos_step(W, x, None, torch.zeros_like(x), scal[:4])
    L, Nh, Nd, kx, ky = key
    cfg = configs.Eigenpair_Config(
        hamiltonian={"num_rungs": L, "num_holes": Nh, "weights": W, "symmetry_qs": {"leg": kx, "rung": ky},
                     "num_threads": 1, "total_spin_projection": 2 * L - Nh - 2 * Nd},
        eigenpair={"num_eigenpairs": 2})
    vals, vecs = api.get_eigenpairs(cfg)
    assert len(vals) == 0
