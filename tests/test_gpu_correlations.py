"""GPU: hole and S^z position correlations against the oracle and the reference's fixtures."""

import numpy as np
import pytest

from conftest import seeded_vector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("key", [(6, 2, 5, 0, 0), (6, 2, 5, 2, 1), (5, 1, 4, 1, 0), (6, 4, 4, 3, 1), (5, 0, 5, 0, 1)])
@pytest.mark.parametrize("name", ["hole_correlations", "Sz_correlations"])
@pytest.mark.parametrize("fixed", [(), ((1, 1),), ((0, 1), (-2, 0))])
def test_position_correlations_vs_oracle(cuda, oracle, key, name, fixed):
    torch = cuda
    from exactdiag_gb300.engine import DeviceSector

    sec = DeviceSector(*key)
    osec = oracle.Sector(*key)
    bas = oracle.basis(osec)
    psi = seeded_vector(len(bas[0]), 9, not sec.is_real)
    if sec.is_real:
        psi = psi.real
    psi = psi / np.linalg.norm(psi)
    want = oracle.position_correlations(osec, bas, psi, name, fixed)
    dev = torch.as_tensor(psi, device=sec.device)
    got = sec.position_correlations(dev, name, fixed)
    assert np.max(np.abs(got - want)) < 1e-12


def test_hole_correlations_match_reference_fixtures(cuda, reference_correlations, in_tmp):
    """The reference's published hole correlations (its test_position_correlations.py), to the
    listed precision 1e-3, normalised to the first entry like the reference's test."""
    from exactdiag_gb300.tJ_spin_half_ladder import api
    from exactdiag_gb300.tJ_spin_half_ladder import configs as lc

    checked = 0
    for d in reference_correlations:
        if d["correlations"]["name"] != "hole_correlations":
            continue
        d = {k: v for k, v in d.items() if k != "file"}
        target = d.pop("probabilities")
        config = lc.Full_Position_Correlation_Config(**d)
        probabilities = api.get_position_correlations(config).spectrum.flatten()
        probabilities = probabilities / probabilities[0]
        diff = probabilities[: len(target)] - np.asarray(target)
        assert np.all(np.abs(diff) < 1e-3), (d["hamiltonian"], diff)
        checked += 1
    assert checked == 16


@pytest.mark.parametrize("key", [(5, 2, 4, 0, 0), (6, 4, 4, 0, 0), (5, 3, 3, 2, 1), (6, 2, 5, 1, 0)])
@pytest.mark.parametrize("fixed", [((1, 1), (1, 1)), ((1, 0), (0, 1)), ((0, 1), (1, 0))])
def test_singlet_correlations_vs_oracle(cuda, oracle, key, fixed):
    torch = cuda
    from exactdiag_gb300.engine import DeviceSector

    sec = DeviceSector(*key)
    osec = oracle.Sector(*key)
    bas = oracle.basis(osec)
    psi = seeded_vector(len(bas[0]), 13, not sec.is_real)
    if sec.is_real:
        psi = psi.real
    psi = psi / np.linalg.norm(psi)
    want = oracle.singlet_correlations(osec, bas, psi.astype(np.complex128), fixed)
    got = sec.singlet_correlations(torch.as_tensor(psi, device=sec.device), fixed)
    assert np.max(np.abs(got - want)) < 1e-12


def test_singlet_correlations_match_reference_fixtures(cuda, reference_correlations, in_tmp):
    """The reference's published singlet-singlet correlations (its test_position_correlations.py),
    unnormalised, to the listed precision 1e-3."""
    from exactdiag_gb300.tJ_spin_half_ladder import api
    from exactdiag_gb300.tJ_spin_half_ladder import configs as lc

    checked = 0
    for d in reference_correlations:
        if d["correlations"]["name"] != "singlet-singlet":
            continue
        d = {k: v for k, v in d.items() if k != "file"}
        target = d.pop("probabilities")
        config = lc.Full_Position_Correlation_Config(**d)
        values = api.get_position_correlations(config).spectrum.flatten()
        diff = values[: len(target)] - np.asarray(target)
        assert np.all(np.abs(diff) < 1e-3), (d["hamiltonian"]["weights"], d["correlations"], diff)
        checked += 1
    assert checked == 18
