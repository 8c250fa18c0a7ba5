import json
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger CPU cases")


@pytest.fixture(scope="session")
def reference_fixtures():
    """The reference's 68 basis-size / eigenvalue fixtures (tests/golden/reference_fixtures.json)."""
    return json.loads((GOLDEN / "reference_fixtures.json").read_text())


@pytest.fixture(scope="session")
def reference_correlations():
    """The reference's position-correlation fixtures (tests/golden/reference_correlations.json)."""
    return json.loads((GOLDEN / "reference_correlations.json").read_text())


@pytest.fixture(scope="session")
def golden_sectors():
    return np.load(GOLDEN / "sectors.npz")


@pytest.fixture(scope="session")
def golden_excitations():
    return np.load(GOLDEN / "excitations.npz")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from exactdiag_gb300 import build

    build.build()
    return torch


def seeded_vector(n, seed, complex_):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, n)
    if complex_:
        x = x + 1j * rng.uniform(-1, 1, n)
    return x.astype(np.complex128)


def fixture_sector(d):
    return (d["num_rungs"], d["num_holes"], d["num_down_spins"], d["symmetry_qs"][0], d["symmetry_qs"][1])


@pytest.fixture()
def in_tmp(tmp_path, monkeypatch):
    """Run in a temporary folder (the API writes its cache files under ./calculations)."""
    monkeypatch.chdir(tmp_path)
    from exactdiag_gb300.tJ_spin_half_ladder import matrix_setup

    yield tmp_path
    matrix_setup.clear_sector_cache()
