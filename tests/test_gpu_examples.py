"""GPU: the calculations of the reference's examples (examples/tJ_spin_half_ladder/*.py) run through
this package on the examples' own configurations (tests/golden/reference_examples.json).

Each test follows one example's API calls (loading the config, the api/configs/sparse_matrices
calls it makes) and checks the result against the oracle or an exact property instead of plotting.
"""

import json
import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXAMPLES = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_examples.json").read_text())


def test_all_ks_eigvals_example(cuda, oracle, in_tmp):
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    config = configs.Eigenpair_Config(**EXAMPLES["all_ks_eigvals"])
    k_to_pairs = api.get_all_k_eigenpairs(config)
    h = config.hamiltonian
    assert len(k_to_pairs) == 2 * (h.num_rungs // 2 + 1)
    for (kx, ky), (vals, vecs) in k_to_pairs.items():
        osec = oracle.Sector(h.num_rungs, h.num_holes, h.num_down_spins, kx, ky)
        bas = oracle.basis(osec)
        want = oracle.lowest_eigvals(oracle.hamiltonian(osec, vars(h.weights), bas), len(vals))
        assert vecs.shape[0] == len(bas[0])
        assert np.max(np.abs(np.asarray(vals) - want)) < 1e-8, (kx, ky)


def test_load_matrix_example(cuda, in_tmp):
    import dataclasses

    from exactdiag_gb300.general.sparse_matrices import Added_Sparse_Matrices, Sparse_Matrix
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    config = configs.Eigenpair_Config(**EXAMPLES["load_matrix"])
    eigvals, eigvecs = api.get_eigenpairs(config)
    ground_state = eigvecs[:, 0]
    weights = dataclasses.asdict(config.hamiltonian.weights)
    matrices = Added_Sparse_Matrices(*zip(*[[Sparse_Matrix.from_name(name=name, config=config.hamiltonian), weight]
                                            for name, weight in weights.items()]))
    trial_vec = matrices.dot(ground_state)
    assert np.linalg.norm(eigvals[0] * ground_state - trial_vec) < 1e-8


def test_multiple_spectra_example(cuda, in_tmp):
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    config = configs.Full_Spectrum_Config(**EXAMPLES["multiple_spectra"])
    omega_mins = {"current_rung": 0, "current_leg": -0.5, "Szq": 0, "spectral_function_plus": -2}
    L = config.hamiltonian.num_rungs
    for name, omega_min in omega_mins.items():
        config.spectrum.name = name
        config.spectrum.omega_min = omega_min
        spectrum = api.plot_excitation_spectrum(config=config, show=False, limited_qs=False)
        data = np.asarray(spectrum.spectrum)
        assert data.shape[-1] == config.spectrum.omega_steps and np.all(np.isfinite(data)), name
        if name == "Szq":
            assert data.shape[:2] == (L, 2)
        if name == "spectral_function_plus":  # one hole present: the plus and the minus parts
            assert data.shape[:2] == (2, 2 * L)


def test_rung_current_spectrum_example(cuda, in_tmp):
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    config = configs.Full_Spectrum_Config(**EXAMPLES["rung_current_spectrum"])
    spectrum = api.plot_excitation_spectrum(config=config, show=False)
    data = np.asarray(spectrum.spectrum)
    assert data.shape == (config.spectrum.omega_steps,) and np.all(np.isfinite(data)) and np.max(data) > 0


@pytest.mark.parametrize("example", ["hole_position_correlations", "untested_Sz_position_correlations"])
def test_hole_and_sz_correlation_examples(cuda, in_tmp, example):
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    config = configs.Full_Position_Correlation_Config(**EXAMPLES[example])
    spectrum = api.plot_position_correlation(config=config, show=False)
    corrs = np.asarray(spectrum.spectrum)
    h = config.hamiltonian
    assert corrs.shape == (h.num_nodes,)
    if not config.correlations.fixed_distances:  # summed over distances: Nh^2 or (2 Sz)^2
        want = h.num_holes ** 2 if config.correlations.name == "hole_correlations" else h.total_spin_projection ** 2
        assert abs(corrs.sum() - want) < 1e-9


def test_singlet_correlations_example(cuda, in_tmp):
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    config = configs.Full_Position_Correlation_Config(**EXAMPLES["singlet-singlet_correlations"])
    corrs = np.asarray(api.plot_position_correlation(config=config, show=False).spectrum)
    assert corrs.shape == (config.hamiltonian.num_nodes,) and np.all(np.isfinite(corrs))


def test_custom_figure_example_operator_is_rejected_like_the_reference(cuda, in_tmp):
    """Its off-diagonal spectral function is not supported by the reference either (api.py:83-101)."""
    from exactdiag_gb300.tJ_spin_half_ladder import api, configs

    config = configs.Full_Spectrum_Config(**EXAMPLES["custom_figure"])
    with pytest.raises(ValueError):
        api.get_excitation_spectrum(config=config)
