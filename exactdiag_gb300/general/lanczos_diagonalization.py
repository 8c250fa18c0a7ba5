"""Eigenpairs and dynamical spectra on the GPU (mirrors general/lanczos_diagonalization.py).

Same function names, arguments, cache files and averaging rules as the
reference (:21-175); the eigen-solver is the device Lanczos of
exactdiag_gb300.eigensolver, the spectrum recursion runs on the device
(fused steps, FP64 reductions) and the continued fraction is evaluated on the
device over the omega grid.
"""

from __future__ import annotations

import logging
import pathlib
from os import makedirs

import numpy as np
import torch

from exactdiag_gb300.utils import load_calculate_save

_logger = logging.getLogger(__name__)


def get_lowest_eigenpairs(config):
    """Load or calculate and save the lowest eigenpairs (:21-34)."""
    eigvals, eigvecs = load_calculate_save(*config.get_eigenpair_paths(), load_fun=load_eigenpairs,
                                           calc_fun=lambda: calculate_eigenpairs(config), save_fun=save_eigenpairs)
    _logger.info(f"Got lowest eigenpairs with k={config.hamiltonian.symmetry_qs.to_npint32()!s}, {eigvals=}")
    return eigvals, eigvecs


def load_eigenpairs(vals_path: pathlib.Path, vecs_path: pathlib.Path):
    return np.load(vals_path, allow_pickle=False), np.load(vecs_path, allow_pickle=False)


def save_eigenpairs(eigenpairs, vals_path: pathlib.Path, vecs_path: pathlib.Path) -> None:
    makedirs(vals_path.parent, exist_ok=True)
    makedirs(vecs_path.parent, exist_ok=True)
    eigvals, eigvecs = eigenpairs
    np.save(vals_path, eigvals)
    np.save(vecs_path, eigvecs)


def calculate_eigenpairs(config):
    """Lowest config.eigenpair.num_eigenpairs eigenpairs, eigvecs[:, i] normalised (:53-78)."""
    from exactdiag_gb300.eigensolver import lowest_eigenpairs

    hamiltonian = config.hamiltonian.setup()()
    if hamiltonian.shape[0] == 0:
        _logger.warning("hamiltonian has 0 rows, skipping eigen problem")
        return [], []
    k = config.eigenpair.num_eigenpairs
    # "mixed": FP32 Krylov vectors with FP64 reductions, each eigenpair refined in FP64 (eigensolver)
    eigvals, eigvecs = lowest_eigenpairs(hamiltonian.sector, hamiltonian.weights_tuple, k,
                                         precision=hamiltonian.precision)
    eigvals = np.real(eigvals)
    order = eigvals.argsort()[:k]
    return eigvals[order], eigvecs[:, order]


def get_spectrum(config, suffix: str = ""):
    """Load or calculate and save one spectrum (:124-143)."""

    def calculate():
        eigvals, eigvecs = get_lowest_eigenpairs(config)
        get_operator, _, get_excited_h = config.setup_excitation_operator()
        return calculate_spectrum(ws=config.spectrum.get_omegas(), broadening=config.spectrum.broadening,
                                  excited_state_hamiltonian=get_excited_h(), excitation_operator=get_operator(),
                                  eigvecs=eigvecs, eigvals=eigvals, num_lanczos_vecs=config.spectrum.num_lanczos_vecs,
                                  num_threads=config.spectrum.num_threads)

    ws, spectrum = load_calculate_save(config.get_spectrum_path(suffix), load_fun=load_spectrum, calc_fun=calculate,
                                       save_fun=save_spectrum)
    return ws, spectrum


def load_spectrum(path):
    npz_file = np.load(path, allow_pickle=True)
    ws, spectrum = npz_file.values()
    return ws, spectrum


def save_spectrum(ws_spectrum, path) -> None:
    path = pathlib.Path(path)
    makedirs(path.parent, exist_ok=True)
    np.savez(path, *ws_spectrum)


def _start_dtype(hamiltonian) -> torch.dtype:
    return torch.complex128 if hamiltonian.precision == "fp64" else torch.complex64


def calculate_spectrum(ws, broadening, num_lanczos_vecs, excited_state_hamiltonian, excitation_operator, eigvecs,
                       eigvals, num_threads):
    """Average the response over degenerate ground states, |E_j - E_0| <= 1e-6 (:158-175)."""
    gs_energy = eigvals[0]
    num_degenerate_states = 0
    spectrum = np.zeros(len(ws))
    zs = ws + gs_energy + 1j * broadening
    for j in range(len(eigvals)):
        if abs(gs_energy - eigvals[j]) > 1e-6:
            break
        num_degenerate_states += 1
        spectrum += lanczos_dynamical_response(eigvecs[:, j], excitation_operator, excited_state_hamiltonian, zs,
                                               num_lanczos_vecs, num_threads)
    spectrum /= num_degenerate_states
    return ws, spectrum


def lanczos_dynamical_response(initial_state, excitation_operator, excited_state_hamiltonian, zs, num_lanczos_vecs,
                               num_threads=1):
    """Spectrum of an operator applied to a state (general/cython_lanczos_diagonalization.pyx:18-40), on the GPU."""
    from exactdiag_gb300.engine import continued_fraction
    from exactdiag_gb300.lanczos import lanczos_coefficients

    zs = np.asarray(zs)
    src = excitation_operator.src
    dt = _start_dtype(excited_state_hamiltonian)
    gs = torch.as_tensor(np.asarray(initial_state, np.complex128)).to(device=src.device, dtype=dt)
    phi = excitation_operator.device_dot(gs)
    if phi.numel() == 0:
        return np.zeros(len(zs))
    sector = excited_state_hamiltonian.sector
    a, b, norm = lanczos_coefficients(sector, excited_state_hamiltonian.weights_tuple, phi, int(num_lanczos_vecs))
    if norm < 1e-8:
        return np.zeros(len(zs))
    dev = sector.device
    e0 = 0.0
    omegas = torch.as_tensor(zs.real - e0, dtype=torch.float64, device=dev)
    eta = float(zs.imag[0]) if len(zs) else 0.0
    s = continued_fraction(torch.as_tensor(a, device=dev), torch.as_tensor(b, device=dev), omegas, e0, eta, norm ** 2)
    return s.cpu().numpy()
