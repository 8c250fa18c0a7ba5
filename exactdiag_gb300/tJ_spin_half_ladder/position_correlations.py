"""Position correlations of the ground state (mirrors tJ_spin_half_ladder/position_correlations.pyx).

Hole and S^z correlations are one pass of ed_position_correlations over the device basis per
(degenerate) ground state; results are averaged over ground states within 1e-6 of the lowest
energy and cached under the reference's result path, like the reference (:28-52).  Singlet-singlet
correlations are <gs|O|gs> of the reference's singlet-pair operator (matrix_setup.pyx:434-469),
evaluated by ed_singlet_correlations from the operator's column rule without storing it.
"""

from __future__ import annotations

import numpy as np
import torch

from exactdiag_gb300.general.lanczos_diagonalization import get_lowest_eigenpairs, load_spectrum, save_spectrum
from exactdiag_gb300.tJ_spin_half_ladder import configs
from exactdiag_gb300.tJ_spin_half_ladder.matrix_setup import sector_of
from exactdiag_gb300.utils import load_calculate_save


def varied_shifts(num_nodes: int) -> np.ndarray:
    """(leg, rung) of each distance index (symmetry_ladder.h:103-108 get_unit_shifts_from_index)."""
    return np.array([[d // 2, d % 2] for d in range(num_nodes)], dtype=np.int32)


def calculate_hole_spin_projection_correlations(config, eigvec: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(varied shifts, correlations over distances) of one state (:83-118)."""
    sec = sector_of(config.hamiltonian)
    dt = torch.float64 if sec.is_real else torch.complex128
    vec = np.asarray(eigvec)
    if sec.is_real:
        vec = vec.real
    psi = torch.as_tensor(np.ascontiguousarray(vec), device=sec.device).to(dt)
    fixed = [shift.to_npint32() for shift in config.correlations.fixed_distances]
    corrs = sec.position_correlations(psi, str(config.correlations.name), fixed)
    return varied_shifts(config.hamiltonian.num_nodes), corrs


def get_hole_spin_projection_correlations(config: configs.Full_Position_Correlation_Config):
    """Correlations averaged over the degenerate ground states, loaded or computed and saved (:28-52)."""

    def calculate():
        eigvals, eigvecs = get_lowest_eigenpairs(config)
        num_degenerate_states = 0
        spectrum = None
        shifts = None
        for j in range(len(eigvals)):
            if abs(eigvals[0] - eigvals[j]) > 1e-6:
                break
            num_degenerate_states += 1
            shifts, corrs = calculate_hole_spin_projection_correlations(config, eigvecs[:, j])
            spectrum = corrs if spectrum is None else spectrum + corrs
        return shifts, spectrum / num_degenerate_states

    return load_calculate_save(config.get_spectrum_path(), load_fun=load_spectrum, calc_fun=calculate,
                               save_fun=save_spectrum)


def calculate_singlet_singlet_correlations(config, eigvec: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(varied shifts, Re <gs|O(shift)|gs> per free shift) of one state (:112-124) with the
    singlet-pair operator of matrix_setup.pyx:434-469; fixed_distances = [y, x] (the creation and
    annihilation singlets' structure)."""
    fixed = config.correlations.fixed_distances
    if len(fixed) != 2:
        raise ValueError("singlet-singlet correlations take two fixed distances (the two singlets' bonds)")
    sec = sector_of(config.hamiltonian)
    dt = torch.float64 if sec.is_real else torch.complex128
    vec = np.asarray(eigvec)
    if sec.is_real:
        vec = vec.real
    psi = torch.as_tensor(np.ascontiguousarray(vec), device=sec.device).to(dt)
    corrs = sec.singlet_correlations(psi, [fixed[0].to_npint32(), fixed[1].to_npint32()])
    return varied_shifts(config.hamiltonian.num_nodes), corrs


def get_singlet_singlet_correlations(config: configs.Full_Position_Correlation_Config):
    """Singlet-singlet correlations averaged over the degenerate ground states, loaded or computed and
    saved (:54-77)."""

    def calculate():
        eigvals, eigvecs = get_lowest_eigenpairs(config)
        num_degenerate_states = 0
        spectrum = None
        shifts = None
        for j in range(len(eigvals)):
            if abs(eigvals[0] - eigvals[j]) > 1e-6:
                break
            num_degenerate_states += 1
            shifts, corrs = calculate_singlet_singlet_correlations(config, eigvecs[:, j])
            spectrum = corrs if spectrum is None else spectrum + corrs
        return shifts, spectrum / num_degenerate_states

    return load_calculate_save(config.get_spectrum_path(), load_fun=load_spectrum, calc_fun=calculate,
                               save_fun=save_spectrum)
