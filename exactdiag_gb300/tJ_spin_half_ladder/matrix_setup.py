"""Sector translators, the Hamiltonian and excitation operators on the GPU.

Mirrors tJ_spin_half_ladder/matrix_setup.pyx: setup_hamiltonian (:41-129),
setup_excitation_operator (:195-374) and py_get_ladder_translators (:377-406),
with the stored matrices replaced by the matrix-free device operators.
Sectors are built once per (L, Nh, Nd, kx mod L, ky) and cached for the
process (clear_sector_cache() releases them).
"""

from __future__ import annotations

import copy
import logging
import os
import pathlib
from functools import partial

import numpy as np

from exactdiag_gb300.engine import DeviceSector
from exactdiag_gb300.general.sparse_matrices import Device_Hamiltonian, Device_Operator
from exactdiag_gb300.tJ_spin_half_ladder import configs

_logger = logging.getLogger(__name__)
_SECTORS: dict[tuple, DeviceSector] = {}

IMPLEMENTED_OPERATORS = (configs.Spectrum_Name.SZQ, configs.Spectrum_Name.SPECTRAL_FUNCTION_MINUS,
                         configs.Spectrum_Name.SPECTRAL_FUNCTION_PLUS, configs.Spectrum_Name.CURRENT_RUNG,
                         configs.Spectrum_Name.CURRENT_LEG)


def get_sector(num_rungs: int, num_holes: int, num_down_spins: int, kx: int, ky: int) -> DeviceSector:
    key = (int(num_rungs), int(num_holes), int(num_down_spins), int(kx) % int(num_rungs), int(ky))
    sec = _SECTORS.get(key)
    if sec is None:
        sec = DeviceSector(num_rungs, num_holes, num_down_spins, kx, ky)
        _SECTORS[key] = sec
    return sec


def clear_sector_cache() -> None:
    for s in _SECTORS.values():
        s.close()
    _SECTORS.clear()


def sector_of(config: configs.Hamiltonian_Config) -> DeviceSector:
    if config.symmetry_qs is None:
        raise ValueError("symmetry_qs must be set to build a sector")
    return get_sector(*config.sector_key())


def setup_hamiltonian(config: configs.Hamiltonian_Config):
    """Callable returning the sector's Hamiltonian (matrix_setup.pyx:41-129)."""
    return partial(_make_hamiltonian, config)


def _make_hamiltonian(config: configs.Hamiltonian_Config) -> Device_Hamiltonian:
    return Device_Hamiltonian(sector_of(config), config.weights, config.num_threads, config.precision)


def target_sector_config(initial_config, name, qx: int, qy: int) -> configs.Hamiltonian_Config:
    """Final Hamiltonian config of an excitation (matrix_setup.pyx:248-330)."""
    h = initial_config.hamiltonian
    final = copy.deepcopy(h)
    L = h.num_rungs
    kx, ky = h.symmetry_qs.leg, h.symmetry_qs.rung
    if name in (configs.Spectrum_Name.SZQ, configs.Spectrum_Name.CURRENT_LEG):
        pass
    elif name == configs.Spectrum_Name.CURRENT_RUNG:
        qy += 1  # the rung current's hopping-direction sign is carried by the target's rung parity (:251)
    elif name == configs.Spectrum_Name.SPECTRAL_FUNCTION_MINUS:
        final.num_holes += 1
        if h.total_spin_projection <= 0:
            final.total_spin_projection += 1
        else:
            final.total_spin_projection -= 1
    elif name == configs.Spectrum_Name.SPECTRAL_FUNCTION_PLUS:
        if h.num_holes < 1:
            raise ValueError("spectral_function_plus needs a hole to fill")
        final.num_holes -= 1
        if h.total_spin_projection > 0:
            final.total_spin_projection -= 1
        else:
            final.total_spin_projection += 1
    else:
        raise ValueError(f"{name} not supported")
    final.symmetry_qs = configs.Quantum_Numbers(leg=(kx + qx + (L - 1) // 2) % L - (L - 1) // 2, rung=(ky + qy) % 2)
    return final


def setup_excitation_operator(initial_config):
    """(get_operator, final hamiltonian config, get_excited_H) (matrix_setup.pyx:195-374)."""
    name = initial_config.spectrum.name
    qs = initial_config.spectrum.operator_symmetry_qs
    qx, qy = (int(qs.leg), int(qs.rung)) if qs is not None else (0, 0)
    final_h = target_sector_config(initial_config, name, qx, qy)
    h = initial_config.hamiltonian

    def get_operator():
        return Device_Operator(str(name), sector_of(h), sector_of(final_h), qx, qy, h.total_spin_projection,
                               initial_config.spectrum.num_threads, h.precision)

    return get_operator, final_h, final_h.setup()


BASIS_MAP_FILE = "Sz_local-momentum_map.dat"  # matrix_setup.pyx:390


def save_basis_map(path, sparse: np.ndarray, orbit: np.ndarray) -> None:
    """Write a basis in the reference's binary format (basis_indexing.h:128-146): the number of
    representatives as an unsigned 64-bit count, then dense_to_sparse as int64 and
    num_sparse_states_in_dense as int32, native little-endian."""
    path = pathlib.Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    n = len(sparse)
    if len(orbit) != n:
        raise ValueError("dense_to_sparse and num_sparse_states_in_dense differ in length")
    tmp = path.with_name(path.name + ".tmp")
    with open(tmp, "wb") as f:
        np.array([n], dtype="<u8").tofile(f)
        np.ascontiguousarray(sparse, dtype="<i8").tofile(f)
        np.ascontiguousarray(orbit, dtype="<i4").tofile(f)
    os.replace(tmp, path)


def load_basis_map(path) -> tuple[np.ndarray, np.ndarray]:
    """Read a basis written by the reference or by save_basis_map (basis_indexing.h:72-100)."""
    path = pathlib.Path(path)
    with open(path, "rb") as f:
        head = np.fromfile(f, dtype="<u8", count=1)
        if len(head) != 1:
            raise ValueError(f"{path}: truncated basis file")
        n = int(head[0])
        sparse = np.fromfile(f, dtype="<i8", count=n)
        orbit = np.fromfile(f, dtype="<i4", count=n)
        rest = f.read(1)
    if len(sparse) != n or len(orbit) != n or rest:
        raise ValueError(f"{path}: basis file does not hold {n} representatives")
    return sparse, orbit


class Py_Basis_Index_Map:
    """Host view of a device basis with the reference's query methods (basis_indexing.pxd:40-53)."""

    def __init__(self, sparse: np.ndarray, orbit: np.ndarray):
        self.dense_to_sparse = sparse
        self.num_sparse_in_dense = orbit

    def save(self, path) -> None:
        """The basis .dat file (basis_indexing.h:128-146)."""
        save_basis_map(path, self.dense_to_sparse, self.num_sparse_in_dense)

    def get_num_states(self) -> int:
        return len(self.dense_to_sparse)

    def get_sparse(self, dense_index: int) -> int:
        return int(self.dense_to_sparse[dense_index])

    def get_dense(self, sparse_index: int) -> int:
        if sparse_index < 0:
            return -1
        i = int(np.searchsorted(self.dense_to_sparse, sparse_index))
        return i if i < len(self.dense_to_sparse) and self.dense_to_sparse[i] == sparse_index else -1

    def get_num_sparse_in_dense(self, dense_index: int) -> int:
        return int(self.num_sparse_in_dense[dense_index])

    def get_num_sparse_in_dense_from_sparse(self, sparse_index: int) -> int:
        d = self.get_dense(sparse_index)
        return int(self.num_sparse_in_dense[d]) if d > -1 else 0


class Py_State_Index_Amplitude_Translator:
    """Sparse index <-> site values (symmetry_ladder.h:314-361); 0 hole, 1 down, 2 up."""

    def __init__(self, config: configs.Hamiltonian_Config):
        self.num_nodes = config.num_nodes
        self.num_holes = config.num_holes
        self.num_down_spins = config.num_down_spins
        self.comb = configs.set_combinatorics(self.num_nodes)
        self.num_spin_states = int(self.comb[self.num_down_spins, self.num_nodes - self.num_holes])

    def get_num_minor_sparse_states(self) -> int:
        return self.num_spin_states

    def sparse_index_to_state(self, sparse_index: int) -> np.ndarray:
        rh, rs = self.num_holes, self.num_down_spins
        hole_ind, spin_ind = divmod(int(sparse_index), self.num_spin_states)
        state = np.empty(self.num_nodes, np.int16)
        for j in range(self.num_nodes - 1, -1, -1):
            if rh > 0 and hole_ind >= self.comb[rh, j]:
                state[j] = 0
                hole_ind -= self.comb[rh, j]
                rh -= 1
                continue
            if rs > 0 and j - rh >= 0 and spin_ind >= self.comb[rs, j - rh]:
                state[j] = 1
                spin_ind -= self.comb[rs, j - rh]
                rs -= 1
                continue
            state[j] = 2
        return state

    def state_to_sparse_index(self, state) -> int:
        hole_index = spin_index = 0
        ah = int(state[0] == 0)
        ad = int(state[0] == 1)
        for i in range(1, self.num_nodes):
            if state[i] == 0:
                ah += 1
                hole_index += int(self.comb[ah, i])
            elif state[i] == 1:
                ad += 1
                spin_index += int(self.comb[ad, i - ah])
        return spin_index + hole_index * self.num_spin_states


class Py_Symmetry_Generator:
    """Translation x mirror group of the two-leg ladder (symmetry_ladder.h:55-111)."""

    def __init__(self, config: configs.Hamiltonian_Config):
        self.num_rungs = config.num_rungs
        self.symmetry_qs = config.symmetry_qs.to_npint32()

    def get_basis_length(self) -> int:
        return 2 * self.num_rungs

    def get_shift_periodicities(self) -> list[int]:
        return [self.num_rungs, 2]

    def get_num_shifts(self) -> int:
        return 2


def py_get_ladder_translators(config: configs.Hamiltonian_Config):
    """(translator, basis map, symmetry generator) (matrix_setup.pyx:377-406).

    The basis is built on the GPU.  Like the reference (basis_indexing.h:58-66), the basis file in the
    sector's calculation folder is written when absent; when present (written by the reference or by
    this package) it must hold the same basis, else ValueError names the file.
    """
    sec = sector_of(config)
    sparse, orbit = sec.export_basis()
    path = config.get_calc_folder() / BASIS_MAP_FILE
    if path.exists():
        f_sparse, f_orbit = load_basis_map(path)
        if not (np.array_equal(f_sparse, sparse) and np.array_equal(f_orbit, orbit.astype(np.int32))):
            raise ValueError(f"{path} holds a different basis than sector {config.sector_key()}")
    else:
        save_basis_map(path, sparse, orbit)
    return Py_State_Index_Amplitude_Translator(config), Py_Basis_Index_Map(sparse, orbit), Py_Symmetry_Generator(config)
