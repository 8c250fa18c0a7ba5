"""Public API of the t-J ladder engine (mirrors tJ_spin_half_ladder/api.py).

get_eigenpairs, get_all_k_eigenpairs, get_excitation_spectrum, get_Szq_spectra
and get_spectral_function_spectra keep the reference's signatures, loops over
momenta, result shapes and cache files (:33-199).  With batched=True (default)
the spectra of all momenta q of one call are computed together: every q's
excited state O_q|gs> is formed on the GPU, then all target sectors' Lanczos
recursions run as one batched, graph-captured recursion (ed_batch_lanczos) and
the continued fractions are evaluated on the device.  batched=False runs them
one by one through get_spectrum, exactly the reference's call sequence.
Plotting is not part of this package.
"""

from __future__ import annotations

import copy
import dataclasses
import itertools
import typing

import numpy as np
import torch

from exactdiag_gb300.general import lanczos_diagonalization as ld
from exactdiag_gb300.tJ_spin_half_ladder import configs, matrix_setup
from exactdiag_gb300.utils import load_calculate_save


class IntSymmetryQs(typing.NamedTuple):
    leg: int
    rung: typing.Literal[0, 1]


def get_eigenpairs(config: configs.Eigenpair_Config):
    """Eigenvalues and eigenvectors; all momenta when symmetry_qs is None (:33-42)."""
    if config.hamiltonian.symmetry_qs is None:
        return get_all_k_eigenpairs(config)
    return ld.get_lowest_eigenpairs(config)


def get_all_k_eigenpairs(config: configs.Eigenpair_Config) -> dict:
    """{(kx, ky): (eigvals, eigvecs)} for kx in [0, L//2], ky in {0, 1} (:45-59)."""
    mut_config = copy.deepcopy(config)
    mkx = config.hamiltonian.num_rungs // 2 + 1
    collected = {}
    for kx in range(mkx):
        for ky in range(2):
            mut_config.hamiltonian.symmetry_qs = {"leg": kx, "rung": ky}
            collected[(kx, ky)] = ld.get_lowest_eigenpairs(mut_config)
    return collected


@dataclasses.dataclass
class Spectrum:
    ws: np.ndarray
    spectrum: np.ndarray
    config: typing.Any
    info: dict = dataclasses.field(default_factory=dict)


def get_excitation_spectrum(config: configs.Full_Spectrum_Config, limited_qs: bool = True,
                            batched: bool = True) -> Spectrum:
    """The spectrum the config names, over the momenta the reference loops over (:83-101)."""
    base_name = config.spectrum.name
    info = {}
    if base_name in {"current_rung", "current_leg"}:
        ws, spectrum = ld.get_spectrum(config)
    elif base_name == "Szq":
        ws, spectrum, info = get_Szq_spectra(config=config, limited_qs=limited_qs, batched=batched)
    elif base_name in {"spectral_function_plus", "spectral_function_minus"}:
        ws, spectrum, info = get_spectral_function_spectra(config=config, limited_qs=limited_qs, batched=batched)
    else:
        raise ValueError(f"{base_name} is not supported")
    return Spectrum(ws, spectrum, config, info)


def get_mkx_qxs_qys(config, limited_qs: bool):
    """(:186-199)"""
    mkx = config.hamiltonian.num_rungs
    qxs = range(mkx // 2 + 1) if limited_qs else range(mkx)
    return mkx, qxs, range(2)


def _spectra_batched(configs_list: list) -> list[tuple[np.ndarray, np.ndarray]]:
    """Spectra of several Full_Spectrum_Configs that share the Hamiltonian and the operator name.

    Cached spectra are loaded; the rest are computed together and saved under the reference's paths.
    """
    results: list = [None] * len(configs_list)
    todo = []
    for i, cfg in enumerate(configs_list):
        path = cfg.get_spectrum_path("")
        if path.is_file():
            results[i] = ld.load_spectrum(path)
        else:
            todo.append(i)
    if not todo:
        return results
    base = configs_list[todo[0]]
    eigvals, eigvecs = ld.get_lowest_eigenpairs(base)
    h = base.hamiltonian
    dt = torch.complex128 if h.precision == "fp64" else torch.complex64
    ops, hams = [], []
    for i in todo:
        get_operator, _, get_excited_h = configs_list[i].setup_excitation_operator()
        ops.append(get_operator())
        hams.append(get_excited_h())
    ws = base.spectrum.get_omegas()
    gs_energy = eigvals[0]
    spectra = np.zeros((len(todo), len(ws)))
    ndeg = 0
    from exactdiag_gb300.engine import batch_lanczos, continued_fraction

    for j in range(len(eigvals)):
        if abs(gs_energy - eigvals[j]) > 1e-6:
            break
        ndeg += 1
        src = ops[0].src
        gs = torch.as_tensor(np.asarray(eigvecs[:, j], np.complex128)).to(device=src.device, dtype=dt)
        live, v0s = [], []
        for q, op in enumerate(ops):
            if op.shape[0] == 0:
                continue
            live.append(q)
            v0s.append(op.device_dot(gs))
        if not live:
            continue
        coefs = batch_lanczos([hams[q].sector for q in live], h.weights, v0s, base.spectrum.num_lanczos_vecs)
        dev = src.device
        zs = ws + gs_energy + 1j * base.spectrum.broadening
        om = torch.as_tensor(zs.real, dtype=torch.float64, device=dev)
        for q, (a, b, norm) in zip(live, coefs):
            if norm < 1e-8:
                continue
            s = continued_fraction(torch.as_tensor(a, device=dev), torch.as_tensor(b, device=dev), om, 0.0,
                                   base.spectrum.broadening, norm ** 2)
            spectra[q] += s.cpu().numpy()
    spectra /= max(ndeg, 1)
    for q, i in enumerate(todo):
        results[i] = (ws, spectra[q])
        ld.save_spectrum(results[i], configs_list[i].get_spectrum_path(""))
    return results


def get_Szq_spectra(config: configs.Full_Spectrum_Config, limited_qs: bool, batched: bool = True):
    """S^z_q spectra for every qx, qy (:116-132); returns (ws, spectra[qx, qy, w], info)."""
    config = copy.deepcopy(config)
    mkx, qxs, qys = get_mkx_qxs_qys(config, limited_qs=False)
    qs_list = itertools.product(qxs, qys)
    spectra = np.empty((len(qxs), len(qys), config.spectrum.omega_steps))
    ws = np.empty((len(qxs), len(qys), config.spectrum.omega_steps))
    cfgs, slots = [], []
    for i, qx in enumerate(qxs):
        for j, qy in enumerate(qys):
            if limited_qs and qx > mkx // 2:
                qx = mkx - qx
            c = copy.deepcopy(config)
            c.spectrum.operator_symmetry_qs = {"leg": qx, "rung": qy}
            cfgs.append(c)
            slots.append((i, j))
    results = _spectra_batched(cfgs) if batched else [ld.get_spectrum(c) for c in cfgs]
    for (i, j), (w, s) in zip(slots, results):
        ws[i, j, :], spectra[i, j, :] = w, s
    return ws, spectra, {"qs_list": qs_list}


def get_spectral_function_spectra(config: configs.Full_Spectrum_Config, limited_qs: bool, batched: bool = True):
    """One-particle spectral functions over q (:135-161); returns (ws, spectra[op, q, w], info)."""
    config = copy.deepcopy(config)
    mkx, qxs, qys = get_mkx_qxs_qys(config=config, limited_qs=limited_qs)
    plus_minus_conditions = [
        (configs.Spectrum_Name.SPECTRAL_FUNCTION_PLUS, config.hamiltonian.num_holes > 0),
        (configs.Spectrum_Name.SPECTRAL_FUNCTION_MINUS, config.hamiltonian.num_holes < config.hamiltonian.num_nodes),
    ]
    qs_list = list(itertools.product(qxs, qys))
    shape = [sum(c for _, c in plus_minus_conditions), len(qs_list), config.spectrum.omega_steps]
    spectra = np.empty(shape, dtype=float)
    ws = np.empty(shape, dtype=float)
    cfgs, slots = [], []
    for i, (qx, qy) in enumerate(qs_list):
        if limited_qs and qx > mkx // 2 + 1:
            continue
        qs = np.array([qx, qy], dtype=int)
        for o, (name, condition) in enumerate(plus_minus_conditions):
            if not condition:
                continue
            if name == configs.Spectrum_Name.SPECTRAL_FUNCTION_MINUS:
                qs = -qs
            c = copy.deepcopy(config)
            c.spectrum.operator_symmetry_qs = {"leg": int(qs[0]), "rung": int(qs[1] % 2)}
            c.spectrum.name = name
            cfgs.append(c)
            slots.append((o - int(not plus_minus_conditions[0][1]), i))
    if batched:  # one batched recursion per operator: plus and minus targets differ in Nh and Nd
        results = [None] * len(cfgs)
        for name, _ in plus_minus_conditions:
            pick = [k for k, c in enumerate(cfgs) if c.spectrum.name == name]
            if pick:
                for k, r in zip(pick, _spectra_batched([cfgs[k] for k in pick])):
                    results[k] = r
    else:
        results = [ld.get_spectrum(c) for c in cfgs]
    for (o, i), (w, s) in zip(slots, results):
        ws[o, i, :], spectra[o, i, :] = w, s
    return ws, spectra, {"qs_list": qs_list}


def get_position_correlations(config: configs.Full_Position_Correlation_Config) -> Spectrum:
    """Hole or S^z position correlations of the ground state (:104-113)."""
    from exactdiag_gb300.tJ_spin_half_ladder import position_correlations

    base_name = config.correlations.name
    if base_name in {"hole_correlations", "Sz_correlations"}:
        ws, spectrum = position_correlations.get_hole_spin_projection_correlations(config)
    elif base_name == "singlet-singlet":
        ws, spectrum = position_correlations.get_singlet_singlet_correlations(config)
    else:
        raise ValueError(f"{base_name} is not supported")
    info = {"fixed_distances": config.correlations.fixed_distances}
    return Spectrum(ws, spectrum, config, info)


def _plot(name: str, spectrum: Spectrum, show: bool) -> None:
    """A plain figure of a computed spectrum or correlation when matplotlib is installed; the
    reference's styled figures (plotting.py) are not part of this package."""
    try:
        import matplotlib.pyplot as plt
    except ImportError:
        return
    data = np.asarray(spectrum.spectrum)
    fig, ax = plt.subplots()
    if data.ndim == 1:
        ax.plot(data)
    else:
        ax.imshow(data.reshape(-1, data.shape[-1]), aspect="auto", origin="lower")
    ax.set_title(str(name))
    if show:
        plt.show()


def plot_excitation_spectrum(config: configs.Full_Spectrum_Config, show: bool = False, **kwargs) -> Spectrum:
    """Compute the spectra get_excitation_spectrum gives (:202-204) and draw them if matplotlib is
    installed; returns the Spectrum."""
    spectrum = get_excitation_spectrum(config=config, **kwargs)
    _plot(config.spectrum.name, spectrum, show)
    return spectrum


def plot_position_correlation(config: configs.Full_Position_Correlation_Config, show: bool = False) -> Spectrum:
    """Compute the position correlations (:207-209) and draw them if matplotlib is installed."""
    spectrum = get_position_correlations(config=config)
    _plot(config.correlations.name, spectrum, show)
    return spectrum


__all__ = ["get_eigenpairs", "get_all_k_eigenpairs", "Spectrum", "get_excitation_spectrum", "get_Szq_spectra",
           "get_spectral_function_spectra", "get_position_correlations", "plot_excitation_spectrum",
           "plot_position_correlation", "get_mkx_qxs_qys", "load_calculate_save", "matrix_setup"]
