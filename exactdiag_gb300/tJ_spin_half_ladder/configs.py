"""Configurations of the anisotropic spin-1/2 t-J ladder (mirrors tJ_spin_half_ladder/configs.py).

Same classes, field names, defaults, derived quantities and result paths as the
reference (:24-389), so existing JSON configs and cached results carry over.
One addition: Hamiltonian_Config.precision selects the GPU arithmetic --
"fp64" (default; FP64/complex128 vectors, the reference's precision) or
"mixed" (FP32/complex64 vectors and per-term arithmetic with FP64 reductions).
num_threads is accepted and kept for compatibility; the GPU path ignores it.
"""

from __future__ import annotations

import copy
import dataclasses
import enum
import logging
import os
import pathlib
import typing

import numpy as np

from exactdiag_gb300.general import configs as gc

_logger = logging.getLogger(__name__)


def set_combinatorics(size: int) -> np.ndarray:
    """comb[j, i] = C(i, j) (general/matrix_rules_utils.pyx:122-134), exact integers."""
    comb = np.zeros((size + 1, size + 1), dtype=np.int64)
    for i in range(size + 1):
        comb[0, i] = 1
        for j in range(1, i + 1):
            comb[j, i] = comb[j - 1, i - 1] + (comb[j, i - 1] if j <= i - 1 else 0)
    return comb


@dataclasses.dataclass(kw_only=True)
class Weights:
    """Weights of the Hamiltonian terms (:24-31)."""

    tl: float
    tr: float
    jl: float
    jr: float


@dataclasses.dataclass(kw_only=True)
class Quantum_Numbers:
    """Leg momentum and rung parity (:34-37)."""

    leg: int
    rung: typing.Literal[0, 1]

    def __post_init__(self):
        self.leg = int(self.leg)
        if int(self.rung) not in (0, 1):
            raise ValueError("rung must be 0 or 1")
        self.rung = int(self.rung)

    def to_npint32(self):
        return np.array([self.leg, self.rung], dtype=np.int32)


def _weights(value) -> Weights:
    if isinstance(value, Weights):
        return value
    gc._check_fields(Weights, value)
    return Weights(**value)


def _qs(value) -> Quantum_Numbers | None:
    if value is None or isinstance(value, Quantum_Numbers):
        return value
    gc._check_fields(Quantum_Numbers, value)
    return Quantum_Numbers(**value)


@dataclasses.dataclass(kw_only=True)
class Hamiltonian_Config(gc._Json_Loadable):
    """Information necessary to construct a Hamiltonian (:40-147)."""

    CALCULATIONS_FOLDER_NAME: typing.ClassVar[str] = "calculations"
    FIGURES_FOLDER_NAME: typing.ClassVar[str] = "figures"

    num_rungs: int
    num_holes: int
    weights: Weights
    symmetry_qs: Quantum_Numbers | None
    num_threads: int
    total_spin_projection: int | None = None
    major: typing.Literal["row", "column"] = "row"
    triangle_only: bool = True
    precision: typing.Literal["fp64", "mixed"] = "fp64"

    def __post_init__(self):
        self.weights = _weights(self.weights)
        self.symmetry_qs = _qs(self.symmetry_qs)
        if self.precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        if self.total_spin_projection is None:
            self.total_spin_projection = self._get_default_spin_projection()
        elif (self.num_spins - self.total_spin_projection) % 2 != 0:
            raise ValueError(
                f"Incompatible total_spin_projection {self.total_spin_projection}/2 with {self.num_spins} spins.")

    def __setattr__(self, name, value):
        if name == "weights" and value is not None and not isinstance(value, Weights):
            value = _weights(value)
        if name == "symmetry_qs" and value is not None and not isinstance(value, Quantum_Numbers):
            value = _qs(value)
        object.__setattr__(self, name, value)

    @property
    def combinatorics_table(self) -> np.ndarray:
        return set_combinatorics(self.num_nodes)

    def _get_default_spin_projection(self) -> int:
        return self.num_spins % 2

    @property
    def num_spin_states(self) -> int:
        return int(self.combinatorics_table[self.num_down_spins, self.num_spins])

    @property
    def num_spins(self) -> int:
        return self.num_nodes - self.num_holes

    @property
    def num_down_spins(self) -> int:
        return (self.num_spins - self.total_spin_projection) // 2

    @property
    def periodicities(self) -> tuple[int, int]:
        return (self.num_rungs, 2)

    @property
    def num_nodes(self) -> int:
        return 2 * self.num_rungs

    def _get_relative_path(self) -> pathlib.Path:
        if self.symmetry_qs is None:
            raise ValueError("symmetry_qs must not be None to specify a path.")
        rungs_holes = f"rungs{self.num_rungs}_holes{self.num_holes}"
        qs_spins = f"kx{self.symmetry_qs.leg}_ky{self.symmetry_qs.rung}_down_spins{self.num_down_spins}"
        return pathlib.Path(rungs_holes) / qs_spins

    def get_calc_folder(self) -> pathlib.Path:
        path = self.CALCULATIONS_FOLDER_NAME / self._get_relative_path()
        os.makedirs(path, exist_ok=True)
        return path

    def get_figures_folder(self) -> pathlib.Path:
        path = self.FIGURES_FOLDER_NAME / self._get_relative_path()
        os.makedirs(path, exist_ok=True)
        return path

    def sector_key(self) -> tuple[int, int, int, int, int]:
        return (self.num_rungs, self.num_holes, self.num_down_spins, self.symmetry_qs.leg, self.symmetry_qs.rung)

    def get_translators(self):
        """(translator, basis map, symmetry generator) of the sector (matrix_setup.pyx:377-406)."""
        from exactdiag_gb300.tJ_spin_half_ladder import matrix_setup

        return matrix_setup.py_get_ladder_translators(self)

    def setup(self):
        """Callable returning the Hamiltonian object with .dot/.shape/.toarray (matrix_setup.pyx:41-129)."""
        from exactdiag_gb300.tJ_spin_half_ladder import matrix_setup

        return matrix_setup.setup_hamiltonian(self)

    def get_symmetry_info(self) -> dict:
        symmetry_qs = None if self.symmetry_qs is None else [int(i) for i in self.symmetry_qs.to_npint32()]
        dic = {"num_rungs": self.num_rungs, "num_holes": self.num_holes, "symmetry_qs": symmetry_qs}
        if self.total_spin_projection != self._get_default_spin_projection():
            dic["total_spin_projection"] = self.total_spin_projection
        return dic


def _hamiltonian(value) -> Hamiltonian_Config:
    if isinstance(value, Hamiltonian_Config):
        return value
    gc._check_fields(Hamiltonian_Config, value)
    return Hamiltonian_Config(**value)


@dataclasses.dataclass(kw_only=True)
class Eigenpair_Config(gc._Json_Loadable):
    """Hamiltonian plus the eigenpair request (general/configs.py:134-160)."""

    hamiltonian: Hamiltonian_Config
    eigenpair: gc.Eigenpair_Part

    def __post_init__(self):
        self.hamiltonian = _hamiltonian(self.hamiltonian)
        if not isinstance(self.eigenpair, gc.Eigenpair_Part):
            gc._check_fields(gc.Eigenpair_Part, self.eigenpair)
            self.eigenpair = gc.Eigenpair_Part(**self.eigenpair)
        if self.eigenpair.num_threads is None:
            self.eigenpair.num_threads = self.hamiltonian.num_threads

    def get_eigenpair_paths(self) -> tuple[pathlib.Path, pathlib.Path]:
        hamiltonian_string = "_".join(
            [f"{name}{weight:g}" for name, weight in gc.asdict_shallow(self.hamiltonian.weights).items()])
        suffix = f"_{hamiltonian_string}_eigenpairs{self.eigenpair.num_eigenpairs}.npy"
        eigen_folder = self.hamiltonian.get_calc_folder() / "eigenpairs"
        return eigen_folder / f"eigenvals{suffix}", eigen_folder / f"eigenvecs{suffix}"


class Spectrum_Name(enum.StrEnum):
    """Names of the operators (:163-172)."""

    CURRENT_RUNG = enum.auto()
    CURRENT_LEG = enum.auto()
    SZQ = "Szq"
    SPECTRAL_FUNCTION_PLUS = enum.auto()
    SPECTRAL_FUNCTION_MINUS = enum.auto()
    OFFIDAG_SPEC_FUNC_PLUS = "offdiagonal_spectral_function_plus"
    OFFIDAG_SPEC_FUNC_MINUS = "offdiagonal_spectral_function_minus"


@dataclasses.dataclass(kw_only=True)
class Spectrum_Part(gc.Spectrum_Part_Base):
    def __post_init__(self):
        if not isinstance(self.name, Spectrum_Name):
            self.name = Spectrum_Name(self.name)
        self.operator_symmetry_qs = _qs(self.operator_symmetry_qs)

    def __setattr__(self, name, value):
        if name == "operator_symmetry_qs" and value is not None and not isinstance(value, Quantum_Numbers):
            value = _qs(value)
        if name == "name" and not isinstance(value, Spectrum_Name):
            value = Spectrum_Name(value)
        object.__setattr__(self, name, value)


def _spectrum(value) -> Spectrum_Part:
    if isinstance(value, Spectrum_Part):
        return value
    gc._check_fields(Spectrum_Part, value)
    return Spectrum_Part(**value)


@dataclasses.dataclass(kw_only=True)
class Limited_Spectrum_Config(gc._Json_Loadable):
    """Hamiltonian plus operator (:193-211)."""

    hamiltonian: Hamiltonian_Config
    spectrum: Spectrum_Part

    def __post_init__(self):
        self.hamiltonian = _hamiltonian(self.hamiltonian)
        self.spectrum = _spectrum(self.spectrum)
        if self.spectrum.num_threads is None:
            self.spectrum.num_threads = self.hamiltonian.num_threads

    def setup_excitation_operator(self):
        from exactdiag_gb300.tJ_spin_half_ladder import matrix_setup

        return matrix_setup.setup_excitation_operator(self)


@dataclasses.dataclass(kw_only=True)
class Full_Spectrum_Config(gc._Json_Loadable):
    """Hamiltonian, eigenpair request and operator (:214-233)."""

    hamiltonian: Hamiltonian_Config
    spectrum: Spectrum_Part
    eigenpair: gc.Eigenpair_Part

    def __post_init__(self):
        self.hamiltonian = _hamiltonian(self.hamiltonian)
        self.spectrum = _spectrum(self.spectrum)
        if not isinstance(self.eigenpair, gc.Eigenpair_Part):
            gc._check_fields(gc.Eigenpair_Part, self.eigenpair)
            self.eigenpair = gc.Eigenpair_Part(**self.eigenpair)
        if self.spectrum.num_threads is None:
            self.spectrum.num_threads = self.hamiltonian.num_threads
        if self.eigenpair.num_threads is None:
            self.eigenpair.num_threads = self.hamiltonian.num_threads

    get_eigenpair_paths = Eigenpair_Config.get_eigenpair_paths

    def setup_excitation_operator(self):
        from exactdiag_gb300.tJ_spin_half_ladder import matrix_setup

        return matrix_setup.setup_excitation_operator(self)

    def get_spectrum_path(self, operator_name_suffix: str = "") -> pathlib.Path:
        system_folder = self.hamiltonian.get_calc_folder()
        folder = system_folder / f"{self.spectrum.name}_spectra"
        suffix = _get_spectrum_figure_suffix(self.hamiltonian, self.spectrum, operator_name_suffix)
        return folder / f"{self.spectrum.name}{suffix}.npz"

    def copy(self) -> "Full_Spectrum_Config":
        return copy.deepcopy(self)


def _get_spectrum_figure_suffix(hamiltonian_config: Hamiltonian_Config, spectrum_config: Spectrum_Part,
                                operator_name_suffix: str) -> str:
    """tJ_spin_half_ladder/configs.py:366-379."""
    weight_string = "_".join([f"{name}{weight}" for name, weight in
                              gc.asdict_shallow(hamiltonian_config.weights).items()])
    operator_name_suffix = f"_{operator_name_suffix}" if operator_name_suffix else ""
    if spectrum_config.operator_symmetry_qs is None:
        q_string = ""
    else:
        q_string = f"_q{spectrum_config.operator_symmetry_qs.to_npint32()}"
    ws_string = f"_ws{spectrum_config.omega_min:g},{spectrum_config.omega_max:g},{spectrum_config.omega_steps:g}"
    broad_string = f"_broad{spectrum_config.broadening}"
    vecs_string = f"_vecs{spectrum_config.num_lanczos_vecs}"
    # FP64 results keep the reference's file names; mixed-precision ones are stored beside them
    precision_string = "_mixed" if getattr(hamiltonian_config, "precision", "fp64") == "mixed" else ""
    return (f"{operator_name_suffix}{q_string}{ws_string}{broad_string}{vecs_string}_{weight_string}"
            f"{precision_string}")


class Position_Correlation_Name(enum.StrEnum):
    """Names of the position correlations (:236-241)."""

    HOLE_CORRELATIONS = "hole_correlations"
    SZ_CORRELATIONS = "Sz_correlations"
    SINGLET_SINGLET = "singlet-singlet"


@dataclasses.dataclass(kw_only=True)
class Position_Shift:
    """A relative node position (:244-247, general/configs.py:47-52)."""

    leg: int
    rung: typing.Literal[0, 1]

    def __post_init__(self):
        self.leg = int(self.leg)
        if int(self.rung) not in (0, 1):
            raise ValueError("rung must be 0 or 1")
        self.rung = int(self.rung)

    def to_npint32(self):
        return np.array([self.leg, self.rung], dtype=np.int32)


def _shift(value) -> Position_Shift:
    if isinstance(value, Position_Shift):
        return value
    gc._check_fields(Position_Shift, value)
    return Position_Shift(**value)


@dataclasses.dataclass(kw_only=True)
class Position_Correlation_Part:
    """Correlation request (:250-275): fixed_distances are the shifts of the fixed number operators
    relative to the first one (hole and S^z correlations)."""

    name: Position_Correlation_Name
    fixed_distances: list
    num_threads: int | None = None

    def __post_init__(self):
        self.name = Position_Correlation_Name(self.name)
        self.fixed_distances = [_shift(e) for e in self.fixed_distances]


def _correlations(value) -> Position_Correlation_Part:
    if isinstance(value, Position_Correlation_Part):
        return value
    gc._check_fields(Position_Correlation_Part, value)
    return Position_Correlation_Part(**value)


@dataclasses.dataclass(kw_only=True)
class Limited_Position_Correlation_Config(gc._Json_Loadable):
    """Hamiltonian plus correlation request (:278-310)."""

    hamiltonian: Hamiltonian_Config
    correlations: Position_Correlation_Part

    def __post_init__(self):
        self.hamiltonian = _hamiltonian(self.hamiltonian)
        self.correlations = _correlations(self.correlations)
        if self.correlations.num_threads is None:
            self.correlations.num_threads = self.hamiltonian.num_threads

    def setup_excitation_operator(self, free_shift):
        """The position-projection operator (:296-310) is the building block of the singlet-singlet
        correlations, which are not computed by this engine."""
        raise NotImplementedError("position-correlation operators (singlet-singlet correlations) are not on the GPU path")


@dataclasses.dataclass(kw_only=True)
class Full_Position_Correlation_Config(Limited_Position_Correlation_Config):
    """Hamiltonian, eigenpair request and correlation request (:313-331)."""

    eigenpair: gc.Eigenpair_Part

    def __post_init__(self):
        super().__post_init__()
        if not isinstance(self.eigenpair, gc.Eigenpair_Part):
            gc._check_fields(gc.Eigenpair_Part, self.eigenpair)
            self.eigenpair = gc.Eigenpair_Part(**self.eigenpair)
        if self.eigenpair.num_threads is None:
            self.eigenpair.num_threads = self.hamiltonian.num_threads

    get_eigenpair_paths = Eigenpair_Config.get_eigenpair_paths

    def get_spectrum_path(self, operator_name_suffix: str = "") -> pathlib.Path:
        system_folder = self.hamiltonian.get_calc_folder()
        folder = system_folder / f"{self.correlations.name}_spectra"
        suffix = _get_position_correlation_figure_suffix(self.hamiltonian, self.correlations, operator_name_suffix)
        return folder / f"{self.correlations.name}{suffix}.npz"


def _get_position_correlation_figure_suffix(hamiltonian_config: Hamiltonian_Config,
                                            correlation_config: Position_Correlation_Part,
                                            operator_name_suffix: str) -> str:
    """(:382-389)"""
    weight_string = "_".join([f"{name}{weight}" for name, weight in
                              gc.asdict_shallow(hamiltonian_config.weights).items()])
    operator_name_suffix = f"_{operator_name_suffix}" if operator_name_suffix else ""
    fixed_string = f"{[shift.to_npint32().tolist() for shift in correlation_config.fixed_distances]}"
    return f"{operator_name_suffix}_fixed{fixed_string}_{weight_string}"
