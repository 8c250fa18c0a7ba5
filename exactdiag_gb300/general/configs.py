"""Model-independent configuration parts (mirrors general/configs.py of the reference).

Plain dataclasses with explicit validation: the same field names, defaults and
JSON loading as the reference's pydantic dataclasses, without the pydantic
dependency.
"""

from __future__ import annotations

import dataclasses
import json
import pathlib
import typing

import numpy as np


def _check_fields(cls, data: dict) -> None:
    names = {f.name for f in dataclasses.fields(cls) if f.init}
    extra = set(data) - names
    if extra:
        raise ValueError(f"{cls.__name__}: unexpected fields {sorted(extra)}")


class _Json_Loadable:
    @classmethod
    def load(cls, path: pathlib.Path | str) -> typing.Self:
        """Load from a JSON file (general/configs.py:60-66)."""
        with open(path, mode="r", encoding="utf-8") as fp:
            d = json.load(fp)
        return cls(**d)


@dataclasses.dataclass(kw_only=True)
class Eigenpair_Part:
    """num_eigenpairs lowest eigenpairs (general/configs.py:116-128)."""

    num_eigenpairs: int
    num_recalculated_vecs_per_iteration: int = 4
    num_threads: int | None = None

    def __post_init__(self):
        if int(self.num_eigenpairs) < 1:
            raise ValueError("num_eigenpairs must be >= 1")
        self.num_eigenpairs = int(self.num_eigenpairs)


def asdict_shallow(obj) -> dict:
    return {f.name: getattr(obj, f.name) for f in dataclasses.fields(obj)}


@dataclasses.dataclass(kw_only=True)
class Spectrum_Part_Base:
    """Spectrum parameters (general/configs.py:174-191)."""

    name: typing.Any
    operator_symmetry_qs: typing.Any
    broadening: float
    omega_max: float
    omega_min: float = 0
    omega_steps: int = 1000
    num_lanczos_vecs: int = 250
    num_threads: int | None = None

    def get_omegas(self) -> np.ndarray:
        """Uniformly spaced energies (general/configs.py:189-191)."""
        return np.linspace(self.omega_min, self.omega_max, self.omega_steps)
