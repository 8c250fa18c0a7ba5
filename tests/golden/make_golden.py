"""Generate the committed golden fixtures under tests/golden/.

Run in a checkout where the reference tree exists (it reads the reference's
test fixtures and uses the reference's own C++ compiled into oracle/_ref):

    python tests/golden/make_golden.py [--ref-root PATH]

Outputs
  reference_fixtures.json  the reference's basis-size / eigenvalue fixtures
                           (tests/tJ_spin_half_ladder/precalculated_basis_size_eigenvalues/*.txt),
                           gathered into one file so the GPU tests can read them
                           where the reference is absent;
  sectors.npz              per small sector: the basis (dense_to_sparse, orbit
                           sizes) and y = H x for a seeded x, both computed by
                           the reference's compiled code, plus 30 spectrum-Lanczos
                           coefficients from the numpy restatement on that matrix;
  excitations.npz          O x for the Szq, spectral_function_minus, spectral_function_plus,
                           current_rung and current_leg operators;
  reference_correlations.json  the reference's position-correlation fixtures
                           (tests/tJ_spin_half_ladder/precalculated_position_correlations/*.txt);
  reference_examples.json  the configurations of examples/tJ_spin_half_ladder/*.json.
"""

from __future__ import annotations

import argparse
import glob
import json
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as O  # noqa: E402

OUT = pathlib.Path(__file__).resolve().parent
WEIGHTS = {"tl": 1.0, "tr": 1.0, "jl": 0.5, "jr": 0.5}
SECTORS = [
    (3, 0, 3, 0, 0),
    (4, 2, 3, 0, 0),
    (4, 2, 3, 1, 0),
    (4, 1, 3, 2, 1),
    (5, 2, 4, 1, 1),
    (5, 3, 3, 2, 0),
    (6, 0, 6, 0, 0),
    (6, 0, 6, 3, 1),
    (6, 1, 5, 2, 1),
    (6, 2, 5, 3, 0),
    (6, 4, 4, 1, 1),
    (7, 2, 6, 2, 1),
    (8, 2, 7, 0, 0),
]
EXCITATIONS = [
    ((6, 2, 5, 0, 0), "Szq", 1, 0),
    ((6, 2, 5, 0, 0), "Szq", 3, 1),
    ((5, 2, 4, 1, 0), "Szq", 2, 1),
    ((6, 0, 6, 0, 0), "spectral_function_minus", -1, 0),
    ((6, 0, 6, 0, 0), "spectral_function_minus", -2, 1),
    ((5, 1, 4, 0, 1), "spectral_function_minus", -3, 0),
    ((6, 2, 5, 0, 0), "spectral_function_plus", 1, 0),
    ((6, 2, 4, 1, 0), "spectral_function_plus", 2, 1),
    ((6, 2, 5, 1, 1), "current_rung", 2, 1),
    ((7, 1, 6, 3, 0), "current_rung", -2, 0),
    ((6, 2, 5, 2, 1), "current_leg", 0, 1),
    ((8, 2, 7, 0, 0), "current_leg", 4, 0),
]


def seeded_vector(n: int, seed: int, complex_: bool) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, n)
    if complex_:
        x = x + 1j * rng.uniform(-1, 1, n)
    return x.astype(np.complex128)


def is_real(sec: O.Sector) -> bool:
    return (2 * (sec.kx % sec.L)) % sec.L == 0


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=str(O.REF_SRC.parents[1]) if O.REF_SRC else None, required=O.REF_SRC is None,
                    help="the reference checkout (default: two levels above EXACTDIAG_REF_SRC)")
    args = ap.parse_args()
    ref_root = pathlib.Path(args.ref_root)
    O.build(ref=True)
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref is required to generate the golden fixtures")

    fixtures = []
    pattern = ref_root / "tests" / "tJ_spin_half_ladder" / "precalculated_basis_size_eigenvalues" / "*.txt"
    for f in sorted(glob.glob(str(pattern))):
        d = json.load(open(f))
        d["file"] = pathlib.Path(f).name
        fixtures.append(d)
    (OUT / "reference_fixtures.json").write_text(json.dumps(fixtures, indent=1))

    corr = []
    folder = ref_root / "tests" / "tJ_spin_half_ladder" / "precalculated_position_correlations"
    for f in sorted(folder.glob("*.txt")):
        for d in json.load(open(f)):
            d["file"] = f.name
            corr.append(d)
    (OUT / "reference_correlations.json").write_text(json.dumps(corr, indent=1))

    # the example configurations (examples/tJ_spin_half_ladder/*.json) for the drop-in test
    examples = {}
    for f in sorted((ref_root / "examples" / "tJ_spin_half_ladder").glob("*.json")):
        examples[f.stem] = json.load(open(f))
    (OUT / "reference_examples.json").write_text(json.dumps(examples, indent=1))

    arrays = {}
    for idx, key in enumerate(SECTORS):
        sec = O.Sector(*key)
        bas = O.basis(sec, impl="ref")
        h = O.hamiltonian(sec, WEIGHTS, bas, impl="ref")
        x = seeded_vector(len(bas[0]), 1000 + idx, not is_real(sec))
        y = h @ x
        a, b = O.lanczos_get_anbn(seeded_vector(len(bas[0]), 2000 + idx, False), 30, lambda v: h @ v)
        tag = "s%d_%d_%d_%d_%d" % key
        arrays[f"{tag}_sparse"] = bas[0]
        arrays[f"{tag}_orbit"] = bas[1].astype(np.int8)
        arrays[f"{tag}_y"] = y.real if is_real(sec) else y
        arrays[f"{tag}_a"] = a
        arrays[f"{tag}_b"] = b
        arrays[f"{tag}_seed"] = np.array([1000 + idx, 2000 + idx])
    arrays["sectors"] = np.array(SECTORS, dtype=np.int64)
    arrays["weights"] = np.array([WEIGHTS[t] for t in O.TERMS])
    np.savez_compressed(OUT / "sectors.npz", **arrays)

    ex = {}
    for idx, (key, name, qx, qy) in enumerate(EXCITATIONS):
        sec = O.Sector(*key)
        bas = O.basis(sec, impl="ref")
        fsec = O.target_sector(sec, name, qx, qy)
        fbas = O.basis(fsec, impl="ref")
        op = O.excitation_matrix(sec, bas, name, qx, qy, fsec, fbas, impl="ref")
        x = seeded_vector(len(bas[0]), 3000 + idx, True)
        ex[f"e{idx}_y"] = op @ x
        ex[f"e{idx}_seed"] = np.array([3000 + idx])
        ex[f"e{idx}_target"] = np.array(fsec.args())
    ex["cases"] = np.array([[*k, O.OPS[n], qx, qy] for k, n, qx, qy in EXCITATIONS])
    np.savez_compressed(OUT / "excitations.npz", **ex)
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")), "and reference_fixtures.json")


if __name__ == "__main__":
    main()
