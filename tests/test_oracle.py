"""CPU: pin the oracle against the reference's fixtures, its compiled code and the golden vectors."""

import numpy as np
import pytest
import scipy.special

from conftest import fixture_sector, seeded_vector

EIGENVALUE_TOLERANCE = 1e-8  # tests/tJ_spin_half_ladder/test_eigvals.py:6


def test_basis_sizes_match_reference_fixtures(oracle, reference_fixtures):
    assert len(reference_fixtures) == 68
    for d in reference_fixtures:
        sp, orb = oracle.basis(oracle.Sector(*fixture_sector(d)))
        assert len(sp) == d["basis_size"], d["file"]


def test_eigenvalues_match_reference_fixtures(oracle, reference_fixtures):
    checked = 0
    for d in reference_fixtures:
        if d.get("eigvals") is None:
            continue
        sec = oracle.Sector(*fixture_sector(d))
        bas = oracle.basis(sec)
        h = oracle.hamiltonian(sec, d["weights"], bas)
        ev = oracle.lowest_eigvals(h, len(d["eigvals"]))
        assert np.all(np.abs(ev - np.array(d["eigvals"])) < EIGENVALUE_TOLERANCE), d["file"]
        checked += 1
    assert checked == 51


def test_sum_over_k_matches_combinatorics(oracle):
    # tests/tJ_spin_half_ladder/test_basis_size.py:61-113 invariants
    for L, Nh in [(4, 2), (5, 1), (6, 0), (6, 3)]:
        N = 2 * L
        for Nd in range(N - Nh + 1):
            total = 0
            for kx in range(L // 2 + 1):
                mult = 1 + (kx != 0 and (kx != L // 2 or L % 2))
                for ky in (0, 1):
                    total += mult * len(oracle.basis(oracle.Sector(L, Nh, Nd, kx, ky))[0])
            assert total == scipy.special.comb(N, Nh, exact=True) * scipy.special.comb(N - Nh, Nd, exact=True)


def test_negative_and_periodic_k(oracle):
    for kx in range(1, 4):
        for ky in (0, 1):
            n = len(oracle.basis(oracle.Sector(6, 0, 6, kx, ky))[0])
            assert len(oracle.basis(oracle.Sector(6, 0, 6, -kx, ky))[0]) == n
            for mult in (-2, 1, 3):
                assert len(oracle.basis(oracle.Sector(6, 0, 6, kx + 6 * mult, ky))[0]) == n


def test_term_matrices_are_hermitian(oracle):
    for key in [(5, 2, 4, 1, 1), (6, 1, 5, 2, 0), (4, 0, 4, 1, 1)]:
        sec = oracle.Sector(*key)
        bas = oracle.basis(sec)
        n = len(bas[0])
        import scipy.sparse as sps

        for t in oracle.TERMS:
            cp, r, v = oracle.term_columns(sec, t, bas, triangle=False)
            m = sps.csc_matrix((v, r, cp), shape=(n, n))
            if m.nnz:
                assert abs(m - m.conj().T).max() < 1e-13


def test_oracle_matches_golden(oracle, golden_sectors):
    secs = golden_sectors["sectors"]
    w = dict(zip(oracle.TERMS, golden_sectors["weights"]))
    for key in secs:
        key = tuple(int(v) for v in key)
        tag = "s%d_%d_%d_%d_%d" % key
        sec = oracle.Sector(*key)
        sp, orb = oracle.basis(sec)
        assert np.array_equal(sp, golden_sectors[f"{tag}_sparse"])
        assert np.array_equal(orb, golden_sectors[f"{tag}_orbit"].astype(np.int32))
        h = oracle.hamiltonian(sec, w, (sp, orb))
        real = (2 * (key[3] % key[0])) % key[0] == 0
        seed = int(golden_sectors[f"{tag}_seed"][0])
        y = h @ seeded_vector(len(sp), seed, not real)
        assert np.max(np.abs(y - golden_sectors[f"{tag}_y"])) < 1e-12


def test_oracle_excitations_match_golden(oracle, golden_excitations):
    names = {code: name for name, code in oracle.OPS.items()}
    for idx, case in enumerate(golden_excitations["cases"]):
        L, Nh, Nd, kx, ky, op, qx, qy = (int(v) for v in case)
        sec = oracle.Sector(L, Nh, Nd, kx, ky)
        bas = oracle.basis(sec)
        fsec = oracle.target_sector(sec, names[op], qx, qy)
        assert list(fsec.args()) == list(golden_excitations[f"e{idx}_target"])
        fbas = oracle.basis(fsec)
        m = oracle.excitation_matrix(sec, bas, names[op], qx, qy, fsec, fbas)
        y = m @ seeded_vector(len(bas[0]), int(golden_excitations[f"e{idx}_seed"][0]), True)
        assert np.max(np.abs(y - golden_excitations[f"e{idx}_y"])) < 1e-12


def test_oracle_bit_exact_against_reference_code(oracle):
    if oracle.ref_lib() is None and oracle.REF_SRC is not None and oracle.REF_SRC.is_dir():
        oracle.build(ref=True)
    if oracle.ref_lib() is None:
        pytest.skip("oracle/_ref not built (EXACTDIAG_REF_SRC unset and no prebuilt library)")
    for key in [(4, 2, 3, 1, 0), (5, 2, 4, 2, 1), (6, 0, 6, 1, 1), (6, 3, 4, 0, 0), (7, 1, 6, 3, 1)]:
        sec = oracle.Sector(*key)
        a = oracle.basis(sec)
        b = oracle.basis(sec, impl="ref")
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        for t in oracle.TERMS:
            c1 = oracle.term_columns(sec, t, a)
            c2 = oracle.term_columns(sec, t, a, impl="ref")
            assert np.array_equal(c1[0], c2[0]) and np.array_equal(c1[1], c2[1])
            assert np.max(np.abs(c1[2] - c2[2]), initial=0) < 1e-14


def test_continued_fraction_restatement(oracle):
    rng = np.random.default_rng(5)
    a = rng.uniform(-2, 2, 40)
    b = np.concatenate([[0.0], rng.uniform(0.1, 1.0, 39)])
    zs = np.linspace(-3, 3, 17) + 0.1j
    vec = oracle.continued_fraction(a, b, zs, 2.5)
    for k, z in enumerate(zs):
        assert abs(vec[k] - (-1 / np.pi * 2.5 * oracle.spectral_value_at_z(a, b, z))) < 1e-12


def test_basis_map_file_format_matches_reference(oracle, tmp_path):
    """The basis .dat writer/reader against the reference's own Basis_Index_Map save/load."""
    import ctypes

    from exactdiag_gb300.tJ_spin_half_ladder.matrix_setup import load_basis_map, save_basis_map

    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("the reference's code is not built here")
    i64p, i32p = ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)
    for key in [(6, 2, 5, 1, 1), (8, 2, 7, 0, 0), (5, 0, 5, 2, 0)]:
        sp, orb = oracle.basis(oracle.Sector(*key))
        orb = orb.astype(np.int32)
        ours = tmp_path / f"ours_{key}.dat"
        save_basis_map(ours, sp, orb)
        n = ctypes.c_int64()
        assert ref.ref_basis_load(str(ours).encode(), None, None, ctypes.c_int64(0), ctypes.byref(n)) == 0
        rs, ro = np.zeros(n.value, np.int64), np.zeros(n.value, np.int32)
        assert ref.ref_basis_load(str(ours).encode(), rs.ctypes.data_as(i64p), ro.ctypes.data_as(i32p),
                                  ctypes.c_int64(n.value), ctypes.byref(n)) == 0
        assert np.array_equal(rs, sp) and np.array_equal(ro, orb)
        theirs = tmp_path / f"theirs_{key}.dat"
        assert ref.ref_basis_save(str(theirs).encode(), sp.ctypes.data_as(i64p), orb.ctypes.data_as(i32p),
                                  ctypes.c_int64(len(sp))) == 0
        assert theirs.read_bytes() == ours.read_bytes()
        ls, lo = load_basis_map(theirs)
        assert np.array_equal(ls, sp) and np.array_equal(lo, orb)


def test_basis_map_file_rejects_truncation(tmp_path):
    from exactdiag_gb300.tJ_spin_half_ladder.matrix_setup import load_basis_map, save_basis_map

    p = tmp_path / "b.dat"
    save_basis_map(p, np.arange(10, dtype=np.int64), np.full(10, 4, np.int32))
    data = p.read_bytes()
    p.write_bytes(data[:-3])
    with pytest.raises(ValueError):
        load_basis_map(p)


EXCITATION_SOURCES = [(4, 1, 2, 1, 0), (5, 2, 4, 2, 1), (5, 1, 4, 0, 0), (6, 2, 5, 3, 0), (6, 1, 5, 1, 1),
                      (6, 0, 6, 2, 0), (4, 2, 2, 0, 1), (7, 3, 5, 1, 0)]


@pytest.mark.parametrize("name", ["Szq", "spectral_function_minus", "spectral_function_plus", "current_rung",
                                  "current_leg"])
def test_oracle_excitations_bit_exact_against_reference_code(oracle, name):
    """Operator columns of the restatement against the reference's own column functions."""
    if oracle.ref_lib() is None:
        pytest.skip("the reference's code is not built here")
    cases = 0
    for key in EXCITATION_SOURCES:
        sec = oracle.Sector(*key)
        if name == "spectral_function_plus" and sec.Nh == 0:
            continue
        if name == "spectral_function_minus" and sec.Nh == sec.N:
            continue
        bas = oracle.basis(sec)
        for qx in range(sec.L):
            for qy in (0, 1):
                fsec = oracle.target_sector(sec, name, qx, qy)
                fbas = oracle.basis(fsec)
                a = oracle.excitation_columns(sec, bas, name, qx, qy, fsec, fbas)
                b = oracle.excitation_columns(sec, bas, name, qx, qy, fsec, fbas, impl="ref")
                assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (key, qx, qy)
                assert np.max(np.abs(a[2] - b[2]), initial=0) < 1e-14, (key, qx, qy)
                cases += 1
    assert cases > 0


def test_oracle_position_correlation_sum_rules(oracle):
    """Summed over distances, hole correlations give Nh^2 and S^z correlations (2 S^z)^2 per unit norm."""
    rng = np.random.default_rng(4)
    for key in [(4, 2, 3, 0, 0), (5, 1, 4, 1, 1), (4, 0, 3, 1, 0)]:
        sec = oracle.Sector(*key)
        bas = oracle.basis(sec)
        psi = rng.normal(size=len(bas[0])) + 1j * rng.normal(size=len(bas[0]))
        psi /= np.linalg.norm(psi)
        holes = oracle.position_correlations(sec, bas, psi, "hole_correlations")
        spins = oracle.position_correlations(sec, bas, psi, "Sz_correlations")
        assert abs(holes.sum() - sec.Nh ** 2) < 1e-12
        assert abs(spins.sum() - sec.Sz2 ** 2) < 1e-12
        assert abs(holes[0] - sec.Nh) < 1e-12 and abs(spins[0] - (sec.N - sec.Nh)) < 1e-12


def test_oracle_singlet_operator_bit_exact_against_reference_code(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("the reference's code is not built here")
    for key in [(5, 2, 4, 0, 0), (6, 4, 4, 0, 0), (5, 3, 3, 2, 1), (6, 2, 5, 1, 0)]:
        sec = oracle.Sector(*key)
        bas = oracle.basis(sec)
        for fixed in [((1, 1), (1, 1)), ((1, 0), (0, 1)), ((0, 1), (1, 0))]:
            for d in range(sec.N):
                shifts = [fixed[0], fixed[1], (d // 2, d % 2)]
                a = oracle.singlet_columns(sec, bas, shifts)
                b = oracle.singlet_columns(sec, bas, shifts, impl="ref")
                assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (key, fixed, d)
                assert np.max(np.abs(a[2] - b[2]), initial=0) < 1e-14, (key, fixed, d)
