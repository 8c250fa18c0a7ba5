"""CPU: the C-ABI library builds for sm_103a, loads, and exports every symbol include/*.h declares.

No compute call is made (there is no GPU here); device behaviour is covered by the gpu-marked tests.
"""

import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(ed_[a-z_0-9]+)\s*\(", text, flags=re.M))
    return names


def test_header_declares_the_boundary():
    names = declared_symbols()
    for required in ("ed_sector_create", "ed_basis_build", "ed_hv", "ed_lanczos_step", "ed_continued_fraction",
                     "ed_last_error_string"):
        assert required in names


def test_library_builds_and_exports_every_declared_symbol():
    from exactdiag_gb300 import build, _native

    lib_path = build.build()
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the Python binding
    assert declared_symbols() <= set(_native.SIGNATURES)


def test_error_string_without_gpu():
    from exactdiag_gb300 import _native

    lib = _native.load(build_if_missing=True)
    # argument validation happens before any device work
    rc = lib.ed_sector_create(1, 0, 0, 0, 0, None)
    assert rc == -1
    assert b"out is NULL" in lib.ed_last_error_string()
    out = ctypes.c_void_p()
    rc = lib.ed_sector_create(20, 0, 0, 0, 0, ctypes.byref(out))
    assert rc == -1 and b"L must be" in lib.ed_last_error_string()
    rc = lib.ed_sector_create(4, 2, 3, 0, 2, ctypes.byref(out))
    assert rc == -1 and b"ky" in lib.ed_last_error_string()


def test_device_ops_refuse_without_cuda():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    from exactdiag_gb300.engine import DeviceSector

    with pytest.raises(RuntimeError, match="CUDA"):
        DeviceSector(4, 2, 3, 0, 0)
