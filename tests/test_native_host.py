"""CPU: host-compiled checks of the descriptor builder (tests/native/*.cu), built with nvcc as host
code -- no GPU is touched."""

import pathlib
import shutil
import subprocess

import pytest

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE.parent / "exactdiag_gb300" / "csrc"


def _nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not pathlib.Path(exe).exists():
        pytest.skip("nvcc not available")
    return exe


def _build_and_run(tmp_path, name: str) -> str:
    exe = tmp_path / name
    build = subprocess.run([_nvcc(), "-std=c++17", "--expt-relaxed-constexpr", "-O2",
                            "-gencode", "arch=compute_103a,code=sm_103a", f"-I{CSRC}",
                            f"-I{HERE.parent / 'include'}", str(HERE / "native" / f"{name}.cu"), "-o", str(exe)],
                           capture_output=True, text=True, timeout=600)
    assert build.returncode == 0, build.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout[-3000:]
    assert "differences 0" in run.stdout
    return run.stdout


def test_coset_phases_compose_with_the_stabiliser(tmp_path):
    """Resolving through a hole mask's coset equals mapping by its first element and resolving with
    the canonical mask's stabiliser, phases added (L = 4..8, 1-4 holes, every momentum)."""
    _build_and_run(tmp_path, "coset_phase_check")


def test_rank_tables_unrank_and_next_combination(tmp_path):
    """The spin-rank tables of every (Ns, Nd) give the colex rank; unranking and the
    next-combination step of the stabiliser expansion invert and advance it."""
    _build_and_run(tmp_path, "rank_tables_check")


def test_chunk_plan_cuts_each_sector_the_same_alone_and_batched(tmp_path):
    """plan_chunks on synthetic sectors: row chunks tile the rows inside their blocks with the
    per-kind lengths, segment chunks tile every class of every free block, a sector is cut
    identically alone and in a batch, stabiliser chunks point at their block's expanded copy."""
    _build_and_run(tmp_path, "chunk_plan_check")


def test_segment_layout_reaches_every_target_rank(tmp_path):
    """The segment kernel's index arithmetic (ed_seg.cuh helpers, seg_tables) against the colex rank:
    segments tile each block, and every exchange pair and hop permutation reaches the rank of the
    flipped or permuted configuration, for Ns = 3 .. 31."""
    _build_and_run(tmp_path, "seg_layout_check")
