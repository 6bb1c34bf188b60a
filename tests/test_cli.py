"""The command-line driver doug_gpu (flags of the reference's executables,
util_parseArgs in DOUG_utils.F90): usage, version, control-word list, errors,
and (GPU) a full run on the reference's lap16x16 fixture writing its solution."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from doug_gb300 import build as B

from conftest import GOLDEN


def _cli(*args, cwd=None, exe=None):
    exe = exe or B.CLI
    if not os.path.exists(exe):
        B.build()
    return subprocess.run([exe, *args], capture_output=True, text=True, cwd=cwd, timeout=300)


def test_usage_version_words():
    r = _cli("-h")
    assert r.returncode == 0 and "-f file.name" in r.stdout
    r = _cli("-v")
    assert r.returncode == 0 and "DOUG version" in r.stdout
    r = _cli("-i")
    assert r.returncode == 0
    words = r.stdout.split()
    for w in ("solve_tolerance", "fine_method", "assembled_mtx_file", "precision"):
        assert w in words


def test_geom_driver_usage():
    r = _cli("-h", exe=B.CLI_GEOM)
    assert r.returncode == 0 and "doug_geom_gpu" in r.stdout
    assert "executable" in _cli("-i").stdout.split()


def test_errors():
    r = _cli("-x")
    assert r.returncode != 0 and "Unrecognised command line parameter: -x" in r.stdout
    r = _cli("-f")
    assert r.returncode != 0 and "no control file given" in r.stdout
    r = _cli("-f", "/nonexistent/DOUG.ctl")
    assert r.returncode != 0 and "DOUG error" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("quiet", [False, True])
def test_run_lap16x16(tmp_path, quiet):
    src = os.path.join(GOLDEN, "lap16x16")
    text = open(os.path.join(src, "DOUG.ctl")).read()
    lines = []
    for line in text.splitlines():
        w = line.split()
        if w and w[0] in ("solution_file", "solution_format"):
            continue                     # the first value of a word wins: set below
        if w and w[0] in ("assembled_mtx_file", "assembled_rhs_file"):
            line = f"{w[0]} {os.path.join(src, os.path.basename(w[1]))}"
        lines.append(line)
    lines += ["fine_method 1", "solution_file sol.xdr", "solution_format 2"]
    (tmp_path / "DOUG.ctl").write_text("\n".join(lines) + "\n")
    args = ["-f", "DOUG.ctl", "-p", "prof"] + (["-q", "run.log"] if quiet else [])
    r = _cli(*args, cwd=str(tmp_path))
    out = (tmp_path / "run.log").read_text() if quiet else r.stdout
    assert r.returncode == 0, out + r.stderr
    assert "#it:" in out and "solution written" in out
    assert (tmp_path / "prof.00").exists()
    x = O.read_vector(str(tmp_path / "sol.xdr"), 2, 225)
    ref = O.read_vector(os.path.join(src, "csolution.xdr"), 2, 225)
    assert np.linalg.norm(x - ref) <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("levels", [1, 2])
def test_geom_driver_e4x4(tmp_path, levels):
    """doug_geom_gpu on the reference's e4x4 fixture (its test matrix runs
    doug_geom at levels 1 and 2, tests/tests_all.conf:34-62)."""
    src = os.path.join(GOLDEN, "e4x4")
    lines = []
    for line in open(os.path.join(src, "DOUG.ctl")).read().splitlines():
        w = line.split()
        if w and w[0] in ("solution_file", "solution_format", "levels"):
            continue
        if w and w[0].endswith("_file") and not w[1].startswith("./NOT"):
            line = f"{w[0]} {os.path.join(src, w[1])}"
        lines.append(line)
    lines += [f"levels {levels}", "solution_file sol.xdr", "solution_format 2"]
    (tmp_path / "DOUG.ctl").write_text("\n".join(lines) + "\n")
    r = _cli("-f", "DOUG.ctl", cwd=str(tmp_path), exe=B.CLI_GEOM)
    assert r.returncode == 0, r.stdout + r.stderr
    x = O.read_vector(str(tmp_path / "sol.xdr"), 2, 9)
    ref = O.read_vector(os.path.join(src, "csolution.xdr"), 2, 9)
    assert np.linalg.norm(x - ref) <= 1e-9
