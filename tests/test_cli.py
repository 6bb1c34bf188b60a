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


def _cli(*args, cwd=None):
    if not os.path.exists(B.CLI):
        B.build()
    return subprocess.run([B.CLI, *args], capture_output=True, text=True, cwd=cwd, timeout=300)


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
