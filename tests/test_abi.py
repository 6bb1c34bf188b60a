"""The C-ABI library loads and exports every entry point of include/doug_gpu.h."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared():
    txt = open(os.path.join(ROOT, "include", "doug_gpu.h")).read()
    return sorted(set(re.findall(r"\b(dg_[a-z_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from doug_gb300.build import build
    return ctypes.CDLL(build())


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert "dg_solve" in names and "dg_setup" in names
    for nm in names:
        assert hasattr(lib, nm), nm


def test_python_mirror_lists_the_same_symbols():
    import doug_gb300 as D
    assert sorted(D.EXPORTED_SYMBOLS) == _declared()


def test_solve_before_setup_is_an_error_not_a_crash(lib):
    import doug_gb300 as D
    s = D.DougSolver()
    with pytest.raises(D.DougError) as e:
        s.solve()
    assert e.value.status == D.DG_NOT_READY


def test_bad_control_value_is_rejected():
    import doug_gb300 as D
    s = D.DougSolver()
    with pytest.raises(D.DougError) as e:
        s.set_option("levels", "two")
    assert e.value.status == D.DG_BAD_INPUT


def test_missing_control_file_is_rejected():
    import doug_gb300 as D
    s = D.DougSolver()
    with pytest.raises(D.DougError) as e:
        s.load_ctl("/nonexistent/DOUG.ctl")
    assert e.value.status == D.DG_BAD_INPUT
