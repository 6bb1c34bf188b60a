"""doug_geom: one subdomain of all unknowns (or imported parts) and, for
elemental input with levels 2, the geometric coarse grid
(CoarsePreconditioner_geometric.F90:34-115, coarse/geom/*).

No reference fixture pins the coarse grid itself; the reference's own test
matrix runs the e4x4 fixture through doug_geom at levels 1 and 2
(tests/tests_all.conf:34-62) and checks the solution against csolution.xdr.
Here: the oracle's multilinear restriction with box centres reproduces
constants and linear functions exactly (its defining property), the oracle
solves the e4x4 fixture, the product's host setup gives R, AC, subdomains and
coarse coordinates bit-equal to the oracle, and (GPU) the solutions match the
oracle's (FP64: relative 1e-10, iterations +-1; mixed: 1e-7).
"""
import os

import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

from conftest import GOLDEN

BASE = "input_type 1\nsolver 2\nmethod 1\nsolve_tolerance 1.0e-10\nsolve_maxiters 500\n"
E4 = os.path.join(GOLDEN, "e4x4")
GEOM = "executable geom\nlevels 2\n"
WORDS = [GEOM, GEOM + "maxcie 16\nmaxnd 60\ncutbal 3\n", GEOM + "maxcie 9\nmaxnd 200\ncutbal 2\ncenter_type 2\n",
         GEOM + "interpolation_type 2\nmaxnd 60\ncutbal 3\nmaxcie 16\n",
         GEOM + "interpolation_type 3\nmaxnd 60\ncutbal 3\nmaxcie 16\n", "executable geom\nlevels 1\noverlap 2\n"]


def _mesh(folder, gen):
    ngf, eptr, efree, emat, erhs, info = gen
    files = P.write_elemental_files(str(folder), ngf, eptr, efree, emat, erhs, info)
    text = "".join(f"{k} {v}\n" for k, v in files.items()) + BASE
    (folder / "DOUG.ctl").write_text(text)
    return str(folder / "DOUG.ctl"), info


@pytest.fixture(scope="module")
def p1(tmp_path_factory):
    return _mesh(tmp_path_factory.mktemp("p1"), P.poisson2d_p1_elements(33, seed=3))


@pytest.fixture(scope="module")
def elas(tmp_path_factory):
    return _mesh(tmp_path_factory.mktemp("elas"), P.elasticity3d_p1_elements(6, seed=2))


def _product(ctl, words, part=None):
    s = D.DougSolver({})
    for line in words.strip().splitlines():
        k, v = line.split()
        s.set_option(k, v)
    s.load_ctl(ctl)
    if part is not None:
        s.set_partition(part)
    return s


@pytest.mark.parametrize("mesh", ["p1", "elas"])
@pytest.mark.parametrize("extra", ["", "maxcie 16\nmaxnd 60\ncutbal 3\n", "maxcie 8\nmaxnd 120\ncutbal 2\n"])
def test_oracle_multilinear_reproduces_linear_functions(request, mesh, extra):
    ctl, info = request.getfixturevalue(mesh)
    r = O.run_ctl(ctl, GEOM + extra)
    assert r["status"] == 0, r["errmsg"]
    _, _, ri, rj, rv = r["R"]
    X = r["coarse_xyz"]
    xf = info["coords"][info["freemap"] - 1]
    n = r["n"]
    one = np.zeros(n)
    lin = np.zeros((n, X.shape[1]))
    np.add.at(one, rj - 1, rv)
    np.add.at(lin, rj - 1, rv[:, None] * X[ri - 1])
    # entries <= 1e-9 are dropped (GeomInterp.f90:200-214)
    assert np.abs(one - 1).max() < 1e-8
    assert np.abs(lin - xf).max() < 1e-8
    assert r["R"][0] > 0 and r["iterations"] >= 1


@pytest.mark.parametrize("words", ["executable geom\nlevels 1\n", GEOM, GEOM + "interpolation_type 2\n",
                                   GEOM + "interpolation_type 3\n", GEOM + "center_type 2\nmaxcie 9\ncutbal 1\n",
                                   GEOM + "overlap 1\n"])
def test_oracle_e4x4_fixture(words):
    r = O.run_ctl(os.path.join(E4, "DOUG.ctl"), words)
    assert r["status"] == 0, r["errmsg"]
    ref = O.read_vector(os.path.join(E4, "csolution.xdr"), 2, 9)
    assert np.linalg.norm(r["x"] - ref) <= 1e-9
    assert len(r["subdomains"]) == 1 and len(r["subdomains"][0]) == 9


# the reference harness's doug_geom runs on the e4x4 fixture
# (tests/tests_all.conf:34-62): e1lev = levels 1, fine_methods 1,2, smoothers 0,
# overlaps -1,0,1,2; e2lev = levels 2, fine_methods 1,2, smoothers 0,1,2, overlaps -1,0
HARNESS = ([(1, f, 0, o) for f in (1, 2) for o in (-1, 0, 1, 2)] +
           [(2, f, sm, o) for f in (1, 2) for sm in (0, 1, 2) for o in (-1, 0)])


def _harness_words(levels, fine, smoothers, overlap):
    return (f"executable geom\nlevels {levels}\nfine_method {fine}\nsmoothers {smoothers}\n"
            f"overlap {overlap}\n")


@pytest.mark.parametrize("levels,fine,smoothers,overlap", HARNESS)
def test_oracle_e4x4_harness_matrix(levels, fine, smoothers, overlap):
    r = O.run_ctl(os.path.join(E4, "DOUG.ctl"), _harness_words(levels, fine, smoothers, overlap))
    assert r["status"] == 0, r["errmsg"]
    ref = O.read_vector(os.path.join(E4, "csolution.xdr"), 2, 9)
    assert np.linalg.norm(r["x"] - ref) <= 1e-9   # the harness accepts 1e-6
    assert r["smoothers"] == (0 if levels == 2 else smoothers)


@pytest.mark.parametrize("mesh", ["p1", "elas"])
@pytest.mark.parametrize("words", WORDS)
def test_host_setup_equals_oracle(request, mesh, words):
    ctl, info = request.getfixturevalue(mesh)
    ro = O.run_ctl(ctl, words)
    assert ro["status"] == 0, ro["errmsg"]
    s = _product(ctl, words)
    s.setup_host_only()
    ri, rj, rv = s.restriction()
    ci, cj, cv = s.coarse_matrix()
    assert np.array_equal(ri, ro["R"][2]) and np.array_equal(rj, ro["R"][3])
    assert np.array_equal(rv.view(np.int64), ro["R"][4].view(np.int64))
    assert np.array_equal(ci, ro["AC"][1]) and np.array_equal(cj, ro["AC"][2])
    assert np.array_equal(cv.view(np.int64), ro["AC"][3].view(np.int64))
    sd = s.subdomains()
    assert len(sd) == len(ro["subdomains"]) == 1
    assert np.array_equal(sd[0], ro["subdomains"][0])
    if ro["coarse_xyz"] is not None:
        assert np.array_equal(s.coarse_coords(), ro["coarse_xyz"])
    assert s.sizes()["nagr_fine"] == 0


def test_host_setup_with_partition_equals_oracle(p1):
    ctl, info = p1
    part = np.where(info["coords"][info["freemap"] - 1][:, 0] < 0.5, 1, 2)
    words = GEOM + "maxcie 16\nmaxnd 60\ncutbal 3\noverlap 2\n"
    ro = O.run_ctl(ctl, words, part=part)
    s = _product(ctl, words, part)
    s.setup_host_only()
    sd = s.subdomains()
    assert len(sd) == 2 and all(np.array_equal(a, b) for a, b in zip(sd, ro["subdomains"]))
    ci, cj, cv = s.coarse_matrix()
    assert np.array_equal(cv.view(np.int64), ro["AC"][3].view(np.int64))


def test_geom_input_errors(p1, tmp_path):
    ctl, _ = p1
    # levels 2 needs elemental input with coordinates
    n, r, c, v = P.laplace2d(6)[:4]
    s = D.DougSolver({})
    s.set_option("executable", "geom")
    s.set_option("levels", 2)
    s.set_matrix_coo(n, r, c, v)
    with pytest.raises(D.DougError) as ei:
        s.setup_host_only()
    assert ei.value.status == D.DG_BAD_INPUT
    text = open(ctl).read()
    folder = os.path.dirname(ctl)
    nocoords = "".join(l + "\n" for l in text.splitlines() if not l.startswith(("coords_file", "freemap_file")))
    (tmp_path / "DOUG.ctl").write_text(nocoords.replace("doug_", os.path.join(folder, "doug_")))
    s = _product(str(tmp_path / "DOUG.ctl"), GEOM)
    with pytest.raises(D.DougError):
        s.setup_host_only()
    for words in (GEOM + "hanging_nodes T\n", GEOM + "center_type 3\n", GEOM + "interpolation_type 4\n",
                  "executable geom\nlevels 3\n"):
        s = _product(ctl, words)
        with pytest.raises(D.DougError):
            s.setup_host_only()
    with pytest.raises(D.DougError):
        D.DougSolver({}).set_option("executable", "aggregate")


def test_node_geometry_in_memory_equals_files(p1):
    ctl, info = p1
    ngf, eptr, efree, emat, erhs, info2 = P.poisson2d_p1_elements(33, seed=3)
    words = GEOM + "maxcie 16\nmaxnd 60\ncutbal 3\n"
    a = _product(ctl, words)
    a.setup_host_only()
    b = D.DougSolver({})
    for line in (BASE + words).strip().splitlines():
        k, v = line.split()
        b.set_option(k, v)
    b.set_elements(ngf, eptr, efree, emat, erhs)
    b.set_node_geometry(info2["coords"], info2["freemap"])
    b.setup_host_only()
    for x, y in zip(a.restriction() + a.coarse_matrix(), b.restriction() + b.coarse_matrix()):
        assert np.array_equal(np.asarray(x).view(np.int64) if x.dtype == np.float64 else x,
                              np.asarray(y).view(np.int64) if y.dtype == np.float64 else y)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("mesh,words,parts", [
    ("p1", GEOM + "maxcie 16\nmaxnd 60\ncutbal 3\noverlap 1\n", 4),
    ("p1", GEOM + "interpolation_type 2\nmaxcie 16\nmaxnd 60\ncutbal 3\n", 4),
    ("elas", GEOM + "maxcie 8\nmaxnd 40\ncutbal 4\noverlap 1\n", 2),
    ("p1", GEOM, 0),
])
def test_geom_gpu_matches_oracle(request, precision, mesh, words, parts):
    ctl, info = request.getfixturevalue(mesh)
    part = None
    if parts:
        x = info["coords"][info["freemap"] - 1]
        part = (np.minimum((x[:, 0] * parts).astype(int), parts - 1) + 1).astype(np.int32)
    ro = O.run_ctl(ctl, words, part=part)
    assert ro["status"] == 0, ro["errmsg"]
    s = _product(ctl, words, part)
    s.set_option("precision", precision)
    s.setup()
    x, st = s.solve()
    if precision == 0:
        assert abs(st.iterations - ro["iterations"]) <= 1
        assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
    else:
        assert st.true_rel_residual <= 1.01e-10
        assert np.linalg.norm(x - ro["x"]) <= 1e-7 * np.linalg.norm(ro["x"])


@pytest.mark.gpu
@pytest.mark.parametrize("words", ["executable geom\nlevels 1\n", GEOM, GEOM + "interpolation_type 2\n",
                                   GEOM + "center_type 2\nmaxcie 9\ncutbal 1\n"] +
                         [_harness_words(*h) for h in HARNESS])
def test_geom_gpu_e4x4_fixture(words):
    s = _product(os.path.join(E4, "DOUG.ctl"), words)
    s.setup()
    x, st = s.solve()
    ref = O.read_vector(os.path.join(E4, "csolution.xdr"), 2, 9)
    assert np.linalg.norm(x - ref) <= 1e-9
