"""Restart files (checkpoint / resume) in the reference's formats.

tests/golden/resume_bump holds a restart set written by the reference's own
Resume.c (compiled through the harness, tests/golden/make_golden.py).  The
numpy restatement (oracle/resume_format.py) must reproduce those files byte
for byte, and the library's host-side writers and readers (no GPU needed)
must agree with both."""
import filecmp
import json
import os

import numpy as np
import pytest

from oracle import resume_format as F
from tests import _cases

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "resume_bump")


def golden():
    meta = json.load(open(os.path.join(GOLD, "case.json")))
    c = meta["case"]
    case = _cases.bump_small(c["nx"], c["ny"], c["nz"])
    return case, meta


def decoded(case):
    g, p = case.grid, case.params
    shape = (g.nz + 1, g.ny + 1, g.nx + 1)
    st = {key: F.read_vec(os.path.join(GOLD, name), shape) for name, key in F.field_files(p.nconc, grid=True)}
    dep = np.zeros((p.nconc, g.nz + 1, g.nx + 1))
    for ic in range(p.nconc):
        if p.ctype[ic] == 2:
            dep[ic] = np.fromfile(os.path.join(GOLD, F.deposit_file(ic)), dtype=np.float64).reshape(g.nz + 1, g.nx + 1)
    return st, dep


def test_golden_set_matches_case():
    case, meta = golden()
    st, dep = decoded(case)
    s = _cases.random_state(case, seed=meta["case"]["seed"])
    for k in ("u", "v", "w", "dpx", "dpy", "dpz", "c0"):
        assert np.array_equal(st[k], s[k]), k
    assert np.array_equal(st["status_c"], case.grid.status["c"].astype(np.float64))
    assert dep.max() > 0.0


def test_oracle_restatement_reproduces_reference_files(tmp_path):
    case, meta = golden()
    st, dep = decoded(case)
    p = case.params
    F.write_set(str(tmp_path), st, p.nconc, meta["prim"], grid_status=case.grid.status["c"], deposit=dep,
                particle=[i for i in range(p.nconc) if p.ctype[i] == 2])
    names = sorted(f for f in os.listdir(GOLD) if f.startswith("Resume_"))
    assert names == sorted(os.listdir(tmp_path))
    for f in names:
        assert filecmp.cmp(os.path.join(GOLD, f), os.path.join(tmp_path, f), shallow=False), f
    prim = F.read_primary(os.path.join(GOLD, "Resume_primary.dat"))
    assert prim["iter"] == meta["prim"]["iter"] and prim["time"] == round(meta["prim"]["time"], 6)


def test_library_host_writers_and_readers(tmp_path):
    from turbins_gb300 import api as A
    try:
        A.load_library()
    except A.TurbError:
        pytest.skip("libturbgpu.so not built")
    case, meta = golden()
    st, dep = decoded(case)
    shape = st["u"].shape
    for name, key in F.field_files(case.params.nconc, grid=True):
        out = os.path.join(tmp_path, name)
        A.petsc_vec_write(out, st[key])
        assert filecmp.cmp(out, os.path.join(GOLD, name), shallow=False), name
        assert np.array_equal(A.petsc_vec_read(os.path.join(GOLD, name), shape), st[key])
    A.resume_primary_write(str(tmp_path), meta["prim"])
    assert filecmp.cmp(os.path.join(tmp_path, "Resume_primary.dat"), os.path.join(GOLD, "Resume_primary.dat"),
                       shallow=False)
    q = A.resume_primary_read(GOLD)
    assert q == F.read_primary(os.path.join(GOLD, "Resume_primary.dat"))
    f2 = os.path.join(tmp_path, F.deposit_file(0))
    A.resume_2d_write(f2, dep[0])
    assert filecmp.cmp(f2, os.path.join(GOLD, F.deposit_file(0)), shallow=False)
    assert np.array_equal(A.resume_2d_read(os.path.join(GOLD, F.deposit_file(0)), *dep[0].shape), dep[0])
    # a missing file is an I/O error, a vector of another size a format error
    with pytest.raises(A.TurbError) as e:
        A.petsc_vec_read(os.path.join(tmp_path, "absent.bin"), shape)
    assert e.value.code == 7
    with pytest.raises(A.TurbError) as e:
        A.petsc_vec_read(os.path.join(GOLD, "Resume_u.bin"), (3, 4))
    assert e.value.code == 8


def test_reference_regenerates_golden(tmp_path):
    """the committed files are what the reference writes (here only)"""
    from oracle import refbuild
    if not refbuild.available():
        pytest.skip("reference sources not present")
    from oracle.refcheck import Reference
    case, meta = golden()
    s = _cases.random_state(case, seed=meta["case"]["seed"])
    st, dep = decoded(case)
    ref = Reference(case.grid, case.params)
    ref.resume_write(str(tmp_path), s, meta["prim"], grid=True, dep=dep)
    for f in sorted(os.listdir(tmp_path)):
        assert filecmp.cmp(os.path.join(GOLD, f), os.path.join(tmp_path, f), shallow=False), f
    back, prim, d = ref.resume_read(GOLD, grid=True, dep=True)
    for k in back:
        assert np.array_equal(back[k], st[k]), k
    assert np.array_equal(d, dep)
