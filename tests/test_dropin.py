"""The drop-in layer: the reference's own routine names and signatures
(include/turbins_dropin.h, libturbdropin.so).

CPU tests: the layer compiles against the reference's own headers with every
definition checked against the reference prototype (a conflicting type is a
compile error); the library exports every routine the header declares; and,
preloaded into a program linked against the reference's compiled routines,
it takes their calls (symbol interposition, the way a TURBINS build would
pick it up).  GPU test: a C host step written with the reference's names
(tests/dropin/dropin_step.c) runs one TVD-RK2 step through the layer; it
must give the same bits as the library's own turb_step and agree with the
oracle's step.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "turbins_dropin.h")
SRC = os.path.join(ROOT, "turbins_gb300", "dropin", "turbins_dropin.c")
SHIM = os.path.join(ROOT, "oracle", "shim")


def _declared():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:void|int|double)\s+\**\s*(\w+)\s*\(", txt, flags=re.M)))


def _lib():
    from turbins_gb300 import build
    build.build()
    return build.DROPIN


def test_dropin_prototypes_match_reference():
    from oracle import refbuild
    if not refbuild.available():
        pytest.skip("reference checkout not present")
    r = subprocess.run(["gcc", "-fsyntax-only", "-Wall", "-Werror", "-DTURB_DROPIN_REFERENCE_HEADERS",
                        "-I", SHIM, "-I", os.path.join(refbuild.SRC, "Include"), SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_dropin_exports_every_declared_routine():
    names = _declared()
    assert "Pressure_solve" in names and "Velocity_u_set_RHS" in names and len(names) >= 28
    out = subprocess.run(["nm", "-D", "--defined-only", _lib()], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_dropin_interposes_the_reference(tmp_path):
    """a program linked against the reference's compiled routines, with the
    layer preloaded: its call of Velocity_solve reaches the layer (which
    reports the unbound struct) instead of the reference's routine"""
    from oracle import refbuild
    if not refbuild.available():
        pytest.skip("reference checkout not present")
    ref = refbuild.build()
    drv = tmp_path / "drv.c"
    drv.write_text('#include <stdio.h>\n'
                   'typedef struct velocity Velocity;\n'
                   'int Velocity_solve(Velocity *vel);\n'
                   'int main(void) { static char key; int it = Velocity_solve((Velocity *)&key);'
                   ' printf("iters=%d\\n", it); return 0; }\n')
    exe = tmp_path / "drv"
    subprocess.check_call(["gcc", str(drv), "-o", str(exe), ref, "-Wl,-rpath," + os.path.dirname(ref), "-lm"])
    env = dict(os.environ, LD_PRELOAD=_lib())
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=60)
    assert r.returncode == 0, r.stderr
    assert "iters=-1" in r.stdout
    assert "turbins_dropin: Velocity_solve" in r.stderr


def _build_driver(tmp):
    lib = _lib()
    so = os.path.join(tmp, "libdropinstep.so")
    libdir = os.path.dirname(lib)
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-o", so,
                           os.path.join(ROOT, "tests", "dropin", "dropin_step.c"), os.path.join(SHIM, "shim.c"),
                           "-I", SHIM, "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lturbdropin", "-lturbgpu",
                           "-Wl,-rpath," + libdir, "-lm"])
    return so


def test_dropin_step_refuses_unbound_keys(tmp_path):
    """the fused step through a GVG_bag: a bag whose grid has no context, or
    an unbound bag, is refused with TURB_ERR_ARG, which turb_dropin_status
    reports once (CPU: no device call is reached)"""
    lib = _lib()
    libdir = os.path.dirname(lib)
    prog = tmp_path / "bag.c"
    prog.write_text(
        '#include <stdio.h>\n#include "turbins_dropin.h"\n'
        'int main(void) {\n'
        '  static char bag_key, grid_key; GVG_bag *bag = (GVG_bag *)&bag_key;\n'
        '  MAC_grid *grid = (MAC_grid *)&grid_key; int st = 12345;\n'
        '  int a = turb_dropin_bind_bag(NULL, grid), b = turb_dropin_bind_bag(bag, grid);\n'
        '  int c = turb_dropin_step(bag, 1e-3, &st), d = turb_dropin_status(), e = turb_dropin_status();\n'
        '  int f = turb_dropin_step(NULL, 1e-3, NULL);\n'
        '  printf("%d %d %d %d %d %d %d %d\\n", TURB_ERR_ARG, a, b, c, st, d, e, f);\n'
        '  return 0;\n}\n')
    exe = tmp_path / "bag"
    subprocess.check_call(["gcc", "-O2", str(prog), os.path.join(SHIM, "shim.c"), "-I", SHIM,
                           "-I", os.path.join(ROOT, "include"), "-o", str(exe), "-L", libdir, "-lturbdropin",
                           "-lturbgpu", "-Wl,-rpath," + libdir, "-lm"])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    err, a, b, c, st, d, e, f = map(int, r.stdout.split())
    assert err != 0
    assert (a, b, c, st, d, e, f) == (err, err, err, err, err, 0, err)
    assert "turbins_dropin: turb_dropin_step" in r.stderr


def test_driver_builds_without_reference(tmp_path):
    """the host step compiles and links against the layer with no reference
    header in sight (CPU: build only)"""
    assert os.path.exists(_build_driver(str(tmp_path)))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lock", "multi"])
def test_dropin_step_matches_library_and_oracle(tmp_path, name):
    from oracle.oracle import Oracle
    from tests import _cases
    from turbins_gb300 import api
    case = _cases.lock_small() if name == "lock" else _cases.multi_small()
    g, p = case.grid, case.params
    drv = C.CDLL(_build_driver(str(tmp_path)))
    keys = ["u", "v", "w", "phi", "dpx", "dpy", "dpz"] + ["c%d" % i for i in range(p.nconc)]
    fields = [np.ascontiguousarray(case.state[k], dtype=np.float64).copy() for k in keys]
    arr = (C.c_void_p * len(fields))(*[f.ctypes.data for f in fields])
    ctx = api.Context(g, p)
    divs = (C.c_double * 2)()
    its = (C.c_int * 5)()
    rc = drv.dropin_step(ctx.ctx, g.nx, g.ny, g.nz, p.nconc, C.c_double(case.dt), arr, divs, its)
    assert rc == 0, api.load_library().turb_status_string(rc)
    ctx.close()
    assert max(divs) <= 1e-10 and its[4] > 0
    # the library's own step from the same state: the same calls, the same bits
    ctx2 = api.Context(g, p)
    ctx2.load_state(case.state)
    ctx2.step(case.dt)
    lib_state = ctx2.state()
    ctx2.close()
    got = dict(zip(keys, fields))
    for k in keys:
        assert np.array_equal(got[k], lib_state[k]), k
    # and the oracle's step (tolerances of the step comparisons: solvers to
    # their relative residuals, velocities within 1e-7 of their scale)
    ref = {k: v.copy() for k, v in case.state.items()}
    Oracle(g, p).step(ref, case.dt)
    vscale = max(float(np.abs(ref[k]).max()) for k in "uvw")
    for k in ("u", "v", "w"):
        assert float(np.abs(got[k] - ref[k]).max()) <= 1e-7 * vscale, k
    for i in range(p.nconc):
        k = "c%d" % i
        assert float(np.abs(got[k] - ref[k]).max()) <= 1e-6 * max(float(np.abs(ref[k]).max()), 1.0), k
