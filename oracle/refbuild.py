"""Build recipe of the reference-compiled checker (TEST INFRASTRUCTURE ONLY).

Compiles the reference's own hot-path C files, unmodified, from where they lie
in the read-only reference checkout, against the single-rank PETSc shim
(oracle/shim), together with ref_harness.c, into oracle/_ref/libturbins_ref.so.
Symbols the compiled files reference but never reach on the harness's paths
(surface/level-set set-up, KSP factories, output) get stubs that abort if
called.  Requires gcc; does not run the reference's own build system (it has
none in the checkout).  Output goes to oracle/_ref/ only.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: TURB_REFERENCE_ROOT, else a checkout named
# "reference" beside this repository
REF = os.environ.get("TURB_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
SRC = os.path.join(REF, "src")
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libturbins_ref.so")
FILES = ["ENO", "Velocity", "Conc", "Pressure", "Grid", "Immersed", "MyMath", "Memory", "Communication", "Extract",
         "Resume", "Solver", "Inflow", "Outflow", "Surface", "Levelset"]
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w"]


def available():
    return all(os.path.exists(os.path.join(SRC, f + ".c")) for f in FILES)


def build(force=False):
    if not available():
        raise FileNotFoundError("reference sources not found under %s" % SRC)
    own = [os.path.join(HERE, "ref_harness.c")] + [os.path.join(HERE, "shim", f)
                                                    for f in os.listdir(os.path.join(HERE, "shim"))]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in own):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "shim"), "-I" + os.path.join(SRC, "Include")]
    objs = []
    for f in FILES:
        o = os.path.join(OUT, f + ".o")
        subprocess.check_call(["gcc", "-c"] + CFLAGS + inc + [os.path.join(SRC, f + ".c"), "-o", o])
        objs.append(o)
    for src in (os.path.join(HERE, "shim", "shim.c"), os.path.join(HERE, "ref_harness.c")):
        o = os.path.join(OUT, os.path.basename(src)[:-2] + ".o")
        subprocess.check_call(["gcc", "-c"] + CFLAGS + inc + [src, "-o", o])
        objs.append(o)
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-shared", "-o", tmp] + objs + ["-lm"])
    und = subprocess.run(["nm", "-u", tmp], capture_output=True, text=True).stdout.split("\n")
    names = [ln.split()[-1] for ln in und if ln.strip().startswith("U ") and "@" not in ln]
    if names:
        with tempfile.NamedTemporaryFile("w", suffix=".c", delete=False, dir=OUT) as fh:
            fh.write("#include <stdio.h>\n#include <stdlib.h>\n")
            for nm in names:
                if nm.startswith("Display_"):   # console output only
                    fh.write("void %s(void) { }\n" % nm)
                else:
                    fh.write("void %s(void) { fprintf(stderr, \"ref stub %s called\\n\"); abort(); }\n" % (nm, nm))
            stub = fh.name
        so = stub[:-2] + ".o"
        subprocess.check_call(["gcc", "-c"] + CFLAGS + [stub, "-o", so])
        subprocess.check_call(["gcc", "-shared", "-o", tmp] + objs + [so, "-lm"])
    os.replace(tmp, LIB)
    return LIB


def build_if_available():
    if available():
        return build()
    return None


if __name__ == "__main__":
    print(build(force=True))
