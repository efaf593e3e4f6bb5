"""Restart-file formats of the reference (Resume.c), restated with numpy.

TEST INFRASTRUCTURE ONLY: the checker of the library's restart writer and
reader (tests/); nothing in the product imports it.

* 3-D fields: PETSc binary vectors as Resume_write_data (Resume.c:98-121)
  writes them through VecView, and Resume_read_data (Resume.c:124-151) loads
  them through VecLoadIntoVector.  PETSc is a third-party dependency of the
  reference (PETSc 3.1, README.md:18) and not part of the checkout; its
  published binary layout for a vector is the int32 pair
  {VEC_FILE_COOKIE = 1211214, N} followed by N doubles, every word
  big-endian.  On one rank a DA vector's natural order is its DA order
  [k][j][i].
* Resume_primary.dat: Resume_write_primary_data (Resume.c:248-279), C's %lf
  (6 decimals) and %d.
* 2-D [NZ][NX] arrays: Resume_write_2D_data (Resume.c:321-351), raw doubles in
  the host's byte order.
* The vector set and its file names: Resume_set_data (Resume.c:208-244).
"""
from __future__ import annotations

import os

import numpy as np

VEC_COOKIE = 1211214


def vec_bytes(a):
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    return np.array([VEC_COOKIE, a.size], dtype=">i4").tobytes() + a.astype(">f8").tobytes()


def write_vec(path, a):
    with open(path, "wb") as f:
        f.write(vec_bytes(a))


def read_vec(path, shape=None):
    raw = open(path, "rb").read()
    cookie, n = np.frombuffer(raw[:8], dtype=">i4")
    if cookie != VEC_COOKIE or len(raw) != 8 + 8 * int(n):
        raise ValueError("%s: not a PETSc binary vector" % path)
    a = np.frombuffer(raw[8:], dtype=">f8").astype(np.float64)
    return a.reshape(shape) if shape is not None else a


def primary_text(time, dt, dt_old, iteration, output_iter):
    return "time=\n%f\ndt=\n%f\ndt_old=\n%f\niteration=\n%d\noutput_iter=\n%d\n" % (
        time, dt, dt_old, iteration, output_iter)


def read_primary(path):
    t = open(path).read().split()
    return dict(time=float(t[1]), dt=float(t[3]), dt_old=float(t[5]), iter=int(t[7]), output_iter=int(t[9]))


def field_files(nconc, grid=False):
    """(file name, state key) of the restart set, in Resume_set_data's order"""
    out = [("Resume_u.bin", "u"), ("Resume_v.bin", "v"), ("Resume_w.bin", "w"), ("Resume_dpdx.bin", "dpx"),
           ("Resume_dpdy.bin", "dpy"), ("Resume_dpdz.bin", "dpz")]
    if grid:
        out.append(("Resume_gridc.bin", "status_c"))
    out += [("Resume_conc%d.bin" % i, "c%d" % i) for i in range(nconc)]
    return out


def deposit_file(ic):
    return "Resume_deposit_height%d.bin" % ic


def write_set(dirname, state, nconc, prim, grid_status=None, deposit=None, particle=()):
    """the whole restart set, as the reference writes it"""
    for name, key in field_files(nconc, grid_status is not None):
        write_vec(os.path.join(dirname, name), grid_status.astype(np.float64) if key == "status_c" else state[key])
    with open(os.path.join(dirname, "Resume_primary.dat"), "w") as f:
        f.write(primary_text(prim["time"], prim["dt"], prim["dt_old"], prim["iter"], prim["output_iter"]))
    if deposit is not None:
        for ic in range(nconc):
            if ic in particle:
                np.ascontiguousarray(deposit[ic], dtype=np.float64).tofile(os.path.join(dirname, deposit_file(ic)))
