"""Host binding of the learned pressure guess (turb_net_* / turb_snaps_* of
include/turbins_gb300.h).

``Net`` is the 4-level 3-D U-Net (channels 16-32-64-128) that proposes an
initial guess for the Poisson solve; ``Snapshots`` is the device store of its
inputs, recorded by a ``Context`` during plain solves and read by training.
The solver uses a network guess only when it lowers the initial residual, so
the network changes iteration counts, never the converged pressure.  Device
arrays passed to the raw entry points are torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .api import TurbError, _check, load_library

_vp = C.c_void_p


def _dev(t):
    return _vp(t.data_ptr())


class Net:
    def __init__(self, nx, ny, nz, train=False):
        self.lib = load_library()
        self.lib.turb_net_num_params.restype = C.c_longlong
        h = _vp()
        _check(self.lib.turb_net_create(nx, ny, nz, 1 if train else 0, C.byref(h)), "turb_net_create")
        self.h = h
        self.dims = (nx, ny, nz)
        self.train = train

    def close(self):
        if self.h:
            self.lib.turb_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self):
        return int(self.lib.turb_net_num_params(self.h))

    def init_params(self, seed=0):
        _check(self.lib.turb_net_init_params(self.h, C.c_ulonglong(seed)), "turb_net_init_params")

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params:
            raise TurbError(1, "parameter vector of %d values, net has %d" % (p.size, self.num_params))
        _check(self.lib.turb_net_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), C.c_longlong(p.size)),
               "turb_net_set_params")

    def get_params(self):
        p = np.zeros(self.num_params, dtype=np.float32)
        _check(self.lib.turb_net_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), C.c_longlong(p.size)),
               "turb_net_get_params")
        return p

    def get_grads(self):
        g = np.zeros(self.num_params, dtype=np.float32)
        _check(self.lib.turb_net_get_grads(self.h, g.ctypes.data_as(C.POINTER(C.c_float)), C.c_longlong(g.size)),
               "turb_net_get_grads")
        return g

    ACTS = ("x0", "a0", "p0", "a1", "p1", "a2", "p2", "a3", "b3", "c2", "s2", "b2", "c1", "s1", "b1", "c0", "s0", "b0")
    ACT_SHAPE = dict(x0=(0, 16), a0=(0, 16), p0=(1, 16), a1=(1, 32), p1=(2, 32), a2=(2, 64), p2=(3, 64), a3=(3, 128),
                     b3=(3, 128), c2=(3, 64), s2=(2, 64), b2=(2, 64), c1=(2, 32), s1=(1, 32), b1=(1, 32), c0=(1, 16),
                     s0=(0, 16), b0=(0, 16))

    def activation(self, name):
        """Forward activation as float64 [C, Z, Y, X] (BF16 values)."""
        lev, c = self.ACT_SHAPE[name]
        nx, ny, nz = (d >> lev for d in self.dims)
        raw = np.zeros((c // 8, nz, ny, nx, 8), dtype=np.uint16)
        _check(self.lib.turb_net_get_activation(self.h, self.ACTS.index(name),
                                                raw.ctypes.data_as(C.POINTER(C.c_uint16)), C.c_longlong(raw.size)),
               "turb_net_get_activation")
        f = (raw.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        return np.ascontiguousarray(f.transpose(0, 4, 1, 2, 3).reshape(c, nz, ny, nx))

    def forward(self, in3, out):
        """in3: torch float32 CUDA tensor [3, nz, ny, nx]; out: [nz, ny, nx]."""
        _check(self.lib.turb_net_forward(self.h, _dev(in3), _dev(out), None), "turb_net_forward")

    def backward(self, gout):
        _check(self.lib.turb_net_backward(self.h, _dev(gout), None), "turb_net_backward")

    def adam(self, lr):
        _check(self.lib.turb_net_adam(self.h, C.c_float(lr), None), "turb_net_adam")

    def train_on(self, ctx, snaps, steps, lr=1e-3, seed=0):
        loss = C.c_double()
        _check(self.lib.turb_net_train(self.h, ctx.ctx, snaps.h, steps, C.c_float(lr), C.c_ulonglong(seed),
                                       C.byref(loss)), "turb_net_train")
        return loss.value

    def set_loss(self, w_residual=1.0, w_energy=0.0):
        """Training loss weights: relative squared initial residual and relative
        energy-norm (A-norm) error of the corrected guess."""
        _check(self.lib.turb_net_set_loss(self.h, C.c_double(w_residual), C.c_double(w_energy)), "turb_net_set_loss")

    def eval_on(self, ctx, snaps, first, count):
        """(mean relative squared residual, mean relative energy error) of the
        candidates over snapshots first .. first+count-1."""
        lr, le = C.c_double(), C.c_double()
        _check(self.lib.turb_net_eval(self.h, ctx.ctx, snaps.h, first, count, C.byref(lr), C.byref(le)),
               "turb_net_eval")
        return lr.value, le.value


class Snapshots:
    def __init__(self, nx, ny, nz, capacity):
        self.lib = load_library()
        h = _vp()
        _check(self.lib.turb_snaps_create(nx, ny, nz, capacity, C.byref(h)), "turb_snaps_create")
        self.h = h
        self.capacity = capacity

    def close(self):
        if self.h:
            self.lib.turb_snaps_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return int(self.lib.turb_snaps_count(self.h))

    def device_ptr(self, i):
        p = C.c_void_p()
        _check(self.lib.turb_snaps_data(self.h, i, C.byref(p)), "turb_snaps_data")
        return p.value


def set_snapshot_store(ctx, snaps):
    _check(ctx.lib.turb_set_snapshot_store(ctx.ctx, snaps.h if snaps is not None else None),
           "turb_set_snapshot_store")


def set_learned_net(ctx, net):
    _check(ctx.lib.turb_set_learned_net(ctx.ctx, net.h if net is not None else None), "turb_set_learned_net")


def selftest_umma(mn_major, swap=0):
    bad = C.c_ulonglong()
    _check(load_library().turb_selftest_umma(mn_major, swap, C.byref(bad)), "turb_selftest_umma")
    return bad.value


def conv3(X, Y, Z, cin, cout, x, W, bias=None, relu=False, dgrad=False, out=None):
    """One network convolution on torch CUDA tensors (channel-blocked BF16)."""
    _check(load_library().turb_conv3_test(X, Y, Z, cin, cout, _dev(x), _dev(W),
                                          _dev(bias) if bias is not None else None, 1 if relu else 0,
                                          1 if dgrad else 0, _dev(out), None), "turb_conv3_test")
    return out


def conv3_wgrad(X, Y, Z, cin, cout, x, dy, dw):
    _check(load_library().turb_conv3_wgrad_test(X, Y, Z, cin, cout, _dev(x), _dev(dy), _dev(dw), None),
           "turb_conv3_wgrad_test")
    return dw


def _main():
    """Time the network forward on random inputs (3 warm-up passes, then the
    timed ones, CUDA events):  python -m turbins_gb300.net NX NY NZ [REPS]"""
    import json
    import sys

    import torch

    nx, ny, nz = (int(v) for v in sys.argv[1:4])
    reps = int(sys.argv[4]) if len(sys.argv) > 4 else 5
    net = Net(nx, ny, nz, train=False)
    net.init_params(1)
    x = torch.randn(3, nz, ny, nx, device="cuda")
    out = torch.zeros(nz, ny, nx, device="cuda")
    for _ in range(3):
        net.forward(x, out)
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        net.forward(x, out)
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    flop = 2.0 * 25920 * nx * ny * nz
    print(json.dumps({"dims": [nx, ny, nz], "forward_ms": ts, "tflops": flop / (min(ts) / 1e3) / 1e12}))
    net.close()


if __name__ == "__main__":
    _main()
