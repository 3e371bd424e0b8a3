"""Build and load ``oracle/liboracle.so`` (gcc, OpenMP, FP64).

Test infrastructure: the C restatement of the reference path, used as the
timed CPU baseline and as a second oracle.  Portable flags only (the same
source builds on the x86 container and the Arm GPU host).
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "fem_oracle.c"
LIB = HERE / "liboracle.so"


def build(force: bool = False) -> pathlib.Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


class Params(ctypes.Structure):
    _fields_ = [("max_steps", ctypes.c_int), ("rtol", ctypes.c_double), ("atol", ctypes.c_double),
                ("max_bt", ctypes.c_int), ("c", ctypes.c_double), ("overstep", ctypes.c_double),
                ("beta_max", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("result", ctypes.c_int), ("n_steps", ctypes.c_int), ("grad_norm", ctypes.c_double),
                ("grad_norm_first", ctypes.c_double), ("energy", ctypes.c_double)]


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(LIB))
        vp = ctypes.c_void_p
        lib.orc_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [vp] * 5 + [vp, vp, ctypes.c_uint] + [vp] * 5
        lib.orc_eval.restype = ctypes.c_int
        lib.orc_pncg.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [vp] * 5 + [vp, vp, vp,
                                                                                     ctypes.POINTER(Params),
                                                                                     ctypes.POINTER(Stats)]
        lib.orc_pncg.restype = ctypes.c_int
        lib.orc_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class CModel:
    """One FEM potential + fixed DOFs + per-vertex force, FP64 arrays."""

    def __init__(self, material: int, cells, dhdX, dV, mu, lam, n_points, mask=None, force=None):
        self.material = int(material)
        self.cells = np.ascontiguousarray(cells, np.int32)
        self.dhdX = np.ascontiguousarray(dhdX, np.float64)
        self.dV = np.ascontiguousarray(dV, np.float64)
        n = self.cells.shape[0]
        self.mu = np.ascontiguousarray(np.broadcast_to(mu, (n,)), np.float64)
        self.lam = np.ascontiguousarray(np.broadcast_to(lam if lam is not None else 0.0, (n,)), np.float64)
        self.n_points = int(n_points)
        self.mask = np.ascontiguousarray(np.zeros((n_points, 3), np.uint8) if mask is None else mask, np.uint8)
        self.force = None if force is None else np.ascontiguousarray(force, np.float64)

    def eval(self, u, p=None, flags=31):
        lib = load()
        u = np.ascontiguousarray(u, np.float64)
        p = None if p is None else np.ascontiguousarray(p, np.float64)
        e = np.zeros(1)
        q = np.zeros(1)
        g = np.zeros((self.n_points, 3))
        d = np.zeros((self.n_points, 3))
        hp = np.zeros((self.n_points, 3))
        if p is None:
            flags &= 7
        lib.orc_eval(self.material, self.n_points, self.cells.shape[0], _p(self.cells), _p(self.dhdX), _p(self.dV),
                     _p(self.mu), _p(self.lam), _p(u), _p(p), flags, _p(e), _p(g), _p(d), _p(hp), _p(q))
        return {"fun": e[0], "grad": g, "hess_diag": d, "hess_prod": hp, "hess_quad": q[0]}

    def pncg(self, u, *, max_steps=1500, rtol=1e-9, atol=0.0, max_bt=8, c=1e-4, overstep=1.0, beta_max=10.0):
        lib = load()
        u = np.array(u, np.float64, order="C")
        prm = Params(max_steps, rtol, atol, max_bt, c, overstep, beta_max)
        st = Stats()
        lib.orc_pncg(self.material, self.n_points, self.cells.shape[0], _p(self.cells), _p(self.dhdX), _p(self.dV),
                     _p(self.mu), _p(self.lam), _p(self.mask), _p(self.force), _p(u), ctypes.byref(prm),
                     ctypes.byref(st))
        return u, st


def threads() -> int:
    return int(load().orc_threads())
