"""Build and bind oracle/cpu_ref.c (OpenMP C restatement) -- TEST INFRASTRUCTURE.

Used by tests as a second checker and by bench.py as the timed CPU baseline
("port"); the product never imports it.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_ref.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmandoct_cpu_ref.so")
_lib = None


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = shutil.which("gcc") or "cc"
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", LIB + ".tmp", SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("cpu_ref build failed:\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.cpu_threads.restype = ctypes.c_int
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def threads():
    return int(load().cpu_threads())


def weight(geom, sgm):
    load().cpu_weight(ctypes.byref(geom), _p(sgm))


def filter_rows(geom, x, taps, y, r0, r1):
    load().cpu_filter(ctypes.byref(geom), _p(x), _p(taps), _p(y), ctypes.c_int64(r0), ctypes.c_int64(r1))


def fdk_bp(geom, angles, F, vol, alive, v0, v1):
    load().cpu_fdk_bp(ctypes.byref(geom), _p(angles), _p(F), _p(vol), _p(alive), ctypes.c_int(v0), ctypes.c_int(v1))


def fp(geom, angles, u, v, vol, out, v0, v1):
    load().cpu_fp(ctypes.byref(geom), _p(angles), _p(u), _p(v), _p(vol), _p(out), ctypes.c_int(v0), ctypes.c_int(v1))
