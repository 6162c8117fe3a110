"""Builds the oracle's C code (test infrastructure, see ``oracle/__init__``)
into oracle/_build/libnqport.so with gcc -O3 -fopenmp: cport.c (the C
restatement of the reference VMC iteration) and lanczos.c (the matrix-free
Lanczos recurrence that pins the 2D Ising convention).  No reference sources
are compiled: the reference is Julia and has no C/C++ path."""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "cport.c"), os.path.join(HERE, "lanczos.c")]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnqport.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in SRCS):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", *SRCS, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        d, i, u64, u32, vp = ctypes.c_double, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p
        L.port_sample.restype = ctypes.c_long
        L.port_sample.argtypes = [i, i, i, i, vp, i, i, i, i, u64, u32, i, vp]
        L.port_eval.restype = None
        L.port_eval.argtypes = [i, i, i, vp, i, vp, vp, vp]
        L.port_eloc.restype = None
        L.port_eloc.argtypes = [i, i, i, i, vp, i, vp, vp, i] + [vp] * 8 + [vp]
        L.tfim2d_lanczos.restype = i
        L.tfim2d_lanczos.argtypes = [i, i, d, d, i, i, vp, vp]
        _lib = L
    return _lib
