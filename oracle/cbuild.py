"""Builds the oracle's C code (test infrastructure, see ``oracle/__init__``)
into oracle/_build/libnqport.so with gcc -O3 -fopenmp: cport.c (the C
restatement of the reference VMC iteration, compiled in FP64 and in FP32) and
lanczos.c (the matrix-free
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
    # cport.c twice: FP64 (port_*) and FP32 (port_*_f32, -DPORT_F32)
    units = [(SRCS[0], "cport64.o", []), (SRCS[0], "cport32.o", ["-DPORT_F32"]), (SRCS[1], "lanczos.o", [])]
    objs = []
    for src, obj, extra in units:
        out = os.path.join(OUT_DIR, obj)
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-std=c11", *extra, "-c", src, "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gcc failed for {src}:\n{r.stderr}")
        objs.append(out)
    cmd = ["gcc", "-shared", "-fopenmp", *objs, "-o", LIB + ".tmp", "-lm"]
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
        for sfx in ("", "_f32"):
            getattr(L, "port_sample" + sfx).restype = ctypes.c_long
            getattr(L, "port_sample" + sfx).argtypes = [i, i, i, i, vp, i, i, i, i, u64, u32, i, vp]
            getattr(L, "port_eval" + sfx).restype = None
            getattr(L, "port_eval" + sfx).argtypes = [i, i, i, vp, i, vp, vp, vp]
            getattr(L, "port_eloc" + sfx).restype = None
            getattr(L, "port_eloc" + sfx).argtypes = [i, i, i, i, vp, i, vp, vp, i] + [vp] * 8 + [vp]
        L.tfim2d_lanczos.restype = i
        L.tfim2d_lanczos.argtypes = [i, i, d, d, i, i, vp, vp]
        _lib = L
    return _lib
