"""Build recipe of the C restatement (bp_ref.c -> libbpref.so, gcc -O3
-fopenmp).  Test/bench infrastructure only; the product library never links
it.  The reference itself is Julia (no julia binary here), so there is no
oracle/_ref build of the reference's own sources."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "bp_ref.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libbpref.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", str(SRC), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        ip = C.POINTER(C.c_int32)
        dp = C.POINTER(C.c_double)
        lib.bpref_run.restype = C.c_int
        lib.bpref_run.argtypes = [C.c_int, C.c_int, ip, ip, ip, ip, ip, ip, dp, dp, C.c_int, ip, C.c_int, C.c_int,
                                  C.c_double, C.c_int, ip, dp]
        _lib = lib
    return _lib


def run(g, A_flat, msgs_flat, schedule, seq, maxiter, tol=None, nthreads=0):
    """Run the C restatement on an oracle Graph; returns (msgs, iters, mean_diff)."""
    lib = load()
    i32 = lambda x: np.ascontiguousarray(x if len(x) else [0], dtype=np.int32)
    eu = i32([u for u, _ in g.edges])
    ev = i32([v for _, v in g.edges])
    ed = i32(g.edge_dims)
    sd = i32(g.site_dims)
    lp = np.zeros(g.nv + 1, dtype=np.int32)
    for v in range(g.nv):
        lp[v + 1] = lp[v] + len(g.legs[v])
    le = i32([e for l in g.legs for e in l])
    fac = np.ascontiguousarray(A_flat, dtype=np.float64)
    msgs = np.ascontiguousarray(msgs_flat, dtype=np.float64).copy()
    sq = i32(seq if seq is not None else [0])
    it = np.zeros(1, dtype=np.int32)
    md = np.zeros(1)
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    rc = lib.bpref_run(g.nv, g.ne, P(eu, C.c_int32), P(ev, C.c_int32), P(ed, C.c_int32), P(sd, C.c_int32),
                       P(lp, C.c_int32), P(le, C.c_int32), P(fac, C.c_double), P(msgs, C.c_double),
                       0 if schedule == "sequential" else 1, P(sq, C.c_int32), len(seq) if seq is not None else 0,
                       int(maxiter), -1.0 if tol is None else float(tol), int(nthreads), P(it, C.c_int32),
                       P(md, C.c_double))
    if rc != 0:
        raise RuntimeError(f"bpref_run failed ({rc})")
    return msgs, int(it[0]), float(md[0])


if __name__ == "__main__":
    print(build(force=True))
