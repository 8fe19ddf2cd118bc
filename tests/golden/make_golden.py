"""Generates the gather-scatter golden vectors in tests/golden/ from the
reference's own jl library (src/jl/gs.c, gs_local.c ...), compiled from the
reference sources by ``make -C oracle ref`` into oracle/_ref/libjl_ref.so.

Run in a container that has the reference checkout:
    make -C oracle ref REF=<reference root> && python tests/golden/make_golden.py

Each case stores the ids, the three jl local maps (unflagged, all, flagged
primaries, exactly as local_map / flagged_primaries_map write them) and, for
every (dom, op, transpose), an input vector and the output of jl's gs().
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def cases():
    rng = np.random.default_rng(20260)
    yield "gs_test", np.array([-11, -1, 1, 1, 1], dtype=np.int64)   # jl/gs_test.c:21-27 at np=1
    yield "gs_unique", np.array([1, 1], dtype=np.int64)             # jl/gs_unique_test.c:20
    yield "empty", np.zeros(0, dtype=np.int64)
    yield "all_zero", np.zeros(7, dtype=np.int64)
    yield "random_small", rng.integers(-6, 7, size=40).astype(np.int64)
    yield "random_flags", rng.integers(-30, 31, size=600).astype(np.int64)
    ids = rng.integers(1, 200, size=1500).astype(np.int64)
    ids[rng.random(1500) < 0.3] *= -1
    yield "random_mostly_flagged", ids
    ids = rng.integers(1, 50, size=400).astype(np.int64) * 1000003
    yield "large_ids", ids
    # a 2x2x1 box of lx1=3 elements numbered as set_vert_box does
    yield "box_2x2x1_lx3", box_ids(2, 2, 1, 3)
    yield "box_3x2x2_lx4", box_ids(3, 2, 2, 4)


def box_ids(nelx, nely, nelz, nx):
    nn = nx - 1
    out = []
    for ez in range(nelz):
        for ey in range(nely):
            for ex in range(nelx):
                for k in range(nx):
                    for j in range(nx):
                        for i in range(nx):
                            ig, jg, kg = nn * ex + i, nn * ey + j, nn * ez + k
                            out.append(1 + ig + jg * (nn * nelx + 1)
                                       + kg * (nn * nelx + 1) * (nn * nely + 1))
    return np.array(out, dtype=np.int64)


def main():
    jl = C.CDLL(str(ROOT / "oracle" / "_ref" / "libjl_ref.so"))
    jl.jlp_gs_setup.restype = C.c_void_p
    rng = np.random.default_rng(7)
    dtypes = {1: np.float64, 2: np.float32, 3: np.int32, 4: np.int64}
    for name, ids in cases():
        n = len(ids)
        h = jl.jlp_gs_setup(_ptr(ids), C.c_int(n))
        rec = {"ids": ids}
        for which in range(3):
            ln = jl.jlp_map_len(C.c_void_p(h), C.c_int(which))
            m = np.zeros(ln, dtype=np.uint32)
            jl.jlp_map_copy(C.c_void_p(h), C.c_int(which), _ptr(m))
            rec[f"map{which}"] = m
        for dom, dt in dtypes.items():
            for op in (1, 2, 3, 4):
                for tr in (0, 1):
                    if dom <= 2:
                        u = (rng.standard_normal(n) * 2).astype(dt)
                        if op == 2:
                            u = (1 + 0.1 * rng.standard_normal(n)).astype(dt)
                    else:
                        u = rng.integers(-4, 5, size=n).astype(dt)
                    v = u.copy()
                    if n:
                        jl.jlp_gs_op(C.c_void_p(h), _ptr(v), C.c_int(dom), C.c_int(op), C.c_int(tr))
                    rec[f"in_{dom}_{op}_{tr}"] = u
                    rec[f"out_{dom}_{op}_{tr}"] = v
        jl.jlp_gs_free(C.c_void_p(h))
        np.savez_compressed(OUT / f"gs_{name}.npz", **rec)
        print("wrote", name, n)


if __name__ == "__main__":
    main()
