"""The reference's own driver program, recorded at the library's boundary.

driver.f's `program nekbone` (driver.f:2-86) runs unmodified in the Fortran
77 subset executor ``oracle/f77.py`` over the reference's solver sources and
jl library (the set-up of make_golden_fortran.py).  Every call the program
makes into a routine the library replaces -- gs_setup, gs_op, gs_free,
dssum, h1mg_setup, cg -- is recorded in order with its arguments as passed
and as returned by the reference's implementation.  Calls those routines make
themselves (cg's dssum and gs_op, ...) are inside the library and are not
recorded.  The hand-off lines the link step adds to driver.f are recorded
where they go: `nekbone_mask_reset` after each init_mesh (init_mesh sets
cmask(-1) = 1, driver.f:125), and `nekbone_common` / `nekbone_set_mask_mode`
/ `nekbone_set_mgrid` after each proxy_setup, with the values of /dimn/,
/hcglb/ lglel, /dxyz/ dxm1 and /comm_handles/ gsh at that point.

What the executor cannot run is supplied from outside:
  * read_param (driver.f:402-484) reads data.rea; the executor has no
    I/O, so the five records are given here (ifmgrid as the MGRID build sets
    it);
  * iniproc (comm_mpi.f) sets one process (nid 0, np 1) and its word sizes;
  * dnekclock counts up by one per call (set_timer_flop_cnt divides by it),
    nekgsync, init_delay and gop are no-ops, and exitt0 ends the run.

The trace runs on the GPU through the library's gfortran-convention entry
points in tests/test_gpu_driver_trace.py.  Outputs: tests/golden/
driver_trace_<case>.npz.

    make -C oracle all ref
    python tests/golden/make_golden_driver.py [--ref <root>]
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import make_golden_fortran as MGF  # noqa: E402
from make_golden_fortran import f77, Ref  # noqa: E402


class _Exit(Exception):
    """exitt0: the program's end."""


# the data.rea records of each recorded case: ifbrick, (iel0, ielN, ielD),
# (nx0, nxN, nxD), (npx, npy, npz), (mx, my, mz), and the MGRID build
CASES = {
    # two polynomial orders (nx1 = 4 runs below SIZE's lx1 = 6) and two
    # element counts: four meshes, each set up, solved twice and freed (one
    # element is left out: its mask leaves r = 0 and cg divides 0 by 0,
    # which the executor raises where the compiled program makes NaNs)
    "plain": dict(ifbrick=True, iel=(2, 9, 7), nx=(4, 6, 2), mgrid=False),
    # the MGRID build: hsmg set-up per mesh, h1mg_solve as cg's solveM
    "mgrid": dict(ifbrick=True, iel=(2, 2, 1), nx=(6, 6, 1), mgrid=True),
}


class Recorder:
    """Wraps routines of the executor so that top-level calls are recorded."""

    def __init__(self, rt):
        self.rt = rt
        self.calls = []        # (name, [(kind, in, out)])
        self.depth = 0

    def cur_n(self):
        d = self.rt.common("dimn")
        nx1, nelt = int(d[4][0]), int(d[3][0])
        return nx1 ** 3 * nelt

    @staticmethod
    def grab(ref, kind, length):
        vals = ref.b[ref.o:ref.o + length]
        if len(vals) != length:
            raise RuntimeError("argument shorter than its declared length")
        dt = {"f8": np.float64, "i4": np.int32, "i8": np.int64}[kind]
        return np.array(vals, dtype=dt)

    def wrap(self, name, inner, layout):
        """layout(args) -> [(kind, length)] per argument."""

        def wrapped(*args):
            if self.depth > 0:
                return inner(*args)
            lay = layout(args)
            ins = [self.grab(a, k, m) for a, (k, m) in zip(args, lay)]
            self.depth += 1
            try:
                v = inner(*args)
            finally:
                self.depth -= 1
            outs = [self.grab(a, k, m) for a, (k, m) in zip(args, lay)]
            self.calls.append((name, [(k, i, o) for (k, _), i, o in zip(lay, ins, outs)]))
            return v

        return wrapped

    def note(self, name, args):
        """A hand-off call with given argument values (kind, array)."""
        self.calls.append((name, [(k, a, a) for k, a in args]))


def run_case(gs, tag, spec):
    lx = spec["nx"][1]
    lelt = spec["iel"][1]
    rt = MGF.runtime(lx, lelt, spec["mgrid"], gs)
    for blk in ("dimn", "cube1", "nekmpi", "mymask", "comm_handles", "precsl", "lmgrid",
                "hcglb", "dxyz"):
        rt.ensure_common(blk)
    rec = Recorder(rt)
    ticks = [0.0]

    def dnekclock(*a):
        ticks[0] += 1.0
        return ticks[0]

    def iniproc(comm):
        rt.common("dimn")[9][0] = 0        # nid (SIZE's /dimn/)
        rt.common("cube1")[2][0] = 1       # np (PARALLEL's /cube1/)
        rt.common("nekmpi")[0][0] = 0      # nid_
        rt.common("nekmpi")[1][0] = 1      # np_
        rt.common("precsl")[0][0] = True   # ifdblas: REAL is 8 bytes

    def exitt0(*a):
        raise _Exit()

    def read_param(ifbrick, iel0, ieln, ield, nx0, nxn, nxd, npx, npy, npz, mx, my, mz):
        ifbrick.b[ifbrick.o] = spec["ifbrick"]
        for r, v in zip((iel0, ieln, ield), spec["iel"]):
            r.b[r.o] = v
        for r, v in zip((nx0, nxn, nxd), spec["nx"]):
            r.b[r.o] = v
        for r in (npx, npy, npz, mx, my, mz):
            r.b[r.o] = 0
        rt.common("lmgrid")[0][0] = spec["mgrid"]

    for k, v in (("dnekclock", dnekclock), ("iniproc", iniproc), ("exitt0", exitt0),
                 ("init_delay", lambda *a: None), ("nekgsync", lambda *a: None),
                 ("gop", lambda *a: None)):
        rt.externals[k] = v
    rt.compiled["read_param"] = read_param

    # boundary routines
    gsn = {}

    def gs_setup_layout(a):
        return [("i4", 1), ("i8", int(a[2].b[a[2].o])), ("i4", 1), ("i4", 1), ("i4", 1)]

    def gs_setup(h, glo, n, comm, np_):
        gs.gs_setup(h, glo, n, comm, np_)
        gsn[int(h.b[h.o])] = int(n.b[n.o])

    rt.externals["gs_setup"] = rec.wrap("gs_setup", gs_setup, gs_setup_layout)
    rt.externals["gs_op"] = rec.wrap(
        "gs_op", gs.gs_op,
        lambda a: [("i4", 1), ("f8", gsn[int(a[0].b[a[0].o])]), ("i4", 1), ("i4", 1), ("i4", 1)])
    rt.externals["gs_free"] = rec.wrap("gs_free", gs.gs_free, lambda a: [("i4", 1)])
    rt.compiled["dssum"] = rec.wrap("dssum", rt.routine("dssum"),
                                    lambda a: [("f8", rec.cur_n())])
    rt.compiled["h1mg_setup"] = rec.wrap("h1mg_setup", rt.routine("h1mg_setup"), lambda a: [])

    def cg_layout(a):
        n = int(a[8].b[a[8].o])
        return [("f8", n), ("f8", n), ("f8", 6 * n), ("f8", n), ("f8", n), ("f8", n),
                ("f8", n), ("f8", n), ("i4", 1), ("i4", 1), ("f8", 1)]

    rt.compiled["cg"] = rec.wrap("cg", rt.routine("cg"), cg_layout)

    # the link step's hand-off lines
    init_mesh = rt.routine("init_mesh")

    def init_mesh_then_reset(*a):
        init_mesh(*a)
        rec.note("nekbone_mask_reset", [])

    rt.compiled["init_mesh"] = init_mesh_then_reset
    proxy_setup = rt.routine("proxy_setup")

    def proxy_setup_then_publish(*a):
        proxy_setup(*a)
        d = rt.common("dimn")
        nelx, nely, nelz, nelt, nx1 = (int(d[k][0]) for k in range(5))
        lglel = np.array(rt.common("hcglb")[2][:nelt], dtype=np.int32)   # after nvtot, nelgf
        dxm1 = np.array(rt.common("dxyz")[0][:nx1 * nx1], dtype=np.float64)
        gsh = int(rt.common("comm_handles")[1][0])
        i4 = lambda v: ("i4", np.array([v], dtype=np.int32))
        rec.note("nekbone_common", [i4(nelx), i4(nely), i4(nelz), i4(nelt), i4(nx1),
                                    ("i4", lglel), ("f8", dxm1), i4(gsh)])
        rec.note("nekbone_set_mask_mode", [i4(0)])
        rec.note("nekbone_set_mgrid", [i4(1 if spec["mgrid"] else 0)])

    rt.compiled["proxy_setup"] = proxy_setup_then_publish

    t0 = time.time()
    try:
        rt.call("nekbone")
    except _Exit:
        pass
    dt = time.time() - t0
    out = {}
    meta = []
    for k, (name, args) in enumerate(rec.calls):
        meta.append({"name": name, "kinds": [a[0] for a in args]})
        for j, (kind, ain, aout) in enumerate(args):
            out[f"c{k}_a{j}_in"] = ain
            out[f"c{k}_a{j}_out"] = aout
    out["calls"] = np.array(json.dumps(meta))
    out["spec"] = np.array(json.dumps(spec))
    np.savez_compressed(HERE / f"driver_trace_{tag}.npz", **out)
    names = [m["name"] for m in meta]
    print(f"{tag}: {len(names)} boundary calls in {dt:.1f} s: "
          + ", ".join(f"{n} x{names.count(n)}" for n in dict.fromkeys(names)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="root of the reference checkout")
    ap.add_argument("--only", choices=sorted(CASES), default=None)
    a = ap.parse_args()
    MGF.REF = MGF.reference_src(a.ref)
    if not MGF.JL.exists():
        sys.exit("build the jl library first: make -C oracle ref")
    gs = MGF.JlGs()
    for tag, spec in CASES.items():
        if a.only in (None, tag):
            run_case(gs, tag, spec)


if __name__ == "__main__":
    main()
