"""Golden vectors from the reference's own Fortran sources.

No Fortran compiler exists in this image, so the reference's solver sources
(src/*.f: driver.f, cg.f, math.f, mxm_std.f, speclib.f, semhat.f,
prox_setup.f, prox_dssum.f, hsmg.f) are run by the Fortran 77 subset executor
``oracle/f77.py``.  It gives gfortran -fdefault-real-8 semantics without FMA
contraction (the x86-64 build).  Gather-scatter calls go to the reference's
own jl library, compiled by ``make -C oracle ref`` into oracle/_ref/.
dsygv (hsmg's generalised eigensolver, vendored LAPACK in the reference) is
scipy's LAPACK dsygv with the same arguments.

The driver sequence is driver.f's own: init_mesh (brick), proxy_setupds,
set_multiplicity, proxy_setup, set_f, then cg twice (the warm-up and the timed
call; the second one sees the reference's element-1 mask list, cg.f:214-258).
Every glsc3 value the solver computes is recorded, in order.

Run where the reference checkout exists (--ref <root>, else
$NEKBONE_REFERENCE, else a checkout named "reference" beside this
repository):

    make -C oracle all ref
    python tests/golden/make_golden_fortran.py [--ref <root>] [--c1]

--c1 adds the C1 configuration (4^3 elements, lx1=10, 100 iterations per cg
call, a few minutes).  Outputs: tests/golden/fortran_*.npz.
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
import f77  # noqa: E402
from f77 import Ref  # noqa: E402

REF = None  # the reference's src/ directory, set by main() from --ref
JL = ROOT / "oracle" / "_ref" / "libjl_ref.so"


def reference_src(arg: str | None) -> Path:
    """src/ of the reference checkout: --ref, $NEKBONE_REFERENCE, or a
    checkout named "reference" beside this repository."""
    import os
    root = Path(arg or os.environ.get("NEKBONE_REFERENCE") or ROOT.parent / "reference")
    if not (root / "src" / "cg.f").exists():
        raise SystemExit(f"no reference checkout at {root} (pass --ref or set NEKBONE_REFERENCE)")
    return root / "src"


# ------------------------------------------------------ external routines --
class JlGs:
    """gs_setup / gs_op / gs_free of the reference's jl library."""

    def __init__(self):
        self.lib = C.CDLL(str(JL))
        self.n = {}

    def gs_setup(self, h, glo, n, comm, np_):
        nn = n.b[n.o]
        ids = np.array(glo.b[glo.o:glo.o + nn], dtype=np.int64)
        if len(ids) != nn:
            raise RuntimeError("gs_setup: id array too short")
        hh, ni, cm, npp = C.c_int(0), C.c_int(nn), C.c_int(0), C.c_int(1)
        self.lib.gs_setup_(C.byref(hh), ids.ctypes.data_as(C.c_void_p), C.byref(ni),
                           C.byref(cm), C.byref(npp))
        h.b[h.o] = hh.value
        self.n[hh.value] = nn

    def gs_op(self, h, u, dom, op, tr):
        hv = h.b[h.o]
        nn = self.n[hv]
        if dom.b[dom.o] != 1:
            raise RuntimeError("gs_op: only dom=1 (double) is used by the solver")
        a = np.array(u.b[u.o:u.o + nn], dtype=np.float64)
        if len(a) != nn:
            raise RuntimeError("gs_op: array too short")
        hh, d = C.c_int(hv), C.c_int(1)
        o, t = C.c_int(op.b[op.o]), C.c_int(tr.b[tr.o])
        self.lib.gs_op_(C.byref(hh), a.ctypes.data_as(C.c_void_p), C.byref(d), C.byref(o),
                        C.byref(t))
        u.b[u.o:u.o + nn] = a.tolist()

    def gs_free(self, h):
        hh = C.c_int(h.b[h.o])
        self.lib.gs_free_(C.byref(hh))


def dsygv(itype, jobz, uplo, n, a, lda, b, ldb, w, work, lwork, info):
    import scipy.linalg.lapack as LA
    nn, la, lb = n.b[n.o], lda.b[lda.o], ldb.b[ldb.o]
    A = np.array(a.b[a.o:a.o + la * nn]).reshape(nn, la).T[:nn, :nn].copy(order="F")
    B = np.array(b.b[b.o:b.o + lb * nn]).reshape(nn, lb).T[:nn, :nn].copy(order="F")
    res = LA.dsygv(A, B, itype=itype.b[itype.o], jobz=jobz.b[jobz.o].strip().upper(),
                   uplo=uplo.b[uplo.o].strip().upper())
    vals, vecs, inf = res[0], res[1], res[-1]
    for j in range(nn):
        for i in range(nn):
            a.b[a.o + i + la * j] = float(vecs[i, j])
    for i in range(nn):
        w.b[w.o + i] = float(vals[i])
    info.b[info.o] = int(inf)


def size_include(lx, lelt):
    """The case's SIZE file (test/example1/SIZE's parameters, sized here)."""
    return (f"      parameter (ldim=3)\n"
            f"      parameter (lx1={lx},ly1=lx1,lz1=lx1)\n"
            f"      parameter (lp = 1)\n"
            f"      parameter (lelt={lelt})\n"
            f"      parameter (lelg=lelt*lp)\n"
            f"      parameter (ldimt=1,ldimt1=ldimt+1)\n"
            f"      common /dimn/ nelx,nely,nelz,nelt\n"
            f"     $            , nx1,ny1,nz1,ndim,nfield,nid\n")


def runtime(lx, lelt, mgrid, gs):
    files = ["math.f", "speclib.f", "semhat.f", "mxm_wrapper.f", "mxm_std.f", "driver.f",
             "prox_setup.f", "prox_dssum.f", "cg.f", "hsmg.f" if mgrid else "hsmg_dum.f"]
    ext = {"gs_setup": gs.gs_setup, "gs_op": gs.gs_op, "gs_free": gs.gs_free,
           "gop": lambda *a: None,          # one process: the allreduce is the identity
           "adelay": lambda *a: None, "nekgsync": lambda *a: None,
           "dnekclock": lambda *a: 0.0, "dsygv": dsygv}
    rt = f77.F77([str(REF / f) for f in files], [str(REF)],
                 overrides={"SIZE": size_include(lx, lelt), "mpif.h": ""}, externals=ext)
    for blk in ("dimn", "cube1", "nekmpi", "mymask", "comm_handles", "precsl"):
        rt.ensure_common(blk)
    return rt


def driver_setup(rt, nx, ny, nz, lx):
    """driver.f:38-52 for one mesh: returns (n, c, g, f)."""
    nelt = nx * ny * nz
    dimn = rt.common("dimn")
    for k, v in enumerate([nx, ny, nz, nelt, lx, lx, lx, 3, 1, 0]):
        dimn[k][0] = v
    rt.common("cube1")[2][0] = 1        # np (iniproc)
    rt.common("nekmpi")[1][0] = 1       # mp
    rt.common("precsl")[0][0] = True    # ifdblas: REAL is 8 bytes (comm_mpi.f:54-55)
    cmask = rt.common("mymask")[0]
    rt.call("init_mesh", Ref([True]), Ref(cmask), 1, 1, 1, nx, ny, nz)
    rt.call("proxy_setupds", Ref(rt.common("comm_handles")[1]), lx)
    n = nelt * lx ** 3
    c = [0.0] * n
    rt.call("set_multiplicity", c)
    g = [0.0] * (6 * n)
    ah, bh, ch, dh = [0.0] * lx * lx, [0.0] * lx, [0.0] * lx * lx, [0.0] * lx * lx
    zh, wh = [0.0] * lx, [0.0] * 2 * lx
    rt.call("proxy_setup", ah, bh, ch, dh, zh, wh, g)
    rt.call("h1mg_setup")
    f = [0.0] * n
    rt.call("set_f", f, c, n)
    return n, c, g, f


def log_glsc3(rt):
    log = []
    inner = rt.routine("glsc3")

    def logged(*a):
        v = inner(*a)
        log.append(v)
        return v

    rt.compiled["glsc3"] = logged
    return log


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# ----------------------------------------------------------------- cases --
def speclib_case(gs):
    rt = runtime(16, 1, False, gs)
    zs, ws = [], []
    for npt in range(2, 17):
        z, w = [0.0] * npt, [0.0] * npt
        rt.call("zwgll", z, w, npt)
        zs.extend(z)
        ws.extend(w)
    sem = {k: [] for k in "abcdz"}
    for n in range(1, 16):
        np1 = n + 1
        a, b, c, d, z = ([0.0] * np1 * np1, [0.0] * np1, [0.0] * np1 * np1,
                         [0.0] * np1 * np1, [0.0] * np1)
        rt.call("semhat", a, b, c, d, z, [0.0] * (2 * n + 2), n)   # as proxy_setup sizes it
        for k, v in zip("abcdz", (a, b, c, d, z)):
            sem[k].extend(v)
    cub = []
    for npr in range(1, 401):
        mx, my, mz = [0], [0], [0]
        rt.call("cubic", mx, my, mz, npr)
        cub.append((mx[0], my[0], mz[0]))
    np.savez_compressed(HERE / "fortran_speclib.npz", zwgll_z=np.array(zs),
                        zwgll_w=np.array(ws), semhat_a=np.array(sem["a"]),
                        semhat_b=np.array(sem["b"]), semhat_c=np.array(sem["c"]),
                        semhat_d=np.array(sem["d"]), semhat_z=np.array(sem["z"]),
                        cubic=np.array(cub, dtype=np.int32))


def box_case(gs, nx, ny, nz, lx, niter, full=True, tag=None):
    rt = runtime(lx, nx * ny * nz, False, gs)
    n, c, g, f = driver_setup(rt, nx, ny, nz, lx)
    glo = [0] * n
    rt.call("set_vert_box", glo, lx)
    out = {"dims": np.array([nx, ny, nz, lx, niter])}
    # ax on a seeded field, before the mask list exists (the call that builds
    # it) and after (the element-1 list semantics)
    rng = np.random.default_rng(1000 * lx + nx)
    u = rng.uniform(-1, 1, n).tolist()
    lt = n
    w1 = [0.0] * n
    wk = [[0.0] * lt for _ in range(4)]
    if full:
        rt2 = runtime(lx, nx * ny * nz, False, gs)
        driver_setup(rt2, nx, ny, nz, lx)
        rt2.call("ax", w1, list(u), g, *wk, n)
        w2 = [0.0] * n
        rt2.call("ax", w2, list(u), g, *wk, n)
        out.update(ax_u=np.array(u), ax_w_first=np.array(w1), ax_w_second=np.array(w2))
    log = log_glsc3(rt)
    x, r, w, p, z = ([0.0] * n for _ in range(5))
    flop = [0.0]
    t0 = time.time()
    rt.call("cg", x, f, g, c, r, w, p, z, n, niter, flop)
    x1, r1, nlog1 = np.array(x), np.array(r), len(log)
    rt.call("cg", x, f, g, c, r, w, p, z, n, niter, flop)
    x2, r2 = np.array(x), np.array(r)
    dt = time.time() - t0
    # the mask list of /mymask/: pmask(-1) < 0 once built, pmask(0) = count,
    # pmask(1..count) = indices (cg.f:222-253)
    cm = rt.common("mymask")[0]
    mask = np.array(cm[2:2 + int(cm[1])]) if cm[0] < 0 else np.zeros(0)
    out.update(log_warmup=np.array(log[:nlog1]), log_timed=np.array(log[nlog1:]),
               mask_list=mask, flop_cg=np.array(flop[0]))
    arrays = dict(glo=np.array(glo, dtype=np.int64), c=np.array(c), g=np.array(g),
                  f=np.array(f), x_warmup=x1, r_warmup=r1, x_timed=x2, r_timed=r2)
    if full:
        out.update(arrays)
    else:
        for k, v in arrays.items():
            out["sha_" + k] = np.array(sha(v))
        out["x_timed_sample"] = x2[::37]
        out["r_timed_sample"] = r2[::37]
        out["x_warmup_sample"] = x1[::37]
    name = tag or f"box_{nx}x{ny}x{nz}_lx{lx}"
    np.savez_compressed(HERE / f"fortran_{name}.npz", **out)
    print(f"{name}: n={n}, 2 x {niter} CG iterations in {dt:.1f} s")


def hsmg_case(gs, nx, ny, nz, lx, niter):
    rt = runtime(lx, nx * ny * nz, True, gs)
    n, c, g, f = driver_setup(rt, nx, ny, nz, lx)
    rhs = list(f)
    zz = [0.0] * n
    rt.call("h1mg_solve", zz, rhs, n)
    # preconditioned cg (solveM = h1mg_solve), the warm-up call of driver.f
    rt2 = runtime(lx, nx * ny * nz, True, gs)
    n, c, g, f2 = driver_setup(rt2, nx, ny, nz, lx)
    log = log_glsc3(rt2)
    x, r, w, p, z = ([0.0] * n for _ in range(5))
    rt2.call("cg", x, f2, g, c, r, w, p, z, n, niter, [0.0])
    lev = rt.common("mghs")
    np.savez_compressed(HERE / f"fortran_hsmg_{nx}x{ny}x{nz}_lx{lx}.npz",
                        dims=np.array([nx, ny, nz, lx, niter]), f=np.array(f),
                        rhs_after=np.array(rhs), z=np.array(zz), pcg_x=np.array(x),
                        pcg_log=np.array(log),
                        mg_lmax=np.array(rt.common("mgh1i")[0][0]),
                        mg_nx=np.array(lev[1], dtype=np.int32))
    print(f"hsmg {nx}x{ny}x{nz} lx{lx}: done")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--c1", action="store_true", help="also the 4^3, lx1=10 C1 case")
    ap.add_argument("--only", choices=["speclib", "box", "hsmg", "c1"], default=None)
    ap.add_argument("--ref", default=None, help="root of the reference checkout")
    a = ap.parse_args()
    global REF
    REF = reference_src(a.ref)
    if not JL.exists():
        sys.exit("build the jl library first: make -C oracle ref")
    gs = JlGs()
    want = lambda k: a.only in (None, k)
    if want("speclib"):
        speclib_case(gs)
    if want("box"):
        box_case(gs, 2, 2, 2, 6, 20)
        box_case(gs, 3, 2, 1, 5, 15)
    if want("hsmg"):
        hsmg_case(gs, 2, 2, 2, 6, 10)
    if (a.c1 and a.only is None) or a.only == "c1":
        box_case(gs, 4, 4, 4, 10, 100, full=False, tag="c1_4x4x4_lx10")


if __name__ == "__main__":
    main()
