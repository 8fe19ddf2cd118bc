"""Benchmark of the Nekbone CG hot path on one GB300.

Workload (the headline metric's configuration): a 32x32x32 box of undeformed
hexahedral elements, lx1=12 GLL points per direction (n = 56,623,104 local
points), full Dirichlet mask, seeded uniform RHS; one step = one call of the
reference's cg (cg.f:2-84): 100 plain FP64 CG iterations with the identity
preconditioner.  Metric: GDOF*iter/s = n * 100 / seconds / 1e9 (the
reference's DOF convention, n = nelt*lx1^3).

  value  -- device-resident solve (inputs already in HBM), CUDA events on
            the library's stream, K steps after W warm-up steps.  Every
            vector (453 MB) is larger than L2 (129 MB).
  e2e    -- the same solve through the drop-in C ABI call cg_ with pinned
            HOST buffers: f, g, c copied in and x, r, w, p, z copied out inside
            the timed region, every step.
  roofline -- the dominant kernel (the fused element operator k_ax), from its
            own CUDA-event time over a timed CG iteration loop.
  mixed  -- time to relative residual 1e-10 of plain FP64 CG and of the
            mixed-precision solver (FP32 inner CG in FP64 defect correction),
            each solution's true residual recomputed on the host by the
            oracle's own ax (cpu_relres).
  cpu_baseline -- the oracle (CPU restatement, OpenMP over elements) on the
            host cores, on a bounded sample of the same workload (the same
            32^3 mesh, fewer iterations).

--impl reference runs the reference's CPU algorithm (the oracle port; the
Fortran reference has no compiler in this image) on the same configuration:
the same 32^3 mesh and right-hand side, a bounded number of CG iterations
per step (the metric is a per-iteration rate).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GDOF·iter/s (lx1=12, 32^3 elems); mixed vs FP64 GPU time to rel. resid 1e-10"
UNIT = "GDOF*iter/s"
# DRAM read + write bytes per point of each FP64 element operator at lx1 = 12
# from one ncu capture on 16^3 elements (7,077,888 points); the kernels
# stream, so traffic scales with n.  Source: the profiles/ summaries named.
DRAM_BYTES_PER_POINT = {
    1: ((531.699456e6 + 120.930048e6) / 7077888, "profiles/k_ax_eo_fp64_lx12_16cubed.md"),
    2: ((511.710208e6 + 98.418944e6) / 7077888, "profiles/k_ax_fx_fp64_lx12_16cubed.md"),
}
RHS_SEED = 20260


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nel", type=int, default=32, help="elements per direction")
    ap.add_argument("--lx", type=int, default=12)
    ap.add_argument("--niter", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--order", type=int, default=2, choices=[0, 1, 2],
                    help="FP64 operator form: 0 the reference's summation order, 1 even-odd "
                         "on the FP64 pipe, 2 even-odd in 64-bit fixed point on the integer "
                         "pipes")
    ap.add_argument("--cpu-sample-iters", type=int, default=8,
                    help="CG iterations per CPU sample of the 32^3 workload")
    ap.add_argument("--case", choices=["cg", "tc", "batch", "hsmg", "mixed"], default="cg",
                    help="cg: the benchmark; tc / batch / hsmg / mixed: a small case of the "
                         "tensor-core operator / the batched solver / hsmg PCG / the mixed "
                         "solver, for profiling")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"nekbone_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])),
                "sm_max_mhz": float(max(r[1] for r in rows)),
                "power_w_max": float(max(r[2] for r in rows)),
                "samples": len(rows), "reasons": reasons}


# ------------------------------------------------------------- CPU oracle --
def uniform_pm1(seed: int, ids: np.ndarray) -> np.ndarray:
    """The library's counter-based uniform [-1, 1) of (seed, global id)
    (splitmix64 finaliser), restated in numpy for the CPU side."""
    z = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + ids.astype(np.uint64)
         + np.uint64(0x632BE59BD9B4E019))
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def global_ids(nel: int, lx: int) -> np.ndarray:
    """set_vert_box's global numbering (prox_dssum.f:42-73) of a nel^3 brick,
    in the local point order (element ex fastest, then i, j, k)."""
    nn = lx - 1
    ax = nn * nel + 1
    e = np.arange(nel, dtype=np.int64)
    q = np.arange(lx, dtype=np.int64)
    ez, ey, ex, k, j, i = np.ix_(e, e, e, q, q, q)
    return (1 + (nn * ex + i) + (nn * ey + j) * ax + (nn * ez + k) * ax * ax).reshape(-1)


class CpuCase:
    """The oracle on the headline mesh with the headline inputs: setup_g's
    metric, the inverse multiplicity and nb_rhs_uniform's right-hand side
    (uniform per global point, dssum, times c, masked)."""

    def __init__(self, nel: int, lx: int, threads: int, seed: int = RHS_SEED):
        sys.path.insert(0, str(ROOT / "tests"))
        import oracle_lib as O
        t0 = time.perf_counter()
        self.ctx = O.Ctx(nel, nel, nel, lx, mask_mode=1, nthreads=threads, fma=False)
        self.g = self.ctx.setup_g()
        self.c = self.ctx.set_multiplicity()
        f = uniform_pm1(seed, global_ids(nel, lx))
        self.ctx.dssum(f)
        f *= self.c
        self.ctx.maskit(f)
        self.f = f
        self.n = self.ctx.n
        self.threads = threads
        self.setup_s = time.perf_counter() - t0
        self.work = tuple(np.zeros(self.n) for _ in range(5))

    def cg(self, iters: int):
        t0 = time.perf_counter()
        o = self.ctx.cg(self.f, self.g, self.c, iters, work=self.work)
        return o, time.perf_counter() - t0

    def rate(self, iters: int):
        _, dt = self.cg(iters)
        return self.n * iters / dt / 1e9, dt

    def relres(self, x: np.ndarray) -> float:
        """sqrt(r'Cr) / sqrt(f'Cf), r = mask(f - A x), A the oracle's ax."""
        r = self.f - self.ctx.ax(x, self.g)
        self.ctx.maskit(r)
        return float(np.sqrt(np.dot(r * self.c, r)) / np.sqrt(np.dot(self.f * self.c, self.f)))


def replica_rate(ms, n, niter, steps, world, device=None):
    """Whole-job rate of `world` independent replicas (one mesh of n points
    per rank, niter iterations per step): every rank's work over the slowest
    rank's time.  Returns (max ms over ranks, GDOF*iter/s)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * n * niter * steps / (ms / 1e3) / 1e9


def workload_config(nel: int, lx: int, niter: int) -> dict:
    """The workload, identical in both arms' lines."""
    n = nel ** 3 * lx ** 3
    return {"workload": f"cg, {nel}^3 elements, lx1={lx}, {niter} FP64 iterations per step",
            "n": n, "mask": "full Dirichlet", "rhs": "seeded uniform[-1,1] per global DOF",
            "l2": f"inputs larger than L2 ({8 * n / 1e6:.0f} MB per vector)"}


def run_reference(a, rank, world):
    """The reference's CPU algorithm (the oracle port, OpenMP over elements,
    every host thread) on the headline mesh and right-hand side; each step
    is a bounded sample of --cpu-sample-iters CG iterations of that solve."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    t_all = time.perf_counter()
    case = CpuCase(a.nel, a.lx, threads)
    for _ in range(a.warmup):
        case.rate(1)
    rates, times = [], []
    t_steps = time.perf_counter()
    for _ in range(a.steps):
        r, dt = case.rate(a.cpu_sample_iters)
        rates.append(r)
        times.append(dt)
    steps_s = time.perf_counter() - t_steps
    v = float(np.median(rates))
    sample = (f"{a.nel}^3 elements, lx1={a.lx} (n={case.n}), the headline solve's first "
              f"{a.cpu_sample_iters} CG iterations per step")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": float(np.median(times)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(a.nel, a.lx, a.niter),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": case.setup_s, "steps_s": steps_s,
            "wall_s": time.perf_counter() - t_all}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- extras --
def _time_on(stream, torch, fn, reps=10):
    """Average milliseconds of fn() over reps calls, CUDA events on stream."""
    fn()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def extras(nb, torch, dev, order=2):
    """Deformed-geometry operator error per lx1 (16^3 elements) for the
    CUDA-core FP32 and the tensor-core (FP16 hi+lo split) operators and the
    FP64 operator in fixed point, each against the FP64 operator in the
    reference's summation order, with each operator's time; and
    hsmg-preconditioned CG against plain CG (16^3 deformed, lx1=12, levels
    12 -> 6 -> 3), to relative residual 1e-10, with the FP64 operator form
    `order`."""
    res = {"deformed_operator_error": {}, "hsmg_pcg": {}}
    stream = torch.cuda.ExternalStream(nb.stream_handle(), device=dev)
    for lx in (8, 12, 16):
        m = nb.DeviceMesh(16, 16, 16, lx, mask_mode=1)
        n = m.n
        g = torch.empty(6 * n, dtype=torch.float64, device=dev)
        m.setup_g_deformed(g.data_ptr(), 11, 0.1)
        u = torch.rand(n, dtype=torch.float64, device=dev) * 2 - 1
        m.dssum(u.data_ptr(), 1)        # continuous field
        w64 = torch.empty_like(u)
        m.set_order(0)
        m.ax(w64.data_ptr(), u.data_ptr(), g.data_ptr())
        wfx = torch.empty_like(u)
        m.set_order(2)
        m.ax(wfx.data_ptr(), u.data_ptr(), g.data_ptr())
        t_fx = _time_on(stream, torch, lambda: m.ax(wfx.data_ptr(), u.data_ptr(), g.data_ptr()))
        m.set_order(1)
        w32 = torch.empty(n, dtype=torch.float32, device=dev)
        u32, g32 = u.float(), g.float()
        m.ax_f32(w32.data_ptr(), u32.data_ptr(), g32.data_ptr())
        wtc = torch.empty(n, dtype=torch.float32, device=dev)
        m.ax_tc(wtc.data_ptr(), u32.data_ptr(), g32.data_ptr())
        torch.cuda.synchronize()
        sc = w64.abs().max().item()
        d = (w32.double() - w64).abs().max().item() / sc
        dtc = (wtc.double() - w64).abs().max().item() / sc
        dfx = (wfx - w64).abs().max().item() / sc
        ms = {
            "fp64": _time_on(stream, torch, lambda: m.ax(w64.data_ptr(), u.data_ptr(), g.data_ptr())),
            "fp64_fixed_point": t_fx,
            "fp32": _time_on(stream, torch,
                             lambda: m.ax_f32(w32.data_ptr(), u32.data_ptr(), g32.data_ptr())),
            "tc": _time_on(stream, torch,
                           lambda: m.ax_tc(wtc.data_ptr(), u32.data_ptr(), g32.data_ptr())),
        }
        res["deformed_operator_error"][f"lx1={lx}"] = {"fp32": d, "tc": dtc,
                                                       "fp64_fixed_point": dfx, "n": n,
                                                       "apply_ms": ms}
        del g, u, w64, wfx, w32, u32, g32, wtc
        m.close()
        torch.cuda.empty_cache()
    m = nb.DeviceMesh(16, 16, 16, 12, mask_mode=1)
    m.set_order(order)
    n = m.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    m.setup_g_deformed(g.data_ptr(), 11, 0.1)
    m.set_multiplicity(c.data_ptr())
    m.rhs_uniform(f.data_ptr(), c.data_ptr(), 5)
    x = torch.zeros_like(f)
    m.cg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
             max_iter=20000, check_every=10)          # warm-up (scratch, kernel loading)
    x.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it, rr = m.cg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                      max_iter=20000, check_every=10)
    tcg = time.perf_counter() - t0
    res["hsmg_pcg"]["cg"] = {"iters": it, "relres": rr, "s": tcg}
    for prec in (32, 64):
        t0 = time.perf_counter()
        m.mg_setup([2, 5, 11], precision=prec)
        tset = time.perf_counter() - t0
        x.zero_()
        m.pcg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                  max_iter=2000, check_every=2)      # warm-up
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, rr = m.pcg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                           max_iter=2000, check_every=2)
        tp = time.perf_counter() - t0
        res["hsmg_pcg"][f"pcg_fp{prec}_smoother"] = {"iters": it, "relres": rr, "s": tp,
                                                     "setup_s": tset}
    # the exact Galerkin coarse solve needs a vertex (order-1) coarsest
    # level: levels 12 -> 6 -> 2 points
    for prec in (32,):
        t0 = time.perf_counter()
        m.mg_setup([1, 5, 11], precision=prec)
        m.mg_setup_coarse(g.data_ptr())
        tset = time.perf_counter() - t0
        x.zero_()
        m.pcg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                  max_iter=2000, check_every=2)      # first call: scratch, kernel loading
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, rr = m.pcg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                           max_iter=2000, check_every=2)
        tp = time.perf_counter() - t0
        res["hsmg_pcg"][f"pcg_fp{prec}_smoother_exact_coarse_12_6_2"] = {
            "iters": it, "relres": rr, "s": tp, "setup_s": tset}
    res["hsmg_pcg"]["workload"] = ("16^3 deformed elements, lx1=12, levels 12->6->3, tol 1e-10, "
                                   f"FP64 operator order {order}")
    m.close()
    del g, c, f, x
    torch.cuda.empty_cache()
    res["batched_uneven"] = batched(nb, torch, dev)
    return res


def batch_boxes(nprob=256, seed=4096):
    """The batched workload: element counts log-uniform in [8, 4096]
    factorised by cubic (driver.f:196-247), lx1 uniform over {6, 8, 10, 12}."""
    import nekbone_gb300 as nb
    rng = np.random.default_rng(seed)
    e = np.rint(np.exp(rng.uniform(np.log(8), np.log(4096), nprob))).astype(int)
    lx = rng.choice([6, 8, 10, 12], nprob)
    return [(*nb.cubic(int(ei)), int(li)) for ei, li in zip(e, lx)]


# batched inner CG: per-problem stop at a residual reduction of INNER_TOL, at
# most INNER_MAX iterations per cycle (two cycles reach 1e-10)
INNER_TOL, INNER_MAX = 1e-5, 80


def batched(nb, torch, dev, reps=3):
    """256 independent Dirichlet problems solved to 1e-10 by one graph launch
    (FP32 inner CG, each problem's stopping once its residual fell by 1e-5 or
    after 80 iterations, FP64 defect correction), after the autotuner picked
    each lx1's operator shapes."""
    boxes = batch_boxes()
    t0 = time.perf_counter()
    b = nb.Batch(boxes)
    b.setup(777)
    setup_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.tune(3)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(nb.stream_handle(), device=dev)
    b.set_inner_tol(INNER_TOL)
    b.solve(1e-10, INNER_MAX, 60)       # warm-up (builds and instantiates the graph)
    nb.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.solve(1e-10, INNER_MAX, 60)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    res = [b.result(p) for p in range(b.nprob)]
    work = sum(b.problem(p)[1] * res[p][1] for p in range(b.nprob))
    # end to end: pinned host f in, solve, x out
    fh = torch.empty(b.n, dtype=torch.float64).pin_memory()
    xh = torch.empty(b.n, dtype=torch.float64).pin_memory()
    fdev = torch.as_tensor(_DevArray(b.arrays()[1], b.n), device=dev)
    fh.copy_(fdev.cpu())
    nb.sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        b.rhs_in(fh.data_ptr())
        b.solve(1e-10, INNER_MAX, 60)
        b.x_out(xh.data_ptr())
        nb.sync()
    e2e_ms = (time.perf_counter() - t0) / reps * 1e3
    # per-phase device times of one solve, launched cycle by cycle with an
    # event after every kernel (the graph solve runs them without the events)
    phases, _ = b.time_phases(1e-10, INNER_MAX, 60)
    lxs = sorted({bx[3] for bx in boxes})
    out = {
        "workload": "256 box problems, elements log-uniform in [8,4096] (cubic factorisation), "
                    "lx1 uniform over {6,8,10,12}, seeded uniform RHS, full Dirichlet mask; "
                    "FP32 inner CG (each problem's to a 1e-5 residual reduction, at most 80 iterations "
                    "per cycle) in FP64 defect correction to 1e-10",
        "problems": b.nprob, "points": b.n, "elements": b.nelt, "setup_s": setup_s,
        "tune_s": tune_s, "tuning": {str(l): b.tuning(l) for l in lxs},
        "solve_ms": ms, "graph_launches_per_solve": 1, "cycles": b.cycles(),
        "max_relres": max(r[2] for r in res), "max_outer": max(r[0] for r in res),
        "min_outer": min(r[0] for r in res),
        "inner_gdof_iter_per_s": work / (ms * 1e-3) / 1e9,
        "e2e_ms": e2e_ms, "e2e_h2d_bytes": 8 * b.n, "e2e_d2h_bytes": 8 * b.n,
        "phase_ms": {k: round(v, 4) for k, v in phases.items()},
        "phase_ms_sum": round(sum(phases.values()), 4),
    }
    b.close()
    return out


class _DevArray:
    """A float64 device array given by pointer, for torch.as_tensor."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8",
                                         "data": (ptr, False), "version": 3}


# --------------------------------------------------------------- GPU arm --
def _host(t):
    return t.detach().cpu().numpy()


def run_ours(a, rank, world, local):
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    import nekbone_gb300 as nb

    nel, lx, niter, order = a.nel, a.lx, a.niter, a.order
    t0 = time.perf_counter()
    mesh = nb.DeviceMesh(nel, nel, nel, lx, mask_mode=1)   # topology built on the device
    setup_s = time.perf_counter() - t0
    mesh.set_order(order)
    setup_host_s = None
    if not a.no_extras and world == 1:
        # the same mesh with jl's sort-based topology on the host, for comparison
        nb.set_setup_on_device(False)
        t0 = time.perf_counter()
        mh = nb.DeviceMesh(nel, nel, nel, lx, mask_mode=1)
        setup_host_s = time.perf_counter() - t0
        nb.set_setup_on_device(True)
        mh.close()
    n = mesh.n
    g = torch.empty(6 * n, dtype=torch.float64, device=dev)
    c = torch.empty(n, dtype=torch.float64, device=dev)
    f = torch.empty(n, dtype=torch.float64, device=dev)
    mesh.setup_g(g.data_ptr())
    mesh.set_multiplicity(c.data_ptr())
    mesh.rhs_uniform(f.data_ptr(), c.data_ptr(), RHS_SEED + rank)
    x, r, w, p, z = (torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(5))
    ptrs = [t.data_ptr() for t in (x, f, g, c, r, w, p, z)]
    stream = torch.cuda.ExternalStream(nb.stream_handle(), device=dev)
    torch.cuda.synchronize()

    def step():
        mesh.cg(*ptrs, niter)

    for _ in range(a.warmup):
        step()
    nb.sync()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        e0.record(stream)
        for _ in range(a.steps):
            step()
        e1.record(stream)
        e1.synchronize()
    nb.sync()
    torch.cuda.synchronize()
    ms, value = replica_rate(e0.elapsed_time(e1), n, niter, a.steps, world, dev)
    unique = ((lx - 1) * nel + 1) ** 3
    clocks = clk.summary()
    ms_per_step = ms / a.steps
    # per step: x = 0 / r = mask(f) / r'Cr (3), the fixed-point metric (order 2),
    # then 3 kernels per iteration
    launches_per_step = 3 + (1 if order == 2 else 0) + 3 * niter
    x100 = _host(x) if rank == 0 and world == 1 and not a.no_cpu else None

    # each kernel of one iteration on the same stream, for both FP64
    # operator forms on the integer / FP64 pipes (the chosen one first)
    kms = {}
    for o in [order] + [q for q in (2, 1) if q != order]:
        mesh.set_order(o)
        kms[o] = mesh.time_cg_kernels(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(),
                                      r.data_ptr(), w.data_ptr(), p.data_ptr(), reps=10)
    mesh.set_order(order)
    ax_bytes = 64 * n   # u 8 + g 48 + w 8 per point (ax, stored metric)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    rates = nb.pipe_rates()
    achieved = ax_bytes / (kms[order][0] * 1e-3) / 1e9
    flops_pt = 19 + 12 * lx
    names = {2: f"k_ax_fx<{lx},1> (fused FP64 element operator in 64-bit fixed point on the "
                f"integer pipes, even-odd contractions)",
             1: f"k_ax_eo4<double,{lx},1> (fused FP64 element operator, even-odd contractions "
                f"on the FP64 pipe)",
             0: f"k_ax_impl<double,{lx},1,false> (fused FP64 element operator, reference order)"}
    trf = DRAM_BYTES_PER_POINT.get(order) if lx == 12 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": trf[0] * n if trf else None,
                "traffic_source": trf[1] if trf else None,
                "kernel": names[order],
                "algorithmic_bytes_per_point": 64,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback",
                "kernel_ms": {"ax": kms[order][0], "gs_fin": kms[order][1],
                              "update": kms[order][2]},
                "iteration_ms_by_operator": {
                    ("fixed_point" if o == 2 else "fp64_pipe" if o == 1 else "reference_order"):
                        {"ax": kms[o][0], "gs_fin": kms[o][1], "update": kms[o][2],
                         "iteration": float(sum(kms[o]))} for o in kms},
                # live issue rates of the pipes (nb_pipe_rates) and the reference's flop
                # count per point (cg.f:122) at the operator's time
                "pipes": {"measured_ops_per_s": rates,
                          "reference_flops_per_point": flops_pt,
                          "tflops_reference_count": flops_pt * n / (kms[order][0] * 1e-3) / 1e12}}

    # the FP32 iteration of the mixed solver's inner CG, same mesh
    f32, g32, c32 = f.float(), g.float(), c.float()
    x32, r32, w32, p32 = (torch.zeros(n, dtype=torch.float32, device=dev) for _ in range(4))
    torch.cuda.synchronize()
    kms32 = mesh.time_cg_kernels_f32(x32.data_ptr(), f32.data_ptr(), g32.data_ptr(),
                                     c32.data_ptr(), r32.data_ptr(), w32.data_ptr(),
                                     p32.data_ptr(), reps=10)
    ax32_bytes = 32 * n
    roofline["fp32_inner_iteration"] = {
        "kernel_ms": {"ax": kms32[0], "gs_fin": kms32[1], "update": kms32[2]},
        "ax_achieved_gbs": ax32_bytes / (kms32[0] * 1e-3) / 1e9,
        "ax_frac": ax32_bytes / (kms32[0] * 1e-3) / 1e9 / peak,
        "iteration_ms": float(sum(kms32))}
    del f32, g32, c32, x32, r32, w32, p32

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(nel, lx, niter),
           "operator_order": order,
           "setup": {"device_topology_s": setup_s, "host_topology_s": setup_host_s,
                     # unique global DOFs of the box, (N nelx + 1)(N nely + 1)(N nelz + 1)
                     "unique_dofs": unique, "value_unique_gdof_iter_per_s": value * unique / n},
           "gpu_launches": launches_per_step * a.steps, "clocks": clocks, "roofline": roofline}

    # ---- the CPU oracle on the same mesh and inputs (rank 0, one GPU)
    case = None
    if rank == 0 and world == 1 and not a.no_cpu:
        threads = os.cpu_count() or 1
        case = CpuCase(nel, lx, threads)
        assert np.array_equal(case.g, _host(g)) and np.array_equal(case.c, _host(c))
        assert np.array_equal(case.f, _host(f))
        ok, dt = case.cg(a.cpu_sample_iters)
        v = n * a.cpu_sample_iters / dt / 1e9
        # the GPU's iterate after the same number of iterations
        mesh.cg(*ptrs, a.cpu_sample_iters)
        nb.sync()
        xk = _host(x)
        scale_f = float(np.max(np.abs(case.f)))
        out["cpu_check"] = {
            "iterate_iters": a.cpu_sample_iters,
            "x_rel_err": float(np.max(np.abs(xk - ok["x"])) / np.max(np.abs(ok["x"]))),
            "r_err_on_f_scale": float(np.max(np.abs(_host(r) - ok["r"])) / scale_f),
            "headline_x_cpu_relres": case.relres(x100),
            "oracle_setup_s": case.setup_s}
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{nel}^3 elements, lx1={lx} (n={n}), the headline "
                                         f"solve's first {a.cpu_sample_iters} FP64 CG iterations, "
                                         f"{dt:.1f} s"}
        # the same port on one core (the reference has no threading of its own)
        case.ctx.set_threads(1)
        v1, dt1 = case.rate(1)
        case.ctx.set_threads(threads)
        out["cpu_baseline_single_core"] = {
            "value": v1, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{nel}^3 elements, lx1={lx} (n={n}), 1 FP64 CG iteration, {dt1:.1f} s"}

    # ---- mixed vs FP64 time to tolerance
    if not a.no_mixed:
        xt = torch.zeros(n, dtype=torch.float64, device=dev)
        xm = torch.zeros(n, dtype=torch.float64, device=dev)
        args = (f.data_ptr(), g.data_ptr(), c.data_ptr())
        # one untimed solve of each kind first (first-use scratch allocation,
        # kernel loading), as the FP64 headline has its warm-up steps
        mesh.cg_tol(xt.data_ptr(), *args, a.tol, max_iter=20000, check_every=1)
        mesh.cg_mixed(xm.data_ptr(), *args, a.tol, 20, 5000)

        def timed(fn):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = fn()
            torch.cuda.synchronize()
            return res, time.perf_counter() - t0

        # FP64 CG polled every iteration: charged the iterations it needs
        xt.zero_()
        (it64, rr64), t64 = timed(lambda: mesh.cg_tol(xt.data_ptr(), *args, a.tol,
                                                      max_iter=20000, check_every=1))
        mx = {}
        try:
            for key, shared, tc in (("per_element_metric", False, False),
                                    ("shared_metric_block", True, False),
                                    ("tensor_cores", False, True)):
                nb.set_shared_metric(shared)
                nb.set_mixed_tensor_cores(tc)
                if tc:
                    mesh.cg_mixed(xm.data_ptr(), *args, a.tol, 20, 5000)   # warm-up
                xm.zero_()
                (o_, i_, rr_), t_ = timed(lambda: mesh.cg_mixed(xm.data_ptr(), *args, a.tol,
                                                                20, 5000))
                d = float((xm - xt).abs().max().item() / max(xt.abs().max().item(), 1e-300))
                mx[key] = {"s": t_, "outer": o_, "inner_iters": i_, "relres": rr_,
                           "speedup_vs_fp64": t64 / t_, "x_rel_diff_vs_fp64": d}
                if case is not None:
                    mx[key]["cpu_relres"] = case.relres(_host(xm))
        finally:
            nb.set_shared_metric(True)
            nb.set_mixed_tensor_cores(False)
        fp64 = {"s": t64, "iters": it64, "relres": rr64, "check_every": 1}
        if case is not None:
            fp64["cpu_relres"] = case.relres(_host(xt))
        out["mixed_detail"] = {"tol": a.tol, "fp64_cg": fp64, **mx,
                               "note": "per_element_metric is the headline mixed figure: "
                                       "the inner FP32 operator reads each element's metric; "
                                       "shared_metric_block reads one block for all (box "
                                       "meshes only) and is reported separately"}
        out["_mixed"] = {"tol": a.tol, "fp64_s": t64, "fp64_iters": it64,
                         "mixed_s": mx["per_element_metric"]["s"],
                         "speedup": mx["per_element_metric"]["speedup_vs_fp64"],
                         "mixed_relres": mx["per_element_metric"]["relres"],
                         "cpu_relres_fp64": fp64.get("cpu_relres"),
                         "cpu_relres_mixed": mx["per_element_metric"].get("cpu_relres"),
                         "speedup_shared_metric": mx["shared_metric_block"]["speedup_vs_fp64"],
                         "speedup_tensor_cores": mx["tensor_cores"]["speedup_vs_fp64"]}
        del xt, xm
    case = None

    # ---- the other workloads, one measurement each (not the headline)
    if not a.no_extras and world == 1:
        del x, r, w, p, z
        torch.cuda.empty_cache()
        out["extras"] = extras(nb, torch, dev, order)
        x = r = w = p = z = None

    # ---- end to end through the drop-in cg_ with pinned host buffers
    if not a.no_e2e:
        x = r = w = p = z = None
        torch.cuda.empty_cache()
        hb = nb.Nekbone(nel, nel, nel, lx, mask_mode=1)
        nb.Nekbone.set_order(order)
        pin = lambda t: t.cpu().pin_memory()
        fh, gh, ch = pin(f), pin(g), pin(c)
        work = [torch.zeros(n, dtype=torch.float64).pin_memory() for _ in range(5)]
        fn, gn, cn = fh.numpy(), gh.numpy(), ch.numpy()
        wn = tuple(t.numpy() for t in work)
        hb.cg(fn, gn, cn, niter, 0.0, wn)      # warm-up
        torch.cuda.synchronize()
        calls = []
        with Clocks(local) as clk_e2e:
            t0 = time.perf_counter()
            for _ in range(a.steps):
                t1 = time.perf_counter()
                hb.cg(fn, gn, cn, niter, 0.0, wn)
                calls.append((time.perf_counter() - t1) * 1e3)
            e2e_s = (time.perf_counter() - t0) / a.steps
        out["e2e"] = {"value": world * n * niter / e2e_s / 1e9, "unit": UNIT,
                      "h2d_bytes_per_step": 64 * n, "d2h_bytes_per_step": 40 * n,
                      "ms_per_step": e2e_s * 1e3, "call": "cg_ (C ABI, host arrays)",
                      "calls_ms": [round(v, 2) for v in calls],
                      "clocks": clk_e2e.summary()}

    if "_mixed" in out:
        out["mixed"] = out.pop("_mixed")       # last key: the driver's tail shows it
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_case(a):
    """Small cases for kernel profiles (one JSON line of timings, not a bench
    line): 'tc' applies the tensor-core and CUDA-core FP32 operators on 16^3
    deformed elements (lx1 = --lx); 'batch' solves the first 32 problems of
    the batched workload once after tuning; 'hsmg' runs 6 PCG iterations with
    the FP32-smoother V-cycle (levels 12 -> 6 -> 2 points, exact coarse solve)
    on 16^3 deformed elements, lx1 = 12; 'mixed' runs one mixed-precision
    solve (20 FP32 inner iterations per cycle) to 1e-10 on the --nel^3 box,
    lx1 = --lx."""
    import torch
    import nekbone_gb300 as nb
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    stream = torch.cuda.ExternalStream(nb.stream_handle(), device=dev)
    if a.case == "tc":
        m = nb.DeviceMesh(16, 16, 16, a.lx, mask_mode=1)
        n = m.n
        g = torch.empty(6 * n, dtype=torch.float64, device=dev)
        m.setup_g_deformed(g.data_ptr(), 11, 0.1)
        g32 = g.float()
        u = torch.rand(n, dtype=torch.float32, device=dev)
        w = torch.empty_like(u)
        torch.cuda.synchronize()
        out = {"case": "tc", "n": n, "lx": a.lx,
               "tc_ms": _time_on(stream, torch, lambda: m.ax_tc(w.data_ptr(), u.data_ptr(),
                                                                g32.data_ptr()), reps=3),
               "fp32_ms": _time_on(stream, torch, lambda: m.ax_f32(w.data_ptr(), u.data_ptr(),
                                                                   g32.data_ptr()), reps=3)}
    elif a.case == "hsmg":
        m = nb.DeviceMesh(16, 16, 16, 12, mask_mode=1)
        n = m.n
        g = torch.empty(6 * n, dtype=torch.float64, device=dev)
        c = torch.empty(n, dtype=torch.float64, device=dev)
        f = torch.empty(n, dtype=torch.float64, device=dev)
        m.setup_g_deformed(g.data_ptr(), 11, 0.1)
        m.set_multiplicity(c.data_ptr())
        m.rhs_uniform(f.data_ptr(), c.data_ptr(), 5)
        m.mg_setup([1, 5, 11], precision=32)
        m.mg_setup_coarse(g.data_ptr())
        x = torch.zeros_like(f)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it, rr = m.pcg_tol(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(), 1e-10,
                           max_iter=6, check_every=6)
        out = {"case": "hsmg", "n": n, "iters": it, "relres": rr,
               "s": time.perf_counter() - t0}
        m.close()
    elif a.case == "mixed":
        m = nb.DeviceMesh(a.nel, a.nel, a.nel, a.lx, mask_mode=1)
        n = m.n
        g = torch.empty(6 * n, dtype=torch.float64, device=dev)
        c = torch.empty(n, dtype=torch.float64, device=dev)
        f = torch.empty(n, dtype=torch.float64, device=dev)
        m.setup_g(g.data_ptr())
        m.set_multiplicity(c.data_ptr())
        m.rhs_uniform(f.data_ptr(), c.data_ptr(), 20260)
        x = torch.zeros_like(f)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        outer, inner, rr = m.cg_mixed(x.data_ptr(), f.data_ptr(), g.data_ptr(), c.data_ptr(),
                                      a.tol, 20, 500)
        out = {"case": "mixed", "n": n, "outer": outer, "inner": inner, "relres": rr,
               "s": time.perf_counter() - t0}
        m.close()
    else:
        b = nb.Batch(batch_boxes()[:32])
        b.setup(777)
        b.tune(1)
        b.set_inner_tol(INNER_TOL)
        torch.cuda.synchronize()
        b.solve(1e-10, INNER_MAX, 60)
        nb.sync()
        out = {"case": "batch", "problems": b.nprob, "points": b.n, "cycles": b.cycles(),
               "max_relres": max(b.result(p)[2] for p in range(b.nprob))}
        b.close()
    print(json.dumps(out), flush=True)


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    if a.case != "cg":
        run_case(a)
        return
    run_ours(a, rank, world, local)


if __name__ == "__main__":
    main()
