"""Benchmark: ms per RK3 step and Mcells/s of the four-block turbulent channel on one GB300.

Workload (the configuration the headline metric is quoted on): four uneven blocks
(x: 96|160, y: 64|80, z: 128) tiling 256x144x128 = 4.72M cells on a
4pi x 2 x 4pi/3 box, periodic x and z through friend links, no-slip walls in y
with a global tanh-stretched wall-normal grid (alpha = 1.8), Re_tau = 180,
FFT along z, every Poisson solve to a relative residual of 1e-12.  Initial
field: laminar Poiseuille profile scaled to U_b plus seeded uniform noise of
0.1 U_b (synthetic; the reference publishes no dataset for this case).

A "step" is one full RK3 step (3 stages: momentum, halo/BC, divergence,
transform, 128 batched 2-D solves, back-transform, projection, pressure
update; chkdt every icheck=10 steps).  `value` is the mixed path (FP32 V-cycles
inside FP64 refinement, with the solver settings snac_autotune picks after the warm-up steps: tile
shape, CTA waves, inner iterations, coarse sweeps); the plain FP64 path (library defaults) and the mixed
path with the learned
initial guess (pairs recorded from 8 steps, the network trained on the GPU, then
timed) are reported beside it at the same solver tolerance.  Inputs (~0.5 GB of
fields + solver vectors) exceed L2.

--impl reference times the CPU restatement of the reference (the Fortran/HYPRE
reference cannot be built on these machines) on the host cores, same case.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per RK3 step & Mcells/s on 1 GB300, learned+mixed vs plain, equal |div u|"


def max_over_ranks(x, device=0):
    """Largest value of x over the ranks of the job (x itself when not distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return x
    on_gpu = dist.get_backend() == "nccl"
    t = torch.tensor([float(x)], dtype=torch.float64, device=f"cuda:{device}" if on_gpu else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_barrier(device=0):
    """Barrier over the job's ranks, with the device drained on both sides."""
    import torch
    import torch.distributed as dist
    if torch.cuda.is_available():
        torch.cuda.synchronize(device)
    if dist.is_available() and dist.is_initialized():
        if dist.get_backend() == "nccl":
            dist.barrier(device_ids=[device])
        else:
            dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize(device)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for q, n in enumerate(names):
                if len(r) > 5 + q and r[5 + q].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def init_channel(dom, case):
    from snac_gb300 import capi, cases
    ic = cases.channel_initial_condition(case, lambda ib: dom.grid(ib, 1, capi.G_XC))
    for ib, (u, v, w) in ic.items():
        dom.set(ib, capi.U, u)
        dom.set(ib, capi.V, v)
        dom.set(ib, capi.W, w)
    dom.bounduvw(False)
    dom.boundp(capi.P)


# algorithmic bytes / FP64 flops per cell and launch of the profiled kernels (FP64 state)
KERNEL_WORK = {
    # kid: (name, bytes per cell, flops per cell, cells-per-launch key)
    1: ("k_rk_mom", 104.0, 180.0, "cells"),
    4: ("k_fft_fwd_box", 16.0, 22.0, "cells"),
    2: ("k_rbgs<float>", 12.0, 0.0, "cells"),
}


USE_GRAPH = 1  # the mixed path replays its refinement steps as CUDA graphs (bench.py --no-graph: off)


def other_configs():
    """The reference configurations other than the headline channel, at their stated sizes: (case, initial
    state, description).  The L-shaped box is three 144 x 144 x 96 blocks (5.97 M cells, the configuration's
    "~6M cells" in three blocks)."""
    from snac_gb300 import cases
    return {
        "c1_ldc64": (lambda: cases.lid_driven_cavity(64), init_rest,
                     "lid-driven cavity 64^3, Re=1000, CFL 0.5, 3-D multigrid, from rest"),
        "c2_tgv128": (lambda: cases.taylor_green(128), init_tgv,
                      "Taylor-Green vortex 128^3, Re=1600, FFT along z (128 systems of 128x128)"),
        "c4_lbox": (lambda: cases.l_shaped_box(144, 96), init_rest,
                    "L-shaped closed box, 3 blocks of 144x144x96, lid-driven, Re=2000, 3-D multigrid, from rest"),
        "c5_dhc512": (lambda: cases.heated_cavity((512, 512, 256), dt_f=1e-3), init_dhc,
                      "heated cavity 512x512x256, stretched 1.5, Ra=1e8, Pr=0.71, IMPDIFF (u,v,w,T Helmholtz) + "
                      "3-D pressure multigrid, T noise 1e-3, fixed dt 1e-3 (dt_f of the reference's heated-cavity "
                      "test: from rest the CFL limit is unbounded and IMPDIFF has no viscous one)"),
    }


def bench_configs(names, steps, warmup, device, learned_c4=1500):
    """ms per RK3 step, Mcells/s and max|div u| of the plain FP64 and the mixed path on each configuration."""
    out = {}
    cfgs = other_configs()
    for name in names:
        case_fn, init, desc = cfgs[name]
        row = {"workload": desc, "cells": case_fn().ncell}
        for label, prec in (("mixed", 1), ("plain_fp64", 0)):
            r = run_gpu_path(case_fn, prec, steps, warmup, device, init=init)
            row[label] = {"ms_per_step": r["ms"], "mcells_per_s": r["ncell"] / (r["ms"] * 1e-3) / 1e6,
                          "max_div_u": r["divmax"], "solve_iters_max": r["iters"],
                          "solve_residual_max": r["residual"], "helm_iters_max": r["helm_iters"],
                          "setup_s": r["setup_s"], "rc": r["rc"]}
        row["speedup_mixed_vs_plain"] = row["plain_fp64"]["ms_per_step"] / row["mixed"]["ms_per_step"]
        if name == "c4_lbox" and learned_c4:
            # the configuration's learned guess: 2,000 crops (4 per solve, 3 solves per step) recorded from the
            # case's own solves, the U-Net trained on them, then guided steps at the same 1e-12 tolerance
            lr_ = run_learned_path(case_fn, steps, warmup, device, record=167, train_iters=learned_c4, init=init)
            row["learned_mixed"] = {k: lr_[k] for k in ("ms_per_step", "solve_iters_max", "solve_residual_max",
                                                       "max_div_u", "pairs", "train_iters", "train_s", "loss_first",
                                                       "loss_last", "residual_ratio_median")}
            row["learned_mixed"]["mcells_per_s"] = row["cells"] / (lr_["ms_per_step"] * 1e-3) / 1e6
        out[name] = row
    return out


def init_rest(dom, case):
    """Zero velocity and pressure (the lid-driven cavities); only the boundary conditions."""
    from snac_gb300 import capi
    dom.bounduvw(False)
    dom.boundp(capi.P)


def init_tgv(dom, case):
    """Taylor-Green vortex with its analytic pressure."""
    from snac_gb300 import capi, cases
    for ib, (u, v, w, p) in cases.tgv_initial_condition(case, dom.grid).items():
        for k, f in ((capi.U, u), (capi.V, v), (capi.W, w), (capi.P, p)):
            dom.set(ib, k, f)
    dom.bounduvw(False)
    dom.boundp(capi.P)


def init_dhc(dom, case):
    """Heated cavity: zero velocity, T = seeded uniform noise of amplitude 1e-3 (splitmix64, seed 0x5EED)."""
    from snac_gb300 import capi, cases
    for ib, b in enumerate(case.blocks):
        n = [int(x) for x in b.ng]
        t = np.zeros([x + 2 for x in n], order="F")
        r = cases.splitmix64_uniform_fast(0x5EED, n[0] * n[1] * n[2]).reshape(n, order="F")
        t[1:-1, 1:-1, 1:-1] = 2e-3 * (r - 0.5)
        dom.set(ib, capi.S0, t)
    dom.bounduvw(False)
    dom.boundp(capi.P)
    dom.boundp(capi.S0)


def run_gpu_path(case_fn, precision, steps, warmup, device, profile_kid=0, init=None, tune=0, **solver):
    """solver: snac_options fields passed to the domain (the library defaults when absent); init(dom, case)
    sets the initial state (default: the channel's); tune > 0: snac_autotune with that many timed steps per
    candidate after the warm-up (its choice is returned in `tuned`, as snac_options fields)."""
    from snac_gb300 import capi
    from snac_gb300.domain import Domain
    case = case_fn()
    t0 = time.perf_counter()
    dom = Domain(case, precision=precision, device=device, use_graph=USE_GRAPH if precision else 0, **solver)
    setup_s = time.perf_counter() - t0
    try:
        (init or init_channel)(dom, case)
        dom.step(warmup, allow_not_converged=True)
        tuned = None
        if tune:
            r = dom.autotune(tune)
            tuned = dict(precision=r["precision"], inner_iters=r["inner_iters"], nu_coarse=r["nu_coarse"],
                         mg_tile=r["mg_tile"], mg_waves=r["mg_waves"], mg_cta_level=r["mg_cta_level"],
                         refine_steps=r["refine_steps"], ms_before=r["ms_before"], ms_tuned=r["ms_per_step"],
                         candidates=r["candidates"])
            dom.step(1, allow_not_converged=True)
        L = capi.lib()
        if profile_kid:
            capi.check(L.snac_profile_kernel(profile_kid))
        n0 = C.c_longlong()
        capi.check(L.snac_launch_count(C.byref(n0)))
        rank_barrier(device)
        rc = dom.step(steps, allow_not_converged=True)
        rank_barrier(device)
        n1 = C.c_longlong()
        capi.check(L.snac_launch_count(C.byref(n1)))
        st = dom.stats()
        prof = None
        if profile_kid:
            n = C.c_int(); tot = C.c_double()
            capi.check(L.snac_profile_read(C.byref(n), C.byref(tot)))
            capi.check(L.snac_profile_kernel(0))
            prof = (n.value, tot.value)
        divtot, divmax = dom.chkdiv()
        ke = dom.kinetic_energy()
        return dict(ms=st["device_ms"] / steps, iters=st["iters"], residual=st["residual"], divmax=divmax, ke=ke,
                    rc=rc, prof=prof, ncell=case.ncell, dt=st["dt"], launches=n1.value - n0.value,
                    helm_iters=st["helm_iters"], helm_residual=st["helm_residual"], setup_s=setup_s, tuned=tuned)
    finally:
        dom.close()


def run_learned_path(case_fn, steps, warmup, device, record=8, train_iters=1500, lr=2e-3, init=None, **solver):
    """Mixed path with the learned initial guess: pairs recorded from `record` steps after the warm-up, the
    network trained on the GPU, then `steps` timed steps with the guess applied (and one more that measures
    the residual it leaves relative to the previous solution's, per wavenumber system; one ratio for the
    3-D solve).  With a transform axis the network is the plane network, with the 3-D solve the U-Net, whose
    pairs are four 32^3 crops per solve."""
    from snac_gb300 import capi
    from snac_gb300.domain import Domain
    case = case_fn()
    L = capi.lib()
    dom = Domain(case, precision=1, device=device, use_graph=USE_GRAPH, **solver)
    try:
        (init or init_channel)(dom, case)
        dom.step(warmup, allow_not_converged=True)
        capi.check(L.snac_guess_mode(1))
        dom.step(record, allow_not_converged=True)
        lf, ll, npairs = C.c_double(), C.c_double(), C.c_int()
        t0 = time.time()
        capi.check(L.snac_guess_train(train_iters, lr, C.byref(lf), C.byref(ll), C.byref(npairs)))
        train_s = time.time() - t0
        capi.check(L.snac_guess_mode(2))
        dom.step(1, allow_not_converged=True)
        dom.step(steps, allow_not_converged=True)
        st = dom.stats()
        capi.check(L.snac_guess_measure(1, None, None))
        dom.step(1, allow_not_converged=True)
        med, mx = C.c_double(), C.c_double()
        capi.check(L.snac_guess_measure(0, C.byref(med), C.byref(mx)))
        divtot, divmax = dom.chkdiv()
        return {"ms_per_step": st["device_ms"] / steps, "solve_iters_max": st["iters"],
                "solve_residual_max": st["residual"], "max_div_u": divmax, "pairs": npairs.value,
                "train_iters": train_iters, "train_s": train_s, "loss_first": lf.value, "loss_last": ll.value,
                "residual_ratio_median": med.value, "residual_ratio_max": mx.value}
    finally:
        L.snac_guess_mode(0)
        dom.close()


def bench_smoother(case_fn, device, levels=(0, 1, 2), reps=20, **solver):
    """CUDA-event timing of the FP32 tiled pre-smoother (the dominant kernel) on the bench workload,
    inputs resident in HBM, all systems active: ms and algorithmic bytes per launch per level."""
    from snac_gb300 import capi
    from snac_gb300.domain import Domain
    case = case_fn()
    dom = Domain(case, precision=1, device=device, **solver)
    out = {}
    try:
        init_channel(dom, case)
        dom.step(1, allow_not_converged=True)
        L = capi.lib()
        for lev in levels:
            ms = C.c_double(); nb = C.c_double()
            if L.snac_bench_smoother(lev, reps, C.byref(ms), C.byref(nb)) == 0:
                out[lev] = (ms.value, nb.value)
    finally:
        dom.close()
    return out


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (None when absent)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f).get(kernel, {}).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        return None


def run_e2e(case_fn, precision, steps, device, **solver):
    """Through the C ABI with host buffers: upload u,v,w,p of every block from pinned host memory in one
    snac_set_fields call, one step, read them back with snac_get_fields."""
    import torch
    from snac_gb300 import capi
    from snac_gb300.domain import Domain
    case = case_fn()
    dom = Domain(case, precision=precision, device=device, use_graph=USE_GRAPH if precision else 0, **solver)
    try:
        init_channel(dom, case)
        dom.step(1, allow_not_converged=True)
        host = {}
        for ib in range(dom.nblocks):
            for k in (capi.U, capi.V, capi.W, capi.P):
                shp = dom.shape(ib, k)
                t = torch.empty(int(np.prod(shp)), dtype=torch.float64, pin_memory=True)
                a = t.numpy().reshape(shp, order="F")
                a[...] = dom.get(ib, k)
                host[(ib, k)] = (t, a)
        nbytes = sum(a.nbytes for (_, a) in host.values())
        items = [(ib, k, a) for (ib, k), (_, a) in host.items()]
        t0 = time.perf_counter()
        for _ in range(steps):
            dom.set_many(items)  # snac_set_fields: every field's copy issued, one synchronisation
            dom.step(1, allow_not_converged=True)
            dom.get_many(items)  # snac_get_fields
        el = time.perf_counter() - t0
        return dict(s_per_step=el / steps, h2d=nbytes, d2h=nbytes, ncell=case.ncell)
    finally:
        dom.close()


def cpu_reference(case_fn, steps, warmup, budget_s=60.0):
    """The oracle (CPU restatement of the reference) on all host cores, bounded to ~budget_s of stepping."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from snac_gb300 import cases
    case = case_fn()
    d = O.OracleDomain(case)
    ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, O.G_XC))
    for ib, (u, v, w) in ic.items():
        d.field(ib, O.U)[...] = u
        d.field(ib, O.V)[...] = v
        d.field(ib, O.W)[...] = w
    d.bounduvw(False)
    d.boundp(O.P)
    t0 = time.perf_counter()
    d.step(1)                       # warm-up (first-touch, dt) -- always one
    first = time.perf_counter() - t0
    nrun = max(1, min(steps, int(budget_s / max(first, 1e-3))))
    t0 = time.perf_counter()
    d.step(nrun)
    el = time.perf_counter() - t0
    d.close()
    return dict(ms=1e3 * el / nrun, nrun=nrun, ncell=case.ncell, cores=os.cpu_count())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--case", choices=["channel", "small"], default="channel",
                    help="channel: the benchmark workload; small: the same layout at test size")
    ap.add_argument("--no-graph", action="store_true", help="launch the refinement steps one kernel at a time")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-guess path (record, train, time)")
    ap.add_argument("--configs", default="c1_ldc64,c2_tgv128,c4_lbox,c5_dhc512",
                    help="other reference configurations timed beside the headline (comma list; empty: none)")
    ap.add_argument("--config-steps", type=int, default=3, help="timed steps per configuration and path")
    ap.add_argument("--c4-train", type=int, default=1500,
                    help="Adam steps of the U-Net guess on the L-shaped box's 2,000 recorded crops (0: no learned "
                         "path for that configuration)")
    ap.add_argument("--tune", type=int, default=3,
                    help="snac_autotune with this many timed steps per candidate before the headline path is "
                         "timed (0: the library defaults)")
    ap.add_argument("--only", choices=["mixed", "plain", "learned"], default=None,
                    help="run one path once and print its timing only (used for ncu launch lists; learned: "
                         "1 recorded step and 20 training iterations)")
    args = ap.parse_args()
    global USE_GRAPH
    if args.no_graph:
        USE_GRAPH = 0
    rank, world, local = dist_env()
    from snac_gb300 import cases
    if args.case == "small":  # the same four-block layout at 48x24x16 (tests of the multi-rank logic)
        case_fn = lambda: cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
        cfg = {"workload": "channel4 48x24x16 (4 uneven blocks 16|32 x 8|16 x 16), FFT along z",
               "cells": case_fn().ncell, "solver_tol": 1e-12, "blocks": 4, "l2_policy": "fits in L2 (test size)"}
    else:
        case_fn = lambda: cases.channel_4block()
        cfg = {"workload": "channel4 256x144x128 (4 uneven blocks 96|160 x 64|80 x 128), Re_tau=180, FFT along z",
               "cells": cases.channel_4block().ncell, "solver_tol": 1e-12, "blocks": 4,
               "l2_policy": "inputs larger than L2 (fields + solver vectors ~1.3 GB)"}

    if args.impl == "reference":
        if rank != 0:
            return
        r = cpu_reference(case_fn, args.steps, args.warmup)
        mcells = r["ncell"] / (r["ms"] * 1e-3) / 1e6
        line = {"metric": METRIC, "impl": "reference", "value": mcells, "unit": "Mcells/s", "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "cpu_baseline": {"value": mcells, "unit": "Mcells/s", "cores": r["cores"], "kind": "port",
                                 "sample": f"{r['nrun']} RK3 step(s) of the full case after 1 warm-up step "
                                           "(the Fortran/HYPRE reference cannot be built here; its C restatement "
                                           "with OpenMP on all host cores)"},
                "e2e": {"value": mcells, "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local
    if args.only == "learned":
        r = run_learned_path(case_fn, args.steps, args.warmup, device, record=1, train_iters=20)
        if rank == 0:
            print(json.dumps({"path": "learned", **r}), flush=True)
        return
    if args.only:
        r = run_gpu_path(case_fn, 1 if args.only == "mixed" else 0, args.steps, args.warmup, device)
        if rank == 0:
            print(json.dumps({"path": args.only, "ms_per_step": r["ms"], "max_div_u": r["divmax"],
                              "solve_iters_max": r["iters"]}), flush=True)
        return
    sampler = ClockSampler(device)
    # plain FP64 path
    plain = run_gpu_path(case_fn, 0, args.steps, args.warmup, device)
    # mixed path, the headline; clocks sampled over its timed region
    sampler.start()
    mixed = run_gpu_path(case_fn, 1, args.steps, args.warmup, device, tune=args.tune)
    clocks = sampler.stop()
    # the settings the autotuner chose (tile shape, waves, coarse-cycle level, inner iterations ...) for every
    # further run of the mixed path
    opts = {k: mixed["tuned"][k] for k in ("inner_iters", "nu_coarse", "mg_tile", "mg_waves", "mg_cta_level",
                                           "refine_steps")} if mixed["tuned"] else {}
    # live CUDA-event timing of the kernel classes over timed runs of the mixed path
    shares = {}
    for kid, name in ((10, "pressure_solve"), (2, "smoother"), (9, "coarse_vcycle"), (3, "restriction"),
                      (6, "operator_apply"), (1, "k_rk_mom"), (4, "fft_forward_box")):
        n, tot = run_gpu_path(case_fn, 1, args.steps, args.warmup, device, profile_kid=kid, **opts)["prof"]
        shares[name] = {"launches_per_step": n / args.steps, "ms_per_step": tot / args.steps,
                        "mean_launch_ms": tot / max(n, 1)}
    prof_mom = (shares["k_rk_mom"]["launches_per_step"] * args.steps, shares["k_rk_mom"]["ms_per_step"] * args.steps)
    learned = run_learned_path(case_fn, args.steps, args.warmup, device, **opts) if not args.no_learned else None
    smoother = bench_smoother(case_fn, device, **opts)
    ms = mixed["ms"]
    ms = max_over_ranks(ms, device)
    ncell = mixed["ncell"]
    value = world * ncell / (ms * 1e-3) / 1e6
    e2e = None
    if not args.no_e2e:
        e = run_e2e(case_fn, 1, max(2, min(args.steps, 5)), device, **opts)
        e2e = {"value": world * e["ncell"] / e["s_per_step"] / 1e6, "unit": "Mcells/s",
               "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"],
               "ms_per_step": 1e3 * e["s_per_step"]}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    from snac_gb300 import capi
    f64 = C.c_double(); f32 = C.c_double()
    capi.check(capi.lib().snac_probe_peaks(C.byref(f64), C.byref(f32)))
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # roofline of the k_rk_mom kernel (FP64 state, FP64-pipe bound on GB300)
    n, tot = prof_mom
    launch_ms = tot / max(n, 1)
    mom_bytes = 104.0 * ncell
    mom_flops = KERNEL_WORK[1][2] * ncell
    peak_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s"
    roof_mom = {"kernel": "k_rk_mom", "bound": "fp64", "achieved": mom_bytes / (launch_ms * 1e-3) / 1e9,
                "peak": hbm_peak, "unit": "GB/s", "frac": None, "traffic": ncu_traffic("k_rk_mom"),
                "peak_source": peak_src, "launch_ms": launch_ms, "launches": n,
                "fp64": {"achieved_gflops": mom_flops / (launch_ms * 1e-3) / 1e9, "peak_gflops": f64.value,
                         "frac": mom_flops / (launch_ms * 1e-3) / 1e9 / f64.value,
                         "note": "FP64 FMA-stream peak measured on this GPU by snac_probe_peaks"}}
    roof_mom["frac"] = roof_mom["achieved"] / roof_mom["peak"]
    # dominant kernel: the FP32 tiled red-black smoother of the pressure solve (level-0 pre-smoother)
    roof = None
    if 0 in smoother:
        sm_ms, sm_bytes = smoother[0]
        restricting = opts.get("mg_restrict", 0) != -1
        name = ("k_rbgs_tile2d_restrict<float> level 0 pre-smoother" if restricting
                else "k_rbgs_tile2d<float> level 0 pre-smoother")
        roof = {"kernel": name, "bound": "hbm", "achieved": sm_bytes / (sm_ms * 1e-3) / 1e9, "peak": hbm_peak,
                "unit": "GB/s", "frac": None, "traffic": ncu_traffic(name), "peak_source": peak_src,
                "launch_ms": sm_ms, "bytes_per_launch": sm_bytes,
                "algorithmic_bytes": "12 B per cell and system: b and 1/diagonal read, x written (FP32); the "
                                     "restricting form also writes the coarse right-hand side, 4 B per coarse "
                                     "cell and system (2 B per cell on the channel's y-halved level 1)"
                                     if restricting else
                                     "12 B per cell and system: b and 1/diagonal read, x written (FP32)",
                "share_of_step": shares["smoother"]["ms_per_step"] / mixed["ms"],
                "levels": {str(k): {"launch_ms": v[0], "achieved_gbs": v[1] / (v[0] * 1e-3) / 1e9}
                           for k, v in smoother.items()}}
        roof["frac"] = roof["achieved"] / roof["peak"]
    configs = bench_configs([c for c in args.configs.split(",") if c], args.config_steps, 2, device, args.c4_train) \
        if args.configs else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_reference(case_fn, args.steps, args.warmup, budget_s=30.0)
        cpu = {"value": r["ncell"] / (r["ms"] * 1e-3) / 1e6, "unit": "Mcells/s", "cores": r["cores"], "kind": "port",
               "sample": f"{r['nrun']} RK3 step(s) of the same case after 1 warm-up step, C restatement with OpenMP",
               "ms_per_step": r["ms"]}
    line = {"metric": METRIC, "value": value, "unit": "Mcells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "paths": {"mixed": {"ms_per_step": mixed["ms"], "max_div_u": mixed["divmax"],
                                "solve_iters_max": mixed["iters"], "solve_residual_max": mixed["residual"],
                                "kinetic_energy": mixed["ke"], "autotuned": mixed["tuned"]},
                      "plain_fp64": {"ms_per_step": plain["ms"], "max_div_u": plain["divmax"],
                                     "solve_iters_max": plain["iters"], "solve_residual_max": plain["residual"],
                                     "kinetic_energy": plain["ke"]},
                      "speedup_mixed_vs_plain": plain["ms"] / mixed["ms"],
                      "learned_mixed": learned,
                      "headline_path": "mixed, with the settings snac_autotune chose after the warm-up (the "
                                       "learned guess is measured beside it and left off: it lowers "
                                       "the starting residual but not the refinement-step count)"},
            "roofline": roof if roof else roof_mom, "roofline_rk_mom": roof_mom,
            "gpu_launches": mixed["launches"], "gpu_launches_per_step": mixed["launches"] / args.steps,
            "kernels": shares,
            "peaks_measured_here": {"fp64_gflops": f64.value, "fp32_gflops": f32.value},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "configs": configs}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
