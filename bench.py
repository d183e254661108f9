#!/usr/bin/env python
"""Benchmark of the GB300 femmd2D timestep (atom-steps/s).

A bench "step" is one System.run(S) call (S leapfrog steps, default 100) on
the workload's synthetic, seeded system -- the reference's run loop
(femmd2D/src/integrator.cpp:31-57): forced neighbour rebuild, initial force
pass, S steps with half-skin rebuilds.  Default workload: the large mixed
system (4096 hex-ring elastomer disks = 520,192 vertices + 1,000,000 LJ
solvent, 1,520,192 atoms), the largest single-GPU configuration, on which the
HBM-roofline target is stated.  Other workloads: suspension (256 disks,
32,512 atoms), lj_fluid (N = 4096).

  value   atom-steps/s with the state resident in HBM: CUDA events on the
          library's stream around the timed run() calls.
  e2e     the same through the C ABI with host buffers: per step the pinned
          host positions+velocities are copied in (femmd_set_state), run(S),
          and positions+velocities copied out (femmd_get_state); wall clock.
  roofline  the step kernel (k_step, the dominant kernel): algorithmic bytes
          per launch / its mean CUDA-event duration from a direct-launch pass,
          against the measured HBM copy bandwidth.
  cpu_baseline  the oracle's CPU restatement (C, OpenMP over the pair loop)
          timed on this host's cores on a bounded sample of the same system.

Multi-GPU (torchrun, one rank per GPU): independent replicas, no collective
on the data path; value = all ranks' atom-steps / max rank time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload large_mixed|suspension|lj_fluid] [--md-steps S]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from femmd_old_gb300 import scene as S  # noqa: E402

WORKLOADS = {
    "large_mixed": ("large mixed: 4096 hex-ring disks (127 vertices, 216 triangles, boundary bonds k=100, E=50, "
                    "nu=0.3) + 1,000,000 LJ solvent (rho=0.8, rc=2.5; vertex pairs WCA), T=1, dt=0.005, skin 0.3",
                    lambda: S.large_mixed()),
    "suspension": ("elastomer suspension: 256 hex-ring disks (127 vertices), E=50, nu=0.3, boundary bonds k=100, "
                   "WCA, phi=0.5, T=0.1, dt=0.002, skin 0.3", lambda: S.suspension()),
    "lj_fluid": ("plain LJ fluid: N=4096, rho=0.8, rc=2.5, skin 0.3, dt=0.005", lambda: S.lj_fluid()),
    "lj_1m": ("plain LJ fluid, the solvent class of the large mixed system: N=1,000,000 (1000x1000 jittered "
              "lattice), rho=0.8, rc=2.5, skin 0.3, dt=0.005, T=1", lambda: S.lj_fluid(n_side=1000)),
}
FORCE_MODES = {"fast": 1, "reference": 0}
# workloads without bonded particles: the fast mode's persistent step and list
# kernels apply (with bonded particles the reference-exact kernels are faster)
UNBONDED = ("lj_fluid", "lj_1m")
AUTO_RULE = "auto: fast mode without bonded particles, reference-exact mode with them"


def resolve_mode(workload, mode):
    """The force mode a workload runs in: 'auto' picks the faster kind."""
    if mode != "auto":
        return mode
    return "fast" if workload in UNBONDED else "reference"
BATCHED_DESC = ("batched ensemble: 512 independent LJ+elastomer replicas, atom counts log-uniform in [500, 20000] "
                "(seed 8), density U(0.6, 0.85) and T U(0.1, 1.5) (seed 9), 90 % solvent + hex-ring disks, "
                "dt=0.005, skin 0.3, one persistent launch per run() under a CUDA graph, autotuned block shape")
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_mixed", choices=sorted(WORKLOADS) + ["batched"])
    ap.add_argument("--md-steps", type=int, default=100)
    ap.add_argument("--force-mode", default="auto", choices=sorted(FORCE_MODES) + ["auto"],
                    help="fast: same sets, forces within 1e-5 of FP64, cell-ordered storage; "
                         "reference: the reference's float operations and list order; "
                         "auto (default): fast without bonded particles, reference otherwise")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--probe", default=None,
                    choices=["midrun_rebuild", "batch_run10", "batch_run10_single", "adjoint", "extras", "lj_1m",
                             "lj_1m_rebuild", "lj_small_rebuild"],
                    help="run one small fixed workload for a profiler capture and exit (no JSON line)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched and adjoint measurements added to the default line")
    return ap.parse_args()


# ------------------------------------------------------------- distributed

# one process per GPU, replicas only (femmd_old_gb300.replicas.Group: NCCL
# barrier and max over ranks; nothing with one process)
def Dist():
    from femmd_old_gb300.replicas import Group
    return Group()


class _Solo:
    """Single-process stand-in for Dist (the extra measurements run on rank 0)."""
    world, rank, local = 1, 0, 0

    def barrier(self):
        pass

    def max(self, x):
        return x

    def sum(self, x):
        return x


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.p = None
        self.out = os.path.join("/tmp", f"femmd_clocks_{os.getpid()}.csv")
        try:
            self.f = open(self.out, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.out):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# --------------------------------------------------------------- CPU side

def cpu_baseline(sc, natoms, budget_s, threads):
    """The oracle's C restatement on this host: a bounded sample of run()."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    o = O.Oracle(image_mode=0, log_mode=0, threads=threads)
    sc.replay(o)
    t0 = time.perf_counter()
    o.run(1)
    t1 = time.perf_counter() - t0
    m = max(1, min(1000, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.run(m)
    dt = time.perf_counter() - t0
    return {"value": natoms * m / dt, "unit": "atom-steps/s", "cores": threads, "kind": "port",
            "sample": f"{m} leapfrog steps (one run({m}) call incl. its initial rebuild and force pass) of the "
                      f"same {natoms}-atom system, {dt:.2f} s wall, oracle/femmd_oracle.c with OpenMP pair loop"}


def reference_arm(args, dist):
    """--impl reference: the reference's CPU path as restated by the oracle
    (the reference's own binary is x86-only here), all host threads.  For the
    batched ensemble the replicas are advanced one after another (the
    reference has no batched form) on a seeded sample of 8 replicas."""
    if dist.rank != 0:
        return None
    if args.workload == "batched":
        desc = BATCHED_DESC
        ens = S.batched_ensemble()
        pick = np.random.Generator(np.random.PCG64(11)).choice(len(ens), size=8, replace=False)
        scenes = [ens[int(r)] for r in sorted(pick)]
    else:
        desc, make = WORKLOADS[args.workload]
        scenes = [make()]
    natoms = sum(int(sc.meta["N"]) for sc in scenes)
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    systems = []
    for sc in scenes:
        o = O.Oracle(image_mode=0, log_mode=0, threads=threads)
        sc.replay(o)
        systems.append(o)
    # every bench step is the repo arm's run(S): one forced rebuild and initial
    # force pass per S leapfrog steps, the same schedule; the number of timed
    # steps is cut so that the whole arm ends within about two minutes
    md = args.md_steps
    t0 = time.perf_counter()
    for o in systems:
        o.run(1)
    per_run = (time.perf_counter() - t0) * md
    steps = max(1, min(args.steps, int(120.0 / max(per_run, 1e-6))))
    warmup = min(args.warmup, 1) if per_run < 30.0 else 0
    for _ in range(warmup):
        for o in systems:
            o.run(md)
    t0 = time.perf_counter()
    for _ in range(steps):
        for o in systems:
            o.run(md)
    dt = time.perf_counter() - t0
    value = natoms * md * steps / dt
    what = (f"{len(scenes)} replicas ({natoms} atoms) each run({md}) in turn" if len(scenes) > 1 else
            f"run({md}) of the {natoms}-atom system")
    return {"metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": steps, "warmup": warmup,
            "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "description": desc, "atoms": natoms, "md_steps_per_step": md,
                       "parallelism": "replicas" if len(scenes) > 1 else "single"},
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{what} per step, {steps} timed steps of the requested {args.steps}; the "
                                       "reference's own binary (oracle/_ref) is built for x86 and cannot run on "
                                       "this host"},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------- GPU arm

def load_traffic(kernel, workload):
    """DRAM bytes per launch of the step kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def step_kernel_bytes(s, sc):
    """Algorithmic HBM bytes of one step-kernel launch, by the contract's
    per-unit figure: per atom B_state 48 (pos, vel, acc read and written) +
    B_param 8 (mass, type) + 4 (1 + n̄) (list count and entries); per
    elastomer triangle 32 (3 indices + Bm + A0) and per bond 16 (two
    incidences of 8).  Neighbour and partner gathers count as cache hits.
    Also returned: the kernel's own minimum in the steady state (pos in/out,
    vel in/out, mass, count: 40 per atom, + 4 type with several types, 4 per
    entry; per vertex 8 incidence starts, 16 per bond, 36 per triangle
    incidence), which the fused kick-drift-kick meets without acc traffic."""
    n = s.N
    st = s.nn_stats()
    c = s.counts()
    nb = st["mean_neighbors"]
    contract = (48 + 8 + 4 * (1 + nb)) * n + 32 * c["triangles"] + 16 * c["bonds"]
    per = 40 + (4 if sc.meta.get("types", 1) > 1 else 0)
    nbonded = s._vertex_count()
    minimum = per * n + 4 * nb * n + 8 * nbonded + 8 * 2 * c["bonds"] + 12 * 3 * c["triangles"]
    return contract, minimum, st


SMALL_RUN_MAX_ATOMS = 128 * 128  # 128 step blocks of 128 slots


def small_run_path(sc, n, bonded):
    """Whether run() advances its middle steps in the cooperative small-system
    run (k_fsmall) in the fast mode: one particle kind, no bonded particles,
    walls, gravity or area springs, an XY-periodic box, at most 128 step
    blocks (the library's small_run_fits, as far as a scene shows it)."""
    names = {nm for nm, a in sc.calls}
    pbc = [a[0] for nm, a in sc.calls if nm == "PBC"]
    return (not bonded and n <= SMALL_RUN_MAX_ATOMS and sc.meta.get("types", 1) == 1 and pbc and pbc[-1] == 2
            and not names & {"set_moving_wall", "set_gravity", "set_kArea"})


def ours(args, dist):
    import femmd_old_gb300 as F
    desc, make = WORKLOADS[args.workload]
    sc = make()
    sc.meta["types"] = max([a[0] for nm, a in sc.calls if nm == "set_numTypes"] or [1])
    dev = dist.local
    mode = resolve_mode(args.workload, args.force_mode)
    s = F.System(dev)
    s.set_force_mode(FORCE_MODES[mode])
    sc.replay(s)
    n = s.N
    md = args.md_steps
    s.run(0)
    for _ in range(args.warmup):
        s.run(md)
    flush = None
    try:
        import torch
        torch.cuda.set_device(dev)
        working = n * (8 * 5 + 4 * 24 + 16 + 8)
        if working < 2 * L2_BYTES:
            flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{dev}")
    except Exception:
        torch = None

    # ---- timed region: state resident in HBM
    dist.barrier()
    s.sync()
    clk = ClockSampler(dev)
    t_ms = 0.0
    rebuilds = 0
    for k in range(args.steps):
        if flush is not None:
            flush.zero_()
            torch.cuda.synchronize()
        s.event_record(0)
        s.run(md)
        s.event_record(1)
        t_ms += s.event_elapsed_ms(0, 1)
        rebuilds += s.total_updates() - 1
    s.sync()
    clocks = clk.stop()
    dist.barrier()
    t_max = dist.max(t_ms)
    units = n * md * args.steps * dist.world
    value = units / (t_max / 1e3)
    nst = s.nn_stats()

    # kernel launches inside the timed region
    has_tri = 1 if s.counts()["triangles"] else 0
    bonded = s._vertex_count() > 0
    small = mode == "fast" and small_run_path(sc, n, bonded)
    if mode != "fast":
        rebuild_kernels = 7  # k_rebuild_begin, count, scan x2, scatter, cell sort, list build
    elif not bonded and n <= SMALL_RUN_MAX_ATOMS:
        rebuild_kernels = 2  # k_fbin_small (binning and placement in one block), k_flist_p
    elif not bonded:
        rebuild_kernels = 7  # k_rebuild_begin, count, scan x2, scatter, k_fplace, k_flist_p
    else:
        rebuild_kernels = 10  # + k_ffree_count, k_fperm, k_fwindows, k_flist in place of k_flist_p
    if small:
        # run start, its forced rebuild, the first step, one k_fsmall (the
        # middle steps and their rebuilds in one cooperative launch), the last step
        launches = args.steps * (1 + rebuild_kernels + 3)
    else:
        launches = args.steps * (1 + rebuild_kernels + (md + 1) * (1 + has_tri)) + rebuild_kernels * rebuilds

    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    if torch is not None:
        pos = torch.empty((n, 2), dtype=torch.float32, pin_memory=True)
        vel = torch.empty((n, 2), dtype=torch.float32, pin_memory=True)
        s.get_state_ptr(pos.data_ptr(), vel.data_ptr())
        dist.barrier()
        s.sync()
        t0 = time.perf_counter()
        for k in range(args.steps):
            s.set_state_ptr(pos.data_ptr(), vel.data_ptr())
            s.run(md)
            s.get_state_ptr(pos.data_ptr(), vel.data_ptr())
        s.sync()
        dt = time.perf_counter() - t0
        dist.barrier()
        dt = dist.max(dt)
        e2e = {"value": units / dt, "unit": "atom-steps/s", "h2d_bytes_per_step": 16 * n,
               "d2h_bytes_per_step": 16 * n}

    # ---- roofline of the step kernel: direct launches with events
    s.set_profiling(True)
    for k in range(max(1, min(3, args.steps))):
        s.run(md)
    prof = s.profile()
    s.set_profiling(False)
    kbytes, kmin, st = step_kernel_bytes(s, sc)
    kms = prof["force_ms"] / max(prof["force_launches"], 1)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = kbytes / (kms / 1e3) / 1e9
    fast = mode == "fast"
    kname = ("k_fstep" if bonded else "k_fstep_p") if fast else "k_step"
    traffic = load_traffic(kname, args.workload)
    what = ("fast mode: cell-ordered storage, windows in shared memory, fused multiply-adds, hardware "
            "reciprocal" + ("" if bonded else "; persistent, a producer warp stages list rows and windows by "
                            "bulk asynchronous copies, packed float2 pair arithmetic")
            if fast else "reference-exact arithmetic and list order")
    if small:
        what += ("; timed by its own direct launches: inside run() the middle steps and their rebuilds run in "
                 "k_fsmall, one cooperative launch with the same pair arithmetic")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic,
                "kernel": f"{kname} (fused LJ+bond+triangle gather, leapfrog, fixed-point energy sums; {what})",
                "algorithmic_bytes_per_launch": kbytes, "kernel_minimum_bytes_per_launch": kmin,
                "bytes_rule": "contract per-unit figure: 48 + 8 + 4 (1 + mean list) per atom, 32 per triangle, "
                              "16 per bond", "mean_launch_ms": kms,
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(make(), n, args.cpu_seconds, os.cpu_count() or 1)

    rb_per_run = rebuilds / max(args.steps, 1)
    kbar = md / max(rb_per_run, 1e-9) if rebuilds else None
    # the contract's whole-job figure: atom-steps/s x bytes per atom-step, the
    # rebuild's bytes (pos read, cell key and order, count, list write) spread
    # over the steps between rebuilds
    nb = nst["mean_neighbors"]
    cnt = s.counts()
    b_atom = 48 + 8 + 4 * (1 + nb) + ((8 + 12 + 4 + 4 * nb) / kbar if kbar else 0.0)
    b_atom += (32 * cnt["triangles"] + 16 * cnt["bonds"]) / max(n, 1)
    job = value * b_atom / 1e9
    roofline_job = {"achieved": job, "peak": peak, "unit": "GB/s", "frac": job / peak,
                    "bytes_per_atom_step": b_atom, "mean_list": nb, "steps_between_rebuilds": kbar,
                    "rule": "atom-steps/s x (56 + 4 (1 + n) + (24 + 4 n) / k + elastomer bytes per atom)"}
    line = {"metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": args.workload, "description": desc, "atoms": n, "md_steps_per_step": md,
                       "neighbors_mean": nst["mean_neighbors"], "steps_between_rebuilds": kbar,
                       "parallelism": "replicas" if dist.world > 1 else "single",
                       "l2": "L2 flushed between timed steps" if flush is not None else
                             "inputs larger than L2 (state + lists > 129 MB)",
                       "image_mode": "exact", "fea_law": "neo-Hookean", "force_mode": mode,
                       "force_mode_rule": AUTO_RULE if args.force_mode == "auto" else "requested"},
            "roofline": roofline, "roofline_job": roofline_job, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clocks}
    return line


def batched(args, dist):
    """The ensemble advanced by femmd_batch_run (one persistent launch per
    run() call), next to the same replicas advanced one by one through the
    plain path (System.run per replica), on the same total atom count."""
    import femmd_old_gb300 as F
    import torch
    dev = dist.local
    torch.cuda.set_device(dev)
    # several ranks split the ensemble (strong scaling: the total is fixed)
    scenes = ensemble_share(S.batched_ensemble(), dist.world, dist.rank)
    systems = []
    b = F.Batch(dev)
    for sc in scenes:
        s = F.System(dev)
        sc.replay(s)
        systems.append(s)
        b.add(s)
    natoms = sum(s.N for s in systems)
    md = args.md_steps
    b.run(0)
    tune = b.autotune(20)
    for _ in range(args.warmup):
        b.run(md)
    launch = b.launch()

    dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(dev)
    t_ms = 0.0
    for k in range(args.steps):
        b.event_record(0)
        b.run(md)
        b.event_record(1)
        t_ms += b.event_elapsed_ms(0, 1)
    torch.cuda.synchronize()
    clocks = clk.stop()
    dist.barrier()
    t_max = dist.max(t_ms)
    natoms_all = int(dist.sum(natoms))
    value = natoms_all * md * args.steps / (t_max / 1e3)
    rebuilds = sum(s.total_updates() for s in systems)

    # end to end: every replica's positions and velocities in from pinned host
    # memory and out again around each batched run()
    host = [(torch.empty((s.N, 2), dtype=torch.float32, pin_memory=True),
             torch.empty((s.N, 2), dtype=torch.float32, pin_memory=True)) for s in systems]
    for s, (hp, hv) in zip(systems, host):
        s.get_state_ptr(hp.data_ptr(), hv.data_ptr())
    dist.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        for s, (hp, hv) in zip(systems, host):
            s.set_state_ptr(hp.data_ptr(), hv.data_ptr())
        b.run(md)
        for s, (hp, hv) in zip(systems, host):
            s.get_state_ptr(hp.data_ptr(), hv.data_ptr())
    torch.cuda.synchronize()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e = {"value": natoms_all * md * args.steps / e2e_s, "unit": "atom-steps/s",
           "h2d_bytes_per_step": 16 * natoms_all, "d2h_bytes_per_step": 16 * natoms_all}

    # the plain form on the same replicas: one System.run per replica
    md_plain = max(1, min(md, 100))
    t0 = time.perf_counter()
    for s in systems:
        s.run(md_plain)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain_value = natoms * md_plain / plain_s

    # the plain form on one system of the same total atom count (LJ fluid,
    # rho = 0.8, rc = 2.5, the plain-LJ composition scaled up)
    side = int(round(math.sqrt(natoms)))
    big = F.System(dev)
    S.lj_fluid(n_side=side).replay(big)
    big.run(0)
    big.run(md)
    big_ms = []
    for k in range(max(1, min(args.steps, 3))):
        big.event_record(0)
        big.run(md)
        big.event_record(1)
        big_ms.append(big.event_elapsed_ms(0, 1))
    single_value = side * side * md / (statistics.median(big_ms) / 1e3)
    del big
    # and one system of the ensemble's composition (2025 hex-ring disks, about
    # 10 % of the atoms, in LJ solvent at rho 0.8) with the same atom count
    mix = F.System(dev)
    mixed_scene = S.large_mixed(n_side=45, n_solvent=natoms - 45 * 45 * 127)
    mixed_scene.replay(mix)
    mix.run(0)
    mix.run(md)
    mix_ms = []
    for k in range(max(1, min(args.steps, 3))):
        mix.event_record(0)
        mix.run(md)
        mix.event_record(1)
        mix_ms.append(mix.event_elapsed_ms(0, 1))
    mixed_value = mix.N * md / (statistics.median(mix_ms) / 1e3)
    mixed_atoms = mix.N
    del mix

    # the tuner's search over rebuild cadence (skin) and cell size (cell
    # factor): it changes rounding, not physics, and is reported beside the
    # reference-exact figure
    tuned = b.autotune_lists(20, skins=(0.3, 0.45, 0.6), factors=(1.0, 1.2, 1.5))
    for _ in range(2):
        b.run(md)
    tms = []
    for k in range(max(1, min(args.steps, 3))):
        b.event_record(0)
        b.run(md)
        b.event_record(1)
        tms.append(b.event_elapsed_ms(0, 1))
    tuned_value = natoms * md / (statistics.median(tms) / 1e3)

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        # one mid-sized replica on the host, scaled by atoms
        mid = sorted(range(len(scenes)), key=lambda r: scenes[r].meta["N"])[len(scenes) // 2]
        cpu = cpu_baseline(scenes[mid], int(scenes[mid].meta["N"]), args.cpu_seconds, os.cpu_count() or 1)
        cpu["sample"] = "median-size replica: " + cpu["sample"]
    launches_per_run = 1
    return {"metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
            "higher_is_better": True, "scaling": "strong" if dist.world > 1 else "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched", "description": BATCHED_DESC, "replicas": len(S.batched_ensemble()),
                       "replicas_this_rank": len(systems), "atoms": natoms_all, "md_steps_per_step": md,
                       "launch": launch, "autotune": tune, "rebuilds_last_run": rebuilds,
                       "parallelism": f"replicas split over {dist.world} ranks" if dist.world > 1 else "single",
                       "l2": "inputs larger than L2 (512 replicas' state + lists > 129 MB)"},
            "plain_same_atoms": {"value": plain_value, "unit": "atom-steps/s", "md_steps": md_plain,
                                 "how": "System.run on each replica in turn, wall clock"},
            "plain_single_system": {"value": single_value, "unit": "atom-steps/s", "atoms": side * side,
                                    "how": f"one LJ fluid of {side}x{side} atoms (rho 0.8, rc 2.5), run({md}), "
                                           "CUDA events"},
            "plain_single_system_same_mix": {"value": mixed_value, "unit": "atom-steps/s", "atoms": mixed_atoms,
                                             "how": "one system of 2025 hex-ring disks in LJ solvent (rho 0.8), "
                                                    f"run({md}), CUDA events"},
            "batched_tuned_lists": {"value": tuned_value, "unit": "atom-steps/s", "skin": tuned["skin"],
                                    "cell_factor": tuned["cell_factor"],
                                    "note": "opt-in skin/cell-size tuning: same physics, other rounding"},
            "batched_over_plain": value / plain_value,
            "batched_over_single_system": value / single_value,
            "batched_over_single_system_same_mix": value / mixed_value,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches_per_run * args.steps, "clocks": clocks}


def adjoint_ratio(dev, reps=3, steps=200, every=20):
    """Config 5: wall time of femmd_adjoint_backward (recompute of every
    checkpoint segment + reverse steps) over femmd_adjoint_forward (the same
    200 steps as run(20) segments with checkpoints), each call synchronous;
    a fresh system per repetition."""
    import femmd_old_gb300 as F
    sc = S.compression(steps=steps)
    fw, bw, plain = [], [], []
    for r in range(reps + 1):
        s = F.System(dev)
        sc.replay(s)
        s.run(0)
        t0 = time.perf_counter()
        s.adjoint_forward(steps, every)
        t1 = time.perf_counter()
        s.adjoint_backward()
        t2 = time.perf_counter()
        p = F.System(dev)
        sc.replay(p)
        p.run(0)
        p.sync()
        t3 = time.perf_counter()
        p.run(steps)
        p.sync()
        t4 = time.perf_counter()
        if r:  # the first repetition builds graphs and buffers
            fw.append(t1 - t0)
            bw.append(t2 - t1)
            plain.append(t4 - t3)
    f, b, pl = statistics.median(fw), statistics.median(bw), statistics.median(plain)
    return {"workload": "compression: 64 hex-ring disks (8128 vertices), XPBC, harmonic top wall k=100 moving "
                        "2% of L in 200 steps, per-disk E~U(20,80), nu~U(0.2,0.45), dt=0.002",
            "steps": steps, "checkpoint_every": every, "forward_ms": 1e3 * f, "backward_ms": 1e3 * b,
            "plain_run_ms": 1e3 * pl, "adjoint_over_forward": b / f, "adjoint_over_plain_run": b / pl,
            "observable": "mean wall stress + FEA energy at the final step",
            "gradients": "initial positions and velocities, per-disk E and nu, log eps, log sigma"}


# ------------------------------------------------------------------ probes
#
# Small fixed workloads for profiler captures (the commands in profiles/):
# each runs once on cuda:0, prints "ok" and no JSON line.

def probe(name, mode="fast"):
    import femmd_old_gb300 as F
    import torch
    if name == "midrun_rebuild":
        # one neighbour rebuild of the large mixed system after 200 steps,
        # inside the NVTX range "midrun", then run(12) launched directly
        s = F.System()
        s.set_force_mode(FORCE_MODES[mode])
        S.large_mixed().replay(s)
        s.run(0)
        s.run(200)
        s.sync()
        torch.cuda.nvtx.range_push("midrun")
        s.build_nn()
        s.set_profiling(True)
        s.run(12)
        s.sync()
        torch.cuda.nvtx.range_pop()
    elif name in ("batch_run10", "batch_run10_single"):
        # the 512-replica ensemble, run(0) then run(10) in one launch each:
        # 1024 threads x 2 CTAs per SM with the heaviest replicas on CTA
        # pairs, or 1024 x 1 with every replica on one CTA
        b = F.Batch(0)
        keep = []
        for sc in S.batched_ensemble():
            s = F.System(0)
            sc.replay(s)
            keep.append(s)
            b.add(s)
        if name == "batch_run10":
            b.set_launch(1024, 2)
        else:
            b.set_launch(1024, 1)
            b.set_split(False)
        b.run(0)
        b.run(10)
        keep[0].sync()
    elif name == "lj_1m":
        # the 1M-atom LJ fluid in the force mode of --force-mode: run(0),
        # run(50), then run(12) launched directly (no graph) inside the NVTX
        # range "steps"
        s = F.System()
        s.set_force_mode(FORCE_MODES[mode])
        S.lj_fluid(n_side=1000).replay(s)
        s.run(0)
        s.run(50)
        s.sync()
        torch.cuda.nvtx.range_push("steps")
        s.set_profiling(True)
        s.run(12)
        s.sync()
        torch.cuda.nvtx.range_pop()
    elif name == "lj_1m_rebuild":
        # three full neighbour rebuilds of the 1M-atom LJ fluid after run(50),
        # in the force mode of --force-mode, inside the NVTX range "rebuild"
        s = F.System()
        s.set_force_mode(FORCE_MODES[mode])
        S.lj_fluid(n_side=1000).replay(s)
        s.run(0)
        s.run(50)
        s.sync()
        torch.cuda.nvtx.range_push("rebuild")
        for _ in range(3):
            s.build_nn()
        s.sync()
        torch.cuda.nvtx.range_pop()
    elif name == "lj_small_rebuild":
        # three full neighbour rebuilds of config 1 (4096 LJ atoms) after
        # run(200), in the force mode of --force-mode, inside the NVTX range
        # "rebuild" (the fast mode's one-block binning and list build)
        s = F.System()
        s.set_force_mode(FORCE_MODES[mode])
        S.lj_fluid().replay(s)
        s.run(0)
        s.run(200)
        s.sync()
        torch.cuda.nvtx.range_push("rebuild")
        for _ in range(3):
            s.build_nn()
        s.sync()
        torch.cuda.nvtx.range_pop()
    elif name == "adjoint":
        # config 5: forward with checkpoints every 20 steps, then the backward
        c = F.System()
        S.compression().replay(c)
        c.run(0)
        c.adjoint_forward(200, 20)
        c.adjoint_observable()
        c.adjoint_backward()
        c.sync()
    elif name == "extras":
        # area springs (kArea 0.3) on the large mixed system: run(4), the
        # observables, the cluster getter and three averaged steps; then the
        # compression case through adjoint_forward(40, 20) and the backward
        sc = S.large_mixed()
        calls = []
        for n, a in sc.calls:
            calls.append((n, a))
            if n == "set_elastomer_bonds":
                calls.append(("set_kArea", (0.3,)))
        s = F.System()
        S.Scene(calls=calls, meta=sc.meta).replay(s)
        s.run(0)
        s.run(4)
        s.properties()
        s.clusters()
        s.set_property_averaging(True, 5, 0)
        s.run(3)
        s.sync()
        del s
        c = F.System()
        S.compression().replay(c)
        c.adjoint_forward(40, 20)
        c.adjoint_observable()
        c.adjoint_backward()
        c.sync()
    else:
        raise SystemExit(f"unknown probe {name}")
    print("ok", flush=True)


def relaunch_cmd(gpus, argv):
    """The command that runs this bench as one process per GPU (torchrun on
    the loopback rendezvous with a free port)."""
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
            "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + list(argv)


def ensemble_share(scenes, world, rank):
    """The replicas of an ensemble one rank advances: the atom counts split
    over the ranks heaviest first (replicas.partition), the same split on
    every rank without communication."""
    from femmd_old_gb300.replicas import partition
    if world <= 1:
        return list(scenes)
    mine = partition([int(sc.meta["N"]) for sc in scenes], world)[rank]
    return [scenes[i] for i in sorted(mine)]


def main():
    args = parse()
    if args.probe:
        probe(args.probe, "fast" if args.force_mode == "auto" else args.force_mode)
        return
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: launch the ranks here when no launcher did
        raise SystemExit(subprocess.call(relaunch_cmd(args.gpus, sys.argv[1:])))
    dist = Dist()
    try:
        if args.impl == "reference":
            line = reference_arm(args, dist)
        elif args.workload == "batched":
            line = batched(args, dist)
        else:
            line = ours(args, dist)
            if dist.rank == 0 and args.workload == "large_mixed" and not args.no_extras:
                dev = dist.local
                # the 1M-atom LJ fluid (the solvent class, where the HBM-roofline
                # target is stated) and the headline system in the other force mode
                keep = ("value", "unit", "ms_per_step", "roofline", "roofline_job", "e2e", "gpu_launches", "clocks")
                main_mode = resolve_mode("large_mixed", args.force_mode)
                for key, wl, mode in (("lj_1m", "lj_1m", resolve_mode("lj_1m", args.force_mode)),
                                      ("other_mode", "large_mixed", "reference" if main_mode == "fast" else "fast"),
                                      ("lj_fluid", "lj_fluid", resolve_mode("lj_fluid", args.force_mode)),
                                      ("suspension", "suspension", resolve_mode("suspension", args.force_mode))):
                    sub = argparse.Namespace(**vars(args))
                    sub.workload, sub.force_mode = wl, mode
                    sub.steps, sub.warmup, sub.no_cpu_baseline = max(3, min(args.steps, 10)), 3, True
                    r = ours(sub, _Solo())
                    line[key] = {k: r[k] for k in keep}
                    line[key]["config"] = r["config"]
                line["adjoint"] = adjoint_ratio(dev)
                sub = argparse.Namespace(**vars(args))
                sub.steps, sub.warmup, sub.md_steps, sub.no_cpu_baseline = 3, 3, 100, True
                b = batched(sub, _Solo())
                line["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "plain_same_atoms",
                                                     "plain_single_system", "plain_single_system_same_mix",
                                                     "batched_tuned_lists",
                                                     "batched_over_plain", "batched_over_single_system",
                                                     "batched_over_single_system_same_mix", "e2e", "clocks")}
                line["batched"]["config"] = {k: b["config"][k] for k in ("description", "replicas", "atoms",
                                                                         "md_steps_per_step", "launch")}
        if dist.rank == 0 and line is not None:
            print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
