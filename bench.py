#!/usr/bin/env python
"""Benchmark of the contact hot path on GB300.

Workload (N=1): the 256-scene batch -- 256 uneven two-sheet scenes (grid side
log-uniform in [16, 256], 5,911,266 vertices in all; per-scene dhat
log-uniform in [1e-4, 1e-2], gap U(0.2, 0.9) dhat, stiffness 1e4) --
seeded synthetic data (numpy PCG64, seed 3).  One step = BarrierPotential
energy + gradient + PSD-projected (CLAMP) Hessian with CSR assembly of every
scene over the prebuilt collision sets (76.6 M contacts), in one batched call
(SceneBatch, mixed FP32/FP64: every contact but near-parallel edge-edge ones
computes its distance derivatives in FP32; the PSD eigen-projection, the
mollifier and assembly are FP64), replayed as one CUDA graph.

    value   contacts/s of the batched call, positions resident in HBM
    e2e     the same call through the public API with host positions (pinned)
            copied in and the per-scene energies and the gradient copied out
            every step; the Hessian stays on the device (DeviceCSR)
    plain   the same work as the reference is used: one CollisionMesh and
            one FP64 energy + gradient + Hessian call per scene
    roofline  the dominant kernel's FP64 rate (ncu flop count per launch over
            its CUDA-event launch time) against the measured cuBLAS DGEMM
            rate, and its algorithmic HBM bytes per launch against the
            measured copy bandwidth
    cpu_baseline  the CPU restatement (oracle/) on this host's cores, on a
            bounded sample of the same scenes

--impl reference times the reference algorithm on the host cores (the CPU
restatement under oracle/, since the reference itself cannot be built here)
on that sample and prints the same line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ipc-toolkit_gb300")
sys.path.insert(0, PKG)

METRIC = "barrier E+grad+Hess contacts/s"
UNIT = "contacts/s"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-legs", action="store_true",
                    help="skip the legs beside the headline (served, layered cloth, friction, sphere pack)")
    ap.add_argument("--profile-case", choices=["egh", "ccd"],
                    help="for ncu captures: a 24-scene batch of the headline's distribution (sides 48-96, seed 5), "
                         "one energy/gradient/Hessian call per mode of --modes (egh) or two batched step sizes (ccd); "
                         "prints one line, times nothing")
    ap.add_argument("--modes", default="local,local_df64", help="precision modes of --profile-case egh")
    return ap.parse_args()


def run_profile_case(args):
    import torch
    import ipctk_gb300 as ipctk
    from ipctk_gb300 import scenes
    scs = scenes.batch(n_scenes=24, side_lo=48, side_hi=96, seed=5)
    batch = ipctk.SceneBatch([(s["V"], s["E"], s["F"]) for s in scs])
    Vd = torch.from_numpy(batch.pack([s["V"] for s in scs])).cuda()
    dh = np.array([s["dhat"] for s in scs])
    kap = np.array([s["kappa"] for s in scs])
    out = {"case": args.profile_case, "scenes": len(scs)}
    if args.profile_case == "egh":
        col = ipctk.NormalCollisions()
        col.build(batch, Vd, dh)
        out["contacts"] = len(col)
        for mode in args.modes.split(","):
            BB = ipctk.BatchBarrierPotential(dh, kap, mixed_precision=mode)
            e, g, H = BB.evaluate(col, batch, Vd, energy=True, gradient=True, hessian=True,
                                  project_hessian_to_psd=ipctk.PSDProjectionMethod.CLAMP, device=True)
            torch.cuda.synchronize()
            H.free()
            out[mode] = float(np.sum(e))
    else:
        V1d = torch.from_numpy(batch.pack([s["V1"] for s in scs])).cuda()
        for _ in range(2):
            steps = ipctk.compute_collision_free_stepsize_batch(batch, Vd, V1d)
            torch.cuda.synchronize()
        out["steps"] = [float(x) for x in steps[:4]]
    print(json.dumps(out), flush=True)


BATCH_DESC = ("256 uneven two-sheet scenes (5,911,266 verts; side log-uniform [16, 256], dhat log-uniform "
              "[1e-4, 1e-2], gap U(0.2, 0.9) dhat, stiffness 1e4; seed 3)")
BATCH_CONTACTS = 76_649_164  # merged collisions of the batch (oracle and GPU agree)
# the headline's precision: FP32 distance derivatives and barrier terms for
# every contact but near-parallel edge-edge ones, FP64 PSD eigen-projection
HEADLINE_MODE = "local"
PRECISION = {
    "local": "mixed: FP32 distance derivatives and barrier terms except near-parallel edge-edge and degenerate "
             "point-triangle; FP64 PSD eigen-projection, mollifier, assembly",
    "fp64": "FP64 throughout",
    "psd_df64": "FP64 local Hessians; PSD eigenpairs in df64 (pairs of FP32), contrasts and correction FP64",
    "local_df64": "the mixed mode with the PSD eigenpairs in df64",
}


def ranks_max(x, device):
    """The largest of every rank's x (the job's time is its slowest rank's),
    once all ranks have arrived; x itself with one process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def ranks_sum(n, device):
    """The units all ranks processed (each replica its own batch)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return int(n)
    t = torch.tensor([int(n)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())


def batch_config(contacts=BATCH_CONTACTS):
    """The config dict both arms print (same keys, same workload)."""
    return {"workload": BATCH_DESC, "contacts": contacts, "psd": "clamp", "scenes": 256,
            "l2": "inputs larger than L2 (5.9 M vertices; ~80 GB of Hessian slots per step)",
            "parallelism": "single"}


def cpu_sample(scs, vertex_budget=40_000):
    """A bounded, deterministic sample of the batch for the CPU arms: every
    8th scene (by index) whose vertex count fits the running budget."""
    out, tot = [], 0
    for k in range(0, len(scs), 8):
        nv = scs[k]["V"].shape[0]
        if tot + nv <= vertex_budget:
            out.append(k)
            tot += nv
    return out


def make_scene(name):
    from ipctk_gb300 import scenes
    if name == "sphere_pack":
        return scenes.sphere_pack(), "sphere_pack 512 icospheres x 642 verts (328,704 verts, 655,360 tris)"
    if name == "two_sheet":
        return scenes.two_sheet(), "two_sheet 2 x 64x64 grid (8,192 verts, 15,876 tris)"
    return scenes.layered_cloth(), "layered_cloth 8 x 256x256 (524,288 verts)"


# algorithmic bytes per contact of one E+G+H pass: positions + ids + weight
# in, gradient contribution + Hessian values + CSR column indices out
BYTES_PER_CONTACT = {2: 504, 3: 1104, 4: 1944}


# per contact, the PSD pass reads and writes its 3n x 3n local Hessian slab
PSD_BYTES = {2: 2 * 8 * 36, 3: 2 * 8 * 81, 4: 2 * 8 * 144}


def psd_bytes(counts):
    nvv, nev, nee, nfv = (int(x) for x in counts[:4])
    return nvv * PSD_BYTES[2] + nev * PSD_BYTES[3] + (nee + nfv) * PSD_BYTES[4]


def fp64_peak_tflops(dev):
    """Measured FP64 rate: cuBLAS DGEMM (4096^3) through torch, best of 3."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1000.0)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def algorithmic_bytes(counts, ndof):
    nvv, nev, nee, nfv = (int(x) for x in counts[:4])
    b = nvv * BYTES_PER_CONTACT[2] + nev * BYTES_PER_CONTACT[3] + (nee + nfv) * BYTES_PER_CONTACT[4]
    b += nee * 9  # eps_x + dtype
    b += 8 * (ndof + 1)  # CSR row pointers
    return b


def ccd_candidate_count(ipctk, mesh, V0, V1, strict=False):
    """Broad-phase candidate count of one compute_collision_free_stepsize call
    (the C ABI's n_candidates output), or None if it cannot be read."""
    try:
        import ctypes
        d = ipctk.DEFAULT_NARROW_PHASE_CCD
        step, count = np.zeros(1), np.zeros(1, np.int64)
        ipctk._check(ipctk._load().ipcg_collision_free_stepsize(
            mesh._h, ipctk._ptr(V0), ipctk._ptr(V1), 0.0, d.tolerance, int(d.max_iterations),
            d.conservative_rescaling, step.ctypes.data_as(ctypes.c_void_p), count.ctypes.data_as(ctypes.c_void_p)))
        return int(count[0])
    except Exception:
        if strict:
            raise
        return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling around the timed region.

    Rows are timestamped on arrival; start() returns once the first row is in
    (nvidia-smi takes a moment to start), and stop() keeps the rows that
    arrived inside the window given by mark() (the timed region), or the first
    row after its start when the region is shorter than the sampling interval."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 50

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None
        self.window = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", str(self.INTERVAL_MS)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t0 = time.perf_counter()
        while not self.rows and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def mark(self, t_begin, t_end):
        self.window = (t_begin, t_end)

    def stop(self):
        if self.window is not None:
            # let the row that covers the end of the window arrive
            time.sleep(2 * self.INTERVAL_MS / 1000.0)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)
        rows = [r for _, r in self.rows]
        if self.window is not None and self.rows:
            lo, hi = self.window
            inside = [r for t, r in self.rows if lo <= t <= hi + self.INTERVAL_MS / 1000.0]
            after = [r for t, r in self.rows if t >= lo]
            rows = inside or after[:1] or rows[-1:]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "interval_ms": self.INTERVAL_MS}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_counts(kernel, workload):
    """Per-launch DRAM bytes and FP64 flops of `kernel` on `workload` from the
    committed ncu summary (profiles/ncu_counts.json), or {}."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_counts.json")) as f:
            t = json.load(f)
        return t.get(workload, {}).get(kernel, {})
    except Exception:
        return {}


def cpu_baseline_run(scenes_list, steps, budget_s=20.0, warmup=0, desc=None):
    """Time the CPU restatement (oracle/) on this host: E + grad + PSD Hessian
    with CSR assembly over each scene's prebuilt collision set, all host
    threads, after `warmup` untimed passes.  One pass = every scene once."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    nt = os.cpu_count() or 1
    built = [(sc, oracle.build_collisions(sc["V"], sc["E"], sc["F"], sc["dhat"], nthreads=nt)) for sc in scenes_list]
    C = sum(len(col) for _, col in built)

    def one_pass():
        for sc, col in built:
            V, E, F = sc["V"], sc["E"], sc["F"]
            oracle.barrier_energy(col, V, E, F, sc["dhat"], sc["kappa"], nthreads=nt)
            oracle.barrier_gradient(col, V, E, F, sc["dhat"], sc["kappa"], nthreads=nt)
            oracle.barrier_hessian(col, V, E, F, sc["dhat"], sc["kappa"], psd="clamp", nthreads=nt)

    for _ in range(warmup):
        one_pass()
    times = []
    t_start = time.perf_counter()
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        one_pass()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s:
            break
    med = statistics.median(times)
    sample = desc or f"{len(scenes_list)} scenes"
    return {"value": C / med, "unit": UNIT, "cores": nt, "kind": "port",
            "sample": f"{sample}: {C} contacts per pass, {len(times)} passes, median"}, C, times


def ccd_baseline_run(sc, budget_s=20.0):
    """compute_collision_free_stepsize of the CPU restatement on all host
    threads (median of up to 3 runs within the budget)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    nt = os.cpu_count() or 1
    times = []
    t_start = time.perf_counter()
    step = None
    for _ in range(3):
        t0 = time.perf_counter()
        step, _ = oracle.collision_free_stepsize(sc["V"], sc["V1"], sc["E"], sc["F"], nthreads=nt)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s:
            break
    med = statistics.median(times)
    return {"steps_per_s": 1.0 / med, "ms": 1000 * med, "cores": nt, "kind": "port", "step_size": step,
            "sample": f"full scene, {len(times)} runs, median"}


def run_reference(args, rank):
    if rank != 0:
        return
    from ipctk_gb300 import scenes
    scs = scenes.batch()
    idx = cpu_sample(scs)
    desc = f"scenes {idx} of the 256-scene batch"
    warm = max(0, args.warmup)
    # each step is one pass over the sample; the timed passes stop after 120 s
    base, C, times = cpu_baseline_run([scs[k] for k in idx], args.steps, budget_s=120.0, warmup=min(warm, 1),
                                      desc=desc)
    ms = 1000 * statistics.median(times)
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": len(times), "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded numpy PCG64 scenes; the reference publishes no dataset for this path)",
            "config": batch_config(),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def timed_host(fn, n_warm, n_steps):
    """Wall-clock ms of n_steps calls of fn (each ends synchronised)."""
    import torch
    for _ in range(n_warm):
        fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(n_steps):
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        out.append(1000 * (time.perf_counter() - t0))
    return out


def plain_leg(dev, scs, warmup=1, steps=2):
    """The plain FP64 form on the batch, as the reference is used: one
    CollisionMesh, one collision set and one fused FP64 energy + gradient +
    CLAMP Hessian call per scene (device-resident positions), then one
    compute_collision_free_stepsize per scene."""
    import gc
    import torch
    import ipctk_gb300 as ipctk
    CLAMP = ipctk.PSDProjectionMethod.CLAMP
    plain = []
    for s in scs:
        m = ipctk.CollisionMesh(s["V"], s["E"], s["F"])
        Vd = torch.from_numpy(s["V"]).to(dev)
        V1d = torch.from_numpy(s["V1"]).to(dev)
        c = ipctk.NormalCollisions()
        c.build(m, Vd, s["dhat"])
        plain.append((s, m, Vd, V1d, c, ipctk.BarrierPotential(s["dhat"], s["kappa"])))
    C = sum(len(p[4]) for p in plain)

    def egh():
        for s, m, Vd, V1d, c, B in plain:
            B.energy_gradient_hessian_device(c, m, Vd, CLAMP)[2].free()

    l0 = ipctk.launch_count()
    t = timed_host(egh, warmup, steps)
    launches = (ipctk.launch_count() - l0) / (warmup + steps)
    steps_out = []
    t_ccd = timed_host(lambda: steps_out.append(
        [ipctk.compute_collision_free_stepsize(m, Vd, V1d) for s, m, Vd, V1d, c, B in plain]), 0, 1)
    del plain
    gc.collect()
    torch.cuda.synchronize()
    med = statistics.median
    pct = lambda a, q: float(np.percentile(np.array(a), q))
    return {"egh": {"value": C / (med(t) / 1000.0), "unit": UNIT, "p50_ms": pct(t, 50), "p99_ms": pct(t, 99),
                    "steps": steps, "warmup": warmup, "launches_per_step": launches, "contacts": C,
                    "precision": "fp64", "call": "BarrierPotential.energy_gradient_hessian_device per scene"},
            "ccd": {"value": len(scs) / (med(t_ccd) / 1000.0), "unit": "scene-steps/s", "p50_ms": pct(t_ccd, 50)},
            "steps": steps_out[-1]}


def ccd_leg(dev, steps=5):
    """Config 0's step size (two 64x64 sheets, 8,192 verts): the GPU call with
    device positions, and the CPU restatement on all host threads."""
    import torch
    import ipctk_gb300 as ipctk
    sc, desc = make_scene("two_sheet")
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    Vd = torch.from_numpy(sc["V"]).to(dev)
    V1d = torch.from_numpy(sc["V1"]).to(dev)
    t = timed_host(lambda: ipctk.compute_collision_free_stepsize(mesh, Vd, V1d), 2, steps)
    step = ipctk.compute_collision_free_stepsize(mesh, Vd, V1d)
    cpu = ccd_baseline_run(sc)
    return {"workload": desc, "gpu_ms": statistics.median(t), "steps_per_s": 1000.0 / statistics.median(t),
            "step_size": step, "cpu_baseline": cpu, "step_equal_cpu": cpu["step_size"] == step}


def mixed_leg(dev, warmup=2, steps=5):
    """Layered cloth (8 stacked 256x256 sheets, 524,288 verts; dhat 1e-3,
    stiffness 1e4, seed 2): E + grad + CLAMP Hessian in FP64 and in mixed
    precision (face-vertex contacts in FP32), device-resident positions, and
    the mixed results' relative error against the FP64 ones (the FP64 path is
    the one held to the oracle at 1e-10)."""
    import torch
    import ipctk_gb300 as ipctk
    from ipctk_gb300 import scenes
    import scipy.sparse as sp
    sc = scenes.layered_cloth()
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    Vd = torch.from_numpy(sc["V"]).to(dev)
    col = ipctk.NormalCollisions()
    col.build(mesh, Vd, sc["dhat"])
    counts = col.counts()
    C = int(counts[:4].sum())
    CL = ipctk.PSDProjectionMethod.CLAMP
    out = {"workload": "layered cloth 8 x 256^2 (524,288 verts)", "contacts": C,
           "contacts_by_type": {"vv": int(counts[0]), "ev": int(counts[1]), "ee": int(counts[2]),
                                "fv": int(counts[3])}}
    res = {}
    for name, mixed in (("fp64", False), ("mixed", True)):
        B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"], mixed_precision=mixed)
        ts = []
        for i in range(warmup + steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e, g, H = B.energy_gradient_hessian_device(col, mesh, Vd, CL)
            torch.cuda.synchronize()
            if i >= warmup:
                ts.append(time.perf_counter() - t0)
        res[name] = (e, g.cpu().numpy(), H.to_scipy())
        out[name] = {"value": C / statistics.median(ts), "unit": UNIT, "ms": 1000 * statistics.median(ts)}
    (e0, g0, H0), (e1, g1, H1) = res["fp64"], res["mixed"]
    out["rel_error_vs_fp64"] = {"energy": abs(e1 - e0) / abs(e0),
                                "gradient": float(np.linalg.norm(g1 - g0) / np.linalg.norm(g0)),
                                "hessian": float(sp.linalg.norm(H1 - H0) / sp.linalg.norm(H0))}
    return out


def friction_leg(dev, warmup=2, steps=5, eps_v=1e-3):
    """Friction on the sphere pack (512 icospheres, seed 0): TangentialCollisions
    build from the collision set at the same positions (mu_s 0.5, mu_k 0.4) and
    FrictionPotential(eps_v = 1e-3) energy + gradient + CLAMP Hessian (one call) at
    device-resident velocities drawn in [-eps_v, eps_v] (a mix of static and
    sliding contacts), timed on the device."""
    import torch
    import ipctk_gb300 as ipctk
    from ipctk_gb300 import scenes
    sc = scenes.sphere_pack()
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    Vd = torch.from_numpy(sc["V"]).to(dev)
    col = ipctk.NormalCollisions()
    col.build(mesh, Vd, sc["dhat"])
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    tc = ipctk.TangentialCollisions()
    rng = np.random.Generator(np.random.PCG64(5))
    Ud = torch.from_numpy(rng.uniform(-eps_v, eps_v, sc["V"].shape)).to(dev)
    D = ipctk.FrictionPotential(eps_v)
    CL = ipctk.PSDProjectionMethod.CLAMP
    tb, te = [], []
    for i in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tc.build(mesh, Vd, col, B, 0.5, 0.4)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e, g, H = D.energy_gradient_hessian(tc, mesh, Ud, CL)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if i >= warmup:
            tb.append(t1 - t0)
            te.append(t2 - t1)
    n = len(tc)
    return {"workload": "sphere pack 512 x 642 verts, eps_v 1e-3, mu_s 0.5, mu_k 0.4", "tangential_collisions": n,
            "egh": {"value": n / statistics.median(te), "unit": UNIT, "ms": 1000 * statistics.median(te)},
            "build_ms": 1000 * statistics.median(tb), "hessian_nnz": int(H.nnz), "energy": float(e)}


def served_leg(dev, seed=4):
    """Served request stream: 64 resident scenes drawn from the batch size
    distribution plus 4 sphere packs; requests alternate barrier (collision
    set rebuilt at the new positions, E + grad + CLAMP Hessian) and
    step-size, each at the scene's positions perturbed by seeded U(+-0.1
    dhat) noise, arriving as a Poisson stream.  Two runs: the offered rate
    2000 req/s (beyond what one GPU completes on these scenes, so latency is
    queueing) and a rate below the measured capacity.  HBM admission budget
    120 GB.  Latency = completion - submission."""
    import ipctk_gb300 as ipctk
    from ipctk_gb300 import scenes
    rng = np.random.default_rng(seed)
    scs = scenes.batch(n_scenes=64, seed=seed) + [scenes.sphere_pack(seed=10 + i) for i in range(4)]
    # seeded noise pools (4 per scene), reused in turn
    pools = [[rng.uniform(-0.1, 0.1, s["V"].shape) * s["dhat"] for _ in range(4)] for s in scs]
    srv = ipctk.Server(workers=8, hbm_budget_bytes=120e9)
    ids = []
    for s in scs:
        m = ipctk.CollisionMesh(s["V"], s["E"], s["F"])
        ids.append(srv.add_scene(m, ipctk.NormalCollisions(), s["dhat"], 0.0, s["kappa"]))
        srv.set_scene_options(ids[-1], mixed_precision=HEADLINE_MODE)
    for t in [srv.submit_barrier(i, s["V"]) for i, s in zip(ids, scs)]:
        srv.wait(t)  # every scene's collision set and work space resident
    pct = lambda a, q: float(np.percentile(np.array(a), q))

    def stream(rate, n):
        arr = np.cumsum(rng.exponential(1.0 / rate, n))
        picks = rng.integers(len(scs), size=n)
        tick = []
        start = time.perf_counter()
        for j in range(n):
            while time.perf_counter() - start < arr[j]:
                pass
            k = int(picks[j])
            s = scs[k]
            V = s["V"] + pools[k][j % 4]
            tick.append(srv.submit_barrier(ids[k], V) if j % 2 == 0 else srv.submit_stepsize(ids[k], s["V"], V))
        lat = [[], []]
        t_first, t_last = None, 0
        for t in tick:
            r = srv.wait(t)
            lat[r["kind"]].append((r["t_end_ns"] - r["t_submit_ns"]) / 1e6)
            t_first = r["t_submit_ns"] if t_first is None else min(t_first, r["t_submit_ns"])
            t_last = max(t_last, r["t_end_ns"])
        allv = lat[0] + lat[1]
        return {"offered_req_s": rate, "requests": n, "completed_req_s": n / ((t_last - t_first) / 1e9),
                "p50_ms": pct(allv, 50), "p99_ms": pct(allv, 99),
                "barrier": {"p50_ms": pct(lat[0], 50), "p99_ms": pct(lat[0], 99)},
                "stepsize": {"p50_ms": pct(lat[1], 50), "p99_ms": pct(lat[1], 99)}}

    offered = stream(2000.0, 1000)
    below = stream(0.7 * offered["completed_req_s"], 300)
    st = srv.stats()
    srv.close()
    return {"workload": f"64 two-sheet scenes (batch size distribution, seed {seed}) + 4 sphere packs; "
                        f"{sum(s['V'].shape[0] for s in scs):,} verts resident; requests alternate barrier "
                        "(build + E + grad + CLAMP Hessian) and step size, positions +-0.1 dhat noise",
            "workers": 8, "hbm_budget_gb": 120, "precision": PRECISION[HEADLINE_MODE],
            "offered": offered, "below_capacity": below,
            "resident_gb": st["resident_bytes"] / 1e9, "workspace_releases": st["releases"]}


def sphere_pack_leg(dev, steps=20):
    """Config 1: the plain FP64 form on the 512-icosphere pack (31,066
    contacts), one fused E + grad + CLAMP Hessian call per step, device
    positions, L2 flushed between steps."""
    import torch
    import ipctk_gb300 as ipctk
    sc, desc = make_scene("sphere_pack")
    mesh = ipctk.CollisionMesh(sc["V"], sc["E"], sc["F"])
    Vd = torch.from_numpy(sc["V"]).to(dev)
    V1d = torch.from_numpy(sc["V1"]).to(dev)
    col = ipctk.NormalCollisions()
    col.build(mesh, Vd, sc["dhat"])
    C = len(col)
    B = ipctk.BarrierPotential(sc["dhat"], sc["kappa"])
    CL = ipctk.PSDProjectionMethod.CLAMP
    stream = torch.cuda.ExternalStream(mesh.stream, device=dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(3):
        B.energy_gradient_hessian_device(col, mesh, Vd, CL)[2].free()
    per = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        B.energy_gradient_hessian_device(col, mesh, Vd, CL)[2].free()
        b.record(stream)
        torch.cuda.synchronize()
        per.append(a.elapsed_time(b))
    ccd = timed_host(lambda: ipctk.compute_collision_free_stepsize(mesh, Vd, V1d), 1, 5)
    build = timed_host(lambda: col.build(mesh, Vd, sc["dhat"]), 1, 5)
    med = statistics.median(per)
    return {"workload": desc, "contacts": C, "egh": {"value": C / (med / 1000.0), "unit": UNIT, "ms": med},
            "ccd_ms": statistics.median(ccd), "collision_build_ms": statistics.median(build)}


def run_gb300(args, rank, world):
    import gc
    import torch
    import ipctk_gb300 as ipctk
    from ipctk_gb300 import scenes

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # replicas: each rank takes its own batch (seed 3 + rank); rank 0's is the config's
    scs = scenes.batch(seed=3 + rank)
    CLAMP = ipctk.PSDProjectionMethod.CLAMP
    batch = ipctk.SceneBatch([(s["V"], s["E"], s["F"]) for s in scs])
    Vh_np = batch.pack([s["V"] for s in scs])
    Vd = torch.from_numpy(Vh_np).to(dev)
    Vh = torch.from_numpy(Vh_np).pin_memory()
    dh = np.array([s["dhat"] for s in scs])
    kap = np.array([s["kappa"] for s in scs])
    col = ipctk.NormalCollisions()
    t0 = time.perf_counter()
    col.build(batch, Vd, dh)
    torch.cuda.synchronize()
    build_ms = 1000 * (time.perf_counter() - t0)
    counts = col.counts()
    C = int(counts[:4].sum())
    ndof = 3 * batch.num_vertices
    BB = ipctk.BatchBarrierPotential(dh, kap, mixed_precision=HEADLINE_MODE)
    stream = torch.cuda.ExternalStream(batch.stream, device=dev)

    def step(pot=None):
        e, g, H = (pot or BB).evaluate(col, batch, Vd, energy=True, gradient=True, hessian=True,
                                       project_hessian_to_psd=CLAMP, device=True)
        nnz = H.nnz
        H.free()
        return nnz

    def timed_steps(pot, k):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for a, b in evs:
            torch.cuda.synchronize()
            a.record(stream)
            step(pot)
            b.record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    def values(pot):
        e, g, H = pot.evaluate(col, batch, Vd, energy=True, gradient=True, hessian=True,
                               project_hessian_to_psd=CLAMP, device=True)
        v = torch.empty(H.nnz, dtype=torch.float64, device=dev)
        H.values_into(v)
        H.free()
        return e, g, v

    def rel_err(a, b):
        (e1, g1, v1), (e0, g0, v0) = a, b
        return {"energy_max_scene": float(np.max(np.abs(e1 - e0) / np.abs(e0))),
                "gradient": float(torch.linalg.norm(g1 - g0).item() / torch.linalg.norm(g0).item()),
                "hessian": float(torch.linalg.norm(v1 - v0).item() / torch.linalg.norm(v0).item())}

    t0 = time.perf_counter()
    nnz = step()  # builds the cached pattern
    first_ms = 1000 * (time.perf_counter() - t0)
    tune = BB.autotune(col, batch, Vd, CLAMP)
    clocks = ClockSampler(local)
    clocks.start()  # before the warm-up, so the GPU is busy when the timed steps start
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    launches0 = ipctk.launch_count()
    t_region = time.perf_counter()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        torch.cuda.synchronize()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    clocks.mark(t_region, time.perf_counter())
    launches = ipctk.launch_count() - launches0
    clk = clocks.stop()
    per = [a.elapsed_time(b) for a, b in ev]
    total_ms = ranks_max(sum(per), dev)
    ms_per_step = total_ms / args.steps
    # whole job: the contacts of every rank's batch over the slowest rank's time
    C_job = ranks_sum(C, dev)
    value = C_job / (ms_per_step / 1000.0)

    # per-kernel times from one profiled step (direct launches instead of the
    # graph replay, so each kernel is bracketed by events on its stream)
    ipctk.profile_enable(True)
    step()
    torch.cuda.synchronize()
    prof = ipctk.profile_report()
    ipctk.profile_enable(False)
    own = {k: v for k, v in prof.items() if k.startswith("k_")}
    top = max(own, key=lambda k: own[k]["ms"])
    top_ms = own[top]["ms"] / max(1, own[top]["launches"])
    prof_total = sum(v["ms"] for v in own.values())
    step_share = {k: round(v["ms"] / prof_total, 4) for k, v in sorted(own.items(), key=lambda kv: -kv[1]["ms"])}
    peak, peak_kind = measured_peaks()
    fp64_dgemm = fp64_peak_tflops(dev)
    fp64_peak = ipctk.fp64_fma_rate()
    nc = ncu_counts(top, "batch")
    launches_top = own[top]["launches"]
    # the ncu figures were taken on a smaller batch of the same scenes and
    # are per contact; a launch processes one chunk of the batch
    per_launch = C / max(1, launches_top)
    if nc.get("fp64_flops_per_contact"):
        nc = dict(nc, fp64_flops=nc["fp64_flops_per_contact"] * per_launch,
                  dram_bytes=nc["dram_bytes_per_contact"] * per_launch)
    # algorithmic bytes of the fused kernel per launch: the E+G+H bytes per
    # contact over the contacts one launch processes (the batch over its
    # chunks' launches)
    abytes = algorithmic_bytes(counts, ndof) / max(1, launches_top)
    if top == "k_psd_scatter":
        # the projection reads each local Hessian and writes its blocks, reading
        # their slots: 2 x 8 N^2 + 4 n^2 bytes per contact
        contribs = 4 * int(counts[0]) + 9 * int(counts[1]) + 16 * int(counts[2] + counts[3])
        abytes = (psd_bytes(counts) + 4 * contribs) / max(1, launches_top)
    achieved_gbs = abytes / (top_ms / 1000.0) / 1e9
    roof = {"kernel": top, "avg_launch_ms": top_ms, "launches_per_step": launches_top,
            "hbm": {"achieved": achieved_gbs, "peak": peak, "unit": "GB/s", "frac": achieved_gbs / peak,
                    "algorithmic_bytes": abytes, "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)"},
            "traffic": nc.get("dram_bytes"), "traffic_source": nc.get("source")}
    if nc.get("fp64_flops"):
        ach = nc["fp64_flops"] / (top_ms / 1000.0) / 1e12
        roof.update({"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                     "flops_per_launch": nc["fp64_flops"], "fp64_pipe_util_ncu": nc.get("fp64_pipe_pct"),
                     "peak_source": "measured on this GPU: a kernel of independent DFMA chains (ipcg_fp64_fma_rate); "
                                    "MEASURED_PEAKS.json has no FP64 entry",
                     "fp64_dgemm_tflops": fp64_dgemm})
    else:
        roof.update({"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
                     "frac": achieved_gbs / peak, "fp64_fma_tflops": fp64_peak, "fp64_dgemm_tflops": fp64_dgemm})

    # end to end through the public API: pinned host positions in, per-scene
    # energies and the gradient out (host arrays) every step
    e2e = []
    nw = max(2, args.warmup // 2)
    g_pinned = torch.empty(ndof, dtype=torch.float64).pin_memory()
    for i in range(nw + args.steps):
        t0 = time.perf_counter()
        e_h, g_h, H = BB.evaluate(col, batch, Vh.numpy(), energy=True, gradient=True, hessian=True,
                                  project_hessian_to_psd=CLAMP, device=True, out_gradient=g_pinned.numpy())
        H.free()
        if i >= nw:
            e2e.append(1000 * (time.perf_counter() - t0))
    e2e_ms = ranks_max(statistics.median(e2e), dev)
    h2d = Vh_np.nbytes
    d2h = 8 * len(scs) + 8 * ndof

    # the batched form in the other precision modes (each autotuned, a few
    # timed steps), and every mode's error against the batched FP64 results
    ref64 = None
    modes = {}
    for mode in ("fp64", "psd_df64", "local_df64"):
        pot = ipctk.BatchBarrierPotential(dh, kap, mixed_precision=mode)
        step(pot)
        tm = pot.autotune(col, batch, Vd, CLAMP)
        step(pot)
        ms = statistics.median(timed_steps(pot, min(5, args.steps)))
        modes[mode] = {"value": C / (ms / 1000.0), "unit": UNIT, "ms": ms,
                       "tuning": {k: tm[k]["chosen"] for k in ("local", "psd")}}
        if mode == "fp64":
            ref64 = values(pot)
        else:
            modes[mode]["rel_error_vs_fp64"] = rel_err(values(pot), ref64)
        del pot
    err = rel_err(values(BB), ref64)
    del ref64
    # batched CCD: one compute_collision_free_stepsize over every scene
    V1d = torch.from_numpy(batch.pack([s["V1"] for s in scs])).to(dev)
    b_steps = []
    b_ccd = timed_host(lambda: b_steps.append(ipctk.compute_collision_free_stepsize_batch(batch, Vd, V1d)), 0, 1)
    del col, batch, Vd, V1d, BB
    gc.collect()
    torch.cuda.synchronize()
    if rank != 0:
        return
    legs = {}
    plain = plain_leg(dev, scs)
    legs["plain"] = plain["egh"]
    legs["ccd"] = {"unit": "scene-steps/s", "batched": {"value": len(scs) / (b_ccd[0] / 1000.0), "ms": b_ccd[0]},
                   "plain": plain["ccd"], "steps_equal": bool(np.array_equal(np.array(plain["steps"]), b_steps[-1]))}
    legs["collision_build_ms"] = build_ms
    legs["first_call_ms"] = first_ms
    if not args.no_legs:
        for name, fn in (("two_sheet_ccd", ccd_leg), ("served", served_leg), ("layered_cloth_mixed", mixed_leg),
                         ("friction", friction_leg), ("sphere_pack", sphere_pack_leg)):
            gc.collect()
            legs[name] = fn(dev)
    cpu = None
    if not args.no_cpu_baseline:
        idx = cpu_sample(scs)
        cpu, _, _ = cpu_baseline_run([scs[k] for k in idx], 3, budget_s=20.0, warmup=1,
                                     desc=f"scenes {idx} of the 256-scene batch")
    pct = lambda a, q: float(np.percentile(np.array(a), q))
    cfg = batch_config(C)
    cfg.update({"contacts_by_type": {"vv": int(counts[0]), "ev": int(counts[1]), "ee": int(counts[2]),
                                     "fv": int(counts[3])}, "hessian_nnz": int(nnz),
                "precision": PRECISION[HEADLINE_MODE], "mode": HEADLINE_MODE,
                "tuning": {k: tune[k]["chosen"] for k in ("local", "psd")}})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded numpy PCG64 scenes; the reference publishes no dataset for this path)",
        "config": cfg,
        "p50_ms": pct(per, 50), "p99_ms": pct(per, 99),
        "batched_vs_plain": value / plain["egh"]["value"],
        "batched_fp64": {"value": modes["fp64"]["value"], "unit": UNIT, "ms": modes["fp64"]["ms"]},
        "mixed_rel_error_vs_fp64": err,
        "batched_modes": modes,
        "roofline": roof, "kernel_share": step_share,
        "cpu_baseline": cpu,
        "e2e": {"value": C_job / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                "call": "BatchBarrierPotential.evaluate with pinned host positions; energies to host, the "
                        "gradient into a pinned host array (out_gradient), Hessian kept on the device"},
        "gpu_launches": int(launches), "gpu_launches_per_step": launches / args.steps,
        "graph_launches_per_step": 1,
        "clocks": clk,
        "legs": legs,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.profile_case:
        run_profile_case(args)
        return
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        run_gb300(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
