#!/usr/bin/env python3
"""Throughput of the hybrid-PIC step (ion push + collisions + move + CIC
deposit + 19-point potential solve) on one GB300, as particle-steps/s.

Default workload: 128^3 periodic grid, unit spacing, 64 ions/cell
(134,217,728 ions), Maxwellian ions (vT = 1 per component), B = z (Omega_i
= 1), E_x = 1.0, nu = 0.5, equal-mass neutrals at Ti, density
1 + 0.02 sum_m sin(2 pi m x/Lx + phi_m) (3 seeded random-phase modes),
dt = 0.05, mixed precision (FP32 ions and inner solves, FP64 refinement
to rtol 1e-10).  Seeded synthetic plasma generated on the device.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the FP64 CPU restatement of the same step (the
reference's PETSc code does not build here) on the host cores.  Under
torchrun each rank runs an independent replica (the step does not shard:
replicas only) and rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "particle-steps/s incl. potential solve"
UNIT = "particle-steps/s"

WORKLOADS = {
    "128cubed-64ppc-mixed": dict(N=(128, 128, 128), ppc=64, E0=(1.0, 0.0, 0.0), nu=0.5, amp=0.02, modes=3,
                                 rtol=1e-10, precision="mixed", drift=(0.0, 0.0, 0.0), nn=False),
    "128cubed-64ppc-fp64": dict(N=(128, 128, 128), ppc=64, E0=(1.0, 0.0, 0.0), nu=0.5, amp=0.02, modes=3,
                                rtol=1e-10, precision="fp64", drift=(0.0, 0.0, 0.0), nn=False),
    "64cubed-32ppc-mixed": dict(N=(64, 64, 64), ppc=32, E0=(0.5, 0.1, 0.0), nu=0.3, amp=0.02, modes=3,
                                rtol=1e-10, precision="mixed", drift=(0.0, 0.0, 0.0), nn=False),
    "32cubed-16ppc-fp64": dict(N=(32, 32, 32), ppc=16, E0=(0.5, 0.0, 0.0), nu=0.1, amp=0.01, modes=1,
                               rtol=1e-8, precision="fp64", drift=(0.0, 0.0, 0.0), nn=False),
    "256x256x64-32ppc-mixed": dict(N=(256, 256, 64), ppc=32, E0=(0.8, 0.0, 0.0), nu=1.0, amp=0.0, modes=0,
                                   rtol=1e-10, precision="mixed", drift=(0.0, 0.3, 0.0), nn=True),
}
DEFAULT = "128cubed-64ppc-mixed"


def chy():
    return importlib.import_module("collisional-hybrid_gb300")


def make_params(w, seed=1, run=0):
    m = chy()
    N = w["N"]
    kw = dict(precision=m.PRECISION[w["precision"]], E0=w["E0"], nui=w["nu"], ksp_rtol=w["rtol"], seed=seed,
              run=run, vi0=w["drift"], pc_type=m.PC["mg"], sort_period=w.get("sort_period", 4))
    if w["nn"]:
        kw.update(nn_profile=1, nn_center=N[0] / 2.0, nn_sigma=N[0] / 6.0, nn_floor=0.1)
    return m.params_for(N, **kw)


def make_loader(w, seed=1, run=0):
    m = chy()
    amp = [0.0, 0.0, 0.0]
    ph = [0.0, 0.0, 0.0]
    if w["modes"] == 1:
        amp[0] = w["amp"]
    elif w["modes"] == 3:
        amp = [w["amp"]] * 3
        ph = m.mode_phases(seed, run)
    return m.loader(amp=tuple(amp), phase=tuple(ph), v0=w["drift"], vT=(1.0, 1.0, 1.0))


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (read only)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ GPU arm
def measured_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(kernel: str):
    """dram bytes per launch from the committed ncu summary, if present."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


class DeviceTimer:
    """CUDA events on the library's stream."""

    def __init__(self, h):
        import torch

        self.torch = torch
        self.stream = torch.cuda.ExternalStream(h.stream_handle())

    def event(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e


def pass_roofline(w, r, prof, N, K, peak, peak_kind):
    """The ion pass's two launches against HBM: the push launch (push,
    collisions, move; reads and writes the ion state, reads the node field;
    on a step before a sort it also stores each ion's rank in its new cell)
    and the deposit launch (reads the ion state, writes the moment
    accumulators; on a sort step it also reads the ranks and writes every
    ion to its sorted slot).  Algorithmic bytes per launch are averaged over
    the timed steps; the headline kernel is the one with the larger time."""
    np_ = r["np"]
    sorts = prof["sort_calls"]
    dep_calls = max(1, prof["deposit_calls"])
    push_calls = max(1, prof["pass_calls"] - prof["deposit_calls"])
    push_ms = (prof["pass_ms"] - prof["deposit_ms"]) / push_calls
    dep_ms = prof["deposit_ms"] / dep_calls
    if w["precision"] == "mixed":
        push_b = np_ * 64 + N * 16 + np_ * 4 * sorts / push_calls
        dep_b = np_ * 32 + N * 32 + np_ * 36 * sorts / dep_calls
        names = ("k_pass_tiled<PUSH|MOVE>", "k_pass_tiled<DEPOSIT>")
    else:
        push_b = np_ * 104 + N * 24
        dep_b = np_ * 52 + N * 32
        names = ("k_pass_f64<PUSH|MOVE>", "k_pass_f64<DEPOSIT>")
    launches = {}
    for key, name, b, ms in (("push", names[0], push_b, push_ms), ("deposit", names[1], dep_b, dep_ms)):
        tr = committed_traffic(name)
        launches[key] = {"kernel": name, "algorithmic_bytes_per_launch": b, "avg_launch_ms": ms,
                         "achieved": b / (ms / 1e3) / 1e9 if ms > 0 else None,
                         "frac": b / (ms / 1e3) / 1e9 / peak if ms > 0 else None,
                         "traffic": (tr["dram_bytes_per_launch"] * np_ / tr["ions"]
                                     if isinstance(tr, dict) and "dram_bytes_per_launch" in tr else None),
                         "calls": push_calls if key == "push" else dep_calls}
    top = max(launches, key=lambda k: launches[k]["avg_launch_ms"] * launches[k]["calls"])
    L = launches[top]
    both_b = push_b * push_calls + dep_b * dep_calls
    both_ms = push_ms * push_calls + dep_ms * dep_calls
    return {"bound": "hbm", "achieved": L["achieved"], "peak": peak, "unit": "GB/s", "frac": L["frac"],
            "peak_kind": peak_kind, "kernel": L["kernel"],
            "algorithmic_bytes_per_launch": L["algorithmic_bytes_per_launch"], "avg_launch_ms": L["avg_launch_ms"],
            "traffic": L["traffic"],
            "traffic_source": "dram bytes of the committed ncu capture (profiles/traffic.json) scaled by the ion count",
            "launches": launches, "sorts_in_timed_steps": sorts,
            "ion_pass": {"achieved": both_b / (both_ms / 1e3) / 1e9, "frac": both_b / (both_ms / 1e3) / 1e9 / peak,
                         "ms_per_step": both_ms / K}}


def ions_for(w):
    return w["N"][0] * w["N"][1] * w["N"][2] * w["ppc"]


def run_gpu(args, w, rank, world, dist):
    m = chy()
    import torch

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    np_ = ions_for(w)
    p = make_params(w, seed=1 + rank, run=rank)
    h = m.Hybrid(p, device=dev)
    h.load(np_, make_loader(w, seed=1 + rank, run=rank))
    h.CollectVlasovQuantities(copy=False)
    h.ComputePotential(copy=False)
    step = 0
    for _ in range(args.warmup):
        h.step(step, 1)
        step += 1
    timer = DeviceTimer(h)
    h.set_profiling(True)
    h.reset_profile()
    launches0 = h.profile()["launches"]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    infos = []
    with ClockSampler(dev) as clk:
        e0 = timer.event()
        for _ in range(args.steps):
            infos.append(h.step(step, 1))
            step += 1
        e1 = timer.event()
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    prof = h.profile()
    h.set_profiling(False)
    launches = prof["launches"] - launches0
    if dist:
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    res = dict(ms=ms, prof=prof, launches=launches, infos=infos, clocks=clk.summary(), np=np_, step=step)
    # end to end through the C ABI with host buffers (rank-local)
    if not args.no_e2e:
        res["e2e"] = e2e(args, h, w, step)
    h.close()
    return res


def host_link():
    """The host link as the bench sees it: pinned 1 GiB copies each way and
    both ways at once (CUDA events / host clock, best of 3), and the host
    NUMA node nearest the GPU (cudaDevAttrHostNumaId) beside the NUMA nodes
    this process may allocate on."""
    import ctypes as C

    import torch

    out = {}
    n = 1 << 30
    h = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(n, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream()
    for name, dst, src in (("h2d_GBps", d, h), ("d2h_GBps", h, d)):
        best = 1e30
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            dst.copy_(src, non_blocking=True)
            e1.record(st)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = n / (best / 1e3) / 1e9
    # both directions at once (two streams): the host link is nearly duplex
    h2 = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    d2 = torch.empty(n, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    best = 1e30
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    out["duplex_GBps"] = 2 * n / best / 1e9
    del h, d, h2, d2
    try:
        rt = C.CDLL("libcudart.so")
    except OSError:
        try:
            rt = C.CDLL("/usr/local/cuda/lib64/libcudart.so")
        except OSError:
            rt = None
    if rt is not None:
        v = C.c_int(-1)
        if rt.cudaDeviceGetAttribute(C.byref(v), 134, torch.cuda.current_device()) == 0:  # cudaDevAttrHostNumaId
            out["host_numa_node_of_gpu"] = v.value
    try:
        with open("/proc/self/status") as f:
            for ln in f:
                if ln.startswith("Mems_allowed_list"):
                    out["process_numa_nodes"] = ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return out


def e2e(args, h, w, step):
    """Per step, through ch_step_host: the ions from the host's RealVector
    arrays (page-locked, from ch_host_alloc) to the device, the step, the
    ions back into the arrays, then phi into a host array; K >= 10 steps,
    timed by the host clock around synchronised calls.  The link's own copy
    rates are measured beside it, so the transfer floor of a step is known."""
    m = chy()
    import torch

    HP, HV, HF = m.HostArray((h.np, 4)), m.HostArray((h.np, 4)), m.HostArray((h.N,))
    pos, vel, phi = HP.a, HV.a, HF.a
    K = max(1, args.e2e_steps)
    try:
        h.download(pos, vel)
        h.step_host(pos, vel, step, 1)
        torch.cuda.synchronize()
        h.reset_profile()
        h.set_profiling(True)
        t0 = time.perf_counter()
        for s in range(K):
            h.step_host(pos, vel, step + 1 + s, 1)
            h.phi(out=phi)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        prof = h.profile()
        h.set_profiling(False)
        Bi = pos.nbytes + vel.nbytes
        Bo = pos.nbytes + vel.nbytes + phi.nbytes
    finally:
        del pos, vel, phi
        for a in (HP, HV, HF):
            a.free()
    link = host_link()
    link["sequential_floor_ms_per_step"] = 1e3 * (Bi / (link["h2d_GBps"] * 1e9) + Bo / (link["d2h_GBps"] * 1e9))
    link["duplex_floor_ms_per_step"] = 1e3 * (Bi + Bo) / (link["duplex_GBps"] * 1e9)
    return {"value": h.np * K / dt, "unit": UNIT, "h2d_bytes_per_step": int(Bi), "d2h_bytes_per_step": int(Bo),
            "steps": K, "ms_per_step": 1e3 * dt / K, "link": link,
            "host_streamed_pushes": prof["host_push_calls"], "reruns": prof["host_push_reruns"],
            "host_arrays": "ch_host_alloc (page-locked, transparent huge pages)"}


# ------------------------------------------------------------------ forms beside the step
def errors_vs_fp64(w, steps=3):
    """Mixed-form outputs against the FP64 form from the same seeded plasma:
    the initial moments and potential, then `steps` steps.  Collisionless
    steps measure the precision error; with collisions the stochastic
    trajectories of the two forms also part where an FP32 and an FP64
    collision test fall on either side of a threshold, so that line is
    reported separately."""
    m = chy()

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    out = {"norm": "relative L2 against the FP64 form, same seeded ions", "steps": steps}
    for tag, extra in (("collisionless", dict(mn=0.0)), ("collisions", {})):
        res = {}
        for form in ("mixed", "fp64"):
            p = make_params(dict(w, precision=form))
            for k, v in extra.items():
                setattr(p, k, v)
            with m.Hybrid(p) as h:
                h.load(ions_for(w), make_loader(w))
                m0 = h.CollectVlasovQuantities()
                phi0 = h.ComputePotential()
                h.step(0, steps)
                res[form] = (m0, phi0, h.CollectVlasovQuantities(), h.phi())
        (m0m, p0m, m1m, p1m), (m0d, p0d, m1d, p1d) = res["mixed"], res["fp64"]
        if tag == "collisionless":
            out["moments_initial"] = rel(m0m, m0d)
            out["phi_initial"] = rel(p0m, p0d)
        out[f"moments_after_steps_{tag}"] = rel(m1m, m1d)
        out[f"phi_after_steps_{tag}"] = rel(p1m, p1d)
    return out


def ensemble_runs(nruns=64, seed=3):
    """The ensemble workload: grid edge per axis uniform in {16, 24, 32, 48,
    64}, 8-32 ions/cell, E_x ~ U[0.2, 1.5], nu ~ logU[0.01, 2], a distinct
    seed per run; mixed form, rtol 1e-10."""
    m = chy()
    rng = np.random.default_rng(seed)
    edges = np.array([16, 24, 32, 48, 64])
    params, nions, loaders = [], [], []
    for r in range(nruns):
        N = tuple(int(x) for x in rng.choice(edges, 3))
        ppc = int(rng.integers(8, 33))
        Ex = float(rng.uniform(0.2, 1.5))
        nu = float(np.exp(rng.uniform(np.log(0.01), np.log(2.0))))
        p = m.params_for(N, precision=m.PRECISION["mixed"], E0=(Ex, 0.0, 0.0), nui=nu, ksp_rtol=1e-10,
                         pc_type=m.PC["mg"], sort_period=4, seed=1000 + r, run=r)
        params.append(p)
        nions.append(N[0] * N[1] * N[2] * ppc)
        loaders.append(m.loader(amp=(0.01, 0.0, 0.0)))
    return params, nions, loaders


def run_ensemble(steps):
    """Aggregate particle-steps/s of the ensemble in one ch_batch against the
    same runs stepped one by one on a ch_ctx each (CUDA events on each
    stream)."""
    m = chy()
    import torch

    params, nions, loaders = ensemble_runs()
    total = sum(nions)
    with m.Batch(params, nions) as b:
        b.load(loaders)
        b.initialize()
        tune = b.autotune()
        b.step(0, 2)
        st = torch.cuda.ExternalStream(b.stream_handle())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        info = b.step(2, steps)
        e1.record(st)
        torch.cuda.synchronize()
        ms_batch = e0.elapsed_time(e1)
        ok = all(i["status"] == 0 for i in info)
    ms_one = 0.0
    for p, n, L in zip(params, nions, loaders):
        with m.Hybrid(p) as h:
            h.load(n, L)
            h.CollectVlasovQuantities(copy=False)
            h.ComputePotential(copy=False)
            h.step(0, 2)
            t = DeviceTimer(h)
            torch.cuda.synchronize()
            a = t.event()
            h.step(2, steps)
            c = t.event()
            torch.cuda.synchronize()
            ms_one += a.elapsed_time(c)
    v_b = total * steps / (ms_batch / 1e3)
    v_o = total * steps / (ms_one / 1e3)
    return {"value": v_b, "unit": UNIT, "one_by_one": v_o, "speedup": v_b / v_o, "runs": len(params),
            "ions": total, "nodes": sum(p.Nx * p.Ny * p.Nz for p in params), "steps": steps,
            "ms_per_step": ms_batch / steps, "one_by_one_ms_per_step": ms_one / steps, "tuning": tune,
            "all_runs_ok": ok, "workload": "64 runs, edges U{16,24,32,48,64} per axis, 8-32 ions/cell, "
            "E_x U[0.2,1.5], nu logU[0.01,2], mixed form; timed steps are a bounded sample of the 100-step run"}


def run_adjoint(fd=True):
    """Differentiation workload: 64^3 grid, 32 ions/cell, E0 = (0.5, 0.1, 0),
    nu = 0.3, 50 steps, checkpoints every 10, objective over the final 10
    steps (mean x flux + 0.1 mean square potential); gradient w.r.t. E0,
    vn0, amp against central differences of the frozen-event
    forward."""
    m = chy()
    N = (64, 64, 64)
    p = m.params_for(N, precision=m.PRECISION["fp64"], E0=(0.5, 0.1, 0.0), nui=0.3, ksp_rtol=1e-13,
                     pc_type=m.PC["mg"], seed=1)
    L = m.loader(amp=(0.01, 0.0, 0.0))
    np_ = 64 ** 3 * 32
    with m.Adjoint(p, np_, L, nsteps=50, checkpoint_every=10, window=10) as adj:
        th = adj.theta0()
        t0 = time.perf_counter()
        J = adj.forward(th, record=True)
        t1 = time.perf_counter()
        g, _ = adj.gradient()
        t2 = time.perf_counter()
        tim = adj.timing()
        out = {"J": J, "gradient": [float(x) for x in g], "theta": ["E0x", "E0y", "E0z", "vn0x", "vn0y", "vn0z", "amp"],
               "forward_ms": tim["forward_ms"], "gradient_ms": tim["gradient_ms"],
               "recompute_ms": tim["recompute_ms"], "gradient_over_forward": tim["gradient_ms"] / tim["forward_ms"],
               "events": tim["events"], "ions": np_, "steps": 50, "checkpoint_every": 10,
               "wall_s": {"forward": t1 - t0, "gradient": t2 - t1}}
        if fd:
            # every parameter at eps = 1e-6; the amplitude also down to
            # 3e-9.  Its perturbation moves every ion's start by up to
            # eps 2 Lx / (2 pi) / 0.99 cells, and an ion that comes that
            # close to a cell face in some step passes a kink of the CIC
            # weights and biases its difference quotient; the expected number
            # of such ion-steps is 2 x that distance x ions x steps.  J's
            # noise (solves to rtol 1e-13) is about 1e-15, so the smallest
            # step still resolves the quotient to a few 1e-6.
            def central(k, eps):
                e = np.zeros_like(th)
                e[k] = eps
                return (adj.forward(th + e) - adj.forward(th - e)) / (2 * eps)

            fdv = np.array([central(k, 1e-6) for k in range(len(th))])
            scale = np.maximum(np.abs(fdv), 1e-3 * np.abs(fdv).max())
            err = np.abs(g - fdv) / scale
            out["central_fd_eps1e-6"] = [float(x) for x in fdv]
            out["rel_err_vs_fd_eps1e-6"] = [float(x) for x in err]
            sweep = {}
            for eps in (1e-6, 1e-7, 1e-8, 3e-9):
                v = float(fdv[6]) if eps == 1e-6 else central(6, eps)
                reach = eps * 2.0 * N[0] / (2.0 * np.pi) / 0.99
                sweep[f"{eps:g}"] = {"fd": v, "rel_err": float(abs(g[6] - v) / abs(v)),
                                     "kink_ion_steps_expected": 2.0 * reach * np_ * 50}
            out["amp_fd_sweep"] = sweep
            out["amp_rel_err_at_smallest_eps"] = sweep["3e-09"]["rel_err"]
            out["max_rel_err_vs_fd_E0_vn0"] = float(err[:6].max())
    return out


def run_solves(reps=10):
    """The stand-alone solve (src/solver.c's work) on the two production
    grids: a loaded density (n = 1 + 0.02 sum_m sin(2 pi m x/Lx + phase_m),
    flux = the workload's drift times n), then `reps` solves, each from
    phi = 0 (ComputeInitialPhi) to rtol 1e-10 with the workload's solver
    (mixed form: multigrid-preconditioned CG in FP32 inside FP64 refinement),
    timed with the library's CUDA events on its stream."""
    m = chy()
    out = {}
    for name in ("128cubed-64ppc-mixed", "256x256x64-32ppc-mixed"):
        w = WORKLOADS[name]
        N = w["N"]
        p = make_params(w)
        x = (np.arange(N[0]) / N[0])[None, None, :]
        ph = m.mode_phases(1)
        n = 1.0 + 0.02 * sum(np.sin(2 * np.pi * k * x + ph[k - 1]) for k in (1, 2, 3))
        n = np.broadcast_to(n, (N[2], N[1], N[0])).ravel()
        nodes = np.zeros((n.size, 4))
        nodes[:, 0] = n
        for d in range(3):
            nodes[:, 1 + d] = w["drift"][d] * n
        zeros = np.zeros(n.size)
        with m.Hybrid(p) as h:
            h.set_moments(nodes)
            its = []
            for k in range(reps + 2):
                if k == 2:
                    h.set_profiling(True)
                    h.reset_profile()
                h.set_phi(zeros)
                h.ComputePotential(copy=False)
                its.append((h.last_solve["iterations"], h.last_solve["refinements"],
                            h.last_solve["rnorm"] / h.last_solve["bnorm"]))
            prof = h.profile()
            h.set_profiling(False)
        ms = prof["solve_ms"] / max(1, prof["solve_calls"])
        out[name] = {"grid": list(N), "solves_per_s": 1e3 / ms, "ms_per_solve": ms, "solves": reps,
                     "iterations": its[-1][0], "refinements": its[-1][1], "rel_residual": its[-1][2],
                     "start": "phi = 0", "ksp_rtol": w["rtol"]}
    return out


# ------------------------------------------------------------------ CPU arm
# The CPU legs (the reference arm and cpu_baseline) run the FP64 CPU
# restatement of the step, built from the oracle alone: nothing of the product
# package is imported or loaded on these legs.
def oracle_params(w, N, seed=1, run=0):
    """The workload's plasma on grid N for the FP64 CPU restatement (Jacobi-CG
    at the workload's rtol; the CPU has no multigrid)."""
    from oracle import pyoracle as po

    kw = dict(E0=w["E0"], nui=w["nu"], ksp_rtol=w["rtol"], seed=seed, run=run, vi0=w["drift"], pc_type=1,
              precision=0)
    if w["nn"]:
        kw.update(nn_profile=1, nn_center=N[0] / 2.0, nn_sigma=N[0] / 6.0, nn_floor=0.1)
    return po.default_params(tuple(N), **kw)


def oracle_loader(w, seed=1, run=0):
    from oracle import pyoracle as po

    amp, ph = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
    if w["modes"] == 1:
        amp[0] = w["amp"]
    elif w["modes"] == 3:
        amp = [w["amp"]] * 3
        ph = po.mode_phases(seed, run)
    return po.make_loader(amp=tuple(amp), phase=tuple(ph), v0=w["drift"], vT=(1.0, 1.0, 1.0))


def sample_grid(w, div):
    """A sub-box of the workload's grid, 1/div per axis, with the same ions per
    cell: the same plasma at 1/div^3 of the ions and nodes."""
    return tuple(max(8, n // div) for n in w["N"])


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.machine()


def cpu_run(w, div, threads, steps, warmup):
    """The FP64 CPU restatement of the step (push with collisions, move,
    deposit, RHS and Jacobi-CG solve), run for warmup + steps steps on the
    sub-box sample_grid(w, div) with `threads` OpenMP threads; every timed
    step is executed, none is extrapolated."""
    from oracle import pyoracle as po

    po.build()
    po.lib().orc_set_threads(threads)
    N = sample_grid(w, div)
    q = oracle_params(w, N)
    nions = N[0] * N[1] * N[2] * w["ppc"]
    ions = po.load(q, oracle_loader(w), nions)
    run = po.Run(q, ions)
    rc, _ = run.initialize()
    if rc:
        raise RuntimeError(f"oracle initial solve: status {rc}")
    times = []
    for s in range(warmup + steps):
        t0 = time.perf_counter()
        rc, _ = run.step(s)
        t1 = time.perf_counter()
        if rc:
            raise RuntimeError(f"oracle step {s}: status {rc}")
        if s >= warmup:
            times.append(t1 - t0)
    ms = 1e3 * statistics.mean(times)
    return dict(value=nions / (ms / 1e3), ms_per_step=ms, ions=nions, grid=N, threads=threads, steps=steps,
                warmup=warmup, total_s=sum(times))


def cpu_desc(c, w, kind="all host cores"):
    g = c["grid"]
    return (f"FP64 CPU restatement of the step (push with collisions, move, deposit, RHS, Jacobi-CG to rtol "
            f"{w['rtol']:g}; OpenMP, {c['threads']} thread{'s' if c['threads'] > 1 else ''}, {kind}) on a "
            f"{g[0]}x{g[1]}x{g[2]} sub-box of the {w['N'][0]}x{w['N'][1]}x{w['N'][2]} workload at the same "
            f"{w['ppc']} ions/cell ({c['ions']:,} ions): {c['steps']} timed steps after {c['warmup']} warm-up, "
            f"{c['ms_per_step']:.0f} ms per step, all executed")


# ------------------------------------------------------------------ main
def config_of(args, w, world):
    """The workload's config, identical in both arms."""
    return {"workload": args.workload, "grid": list(w["N"]), "ions": ions_for(w), "ions_per_cell": w["ppc"],
            "precision": w["precision"], "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
            "l2": "inputs larger than L2 (ion state 4.3 GB)", "ksp_rtol": w["rtol"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-div", type=int, default=2,
                    help="CPU legs run a sub-box of 1/div of the grid per axis at the same ions per cell")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-form comparison line")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble (ch_batch) measurement")
    ap.add_argument("--ensemble-steps", type=int, default=10)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (ch_adjoint) measurement")
    ap.add_argument("--no-adjoint-fd", action="store_true", help="skip its finite-difference check")
    ap.add_argument("--no-solve", action="store_true", help="skip the stand-alone solves (solves/s)")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        # the reference's PETSc build is unavailable (no PETSc, MPI or HDF5);
        # its CPU algorithm is the FP64 restatement, timed on the host cores
        # by rank 0 alone, every step executed
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        c = cpu_run(w, args.cpu_div, threads, max(1, args.steps), max(0, args.warmup))
        line = {"metric": METRIC, "value": c["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": c["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": config_of(args, w, world),
                "cpu_baseline": {"value": c["value"], "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": cpu_desc(c, w), "cpu_model": cpu_model(),
                                 "timed_s": c["total_s"]},
                "e2e": {"value": c["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("gloo")
    r = run_gpu(args, w, rank, world, dist)
    fp64 = None
    if not args.no_fp64 and w["precision"] == "mixed" and rank == 0:
        w64 = dict(w, precision="fp64")
        a64 = argparse.Namespace(**vars(args))
        a64.steps, a64.warmup, a64.no_e2e = max(2, min(args.steps, 5)), 1, True
        r64 = run_gpu(a64, w64, 0, 1, None)
        fp64 = {"value": r64["np"] * a64.steps / (r64["ms"] / 1e3), "unit": UNIT,
                "ms_per_step": r64["ms"] / a64.steps, "steps": a64.steps}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    K = args.steps
    ms_step = r["ms"] / K
    value = r["np"] * world * K / (r["ms"] / 1e3)
    prof = r["prof"]
    peak, peak_kind = measured_peak()
    N = w["N"][0] * w["N"][1] * w["N"][2]
    roof = pass_roofline(w, r, prof, N, K, peak, peak_kind)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if w["precision"] == "mixed" else "f64", "data": "synthetic",
        "config": config_of(args, w, world),
        "roofline": roof,
        "phase_ms_per_step": {k.replace("_ms", ""): prof[k] / K for k in ("pass_ms", "solve_ms", "sort_ms",
                                                                          "moments_ms")},
        "solve": {"iterations_last": r["infos"][-1]["iterations"], "refinements_last": r["infos"][-1]["refinements"],
                  "rel_residual_last": r["infos"][-1]["rnorm"] / max(r["infos"][-1]["bnorm"], 1e-300)},
        "collisions_last": {"Nc": r["infos"][-1]["Nc"], "events": r["infos"][-1]["collisions"]},
        "gpu_launches": int(r["launches"]),
        "clocks": r["clocks"],
    }
    if fp64:
        line["fp64_form"] = fp64
        line["mixed_over_fp64"] = value / world / fp64["value"]
    if "e2e" in r:
        e = r["e2e"]
        line["e2e"] = {k: e[k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step")}
        line["e2e"]["value"] *= world
        line["e2e"]["ms_per_step"] = e["ms_per_step"]
        for k in ("steps", "link", "host_streamed_pushes", "reruns", "host_arrays"):
            line["e2e"][k] = e[k]
    if not args.no_fp64 and w["precision"] == "mixed":
        line["errors_vs_fp64"] = errors_vs_fp64(w)
    if not args.no_ensemble:
        line["ensemble"] = run_ensemble(args.ensemble_steps)
    if not args.no_solve:
        line["solves"] = run_solves()
    if not args.no_adjoint:
        line["adjoint"] = run_adjoint(fd=not args.no_adjoint_fd)
    if not args.no_cpu:
        # all host cores (the reference arm's leg, 3 timed steps), and one
        # core on a sub-box of 1/4 per axis (the reference's serial loops)
        c = cpu_run(w, args.cpu_div, os.cpu_count() or 1, 3, 1)
        c1 = cpu_run(w, 2 * args.cpu_div, 1, 2, 1)
        line["cpu_baseline"] = {"value": c["value"], "unit": UNIT, "cores": c["threads"], "kind": "port",
                                "sample": cpu_desc(c, w), "cpu_model": cpu_model(),
                                "single_thread": {"value": c1["value"], "unit": UNIT, "cores": 1,
                                                  "sample": cpu_desc(c1, w, "one core")}}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
