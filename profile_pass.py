"""Profiling driver of the hot-path kernels on seeded synthetic plasmas;
prints one JSON line.

    --mode pass (default): the fused step (push + collide + move + deposit)
        against UpdateVelocities, UpdatePositions and CollectVlasovQuantities
        run separately; each phase is one launch of k_pass_tiled<PH> (or
        k_pass_f64<PH>).  Timings are the library's CUDA-event phase times.
    --mode ensemble: a ch_batch of --runs small runs (edges 16-32), --steps
        steps; one k_batch_pass and one k_batch_solve launch per step.
    --mode adjoint: a ch_adjoint run (FP64, --grid^3, --ppc ions per cell,
        --steps steps): one recorded forward and one gradient.
    --mode solve: --steps steps of the plasma of the pass mode; the solves
        inside them (warm start from the previous step's potential) are the
        ones a run makes; prints the solve time, iterations and refinements.
    --mode e2e: the ions through host arrays from ch_host_alloc every step,
        --steps times: upload, ch_step and download as separate calls (wall
        time of each, synchronised), then ch_step_host (the push streams the
        host arrays in and out, k_host_push).

    python profile_pass.py --grid 128 --ppc 64 --nu 0.5
"""
import argparse
import importlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=128, help="nodes per axis (cubic grid, unit spacing)")
    ap.add_argument("--ppc", type=int, default=64, help="ions per cell")
    ap.add_argument("--nu", type=float, default=0.5, help="ion-neutral collision rate (0: no neutrals)")
    ap.add_argument("--Ex", type=float, default=1.0)
    ap.add_argument("--sort-period", type=int, default=4)
    ap.add_argument("--warm", type=int, default=3)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--mode", choices=["pass", "ensemble", "adjoint", "solve", "e2e"], default="pass")
    ap.add_argument("--runs", type=int, default=8)
    ap.add_argument("--steps", type=int, default=4)
    a = ap.parse_args(argv)
    m = importlib.import_module("collisional-hybrid_gb300")
    if a.mode == "ensemble":
        return ensemble(m, a)
    if a.mode == "adjoint":
        return adjoint(m, a)
    if a.mode == "solve":
        return solve(m, a)
    if a.mode == "e2e":
        return e2e(m, a)
    N = a.grid
    p = m.params_for((N, N, N), precision=m.PRECISION[a.precision], E0=(a.Ex, 0.0, 0.0), nui=a.nu, ksp_rtol=1e-10,
                     pc_type=m.PC["mg"], sort_period=a.sort_period, mn=(1.0 if a.nu > 0 else 0.0))
    out = {"grid": N, "ppc": a.ppc, "nu": a.nu, "precision": a.precision}
    with m.Hybrid(p) as h:
        h.load(N ** 3 * a.ppc, m.loader(amp=(0.02, 0.02, 0.02), phase=tuple(m.mode_phases(1))))
        h.CollectVlasovQuantities(copy=False)
        h.ComputePotential(copy=False)
        for s in range(a.warm):
            h.step(s, 1)
        h.set_profiling(True)
        h.reset_profile(); h.step(a.warm, 1); out["fused_ms"] = h.profile()["pass_ms"]
        out["solve_ms"] = h.profile()["solve_ms"]
        h.reset_profile(); h.UpdateVelocities(a.warm + 1); out["push_ms"] = h.profile()["pass_ms"]
        h.reset_profile(); h.UpdatePositions(); out["move_ms"] = h.profile()["pass_ms"]
        h.reset_profile(); h.CollectVlasovQuantities(copy=False); out["deposit_ms"] = h.profile()["pass_ms"]
    print(json.dumps(out))


def solve(m, a):
    N = a.grid
    p = m.params_for((N, N, N), precision=m.PRECISION[a.precision], E0=(a.Ex, 0.0, 0.0), nui=a.nu, ksp_rtol=1e-10,
                     pc_type=m.PC["mg"], sort_period=a.sort_period, mn=(1.0 if a.nu > 0 else 0.0))
    with m.Hybrid(p) as h:
        h.load(N ** 3 * a.ppc, m.loader(amp=(0.02, 0.02, 0.02), phase=tuple(m.mode_phases(1))))
        h.CollectVlasovQuantities(copy=False)
        h.ComputePotential(copy=False)
        h.set_profiling(True)
        rows = []
        for s in range(a.steps):
            h.reset_profile()
            info = h.step(s, 1)
            rows.append([round(h.profile()["solve_ms"], 3), info["iterations"], info["refinements"]])
        print(json.dumps({"mode": "solve", "grid": N, "ppc": a.ppc, "steps[solve_ms, iterations, refinements]": rows}))


def e2e(m, a):
    import time

    import torch

    N = a.grid
    p = m.params_for((N, N, N), precision=m.PRECISION[a.precision], E0=(a.Ex, 0.0, 0.0), nui=a.nu, ksp_rtol=1e-10,
                     pc_type=m.PC["mg"], sort_period=a.sort_period, mn=(1.0 if a.nu > 0 else 0.0))
    out = {"mode": "e2e", "grid": N, "ppc": a.ppc}
    with m.Hybrid(p) as h:
        h.load(N ** 3 * a.ppc, m.loader(amp=(0.02, 0.02, 0.02), phase=tuple(m.mode_phases(1))))
        h.CollectVlasovQuantities(copy=False)
        h.ComputePotential(copy=False)
        for s in range(a.warm):
            h.step(s, 1)
        HP, HV = m.HostArray((h.np, 4)), m.HostArray((h.np, 4))  # ch_host_alloc: page-locked, huge pages
        pos, vel = HP.a, HV.a
        h.download(pos, vel)
        out["bytes_each_way"] = int(pos.nbytes + vel.nbytes)
        try:
            step = a.warm
            rows = []
            for _ in range(a.steps):
                t = [time.perf_counter()]
                h.upload(pos, vel); torch.cuda.synchronize(); t.append(time.perf_counter())
                h.step(step, 1); torch.cuda.synchronize(); t.append(time.perf_counter())
                h.download(pos, vel); torch.cuda.synchronize(); t.append(time.perf_counter())
                step += 1
                rows.append([round(1e3 * (t[i + 1] - t[i]), 2) for i in range(3)])
            out["separate[upload_ms, step_ms, download_ms]"] = rows
            host = []
            h.set_profiling(True)
            h.reset_profile()
            for _ in range(a.steps):
                t0 = time.perf_counter()
                h.step_host(pos, vel, step, 1)
                torch.cuda.synchronize()
                host.append(round(1e3 * (time.perf_counter() - t0), 2))
                step += 1
            prof = h.profile()
            out["step_host_ms"] = host
            out["step_host_pass_ms"] = prof["pass_ms"] / max(1, a.steps)
            out["host_push_calls"], out["host_push_reruns"] = prof["host_push_calls"], prof["host_push_reruns"]
        finally:
            del pos, vel
            HP.free()
            HV.free()
    print(json.dumps(out))


def ensemble(m, a):
    import numpy as np

    rng = np.random.default_rng(7)
    params, nions, loaders = [], [], []
    for r in range(a.runs):
        N = tuple(int(x) for x in rng.choice([16, 24, 32], 3))
        params.append(m.params_for(N, precision=m.PRECISION["mixed"], E0=(a.Ex, 0.0, 0.0), nui=a.nu,
                                   ksp_rtol=1e-10, pc_type=m.PC["mg"], sort_period=a.sort_period, seed=100 + r,
                                   run=r))
        nions.append(N[0] * N[1] * N[2] * a.ppc)
        loaders.append(m.loader(amp=(0.01, 0.0, 0.0)))
    with m.Batch(params, nions) as b:
        b.load(loaders)
        b.initialize()
        info = b.step(0, a.steps)
        print(json.dumps({"mode": "ensemble", "runs": a.runs, "ions": sum(nions), "steps": a.steps,
                          "ok": all(i["status"] == 0 for i in info)}))


def adjoint(m, a):
    N = a.grid
    p = m.params_for((N, N, N), precision=m.PRECISION["fp64"], E0=(0.5, 0.1, 0.0), nui=a.nu, ksp_rtol=1e-13,
                     pc_type=m.PC["mg"], seed=1)
    with m.Adjoint(p, N ** 3 * a.ppc, m.loader(amp=(0.01, 0.0, 0.0)), nsteps=a.steps,
                   checkpoint_every=max(1, a.steps // 2), window=max(1, a.steps // 2)) as adj:
        J = adj.forward(adj.theta0(), record=True)
        g, _ = adj.gradient()
        print(json.dumps({"mode": "adjoint", "J": J, "grad": [float(x) for x in g], **adj.timing()}))


if __name__ == "__main__":
    main()
