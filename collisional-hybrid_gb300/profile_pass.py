"""Per-phase timing of the ion pass: the fused step (push + collide + move +
deposit) against UpdateVelocities, UpdatePositions and CollectVlasovQuantities
run separately, on a seeded synthetic plasma.  Prints one JSON line.

    python collisional-hybrid_gb300/profile_pass.py --grid 128 --ppc 64 --nu 0.5

Timings are CUDA-event phase times of the library (ch_get_profile); the step
that is timed follows `--warm` untimed steps.  Used for the ncu captures of
the pass kernels (each phase is one launch of k_pass_tiled<PH>)."""
import argparse
import importlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=128, help="nodes per axis (cubic grid, unit spacing)")
    ap.add_argument("--ppc", type=int, default=64, help="ions per cell")
    ap.add_argument("--nu", type=float, default=0.5, help="ion-neutral collision rate (0: no neutrals)")
    ap.add_argument("--Ex", type=float, default=1.0)
    ap.add_argument("--sort-period", type=int, default=4)
    ap.add_argument("--warm", type=int, default=3)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    a = ap.parse_args(argv)
    m = importlib.import_module("collisional-hybrid_gb300")
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


if __name__ == "__main__":
    main()
