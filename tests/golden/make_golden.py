"""Generates the golden vectors in tests/golden/ from the reference's own code.

The reference's hot-path sources (src/particles.c, src/lhs.c, src/rhs.c,
src/calculus.c, src/vectors.c, src/random.c) are compiled unmodified
against the PETSc stand-in of oracle/ref (make -C oracle ref) and driven on
seeded inputs.  Inputs come from the oracle's seeded loader, so the fixtures
store outputs plus the parameters needed to rebuild the inputs.

Run:  python tests/golden/make_golden.py      (needs the reference sources)
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from oracle import pyoracle as po  # noqa: E402

ip = C.POINTER(C.c_int)


def grids():
    # (N, L, ions, amp, phase): the 8^3 case of run-case test-collection-8cubed
    # and an uneven 15x10x8 box like test-collection-asymmetric
    return [
        dict(name="g8", N=(8, 8, 8), L=(8.0, 8.0, 8.0), np=8192, amp=(0.25, 0.0, 0.0), phase=(0.0, 0.0, 0.0)),
        dict(name="g15x10x8", N=(15, 10, 8), L=(3.0, 2.0, 1.6), np=4800, amp=(0.1, 0.05, 0.02),
             phase=(0.3, 1.1, 2.9)),
    ]


def main():
    po.build(ref=True)
    R = po.ref()
    if R is None:
        raise SystemExit("reference harness not built (needs the reference sources)")
    out = {}
    for G in grids():
        N, L = G["N"], np.array(G["L"])
        Nn = int(np.prod(N))
        p = po.default_params(N, tuple(L))
        ions = po.load(p, po.make_loader(amp=G["amp"], phase=G["phase"], vT=(1.0, 0.8, 1.2)), G["np"])
        pos, vel = ions.aos()
        tag = G["name"]
        out[f"{tag}_meta"] = np.array([*N, *L, G["np"], *G["amp"], *G["phase"]], dtype=np.float64)
        out[f"{tag}_pos"] = pos[:, :3].copy()
        out[f"{tag}_vel"] = vel[:, :3].copy()
        # CollectVlasovQuantities, one call and two calls (accumulation, D6)
        for ncalls in (1, 2):
            nodes = np.zeros(4 * Nn)
            rc = R.ref_collect(*N, po._ptr(L), ions.np, po._ptr(pos), po._ptr(vel), ncalls, po._ptr(nodes))
            assert rc == 0
            out[f"{tag}_collect{ncalls}"] = nodes
        nodes = out[f"{tag}_collect1"]
        # LHS rows (full / laplacian / identity), two magnetisations
        for ki, kap in enumerate([(0.0, 0.0, 0.0), (0.3, -0.2, 1.0)]):
            kd = np.array(kap)
            for lt in (0, 1, 2):
                ncols = np.zeros(Nn, dtype=np.int32)
                cols = np.zeros(Nn * 27, dtype=np.int32)
                vals = np.zeros(Nn * 27)
                rc = R.ref_lhs(*N, po._ptr(L), po._ptr(kd), lt, po._ptr(nodes),
                               ncols.ctypes.data_as(ip), cols.ctypes.data_as(ip), po._ptr(vals))
                assert rc == 0
                m = int(ncols.max())
                out[f"{tag}_lhs{lt}_k{ki}_cols"] = cols.reshape(Nn, 27)[:, :m].copy()
                out[f"{tag}_lhs{lt}_k{ki}_vals"] = vals.reshape(Nn, 27)[:, :m].copy()
            for rt in (0, 1, 2):
                E0 = np.array([0.5, 0.1, -0.2])
                b = np.zeros(Nn)
                rc = R.ref_rhs(*N, po._ptr(L), po._ptr(kd), po._ptr(E0), 1.0, 0.1, rt, po._ptr(nodes), po._ptr(b))
                assert rc == 0
                out[f"{tag}_rhs{rt}_k{ki}"] = b
        # DifferenceVector at random points, phi random
        rng = np.random.default_rng(7)
        phi = rng.standard_normal(Nn)
        pts = rng.uniform(0.0, 1.0, (64, 3)) * np.array(N)
        pts[:4] = [[N[0] - 0.25, 0.5, 0.5], [0.5, N[1] - 0.1, 0.5], [0.5, 0.5, N[2] - 0.5],
                   [N[0] - 0.5, N[1] - 0.5, N[2] - 0.5]]
        f = np.zeros(3 * len(pts))
        rc = R.ref_difference_vector(*N, po._ptr(phi), len(pts), po._ptr(pts), po._ptr(f))
        assert rc == 0
        out[f"{tag}_dv_phi"] = phi
        out[f"{tag}_dv_pts"] = pts
        out[f"{tag}_dv_f"] = f
        # calculus helpers at every node of a random field
        F = rng.standard_normal(Nn)
        cal = np.zeros((Nn, 12))
        for k in range(N[2]):
            for j in range(N[1]):
                for i in range(N[0]):
                    r = (k * N[1] + j) * N[0] + i
                    o = np.zeros(12)
                    assert R.ref_calculus(*N, po._ptr(L), po._ptr(F), i, j, k, po._ptr(o)) == 0
                    cal[r] = o
        out[f"{tag}_cal_F"] = F
        out[f"{tag}_cal"] = cal
        # UpdatePositions as written (D5): positions unchanged
        pos2 = pos.copy()
        assert R.ref_update_positions(*N, po._ptr(L), 0.05, ions.np, po._ptr(pos2), po._ptr(vel)) == 0
        out[f"{tag}_moved"] = pos2[:, :3].copy()
    # ComputeCollisions statistics on a Maxwellian population (src/random.c
    # generators, seed -12345 as src/hybrid.c:49 for rank 0)
    cases = [dict(np=200000, viT=(1.0, 1.0, 1.0), vi0=(0.0, 0.0, 0.0), nu=0.1, dt=0.05, vnT=1.0,
                  vn0=(0.0, 0.0, 0.0)),
             dict(np=200000, viT=(1.0, 1.0, 1.0), vi0=(0.0, 0.3, 0.0), nu=1.0, dt=0.05, vnT=1.0,
                  vn0=(0.5, 0.0, 0.0))]
    for ci, cs in enumerate(cases):
        p = po.default_params((8, 8, 8))
        ions = po.load(p, po.make_loader(v0=cs["vi0"], vT=cs["viT"]), cs["np"])
        _, vel = ions.aos()
        before = vel[:, :3].copy()
        nc = C.c_int()
        rc = R.ref_collisions(cs["np"], po._ptr(vel), po._ptr(np.array(cs["viT"])), po._ptr(np.array(cs["vi0"])),
                              cs["nu"], cs["dt"], 1.0, 1.0, cs["vnT"], po._ptr(np.array(cs["vn0"])), -12345,
                              C.byref(nc))
        assert rc == 0, rc
        after = vel[:, :3]
        changed = np.any(after != before, axis=1)
        m = after.mean(axis=0)
        var = after.var(axis=0)
        kurt = ((after - m) ** 4).mean(axis=0) / var ** 2
        out[f"coll{ci}_params"] = np.array([cs["np"], *cs["viT"], *cs["vi0"], cs["nu"], cs["dt"], cs["vnT"],
                                            *cs["vn0"]])
        out[f"coll{ci}_stats"] = np.array([nc.value, changed.sum(), *m, *var, *kurt])
        # per-component moments of the collided ions only
        a = after[changed]
        out[f"coll{ci}_collided"] = np.array([*a.mean(axis=0), *a.var(axis=0)])
    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
