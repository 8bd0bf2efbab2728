"""Ensembles (ch_batch): every run of a batch must behave as the same run on
its own ch_ctx.

Given the same phi, the ion pass of a batch is the single-run pass (same
tile code, integer deposit, exact S sums), so ions, moments and collision
counts agree bit for bit.  The potential solves (one thread-block cluster
per run against the single-run graph-captured solver) agree to the solve
tolerance: both meet rtol 1e-10, so phi agrees to about 1e-9 relative.
Graph replay must equal eager launches, and the autotuner must leave the
state as it found it."""
import numpy as np
import pytest

SHAPES = [((16, 24, 32), 8, 0.3, 0.05, 11), ((32, 16, 16), 16, 1.2, 1.0, 12), ((24, 24, 24), 12, 0.7, 0.2, 13),
          ((16, 16, 48), 10, 0.2, 0.01, 14)]


def _runs(chy):
    params, nions, loaders = [], [], []
    for r, (N, ppc, Ex, nu, seed) in enumerate(SHAPES):
        p = chy.params_for(N, precision=chy.PRECISION["mixed"], E0=(Ex, 0.0, 0.0), nui=nu, ksp_rtol=1e-10,
                           pc_type=chy.PC["mg"], sort_period=4, seed=seed, run=r)
        params.append(p)
        nions.append(N[0] * N[1] * N[2] * ppc)
        loaders.append(chy.loader(amp=(0.02, 0.02, 0.02), phase=tuple(chy.mode_phases(seed, r))))
    return params, nions, loaders


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.gpu
def test_batch_matches_single_runs(chy):
    params, nions, loaders = _runs(chy)
    singles = [chy.Hybrid(p) for p in params]
    with chy.Batch(params, nions) as b:
        b.load(loaders)
        b.initialize()
        for r, h in enumerate(singles):
            h.load(nions[r], loaders[r])
            m1 = h.CollectVlasovQuantities()
            phi1 = h.ComputePotential()
            assert np.array_equal(b.moments(r), m1), r
            assert _rel(b.phi(r), phi1) < 1e-8, (r, _rel(b.phi(r), phi1))
            b.set_phi(r, phi1)
        info = b.step(0, 1)
        for r, h in enumerate(singles):
            si = h.step(0, 1)
            assert info[r]["status"] == 0
            assert info[r]["collisions"] == si["collisions"] and info[r]["Nc"] == si["Nc"], (r, info[r], si)
            pb, vb = b.download(r)
            ps, vs = h.download()
            assert np.array_equal(pb, ps) and np.array_equal(vb, vs), r
            assert np.array_equal(b.moments(r), h.CollectVlasovQuantities()), r
            # after the step both solved the same moments
            assert _rel(b.phi(r), h.phi()) < 1e-8, r
        # several steps, each side with its own solves (a sort at step 3)
        info = b.step(1, 5)
        for r, h in enumerate(singles):
            si = h.step(1, 5)
            assert info[r]["status"] == 0 and info[r]["rnorm"] <= 1.01e-10 * info[r]["bnorm"]
            mb = b.moments(r)
            ms = h.CollectVlasovQuantities()
            assert _rel(mb, ms) < 1e-6, (r, _rel(mb, ms))
            assert abs(info[r]["collisions"] - si["collisions"]) <= 5 + 0.01 * si["collisions"], (r, info[r], si)
    for h in singles:
        h.close()


@pytest.mark.gpu
def test_batch_graph_replay_equals_eager(chy):
    params, nions, loaders = _runs(chy)
    out = []
    for eager in (False, True):
        with chy.Batch(params, nions) as b:
            b.load(loaders)
            b.initialize()
            b.set_tuning(4, 2)
            if eager:
                b.set_profiling(True)
            b.step(0, 7)
            out.append([(b.moments(r), b.phi(r), b.download(r)) for r in range(len(params))])
    for (ma, pa, (xa, va)), (mb, pb, (xb, vb)) in zip(*out):
        assert np.array_equal(ma, mb) and np.array_equal(pa, pb)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)


@pytest.mark.gpu
def test_batch_reinitialize_between_sorts_equals_eager(chy):
    """A second initialize swaps the ion buffers with a full sort after the
    step graphs of both buffer parities exist: the replayed steps that follow
    (two more sorts) must still read the current buffers."""
    params, nions, loaders = _runs(chy)
    out = []
    for eager in (False, True):
        with chy.Batch(params, nions) as b:
            b.load(loaders)
            b.initialize()
            if eager:
                b.set_profiling(True)
            b.step(0, 9)
            b.initialize()
            info = b.step(9, 10)
            assert all(i["status"] == 0 for i in info)
            out.append([(b.moments(r), b.phi(r), b.download(r)) for r in range(len(params))])
    for (ma, pa, (xa, va)), (mb, pb, (xb, vb)) in zip(*out):
        assert np.array_equal(ma, mb) and np.array_equal(pa, pb)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)


@pytest.mark.gpu
def test_batch_autotune_restores_state(chy):
    params, nions, loaders = _runs(chy)
    with chy.Batch(params, nions) as b:
        b.load(loaders)
        b.initialize()
        b.step(0, 2)
        before = [(b.phi(r), b.download(r)) for r in range(len(params))]
        t = b.autotune()
        assert t["cluster"] in (1, 2, 4, 8) and t["pass_ctas_per_sm"] in (1, 2, 3)
        assert t["cluster_big"] in (0, 8, 16) and b.tuning() == t
        assert t["pass_ms"] > 0 and t["solve_ms"] > 0
        after = [(b.phi(r), b.download(r)) for r in range(len(params))]
        for (pa, (xa, va)), (pb, (xb, vb)) in zip(before, after):
            assert np.array_equal(pa, pb) and np.array_equal(xa, xb) and np.array_equal(va, vb)
        info = b.step(2, 2)
        assert all(i["status"] == 0 for i in info)


@pytest.mark.gpu
def test_batch_cluster_sizes_agree(chy):
    """Every cluster size solves to the same tolerance from the same state."""
    params, nions, loaders = _runs(chy)
    phis = []
    for C in (1, 2, 8):
        with chy.Batch(params, nions) as b:
            b.set_tuning(C, 2)
            b.load(loaders)
            b.initialize()
            phis.append([b.phi(r) for r in range(len(params))])
    for r in range(len(params)):
        assert _rel(phis[1][r], phis[0][r]) < 1e-8 and _rel(phis[2][r], phis[0][r]) < 1e-8


@pytest.mark.gpu
def test_batch_split_solve_agrees():
    """Runs of at least twice the mean node count may be solved in a launch of
    their own with wider clusters: the potentials agree with the single
    launch to the solve tolerance."""
    import importlib

    chy = importlib.import_module("collisional-hybrid_gb300")
    shapes = [((32, 32, 32), 8, 0.6, 0.2, 21), ((16, 16, 16), 8, 0.4, 0.5, 22), ((16, 16, 24), 8, 0.9, 0.05, 23),
              ((16, 24, 16), 8, 0.3, 1.0, 24)]
    params, nions, loaders = [], [], []
    for r, (N, ppc, Ex, nu, seed) in enumerate(shapes):
        params.append(chy.params_for(N, precision=chy.PRECISION["mixed"], E0=(Ex, 0.0, 0.0), nui=nu, ksp_rtol=1e-10,
                                     pc_type=chy.PC["mg"], sort_period=4, seed=seed, run=r))
        nions.append(N[0] * N[1] * N[2] * ppc)
        loaders.append(chy.loader(amp=(0.02, 0.0, 0.01), phase=tuple(chy.mode_phases(seed, r))))
    phis = []
    for big in (0, 16, 8):
        with chy.Batch(params, nions) as b:
            try:
                b.set_tuning(4, 2, big)
            except chy.HybridError:
                assert big == 16  # clusters of 16 CTAs refused by the device
                continue
            b.load(loaders)
            b.initialize()
            first = [b.phi(r) for r in range(len(params))]
            info = b.step(0, 2)
            assert all(i["status"] == 0 for i in info)
            phis.append((first, [b.phi(r) for r in range(len(params))]))
    assert len(phis) >= 2
    # the same moments solved to rtol 1e-10 either way; after two steps the
    # ions have also moved on slightly different potentials
    for first, later in phis[1:]:
        for r in range(len(params)):
            assert _rel(first[r], phis[0][0][r]) < 1e-8, (r, _rel(first[r], phis[0][0][r]))
            assert _rel(later[r], phis[0][1][r]) < 1e-5, (r, _rel(later[r], phis[0][1][r]))


@pytest.mark.gpu
def test_batch_sorting_does_not_change_the_runs(chy):
    """As for one run: a batch that sorts after every step (the scatter inside
    the step's deposit) equals, bit for bit, one that does not sort in the same
    4 steps (period 5): every run's ions by id, moments and phi."""
    out = []
    for period in (1, 5):
        params, nions, loaders = _runs(chy)
        for p in params:
            p.sort_period = period
        with chy.Batch(params, nions) as b:
            b.load(loaders)
            b.initialize()
            b.step(0, 4)
            out.append([(b.moments(r), b.phi(r), *b.download(r)) for r in range(len(params))])
    for ra, rb in zip(*out):
        for a, c in zip(ra, rb):
            assert np.array_equal(a, c)


@pytest.mark.gpu
def test_batch_autotune_cache_across_batches(chy, tmp_path):
    """ch_batch_autotune_cached: the first batch of a class is timed and its
    launch shape appended to the cache file; a second batch of the same class
    (another process would read the same file) takes the stored shape without
    timing; a batch of another class is timed again."""
    cache = str(tmp_path / "tuning.jsonl")
    params, nions, loaders = _runs(chy)
    shapes = []
    for k in range(2):
        with chy.Batch(params, nions) as b:
            b.load(loaders)
            b.initialize()
            t = b.autotune(cache=cache)
            assert t["cached"] == (k == 1), t
            assert b.tuning()["cluster"] == t["cluster"]
            b.step(0, 1)
            shapes.append((t["cluster"], t["pass_ctas_per_sm"], t["cluster_big"]))
    assert shapes[0] == shapes[1]
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and '"key": "' in lines[0]
    # three runs instead of four: another class
    with chy.Batch(params[:3], nions[:3]) as b:
        b.load(loaders[:3])
        b.initialize()
        assert not b.autotune(cache=cache)["cached"]
    assert len(open(cache).read().splitlines()) == 2
