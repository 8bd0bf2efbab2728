"""The reference's --density-type placements (src/particles.c:9-132,
src/distributions.c:33-232) on the device (ch_particles_load_placed) and in
the oracle (orc_load_placed).

CPU: the oracle's Sobol points are the standard unscrambled Sobol sequence
(Joe & Kuo directions, Gray-code order) as SciPy generates it; the rejection
sampler's x marginal passes a Kolmogorov-Smirnov test against
n = 1 + 0.25 sin(2 pi x); uniform placement fills every cell equally.
GPU: the device loader gives the oracle's positions bit for bit in the FP64
form (velocities to 1e-12, transcendental functions differ in the last bit)
and within one FP32 offset step in the mixed form; the placements the
reference leaves unimplemented are refused as it refuses them."""
import numpy as np
import pytest

SOBOL, UNIFORM, SINUSOIDAL = 0, 3, 4


def sin_cdf(x, L):
    """CDF of n = 1 + 0.25 sin(2 pi x) over [0, L)."""
    return (x + 0.25 * (1.0 - np.cos(2 * np.pi * x)) / (2 * np.pi)) / (L + 0.25 * (1 - np.cos(2 * np.pi * L)) /
                                                                        (2 * np.pi))


def test_oracle_sobol_is_the_standard_sequence(po):
    qmc = pytest.importorskip("scipy.stats").qmc
    n = 4096
    q = po.default_params((8, 8, 8), L=(1.0, 1.0, 1.0))
    ions = po.load_placed(q, po.make_loader(), n, SOBOL)
    ref = qmc.Sobol(d=3, scramble=False).random(n + 1)[1:]  # point 0 is the origin
    d = 1.0 / 8
    # v = r (L + d) - d/2, clamped to [p0 + 0.01 d, p1 - 0.01 d] (src/distributions.c:117-125)
    v = ref * (1.0 + d) - 0.5 * d
    expect = np.where(v < 0.0, 0.01 * d, np.where(v > 1.0, 1.0 - 0.01 * d, v))
    assert np.array_equal(ions.a[0:3].T, expect)


def test_oracle_rejection_sampler_follows_the_sinusoid(po):
    sst = pytest.importorskip("scipy.stats")
    q = po.default_params((8, 4, 4), seed=3)
    n = 200000
    ions = po.load_placed(q, po.make_loader(), n, SINUSOIDAL)
    x = ions.a[0]
    assert (x >= 0).all() and (x < 8).all()
    ks = sst.kstest(x, lambda t: sin_cdf(t, 8.0))
    assert ks.pvalue > 1e-3, ks
    # a uniform x fails the same test: the sampler does shape the density
    assert sst.kstest(x, lambda t: t / 8.0).pvalue < 1e-6


def test_oracle_uniform_fills_every_cell(po):
    q = po.default_params((6, 5, 4))
    ions = po.load_placed(q, po.make_loader(), 6 * 5 * 4 * 3, UNIFORM)
    cells = (np.floor(ions.a[2]) * 5 + np.floor(ions.a[1])) * 6 + np.floor(ions.a[0])
    assert np.array_equal(np.bincount(cells.astype(int), minlength=120), np.full(120, 3))
    assert np.array_equal(ions.a[0] - np.floor(ions.a[0]), np.full(ions.np, 0.5))
    with pytest.raises(ValueError):
        po.load_placed(q, po.make_loader(), 121, UNIFORM)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["flat-sobol", "uniform", "sinusoidal"])
def test_device_placement_matches_oracle(chy, po, precision, kind):
    N, L = (16, 12, 10), (16.0, 6.0, 10.0)
    p = chy.params_for(N, L, precision=chy.PRECISION[precision], seed=9)
    q = po.params_from(p)
    n = 16 * 12 * 10 * 5
    lo = dict(vT=(1.0, 0.8, 1.2), v0=(0.1, 0.0, -0.2))
    with chy.Hybrid(p) as h:
        h.load_placed(n, chy.loader(**lo), kind)
        pos, vel = h.download()
    ref = po.load_placed(q, po.make_loader(**lo), n, chy.DENSITY[kind])
    rp, rv = ref.aos()
    if precision == "fp64":
        assert np.array_equal(pos[:, :3], rp[:, :3])
        assert np.abs(vel[:, :3] - rv[:, :3]).max() < 1e-12 * np.abs(rv).max()
    else:
        d = np.array([L[i] / N[i] for i in range(3)])
        assert (np.abs(pos[:, :3] - rp[:, :3]) <= 2.0 ** -23 * d).all()
        assert np.abs(vel[:, :3] - rv[:, :3]).max() < 2e-7 * np.abs(rv).max()


@pytest.mark.gpu
def test_device_placement_refusals(chy):
    p = chy.params_for((8, 8, 8))
    with chy.Hybrid(p) as h:
        for kind in ("flat-reverse", "flat-normal", "gaussian"):
            with pytest.raises(chy.HybridError) as e:
                h.load_placed(1000, chy.loader(), kind)
            assert e.value.status == -10 and b"Not implemented" in chy.lib().ch_last_error()
        with pytest.raises(chy.HybridError) as e:
            h.load_placed(513, chy.loader(), "uniform")
        assert e.value.status == -1


@pytest.mark.gpu
def test_device_sobol_run_steps(chy):
    """A run started from the default (flat-sobol) placement steps normally:
    the moments sum to the ion count and the solve meets its tolerance."""
    p = chy.params_for((16, 16, 16), precision=chy.PRECISION["mixed"], pc_type=chy.PC["mg"], ksp_rtol=1e-10)
    with chy.Hybrid(p) as h:
        h.load_placed(16 ** 3 * 8, chy.loader(), "flat-sobol")
        m = h.CollectVlasovQuantities()
        h.ComputePotential(copy=False)
        info = h.step(0, 2)
    assert abs(m[:, 0].sum() - 16 ** 3 * 8) < 1e-6 * 16 ** 3 * 8
    assert info["rnorm"] <= 1e-10 * info["bnorm"] * 1.01
