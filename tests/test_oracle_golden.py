"""The CPU oracle against the reference's own outputs (tests/golden) and
against known answers.  CPU only."""
import numpy as np
import pytest

GRIDS = ["g8", "g15x10x8"]


def _case(po, golden, tag, **kw):
    m = golden[f"{tag}_meta"]
    N = tuple(int(v) for v in m[0:3])
    L = tuple(float(v) for v in m[3:6])
    p = po.default_params(N, L, **kw)
    pos = golden[f"{tag}_pos"]
    vel = golden[f"{tag}_vel"]
    ions = po.Ions(pos.shape[0])
    ions.a[0:3] = pos.T
    ions.a[3:6] = vel.T
    return p, ions, N


def test_philox_known_answers(po):
    # Random123 known-answer vectors for Philox4x32-10
    assert po.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert po.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert po.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("tag", GRIDS)
def test_collect_matches_reference(po, golden, tag):
    p, ions, N = _case(po, golden, tag)
    mine = po.collect(p, ions)
    ref = golden[f"{tag}_collect1"]
    assert np.abs(mine - ref).max() <= 1e-13 * np.abs(ref).max()
    # total weight is the ion count (CIC weights sum to 1)
    assert abs(mine[0::4].sum() - ions.np) < 1e-9
    # as-written accumulation across calls (D6)
    acc = po.collect(p, ions, nodes=mine.copy(), accumulate=True)
    ref2 = golden[f"{tag}_collect2"]
    assert np.abs(acc - ref2).max() <= 1e-13 * np.abs(ref2).max()


@pytest.mark.parametrize("tag", GRIDS)
@pytest.mark.parametrize("ki,kappa", [(0, (0.0, 0.0, 0.0)), (1, (0.3, -0.2, 1.0))])
@pytest.mark.parametrize("lt", [0, 1, 2])
def test_lhs_rows_match_reference(po, golden, tag, ki, kappa, lt):
    p, ions, N = _case(po, golden, tag, kappa_e=kappa, lhs_type=lt)
    n = golden[f"{tag}_collect1"][0::4]
    cols = golden[f"{tag}_lhs{lt}_k{ki}_cols"]
    vals = golden[f"{tag}_lhs{lt}_k{ki}_vals"]
    Nn = n.size
    A = np.zeros((Nn, Nn))
    for r in range(Nn):
        for q in range(cols.shape[1]):
            A[r, cols[r, q]] += vals[r, q]
    x = np.random.default_rng(3).standard_normal(Nn)
    y = po.apply(p, n, x)
    assert np.abs(A @ x - y).max() <= 1e-13 * np.abs(A).max() * np.abs(x).max() * 19
    if lt == 2:
        # row-by-row values in the reference's stencil order (src/lhs.c:7-106)
        mv, mc = po.lhs_rows(p, n)
        for r in range(0, Nn, max(1, Nn // 37)):
            ref = {int(c): v for c, v in zip(cols[r], vals[r])}
            got = {}
            for c, v in zip(mc[r], mv[r]):
                got[int(c)] = got.get(int(c), 0.0) + v
            assert set(ref) == set(got)
            for c in ref:
                assert abs(ref[c] - got[c]) <= 1e-13 * max(1.0, abs(ref[c]))
    # constant null space: A 1 = 0
    if lt != 0:
        assert np.abs(po.apply(p, n, np.ones(Nn))).max() < 1e-12 * np.abs(A).max()


@pytest.mark.parametrize("tag", GRIDS)
@pytest.mark.parametrize("ki,kappa", [(0, (0.0, 0.0, 0.0)), (1, (0.3, -0.2, 1.0))])
@pytest.mark.parametrize("rt", [0, 1, 2])
def test_rhs_matches_reference(po, golden, tag, ki, kappa, rt):
    nodes = golden[f"{tag}_collect1"]
    ref = golden[f"{tag}_rhs{rt}_k{ki}"]
    scale = max(np.abs(ref).max(), 1e-300)
    # as written: d2Fdyz uses the x-z stencil (D8)
    p, _, _ = _case(po, golden, tag, kappa_e=kappa, rhs_type=rt, E0=(0.5, 0.1, -0.2), cth=1.0, cG=0.1,
                    faithful=po.CH_FAITHFUL[8])
    b = po.rhs(p, nodes)
    assert np.abs(b - ref).max() <= 1e-12 * scale + 1e-14
    # corrected default differs from the reference exactly when R_yz or R_zy != 0
    p.faithful = 0
    b0 = po.rhs(p, nodes)
    if rt == 2 and ki == 1:
        assert np.abs(b0 - ref).max() > 1e-6 * scale
    else:
        assert np.abs(b0 - ref).max() <= 1e-12 * scale + 1e-14


@pytest.mark.parametrize("tag", GRIDS)
def test_difference_vector_matches_reference(po, golden, tag):
    p, _, N = _case(po, golden, tag)
    phi = golden[f"{tag}_dv_phi"]
    pts = golden[f"{tag}_dv_pts"]
    ref = golden[f"{tag}_dv_f"].reshape(-1, 3)
    fl = po.CH_FAITHFUL[3] | po.CH_FAITHFUL[4]
    got = np.array([po.difference_vector(p, phi, *pt, faithful=fl) for pt in pts])
    assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("tag", GRIDS)
def test_calculus_stencils(po, golden, tag):
    """The RHS's finite differences reproduce the reference's src/calculus.c
    helpers: checked through the RHS of a field put in each moment slot."""
    p, _, N = _case(po, golden, tag)
    F = golden[f"{tag}_cal_F"]
    cal = golden[f"{tag}_cal"]
    Nn = F.size
    d = np.array([p.x1 / N[0], p.y1 / N[1], p.z1 / N[2]])
    Fg = F.reshape(N[2], N[1], N[0])
    roll = lambda a, s, ax: np.roll(a, -s, axis=ax)  # noqa: E731
    dx = (roll(Fg, 1, 2) - roll(Fg, -1, 2)) / (2 * d[0])
    dyy = (roll(Fg, 1, 1) - 2 * Fg + roll(Fg, -1, 1)) / d[1] ** 2
    dxy = (roll(roll(Fg, 1, 2), 1, 1) - roll(roll(Fg, -1, 2), 1, 1) - roll(roll(Fg, 1, 2), -1, 1)
           + roll(roll(Fg, -1, 2), -1, 1)) / (4 * d[0] * d[1])
    assert np.allclose(cal[:, 0], dx.ravel(), rtol=0, atol=1e-12)
    assert np.allclose(cal[:, 4], dyy.ravel(), rtol=0, atol=1e-11)
    assert np.allclose(cal[:, 6], dxy.ravel(), rtol=0, atol=1e-12)
    # d2Fdyz as written equals d2Fdxz (D8)
    assert np.array_equal(cal[:, 10], cal[:, 8] * (4 * d[0] * d[2]) / (4 * d[1] * d[2]) * 1.0) or \
        np.allclose(cal[:, 10] * (4 * d[1] * d[2]), cal[:, 8] * (4 * d[0] * d[2]), atol=1e-12)
    assert Nn == cal.shape[0]


@pytest.mark.parametrize("tag", GRIDS)
def test_update_positions_as_written_is_noop(po, golden, tag):
    p, ions, _ = _case(po, golden, tag)
    assert np.array_equal(golden[f"{tag}_moved"], golden[f"{tag}_pos"])
    before = ions.a[0:3].copy()
    p.faithful = po.CH_FAITHFUL[5]
    po.update_positions(p, ions)
    assert np.array_equal(ions.a[0:3], before)
    p.faithful = 0
    po.update_positions(p, ions)
    assert not np.array_equal(ions.a[0:3], before)
    assert (ions.a[0] >= 0).all() and (ions.a[0] < p.x1).all()
