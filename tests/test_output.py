"""Asynchronous output (OutputHDF5, src/fileio.c:73-126, without HDF5): the
files written beside the following steps hold exactly the fields of the
step they were queued at, under the reference's dataset names."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_output_matches_the_fields_of_its_step(chy, tmp_path):
    p = chy.params_for((12, 10, 8), precision=chy.PRECISION["mixed"], pc_type=chy.PC["mg"])
    stem = str(tmp_path / "run")
    expect = {}
    with chy.Hybrid(p) as h:
        h.load(12 * 10 * 8 * 16, chy.loader(amp=(0.05, 0.0, 0.0)))
        h.output_open(stem)
        nodes = h.CollectVlasovQuantities()
        phi = h.ComputePotential()
        h.output("-initial")
        expect["-initial"] = (nodes, h.rhs(), phi)
        for it in range(3):
            h.step(it, 1)
            h.output(f"-{it:03d}")  # queued; the next step runs meanwhile
            expect[f"-{it:03d}"] = (h.CollectVlasovQuantities(), h.rhs(), h.phi())
            # CollectVlasovQuantities above redeposits the same ions: same moments
        assert h.output_wait() == 4
    for insert, (nodes, rhs, phi) in expect.items():
        out = chy.read_output(stem + insert)
        assert sorted(out) == sorted(["density", "x flux", "y flux", "z flux", "rhs", "potential"])
        for q, name in enumerate(["density", "x flux", "y flux", "z flux"]):
            assert np.array_equal(out[name].ravel(), nodes[:, q]), (insert, name)
        assert np.array_equal(out["rhs"].ravel(), rhs), insert
        assert np.array_equal(out["potential"].ravel(), phi), insert


def test_output_needs_open_and_fields(chy):
    p = chy.params_for((8, 8, 8))
    with chy.Hybrid(p) as h:
        with pytest.raises(chy.HybridError):
            h.output("-x")
