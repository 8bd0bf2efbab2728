"""Transfers through page-locked host arrays.  Arrays registered with
ch_host_register are read and written by the GPU directly (the conversion
kernels read them, a copy kernel writes them); other arrays go through
staging copies.  Both routes must give the same ions bit for bit, and a view
that is not 16-byte aligned inside a registered range must take the staged
route."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_registered_and_plain_transfers_agree(chy, precision):
    p = chy.params_for((16, 12, 20), precision=chy.PRECISION[precision])
    n = 16 * 12 * 20 * 8
    with chy.Hybrid(p) as h:
        h.load(n, chy.loader(amp=(0.05, 0.0, 0.0)))
        pos0, vel0 = h.download()
    outs = []
    for registered in (False, True):
        pos, vel = pos0.copy(), vel0.copy()
        if registered:
            chy.host_register(pos)
            chy.host_register(vel)
        try:
            with chy.Hybrid(p) as h:
                h.upload(pos, vel)
                h.CollectVlasovQuantities(copy=False)
                h.ComputePotential(copy=False)
                h.step(0, 2)
                a = np.zeros_like(pos)
                b = np.zeros_like(vel)
                if registered:
                    chy.host_register(a)
                    chy.host_register(b)
                try:
                    h.download(a, b)
                finally:
                    if registered:
                        chy.host_unregister(a)
                        chy.host_unregister(b)
                outs.append((a, b))
        finally:
            if registered:
                chy.host_unregister(pos)
                chy.host_unregister(vel)
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_misaligned_view_of_a_registered_range_is_staged(chy):
    p = chy.params_for((8, 8, 8), precision=chy.PRECISION["mixed"])
    n = 8 * 8 * 8 * 4
    with chy.Hybrid(p) as h:
        h.load(n, chy.loader())
        pos, vel = h.download()
    # the same data at an 8-byte offset inside a larger registered block
    big = np.zeros(2 * n * 4 + 2)
    chy.host_register(big)
    try:
        view_p = big[1:1 + n * 4].reshape(n, 4)
        view_p[:] = pos
        with chy.Hybrid(p) as h:
            h.upload(view_p, vel)
            a, b = h.download()
        assert np.array_equal(a, pos) and np.array_equal(b, vel)
    finally:
        chy.host_unregister(big)


@pytest.mark.parametrize("extra,period", [(0, 3), (7, 3), (7, 1)])  # 7: partial last warp and copy chunks
def test_round_trip_through_registered_arrays_keeps_the_run(chy, extra, period):
    """A download into registered arrays followed by an upload of the same
    arrays puts every ion back into its slot (no sort); a plain round trip
    re-sorts.  The order of the ions does not enter any result (integer
    deposit sums, per-ion draws), so both runs stay identical bit for bit.
    Sort period 1: every step ends with a sort."""
    p = chy.params_for((16, 12, 20), precision=chy.PRECISION["mixed"], nui=0.4, sort_period=period)
    n = 16 * 12 * 20 * 8 + extra
    outs = []
    for registered in (False, True):
        with chy.Hybrid(p) as h:
            h.load(n, chy.loader(amp=(0.05, 0.02, 0.0)))
            h.CollectVlasovQuantities(copy=False)
            h.ComputePotential(copy=False)
            h.step(0, 2)
            pos, vel = np.zeros((n, 4)), np.zeros((n, 4))
            if registered:
                chy.host_register(pos)
                chy.host_register(vel)
            try:
                for s in range(2, 6):
                    h.download(pos, vel)
                    h.upload(pos, vel)
                    h.step(s, 1)
                h.download(pos, vel)
                outs.append((pos.copy(), vel.copy(), h.CollectVlasovQuantities(), h.phi()))
            finally:
                if registered:
                    chy.host_unregister(pos)
                    chy.host_unregister(vel)
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision,extra,period", [("mixed", 0, 3), ("mixed", 7, 3), ("fp64", 7, 3), ("mixed", 7, 1)])
def test_step_host_equals_upload_step_download(chy, precision, extra, period):
    """ch_step_host, whose download overlaps the last step's deposit and
    potential solve (started after the deposit, from the new order, on a sort
    step), leaves the host arrays and the device state exactly as upload,
    ch_step and download do: with plain and registered arrays, one or two
    steps per call, sort steps (every 3rd) last in a call.  The FP64 form
    downloads after the steps.  Sort period 1 (mixed): every step ends with a
    sort, so every call's download starts from the new order."""
    p = chy.params_for((16, 12, 20), precision=chy.PRECISION[precision], nui=0.4, sort_period=period)
    n = 16 * 12 * 20 * 8 + extra
    outs = []
    for mode in ("separate", "step_host", "step_host_registered"):
        with chy.Hybrid(p) as h:
            h.load(n, chy.loader(amp=(0.05, 0.02, 0.0)))
            h.CollectVlasovQuantities(copy=False)
            h.ComputePotential(copy=False)
            h.step(0, 1)
            pos, vel = h.download()
            registered = mode == "step_host_registered"
            if registered:
                chy.host_register(pos)
                chy.host_register(vel)
            try:
                s = 1
                for nsteps in (1, 1, 2, 1, 1):  # the calls starting at steps 2 and 5 end with a sort
                    if mode == "separate":
                        h.upload(pos, vel)
                        h.step(s, nsteps)
                        h.download(pos, vel)
                    else:
                        h.step_host(pos, vel, s, nsteps)
                    s += nsteps
                outs.append((pos.copy(), vel.copy(), h.CollectVlasovQuantities(), h.phi()))
            finally:
                if registered:
                    chy.host_unregister(pos)
                    chy.host_unregister(vel)
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(a, b)


def test_step_host_rejects_bad_calls(chy):
    """ch_step_host wants ions on the device (their count sizes the host
    arrays) and at least one step."""
    p = chy.params_for((8, 8, 8), precision=chy.PRECISION["mixed"])
    with chy.Hybrid(p) as h:
        pos = np.zeros((8, 4))
        with pytest.raises(chy.HybridError):
            chy._check(chy.lib().ch_step_host(h._h, 0, 1, pos.ctypes.data, pos.ctypes.data, None))
        h.load(8 * 8 * 8 * 4, chy.loader())
        h.CollectVlasovQuantities(copy=False)
        h.ComputePotential(copy=False)
        pos, vel = h.download()
        with pytest.raises(chy.HybridError):
            h.step_host(pos, vel, 0, 0)


@pytest.mark.parametrize("nu", [0.4, 0.0])
def test_step_host_after_the_host_changed_the_ions(chy, nu):
    """Once the host arrays hold the ions in id order, ch_step_host pushes
    them straight from the host arrays and writes the result back in the
    same launch, using the collision-rate normaliser S of the previous step.
    A host that changes velocities between calls changes S: the call then
    runs the step again the ordinary way.  Changed positions need no rerun.
    Either way the host arrays, moments and phi equal those of upload,
    ch_step and download, bit for bit, with sort steps inside the calls;
    arrays from ch_host_alloc and registered numpy arrays give the same."""
    p = chy.params_for((16, 12, 20), precision=chy.PRECISION["mixed"], nui=nu, mn=1.0 if nu > 0 else 0.0,
                       sort_period=3)
    n = 16 * 12 * 20 * 8 + 5
    outs = []
    for mode in ("separate", "registered", "host_alloc"):
        with chy.Hybrid(p) as h:
            h.load(n, chy.loader(amp=(0.05, 0.02, 0.0)))
            h.CollectVlasovQuantities(copy=False)
            h.ComputePotential(copy=False)
            h.step(0, 1)
            held = []
            if mode == "host_alloc":
                held = [chy.HostArray((n, 4)), chy.HostArray((n, 4))]
                pos, vel = held[0].a, held[1].a
                h.download(pos, vel)
            else:
                pos, vel = h.download()
            if mode == "registered":
                chy.host_register(pos)
                chy.host_register(vel)
            h.set_profiling(True)
            try:
                s = 1
                for call, nsteps in enumerate((1, 1, 2, 1, 1, 3)):
                    if call == 2:
                        vel[::97, 0] *= 1.01   # the host edits some velocities
                    if call == 4:
                        pos[::89, 1] += 0.25    # and later some positions
                    if mode == "separate":
                        h.upload(pos, vel)
                        h.step(s, nsteps)
                        h.download(pos, vel)
                    else:
                        h.step_host(pos, vel, s, nsteps)
                    s += nsteps
                prof = h.profile()
                outs.append((pos.copy(), vel.copy(), h.CollectVlasovQuantities(), h.phi()))
            finally:
                if mode == "registered":
                    chy.host_unregister(pos)
                    chy.host_unregister(vel)
                del pos, vel
                for a in held:
                    a.free()
            if mode != "separate" and nu > 0:
                # every call after the first streams the host arrays; only
                # the call after the velocity edit runs its step again
                assert prof["host_push_calls"] >= 5, prof
                assert prof["host_push_reruns"] == 1, prof
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(a, b)
