"""ch_collect_moments_noalloc: the deposit for callers that cannot allocate
device memory -- a host whose device memory all belongs to its own pool
allocator, or a time-critical loop that cannot absorb the device-wide
synchronisation of cudaMalloc/cudaFree.  The caller supplies device buffers
for the ions and the moments; the entry point's scratch is a fixed static
device array.

Checked through the C ABI against ch_collect_moments and against the CPU
oracle on two calls in a row (the second call must not see the first call's
sums), to the deposit tolerance of the other parity tests: 1e-12 relative,
norm-wise.  An ion with a NaN velocity turns every output into NaN (the
asynchronous form of CH_ERR_NAN), and the call after it is clean again.
The argument checks are covered on the CPU (tests/test_abi_cpu.py).  The
file sorts last so that a stop-at-first-failure run has run every other
test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(chy):
    f = chy.lib().ch_collect_moments_noalloc
    f.argtypes = [C.c_void_p] + [C.c_void_p] * 6 + [C.c_int64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int32
    return f


def _ions(po, q, seed, n, amp):
    q.seed = seed
    return po.load(q, po.make_loader(amp=amp, vT=(1.0, 0.7, 1.3), v0=(0.1, -0.2, 0.0)), n)


def _call(chy, f, p, ions, out):
    import torch

    dev = [torch.from_numpy(np.ascontiguousarray(ions.a[k])).to("cuda:0") for k in range(6)]
    stream = torch.cuda.current_stream(0).cuda_stream
    torch.cuda.synchronize()
    rc = f(C.byref(p), *[t.data_ptr() for t in dev], ions.np, out.data_ptr(), stream)
    assert rc == 0, chy.lib().ch_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(4, -1).T.copy()  # (N, 4) GridNode order


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_deposit_matches_collect_moments_and_oracle(chy, po):
    import torch

    f = _noalloc(chy)
    p = chy.params_for((24, 16, 12), (24.0, 16.0, 12.0))
    q = po.params_from(p)
    N = p.Nx * p.Ny * p.Nz
    out = torch.empty(4 * N, dtype=torch.float64, device="cuda:0")
    for call, (seed, amp) in enumerate([(11, (0.2, 0.0, 0.0)), (12, (0.0, 0.1, 0.05))]):
        ions = _ions(po, q, seed, 40000 + 1000 * call, amp)
        pos, vel = ions.aos()
        with chy.Hybrid(p) as h:
            h.upload(pos, vel)
            ref = h.CollectVlasovQuantities()  # (N, 4) GridNode
        orc = po.collect(q, ions).reshape(N, 4)  # oracle nodes: GridNode (dof-4 interleaved)
        got = _call(chy, f, p, ions, out)
        assert np.array_equal(got, ref), (call, np.abs(got - ref).max())  # same fixed-point sums
        assert _rel(got, orc) < TOL, (call, _rel(got, orc))


def test_noalloc_flags_a_nonfinite_ion_with_nan_and_recovers(chy, po):
    import torch

    f = _noalloc(chy)
    p = chy.params_for((16, 16, 16))
    q = po.params_from(p)
    N = p.Nx * p.Ny * p.Nz
    out = torch.empty(4 * N, dtype=torch.float64, device="cuda:0")
    ions = _ions(po, q, 5, 20000, (0.1, 0.0, 0.0))
    bad = ions.copy()
    bad.a[4, 123] = np.nan  # one NaN velocity
    got = _call(chy, f, p, bad, out)
    assert np.isnan(got).all()
    huge = ions.copy()
    huge.a[0, 7] = 1e300  # finite, but no cell index fits
    assert np.isnan(_call(chy, f, p, huge, out)).all()
    clean = _call(chy, f, p, ions, out)  # the status word is cleared per call
    orc = po.collect(q, ions).reshape(N, 4)
    assert _rel(clean, orc) < TOL


def test_noalloc_rejects_grids_beyond_its_scratch(chy):
    f = _noalloc(chy)
    p = chy.params_for((128, 64, 64))  # 2^19 nodes > 2^18
    rc = f(C.byref(p), None, None, None, None, None, None, 0, C.c_void_p(1), None)
    assert rc == -1
    assert b"at most" in chy.lib().ch_last_error()
