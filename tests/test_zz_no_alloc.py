"""ch_collect_moments_noalloc: the deposit for callers that cannot allocate
device memory (a host whose device memory belongs to its own pool, launches
recorded into a CUDA graph, loops that cannot absorb cudaMalloc's device-wide
synchronisation).  The caller supplies device buffers for the ions and the
moments; the entry point's scratch is a fixed static device array.

Checked through the C ABI against ch_collect_moments on two calls in a row
(the second call must not see the first call's sums), to the deposit
tolerance of the other parity tests: 1e-12 relative, norm-wise.  The file
sorts last so that a stop-at-first-failure run has run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(chy):
    f = chy.lib().ch_collect_moments_noalloc
    f.argtypes = [C.c_void_p] + [C.c_void_p] * 6 + [C.c_int64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int32
    return f


def _ions(po, q, seed, n, amp):
    q.seed = seed
    return po.load(q, po.make_loader(amp=amp, vT=(1.0, 0.7, 1.3), v0=(0.1, -0.2, 0.0)), n)


def test_noalloc_deposit_matches_collect_moments(chy, po):
    import torch

    f = _noalloc(chy)
    p = chy.params_for((24, 16, 12), (24.0, 16.0, 12.0))
    q = po.params_from(p)
    N = p.Nx * p.Ny * p.Nz
    out = torch.empty(4 * N, dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream(0).cuda_stream
    for call, (seed, amp) in enumerate([(11, (0.2, 0.0, 0.0)), (12, (0.0, 0.1, 0.05))]):
        ions = _ions(po, q, seed, 40000 + 1000 * call, amp)
        pos, vel = ions.aos()
        with chy.Hybrid(p) as h:
            h.upload(pos, vel)
            ref = h.CollectVlasovQuantities()  # (N, 4) GridNode
        dev = [torch.from_numpy(np.ascontiguousarray(ions.a[k])).to("cuda:0") for k in range(6)]
        torch.cuda.synchronize()
        rc = f(C.byref(p), *[t.data_ptr() for t in dev], ions.np, out.data_ptr(), stream)
        assert rc == 0, chy.lib().ch_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(4, N).T
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 1e-12, (call, err)


def test_noalloc_rejects_grids_beyond_its_scratch(chy):
    f = _noalloc(chy)
    p = chy.params_for((128, 64, 64))  # 2^19 nodes > 2^18
    rc = f(C.byref(p), None, None, None, None, None, None, 0, C.c_void_p(1), None)
    assert rc == -1
    assert b"at most" in chy.lib().ch_last_error()
