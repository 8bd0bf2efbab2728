"""The C-ABI library loads and exports every symbol its header declares;
host-side logic that needs no GPU.  CPU only: no CUDA call is made."""
import ctypes as C
import os
import re

import numpy as np

from conftest import REPO


def _declared(header):
    txt = open(os.path.join(REPO, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ch_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(chy):
    lib = C.CDLL(chy.LIBPATH)
    names = _declared("chybrid.h")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_params_layout_matches_c(chy, po):
    size = po.lib().orc_sizeof_params()
    assert C.sizeof(chy.Params) == size
    assert C.sizeof(po.Params) == size
    for (a, ta), (b, tb) in zip(chy.Params._fields_, po.Params._fields_):
        assert a == b and getattr(chy.Params, a).offset == getattr(po.Params, b).offset


def test_params_default_is_reference_default(chy):
    p = chy.default_params()
    assert (p.Nx, p.Ny, p.Nz) == (7, 7, 7)          # src/setup.c:10-12
    assert p.lhs_type == chy.LHS["full"] and p.rhs_type == chy.RHS["full"]  # src/parameters.c:66,72
    assert p.dt == 1.0 / p.nui                         # src/parameters.c:417
    assert p.mn == p.mi                                # src/parameters.c:337
    assert p.ksp_rtol == 1e-5 and p.ksp_max_it == 10000
    assert chy.lib().ch_abi_version() == 1


def test_host_philox_matches_oracle(chy, po):
    rng = np.random.default_rng(0)
    for _ in range(50):
        ctr = [int(x) for x in rng.integers(0, 2**32, 4)]
        key = [int(x) for x in rng.integers(0, 2**32, 2)]
        assert chy._philox4x32_10(ctr, key) == po.philox(ctr, key)
    assert chy.mode_phases(7) == po.mode_phases(7)


def test_batch_rejects_unsupported_runs_before_touching_the_device(chy):
    """ch_batch_create validates every run on the host first (no CUDA call)."""
    good = chy.params_for((16, 16, 16), precision=chy.PRECISION["mixed"], pc_type=chy.PC["mg"])
    cases = [
        (dict(precision=chy.PRECISION["fp64"]), -10),      # mixed form only
        (dict(pc_type=chy.PC["jacobi"]), -10),             # CG + multigrid only
        (dict(ksp_type=chy.KSP["bcgs"]), -10),
        (dict(kappa_e=(0.1, 0.0, 0.0)), -10),              # A non-symmetric: CG does not apply
        (dict(sort_period=2), -1),                         # must agree across runs
        (dict(Nx=2), -1),
    ]
    for kw, status in cases:
        bad = chy.params_for((16, 16, 16), precision=chy.PRECISION["mixed"], pc_type=chy.PC["mg"])
        for k, v in kw.items():
            if k == "kappa_e":
                bad.kappa_e[:] = v
            else:
                setattr(bad, k, v)
        arr = (chy.Params * 2)(good, bad)
        nions = (C.c_int64 * 2)(1000, 1000)
        h = C.c_void_p()
        rc = chy.lib().ch_batch_create(C.cast(arr, C.c_void_p), C.cast(nions, C.c_void_p), 2, -1, C.byref(h))
        assert rc == status, (kw, rc, chy.lib().ch_last_error())
        assert not h.value
    arr = (chy.Params * 1)(good)
    rc = chy.lib().ch_batch_create(C.cast(arr, C.c_void_p), C.cast((C.c_int64 * 1)(0), C.c_void_p), 1, -1,
                                   C.byref(C.c_void_p()))
    assert rc == -1 and b"no ions" in chy.lib().ch_last_error()


def test_noalloc_deposit_rejects_bad_arguments_before_touching_the_device(chy):
    """ch_collect_moments_noalloc checks every argument on the host before its
    first CUDA call: an axis so long that the node count would wrap int64
    (2^22 per axis), a grid beyond its static scratch, a deposit scale outside
    the FP64 form's [1, 62], an empty domain, np < 0 and null pointers."""
    f = chy.lib().ch_collect_moments_noalloc
    f.argtypes = [C.c_void_p] + [C.c_void_p] * 6 + [C.c_int64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int32
    fake = C.c_void_p(256)  # never dereferenced: every case fails its checks first
    ions = [fake] * 6

    def call(p, np_=10, out=fake, ptrs=ions):
        return f(C.byref(p), *ptrs, np_, out, None)

    cases = []
    p = chy.params_for((8, 8, 8))
    p.Nx = p.Ny = p.Nz = 1 << 22  # 2^66 nodes: wraps to 0 in int64
    cases.append((p, {}, b"exceeds the scratch"))
    cases.append((chy.params_for((128, 64, 64)), {}, b"at most 262144 nodes"))
    cases.append((chy.params_for((1 << 19, 3, 3)), {}, b"exceeds the scratch"))
    for s in (0.5, 63.0, -1.0, float("nan")):
        cases.append((chy.params_for((8, 8, 8), deposit_scale_log2=s), {}, b"deposit_scale_log2"))
    p = chy.params_for((8, 8, 8))
    p.x1 = p.x0
    cases.append((p, {}, b"empty"))
    cases.append((chy.params_for((2, 8, 8)), {}, b"at least 3"))
    cases.append((chy.params_for((8, 8, 8)), dict(np_=-1), b"np < 0"))
    cases.append((chy.params_for((8, 8, 8)), dict(out=None), b"null"))
    cases.append((chy.params_for((8, 8, 8)), dict(ptrs=[fake] * 5 + [None]), b"null"))
    for p, kw, msg in cases:
        rc = call(p, **kw)
        assert rc == -1, (msg, rc)
        assert msg in chy.lib().ch_last_error(), (msg, chy.lib().ch_last_error())
