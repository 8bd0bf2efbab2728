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
