"""ctypes bindings of the CPU oracle and of the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libref.so")
# Where the reference's sources lie (the same REF variable as oracle/Makefile);
# only the recipe that compiles them and the tests that read its headers use it.
REF = os.environ.get("REF", "/root/reference")
REF_SRC = os.path.join(REF, "src")

_dp = C.POINTER(C.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Params(C.Structure):
    """Mirror of ch_params (include/chybrid.h)."""

    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32), ("Nz", C.c_int32), ("precision", C.c_int32),
        ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
        ("x1", C.c_double), ("y1", C.c_double), ("z1", C.c_double),
        ("qi", C.c_double), ("mi", C.c_double), ("nui", C.c_double), ("dt", C.c_double),
        ("vi0", C.c_double * 3), ("viT", C.c_double * 3),
        ("mn", C.c_double), ("vnT", C.c_double), ("vn0", C.c_double * 3),
        ("B0", C.c_double * 3), ("E0", C.c_double * 3),
        ("kappa_e", C.c_double * 3), ("cth", C.c_double), ("cG", C.c_double),
        ("lhs_type", C.c_int32), ("rhs_type", C.c_int32), ("ksp_type", C.c_int32), ("pc_type", C.c_int32),
        ("ksp_rtol", C.c_double), ("ksp_atol", C.c_double), ("ksp_max_it", C.c_int32),
        ("nn_profile", C.c_int32), ("nn_center", C.c_double), ("nn_sigma", C.c_double), ("nn_floor", C.c_double),
        ("seed", C.c_uint64), ("run", C.c_uint32), ("faithful", C.c_uint32), ("push_E0", C.c_int32),
        ("sort_period", C.c_int32), ("deposit_scale_log2", C.c_double),
    ]


class Loader(C.Structure):
    _fields_ = [("amp", C.c_double * 3), ("phase", C.c_double * 3), ("v0", C.c_double * 3), ("vT", C.c_double * 3)]


class Particles(C.Structure):
    _fields_ = [("np", C.c_int64)] + [(n, _dp) for n in ("x", "y", "z", "vx", "vy", "vz")]


class Counters(C.Structure):
    _fields_ = [("Nc", C.c_int64), ("collisions", C.c_int64), ("refused", C.c_int64), ("expected", C.c_double)]


class State(C.Structure):
    _fields_ = [("p", Params), ("P", Particles), ("phi", _dp), ("nodes", _dp), ("rhs", _dp), ("n_frozen", _dp),
                ("sbar", C.c_double), ("solved_once", C.c_int)]


def build(ref: bool = False) -> None:
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True, stdout=subprocess.DEVNULL)
    if ref and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF}"], check=True, stdout=subprocess.DEVNULL)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_load.argtypes = [C.POINTER(Params), C.POINTER(Loader), C.POINTER(Particles)]
        L.orc_load_placed.argtypes = [C.POINTER(Params), C.POINTER(Loader), C.c_int, C.POINTER(Particles)]
        L.orc_difference_vector.argtypes = [C.POINTER(Params), _dp, C.c_double, C.c_double, C.c_double,
                                            C.c_uint32, _dp]
        L.orc_node_efield.argtypes = [C.POINTER(Params), _dp, _dp, _dp, _dp]
        L.orc_gmean.argtypes = [C.c_double, C.c_double]
        L.orc_gmean.restype = C.c_double
        L.orc_collision_count.argtypes = [C.POINTER(Params), C.c_int64]
        L.orc_collision_count.restype = C.c_int64
        L.orc_sbar.argtypes = [C.POINTER(Params), C.POINTER(Particles)]
        L.orc_sbar.restype = C.c_double
        L.orc_update_velocities.argtypes = [C.POINTER(Params), _dp, C.POINTER(Particles), C.c_int64, C.c_double,
                                            _dp, C.POINTER(Counters)]
        L.orc_update_positions.argtypes = [C.POINTER(Params), C.POINTER(Particles)]
        L.orc_collect.argtypes = [C.POINTER(Params), C.POINTER(Particles), _dp, C.c_int]
        L.orc_rhs.argtypes = [C.POINTER(Params), _dp, _dp]
        L.orc_lhs_row.argtypes = [C.POINTER(Params), _dp, C.c_int, C.c_int, C.c_int, _dp, C.POINTER(C.c_int64)]
        L.orc_apply.argtypes = [C.POINTER(Params), _dp, _dp, _dp]
        L.orc_solve.argtypes = [C.POINTER(Params), _dp, _dp, _dp, C.c_double, C.c_int, C.POINTER(C.c_int), _dp, _dp]
        L.orc_step.argtypes = [C.POINTER(State), C.c_int64, C.POINTER(Counters), C.POINTER(C.c_int), _dp, _dp]
        L.orc_initialize.argtypes = [C.POINTER(State), C.POINTER(C.c_int), _dp, _dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_adj_objective.argtypes = [C.POINTER(Params), C.POINTER(Loader), C.c_int64, C.c_int, C.c_int,
                                        C.c_double, C.c_double, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_double, _dp]
        L.orc_get_threads.restype = C.c_int
        L.orc_sizeof_params.restype = C.c_int64
        _lib = L
    return _lib


def ref():
    """The reference's own functions (None when the harness was not built)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REFLIB):
            return None
        R = C.CDLL(REFLIB)
        ip = C.POINTER(C.c_int)
        R.ref_collect.argtypes = [C.c_int] * 3 + [_dp, C.c_int, _dp, _dp, C.c_int, _dp]
        R.ref_update_positions.argtypes = [C.c_int] * 3 + [_dp, C.c_double, C.c_int, _dp, _dp]
        R.ref_difference_vector.argtypes = [C.c_int] * 3 + [_dp, C.c_int, _dp, _dp]
        R.ref_lhs.argtypes = [C.c_int] * 3 + [_dp, _dp, C.c_int, _dp, ip, ip, _dp]
        R.ref_rhs.argtypes = [C.c_int] * 3 + [_dp, _dp, _dp, C.c_double, C.c_double, C.c_int, _dp, _dp]
        R.ref_collisions.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, _dp, C.c_long, ip]
        R.ref_calculus.argtypes = [C.c_int] * 3 + [_dp, _dp, C.c_int, C.c_int, C.c_int, _dp]
        _ref = R
    return _ref


# ---------------------------------------------------------------- helpers
CH_FAITHFUL = {2: 1 << 2, 3: 1 << 3, 4: 1 << 4, 5: 1 << 5, 6: 1 << 6, 7: 1 << 7, 8: 1 << 8}


def default_params(N=(8, 8, 8), L=None, **kw) -> Params:
    """Normalised-unit defaults (e = kB = 1): unit spacing, Maxwellian ions
    with vT = 1, Omega_i = 1 along z, E0 = (0.5, 0, 0), nu = 0.1 with
    equal-mass neutrals (the 32^3 FP64 workload's physics) unless
    overridden."""
    p = Params()
    p.Nx, p.Ny, p.Nz = N
    L = L if L is not None else tuple(float(n) for n in N)
    p.x0 = p.y0 = p.z0 = 0.0
    p.x1, p.y1, p.z1 = L
    p.qi, p.mi = 1.0, 1.0
    p.nui, p.dt = 0.1, 0.05
    p.vi0[:] = (0.0, 0.0, 0.0)
    p.viT[:] = (1.0, 1.0, 1.0)
    p.mn, p.vnT = 1.0, 1.0
    p.vn0[:] = (0.0, 0.0, 0.0)
    p.B0[:] = (0.0, 0.0, 1.0)
    p.E0[:] = (0.5, 0.0, 0.0)
    p.kappa_e[:] = (0.0, 0.0, 0.0)
    p.cth, p.cG = 1.0, 0.1
    p.lhs_type, p.rhs_type = 2, 2
    p.ksp_type, p.pc_type = 0, 1
    p.ksp_rtol, p.ksp_atol, p.ksp_max_it = 1e-8, 0.0, 10000
    p.nn_profile, p.nn_center, p.nn_sigma, p.nn_floor = 0, 0.0, 1.0, 0.0
    p.seed, p.run, p.faithful, p.push_E0 = 1, 0, 0, 0
    p.sort_period, p.deposit_scale_log2 = 0, 0.0
    for k, v in kw.items():
        if isinstance(v, (tuple, list)):
            getattr(p, k)[:] = v
        else:
            setattr(p, k, v)
    return p


def mode_phases(seed: int, run: int = 0):
    """Random phases of the 3-mode density perturbation: 2 pi U from
    Philox(ctr = {m, 0xFFFFFFFF, 4 << 24, run}, key = seed)."""
    out = []
    for m in range(1, 4):
        r = philox([m, 0xFFFFFFFF, 4 << 24, run], [seed & 0xFFFFFFFF, seed >> 32])
        out.append(2.0 * np.pi * ((float(r[0]) + 0.5) * 2.0 ** -32))
    return out


def make_loader(amp=(0.01, 0.0, 0.0), phase=(0.0, 0.0, 0.0), v0=(0.0, 0.0, 0.0), vT=(1.0, 1.0, 1.0)) -> Loader:
    L = Loader()
    L.amp[:] = amp
    L.phase[:] = phase
    L.v0[:] = v0
    L.vT[:] = vT
    return L


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


class Ions:
    """SoA FP64 ions owned by numpy."""

    def __init__(self, np_: int):
        self.np = int(np_)
        self.a = np.zeros((6, self.np), dtype=np.float64)

    @classmethod
    def from_aos(cls, pos, vel):
        s = cls(pos.shape[0])
        s.a[0:3] = pos[:, 0:3].T
        s.a[3:6] = vel[:, 0:3].T
        return s

    def struct(self) -> Particles:
        P = Particles()
        P.np = self.np
        for i, n in enumerate(("x", "y", "z", "vx", "vy", "vz")):
            setattr(P, n, self.a[i].ctypes.data_as(_dp))
        return P

    def aos(self):
        pos = np.zeros((self.np, 4))
        vel = np.zeros((self.np, 4))
        pos[:, 0:3] = self.a[0:3].T
        vel[:, 0:3] = self.a[3:6].T
        return pos, vel

    def copy(self):
        s = Ions(self.np)
        s.a[:] = self.a
        return s


def load(p: Params, L: Loader, np_: int) -> Ions:
    s = Ions(np_)
    P = s.struct()
    lib().orc_load(C.byref(p), C.byref(L), C.byref(P))
    return s


def load_placed(p: Params, L: Loader, np_: int, density_type: int) -> Ions:
    """The reference's --density-type placements (0 flat-sobol, 3 uniform,
    4 sinusoidal rejection) with Maxwellian velocities."""
    s = Ions(np_)
    P = s.struct()
    rc = lib().orc_load_placed(C.byref(p), C.byref(L), int(density_type), C.byref(P))
    if rc:
        raise ValueError(f"orc_load_placed: status {rc}")
    return s


def collect(p: Params, ions: Ions, nodes=None, accumulate=False):
    N = p.Nx * p.Ny * p.Nz
    if nodes is None:
        nodes = np.zeros(4 * N)
    P = ions.struct()
    lib().orc_collect(C.byref(p), C.byref(P), _ptr(nodes), int(accumulate))
    return nodes


def rhs(p: Params, nodes):
    b = np.zeros(p.Nx * p.Ny * p.Nz)
    lib().orc_rhs(C.byref(p), _ptr(np.ascontiguousarray(nodes)), _ptr(b))
    return b


def apply(p: Params, n, x):
    y = np.zeros_like(x)
    lib().orc_apply(C.byref(p), _ptr(np.ascontiguousarray(n)), _ptr(np.ascontiguousarray(x)), _ptr(y))
    return y


def lhs_rows(p: Params, n):
    N = p.Nx * p.Ny * p.Nz
    vals = np.zeros((N, 19))
    cols = np.zeros((N, 19), dtype=np.int64)
    n = np.ascontiguousarray(n)
    v = np.zeros(19)
    c = np.zeros(19, dtype=np.int64)
    for k in range(p.Nz):
        for j in range(p.Ny):
            for i in range(p.Nx):
                lib().orc_lhs_row(C.byref(p), _ptr(n), i, j, k, _ptr(v), c.ctypes.data_as(C.POINTER(C.c_int64)))
                r = (k * p.Ny + j) * p.Nx + i
                vals[r] = v
                cols[r] = c
    return vals, cols


def solve(p: Params, n, b, phi0=None, rtol=None, maxit=None):
    N = p.Nx * p.Ny * p.Nz
    phi = np.zeros(N) if phi0 is None else np.array(phi0, dtype=np.float64)
    its = C.c_int()
    rn = C.c_double()
    bn = C.c_double()
    rc = lib().orc_solve(C.byref(p), _ptr(np.ascontiguousarray(n)), _ptr(np.ascontiguousarray(b)), _ptr(phi),
                         p.ksp_rtol if rtol is None else rtol, p.ksp_max_it if maxit is None else maxit,
                         C.byref(its), C.byref(rn), C.byref(bn))
    return phi, dict(rc=rc, its=its.value, rnorm=rn.value, bnorm=bn.value)


def adj_objective(p: Params, L: Loader, np_: int, nsteps: int, window: int, flux_weight: float, phi_weight: float,
                  events: dict, rtol: float) -> float:
    """The frozen-event objective of the GPU adjoint, replayed in FP64 on the
    CPU (theta enters through p.E0, p.vn0 and L.amp[0])."""
    st = np.ascontiguousarray(events["step"], dtype=np.int32)
    ion = np.ascontiguousarray(events["ion"], dtype=np.uint32)
    fl = np.ascontiguousarray(events["flags"], dtype=np.int32)
    data = np.ascontiguousarray(events["data"], dtype=np.float64)
    J = C.c_double()
    rc = lib().orc_adj_objective(C.byref(p), C.byref(L), int(np_), int(nsteps), int(window), float(flux_weight),
                                 float(phi_weight), len(st), st.ctypes.data, ion.ctypes.data, fl.ctypes.data,
                                 data.ctypes.data, float(rtol), C.byref(J))
    if rc:
        raise RuntimeError(f"orc_adj_objective: {rc}")
    return J.value


def difference_vector(p: Params, phi, X, Y, Z, faithful=0):
    f = np.zeros(3)
    lib().orc_difference_vector(C.byref(p), _ptr(np.ascontiguousarray(phi)), X, Y, Z, faithful, _ptr(f))
    return f


def update_velocities(p: Params, phi, ions: Ions, step: int, sbar: float):
    P = ions.struct()
    cnt = Counters()
    sn = C.c_double()
    rc = lib().orc_update_velocities(C.byref(p), _ptr(np.ascontiguousarray(phi)), C.byref(P), step, sbar,
                                     C.byref(sn), C.byref(cnt))
    return rc, sn.value, cnt


def update_positions(p: Params, ions: Ions):
    P = ions.struct()
    lib().orc_update_positions(C.byref(p), C.byref(P))


def sbar(p: Params, ions: Ions) -> float:
    P = ions.struct()
    return lib().orc_sbar(C.byref(p), C.byref(P))


class Run:
    """Whole-run oracle state (initial moments + first solve, then steps)."""

    def __init__(self, p: Params, ions: Ions):
        N = p.Nx * p.Ny * p.Nz
        self.ions = ions
        self.phi = np.zeros(N)
        self.nodes = np.zeros(4 * N)
        self.rhs = np.zeros(N)
        self.nfz = np.zeros(N)
        self.s = State()
        self.s.p = p
        self.s.P = ions.struct()
        self.s.phi, self.s.nodes, self.s.rhs, self.s.n_frozen = map(_ptr, (self.phi, self.nodes, self.rhs, self.nfz))

    def initialize(self):
        its, rn, bn = C.c_int(), C.c_double(), C.c_double()
        rc = lib().orc_initialize(C.byref(self.s), C.byref(its), C.byref(rn), C.byref(bn))
        return rc, dict(its=its.value, rnorm=rn.value, bnorm=bn.value)

    def step(self, step: int):
        its, rn, bn = C.c_int(), C.c_double(), C.c_double()
        cnt = Counters()
        rc = lib().orc_step(C.byref(self.s), step, C.byref(cnt), C.byref(its), C.byref(rn), C.byref(bn))
        return rc, dict(its=its.value, rnorm=rn.value, bnorm=bn.value, Nc=cnt.Nc, collisions=cnt.collisions,
                        refused=cnt.refused, expected=cnt.expected)

    @property
    def sbar(self):
        return self.s.sbar


def params_from(src) -> Params:
    """Copies a product ch_params mirror (same field names) into the oracle's."""
    p = Params()
    for name, _ in Params._fields_:
        v = getattr(src, name)
        if hasattr(v, "__len__"):
            getattr(p, name)[:] = list(v)
        else:
            setattr(p, name, v)
    return p
