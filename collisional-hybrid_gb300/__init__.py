"""GB300-native hybrid-PIC hot path: Python host mirror of the C ABI.

The reference drives one step as (src/hybrid.c:101-123)::

    UpdateVelocities(ksp, &ctx)        # src/particles.c:628
    UpdatePositions(&ctx)              # src/particles.c:647
    CollectVlasovQuantities(&ctx)      # src/particles.c:136
    ComputePotential(ksp, &ctx)        # src/potential.c:6

:class:`Hybrid` exposes the same four calls (same names, same meaning,
errors raised as :class:`HybridError` carrying the ch_status) over
``libchybrid.so``, whose kernels run on the GPU.  There is no CPU fallback:
constructing a :class:`Hybrid` without the built library or without a CUDA
device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libchybrid.so")

CH_OK = 0
STATUS = {0: "CH_OK", -1: "CH_ERR_ARG", -2: "CH_ERR_CUDA", -3: "CH_ERR_NOMEM", -4: "CH_ERR_NOT_CONVERGED",
          -5: "CH_ERR_COLLISION_LIMIT", -6: "CH_ERR_NAN", -7: "CH_ERR_RANGE", -8: "CH_ERR_TIMEOUT",
          -9: "CH_ERR_STATE", -10: "CH_ERR_UNSUPPORTED"}
LHS = {"identity": 0, "laplacian": 1, "full": 2}
RHS = {"constant": 0, "sinusoidal": 1, "full": 2}
KSP = {"cg": 0, "bcgs": 1}
PC = {"none": 0, "jacobi": 1, "mg": 2}
PRECISION = {"fp64": 0, "mixed": 1}
NN_PROFILE = {"uniform": 0, "gaussian_x": 1}  # CH_NN_*: neutral density n_n(x)
# --density-type (CH_DENSITY_*), the reference's DensityTypes order
DENSITY = {"flat-sobol": 0, "flat-reverse": 1, "flat-normal": 2, "uniform": 3, "sinusoidal": 4, "gaussian": 5}
FAITHFUL = {2: 1 << 2, 3: 1 << 3, 4: 1 << 4, 5: 1 << 5, 6: 1 << 6, 7: 1 << 7, 8: 1 << 8}

_dp = C.POINTER(C.c_double)


class HybridError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Params(C.Structure):
    """ch_params (include/chybrid.h)."""

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

    def update(self, **kw) -> "Params":
        for k, v in kw.items():
            if isinstance(v, (tuple, list, np.ndarray)):
                getattr(self, k)[:] = [float(x) for x in v]
            else:
                setattr(self, k, v)
        return self


class Loader(C.Structure):
    _fields_ = [("amp", C.c_double * 3), ("phase", C.c_double * 3), ("v0", C.c_double * 3), ("vT", C.c_double * 3)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("rnorm", C.c_double),
                ("bnorm", C.c_double)]


class StepInfo(C.Structure):
    _fields_ = [("Nc", C.c_int64), ("collisions", C.c_int64), ("refused", C.c_int64), ("expected", C.c_double),
                ("moment_sum", C.c_double * 4), ("solve", SolveInfo)]

    def as_dict(self):
        return dict(Nc=self.Nc, collisions=self.collisions, refused=self.refused, expected=self.expected,
                    moment_sum=list(self.moment_sum), iterations=self.solve.iterations,
                    refinements=self.solve.refinements, rnorm=self.solve.rnorm, bnorm=self.solve.bnorm)


class RunInfo(C.Structure):
    """ch_run_info: one run of a batch step."""

    _fields_ = [("Nc", C.c_int64), ("collisions", C.c_int64), ("refused", C.c_int64), ("expected", C.c_double),
                ("solve", SolveInfo), ("status", C.c_int32), ("flags", C.c_int32)]

    def as_dict(self):
        return dict(Nc=self.Nc, collisions=self.collisions, refused=self.refused, expected=self.expected,
                    iterations=self.solve.iterations, refinements=self.solve.refinements, rnorm=self.solve.rnorm,
                    bnorm=self.solve.bnorm, status=self.status, flags=self.flags)


class Tuning(C.Structure):
    _fields_ = [("cluster", C.c_int32), ("pass_ctas_per_sm", C.c_int32), ("pass_ms", C.c_double),
                ("solve_ms", C.c_double), ("cluster_big", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjointConfig(C.Structure):
    _fields_ = [("nsteps", C.c_int32), ("checkpoint_every", C.c_int32), ("window", C.c_int32), ("pad", C.c_int32),
                ("flux_weight", C.c_double), ("phi_weight", C.c_double)]


class AdjointTiming(C.Structure):
    _fields_ = [("forward_ms", C.c_double), ("gradient_ms", C.c_double), ("recompute_ms", C.c_double),
                ("events", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Profile(C.Structure):
    _fields_ = [("pass_ms", C.c_double), ("pass_calls", C.c_int64), ("solve_ms", C.c_double),
                ("solve_calls", C.c_int64), ("sort_ms", C.c_double), ("sort_calls", C.c_int64),
                ("moments_ms", C.c_double), ("moments_calls", C.c_int64), ("launches", C.c_int64),
                ("deposit_ms", C.c_double), ("deposit_calls", C.c_int64), ("host_push_calls", C.c_int64),
                ("host_push_reruns", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    """The loaded C ABI; raises if the library was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise HybridError(-2, f"{LIBPATH} not built: run __graft_entry__.build()")
        L = C.CDLL(LIBPATH)
        vp = C.c_void_p
        L.ch_last_error.restype = C.c_char_p
        L.ch_abi_version.restype = C.c_int32
        sig = {
            "ch_params_default": [C.POINTER(Params)],
            "ch_create": [C.POINTER(Params), C.c_int32, C.POINTER(vp)],
            "ch_destroy": [vp],
            "ch_particles_upload": [vp, vp, vp, C.c_int64],
            "ch_particles_download": [vp, vp, vp],
            "ch_particles_load": [vp, C.c_int64, C.POINTER(Loader)],
            "ch_update_velocities": [vp, C.c_int64, C.POINTER(StepInfo)],
            "ch_update_positions": [vp],
            "ch_collect_moments": [vp, vp, C.POINTER(StepInfo)],
            "ch_compute_potential": [vp, vp, C.POINTER(SolveInfo)],
            "ch_step": [vp, C.c_int64, C.c_int32, C.POINTER(StepInfo)],
            "ch_step_host": [vp, C.c_int64, C.c_int32, vp, vp, C.POINTER(StepInfo)],
            "ch_set_moments": [vp, vp],
            "ch_get_phi": [vp, vp],
            "ch_set_phi": [vp, vp],
            "ch_get_rhs": [vp, vp],
            "ch_apply_operator": [vp, vp, vp],
            "ch_set_profiling": [vp, C.c_int32],
            "ch_get_profile": [vp, C.POINTER(Profile)],
            "ch_reset_profile": [vp],
            "ch_get_stream": [vp, C.POINTER(vp)],
            "ch_output_open": [vp, C.c_char_p],
            "ch_output": [vp, C.c_char_p],
            "ch_output_wait": [vp, C.POINTER(C.c_int64)],
            "ch_set_solver": [vp, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32],
            "ch_particles_load_placed": [vp, C.c_int64, vp, C.c_int32],
            "ch_host_register": [vp, C.c_uint64],
            "ch_host_alloc": [C.c_uint64, C.POINTER(vp)],
            "ch_host_free": [vp],
            "ch_host_unregister": [vp],
            "ch_batch_create": [vp, vp, C.c_int32, C.c_int32, C.POINTER(vp)],
            "ch_batch_destroy": [vp],
            "ch_batch_load": [vp, vp],
            "ch_batch_upload": [vp, C.c_int32, vp, vp],
            "ch_batch_download": [vp, C.c_int32, vp, vp],
            "ch_batch_initialize": [vp],
            "ch_batch_step": [vp, C.c_int64, C.c_int32, vp],
            "ch_batch_get_phi": [vp, C.c_int32, vp],
            "ch_batch_set_phi": [vp, C.c_int32, vp],
            "ch_batch_get_moments": [vp, C.c_int32, vp],
            "ch_batch_autotune": [vp, C.POINTER(Tuning)],
            "ch_batch_autotune_cached": [vp, C.c_char_p, C.POINTER(Tuning), C.POINTER(C.c_int32)],
            "ch_batch_set_tuning": [vp, C.POINTER(Tuning)],
            "ch_batch_get_tuning": [vp, C.POINTER(Tuning)],
            "ch_batch_set_profiling": [vp, C.c_int32],
            "ch_batch_get_profile": [vp, C.POINTER(Profile)],
            "ch_batch_get_stream": [vp, C.POINTER(vp)],
            "ch_adjoint_create": [C.POINTER(Params), C.c_int64, C.POINTER(Loader), C.POINTER(AdjointConfig),
                                  C.c_int32, C.POINTER(vp)],
            "ch_adjoint_destroy": [vp],
            "ch_adjoint_forward": [vp, vp, C.c_int32, C.POINTER(C.c_double)],
            "ch_adjoint_gradient": [vp, vp, C.POINTER(C.c_double)],
            "ch_adjoint_events": [vp, C.POINTER(C.c_int64), vp, vp, vp, vp],
            "ch_adjoint_get_timing": [vp, C.POINTER(AdjointTiming)],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int32
        _lib = L
    return _lib


def _check(rc: int):
    if rc != CH_OK:
        raise HybridError(rc, lib().ch_last_error().decode(errors="replace"))


def default_params(**kw) -> Params:
    """ch_params_default (the reference's defaults, normalised units) with overrides."""
    p = Params()
    _check(lib().ch_params_default(C.byref(p)))
    return p.update(**kw)


def params_for(N, L=None, **kw) -> Params:
    """Normalised plasma of the synthetic configurations: unit spacing,
    Omega_i = 1 along z, Maxwellian ions with vT = 1 per component,
    equal-mass neutrals at Ti, isothermal electrons (cth = 1), kappa_e = 0."""
    L = L if L is not None else tuple(float(n) for n in N)
    p = default_params(Nx=N[0], Ny=N[1], Nz=N[2], x0=0.0, y0=0.0, z0=0.0, x1=L[0], y1=L[1], z1=L[2],
                       qi=1.0, mi=1.0, nui=0.1, dt=0.05, vi0=(0, 0, 0), viT=(1, 1, 1), mn=1.0, vnT=1.0,
                       vn0=(0, 0, 0), B0=(0, 0, 1), E0=(0.5, 0, 0), kappa_e=(0, 0, 0), cth=1.0, cG=0.1,
                       ksp_rtol=1e-8, seed=1)
    return p.update(**kw)


def loader(amp=(0.01, 0.0, 0.0), phase=(0.0, 0.0, 0.0), v0=(0.0, 0.0, 0.0), vT=(1.0, 1.0, 1.0)) -> Loader:
    L = Loader()
    L.amp[:] = amp
    L.phase[:] = phase
    L.v0[:] = v0
    L.vT[:] = vT
    return L


def _philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon et al., SC'11) for the few host-side draws."""
    M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
    x0, x1, x2, x3 = ctr
    k0, k1 = key
    for _ in range(10):
        p0, p1 = M0 * x0, M1 * x2
        x0, x1, x2, x3 = ((p1 >> 32) ^ x1 ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, ((p0 >> 32) ^ x3 ^ k1) & 0xFFFFFFFF, \
            p0 & 0xFFFFFFFF
        k0, k1 = (k0 + W0) & 0xFFFFFFFF, (k1 + W1) & 0xFFFFFFFF
    return [x0, x1, x2, x3]


def mode_phases(seed: int, run: int = 0):
    """Random phases of the 3-mode density perturbation: 2 pi U(m) with
    U from Philox(ctr = {m, 0xFFFFFFFF, 4 << 24, run}, key = seed)."""
    out = []
    for m in range(1, 4):
        r = _philox4x32_10([m, 0xFFFFFFFF, 4 << 24, run], [seed & 0xFFFFFFFF, seed >> 32])
        out.append(2.0 * np.pi * ((float(r[0]) + 0.5) * 2.0 ** -32))
    return out


class Hybrid:
    """One run on one GPU: the reference's Context + DMs + KSP."""

    def __init__(self, params: Params, device: int = -1):
        self.p = params
        self.N = params.Nx * params.Ny * params.Nz
        h = C.c_void_p()
        _check(lib().ch_create(C.byref(params), device, C.byref(h)))
        self._h = h
        self.np = 0

    def close(self):
        if getattr(self, "_h", None):
            lib().ch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- ions
    def upload(self, pos: np.ndarray, vel: np.ndarray):
        """DMSwarm 'position'/'velocity' RealVector arrays (np x 4 FP64)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        assert pos.shape == vel.shape and pos.ndim == 2 and pos.shape[1] == 4
        _check(lib().ch_particles_upload(self._h, pos.ctypes.data, vel.ctypes.data, pos.shape[0]))
        self.np = pos.shape[0]

    def load(self, np_: int, L: Loader):
        _check(lib().ch_particles_load(self._h, int(np_), C.byref(L)))
        self.np = int(np_)

    def load_placed(self, np_: int, L: Loader, density_type: str = "flat-sobol"):
        """InitializePositions with the reference's --density-type placement
        and Maxwellian velocities from L (ch_particles_load_placed)."""
        _check(lib().ch_particles_load_placed(self._h, int(np_), C.byref(L), DENSITY[density_type]))
        self.np = int(np_)

    def download(self, pos=None, vel=None):
        pos = np.empty((self.np, 4)) if pos is None else pos
        vel = np.empty((self.np, 4)) if vel is None else vel
        _check(lib().ch_particles_download(self._h, pos.ctypes.data, vel.ctypes.data))
        return pos, vel

    # ---------------------------------------------------------------- the four entry points
    def UpdateVelocities(self, step: int = 0) -> dict:
        info = StepInfo()
        _check(lib().ch_update_velocities(self._h, int(step), C.byref(info)))
        return info.as_dict()

    def UpdatePositions(self):
        _check(lib().ch_update_positions(self._h))

    def CollectVlasovQuantities(self, out: np.ndarray | None = None, copy: bool = True):
        """Returns the dof-4 GridNode array (N x 4: n, Gx, Gy, Gz); with
        copy=False the moments stay on the device and None is returned."""
        if copy:
            out = np.empty((self.N, 4)) if out is None else out
        info = StepInfo()
        _check(lib().ch_collect_moments(self._h, out.ctypes.data if copy else None, C.byref(info)))
        self.last_moments = info.as_dict()
        return out if copy else None

    def ComputePotential(self, out: np.ndarray | None = None, copy: bool = True):
        if copy:
            out = np.empty(self.N) if out is None else out
        info = SolveInfo()
        _check(lib().ch_compute_potential(self._h, out.ctypes.data if copy else None, C.byref(info)))
        self.last_solve = dict(iterations=info.iterations, refinements=info.refinements, rnorm=info.rnorm,
                               bnorm=info.bnorm)
        return out if copy else None

    def step(self, first_step: int, nsteps: int = 1) -> dict:
        info = StepInfo()
        _check(lib().ch_step(self._h, int(first_step), int(nsteps), C.byref(info)))
        return info.as_dict()

    def step_host(self, pos: np.ndarray, vel: np.ndarray, first_step: int, nsteps: int = 1) -> dict:
        """Steps with the ions held by the host (ch_step_host): uploads pos /
        vel (np x 4 FP64, C order), runs the steps and downloads the ions back
        into them.  Registered arrays (host_register) let the download overlap
        the last step's deposit and potential solve."""
        assert pos.shape == vel.shape == (self.np, 4) and pos.dtype == vel.dtype == np.float64
        assert pos.flags.c_contiguous and vel.flags.c_contiguous
        info = StepInfo()
        _check(lib().ch_step_host(self._h, int(first_step), int(nsteps), pos.ctypes.data, vel.ctypes.data,
                                  C.byref(info)))
        return info.as_dict()

    # ---------------------------------------------------------------- grid access
    def set_solver(self, ksp: str = "cg", pc: str = "mg", rtol: float = 1e-8, atol: float = 0.0, max_it: int = 10000):
        """KSPSetType / KSPSetTolerances for the following solves."""
        _check(lib().ch_set_solver(self._h, KSP[ksp], PC[pc], float(rtol), float(atol), int(max_it)))

    def set_moments(self, nodes: np.ndarray):
        nodes = np.ascontiguousarray(nodes, dtype=np.float64).reshape(self.N, 4)
        _check(lib().ch_set_moments(self._h, nodes.ctypes.data))

    def phi(self, out: np.ndarray | None = None):
        if out is None:
            out = np.empty(self.N)
        assert out.dtype == np.float64 and out.size == self.N and out.flags.c_contiguous
        _check(lib().ch_get_phi(self._h, out.ctypes.data))
        return out

    def set_phi(self, phi: np.ndarray):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        _check(lib().ch_set_phi(self._h, phi.ctypes.data))

    def rhs(self):
        out = np.empty(self.N)
        _check(lib().ch_get_rhs(self._h, out.ctypes.data))
        return out

    def apply_operator(self, x: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        _check(lib().ch_apply_operator(self._h, x.ctypes.data, y.ctypes.data))
        return y

    # ---------------------------------------------------------------- output (OutputHDF5)
    def output_open(self, stem: str):
        _check(lib().ch_output_open(self._h, stem.encode()))

    def output(self, insert: str):
        """Queues the current fields for writing as <stem><insert>.*; returns
        at once (the copy and the writes overlap the next steps)."""
        _check(lib().ch_output(self._h, insert.encode()))

    def output_wait(self) -> int:
        n = C.c_int64()
        _check(lib().ch_output_wait(self._h, C.byref(n)))
        return n.value

    # ---------------------------------------------------------------- profiling
    def set_profiling(self, on: bool = True):
        _check(lib().ch_set_profiling(self._h, int(on)))

    def reset_profile(self):
        _check(lib().ch_reset_profile(self._h))

    def profile(self) -> dict:
        pr = Profile()
        _check(lib().ch_get_profile(self._h, C.byref(pr)))
        return pr.as_dict()

    def stream_handle(self) -> int:
        s = C.c_void_p()
        _check(lib().ch_get_stream(self._h, C.byref(s)))
        return s.value or 0


class Batch:
    """An ensemble of independent runs advanced together (ch_batch): every
    phase of a step is one launch over all runs, replayed from a CUDA graph.
    Runs may differ in grid, ion count and parameters (mixed form, full
    operator, CG + multigrid)."""

    def __init__(self, params, nions, device: int = -1):
        self.n = len(params)
        self.params = list(params)
        self._p = (Params * self.n)(*self.params)
        self.np = [int(v) for v in nions]
        self._np = (C.c_int64 * self.n)(*self.np)
        h = C.c_void_p()
        _check(lib().ch_batch_create(C.cast(self._p, C.c_void_p), C.cast(self._np, C.c_void_p), self.n, device,
                                     C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().ch_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def N(self, r: int) -> int:
        p = self.params[r]
        return p.Nx * p.Ny * p.Nz

    def load(self, loaders):
        arr = (Loader * self.n)(*loaders)
        _check(lib().ch_batch_load(self._h, C.cast(arr, C.c_void_p)))

    def upload(self, r: int, pos: np.ndarray, vel: np.ndarray):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        assert pos.shape == vel.shape == (self.np[r], 4)
        _check(lib().ch_batch_upload(self._h, int(r), pos.ctypes.data, vel.ctypes.data))

    def download(self, r: int):
        pos = np.empty((self.np[r], 4))
        vel = np.empty((self.np[r], 4))
        _check(lib().ch_batch_download(self._h, int(r), pos.ctypes.data, vel.ctypes.data))
        return pos, vel

    def initialize(self):
        _check(lib().ch_batch_initialize(self._h))

    def step(self, first_step: int, nsteps: int = 1):
        info = (RunInfo * self.n)()
        rc = lib().ch_batch_step(self._h, int(first_step), int(nsteps), C.cast(info, C.c_void_p))
        self.last_info = [i.as_dict() for i in info]
        _check(rc)
        return self.last_info

    def phi(self, r: int):
        out = np.empty(self.N(r))
        _check(lib().ch_batch_get_phi(self._h, int(r), out.ctypes.data))
        return out

    def set_phi(self, r: int, phi: np.ndarray):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        _check(lib().ch_batch_set_phi(self._h, int(r), phi.ctypes.data))

    def moments(self, r: int):
        out = np.empty((self.N(r), 4))
        _check(lib().ch_batch_get_moments(self._h, int(r), out.ctypes.data))
        return out

    def autotune(self, cache: str | None = None) -> dict:
        """Times the launch shapes and keeps the fastest; with `cache` (a
        file of JSON lines) a batch of the same class takes the stored shape
        instead, and the result says whether it was cached."""
        t = Tuning()
        if cache is None:
            _check(lib().ch_batch_autotune(self._h, C.byref(t)))
            return t.as_dict()
        hit = C.c_int32(0)
        _check(lib().ch_batch_autotune_cached(self._h, os.fsencode(cache), C.byref(t), C.byref(hit)))
        return dict(t.as_dict(), cached=bool(hit.value))

    def tuning(self) -> dict:
        t = Tuning()
        _check(lib().ch_batch_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, cluster: int, pass_ctas_per_sm: int = 2, cluster_big: int = 0):
        t = Tuning(cluster, pass_ctas_per_sm, 0.0, 0.0, cluster_big)
        _check(lib().ch_batch_set_tuning(self._h, C.byref(t)))

    def set_profiling(self, on: bool = True):
        _check(lib().ch_batch_set_profiling(self._h, int(on)))

    def profile(self) -> dict:
        pr = Profile()
        _check(lib().ch_batch_get_profile(self._h, C.byref(pr)))
        return pr.as_dict()

    def stream_handle(self) -> int:
        s = C.c_void_p()
        _check(lib().ch_batch_get_stream(self._h, C.byref(s)))
        return s.value or 0


NTHETA = 7  # E0 (3), vn0 (3), amp (loader amp[0])


class Adjoint:
    """The FP64 step as a differentiable function of theta = (E0, vn0, amp)
    with the collision events of a recorded run frozen (ch_adjoint)."""

    def __init__(self, params: Params, nions: int, L: Loader, nsteps: int, checkpoint_every: int, window: int,
                 flux_weight: float = 1.0, phi_weight: float = 0.1, device: int = -1):
        self.cfg = AdjointConfig(int(nsteps), int(checkpoint_every), int(window), 0, float(flux_weight),
                                 float(phi_weight))
        self.params, self.loader, self.np = params, L, int(nions)
        h = C.c_void_p()
        _check(lib().ch_adjoint_create(C.byref(params), self.np, C.byref(L), C.byref(self.cfg), device, C.byref(h)))
        self._h = h

    def theta0(self):
        p = self.params
        return np.array(list(p.E0) + list(p.vn0) + [self.loader.amp[0]], dtype=np.float64)

    def close(self):
        if getattr(self, "_h", None):
            lib().ch_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def forward(self, theta, record: bool = False) -> float:
        th = np.ascontiguousarray(theta, dtype=np.float64)
        assert th.shape == (NTHETA,)
        J = C.c_double()
        _check(lib().ch_adjoint_forward(self._h, th.ctypes.data, int(bool(record)), C.byref(J)))
        return J.value

    def gradient(self):
        g = np.empty(NTHETA)
        J = C.c_double()
        _check(lib().ch_adjoint_gradient(self._h, g.ctypes.data, C.byref(J)))
        return g, J.value

    def events(self) -> dict:
        n = C.c_int64()
        _check(lib().ch_adjoint_events(self._h, C.byref(n), None, None, None, None))
        step = np.empty(n.value, np.int32)
        ion = np.empty(n.value, np.uint32)
        flags = np.empty(n.value, np.int32)
        data = np.empty((n.value, 5))
        _check(lib().ch_adjoint_events(self._h, C.byref(n), step.ctypes.data, ion.ctypes.data, flags.ctypes.data,
                                       data.ctypes.data))
        return dict(step=step, ion=ion, flags=flags, data=data)

    def timing(self) -> dict:
        t = AdjointTiming()
        _check(lib().ch_adjoint_get_timing(self._h, C.byref(t)))
        return t.as_dict()


def read_output(path: str) -> dict:
    """Reads one output written by Hybrid.output: path = <stem><insert>
    (without extension); returns {dataset name: (Nz, Ny, Nx) array}."""
    import json

    with open(path + ".json") as f:
        man = json.load(f)
    g = man["grid"]
    d = os.path.dirname(path)
    return {name: np.fromfile(os.path.join(d, fn), dtype="<f8").reshape(g["Nz"], g["Ny"], g["Nx"])
            for name, fn in man["datasets"].items()}


def host_register(a: np.ndarray):
    """Page-locks a numpy array for full-speed upload/download."""
    _check(lib().ch_host_register(a.ctypes.data, a.nbytes))


def host_unregister(a: np.ndarray):
    _check(lib().ch_host_unregister(a.ctypes.data))


class HostArray:
    """A numpy array in page-locked host memory from ch_host_alloc (the
    memory the GPU streams at the full host-link rate); free() or leaving
    the with-block releases it, after which the array must not be used."""

    def __init__(self, shape, dtype=np.float64):
        dt = np.dtype(dtype)
        n = int(np.prod(shape)) * dt.itemsize
        p = C.c_void_p()
        _check(lib().ch_host_alloc(n, C.byref(p)))
        self._p = p
        buf = (C.c_char * n).from_address(p.value)
        self.a = np.frombuffer(buf, dtype=dt).reshape(shape)

    def free(self):
        if self._p is not None and self._p.value:
            self.a = None
            _check(lib().ch_host_free(self._p))
            self._p = None

    def __enter__(self):
        return self.a

    def __exit__(self, *exc):
        self.free()
