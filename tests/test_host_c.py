"""The C host side: option parsing (ProcessOptions names and derivations),
the PETSc drop-in's compilation against the reference's own headers, and
the C driver mirroring src/hybrid.c (GPU)."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import REPO
from oracle.pyoracle import REF_SRC

HOST = os.path.join(REPO, "collisional-hybrid_gb300", "host")
PKG = os.path.join(REPO, "collisional-hybrid_gb300")


@pytest.fixture(scope="module")
def optlib(chy):
    chy.lib()
    d = tempfile.mkdtemp()
    so = os.path.join(d, "libchopts.so")
    subprocess.run(["gcc", "-O1", "-shared", "-fPIC", "-std=c11", "-I", os.path.join(REPO, "include"), "-I", HOST,
                    os.path.join(HOST, "ch_options.c"), "-o", so, "-L", PKG, "-lchybrid", f"-Wl,-rpath,{PKG}",
                    "-lm"], check=True)
    L = C.CDLL(so)
    L.ch_parse_options.restype = C.c_int32
    return L


class RunOpts(C.Structure):
    _fields_ = [("Nt", C.c_int32), ("Np", C.c_int64), ("density_type", C.c_int32), ("amp", C.c_double * 3),
                ("phase", C.c_double * 3), ("random_phases", C.c_int32), ("verbose", C.c_int32),
                ("use_modes", C.c_int32)]


def parse(optlib, chy, args):
    argv = ["hybrid"] + args
    arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
    p = chy.Params()
    r = RunOpts()
    err = C.create_string_buffer(256)
    rc = optlib.ch_parse_options(len(argv), arr, C.byref(p), C.byref(r), err, 256)
    return rc, p, r, err.value.decode()


def test_reference_option_names_and_derivations(optlib, chy):
    # the 32^3 case in the reference's option names (run-case style)
    rc, p, r, err = parse(optlib, chy, ["-Nx", "32", "-Ny", "32", "-Nz", "32", "-x1", "32", "-y1", "32", "-z1",
                                        "32", "-Np", "524288", "-viT", "1", "-B0z", "1", "-E0x", "0.5", "-nui",
                                        "0.1", "-dt", "0.05", "-Nt", "100", "-ksp_rtol", "1e-8",
                                        "--lhs-type", "full", "--rhs-type", "full", "-ksp_type", "bcgs"])
    assert rc == 0, err
    assert (p.Nx, p.Ny, p.Nz) == (32, 32, 32) and p.x1 == 32.0
    assert r.Np == 524288 and r.Nt == 100
    assert p.nui == 0.1 and p.dt == 0.05 and p.E0[0] == 0.5 and p.B0[2] == 1.0
    assert tuple(p.viT) == (1.0, 1.0, 1.0)
    # Ti = m vT.r^2 / 2 (src/parameters.c:537), Tn = Ti, vnT = sqrt(2 Tn / mn) (:556)
    assert abs(p.vnT - (2 * 1.5) ** 0.5) < 1e-15
    # electron magnetisation |q B / m| / nu (src/parameters.c:519-528)
    assert abs(p.kappa_e[2] - 1836.15267343) < 1e-6
    assert p.ksp_rtol == 1e-8 and p.ksp_type == 1
    assert p.lhs_type == 2 and p.rhs_type == 2


def test_defaults_and_extensions(optlib, chy):
    rc, p, r, err = parse(optlib, chy, ["-nui", "4", "-ch_vnT", "1", "-ch_precision", "mixed", "-ch_pc", "mg",
                                        "-ch_seed", "7", "-ch_faithful", "256", "-ch_amp1", "0.02"])
    assert rc == 0, err
    assert p.dt == 0.25  # dt = 1/nu (src/parameters.c:417)
    assert (p.Nx, p.Ny, p.Nz) == (7, 7, 7) and r.Np == 343  # src/setup.c:10-12, 44-46
    assert p.vnT == 1.0 and p.precision == 1 and p.pc_type == 2 and p.seed == 7 and p.faithful == 256
    assert r.amp[0] == 0.02


def test_rejects_unsupported_options(optlib, chy):
    rc, p, r, err = parse(optlib, chy, ["--x0-bc", "neumann"])
    assert rc == -1 and "periodic" in err
    rc, p, r, err = parse(optlib, chy, ["--lhs-type", "bogus"])
    assert rc == -1


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference headers not present")
def test_petsc_dropin_compiles_against_reference_headers():
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run(["gcc", "-std=gnu11", "-Wall", "-Werror", "-Wno-unused-function", "-DCH_WITH_PETSC",
                            "-I", os.path.join(REPO, "oracle", "ref", "shim"), "-I", REF_SRC,
                            "-I", os.path.join(REPO, "include"), "-c", os.path.join(HOST, "petsc_dropin.c"),
                            "-o", os.path.join(d, "dropin.o")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        syms = subprocess.run(["nm", os.path.join(d, "dropin.o")], capture_output=True, text=True).stdout
        for f in ("UpdateVelocities", "UpdatePositions", "CollectVlasovQuantities", "ComputePotential"):
            assert f" T {f}" in syms


def _dropin_loop(args):
    """Builds the drop-in with the PETSc stand-in and a recording test double
    of the C ABI (tests/dropin/), runs the reference's loop order through it
    with the given options, and returns what reached the C ABI."""
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "loop")
    dd = os.path.join(REPO, "tests", "dropin")
    r = subprocess.run(["gcc", "-std=gnu11", "-Wall", "-Werror", "-Wno-unused-function", "-DCH_WITH_PETSC",
                        "-I", os.path.join(REPO, "oracle", "ref", "shim"), "-I", os.path.join(REPO, "oracle", "ref"),
                        "-I", REF_SRC, "-I", os.path.join(REPO, "include"), "-I", HOST,
                        os.path.join(REPO, "oracle", "ref", "standin.c"), os.path.join(HOST, "petsc_dropin.c"),
                        os.path.join(dd, "fake_chybrid.c"), os.path.join(dd, "dropin_loop.c"), "-o", exe, "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe] + args, capture_output=True, text=True).stdout
    rec = {}
    for ln in out.splitlines():
        k, _, v = ln.partition(" ")
        rec[k] = v
    return rec


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference headers not present")
def test_petsc_dropin_passes_the_ksp_and_ch_options_down():
    """KSPSetFromOptions' settings (-ksp_type, -ksp_rtol, -ksp_max_it, read
    back with KSPGetTolerances / KSPGetType) and the -ch_ options reach the C
    ABI; kappa_e comes from the Context.  Over the reference's loop order
    (initial deposit and solve, then 3 steps) the ions go up once and come
    back once per step."""
    rec = _dropin_loop(["-ksp_type", "bcgs", "-ksp_rtol", "1e-10", "-ksp_max_it", "500", "-ch_precision", "mixed",
                        "-ch_pc", "mg", "-ch_sort_period", "2", "-test_kappa_z", "1.5"])
    assert rec["status"] == "0"
    assert rec["ksp"] == "1" and float(rec["rtol"]) == 1e-10 and rec["maxit"] == "500" and rec["pc"] == "2"
    assert rec["precision"] == "1" and rec["create_pc"] == "2" and rec["sort_period"] == "2"
    assert [float(x) for x in rec["kappa"].split()] == [0.0, 0.0, 1.5]
    assert rec["uploads"] == "1" and rec["downloads"] == "3" and rec["solves"] == "4"
    # PETSc's default gmres: BiCGStab for the non-symmetric operator, CG otherwise
    assert _dropin_loop(["-test_kappa_z", "1.5"])["ksp"] == "1"
    rec = _dropin_loop([])
    assert rec["ksp"] == "0" and float(rec["rtol"]) == 1e-5 and rec["maxit"] == "10000"
    # a value the drop-in does not know is an error before anything is created
    rec = _dropin_loop(["-ch_precision", "bogus"])
    assert rec["status"] != "0" and rec["creates"] == "0"


@pytest.mark.gpu
def test_c_driver_runs_reference_loop(chy):
    exe = os.path.join(PKG, "hybrid_gpu")
    r = subprocess.run([exe, "-Nx", "16", "-Ny", "16", "-Nz", "16", "-x1", "16", "-y1", "16", "-z1", "16",
                        "-Np", "65536", "-viT", "1", "-B0z", "1", "-E0x", "0.5", "-nui", "0.1", "-dt", "0.05",
                        "-Nt", "5", "-ch_vnT", "1", "-ch_cth", "1", "-ch_cG", "0.1", "-ch_kappa_ez", "0",
                        "-ch_amp1", "0.01", "-ksp_rtol", "1e-8"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("Time step")]
    assert len(lines) == 5
    assert "Elapsed time" in r.stdout
    # the reference's own placements: flat-sobol (its default) and the sinusoid
    for dens in ("flat-sobol", "sinusoidal"):
        r = subprocess.run([exe, "-Nx", "16", "-Ny", "16", "-Nz", "16", "-x1", "16", "-y1", "16", "-z1", "16",
                            "-Np", "65536", "-viT", "1", "-B0z", "1", "-E0x", "0.5", "-nui", "0.1", "-dt", "0.05",
                            "-Nt", "2", "-ch_vnT", "1", "-ch_cth", "1", "-ch_cG", "0.1", "-ch_kappa_ez", "0",
                            "--density-type", dens, "-ksp_rtol", "1e-8"], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, (dens, r.stderr)
        assert len([ln for ln in r.stdout.splitlines() if ln.startswith("Time step")]) == 2


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_driver_solves_a_loaded_density(chy, po, precision):
    """solver_gpu (src/solver.c's work: load a density, form the fluxes as
    --x/y/z-flux-scale times it, one solve from phi = 0, write the datasets)
    on an analytic density of the kind the reference's write_hdf5 script
    makes (n0 + dn times a sinusoid times a Gaussian): the residual meets
    -ksp_rtol, and phi agrees with the oracle's solve of the same system
    (1e-12 in the FP64 form, 1e-6 in the mixed form)."""
    N, L = (32, 16, 24), (1.0, 1.0, 1.0)
    x = (np.arange(N[0]) / N[0])[None, None, :]
    y = (np.arange(N[1]) / N[1])[None, :, None]
    z = (np.arange(N[2]) / N[2])[:, None, None]
    n = 1.0 + 0.4 * np.sin(2 * np.pi * (2 * x + y)) * np.exp(-((z - 0.5) ** 2) / (2 * 0.2 ** 2))
    n = np.ascontiguousarray(n.ravel())
    d = tempfile.mkdtemp()
    src = os.path.join(d, "vlasov.density.f64")
    n.tofile(src)
    exe = os.path.join(PKG, "solver_gpu")
    args = [exe, "-Nx", "32", "-Ny", "16", "-Nz", "24", "-x1", "1", "-y1", "1", "-z1", "1", "--input", src,
            "--x-flux-scale", "0.2", "--output", os.path.join(d, "res"), "-ksp_rtol", "1e-13", "-ch_pc", "mg",
            "-ch_precision", precision, "-ch_cth", "1", "-ch_cG", "0.1", "-ch_kappa_ez", "0", "-E0x", "0.5",
            "-ch_repeat", "3"]
    r = subprocess.run(args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("KSP iterations")][0]
    rr = float(line.split("|r|/|b|")[1].split()[0])
    assert rr <= 1e-13 * 1.01, line
    assert "solves/s" in r.stdout
    phi = np.fromfile(os.path.join(d, "res.potential.f64"))
    p = chy.params_for(N, L, precision=chy.PRECISION[precision], E0=(0.5, 0.0, 0.0), cth=1.0, cG=0.1,
                       ksp_rtol=1e-13)
    q = po.params_from(p)
    nodes = np.zeros((n.size, 4))
    nodes[:, 0], nodes[:, 1], nodes[:, 2], nodes[:, 3] = n, 0.2 * n, n, n
    nodes = nodes.ravel()
    ref, info = po.solve(q, nodes[0::4].copy(), po.rhs(q, nodes), rtol=1e-14, maxit=50000)
    assert info["rc"] == 0
    err = np.abs(phi - ref).max() / np.abs(ref).max()
    assert err < (1e-12 if precision == "fp64" else 1e-6), err
