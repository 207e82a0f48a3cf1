"""The link-level boundary: the reference's own entry points over the C ABI.

* libpetrbf_gb300.so exports RBFInterpolation with the reference's C++ signature and
  linkage (3d/wrapper.cxx:20-23), so a program built against librbf.a relinks unchanged;
* the PETSc glue (petrbf_gb300/glue/petrbf_petsc.cxx: rbf_interpolation and
  vorticity_evaluation on Vecs, the MatShell MATOP_MULT body mymatmult, a PCShell apply)
  compiles against PETSc's declarations -- here the sequential stand-in in oracle/ref_stub
  -- and links against the library (CPU);
* driven the way the reference's callers drive those functions, it returns exactly what
  the C ABI returns for the same inputs (GPU)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

MANGLED = "_Z16RBFInterpolationiPPciPfS1_S1_S1_iS1_S1_S1_S1_fiii"


def _build_driver(tmp):
    from petrbf_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(str(tmp), "glue_driver")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "oracle", "ref_stub"), "-I",
           os.path.join(ROOT, "include"), "-o", exe, os.path.join(ROOT, "tests", "glue", "driver.cxx"),
           os.path.join(ROOT, "petrbf_gb300", "glue", "petrbf_petsc.cxx"), "-L", libdir, "-lpetrbf_gb300",
           "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, lib


def test_reference_symbol_exported_and_glue_links(tmp_path):
    exe, lib = _build_driver(tmp_path)
    assert os.path.exists(exe)
    assert hasattr(ctypes.CDLL(lib), MANGLED)


@pytest.mark.gpu
def test_glue_returns_what_the_c_abi_returns(tmp_path):
    from petrbf_gb300 import workloads as W
    from petrbf_gb300.api import Context, RBFInterpolation
    exe, _ = _build_driver(tmp_path)
    p = W.lamb_oseen_2d(40, jitter=0.25, seed=21)
    n = p.n
    r = np.random.default_rng(3).standard_normal(n)
    xt, yt = p.x[::3] + 0.3 * p.meta["h"], p.y[::3] - 0.2 * p.meta["h"]
    # an unjittered 3D lattice: RBFInterpolation keeps the reference's restricted Schwarz,
    # which stalls on jittered 3D lattices
    x3, y3, z3, h3 = W.lattice_3d(9, jitter=0.0)
    s3 = h3 / 0.8
    wg = np.exp(-(x3 ** 2 + y3 ** 2 + z3 ** 2))
    xp, yp, zp = x3 + 0.3 * h3, y3 - 0.2 * h3, z3 + 0.1 * h3
    gp = np.exp(-(xp ** 2 + yp ** 2 + zp ** 2)) * h3 ** 3
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    inp = os.path.join(str(tmp_path), "in.bin")
    out = os.path.join(str(tmp_path), "out.bin")
    with open(inp, "wb") as fh:
        fh.write(np.array([n, len(xt), len(x3)], np.int32).tobytes())
        fh.write(np.array([p.sigma, s3], np.float64).tobytes())
        fh.write(np.array([p.nsigma_box, p.sigma_buffer, p.sigma_trunc, 2, 6, 16], np.int32).tobytes())
        for a in (p.x, p.y, p.f, r, xt, yt):
            fh.write(np.ascontiguousarray(a, np.float64).tobytes())
        for a in (x3, y3, z3, wg, xp, yp, zp, gp):
            fh.write(f32(a).tobytes())
    run = subprocess.run([exe, inp, out], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr
    raw = open(out, "rb").read()
    head = np.frombuffer(raw[:28], np.int32)
    its, status = int(head[0]), head[1:]
    assert list(status) == [0] * 6, (status, run.stderr)
    d = np.frombuffer(raw[28:28 + 8 * (3 * n + len(xt))], np.float64)
    g, w, Ar, Br = d[:n], d[n:n + len(xt)], d[n + len(xt):2 * n + len(xt)], d[2 * n + len(xt):]
    fl = np.frombuffer(raw[28 + 8 * (3 * n + len(xt)):], np.float32)
    w_solve, w_eval = fl[:len(x3)], fl[len(x3):]
    with Context(dim=2, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                 sigma_trunc=p.sigma_trunc) as c:
        g0, st = c.interpolate(p.x, p.y, None, p.f)
        w0 = c.evaluate(xt, yt, None, p.x, p.y, None, g0)
        c.matvec_setup(p.x, p.y)
        Ar0 = c.matvec(r)
        c.pc_setup("fp64")
        Br0 = c.pc_apply(r)
    assert its == st.its
    np.testing.assert_array_equal(g, g0)
    np.testing.assert_array_equal(w, w0)
    np.testing.assert_array_equal(Ar, Ar0)
    np.testing.assert_array_equal(Br, Br0)
    ws = f32(wg).copy()
    assert RBFInterpolation(x3, y3, z3, ws, x3, y3, z3, wg, s3, 2, 6, 16) == 0
    we = f32(wg).copy()
    assert RBFInterpolation(x3, y3, z3, we, xp, yp, zp, gp, s3, 2, 6, 16) == 0
    np.testing.assert_array_equal(w_solve, ws)
    np.testing.assert_array_equal(w_eval, we)
