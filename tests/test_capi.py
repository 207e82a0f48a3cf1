"""The C-ABI library builds, loads and exports every function include/petrbf_gb300.h
declares (CPU only: no compute calls)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*(?:[\w*]+\s+)+\**(prbf_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from petrbf_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from petrbf_gb300 import _native
    assert set(_declared()) <= set(_native.SIGNATURES)


def test_status_strings_and_defaults():
    from petrbf_gb300 import _native as N
    L = N.lib()
    p = N.Params()
    L.prbf_params_default(ctypes.byref(p))
    assert p.dim == 2 and p.restart == 30 and p.rtol == 1e-13 and p.max_it == 1000
    assert L.prbf_status_string(0) == b"ok"
    assert L.prbf_status_string(N.ERR_STATE) == b"call out of order"


def test_gpumatmult_argument_checks_need_no_gpu():
    # the seam validates its arguments before any CUDA call
    import numpy as np
    from petrbf_gb300 import _native as N
    L = N.lib()
    f = np.zeros(256, np.float32)
    fp = f.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    ok = np.array([0, 3, 5], np.int32)
    bad = np.array([0, 3, 2], np.int32)
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    call = lambda off, iblok, ncl, ntr, sigma=0.1: L.prbf_gpumatmult_2d(fp, fp, fp, fp, fp, fp, ip(off), iblok,
                                                                       sigma, ncl, ntr)
    assert call(ok, 0, 2, 3) == N.OK                 # nothing to do
    assert call(ok, 2, 1, 3) == N.ERR_ARG            # more blocks than the capacity
    assert call(bad, 2, 2, 3) == N.ERR_ARG           # decreasing offsets
    assert call(ok, 2, 2, 2) == N.ERR_CAPACITY       # 5 sources > 2 x 2
    assert call(ok, 2, 2, 3, sigma=0.0) == N.ERR_ARG
    assert L.prbf_gpumatmult_3d(fp, fp, None, fp, fp, fp, fp, fp, ip(ok), 2, 0.1, 2, 3) == N.ERR_ARG


def test_entry_points_refuse_bad_arguments_before_any_cuda_call():
    import numpy as np
    from petrbf_gb300 import _native as N
    L = N.lib()
    d = np.zeros(8)
    dp = d.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    # a null context is an argument error on every context call
    assert L.prbf_interpolate(None, 8, dp, dp, None, dp, 1, dp, None) == N.ERR_ARG
    assert L.prbf_matvec(None, dp, dp) == N.ERR_ARG
    assert L.prbf_pc_apply(None, dp, dp) == N.ERR_ARG
    assert L.prbf_batch_interpolate(None, 1, None, None, None, None) == N.ERR_ARG
    assert L.prbf_ctx_synchronize(None) == N.ERR_ARG
    # RBFInterpolation (3d/wrapper.cxx:20): no grid points, or a particle field to evaluate
    # first (xg[0] != xp[0]) with a missing array
    g = np.arange(4, dtype=np.float32)
    q = g + 1
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    args = lambda ng, yp: (0, None, ng, fp(g), fp(g), fp(g), fp(g), 4, fp(q), yp, fp(q), fp(q), 0.1, 2, 6, 16)
    assert L.prbf_RBFInterpolation(*args(0, fp(q))) == N.ERR_ARG
    assert L.prbf_RBFInterpolation(*args(4, None)) == N.ERR_ARG


def test_python_mirror_checks_array_lengths_before_any_cuda_call():
    import numpy as np
    import pytest
    from petrbf_gb300.api import RBFInterpolation, batch_interpolate, gpumatmult
    a4, a3 = np.zeros(4), np.zeros(3)
    with pytest.raises(ValueError):
        batch_interpolate([dict(x=a4, y=a3, f=a4, sigma=0.1, nsigma_box=4, sigma_buffer=12, sigma_trunc=20)])
    with pytest.raises(ValueError):
        RBFInterpolation(a4, a4, a4, np.zeros(4, np.float32), a4, a3, a4, a4, 0.1, 2, 6, 16)
    t = np.zeros(128)
    with pytest.raises(ValueError):   # sources shorter than offset[-1]
        gpumatmult(t, t, None, a3, a3, None, a3, [0, 4], 0.1)
    with pytest.raises(ValueError):   # targets of different lengths
        gpumatmult(t, np.zeros(127), None, a4, a4, None, a4, [0, 4], 0.1)
