"""Python mirror of PetRBF's solve-path interface, running on the GPU through the C ABI.

``rbf_interpolation`` and ``vorticity_evaluation`` keep the reference's argument
meaning (2d/rbf_interpolation.cxx:25-26, 2d/vorticity_evaluation.cxx:26-27, and the 3d
twins with z coordinates); ``GaussianOperator`` is the MatShell (MATOP_MULT =
mymatmult, 2d/matmult.cxx:6-51). Errors raise ``PrbfError`` with the C status code.
"""
import ctypes

import numpy as np

from . import _native as N
from ._native import PrbfError, Stats

_D = ctypes.POINTER(ctypes.c_double)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_D)


def _check_len(n, **arrays):
    """Every array given (None skipped) holds n entries: the C side reads n of each."""
    for name, a in arrays.items():
        if a is not None and a.shape[0] != n:
            raise ValueError(f"{name} holds {a.shape[0]} entries, expected {n}")


class Context:
    """One GPU context (device memory + one CUDA stream) with fixed solver parameters."""

    def __init__(self, dim=2, sigma=0.025, nsigma_box=8, sigma_buffer=24, sigma_trunc=24,
                 rtol=1e-13, abstol=1e-50, dtol=1e5, restart=30, max_it=1000, precision="fp64",
                 guess="zero", device=0, pc="rasm", block_fallback="shift"):
        L = N.lib()
        p = N.Params()
        L.prbf_params_default(ctypes.byref(p))
        p.dim, p.sigma, p.nsigma_box = int(dim), float(sigma), int(nsigma_box)
        p.sigma_buffer, p.sigma_trunc = int(sigma_buffer), int(sigma_trunc)
        p.rtol, p.abstol, p.dtol = float(rtol), float(abstol), float(dtol)
        p.restart, p.max_it, p.device = int(restart), int(max_it), int(device)
        p.precision = {"fp64": N.PREC_FP64, "mixed": N.PREC_MIXED}[precision]
        p.guess = {"zero": N.GUESS_ZERO, "learned": N.GUESS_LEARNED}[guess]
        p.pc_type = {"rasm": N.PC_RASM, "asm": N.PC_ASM}[pc]
        # "lu": a block whose FP64 Cholesky fails is factored by LU with partial pivoting, as
        # the reference's PETSc LU (a zero pivot raises); "shift": refactored with a shift
        p.block_fallback = {"shift": N.FALLBACK_SHIFT, "lu": N.FALLBACK_LU}[block_fallback]
        self.params = p
        self.dim = p.dim
        h = ctypes.c_void_p()
        st = L.prbf_ctx_create(ctypes.byref(p), ctypes.byref(h))
        if st:
            raise PrbfError(st, "prbf_ctx_create failed")
        self.h = h
        self.n = None

    def _check(self, st):
        if st:
            raise PrbfError(st, N.lib().prbf_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            N.lib().prbf_ctx_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        return N.lib().prbf_ctx_stream(self.h)

    def synchronize(self):
        self._check(N.lib().prbf_ctx_synchronize(self.h))

    # ---- MatShell seam -----------------------------------------------------------
    def matvec_setup(self, x, y, z=None):
        x, y, z = _f64(x), _f64(y), _f64(z)
        _check_len(x.shape[0], y=y, z=z)
        if self.dim == 3 and z is None:
            raise ValueError("a 3D context needs z")
        self.n = x.shape[0]
        self._keep = (x, y, z)
        self._check(N.lib().prbf_matvec_setup(self.h, self.n, _ptr(x), _ptr(y), _ptr(z)))

    def matvec(self, v):
        v = _f64(v)
        if self.n is None:
            raise PrbfError(N.ERR_STATE, "matvec_setup has not been called")
        _check_len(self.n, v=v)
        out = np.empty_like(v)
        self._check(N.lib().prbf_matvec(self.h, _ptr(v), _ptr(out)))
        return out

    def matvec_dev(self, in_ptr, out_ptr, cell_order=False, fp32=False):
        flags = (N.ORDER_CELL if cell_order else 0) | (N.MATVEC_FP32 if fp32 else 0)
        self._check(N.lib().prbf_matvec_dev(self.h, ctypes.c_void_p(in_ptr),
                                             ctypes.c_void_p(out_ptr), flags))

    def matvec_kernels(self, fp32=False):
        """(kernels one cell-order product launches, whether the FP64 product is symmetric)."""
        k, sym = ctypes.c_int(0), ctypes.c_int(0)
        self._check(N.lib().prbf_matvec_kernels(self.h, 1 if fp32 else 0, ctypes.byref(k), ctypes.byref(sym)))
        return k.value, bool(sym.value)

    def matvec_info(self):
        ints = np.zeros(7, np.int32)
        dbls = np.zeros(4, np.float64)
        pairs = ctypes.c_longlong(0)
        self._check(N.lib().prbf_matvec_info(self.h, ints.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                              _ptr(dbls), ctypes.byref(pairs)))
        keys = ["nx", "ny", "nz", "ncell", "nb_trunc", "nb_buffer", "max_trunc"]
        d = dict(zip(keys, (int(v) for v in ints)))
        d.update(xmin=dbls[0], ymin=dbls[1], zmin=dbls[2], box=dbls[3], pairs=int(pairs.value))
        return d

    def permutation(self):
        out = np.empty(self.n, np.int32)
        self._check(N.lib().prbf_get_permutation(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out

    def cell_start(self):
        out = np.empty(self.matvec_info()["ncell"] + 1, np.int32)
        self._check(N.lib().prbf_get_cell_start(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out

    def trunc_counts(self):
        out = np.empty(self.matvec_info()["ncell"], np.int32)
        self._check(N.lib().prbf_get_trunc_counts(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out

    def pc_setup(self, precision="fp64"):
        self._check(N.lib().prbf_pc_setup(self.h, {"fp64": N.PREC_FP64, "mixed": N.PREC_MIXED}[precision]))

    def pc_apply(self, r):
        r = _f64(r)
        if self.n is None:
            raise PrbfError(N.ERR_STATE, "matvec_setup has not been called")
        _check_len(self.n, r=r)
        out = np.empty_like(r)
        self._check(N.lib().prbf_pc_apply(self.h, _ptr(r), _ptr(out)))
        return out

    def pc_buffer_lists(self):
        """The Schwarz subdomains of the last pc_setup (Get_buffer::get_buffer): offsets
        (ncell + 1) and the sorted positions of every cell's subdomain, centre first."""
        ncell = self.matvec_info()["ncell"]
        off = np.empty(ncell + 1, np.int64)
        self._check(N.lib().prbf_pc_buffer_lists(self.h, off.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                                  None))
        idx = np.empty(max(int(off[-1]), 1), np.int32)
        self._check(N.lib().prbf_pc_buffer_lists(self.h, off.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                                  idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return off, idx[:int(off[-1])]

    def pc_block(self, cell, block=True, factor=True):
        """(nb, nc, K, L) of one subdomain: K = 2 pi sigma^2 A_c as the FP64 factorisation
        assembles it (neighbour points first, then the centre), L the packed factor rows as
        stored (row i: L[i][0..i-1], 1/L[i][i]; FP64 set-up only)."""
        nb, nc = ctypes.c_int(0), ctypes.c_int(0)
        self._check(N.lib().prbf_pc_block(self.h, int(cell), ctypes.byref(nb), ctypes.byref(nc), None, None))
        K = np.empty((nb.value, nb.value), np.float64) if block else None
        L = np.empty(nb.value * (nb.value + 1) // 2, np.float64) if factor else None
        if nb.value:
            self._check(N.lib().prbf_pc_block(self.h, int(cell), None, None, _ptr(K), _ptr(L)))
        return nb.value, nc.value, K, L

    # ---- solve and evaluation -------------------------------------------------------
    def interpolate(self, x, y, z, f):
        """Weights g with A g = f (f may hold several right-hand sides as columns)."""
        x, y, z = _f64(x), _f64(y), _f64(z)
        f = np.asarray(f, np.float64)
        n = x.shape[0]
        _check_len(n, y=y, z=z, f=f)
        if self.dim == 3 and z is None:
            raise ValueError("a 3D context needs z")
        nrhs = 1 if f.ndim == 1 else f.shape[1]
        fr = np.ascontiguousarray(f.T if f.ndim == 2 else f)
        g = np.empty_like(fr)
        st = Stats()
        code = N.lib().prbf_interpolate(self.h, n, _ptr(x), _ptr(y), _ptr(z), _ptr(fr), nrhs, _ptr(g),
                                        ctypes.byref(st))
        if code:
            err = PrbfError(code, N.lib().prbf_last_error(self.h).decode())
            err.stats = st  # iterations, residuals and times up to the failure
            raise err
        return (g.T.copy() if f.ndim == 2 else g), st

    def evaluate(self, xt, yt, zt, xs, ys, zs, gs):
        xt, yt, zt, xs, ys, zs, gs = map(_f64, (xt, yt, zt, xs, ys, zs, gs))
        _check_len(xt.shape[0], yt=yt, zt=zt)
        _check_len(xs.shape[0], ys=ys, zs=zs, gs=gs)
        if self.dim == 3 and (zt is None or zs is None):
            raise ValueError("a 3D context needs z coordinates")
        w = np.empty(xt.shape[0], np.float64)
        self._check(N.lib().prbf_evaluate(self.h, xt.shape[0], _ptr(xt), _ptr(yt), _ptr(zt), xs.shape[0],
                                           _ptr(xs), _ptr(ys), _ptr(zs), _ptr(gs), _ptr(w)))
        return w


def batch_interpolate(problems, dim=2, rtol=1e-13, restart=30, max_it=1000, pc="asm", device=0,
                      precision="fp64", block_fallback="shift"):
    """Solves many independent problems together. problems: sequence of dicts with keys x,
    y, (z), f, sigma, nsigma_box, sigma_buffer, sigma_trunc. precision "mixed": FP32 sums
    and block factors inside FP64 refinement per problem. Returns (list of weight arrays,
    iterations per problem, reason per problem, BatchStats)."""
    keep, probs, outs = [], [], []
    for q in problems:
        arrs = [_f64(q[k]) for k in ("x", "y")] + [_f64(q.get("z")), _f64(q["f"])]
        _check_len(arrs[0].shape[0], y=arrs[1], z=arrs[2], f=arrs[3])
        if dim == 3 and arrs[2] is None:
            raise ValueError("3D problems need z")
        g = np.empty(arrs[0].shape[0], np.float64)
        keep.append(arrs)
        outs.append(g)
        ptr = lambda a: a.ctypes.data if a is not None else None
        probs.append(N.Problem(arrs[0].shape[0], ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(arrs[3]),
                               float(q["sigma"]), int(q["nsigma_box"]), int(q["sigma_buffer"]),
                               int(q["sigma_trunc"]), g.ctypes.data))
    arr = (N.Problem * len(probs))(*probs)
    its = np.zeros(len(probs), np.int32)
    reason = np.zeros(len(probs), np.int32)
    st = N.BatchStats()
    with Context(dim=dim, rtol=rtol, restart=restart, max_it=max_it, pc=pc, device=device,
                 precision=precision, block_fallback=block_fallback) as c:
        code = N.lib().prbf_batch_interpolate(c.h, len(probs), arr, its.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                              reason.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                              ctypes.byref(st))
        if code:
            err = PrbfError(code, N.lib().prbf_last_error(c.h).decode())
            err.stats = st
            if code in (N.ERR_NOT_CONVERGED, N.ERR_BREAKDOWN, N.ERR_NAN, N.ERR_DIVERGED):
                err.results = (outs, its, reason)  # every problem's weights and stop reason
            raise err
    return outs, its, reason, st


class GaussianOperator:
    """The truncated Gaussian operator of a point set (the reference's MatShell M)."""

    def __init__(self, x, y, z, sigma, nsigma_box, sigma_buffer, sigma_trunc, device=0):
        self.ctx = Context(dim=3 if z is not None else 2, sigma=sigma, nsigma_box=nsigma_box,
                           sigma_buffer=sigma_buffer, sigma_trunc=sigma_trunc, device=device)
        self.ctx.matvec_setup(x, y, z)

    def mult(self, v):
        return self.ctx.matvec(v)

    __matmul__ = mult


def rbf_interpolation(xi, yi, *args, **opts):
    """rbf_interpolation(xi, yi, [zi,] wi, sigma, nsigma_box, sigma_buffer, sigma_trunc)
    -> (gi, its). Solves for the Gaussian weights gi that reproduce wi at the points
    (2d/rbf_interpolation.cxx:25-26; 3d/rbf_interpolation.cxx:26-27)."""
    if len(args) == 6:
        zi, wi, sigma, nb, nbuf, nt = args
    elif len(args) == 5:
        zi = None
        wi, sigma, nb, nbuf, nt = args
    else:
        raise TypeError("rbf_interpolation(xi, yi, [zi,] wi, sigma, nsigma_box, sigma_buffer, sigma_trunc)")
    with Context(dim=3 if zi is not None else 2, sigma=sigma, nsigma_box=nb, sigma_buffer=nbuf,
                 sigma_trunc=nt, **opts) as c:
        g, st = c.interpolate(xi, yi, zi, wi)
    return g, st.its


def RBFInterpolation(xg, yg, zg, wg, xp, yp, zp, gp, sigma, nsigma_box, sigma_buffer,
                     sigma_trunc):
    """The librbf.a entry (3d/wrapper.cxx:20-105): FP32 arrays; evaluates the particles
    (xp, yp, zp, gp) at the grid first when xg[0] != xp[0], solves on the grid and
    writes the weights over wg (in place). Returns the status code."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (xg, yg, zg, xp, yp, zp, gp)]
    if not (isinstance(wg, np.ndarray) and wg.dtype == np.float32 and wg.flags.c_contiguous):
        raise TypeError("wg must be a contiguous float32 array (it is overwritten)")
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    xg_, yg_, zg_, xp_, yp_, zp_, gp_ = arrs
    _check_len(len(xg_), yg=yg_, zg=zg_, wg=wg)
    _check_len(len(xp_), yp=yp_, zp=zp_, gp=gp_)
    return N.lib().prbf_RBFInterpolation(0, None, len(xg_), fp(xg_), fp(yg_), fp(zg_), fp(wg),
                                         len(xp_), fp(xp_), fp(yp_), fp(zp_), fp(gp_),
                                         float(sigma), int(nsigma_box), int(sigma_buffer),
                                         int(sigma_trunc))


def gpumatmult(tx, ty, tz, sx, sy, sz, sg, offset, sigma, num_cluster=None, num_trunc=None):
    """The reference's GPU seam (2d/gpumatmult.cu:65-67; 3d/gpumatmult.cu:73-75) on packed
    FP32 arrays: tx, ty(, tz) hold iblok blocks of 128 target slots, sx, sy(, sz), sg the
    blocks' truncation sets one after the other, offset the iblok + 1 block starts (tz and
    sz None in 2D). num_cluster / num_trunc default to the tightest capacities. Returns tw
    (128 * iblok FP32 values)."""
    f32 = lambda a: np.ascontiguousarray(a, np.float32) if a is not None else None
    tx, ty, tz, sx, sy, sz, sg = (f32(a) for a in (tx, ty, tz, sx, sy, sz, sg))
    off = np.ascontiguousarray(offset, np.int32)
    iblok = len(off) - 1
    if iblok < 0 or len(tx) != 128 * iblok:
        raise ValueError("targets must hold 128 slots per block and offset iblok + 1 entries")
    _check_len(len(tx), ty=ty, tz=tz)
    for name, a in (("sx", sx), ("sy", sy), ("sz", sz), ("sg", sg)):
        if a is not None and iblok > 0 and len(a) < int(off[-1]):
            raise ValueError(f"{name} holds {len(a)} entries, fewer than offset[-1] = {int(off[-1])}")
    ncl = iblok if num_cluster is None else int(num_cluster)
    ntr = (max(1, -(-int(off[-1]) // max(ncl, 1))) if iblok else 0) if num_trunc is None else int(num_trunc)
    tw = np.zeros(128 * iblok, np.float32)
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    ip = off.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    if tz is None:
        code = N.lib().prbf_gpumatmult_2d(fp(tx), fp(ty), fp(tw), fp(sx), fp(sy), fp(sg), ip, iblok,
                                          float(sigma), ncl, ntr)
    else:
        code = N.lib().prbf_gpumatmult_3d(fp(tx), fp(ty), fp(tz), fp(tw), fp(sx), fp(sy), fp(sz), fp(sg), ip,
                                          iblok, float(sigma), ncl, ntr)
    if code:
        raise PrbfError(code, "prbf_gpumatmult")
    return tw


def vorticity_evaluation(xi, yi, *args, **opts):
    """vorticity_evaluation(xi, yi, [zi,] xj, yj, [zj,] gj, sigma, nsigma_box,
    sigma_buffer, sigma_trunc) -> wi: the interpolant with weights gj at sources
    (xj, yj[, zj]) evaluated at targets (xi, yi[, zi])
    (2d/vorticity_evaluation.cxx:26-27, 2d/get_vorticity.h:9-27)."""
    if len(args) == 9:
        zi, xj, yj, zj, gj, sigma, nb, nbuf, nt = args
    elif len(args) == 7:
        zi = zj = None
        xj, yj, gj, sigma, nb, nbuf, nt = args
    else:
        raise TypeError("vorticity_evaluation(xi, yi, [zi,] xj, yj, [zj,] gj, sigma, ...)")
    with Context(dim=3 if zi is not None else 2, sigma=sigma, nsigma_box=nb, sigma_buffer=nbuf,
                 sigma_trunc=nt, **opts) as c:
        return c.evaluate(xi, yi, zi, xj, yj, zj, gj)
