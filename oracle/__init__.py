"""Test oracle for the PetRBF solve path -- TEST INFRASTRUCTURE ONLY.

``oracle`` wraps two shared libraries with ctypes:

* ``liboracle.so`` -- the C++ restatement of the reference's solve path
  (prbf_oracle.cpp; every function there cites the reference file:line it follows);
* ``libref2d.so`` / ``libref3d.so`` -- the reference's own cell-list, truncation,
  buffer, matvec, block and evaluation code compiled unmodified against a sequential
  PETSc/MPI stand-in (only where the reference tree is present; used to generate the
  golden fixtures in tests/golden).

Only tests/, bench.py's CPU baseline and ``__graft_entry__.smoke()`` may import this
package, and only as the checker. The product (``petrbf_gb300``) never touches it.

Parity status: cell list, truncation/buffer sets, matvec, blocks and evaluation are
pinned against the reference's own code; GMRES, PCASM and the dense LU come from PETSc
(third-party, unversioned, absent here) and are restated from its documented defaults,
so iteration counts are "parity unpinned".
"""
import ctypes
import os

import numpy as np

from . import build as _build

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_L = ctypes.POINTER(ctypes.c_longlong)


class Grid(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("nz", ctypes.c_int), ("ncell", ctypes.c_int), ("nsigma_box", ctypes.c_int),
                ("sigma_buffer", ctypes.c_int), ("sigma_trunc", ctypes.c_int),
                ("nb_trunc", ctypes.c_int), ("nb_buffer", ctypes.c_int),
                ("sigma", ctypes.c_double), ("xmin", ctypes.c_double), ("ymin", ctypes.c_double),
                ("zmin", ctypes.c_double), ("box", ctypes.c_double),
                ("trunc_len", ctypes.c_double), ("buffer_len", ctypes.c_double)]


_lib = None
_ref = {}


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build_oracle())
        _lib.orc_rasm_create.restype = ctypes.c_void_p
        _lib.orc_rasm_apply.argtypes = [ctypes.c_void_p, _D, _D]
        _lib.orc_rasm_destroy.argtypes = [ctypes.c_void_p]
        _lib.orc_rasm_set_type.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib.orc_rasm_create_kind.restype = ctypes.c_void_p
        _lib.orc_rasm_block_info.argtypes = [ctypes.c_void_p, ctypes.c_int, _I, _I, _I]
        _lib.orc_rasm_factor_rows.argtypes = [ctypes.c_void_p, ctypes.c_int, _D]
        _lib.orc_gmres_ex.argtypes = [ctypes.POINTER(Grid), ctypes.c_int, _D, _D, _D, _I,
                                      ctypes.c_void_p, _D, _D, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _I, _I, _D,
                                      ctypes.c_int]
        _lib.orc_gmres.argtypes = [ctypes.POINTER(Grid), ctypes.c_int, _D, _D, _D, _I,
                                   ctypes.c_void_p, _D, _D, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _I, _I, _D]
        _lib.orc_rbf_interpolation.argtypes = [
            ctypes.c_int, ctypes.c_int, _D, _D, _D, _D, ctypes.c_double, ctypes.c_int,
            ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _I, _I,
            ctypes.c_int]
        _lib.orc_vorticity_evaluation.argtypes = [
            ctypes.c_int, ctypes.c_int, _D, _D, _D, ctypes.c_int, _D, _D, _D, _D,
            ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D]
        _lib.orc_grid_make.argtypes = [ctypes.c_int] + [ctypes.c_double] * 7 + [
            ctypes.c_int] * 3 + [ctypes.POINTER(Grid)]
    return _lib


def num_threads():
    return lib().orc_num_threads()


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def _i(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _check(st, what):
    if st != 0:
        raise RuntimeError("oracle %s failed with status %d" % (what, st))


def grid_make(dim, bbox, sigma, nsigma_box, sigma_buffer, sigma_trunc):
    g = Grid()
    b = list(bbox) + [0.0] * (6 - len(bbox))
    _check(lib().orc_grid_make(dim, *[float(v) for v in b], float(sigma), int(nsigma_box),
                               int(sigma_buffer), int(sigma_trunc), ctypes.byref(g)), "grid")
    return g


def bbox(*coords):
    out = []
    for c in coords:
        if c is None:
            continue
        out += [float(np.min(c)), float(np.max(c))]
    return out


def grid_for(x, y, z, sigma, nsigma_box, sigma_buffer, sigma_trunc):
    dim = 3 if z is not None else 2
    return grid_make(dim, bbox(x, y, z), sigma, nsigma_box, sigma_buffer, sigma_trunc)


def cell_sort(g, x, y, z=None):
    x, y, z = _f64(x), _f64(y), _f64(z)
    n = x.shape[0]
    perm = np.empty(n, np.int32)
    cs = np.empty(g.ncell + 1, np.int32)
    _check(lib().orc_cell_sort(ctypes.byref(g), n, _d(x), _d(y), _d(z), _i(perm), _i(cs)),
           "cell_sort")
    return perm, cs


def trunc_counts(g, sx, sy, sz, cs_src, cs_tgt=None):
    cs_tgt = cs_src if cs_tgt is None else cs_tgt
    out = np.empty(g.ncell, np.int32)
    lib().orc_trunc_counts(ctypes.byref(g), _d(_f64(sx)), _d(_f64(sy)), _d(_f64(sz)),
                           _i(cs_src), _i(cs_tgt), _i(out))
    return out


def trunc_list(g, cell, sx, sy, sz, cs_src, cs_tgt=None):
    cs_tgt = cs_src if cs_tgt is None else cs_tgt
    cap = int(cs_src[-1])
    out = np.empty(max(cap, 1), np.int32)
    n = lib().orc_trunc_list(ctypes.byref(g), int(cell), _d(_f64(sx)), _d(_f64(sy)),
                             _d(_f64(sz)), _i(cs_src), _i(cs_tgt), _i(out))
    return out[:n].copy()


def gauss_sum(g, tx, ty, tz, cs_t, sx, sy, sz, sg, cs_s):
    w = np.zeros(len(tx), np.float64)
    lib().orc_gauss_sum(ctypes.byref(g), _d(_f64(tx)), _d(_f64(ty)), _d(_f64(tz)), _i(cs_t),
                        _d(_f64(sx)), _d(_f64(sy)), _d(_f64(sz)), _d(_f64(sg)), _i(cs_s), _d(w))
    return w


def matvec(g, xs, ys, zs, cs, v):
    """Truncated Gaussian matvec in cell order (mymatmult, 2d/matmult.cxx:6-51)."""
    return gauss_sum(g, xs, ys, zs, cs, xs, ys, zs, v, cs)


def buffer_counts(g, xs, ys, zs, cs):
    """Points of every cell's Schwarz block (2d/get_buffer.h:9-90), without the lists."""
    cnt = np.empty(g.ncell, np.int32)
    lib().orc_buffer_counts(ctypes.byref(g), _d(_f64(xs)), _d(_f64(ys)), _d(_f64(zs)),
                            _i(cs), _i(cnt))
    return cnt


def buffer_lists(g, xs, ys, zs, cs):
    cnt = np.empty(g.ncell, np.int32)
    lib().orc_buffer_counts(ctypes.byref(g), _d(_f64(xs)), _d(_f64(ys)), _d(_f64(zs)),
                            _i(cs), _i(cnt))
    off = np.zeros(g.ncell + 1, np.int64)
    np.cumsum(cnt, out=off[1:])
    idx = np.empty(max(int(off[-1]), 1), np.int32)
    lib().orc_buffer_fill(ctypes.byref(g), _d(_f64(xs)), _d(_f64(ys)), _d(_f64(zs)), _i(cs),
                          off.ctypes.data_as(_L), _i(idx))
    return off, idx[:int(off[-1])]


def block(g, idx, xs, ys, zs):
    idx = np.ascontiguousarray(idx, np.int32)
    nb = idx.shape[0]
    A = np.empty((nb, nb), np.float64)
    lib().orc_block(ctypes.byref(g), nb, _i(idx), _d(_f64(xs)), _d(_f64(ys)), _d(_f64(zs)),
                    _d(A))
    return A


def gpu_block(g, idx, nc, xs, ys, zs):
    """The block K = 2 pi sigma^2 A_c of one buffer list (centre first, nc centre points) as
    the GPU library assembles it: rows and columns neighbours first, its table exp; the full
    symmetric nb x nb matrix."""
    idx = np.ascontiguousarray(idx, np.int32)
    nb = idx.shape[0]
    K = np.zeros((nb, nb), np.float64)
    _check(lib().orc_gpu_block(ctypes.byref(g), nb, int(nc), _i(idx), _d(_f64(xs)), _d(_f64(ys)),
                               _d(_f64(zs)), _d(K)), "gpu_block")
    return np.tril(K) + np.tril(K, -1).T


FACTORS = {"lu": 0, "chol": 1, "chol_lu": 2}


class Rasm:
    """Restricted (or, with basic=True, basic) additive Schwarz. factor "lu": dense LU with
    partial pivoting (PETSc's, the reference's); "chol": the GPU library's block arithmetic
    restated (table exp, neighbours first, ordered Cholesky, its substitution order);
    "chol_lu": the same with the GPU's LU fallback for blocks whose Cholesky fails."""

    def __init__(self, g, xs, ys, zs, cs, basic=False, factor="lu"):
        self.g = g
        self.keep = (_f64(xs), _f64(ys), _f64(zs), cs)
        st = ctypes.c_int(0)
        self.h = lib().orc_rasm_create_kind(ctypes.byref(g), len(xs), _d(self.keep[0]),
                                            _d(self.keep[1]), _d(self.keep[2]), _i(cs),
                                            FACTORS[factor], ctypes.byref(st))
        self.status = st.value
        self.factor = factor
        lib().orc_rasm_set_type(self.h, 1 if basic else 0)

    def block_info(self, cell):
        nb, nc, ns = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().orc_rasm_block_info(self.h, int(cell), ctypes.byref(nb), ctypes.byref(nc),
                                         ctypes.byref(ns)), "block_info")
        return nb.value, nc.value, ns.value

    def factor_rows(self, cell):
        """factor "chol": the packed rows of a cell (row i: L_A[i][0..i-1], 1/L_A[i][i])."""
        nb, _, _ = self.block_info(cell)
        out = np.empty(nb * (nb + 1) // 2, np.float64)
        _check(lib().orc_rasm_factor_rows(self.h, int(cell), _d(out)), "factor_rows")
        return out

    def apply(self, r):
        r = _f64(r)
        out = np.zeros_like(r)
        lib().orc_rasm_apply(self.h, _d(r), _d(out))
        return out

    def close(self):
        if self.h:
            lib().orc_rasm_destroy(self.h)
            self.h = None

    __del__ = close


def gmres(g, xs, ys, zs, cs, rasm, b, x0=None, rtol=1e-13, abstol=1e-50, dtol=1e5,
          restart=30, max_it=1000, texp=False):
    """GMRES(restart) with the RASM preconditioner on the left, in cell order; texp: the
    Gaussian sums take the GPU library's table exp."""
    b = _f64(b)
    n = b.shape[0]
    x = np.zeros(n, np.float64)
    its = ctypes.c_int(0)
    reason = ctypes.c_int(0)
    hist = np.zeros(max_it + 2, np.float64)
    lib().orc_gmres_ex(ctypes.byref(g), n, _d(_f64(xs)), _d(_f64(ys)), _d(_f64(zs)), _i(cs),
                       rasm.h, _d(b), _d(_f64(x0)), rtol, abstol, dtol, restart, max_it, _d(x),
                       ctypes.byref(its), ctypes.byref(reason), _d(hist), 4 if texp else 0)
    return x, its.value, reason.value, hist[:its.value + 1].copy()


def rbf_interpolation(x, y, z, f, sigma, nsigma_box, sigma_buffer, sigma_trunc, rtol=1e-13,
                      restart=30, max_it=1000, pc="rasm", factor="lu", texp=False,
                      reverse_sums=False):
    """Weights g with A g = f, in the caller's order (2d/rbf_interpolation.cxx:25-310);
    pc "asm" selects basic additive Schwarz (-pc_asm_type basic); factor "chol" the GPU
    library's block arithmetic instead of the reference's LU; texp its table exp in the
    Gaussian sums; reverse_sums adds every row's terms last to first (same operator,
    another rounding order)."""
    x, y, z, f = _f64(x), _f64(y), _f64(z), _f64(f)
    n = x.shape[0]
    gout = np.zeros(n, np.float64)
    its = ctypes.c_int(0)
    reason = ctypes.c_int(0)
    _check(lib().orc_rbf_interpolation(3 if z is not None else 2, n, _d(x), _d(y), _d(z),
                                       _d(f), sigma, nsigma_box, sigma_buffer, sigma_trunc,
                                       rtol, restart, max_it, _d(gout), ctypes.byref(its),
                                       ctypes.byref(reason),
                                       (1 if pc == "asm" else 0) | (2 if factor != "lu" else 0)
                                       | (16 if factor == "chol_lu" else 0) | (4 if texp else 0)
                                       | (8 if reverse_sums else 0)),
           "rbf_interpolation")
    return gout, its.value, reason.value


def vorticity_evaluation(xt, yt, zt, xs, ys, zs, gs, sigma, nsigma_box, sigma_buffer,
                         sigma_trunc):
    """Interpolant at targets (2d/vorticity_evaluation.cxx:26-299)."""
    xt, yt, zt, xs, ys, zs, gs = map(_f64, (xt, yt, zt, xs, ys, zs, gs))
    w = np.zeros(xt.shape[0], np.float64)
    _check(lib().orc_vorticity_evaluation(
        3 if zt is not None else 2, xt.shape[0], _d(xt), _d(yt), _d(zt), xs.shape[0], _d(xs),
        _d(ys), _d(zs), _d(gs), sigma, nsigma_box, sigma_buffer, sigma_trunc, _d(w)),
        "vorticity_evaluation")
    return w


# ---------------------------------------------------------------------------------------
# The reference's own code (compiled against the PETSc stand-in), where available.
# ---------------------------------------------------------------------------------------
def ref_available(dim, ref_root=None):
    so = os.path.join(os.path.dirname(__file__), "_ref", "libref%dd.so" % dim)
    if os.path.exists(so):
        return True
    if ref_root and os.path.isdir(ref_root):
        _build.build_ref(ref_root)
    return os.path.exists(so)


class Ref:
    """Runs the reference's get_cluster / get_trunc / get_buffer / mymatmult / mysubmat /
    get_vorticity on one process (fixture generation only)."""

    def __init__(self, dim):
        so = os.path.join(os.path.dirname(__file__), "_ref", "libref%dd.so" % dim)
        if not os.path.exists(so):
            raise RuntimeError("reference library not built: %s" % so)
        self.dim = dim
        self.l = ctypes.CDLL(so)
        self.l.ref_blocks.restype = ctypes.c_longlong
        self.l.ref_setup.argtypes = [ctypes.c_int, _D, _D, _D, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int]
        self.l.ref_vorticity.argtypes = [ctypes.c_int, _D, _D, _D, ctypes.c_int, _D, _D, _D, _D,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, _D]

    def setup(self, x, y, z, sigma, nsigma_box, sigma_buffer, sigma_trunc):
        self.x, self.y = _f64(x), _f64(y)
        self.z = _f64(z) if self.dim == 3 else np.zeros_like(self.x)
        self.n = self.x.shape[0]
        self.ncell = self.l.ref_setup(self.n, _d(self.x), _d(self.y), _d(self.z), sigma,
                                      nsigma_box, sigma_buffer, sigma_trunc)
        # The reference sizes its 3D scratch arrays with the 2D formula
        # n_per_cell*(2*nb+1)^2 (3d/get_cluster.h:188-191); larger truncation or buffer
        # sets would overflow its heap, so refuse such inputs instead of running them.
        ints, _ = self.grid()
        zz = self.z if self.dim == 3 else None
        g = grid_for(self.x, self.y, zz, sigma, nsigma_box, sigma_buffer, sigma_trunc)
        perm, cs = cell_sort(g, self.x, self.y, zz)
        xs, ys = self.x[perm], self.y[perm]
        zs = self.z[perm] if self.dim == 3 else None
        need_t = int(trunc_counts(g, xs, ys, zs, cs).max())
        off, _ = buffer_lists(g, xs, ys, zs, cs)
        need_b = int(np.diff(off).max())
        if need_t > ints[6] or need_b > ints[7]:
            raise ValueError("input exceeds the reference's scratch capacity (trunc %d > %d "
                             "or buffer %d > %d)" % (need_t, ints[6], need_b, ints[7]))
        return self.ncell

    def grid(self):
        ints = np.zeros(8, np.int32)
        dbls = np.zeros(4, np.float64)
        self.l.ref_grid(_i(ints), _d(dbls))
        return ints, dbls

    def perm(self):
        p = np.empty(self.n, np.int32)
        self.l.ref_perm(_i(p))
        return p

    def cell_start(self):
        cs = np.empty(self.ncell + 1, np.int32)
        self.l.ref_cell_start(_i(cs))
        return cs

    def trunc_counts(self):
        c = np.empty(self.ncell, np.int32)
        self.l.ref_trunc_counts(_i(c))
        return c

    def trunc_set(self, ic):
        cap = self.n
        xo, yo, zo = (np.empty(cap, np.float64) for _ in range(3))
        k = self.l.ref_trunc_set(int(ic), _d(xo), _d(yo), _d(zo))
        return xo[:k].copy(), yo[:k].copy(), zo[:k].copy()

    def buffer(self, ic):
        idx = np.empty(self.n, np.int32)
        k = self.l.ref_buffer(int(ic), _i(idx))
        return idx[:k].copy()

    def matvec(self, g_sorted):
        g_sorted = _f64(g_sorted)
        y = np.empty(self.n, np.float64)
        st = self.l.ref_matvec(_d(g_sorted), _d(y))
        _check(st, "ref_matvec")
        return y

    def blocks(self, cells):
        cells = np.ascontiguousarray(cells, np.int32)
        tot = self.l.ref_blocks(len(cells), _i(cells), None)
        out = np.empty(max(tot, 1), np.float64)
        self.l.ref_blocks(len(cells), _i(cells), _d(out))
        return out[:tot]

    def vorticity(self, xt, yt, zt, xs, ys, zs, gs, sigma, nsigma_box, sigma_buffer,
                  sigma_trunc):
        xt, yt, xs, ys, gs = map(_f64, (xt, yt, xs, ys, gs))
        zt = _f64(zt) if self.dim == 3 else np.zeros_like(xt)
        zs = _f64(zs) if self.dim == 3 else np.zeros_like(xs)
        w = np.empty(xt.shape[0], np.float64)
        self.l.ref_vorticity(xt.shape[0], _d(xt), _d(yt), _d(zt), xs.shape[0], _d(xs), _d(ys),
                             _d(zs), _d(gs), sigma, nsigma_box, sigma_buffer, sigma_trunc,
                             _d(w))
        return w
