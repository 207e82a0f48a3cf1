"""Generate the golden fixtures in tests/golden from the reference's own code.

Runs the reference's get_cluster / get_trunc / get_buffer / mymatmult / mysubmat /
get_vorticity (2d/ and 3d/ trees, compiled unmodified against the sequential PETSc/MPI
stand-in by oracle/build.py) on small seeded inputs and stores inputs and outputs as
.npz files. The reference tree is only present where the fixtures are generated; the
tests read the committed .npz files.

    python tests/golden/make_golden.py /path/to/petrbf
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402
from oracle import build as _build  # noqa: E402
from petrbf_gb300 import workloads as W  # noqa: E402


def _vec(n, a=0.37, b=1.3):
    k = np.arange(n, dtype=np.float64)
    return np.sin(a * k) + 0.5 * np.cos(b * k)


def _case(name, dim, x, y, z, sigma, nbox, nbuf, ntrunc, blocks=(), eval_targets=None,
          store_inputs=True):
    R = O.Ref(dim)
    ncell = R.setup(x, y, z, sigma, nbox, nbuf, ntrunc)
    ints, dbls = R.grid()
    perm = R.perm()
    cs = R.cell_start()
    tc = R.trunc_counts()
    v = _vec(len(x))
    yv = R.matvec(v)
    bl = [R.buffer(c) for c in range(ncell)]
    boff = np.zeros(ncell + 1, np.int64)
    boff[1:] = np.cumsum([len(b) for b in bl])
    bidx = np.concatenate(bl).astype(np.int32) if boff[-1] else np.zeros(0, np.int32)
    out = dict(dim=dim, sigma=sigma, nsigma_box=nbox, sigma_buffer=nbuf, sigma_trunc=ntrunc,
               grid_ints=ints, grid_dbls=dbls, perm=perm, cell_start=cs, trunc_counts=tc,
               matvec_in=v, matvec_out=yv, buffer_off=boff, buffer_idx=bidx)
    if store_inputs:
        out.update(x=x, y=y)
        if dim == 3:
            out.update(z=z)
    if blocks:
        blocks = [c for c in blocks if boff[c + 1] > boff[c]]
        vals = R.blocks(blocks)
        out.update(block_cells=np.array(blocks, np.int32),
                   block_sha256=np.array([hashlib.sha256(vals.tobytes()).hexdigest()]),
                   block_fro=np.array([np.sqrt(np.sum(vals * vals))]),
                   block_head=vals[:64].copy())
    # evaluation of the interpolant with weights v at the collocation points and, if
    # given, at separate targets (get_vorticity through vorticity_evaluation's set-up)
    gsrc = _vec(len(x), 0.11, 0.7)
    out["eval_g"] = gsrc
    out["eval_self"] = R.vorticity(x, y, z, x, y, z, gsrc, sigma, nbox, nbuf, ntrunc)
    if eval_targets is not None:
        xt, yt, zt = eval_targets
        out.update(eval_xt=xt, eval_yt=yt)
        if dim == 3:
            out.update(eval_zt=zt)
        out["eval_t"] = R.vorticity(xt, yt, zt, x, y, z, gsrc, sigma, nbox, nbuf, ntrunc)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, "N=%d cells=%d pairs=%d" % (len(x), ncell, int((np.diff(cs) * tc).sum())))


def main(ref_root):
    for d in (2, 3):
        if not O.ref_available(d, ref_root):
            raise SystemExit("reference %dd tree not found under %s" % (d, ref_root))
    # 1. the 2D lattice case of the headline workload: N=10^4, h=0.02, sigma=h/0.8
    p = W.lamb_oseen_lattice_1e4()
    xs = -1.0 + np.arange(199) * 0.01  # main2-style half-spacing evaluation grid
    xt, yt = np.repeat(xs, 199), np.tile(xs, 199)
    _case("g2d_lattice100", 2, p.x, p.y, None, *p.params(), blocks=(0, 45, 99),
          eval_targets=(xt, yt, None), store_inputs=False)
    # 2. jittered lattice (cell boundaries fall between jittered points)
    p = W.lamb_oseen_2d(48, jitter=0.25, seed=20261203)
    _case("g2d_jitter48", 2, p.x, p.y, None, *p.params(), blocks=(0, 7))
    # 3. ragged: random points with a dense blob, many empty cells, smaller cells
    rng = np.random.default_rng(99)
    x = np.concatenate([rng.uniform(-1, 1, 600), rng.normal(0.3, 0.05, 900)])
    y = np.concatenate([rng.uniform(-1, 1, 600), rng.normal(-0.2, 0.05, 900)])
    _case("g2d_ragged", 2, x, y, None, 0.02, 4, 12, 20, blocks=(0,))
    # 4. 3D jittered lattice. The reference's 3D scratch arrays hold at most
    #    n_per_cell*(2*nb+1)^2 points (3d/get_cluster.h:188-191), so the widths here keep
    #    every truncation and buffer set inside that: cell 4 sigma, 1 sigma margins.
    x, y, z, h = W.lattice_3d(16, jitter=0.25, seed=424242)
    _case("g3d_jitter16", 3, x, y, z, h / 0.8, 4, 6, 6, blocks=(0, 17),
          eval_targets=(x[::7] + 0.3 * h, y[::7] - 0.2 * h, z[::7] + 0.1 * h))
    # 5. the reference's own scattered-data fixture (2d/cdata, 5346 particles around a
    #    cylinder) with the cylinder driver's parameters (2d/cylinder.cxx:43-55,
    #    2d/Makefile:18); the oracle's solve of it (weights, iterations, error) is stored too
    x, y, g, e = W.read_cdata(os.path.join(ref_root, "2d", "cdata"))
    p = W.cylinder_problem(x, y, e)
    _case("g2d_cdata", 2, x, y, None, *p.params(), blocks=tuple(range(0, 1089, 97)))  # empty cells dropped
    gw, its, reason = O.rbf_interpolation(x, y, None, e, *p.params(), rtol=1e-13, max_it=1000)
    w = O.vorticity_evaluation(x, y, None, x, y, None, gw, *p.params())
    path = os.path.join(HERE, "g2d_cdata.npz")
    d = dict(np.load(path))
    d.update(cdata_g=g, cdata_e=e, solve_weights=gw, solve_its=np.array([its]), solve_reason=np.array([reason]),
             solve_log10_err=np.array([W.log10_rel_error(w, e)]))
    np.savez_compressed(path, **d)
    print("cdata: its %d reason %d log10 err %.4f" % (its, reason, d["solve_log10_err"][0]))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else _build.reference_tree()
    if not root:
        sys.exit("no reference tree: pass its path or set PETRBF_REFERENCE_TREE")
    main(root)
