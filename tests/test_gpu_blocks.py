"""GPU parity of the Schwarz subdomains, blocks, factors and applies, read back through
the C ABI (prbf_pc_buffer_lists, prbf_pc_block, prbf_pc_apply):

* the buffer lists (Get_buffer::get_buffer, 2d/get_buffer.h:9-90) equal the reference's own
  lists in tests/golden, entry for entry;
* the blocks (mysubmat, 2d/matmult.cxx:83-93) agree with the reference's to the rounding
  of its exponent argument, and bit for bit with the oracle's restatement of the GPU
  library's block arithmetic;
* the FP64 factors and the preconditioner applies are bit-identical to that restatement
  (oracle Rasm factor="chol"), so one point moved between subdomains, or one operation
  reordered, fails these tests;
* with block_fallback="lu" the blocks whose Cholesky fails are factored by LU with partial
  pivoting (the reference's -sub_pc_type lu on them): the applies are bit-identical to the
  oracle's restatement of that fallback (factor="chol_lu"), and an exactly singular block
  (duplicated points) is the reference's zero-pivot failure."""
import numpy as np
import pytest

import oracle as O
from petrbf_gb300 import _native as N
from petrbf_gb300 import workloads as W
from petrbf_gb300.api import Context, PrbfError

pytestmark = pytest.mark.gpu

CASES = ["g2d_lattice100", "g2d_jitter48", "g2d_ragged", "g3d_jitter16", "g2d_cdata"]
EPS = 2.0 ** -52


def _ctx(d, **kw):
    return Context(dim=int(d["dim"]), sigma=float(d["sigma"]), nsigma_box=int(d["nsigma_box"]),
                   sigma_buffer=int(d["sigma_buffer"]), sigma_trunc=int(d["sigma_trunc"]), **kw)


def _sorted(d):
    """Coordinates in the reference's cell order and the oracle grid of a fixture."""
    z = d.get("z")
    g = O.grid_for(d["x"], d["y"], z, float(d["sigma"]), int(d["nsigma_box"]), int(d["sigma_buffer"]),
                   int(d["sigma_trunc"]))
    perm = d["perm"]
    return g, d["x"][perm], d["y"][perm], (z[perm] if z is not None else None)


def _gpu_order(nb, nc):
    """Buffer-list entry of each row of the GPU's block order (neighbours first)."""
    return np.r_[np.arange(nc, nb), np.arange(nc)]


@pytest.mark.parametrize("case", CASES)
def test_buffer_lists_equal_reference(golden, case):
    d = golden(case)
    with _ctx(d) as c:
        c.matvec_setup(d["x"], d["y"], d.get("z"))
        c.pc_setup("fp64")
        off, idx = c.pc_buffer_lists()
    np.testing.assert_array_equal(off, d["buffer_off"])
    np.testing.assert_array_equal(idx, d["buffer_idx"])


@pytest.mark.parametrize("case", CASES)
def test_blocks_match_reference_and_oracle(golden, case):
    d = golden(case)
    if "block_cells" not in d:
        pytest.skip("fixture holds no blocks")
    g, xs, ys, zs = _sorted(d)
    sigma = float(d["sigma"])
    two_pi_s2 = 2 * np.pi * sigma * sigma
    vals, bounds = [], []
    with _ctx(d) as c:
        c.matvec_setup(d["x"], d["y"], d.get("z"))
        c.pc_setup("fp64")
        off, idx = c.pc_buffer_lists()
        for cell in d["block_cells"]:
            nb, nc, K, _ = c.pc_block(int(cell), factor=False)
            ids = idx[off[cell]:off[cell + 1]]
            assert nb == len(ids) and nc == d["cell_start"][cell + 1] - d["cell_start"][cell]
            # bit for bit: the oracle's restatement of the GPU's assembly (table exp)
            np.testing.assert_array_equal(K, O.gpu_block(g, ids, nc, xs, ys, zs))
            # the reference's block, centre first: A = K / (2 pi sigma^2) in its order
            inv = np.empty(nb, np.int64)
            inv[_gpu_order(nb, nc)] = np.arange(nb)
            A = K[np.ix_(inv, inv)] / two_pi_s2
            ref = O.block(g, ids, xs, ys, zs)  # bit-identical to the reference's (test_oracle)
            # each side's exponent carries a rounding of relative size eps (the reference's
            # argument -r^2/(2 sigma^2), the table's factor 1024/(2 sigma^2 ln2)), which is
            # |arg| eps in the result: measured within (2 |arg| + 3) ulps on every fixture
            dx = xs[ids][:, None] - xs[ids][None, :]
            dy = ys[ids][:, None] - ys[ids][None, :]
            r2 = dx * dx + dy * dy + ((zs[ids][:, None] - zs[ids][None, :]) ** 2 if zs is not None else 0)
            arg = r2 / (2 * sigma * sigma)
            tol = (2.0 * arg + 8.0) * EPS * np.abs(ref)
            assert np.all(np.abs(A - ref) <= tol)
            vals.append(A.ravel())
            bounds.append(tol.ravel())
    v, b = np.concatenate(vals), np.concatenate(bounds)
    assert np.all(np.abs(v[:64] - d["block_head"]) <= b[:64])
    assert abs(np.sqrt(np.sum(v * v)) - d["block_fro"][0]) <= 1e-14 * d["block_fro"][0]


@pytest.mark.parametrize("case", CASES)
def test_fp64_factors_equal_oracle_restatement(golden, case):
    d = golden(case)
    g, xs, ys, zs = _sorted(d)
    R = O.Rasm(g, xs, ys, zs, d["cell_start"].astype(np.int32), factor="chol")
    assert R.status == 0
    ncell = len(d["cell_start"]) - 1
    cells = [cc for cc in range(ncell) if d["buffer_off"][cc + 1] > d["buffer_off"][cc]]
    if len(cells) > 24:  # the 10^4-point lattice: a spread of 24 of its 100 blocks
        cells = cells[:: len(cells) // 24][:24]
    with _ctx(d) as c:
        c.matvec_setup(d["x"], d["y"], d.get("z"))
        c.pc_setup("fp64")
        for cell in cells:
            nb, nc, _, L = c.pc_block(cell, block=False)
            np.testing.assert_array_equal(L, R.factor_rows(cell), err_msg="cell %d" % cell)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("pc", ["rasm", "asm"])
def test_fp64_apply_equals_oracle_restatement(golden, case, pc):
    d = golden(case)
    g, xs, ys, zs = _sorted(d)
    R = O.Rasm(g, xs, ys, zs, d["cell_start"].astype(np.int32), basic=pc == "asm", factor="chol")
    n = len(d["x"])
    r = np.random.default_rng(11).standard_normal(n)
    perm = d["perm"]
    ref = np.empty(n)
    ref[perm] = R.apply(r[perm])
    with _ctx(d, pc=pc) as c:
        c.matvec_setup(d["x"], d["y"], d.get("z"))
        c.pc_setup("fp64")
        out = c.pc_apply(r)
    np.testing.assert_array_equal(out, ref)
    # and the reference's LU form of the same preconditioner, to the blocks' conditioning,
    # where no block needed the shifted refactorisation (the ragged set's dense blob has
    # near-singular blocks, which LU with partial pivoting solves unshifted)
    if R.block_info(0)[2] > 0:
        return
    L = O.Rasm(g, xs, ys, zs, d["cell_start"].astype(np.int32), basic=pc == "asm")
    lu = np.empty(n)
    lu[perm] = L.apply(r[perm])
    assert np.linalg.norm(out - lu) / np.linalg.norm(lu) < 1e-7


@pytest.mark.parametrize("case", ["g2d_ragged", "g2d_jitter48"])
@pytest.mark.parametrize("pc", ["rasm", "asm"])
def test_lu_fallback_apply_equals_oracle_restatement(golden, case, pc):
    d = golden(case)
    g, xs, ys, zs = _sorted(d)
    R = O.Rasm(g, xs, ys, zs, d["cell_start"].astype(np.int32), basic=pc == "asm", factor="chol_lu")
    assert R.status == 0
    n = len(d["x"])
    r = np.random.default_rng(12).standard_normal(n)
    perm = d["perm"]
    ref = np.empty(n)
    ref[perm] = R.apply(r[perm])
    with _ctx(d, pc=pc, block_fallback="lu") as c:
        c.matvec_setup(d["x"], d["y"], d.get("z"))
        c.pc_setup("fp64")
        out = c.pc_apply(r)
        nlu = R.block_info(0)[2]
        if case == "g2d_ragged":
            assert nlu == 15  # the dense blob's near-singular blocks
            cells = [cc for cc in range(len(d["cell_start"]) - 1) if d["buffer_off"][cc + 1] > d["buffer_off"][cc]]
            refused = 0
            for cell in cells:  # an LU-factored block has no Cholesky factor to read back
                try:
                    c.pc_block(cell, block=False)
                except PrbfError as e:
                    assert e.status == N.ERR_STATE
                    refused += 1
            assert refused == nlu
    np.testing.assert_array_equal(out, ref)


def test_lu_fallback_zero_pivot_is_the_reference_failure():
    # five points repeated: their blocks are exactly singular. The reference's PETSc LU
    # stops on the zero pivot; with the LU fallback the set-up fails the same way (the
    # oracle's restatement and the reference's LU form agree), while the default shift
    # fallback factors the blocks and solves the consistent system
    p = W.lamb_oseen_lattice_1e4()
    idx = np.arange(10, 15)
    x, y = np.concatenate([p.x, p.x[idx]]), np.concatenate([p.y, p.y[idx]])
    f = np.concatenate([p.f, p.f[idx]])
    g = O.grid_for(x, y, None, *p.params())
    perm, cs = O.cell_sort(g, x, y)
    for factor in ("lu", "chol_lu"):
        assert O.Rasm(g, x[perm], y[perm], None, cs, factor=factor).status != 0
    assert O.Rasm(g, x[perm], y[perm], None, cs, factor="chol").status == 0
    kw = dict(dim=2, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
              sigma_trunc=p.sigma_trunc)
    with Context(block_fallback="lu", **kw) as c:
        with pytest.raises(PrbfError) as e:
            c.interpolate(x, y, None, f)
        assert e.value.status == N.ERR_FACTOR and "zero pivot" in str(e.value)
        # the context stays usable: the same call without the duplicates solves
        gs, st = c.interpolate(p.x, p.y, None, p.f)
        assert st.reason == 2 and st.nblocks_fallback == 0
    with Context(**kw) as c:
        _, st = c.interpolate(x, y, None, f)
        assert st.reason == 2 and st.nblocks_fallback > 0
