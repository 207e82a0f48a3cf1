"""GPU parity of the cell list, the truncated Gaussian matvec (FP64 and FP32) and the
evaluation of the interpolant, through the C ABI, against the reference's own outputs
(tests/golden) and the oracle."""
import numpy as np
import pytest

import oracle as O
from petrbf_gb300 import workloads as W
from petrbf_gb300.api import Context, PrbfError

pytestmark = pytest.mark.gpu

CASES = ["g2d_lattice100", "g2d_jitter48", "g2d_ragged", "g3d_jitter16", "g2d_cdata"]
RTOL_FP64 = 1e-12  # plain FP64 matvec vs the reference, relative 2-norm
RTOL_FP32 = 2e-5   # FP32 pair arithmetic (mixed-precision inner matvec)


def _ctx(d):
    dim = int(d["dim"])
    return Context(dim=dim, sigma=float(d["sigma"]), nsigma_box=int(d["nsigma_box"]),
                   sigma_buffer=int(d["sigma_buffer"]), sigma_trunc=int(d["sigma_trunc"]))


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("case", CASES)
def test_cell_list_matches_reference(golden, case):
    d = golden(case)
    z = d.get("z") if int(d["dim"]) == 3 else None
    with _ctx(d) as c:
        c.matvec_setup(d["x"], d["y"], z)
        info = c.matvec_info()
        gi = d["grid_ints"]
        assert (info["nx"], info["ny"], info["nz"], info["ncell"], info["nb_trunc"],
                info["nb_buffer"]) == tuple(int(v) for v in gi[:6])
        assert info["box"] == d["grid_dbls"][3] and info["xmin"] == d["grid_dbls"][0]
        np.testing.assert_array_equal(c.permutation(), d["perm"])
        np.testing.assert_array_equal(c.cell_start(), d["cell_start"])
        np.testing.assert_array_equal(c.trunc_counts(), d["trunc_counts"])
        assert info["pairs"] == int((np.diff(d["cell_start"]) * d["trunc_counts"]).sum())


@pytest.mark.parametrize("case", CASES)
def test_matvec_fp64_matches_reference(golden, case):
    d = golden(case)
    z = d.get("z") if int(d["dim"]) == 3 else None
    perm = d["perm"]
    with _ctx(d) as c:
        c.matvec_setup(d["x"], d["y"], z)
        v = np.empty_like(d["matvec_in"])
        v[perm] = d["matvec_in"]          # golden vectors are in cell order
        y = c.matvec(v)[perm]
    ref = d["matvec_out"]
    assert _rel(y, ref) <= RTOL_FP64
    # per-term accuracy at the reference's level: only the summation order differs
    assert _rel(y, ref) <= 1e-14
    np.testing.assert_allclose(y, ref, rtol=0, atol=1e-14 * np.abs(ref).max())


@pytest.mark.parametrize("case", CASES)
def test_matvec_fp32_close_to_reference(golden, case):
    torch = pytest.importorskip("torch")
    d = golden(case)
    z = d.get("z") if int(d["dim"]) == 3 else None
    with _ctx(d) as c:
        c.matvec_setup(d["x"], d["y"], z)
        vin = torch.tensor(d["matvec_in"], dtype=torch.float64, device="cuda")
        out = torch.empty_like(vin)
        torch.cuda.synchronize()
        c.matvec_dev(vin.data_ptr(), out.data_ptr(), cell_order=True, fp32=True)
        c.synchronize()
        y32 = out.cpu().numpy()
        c.matvec_dev(vin.data_ptr(), out.data_ptr(), cell_order=True, fp32=False)
        c.synchronize()
        y64 = out.cpu().numpy()
    assert _rel(y64, d["matvec_out"]) <= RTOL_FP64
    assert _rel(y32, d["matvec_out"]) <= RTOL_FP32


@pytest.mark.parametrize("case", CASES)
def test_evaluation_matches_reference(golden, case):
    d = golden(case)
    dim = int(d["dim"])
    z = d.get("z") if dim == 3 else None
    with _ctx(d) as c:
        w = c.evaluate(d["x"], d["y"], z, d["x"], d["y"], z, d["eval_g"])
        assert _rel(w, d["eval_self"]) <= RTOL_FP64
        if "eval_t" in d:
            zt = d.get("eval_zt") if dim == 3 else None
            wt = c.evaluate(d["eval_xt"], d["eval_yt"], zt, d["x"], d["y"], z, d["eval_g"])
            assert _rel(wt, d["eval_t"]) <= RTOL_FP64


def test_matvec_medium_jittered_vs_oracle():
    p = W.lamb_oseen_2d(400, jitter=0.25, seed=11)  # 160k points, 8-sigma-cell geometry
    rng = np.random.default_rng(0)
    v = rng.standard_normal(p.n)
    with Context(dim=2, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                 sigma_trunc=p.sigma_trunc) as c:
        c.matvec_setup(p.x, p.y)
        y = c.matvec(v)
        perm = c.permutation()
    g = O.grid_for(p.x, p.y, None, *p.params())
    operm, cs = O.cell_sort(g, p.x, p.y)
    np.testing.assert_array_equal(perm, operm)
    yo = np.empty(p.n)
    yo[operm] = O.matvec(g, p.x[operm], p.y[operm], None, cs, v[operm])
    assert _rel(y, yo) <= RTOL_FP64


def test_matvec_linearity_large():
    """Size-independent property at the headline size class: A(a u + b v) = a Au + b Av."""
    p = W.lamb_oseen_2d(1000, jitter=0.25, seed=3)  # 10^6 points
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal(p.n), rng.standard_normal(p.n)
    with Context(dim=2, sigma=p.sigma, nsigma_box=8, sigma_buffer=24, sigma_trunc=24) as c:
        c.matvec_setup(p.x, p.y)
        au, av, aw = c.matvec(u), c.matvec(v), c.matvec(2.0 * u - 0.5 * v)
        again = c.matvec(u)
    assert _rel(aw, 2.0 * au - 0.5 * av) < 1e-13
    np.testing.assert_array_equal(au, again)  # deterministic


def test_single_point_and_single_cell():
    with Context(dim=2, sigma=0.1, nsigma_box=8, sigma_buffer=24, sigma_trunc=24) as c:
        c.matvec_setup(np.array([0.3]), np.array([-0.2]))
        y = c.matvec(np.array([2.0]))
        assert abs(y[0] - 2.0 / (2 * np.pi * 0.01)) < 1e-12 * y[0]
        x = np.random.default_rng(2).uniform(0, 0.05, 50)
        yy = np.random.default_rng(3).uniform(0, 0.05, 50)
        c.matvec_setup(x, yy)
        assert c.matvec_info()["ncell"] == 1
        gv = np.ones(50)
        r = c.matvec(gv)
        dx = x[:, None] - x[None, :]
        dy = yy[:, None] - yy[None, :]
        ref = np.exp(-(dx * dx + dy * dy) / (2 * 0.01)).sum(1) / (2 * np.pi * 0.01)
        assert _rel(r, ref) < 1e-14


def test_errors_are_reported():
    with Context(dim=2, sigma=0.1) as c:
        with pytest.raises(PrbfError) as e:
            c.matvec(np.ones(3))
        assert e.value.status == 8  # PRBF_ERR_STATE
        with pytest.raises(PrbfError) as e:
            c.matvec_setup(np.array([0.0, np.nan]), np.array([0.0, 1.0]))
        assert e.value.status == 2  # PRBF_ERR_RANGE


def test_bounded_wait_timeout_is_reported_and_the_context_survives():
    # the failure path of the kernels' bounded mbarrier waits, made to run out on purpose by
    # a wait that nothing completes (no copy or MMA in flight): PRBF_ERR_TIMEOUT, then the
    # same context computes correctly
    from petrbf_gb300 import _native as N
    with Context(dim=2, sigma=0.1) as c:
        assert N.lib().prbf_selftest_wait_timeout(c.h, 256) == N.ERR_TIMEOUT
        assert "gave up" in N.lib().prbf_last_error(c.h).decode()
        assert N.lib().prbf_selftest_wait_timeout(c.h, 0) == N.ERR_ARG
        c.matvec_setup(np.array([0.3]), np.array([-0.2]))
        y = c.matvec(np.array([2.0]))
        assert abs(y[0] - 2.0 / (2 * np.pi * 0.01)) < 1e-12 * y[0]


@pytest.mark.parametrize("which", ["lamb_oseen_jitter_4e6", "vortex_ring_3d"])
def test_full_size_matvec_rows_against_oracle(which):
    # the full-size workloads (4x10^6 points in 2D, 128^3 in 3D): 2000 sampled rows of the
    # GPU's FP64 sum against the oracle's evaluation of the same sum at those points, and
    # the FP32 sum's rows within its own tolerance
    p = getattr(W, which)()
    z = p.z if p.dim == 3 else None
    rng = np.random.default_rng(5)
    v = rng.standard_normal(p.n)
    import torch
    with Context(dim=p.dim, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                 sigma_trunc=p.sigma_trunc) as c:
        c.matvec_setup(p.x, p.y, z)
        y = c.matvec(v)
        vt = torch.from_numpy(v).cuda()
        ot = torch.empty_like(vt)
        torch.cuda.synchronize()
        c.matvec_dev(vt.data_ptr(), ot.data_ptr(), cell_order=False, fp32=True)
        c.synchronize()
        y32 = ot.cpu().numpy()
    k = rng.choice(p.n, 2000, replace=False)
    zk = z[k] if z is not None else None
    yo = O.vorticity_evaluation(p.x[k], p.y[k], zk, p.x, p.y, z, v, *p.params())
    scale = np.max(np.abs(yo))
    assert np.max(np.abs(y[k] - yo)) <= 1e-12 * scale
    assert np.max(np.abs(y32[k] - yo)) <= 1e-4 * scale


def test_symmetric_form_where_it_applies():
    # The 10^4-point lattice (5 x 5 window: 12 upper cells): the FP64 product takes the
    # symmetric form (sum + gather); a 3D 7 x 7 x 7 window (171 upper cells) keeps the
    # one-sided kernel; FP32 products are the conversion and the sum
    p = W.lamb_oseen_lattice_1e4()
    with Context(dim=2, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                 sigma_trunc=p.sigma_trunc) as c:
        c.matvec_setup(p.x, p.y)
        assert c.matvec_kernels() == (2, True)
        assert c.matvec_kernels(fp32=True) == (2, False)
    x, y, z, h = W.lattice_3d(12, jitter=0.25, seed=1)
    with Context(dim=3, sigma=h / 0.8, nsigma_box=3, sigma_buffer=7, sigma_trunc=17) as c:
        c.matvec_setup(x, y, z)
        assert c.matvec_info()["nb_trunc"] == 3
        assert c.matvec_kernels() == (1, False)
