"""GPU parity of the RASM preconditioner and of the full solve (plain FP64 and mixed
precision) through the C ABI, against the oracle."""
import numpy as np
import pytest

import oracle as O
from petrbf_gb300 import workloads as W
from petrbf_gb300.api import Context, PrbfError, RBFInterpolation

pytestmark = pytest.mark.gpu

# Solved weights, plain FP64 vs the oracle (relative 2-norm), for solves run to
# convergence (rtol 1e-16): both reach the same discrete solution.
RTOL_WEIGHTS = 1e-10
# The weights' rounding floor on the 10^4-point lattice: the oracle against itself with
# only the summation order of its matvec rows reversed stops after the same iterations with
# weights 1.8e-10 apart, converged or at the reference's rtol 1e-13
# (test_oracle.py::test_weights_move_with_rounding_order_alone). The GPU's pair sums round
# differently from the oracle's row sums, so at that stopping rule the solves are compared
# with equal iteration counts and this envelope.
RTOL_WEIGHTS_AT_1E13 = 5e-10


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _halfgrid():
    """main2's evaluation grid at half the lattice spacing (2d/main2.cxx:125-137)."""
    k = -1.0 + 0.01 * np.arange(197)
    return np.repeat(k, 197), np.tile(k, 197)


def _offgrid_err(p, g, **field):
    xt, yt = _halfgrid()
    wt = O.vorticity_evaluation(xt, yt, None, p.x, p.y, None, g, *p.params())
    return W.log10_rel_error(wt, W.lamb_oseen(xt, yt, **field))


def _ctx(p, **kw):
    return Context(dim=p.dim, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                   sigma_trunc=p.sigma_trunc, **kw)


@pytest.mark.parametrize("jitter", [0.0, 0.25])
def test_rasm_apply_matches_oracle(jitter):
    p = W.lamb_oseen_2d(60, jitter=jitter, seed=4)
    r = np.random.default_rng(5).standard_normal(p.n)
    g = O.grid_for(p.x, p.y, None, *p.params())
    perm, cs = O.cell_sort(g, p.x, p.y)
    R = O.Rasm(g, p.x[perm], p.y[perm], None, cs)
    ref = np.empty(p.n)
    ref[perm] = R.apply(r[perm])
    Rc = O.Rasm(g, p.x[perm], p.y[perm], None, cs, factor="chol")
    refc = np.empty(p.n)
    refc[perm] = Rc.apply(r[perm])
    with _ctx(p) as c:
        c.matvec_setup(p.x, p.y)
        c.pc_setup("fp64")
        z64 = c.pc_apply(r)
        c.pc_setup("mixed")
        z32 = c.pc_apply(r)
    # bit for bit against the oracle's restatement of the GPU's block arithmetic
    np.testing.assert_array_equal(z64, refc)
    # Cholesky (GPU) vs partial-pivoting LU (oracle, the reference's) of the same SPD
    # blocks: both are backward stable, so they agree to about cond(A_c) * eps
    assert _rel(z64, ref) < 1e-7
    assert _rel(z32, ref) < 0.2  # FP32 factors: a preconditioner, not a solve


@pytest.mark.parametrize("case", ["g2d_lattice100", "g2d_jitter48", "g2d_cdata", "lattice400", "cells225"])
def test_mixed_restricted_apply_tracks_fp64_blocks(golden, case):
    # The FP32 restricted form (S_c, the centre rows of A_c^-1 from the tensor-core
    # Cholesky and substitutions) against the FP64 factor form of the same blocks: the
    # applies differ by the FP32 rounding of the inverses, 8e-6 to 8e-3 relative on these
    # point sets; a wrong row, column or scale of S_c shows as O(1). cells225: 15 x 15 points
    # per cell, so S_c is computed in two 128-row panels of centre points.
    if case == "lattice400":
        p = W.lamb_oseen_2d(400, jitter=0.25, seed=1)
        dim, x, y, z, prm = 2, p.x, p.y, None, p.params()
    elif case == "cells225":
        p = W.lamb_oseen_2d(150, jitter=0.25, seed=2, nsigma_box=12)
        dim, x, y, z, prm = 2, p.x, p.y, None, p.params()
    else:
        d = golden(case)
        dim, x, y, z = int(d["dim"]), d["x"], d["y"], d.get("z")
        prm = (float(d["sigma"]), int(d["nsigma_box"]), int(d["sigma_buffer"]), int(d["sigma_trunc"]))
    r = np.random.default_rng(3).standard_normal(len(x))
    with Context(dim=dim, sigma=prm[0], nsigma_box=prm[1], sigma_buffer=prm[2], sigma_trunc=prm[3], pc="rasm") as c:
        c.matvec_setup(x, y, z)
        c.pc_setup("fp64")
        z64 = c.pc_apply(r)
        c.pc_setup("mixed")
        z32 = c.pc_apply(r)
    assert np.all(np.isfinite(z32))
    assert _rel(z32, z64) < 0.03


def test_solve_lamb_oseen_lattice_1e4_fp64_converged_weights_match_oracle():
    p = W.lamb_oseen_lattice_1e4()
    go, its_o, reason_o = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), rtol=1e-16,
                                              max_it=300)
    with _ctx(p, rtol=1e-16, max_it=300) as c:
        g, st = c.interpolate(p.x, p.y, None, p.f)
    assert reason_o == 2 and st.reason == 2
    assert _rel(g, go) <= RTOL_WEIGHTS
    # GMRES stops on its Givens estimate, which can cross 1e-16 while the true residual
    # sits near 1e-13 (1e-13 against the oracle's 5.8e-16 after a restart); where it
    # stops depends on rounding, so the off-grid error (10^-12.43 for this field) agrees
    # within a factor of two here. The exact comparison is the true-residual solve below.
    assert abs(_offgrid_err(p, g) - _offgrid_err(p, go)) < 0.3


def test_true_residual_solve_matches_oracle_converged():
    """The mixed form stops on the true FP64 residual: at rtol 1e-15 it reaches the
    discrete solution, whose interpolation error must match the oracle's converged one."""
    p = W.lamb_oseen_lattice_1e4()
    go, its_o, reason_o = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), rtol=1e-16,
                                              max_it=300)
    with _ctx(p, precision="mixed", rtol=1e-15) as c:
        g, st = c.interpolate(p.x, p.y, None, p.f)
    assert st.reason == 2 and st.true_rel_resid <= 1e-15
    assert _rel(g, go) <= RTOL_WEIGHTS
    assert abs(_offgrid_err(p, g) - _offgrid_err(p, go)) < 1e-3


@pytest.mark.parametrize("case", ["lattice100", "jitter50", "jitter100"])
def test_solve_at_reference_stop_matches_oracle(case):
    """At the reference's stopping rule the GPU takes exactly the oracle's iterations, with
    the reference's LU blocks and with the GPU's own block arithmetic restated, and its
    weights lie within the rounding floor of both."""
    p = {"lattice100": W.lamb_oseen_lattice_1e4,
         "jitter50": lambda: W.lamb_oseen_2d(50, jitter=0.25, seed=8),
         "jitter100": lambda: W.lamb_oseen_2d(100, jitter=0.25, seed=3)}[case]()
    with _ctx(p) as c:
        g, st = c.interpolate(p.x, p.y, None, p.f)
    assert st.reason == 2
    for factor in ("lu", "chol"):
        go, its_o, reason_o = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), factor=factor)
        assert reason_o == 2 and st.its == its_o
        assert _rel(g, go) <= RTOL_WEIGHTS_AT_1E13


def test_solve_lamb_oseen_lattice_1e4_fp64_matches_oracle():
    p = W.lamb_oseen_lattice_1e4()
    go, its_o, reason_o = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params())
    with _ctx(p) as c:
        g, st = c.interpolate(p.x, p.y, None, p.f)
    assert st.reason == 2 and st.its == its_o
    assert st.true_rel_resid < 1e-11
    assert _rel(g, go) <= RTOL_WEIGHTS_AT_1E13
    # At the collocation points the error metric of 2d/main.cxx:130-133 equals the true
    # residual; for this well-resolved field the off-grid error (10^-12.43 converged) is
    # also at solver level, so at the 1e-13 stopping rule both agree in magnitude only.
    w = O.vorticity_evaluation(p.x, p.y, None, p.x, p.y, None, g, *p.params())
    assert W.log10_rel_error(w, p.exact) < -11
    e, eo = _offgrid_err(p, g), _offgrid_err(p, go)
    assert e < -11.5 and eo < -11.5 and abs(e - eo) < 1.0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_interpolation_error_matches_oracle_narrow_core(precision):
    """Narrow Lamb-Oseen core (nu = 0.001): the interpolation error (10^-8.8) dominates
    the solver's, so the reference's error metric must come out the same."""
    p = W.lamb_oseen_lattice_1e4()
    f = W.lamb_oseen(p.x, p.y, nu=0.001)
    go, its_o, reason_o = O.rbf_interpolation(p.x, p.y, None, f, *p.params())
    with _ctx(p, precision=precision) as c:
        g, st = c.interpolate(p.x, p.y, None, f)
    assert reason_o == 2 and st.reason == 2
    e, eo = _offgrid_err(p, g, nu=0.001), _offgrid_err(p, go, nu=0.001)
    assert e < -8 and abs(e - eo) < 1e-3


def test_solve_lamb_oseen_lattice_1e4_mixed_reaches_fp64_answer():
    p = W.lamb_oseen_lattice_1e4()
    with _ctx(p) as c:
        g64, st64 = c.interpolate(p.x, p.y, None, p.f)
    with _ctx(p, precision="mixed") as c:
        g32, st32 = c.interpolate(p.x, p.y, None, p.f)
    assert st32.reason == 2 and st32.true_rel_resid <= 1e-13
    assert st32.outer_its >= 1
    e64, e32 = _offgrid_err(p, g64), _offgrid_err(p, g32)
    assert e32 < -11.5 and abs(e32 - e64) < 1.0


def test_mixed_falls_back_to_fp64_on_ill_conditioned_points():
    # uniform-random points: blocks with smallest eigenvalues near 5e-11 (far below FP32's
    # resolution); the refinement stalls and the call is solved in FP64, to the plain
    # form's answer. A jittered lattice at h/sigma 0.97 stays in the mixed form.
    q = W.batch_scattered(nprob=1, seed=5, nmin=3000, nmax=4000)[0]
    args = (q["sigma"], q["nsigma_box"], q["sigma_buffer"], q["sigma_trunc"])
    kw = dict(sigma=q["sigma"], nsigma_box=q["nsigma_box"], sigma_buffer=q["sigma_buffer"],
              sigma_trunc=q["sigma_trunc"], pc="asm")
    with Context(precision="mixed", **kw) as c:
        gm, sm = c.interpolate(q["x"], q["y"], None, q["f"])
    with Context(**kw) as c:
        gd, sd = c.interpolate(q["x"], q["y"], None, q["f"])
    assert sm.fp64_fallback == 1 and sm.reason == 2 and sd.fp64_fallback == 0
    assert sm.its >= sd.its
    np.testing.assert_array_equal(gm, gd)  # the same FP64 solve from zero
    gr = O.grid_for(q["x"], q["y"], None, *args)
    perm, cs = O.cell_sort(gr, q["x"], q["y"])
    r = O.matvec(gr, q["x"][perm], q["y"][perm], None, cs, gm[perm]) - q["f"][perm]
    assert np.linalg.norm(r) / np.linalg.norm(q["f"]) < 1e-10
    lat = [p for p in W.batch_lattice(nprob=6, seed=9, nmin=500, nmax=6000)
           if p["meta"]["h_over_sigma"] > 0.95][0]
    with Context(precision="mixed", sigma=lat["sigma"], nsigma_box=lat["nsigma_box"],
                 sigma_buffer=lat["sigma_buffer"], sigma_trunc=lat["sigma_trunc"], pc="asm") as c:
        _, sl = c.interpolate(lat["x"], lat["y"], None, lat["f"])
    assert sl.fp64_fallback == 0 and sl.reason == 2 and sl.true_rel_resid <= 1e-13


def test_solve_jittered_and_multiple_rhs():
    p = W.lamb_oseen_2d(50, jitter=0.25, seed=8)
    f2 = np.stack([p.f, np.cos(3 * p.x) * np.sin(2 * p.y)], axis=1)
    with _ctx(p, rtol=1e-16, max_it=300) as c:
        g, st = c.interpolate(p.x, p.y, None, f2)
    for k in range(2):
        go, _, reason = O.rbf_interpolation(p.x, p.y, None, f2[:, k], *p.params(), rtol=1e-16,
                                            max_it=300)
        assert reason == 2
        assert _rel(g[:, k], go) <= RTOL_WEIGHTS


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_six_right_hand_sides(precision):
    # more right-hand sides than one launch carries (four): the sums run in chunks, each
    # right-hand side converges to the oracle's answer
    p = W.lamb_oseen_2d(40, jitter=0.25, seed=9)
    fs = np.stack([p.f * (1 + 0.1 * k) + np.sin((k + 1) * p.x) * np.cos(2 * p.y) for k in range(6)], axis=1)
    rtol = 1e-16 if precision == "fp64" else 1e-14
    with _ctx(p, rtol=rtol, max_it=400, precision=precision) as c:
        g, st = c.interpolate(p.x, p.y, None, fs)
    assert st.reason > 0
    for k in range(6):
        go, _, reason = O.rbf_interpolation(p.x, p.y, None, fs[:, k], *p.params(), rtol=1e-16, max_it=400)
        assert reason == 2
        assert _rel(g[:, k], go) <= (RTOL_WEIGHTS if precision == "fp64" else 1e-8)


def test_solve_3d_small_matches_oracle():
    # 3D jittered lattices need a wider overlap than one 2-sigma cell for RASM to work:
    # sigma_buffer = nsigma_box + 8 (4 sigma on each side); cutoff 7 sigma past the cell
    x, y, z, h = W.lattice_3d(12, jitter=0.25, seed=2)
    wx, wy, wz = W.vortex_ring(x, y, z)
    params = (h / 0.8, 2, 10, 16)
    go, its_o, reason_o = O.rbf_interpolation(x, y, z, wx, *params)
    with Context(dim=3, sigma=params[0], nsigma_box=2, sigma_buffer=10, sigma_trunc=16) as c:
        g, st = c.interpolate(x, y, z, wx)
    assert reason_o == 2 and st.reason == 2
    assert _rel(g, go) <= RTOL_WEIGHTS


def _lattice3d_problem(m, seed):
    x, y, z, h = W.lattice_3d(m, jitter=0.25, seed=seed)
    return x, y, z, (h / 0.8, 2, 6, 16)  # cell 2 sigma, 2-sigma overlap, cutoff 7 sigma


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 5e-3)])
def test_basic_asm_apply_matches_oracle_3d(precision, tol):
    x, y, z, prm = _lattice3d_problem(12, 2)
    g = O.grid_for(x, y, z, *prm)
    perm, cs = O.cell_sort(g, x, y, z)
    R = O.Rasm(g, x[perm], y[perm], z[perm], cs, basic=True)
    r = np.random.default_rng(5).standard_normal(len(x))
    ref = np.empty(len(x))
    ref[perm] = R.apply(r[perm])
    with Context(dim=3, sigma=prm[0], nsigma_box=2, sigma_buffer=6, sigma_trunc=16, pc="asm") as c:
        c.matvec_setup(x, y, z)
        c.pc_setup(precision)
        out = c.pc_apply(r)
    # FP64: Cholesky vs pivoted LU of the same blocks, and atomic adds in any order
    assert _rel(out, ref) < tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 5e-3)])
def test_restricted_apply_matches_oracle_3d(precision, tol):
    # the restricted form of the factor-form applies (back substitution over the centre rows
    # only, which start at an arbitrary row of the block): FP64 and the FP32 warp-per-block
    # substitutions against the oracle's LU blocks
    x, y, z, prm = _lattice3d_problem(12, 2)
    g = O.grid_for(x, y, z, *prm)
    perm, cs = O.cell_sort(g, x, y, z)
    R = O.Rasm(g, x[perm], y[perm], z[perm], cs, basic=False)
    r = np.random.default_rng(6).standard_normal(len(x))
    ref = np.empty(len(x))
    ref[perm] = R.apply(r[perm])
    with Context(dim=3, sigma=prm[0], nsigma_box=2, sigma_buffer=6, sigma_trunc=16, pc="rasm") as c:
        c.matvec_setup(x, y, z)
        c.pc_setup(precision)
        out = c.pc_apply(r)
    assert _rel(out, ref) < tol


def test_basic_asm_solve_3d_matches_oracle():
    # same Krylov path as the oracle's PETSc restatement: identical iteration counts
    x, y, z, prm = _lattice3d_problem(12, 2)
    wx = W.vortex_ring(x, y, z)[0]
    for rtol in (1e-12, 1e-16):
        go, its_o, reason_o = O.rbf_interpolation(x, y, z, wx, *prm, rtol=rtol, max_it=400, pc="asm")
        with Context(dim=3, sigma=prm[0], nsigma_box=2, sigma_buffer=6, sigma_trunc=16, pc="asm", rtol=rtol,
                     max_it=400) as c:
            g, st = c.interpolate(x, y, z, wx)
        assert reason_o == 2 and st.reason == 2
        assert st.its == its_o
        assert _rel(g, go) <= RTOL_WEIGHTS


def test_restricted_schwarz_stalls_on_jittered_3d_where_basic_converges():
    x, y, z, prm = _lattice3d_problem(24, 12345)
    wx = W.vortex_ring(x, y, z)[0]
    with Context(dim=3, sigma=prm[0], nsigma_box=2, sigma_buffer=6, sigma_trunc=16, rtol=1e-12, max_it=150) as c:
        with pytest.raises(PrbfError):
            c.interpolate(x, y, z, wx)
    with Context(dim=3, sigma=prm[0], nsigma_box=2, sigma_buffer=6, sigma_trunc=16, rtol=1e-12, max_it=150,
                 pc="asm") as c:
        _, st = c.interpolate(x, y, z, wx)
    assert st.reason == 2 and st.true_rel_resid < 1e-11


def test_mixed_3d_vortex_ring_components_match_fp64_oracle():
    # the 3D mixed form at small size: FP32 matvec and FP32 block Cholesky inside FP64
    # refinement to a true residual of 1e-12, three right-hand sides, each against the
    # oracle's FP64 solve; omega_z of a ring about the z axis is identically zero
    x, y, z, prm = _lattice3d_problem(16, 3)
    F = np.stack(W.vortex_ring(x, y, z), axis=1)
    with Context(dim=3, sigma=prm[0], nsigma_box=2, sigma_buffer=6, sigma_trunc=16, pc="asm", precision="mixed",
                 rtol=1e-12) as c:
        g, st = c.interpolate(x, y, z, F)
    assert st.reason in (2, 3) and st.true_rel_resid <= 1e-12
    fnorm = np.linalg.norm(F)
    for k in range(3):
        go, _, reason = O.rbf_interpolation(x, y, z, F[:, k], *prm, rtol=1e-12, max_it=400, pc="asm")
        if k == 2:
            assert reason == 3 and np.abs(g[:, k]).max() == 0.0
            continue
        assert reason == 2
        assert _rel(g[:, k], go) < 1e-9


def test_large_subdomains_above_default_shared_memory():
    # 73 x 73-point blocks: the apply kernel needs more than 48 KB of shared memory
    x, y, h = W.lattice_2d(100)
    f = W.lamb_oseen(x, y)
    for pc in ("rasm", "asm"):
        with Context(dim=2, sigma=h / 0.8, nsigma_box=16, sigma_buffer=58, sigma_trunc=32, rtol=1e-12, pc=pc) as c:
            _, st = c.interpolate(x, y, None, f)
        assert st.max_block * 8 + 32 * 33 * 8 > 48 * 1024
        assert st.reason == 2 and st.true_rel_resid < 1e-10


def test_rbfinterpolation_shim_matches_evaluate_then_solve():
    x, y, z, h = W.lattice_3d(10, jitter=0.0)
    sigma = h / 0.8
    xp, yp, zp = x + 0.3 * h, y - 0.2 * h, z + 0.1 * h
    gp = np.exp(-(xp ** 2 + yp ** 2 + zp ** 2)) * h ** 3
    wg = np.zeros(len(x), np.float32)
    st = RBFInterpolation(x, y, z, wg, xp, yp, zp, gp, sigma, 2, 6, 16)
    assert st == 0
    x32, y32, z32 = (np.asarray(a, np.float32).astype(np.float64) for a in (x, y, z))
    xp32, yp32, zp32, gp32 = (np.asarray(a, np.float32).astype(np.float64) for a in (xp, yp, zp, gp))
    s32 = float(np.float32(sigma))
    wi = O.vorticity_evaluation(x32, y32, z32, xp32, yp32, zp32, gp32, s32, 2, 6, 16)
    go, _, reason = O.rbf_interpolation(x32, y32, z32, wi, s32, 2, 6, 16)
    assert reason == 2
    assert _rel(wg.astype(np.float64), go) < 1e-6  # FP32 output


def test_solve_errors():
    p = W.lamb_oseen_lattice_1e4()
    with _ctx(p, max_it=2) as c:
        with pytest.raises(PrbfError) as e:
            c.interpolate(p.x, p.y, None, p.f)
        assert e.value.status == 5  # PRBF_ERR_NOT_CONVERGED
    with _ctx(p) as c:
        bad = p.f.copy()
        bad[7] = np.nan
        with pytest.raises(PrbfError) as e:
            c.interpolate(p.x, p.y, None, bad)
        assert e.value.status == 7  # PRBF_ERR_NAN


def test_cdata_cylinder_matches_oracle(golden):
    # the reference's scattered-data fixture (2d/cdata) with the cylinder driver's
    # parameters: the GPU solve against the oracle's stored solve
    d = golden("g2d_cdata")
    p = W.cylinder_problem(d["x"], d["y"], d["cdata_e"])
    with _ctx(p, rtol=1e-13, max_it=1000) as c:
        g, st = c.interpolate(p.x, p.y, None, p.f)
        w = c.evaluate(p.x, p.y, None, p.x, p.y, None, g)
    assert st.reason == 2 and st.its == int(d["solve_its"][0])
    assert _rel(g, d["solve_weights"]) <= RTOL_WEIGHTS_AT_1E13
    # error metric of the cylinder driver (2d/cylinder.cxx:123-127): residual level
    err = W.log10_rel_error(w, p.f)
    assert err < -13.0 and abs(err - float(d["solve_log10_err"][0])) < 0.5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_edge_point_sets(precision):
    kw = dict(nsigma_box=8, sigma_buffer=24, sigma_trunc=24, precision=precision)
    # one point: g = f 2 pi sigma^2
    with Context(sigma=0.025, **kw) as c:
        g, st = c.interpolate(np.array([0.3]), np.array([-0.2]), None, np.array([1.5]))
    # the one-point block solve is exact, so the first residual can be exactly zero
    # (PETSc's KSP_CONVERGED_ATOL, reason 3)
    assert st.reason in (2, 3) and abs(g[0] - 1.5 * 2 * np.pi * 0.025 ** 2) <= 1e-13 * g[0]
    # collinear points (a degenerate bounding box: one row of cells)
    xl = np.linspace(-1, 1, 1000)
    with Context(sigma=2.0 / 999 / 0.8, **kw) as c:
        g, st = c.interpolate(xl, np.zeros(1000), None, np.exp(-xl ** 2))
    assert st.reason == 2 and st.true_rel_resid < 1e-13
    # collisions: five points repeated with the same value -- singular blocks (the reference's
    # PETSc LU stops on the zero pivot); the blocks are factored with a diagonal shift and the
    # consistent system is still solved to the tolerance (the mixed form with its shifted FP32
    # blocks, or in FP64 when its refinement stalls -- which of the two depends on the
    # rounding of the FP32 factors)
    p = W.lamb_oseen_lattice_1e4()
    idx = np.arange(10, 15)
    x, y = np.concatenate([p.x, p.x[idx]]), np.concatenate([p.y, p.y[idx]])
    f = np.concatenate([p.f, p.f[idx]])
    with _ctx(p, precision=precision) as c:
        g, st = c.interpolate(x, y, None, f)
    assert st.reason == 2 and st.nblocks_fallback > 0 and st.true_rel_resid < 1e-12
    assert st.fp64_fallback in ((0, 1) if precision == "mixed" else (0,))
    # ... and with different values at the same point there is no solution: a clean error
    f2 = f.copy()
    f2[-5:] += 0.1
    with _ctx(p, precision=precision, max_it=200) as c:
        with pytest.raises(PrbfError) as e:
            c.interpolate(x, y, None, f2)
    assert e.value.status in (5, 10)  # PRBF_ERR_NOT_CONVERGED, or PRBF_ERR_DIVERGED (past dtol)
