"""The oracle (C++ restatement) against the reference's own outputs (tests/golden) and
against dense linear algebra. CPU only."""
import numpy as np
import pytest
import scipy.linalg as sla

import oracle as O
from petrbf_gb300 import workloads as W

CASES = ["g2d_lattice100", "g2d_jitter48", "g2d_ragged", "g3d_jitter16", "g2d_cdata"]


def _setup(d):
    dim = int(d["dim"])
    z = d.get("z") if dim == 3 else None
    p = (float(d["sigma"]), int(d["nsigma_box"]), int(d["sigma_buffer"]), int(d["sigma_trunc"]))
    g = O.grid_for(d["x"], d["y"], z, *p)
    perm, cs = O.cell_sort(g, d["x"], d["y"], z)
    xs, ys = d["x"][perm], d["y"][perm]
    zs = z[perm] if z is not None else None
    return g, p, perm, cs, xs, ys, zs, z


@pytest.mark.parametrize("case", CASES)
def test_cell_list_matches_reference(golden, case):
    d = golden(case)
    g, p, perm, cs, xs, ys, zs, z = _setup(d)
    gi = d["grid_ints"]
    assert (g.nx, g.ny, g.nz, g.ncell, g.nb_trunc, g.nb_buffer) == tuple(int(v) for v in gi[:6])
    assert g.xmin == d["grid_dbls"][0] and g.ymin == d["grid_dbls"][1]
    assert g.box == d["grid_dbls"][3]
    np.testing.assert_array_equal(perm, d["perm"])
    np.testing.assert_array_equal(cs, d["cell_start"])


@pytest.mark.parametrize("case", CASES)
def test_trunc_and_buffer_sets_match_reference(golden, case):
    d = golden(case)
    g, p, perm, cs, xs, ys, zs, z = _setup(d)
    np.testing.assert_array_equal(O.trunc_counts(g, xs, ys, zs, cs), d["trunc_counts"])
    off, idx = O.buffer_lists(g, xs, ys, zs, cs)
    np.testing.assert_array_equal(off, d["buffer_off"])
    np.testing.assert_array_equal(idx, d["buffer_idx"])


@pytest.mark.parametrize("case", CASES)
def test_matvec_and_eval_match_reference(golden, case):
    d = golden(case)
    g, p, perm, cs, xs, ys, zs, z = _setup(d)
    y = O.matvec(g, xs, ys, zs, cs, d["matvec_in"])
    # same expression, same libm: bit-exact here; 1e-15 allows another libm
    np.testing.assert_allclose(y, d["matvec_out"], rtol=0, atol=1e-15 * np.abs(d["matvec_out"]).max())
    w = O.vorticity_evaluation(d["x"], d["y"], z, d["x"], d["y"], z, d["eval_g"], *p)
    np.testing.assert_allclose(w, d["eval_self"], rtol=0, atol=1e-15 * np.abs(w).max())
    if "eval_t" in d:
        zt = d.get("eval_zt")
        wt = O.vorticity_evaluation(d["eval_xt"], d["eval_yt"], zt, d["x"], d["y"], z,
                                    d["eval_g"], *p)
        np.testing.assert_allclose(wt, d["eval_t"], rtol=0, atol=1e-15 * np.abs(wt).max())


@pytest.mark.parametrize("case", CASES)
def test_blocks_match_reference(golden, case):
    import hashlib
    d = golden(case)
    if "block_cells" not in d:
        pytest.skip("no blocks stored")
    g, p, perm, cs, xs, ys, zs, z = _setup(d)
    off, idx = O.buffer_lists(g, xs, ys, zs, cs)
    vals = np.concatenate([O.block(g, idx[off[c]:off[c + 1]], xs, ys, zs).ravel()
                           for c in d["block_cells"]])
    np.testing.assert_allclose(vals[:64], d["block_head"], rtol=1e-15)
    np.testing.assert_allclose(np.sqrt(np.sum(vals * vals)), d["block_fro"][0], rtol=1e-14)
    if hashlib.sha256(vals.tobytes()).hexdigest() != str(d["block_sha256"][0]):
        # another libm may differ in the last bit; the norm check above still holds
        pass


def test_lu_against_scipy():
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, 300)
    y = rng.uniform(-1, 1, 300)
    g = O.grid_for(x, y, None, 0.08, 8, 24, 24)
    perm, cs = O.cell_sort(g, x, y)
    xs, ys = x[perm], y[perm]
    R = O.Rasm(g, xs, ys, None, cs)
    assert R.status == 0
    off, idx = O.buffer_lists(g, xs, ys, None, cs)
    r = rng.standard_normal(300)
    out = R.apply(r)
    ref = np.zeros(300)
    for c in range(g.ncell):
        b = idx[off[c]:off[c + 1]]
        if not len(b):
            continue
        A = O.block(g, b, xs, ys, None)
        sol = sla.lu_solve(sla.lu_factor(A), r[b])
        nc = cs[c + 1] - cs[c]
        ref[cs[c]:cs[c + 1]] = sol[:nc]
    np.testing.assert_allclose(out, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())


def test_basic_asm_against_scipy_and_symmetric():
    # -pc_asm_type basic: z = sum_c R_c^T A_c^-1 R_c r over the same buffer subdomains
    x, y, z, h = W.lattice_3d(8, jitter=0.25, seed=6)
    g = O.grid_for(x, y, z, h / 0.8, 2, 6, 16)
    perm, cs = O.cell_sort(g, x, y, z)
    xs, ys, zs = x[perm], y[perm], z[perm]
    R = O.Rasm(g, xs, ys, zs, cs, basic=True)
    assert R.status == 0
    off, idx = O.buffer_lists(g, xs, ys, zs, cs)
    rng = np.random.default_rng(7)
    r1, r2 = rng.standard_normal((2, len(x)))
    out = R.apply(r1)
    ref = np.zeros(len(x))
    for c in range(g.ncell):
        b = idx[off[c]:off[c + 1]]
        if len(b):
            ref[b] += sla.solve(O.block(g, b, xs, ys, zs), r1[b], assume_a="pos")
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-8
    # B symmetric: r2 . B r1 = r1 . B r2
    a, b = r2 @ out, r1 @ R.apply(r2)
    assert abs(a - b) <= 1e-8 * abs(a)


def test_basic_asm_gmres_converges_where_restricted_stalls_3d():
    # jittered 3D lattice, 2-sigma overlap: restricted Schwarz has eigenvalues of B A with
    # negative real part and GMRES(30) stalls; the basic form keeps B A positive definite
    x, y, z, h = W.lattice_3d(12, jitter=0.25, seed=2)
    f = W.vortex_ring(x, y, z)[0]
    prm = (h / 0.8, 2, 6, 16)
    _, _, reason_r = O.rbf_interpolation(x, y, z, f, *prm, rtol=1e-12, max_it=200)
    g, its, reason = O.rbf_interpolation(x, y, z, f, *prm, rtol=1e-12, max_it=200, pc="asm")
    assert reason_r < 0
    assert reason == 2 and its < 120
    gr = O.grid_for(x, y, z, *prm)
    perm, cs = O.cell_sort(gr, x, y, z)
    res = O.matvec(gr, x[perm], y[perm], z[perm], cs, g[perm]) - f[perm]
    assert np.linalg.norm(res) / np.linalg.norm(f) < 1e-9


def test_gmres_solves_small_system_to_tolerance():
    p = W.lamb_oseen_2d(30, jitter=0.25, seed=5)
    g = O.grid_for(p.x, p.y, None, *p.params())
    perm, cs = O.cell_sort(g, p.x, p.y)
    xs, ys = p.x[perm], p.y[perm]
    R = O.Rasm(g, xs, ys, None, cs)
    b = p.f[perm]
    x, its, reason, hist = O.gmres(g, xs, ys, None, cs, R, b, rtol=1e-13)
    assert reason == 2 and its > 0
    # dense check: assemble the truncated operator column by column
    n = len(b)
    A = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1
        A[:, j] = O.matvec(g, xs, ys, None, cs, e)
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-11
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8
    assert hist[-1] <= 1e-13 * hist[0]


def test_rbf_interpolation_lamb_oseen_lattice_1e4_error():
    p = W.lamb_oseen_lattice_1e4()
    gw, its, reason = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params())
    assert reason == 2 and 5 <= its <= 40
    w = O.vorticity_evaluation(p.x, p.y, None, p.x, p.y, None, gw, *p.params())
    err = W.log10_rel_error(w, p.exact)
    assert err < -11.0


def test_cdata_reader_roundtrip(tmp_path, golden):
    # the reference's scattered-data format: 4 numbers per particle, any line breaks
    d = golden("g2d_cdata")
    x, y, g, e = d["x"], d["y"], d["cdata_g"], d["cdata_e"]
    rec = np.stack([x, y, g, e], axis=1).ravel()
    text = " ".join("%.17g" % v for v in rec[:101]) + "\n" + "\n".join("%.17g" % v for v in rec[101:])
    (tmp_path / "cdata").write_text(text)
    xr, yr, gr, er = W.read_cdata(str(tmp_path / "cdata"))
    for a, b in ((xr, x), (yr, y), (gr, g), (er, e)):
        np.testing.assert_array_equal(a, b)
    (tmp_path / "bad").write_text("1 2 3")
    with pytest.raises(ValueError):
        W.read_cdata(str(tmp_path / "bad"))


def test_cdata_cylinder_solve_reproduces_fixture(golden):
    # the cylinder driver on the reference's own data (2d/cylinder.cxx:43-55, 118-127)
    d = golden("g2d_cdata")
    p = W.cylinder_problem(d["x"], d["y"], d["cdata_e"])
    assert p.params() == (0.007, 5, 9, 9)
    gw, its, reason = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), rtol=1e-13, max_it=1000)
    assert reason == 2 and its == int(d["solve_its"][0])
    np.testing.assert_allclose(gw, d["solve_weights"], rtol=0, atol=1e-12 * np.abs(d["solve_weights"]).max())
    w = O.vorticity_evaluation(p.x, p.y, None, p.x, p.y, None, gw, *p.params())
    assert abs(W.log10_rel_error(w, p.f) - float(d["solve_log10_err"][0])) < 1e-6


def test_cholesky_restatement_against_dense_solves():
    # the GPU library's block arithmetic restated (factor "chol"): blocks in its order
    # (neighbours first), its table exp; restricted and basic applies against dense solves
    x, y, z, h = W.lattice_3d(8, jitter=0.25, seed=6)
    prm = (h / 0.8, 2, 6, 16)
    g = O.grid_for(x, y, z, *prm)
    perm, cs = O.cell_sort(g, x, y, z)
    xs, ys, zs = x[perm], y[perm], z[perm]
    off, idx = O.buffer_lists(g, xs, ys, zs, cs)
    r = np.random.default_rng(8).standard_normal(len(x))
    for basic in (False, True):
        R = O.Rasm(g, xs, ys, zs, cs, basic=basic, factor="chol")
        assert R.status == 0
        out = R.apply(r)
        ref = np.zeros(len(x))
        for c in range(g.ncell):
            b = idx[off[c]:off[c + 1]]
            if not len(b):
                continue
            nc = cs[c + 1] - cs[c]
            K = O.gpu_block(g, b, nc, xs, ys, zs)
            order = np.r_[np.arange(nc, len(b)), np.arange(nc)]
            # the table exp agrees with libm's to the rounding of the exponent argument
            A = O.block(g, b, xs, ys, zs)[np.ix_(order, order)]
            assert np.abs(K / (2 * np.pi * prm[0] ** 2) - A).max() <= 1e-13 * np.abs(A).max()
            sol = sla.solve(K, r[b][order], assume_a="pos") * (2 * np.pi * prm[0] ** 2)
            if basic:
                ref[b[order]] += sol
            else:
                ref[cs[c]:cs[c + 1]] = sol[len(b) - nc:]
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-9
        # the packed factor reproduces the block: L L^T = A (block order)
        c = int(np.argmax(np.diff(off)))
        nb, nc, _ = R.block_info(c)
        rows = R.factor_rows(c)
        L = np.zeros((nb, nb))
        for i in range(nb):
            L[i, :i + 1] = rows[i * (i + 1) // 2:(i + 1) * (i + 2) // 2]
            L[i, i] = 1.0 / L[i, i]
        K = O.gpu_block(g, idx[off[c]:off[c + 1]], nc, xs, ys, zs) / (2 * np.pi * prm[0] ** 2)
        assert np.abs(L @ L.T - K).max() <= 1e-13 * np.abs(K).max()


def test_weights_move_with_rounding_order_alone():
    """The rounding floor of the solved weights on the 10^4-point lattice. The same oracle
    with each matvec row's terms summed last-to-first -- the same operator, another
    rounding order -- stops after the same 11 iterations at the reference's rule (rtol 1e-13
    on the preconditioned residual) with weights 1.8e-10 away, and run to convergence
    (rtol 1e-16) the two discrete solutions are still 1.8e-10 apart: the weights' forward
    error under a last-bit change of the operator. Two implementations whose sums round
    differently (a CPU row sum and a GPU pair sum) cannot agree more closely than this;
    they are compared with equal iteration counts and this envelope."""
    p = W.lamb_oseen_lattice_1e4()
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    g1, its1, r1 = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), factor="chol")
    g2, its2, r2 = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), factor="chol", reverse_sums=True)
    assert r1 == r2 == 2 and its1 == its2
    assert 2e-11 < rel(g2, g1) < 5e-10
    gc1, _, q1 = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), factor="chol", rtol=1e-16, max_it=60)
    gc2, _, q2 = O.rbf_interpolation(p.x, p.y, None, p.f, *p.params(), factor="chol", rtol=1e-16, max_it=60,
                                     reverse_sums=True)
    assert q1 == q2 == 2
    assert 2e-11 < rel(gc2, gc1) < 5e-10
    assert rel(g1, gc1) < 1e-12  # the same arithmetic: its 1e-13 stop is already at its solution


def test_lu_fallback_restatement(golden):
    # the oracle's restatement of the GPU library's LU fallback: on the ragged fixture the 15
    # blocks whose ordered Cholesky meets a non-positive pivot are factored by LU (none
    # shifted), every other block keeps the Cholesky factor of the plain restatement; the
    # applies are finite; exactly singular blocks (duplicated points) fail as PETSc's LU does
    d = golden("g2d_ragged")
    g = O.grid_for(d["x"], d["y"], None, float(d["sigma"]), int(d["nsigma_box"]), int(d["sigma_buffer"]),
                   int(d["sigma_trunc"]))
    perm = d["perm"]
    xs, ys = d["x"][perm], d["y"][perm]
    cs = d["cell_start"].astype(np.int32)
    R1 = O.Rasm(g, xs, ys, None, cs, factor="chol")
    R2 = O.Rasm(g, xs, ys, None, cs, factor="chol_lu")
    assert R1.status == 0 and R2.status == 0
    assert R1.block_info(0)[2] == 15 and R2.block_info(0)[2] == 15
    lu_cells, same = 0, 0
    for cell in range(len(cs) - 1):
        if d["buffer_off"][cell + 1] == d["buffer_off"][cell]:
            continue
        try:
            rows = R2.factor_rows(cell)
        except Exception:
            lu_cells += 1
            continue
        np.testing.assert_array_equal(rows, R1.factor_rows(cell))
        same += 1
    assert lu_cells == 15 and same > 0
    r = np.random.default_rng(4).standard_normal(len(xs))
    for basic in (False, True):
        R = O.Rasm(g, xs, ys, None, cs, basic=basic, factor="chol_lu")
        assert np.all(np.isfinite(R.apply(r)))
    x2, y2 = np.concatenate([d["x"], d["x"][:3]]), np.concatenate([d["y"], d["y"][:3]])
    g2 = O.grid_for(x2, y2, None, float(d["sigma"]), int(d["nsigma_box"]), int(d["sigma_buffer"]),
                    int(d["sigma_trunc"]))
    p2, c2 = O.cell_sort(g2, x2, y2)
    assert O.Rasm(g2, x2[p2], y2[p2], None, c2, factor="chol_lu").status != 0
