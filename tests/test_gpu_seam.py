"""The reference's GPU seam gpumatmult (2d/gpumatmult.cu:65-119; 3d/gpumatmult.cu:73-133)
through prbf_gpumatmult_2d/3d, fed exactly as the reference's host packer feeds it
(2d/matmultgpu.cxx:39-71: 128 zero-padded FP32 target slots per cell, the cell's truncation
set packed after the previous cell's, CSR offsets)."""
import numpy as np
import pytest

import oracle as O
from petrbf_gb300.api import gpumatmult

pytestmark = pytest.mark.gpu

CASES = ["g2d_lattice100", "g2d_jitter48", "g2d_ragged", "g3d_jitter16", "g2d_cdata"]


def _pack(d):
    dim = int(d["dim"])
    x, y = d["x"], d["y"]
    z = d["z"] if dim == 3 else None
    prm = (float(d["sigma"]), int(d["nsigma_box"]), int(d["sigma_buffer"]), int(d["sigma_trunc"]))
    g = O.grid_for(x, y, z, *prm)
    perm, cs = O.cell_sort(g, x, y, z)
    xs, ys = x[perm], y[perm]
    zs = z[perm] if z is not None else None
    v = d["matvec_in"]  # cell order
    T = [[] for _ in range(dim)]
    S = [[] for _ in range(dim + 1)]
    off, slots = [0], []
    for ic in range(g.ncell):
        a, b = int(cs[ic]), int(cs[ic + 1])
        tl = O.trunc_list(g, ic, xs, ys, zs, cs)
        # a cell of more than 128 points takes several blocks with the same truncation set
        for t0 in range(a, max(b, a + 1), 128):
            nt = max(0, min(128, b - t0))
            for k, c in enumerate((xs, ys, zs)[:dim]):
                blk = np.zeros(128, np.float32)
                blk[:nt] = c[t0:t0 + nt]
                T[k].append(blk)
            for k, c in enumerate(((xs, ys, zs)[:dim]) + (v,)):
                S[k].append(c[tl].astype(np.float32))
            off.append(off[-1] + len(tl))
            slots.append((t0, nt))
    T = [np.concatenate(t) for t in T]
    S = [np.concatenate(s) if s else np.zeros(0, np.float32) for s in S]
    return dim, prm[0], g, T, S, np.array(off, np.int32), slots


def _expected(dim, sigma, T, S, off):
    """The same sums in FP64 from the FP32 inputs."""
    w, mag = np.zeros(len(T[0])), np.zeros(len(T[0]))
    norm = 1.0 / (2 * np.pi * sigma * sigma)
    for b in range(len(off) - 1):
        j = slice(off[b], off[b + 1])
        i = slice(128 * b, 128 * b + 128)
        d2 = sum((T[k][i].astype(np.float64)[:, None] - S[k][j].astype(np.float64)[None, :]) ** 2
                 for k in range(dim))
        e = np.exp(-d2 / (2.0 * float(np.float32(sigma)) ** 2)) * S[dim][j].astype(np.float64)[None, :]
        w[i] = e.sum(1) * norm
        mag[i] = np.abs(e).sum(1) * norm
    return w, mag


@pytest.mark.parametrize("case", CASES)
def test_gpumatmult_matches_the_sum_and_the_reference_matvec(golden, case):
    d = golden(case)
    dim, sigma, g, T, S, off, slots = _pack(d)
    tw = gpumatmult(T[0], T[1], T[2] if dim == 3 else None, S[0], S[1], S[2] if dim == 3 else None,
                    S[dim], off, np.float32(sigma), num_cluster=len(off) - 1 + 3,
                    num_trunc=int(off[-1]) // max(len(off) - 1, 1) + 1)
    we, mag = _expected(dim, sigma, T, S, off)
    # FP32 pair arithmetic and accumulation: within 1e-5 of the sum of |terms| per slot
    # (padding slots, targets at the origin, included)
    assert np.all(np.abs(tw - we) <= 1e-5 * mag + 1e-30)
    # scattered back, the cells' slots reproduce the reference's FP64 matvec up to the FP32
    # rounding of the coordinates and weights
    y = np.zeros(len(d["matvec_out"]))
    for b, (t0, nt) in enumerate(slots):
        y[t0:t0 + nt] = tw[128 * b:128 * b + nt]
    ref = d["matvec_out"]
    assert np.max(np.abs(y - ref)) <= 2e-4 * np.max(np.abs(ref))


def test_gpumatmult_long_sets_and_empty_blocks():
    # truncation sets spanning several staged chunks (2500 sources, offsets not multiples of
    # 4), an empty set (all slots 0) and a one-source set, against the FP64 sum
    rng = np.random.default_rng(4)
    sizes = [2500, 0, 1, 1031, 7]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    n = int(off[-1])
    sx, sy, sg = (rng.uniform(-0.1, 0.1, n).astype(np.float32) for _ in range(3))
    tx, ty = (rng.uniform(-0.1, 0.1, 128 * len(sizes)).astype(np.float32) for _ in range(2))
    sigma = np.float32(0.03)
    tw = gpumatmult(tx, ty, None, sx, sy, None, sg, off, sigma)
    we, mag = _expected(2, float(sigma), [tx, ty], [sx, sy, sg], off)
    assert np.all(np.abs(tw - we) <= 1e-5 * mag + 1e-30)
    assert np.all(tw[128:256] == 0)


def _ref_kernel(dim):
    from oracle import refgpu
    if not refgpu.available(dim):
        pytest.skip("the reference's gpumatmult.cu is compiled only where the reference tree is (oracle/_ref)")
    return refgpu.RefKernel(dim)


@pytest.mark.parametrize("case", CASES)
def test_gpumatmult_matches_the_reference_kernel(golden, case):
    # the reference's own kernel (2d/gpumatmult.cu:20-63, 3d:22-71, compiled unmodified) on
    # the same packed arrays: both FP32, within 2e-5 of the sum of |terms| of each slot
    d = golden(case)
    dim, sigma, g, T, S, off, slots = _pack(d)
    ref = _ref_kernel(dim)
    tr = ref(T, S, off, np.float32(sigma))
    tw = gpumatmult(T[0], T[1], T[2] if dim == 3 else None, S[0], S[1], S[2] if dim == 3 else None,
                    S[dim], off, np.float32(sigma))
    we, mag = _expected(dim, sigma, T, S, off)
    assert np.all(np.abs(tr - we) <= 2e-5 * mag + 1e-30)  # the reference kernel itself
    assert np.all(np.abs(tw - tr) <= 2e-5 * mag + 1e-30)


def test_gpumatmult_and_reference_kernel_on_a_million_points():
    # 10^6-point lattice packed as the reference's packer packs it (10,000 blocks, 8.9e6
    # sources): the two kernels agree; each runs three times so that a launch list of this
    # test shows both kernels' device times side by side
    from petrbf_gb300.workloads import pack_gpumatmult_2d
    tx, ty, sx, sy, sg, off, sigma, npts = pack_gpumatmult_2d()
    ref = _ref_kernel(2)
    args = ref.device_args([tx, ty], [sx, sy, sg], off, sigma)
    for _ in range(3):
        ref.launch(*args)
    import torch
    torch.cuda.synchronize()
    tr = args[3].cpu().numpy()
    for _ in range(3):
        tw = gpumatmult(tx, ty, None, sx, sy, None, sg, off, sigma)
    scale = np.max(np.abs(tr))
    assert np.max(np.abs(tw - tr)) <= 1e-4 * scale
