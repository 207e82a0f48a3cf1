"""Seeded synthetic inputs and the error metric of the PetRBF drivers.

The reference's drivers generate lattices and analytic fields in ``main``
(2d/main.cxx:69-111, 3d/main.cxx) and report ``log10(||w-e||_2/||e||_2)``
(2d/main.cxx:130-133). This module provides the same kind of inputs for the
workloads this package is measured on, with numpy's PCG64 generator for the seeded
jitter so the same seed gives the same points on every machine.

Parameter mapping (widths are full box widths in units of sigma, as in the reference):
cell edge 8 sigma -> nsigma_box = 8; cutoff 8 sigma past the cell edge ->
sigma_trunc = 8 + 16 = 24 (the reference's "+16" rule, 2d/main2.cxx:64-65);
one cell plus a one-cell overlap buffer -> sigma_buffer = 24.
"""
from dataclasses import dataclass, field
import math

import numpy as np


@dataclass
class Problem:
    name: str
    x: np.ndarray
    y: np.ndarray
    z: object  # np.ndarray or None (2D)
    f: np.ndarray  # right-hand side(s): (n,) or (n, nrhs)
    sigma: float
    nsigma_box: int
    sigma_buffer: int
    sigma_trunc: int
    exact: object = None  # analytic field at the points (same shape as f)
    meta: dict = field(default_factory=dict)

    @property
    def n(self):
        return int(self.x.shape[0])

    @property
    def dim(self):
        return 3 if self.z is not None else 2

    def params(self):
        return (self.sigma, self.nsigma_box, self.sigma_buffer, self.sigma_trunc)


def lamb_oseen(x, y, G=1.0, nu=0.01, t=1.0, xc=0.0, yc=0.0):
    """Lamb-Oseen vorticity G/(4 pi nu t) exp(-r^2/(4 nu t)) (2d/main.cxx:103, nu from
    2d/main2.cxx:44)."""
    r2 = (x - xc) ** 2 + (y - yc) ** 2
    return G / (4.0 * math.pi * nu * t) * np.exp(-r2 / (4.0 * nu * t))


def vortex_ring(x, y, z, R=0.5, a=0.1, gamma=1.0):
    """Gaussian-core vortex ring about the z axis: |omega| = gamma/(pi a^2) exp(-s^2/a^2)
    with s the distance to the core circle (rho = R, z = 0), directed along e_theta.
    Returns (omega_x, omega_y, omega_z); omega_z is identically zero."""
    rho = np.sqrt(x * x + y * y)
    s2 = (rho - R) ** 2 + z * z
    w = gamma / (math.pi * a * a) * np.exp(-s2 / (a * a))
    with np.errstate(invalid="ignore", divide="ignore"):
        ex = np.where(rho > 0, -y / np.where(rho > 0, rho, 1.0), 0.0)
        ey = np.where(rho > 0, x / np.where(rho > 0, rho, 1.0), 0.0)
    return w * ex, w * ey, np.zeros_like(w)


def lattice_2d(m, lo=-1.0, hi=1.0, jitter=0.0, seed=12345):
    """m x m lattice x_k = lo + k h, h = (hi-lo)/m, point i at (x[i//m], y[i%m]) like
    2d/main.cxx:106-108; optional uniform jitter of +/- jitter*h per coordinate."""
    h = (hi - lo) / m
    k = np.arange(m, dtype=np.float64)
    xs = lo + k * h
    x = np.repeat(xs, m)
    y = np.tile(xs, m)
    if jitter:
        rng = np.random.default_rng(seed)
        x = x + rng.uniform(-jitter * h, jitter * h, x.shape[0])
        y = y + rng.uniform(-jitter * h, jitter * h, y.shape[0])
    return x, y, h


def lattice_3d(m, lo=-1.0, hi=1.0, jitter=0.0, seed=12345):
    h = (hi - lo) / m
    k = lo + np.arange(m, dtype=np.float64) * h
    X, Y, Z = np.meshgrid(k, k, k, indexing="ij")
    x, y, z = X.ravel().copy(), Y.ravel().copy(), Z.ravel().copy()
    if jitter:
        rng = np.random.default_rng(seed)
        x += rng.uniform(-jitter * h, jitter * h, x.shape[0])
        y += rng.uniform(-jitter * h, jitter * h, y.shape[0])
        z += rng.uniform(-jitter * h, jitter * h, z.shape[0])
    return x, y, z, h


def lamb_oseen_2d(m, jitter=0.0, seed=12345, overlap=0.8, nsigma_box=8, name=None):
    """2D Lamb-Oseen interpolation on an m x m lattice over [-1,1]^2; sigma = h/overlap,
    cell edge nsigma_box sigma, cutoff 8 sigma past the cell edge, one-cell buffer."""
    x, y, h = lattice_2d(m, jitter=jitter, seed=seed)
    e = lamb_oseen(x, y)
    sigma = h / overlap
    ntrunc = nsigma_box + 16
    return Problem(name or "lamb_oseen_2d_%d" % m, x, y, None, e.copy(), sigma, nsigma_box,
                   3 * nsigma_box, ntrunc, exact=e,
                   meta={"m": m, "h": h, "jitter": jitter, "seed": seed, "overlap": overlap})


def lamb_oseen_lattice_1e4():
    """2D plain FP64, N = 10^4 on a 100x100 lattice over [-1,1]^2 (h = 0.02)."""
    return lamb_oseen_2d(100, name="2d_lamb_oseen_N1e4_lattice")


def lamb_oseen_jitter_4e6(m=2000, seed=12345):
    """2D plain FP64 at scale: N = 4x10^6 on a 2000x2000 lattice, +/-0.25h seeded jitter."""
    return lamb_oseen_2d(m, jitter=0.25, seed=seed, name="2d_lamb_oseen_N4e6_jitter")


def vortex_ring_3d(m=128, seed=12345, nsigma_box=3, sigma_buffer=7):
    """3D vortex ring, N = 128^3 jittered lattice, three right-hand sides; cutoff 7 sigma
    past the cell edge (sigma_trunc = nsigma_box + 14). Cell 3 sigma (~53 points) and a
    7-sigma Schwarz box (2 sigma of overlap on each side, blocks of up to 729 points): on
    GB300 this solves the 128^3 mixed problem in 7.8 s against 12.5 s for a 2-sigma cell
    with a 6-sigma box (blocks of up to 512), with fewer iterations (290 vs 316)."""
    x, y, z, h = lattice_3d(m, jitter=0.25, seed=seed)
    wx, wy, wz = vortex_ring(x, y, z)
    f = np.stack([wx, wy, wz], axis=1)
    sigma = h / 0.8
    sb = sigma_buffer
    return Problem("3d_vortex_ring_N%d" % (m ** 3), x, y, z, f.copy(), sigma, nsigma_box,
                   sb, nsigma_box + 14, exact=f,
                   meta={"m": m, "h": h, "jitter": 0.25, "seed": seed})


def batch_scattered(nprob=256, seed=2024, nmin=2000, nmax=200000, nsigma_box=4):
    """Batched 2D: nprob independent problems, N log-uniform in [nmin, nmax], points
    uniform-random in [-1,1]^2, h = 2/sqrt(N), h/sigma uniform in [0.6, 1.0], Lamb-Oseen
    right-hand side (G = 1, t = 1) with centre uniform in [-0.5,0.5]^2 and core radius
    r_c = sqrt(4 nu t) uniform in [0.1, 0.3]. Cell nsigma_box sigma (blocks of one cell
    plus a one-cell buffer, 3 nsigma_box sigma wide), cutoff 8 sigma past the cell edge.
    Returns a list of problem dicts (the batch_interpolate input) with their metadata."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nprob):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        x = rng.uniform(-1.0, 1.0, n)
        y = rng.uniform(-1.0, 1.0, n)
        h = 2.0 / math.sqrt(n)
        ratio = rng.uniform(0.6, 1.0)
        xc, yc = rng.uniform(-0.5, 0.5, 2)
        rc = rng.uniform(0.1, 0.3)
        nu = rc * rc / 4.0
        f = lamb_oseen(x, y, nu=nu, xc=xc, yc=yc)
        out.append({"x": x, "y": y, "f": f, "sigma": h / ratio, "nsigma_box": nsigma_box,
                    "sigma_buffer": 3 * nsigma_box, "sigma_trunc": nsigma_box + 16,
                    "meta": {"n": n, "h_over_sigma": ratio, "centre": (xc, yc), "core_radius": rc}})
    return out


def read_cdata(path):
    """A scattered-data file in the reference's cdata format: whitespace-separated records
    of four numbers per particle, x y g e (read in that order by 2d/cylinder.cxx:82-90;
    line breaks anywhere). Returns (x, y, g, e) as FP64 arrays."""
    with open(path) as fh:
        v = np.array(fh.read().split(), dtype=np.float64)
    if v.size == 0 or v.size % 4:
        raise ValueError("cdata: expected records of 4 numbers, got %d numbers" % v.size)
    v = v.reshape(-1, 4)
    return (v[:, 0].copy(), v[:, 1].copy(), v[:, 2].copy(), v[:, 3].copy())


def cylinder_problem(x, y, e, overlap=0.9, nsigma_box=5, buffer_factor=1.9):
    """The cylinder driver's parameters (2d/cylinder.cxx:43-55, run line 2d/Makefile:18):
    sigma = 0.007, sigma_buffer = (int)(nsigma_box * 1.9), sigma_trunc = nsigma_box + 4
    for overlap >= 0.8 + epsf (else + 6); the right-hand side is the e column."""
    sigma = 0.007
    sigma_buffer = int(nsigma_box * buffer_factor)
    sigma_trunc = nsigma_box + (6 if overlap < 0.8 + 1e-6 else 4)
    return Problem("2d_cylinder_cdata", x, y, None, e.copy(), sigma, nsigma_box, sigma_buffer, sigma_trunc,
                   exact=e, meta={"overlap": overlap})


def batch_lattice(nprob=256, seed=2025, nmin=2000, nmax=200000, nsigma_box=4):
    """The lattice counterpart of batch_scattered: the same N distribution, each problem an m x m
    lattice (m = round(sqrt(N))) over [-1,1]^2 with +/-0.25h seeded jitter, h = 2/m, h/sigma
    uniform in [0.6, 1.0], Lamb-Oseen right-hand side as in batch_scattered."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nprob):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        m = max(8, int(round(math.sqrt(n))))
        x, y, h = lattice_2d(m, jitter=0.25, seed=int(rng.integers(1 << 30)))
        ratio = rng.uniform(0.6, 1.0)
        xc, yc = rng.uniform(-0.5, 0.5, 2)
        rc = rng.uniform(0.1, 0.3)
        f = lamb_oseen(x, y, nu=rc * rc / 4.0, xc=xc, yc=yc)
        out.append({"x": x, "y": y, "f": f, "sigma": h / ratio, "nsigma_box": nsigma_box,
                    "sigma_buffer": 3 * nsigma_box, "sigma_trunc": nsigma_box + 16,
                    "meta": {"n": m * m, "h_over_sigma": ratio, "centre": (xc, yc), "core_radius": rc}})
    return out


def pack_gpumatmult_2d(m=1000, seed=1):
    """Packs a jittered m x m lattice the way the reference's host packer does
    (2d/matmultgpu.cxx:39-71) for the 8-sigma-cell geometry (cell 8 sigma, sources of a cell =
    the points of its 3 x 3 cells, which the 12 sigma truncation box spans): 128 FP32
    target slots per cell, the cells' source sets one after the other, CSR offsets."""
    x, y, h = lattice_2d(m, jitter=0.25, seed=seed)
    sigma = h / 0.8
    box = 8 * sigma + 1e-6
    x0, y0 = x.min() - 1e-6, y.min() - 1e-6
    nx, ny = int(np.ceil((x.max() + 1e-6 - x0) / box)), int(np.ceil((y.max() + 1e-6 - y0) / box))
    ix = np.minimum(((x - x0) / box).astype(np.int64), nx - 1)
    iy = np.minimum(((y - y0) / box).astype(np.int64), ny - 1)
    cell = ix * ny + iy
    order = np.argsort(cell, kind="stable")
    cs = np.zeros(nx * ny + 1, np.int64)
    np.cumsum(np.bincount(cell, minlength=nx * ny), out=cs[1:])
    xs, ys = x[order].astype(np.float32), y[order].astype(np.float32)
    gs = np.random.default_rng(seed).standard_normal(len(x)).astype(np.float32)
    tx = np.zeros(128 * nx * ny, np.float32)
    ty = np.zeros_like(tx)
    src, off = [], [0]
    for cx in range(nx):
        for cy in range(ny):
            c = cx * ny + cy
            a, b = cs[c], cs[c + 1]
            assert b - a <= 128
            tx[128 * c:128 * c + b - a] = xs[a:b]
            ty[128 * c:128 * c + b - a] = ys[a:b]
            idx = np.concatenate([np.arange(cs[jx * ny + max(cy - 1, 0)], cs[jx * ny + min(cy + 1, ny - 1) + 1])
                                  for jx in range(max(cx - 1, 0), min(cx + 1, nx - 1) + 1)])
            src.append(idx)
            off.append(off[-1] + len(idx))
    idx = np.concatenate(src)
    return tx, ty, xs[idx], ys[idx], gs[idx], np.array(off, np.int32), np.float32(sigma), int(cs[-1])


def log10_rel_error(w, e):
    """log10(||w - e||_2 / ||e||_2), 2d/main.cxx:130-133."""
    w = np.asarray(w, np.float64)
    e = np.asarray(e, np.float64)
    return float(np.log10(np.linalg.norm(w - e) / np.linalg.norm(e)))
