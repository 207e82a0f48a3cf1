"""prbf_cell_sort_static: the cell sort for callers that must not allocate device memory
(an application that keeps the whole GPU in its own memory pool, or a latency-critical
loop that cannot pay for the device synchronisation of cudaMalloc/cudaFree). Its result
must be the allocating cell sort's, bit for bit, on consecutive calls that reuse the
library's fixed scratch array. Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from petrbf_gb300 import _native as N
from petrbf_gb300 import workloads as W
from petrbf_gb300.api import Context

pytestmark = pytest.mark.gpu

MAX_POINTS = 1048576  # PRBF_STATIC_SORT_MAX_POINTS


def _cases():
    x3, y3, z3, h3 = W.lattice_3d(40, jitter=0.25, seed=9)
    # a sparse 3D cloud in cells of 0.01: 200^3 = 8,000,000 cells, so the cell-start scan
    # needs its second level (more than 2048 x 2048 entries)
    rs = np.random.default_rng(17)
    xs, ys, zs = (rs.uniform(-1.0, 1.0, 5000) for _ in range(3))
    return [
        (2, W.lamb_oseen_lattice_1e4().x, W.lamb_oseen_lattice_1e4().y, None, (0.025, 8, 24, 24)),
        (2, *W.lattice_2d(1000, jitter=0.25, seed=3)[:2], None, (1.25e-3 * 2, 8, 24, 24)),
        (3, x3, y3, z3, (h3 / 0.8, 2, 10, 16)),
        (3, xs, ys, zs, (0.01, 1, 3, 3)),
    ]


@pytest.mark.parametrize("case", range(4))
def test_static_sort_equals_allocating_sort_on_two_calls(case):
    torch = pytest.importorskip("torch")
    dim, x, y, z, prm = _cases()[case]
    n = len(x)
    with Context(dim=dim, sigma=prm[0], nsigma_box=prm[1], sigma_buffer=prm[2], sigma_trunc=prm[3]) as c:
        c.matvec_setup(x, y, z)
        perm_ref = c.permutation()
        cs_ref = c.cell_start()
    L = N.lib()
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    yd = torch.tensor(y, dtype=torch.float64, device="cuda")
    zd = torch.tensor(z, dtype=torch.float64, device="cuda") if z is not None else None
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    cs = torch.empty(len(cs_ref) + 16, dtype=torch.int32, device="cuda")
    for _ in range(2):
        perm.fill_(-7)
        cs.fill_(-7)
        torch.cuda.synchronize()
        ncell = ctypes.c_int(-1)
        st = L.prbf_cell_sort_static(dim, n, xd.data_ptr(), yd.data_ptr(),
                                     zd.data_ptr() if zd is not None else None, prm[0], prm[1],
                                     prm[2], prm[3], perm.data_ptr(), cs.data_ptr(), cs.numel(),
                                     ctypes.byref(ncell), None)
        torch.cuda.synchronize()
        assert st == 0
        assert ncell.value == len(cs_ref) - 1
        np.testing.assert_array_equal(perm.cpu().numpy(), perm_ref)
        np.testing.assert_array_equal(cs.cpu().numpy()[: ncell.value + 1], cs_ref)


def test_static_sort_rejects_sizes_beyond_its_limits():
    torch = pytest.importorskip("torch")
    L = N.lib()
    one = torch.zeros(4, dtype=torch.float64, device="cuda")
    ibuf = torch.zeros(4, dtype=torch.int32, device="cuda")
    ncell = ctypes.c_int(-1)
    st = L.prbf_cell_sort_static(2, MAX_POINTS + 1, one.data_ptr(), one.data_ptr(), None, 0.1, 8,
                                 24, 24, ibuf.data_ptr(), ibuf.data_ptr(), 4, ctypes.byref(ncell), None)
    assert st == N.ERR_CAPACITY
    # cell_start capacity smaller than ncell + 1
    p = W.lamb_oseen_lattice_1e4()
    xd = torch.tensor(p.x, device="cuda")
    yd = torch.tensor(p.y, device="cuda")
    perm = torch.empty(p.n, dtype=torch.int32, device="cuda")
    cs = torch.empty(8, dtype=torch.int32, device="cuda")
    ncell.value = -1
    st = L.prbf_cell_sort_static(2, p.n, xd.data_ptr(), yd.data_ptr(), None, p.sigma, 8, 24, 24,
                                 perm.data_ptr(), cs.data_ptr(), cs.numel(), ctypes.byref(ncell), None)
    assert st == N.ERR_CAPACITY
    # the refusal still reports the grid's size, so the caller can allocate and call again
    assert ncell.value == 100
