"""The Krylov iterations launched one kernel at a time (PRBF_KRYLOV_EAGER=1, read once per
process: how a launch list of a solve is taken) compute exactly what the CUDA graph's while
node computes: the same weights, iteration counts and residuals, FP64 and mixed."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, %r)
from petrbf_gb300 import workloads as W
from petrbf_gb300.api import Context
out = {}
p = W.lamb_oseen_2d(120, jitter=0.25, seed=4)
for prec in ("fp64", "mixed"):
    with Context(dim=2, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                 sigma_trunc=p.sigma_trunc, precision=prec, restart=10) as c:
        g, st = c.interpolate(p.x, p.y, None, p.f)
    out[prec] = {"g": g.tobytes().hex(), "its": st.its, "rnorm": st.rnorm, "resid": st.true_rel_resid}
print(json.dumps(out))
"""


def _run(eager):
    env = dict(os.environ)
    env.pop("PRBF_KRYLOV_EAGER", None)
    if eager:
        env["PRBF_KRYLOV_EAGER"] = "1"
    r = subprocess.run([sys.executable, "-c", SCRIPT % ROOT], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_eager_launches_equal_the_graph():
    a, b = _run(False), _run(True)
    for prec in ("fp64", "mixed"):
        assert a[prec]["its"] == b[prec]["its"] and a[prec]["its"] > 0
        assert a[prec]["rnorm"] == b[prec]["rnorm"] and a[prec]["resid"] == b[prec]["resid"]
        np.testing.assert_array_equal(np.frombuffer(bytes.fromhex(a[prec]["g"])),
                                      np.frombuffer(bytes.fromhex(b[prec]["g"])))
