"""The tensor-core kernels' bounded waits, driven to run out on purpose.

A copy of the library is compiled with W90G_SPIN_LIMIT=0 (no tries: every mbarrier wait
that is not skipped gives up at once; the drain limit that follows a timeout is
unchanged).  Each kernel must then record device status 2, wait for the MMAs and bulk
copies it already issued, free its tensor memory and return: the call reports the error,
and the GPU stays usable -- a normal solve in the same test afterwards gives the expected
result.  Four routes: the pipelined M update (num_wann <= 32, FP64 exp so that the M
update runs first; its producer has issued one bulk copy per stage slot, which the drain
must let land) with two accumulator sets (num_wann 8) and with the two half sets of
num_wann 32, the tensor exp (its first product's MMAs are in flight), and the
one-CTA-per-group M update (num_wann > 32, its first bulk copy in flight)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from wannier90_gb300 import build as B

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(root)r)
from wannier90_gb300 import library as w90, synth
out = []
for W, texp in %(cases)r:
    p = synth.make_problem(kind="sc", a=4.0, mp=(2, 2, 2), num_wann=W, rmax=1, eps=0.3, seed=2)
    h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_iter=5, iprint=0,
                  gpu_tensor=1, gpu_tensor_exp=texp)
    m = np.array(p.m, order="F", copy=True)
    u = np.array(p.a, order="F", copy=True)
    w90.w90_set_m_local(h, m)
    w90.w90_set_u_matrix(h, u)
    w90.w90_set_u_opt(h, np.asfortranarray(np.broadcast_to(np.eye(W, dtype=np.complex128)[:, :, None],
                                                           (W, W, len(p.kpoints))).copy()))
    rp = w90.w90_project_overlap(h)
    rw = w90.w90_wannierise(h)
    out.append(dict(W=W, texp=texp, project=rp, ierr=rw, msg=h.last_error()))
print(json.dumps(out))
"""

CASES = [(8, 0), (24, 0), (24, 1), (40, 0)]


def test_timed_out_waits_report_error_and_leave_the_gpu_usable(tmp_path):
    lib = B.build(extra_nvcc=["-DW90G_SPIN_LIMIT=0"], libdir=str(tmp_path / "spin0"))
    env = dict(os.environ, W90G_LIBRARY=lib)
    r = subprocess.run([sys.executable, "-c", CHILD % dict(root=ROOT, cases=CASES)], capture_output=True,
                       text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for c in res:
        assert c["project"] == 0, c
        assert c["ierr"] == 1 and "bounded wait ran out" in c["msg"], c
    # the normal build on the same GPU afterwards
    from oracle import w90_oracle as O
    from tests.engine_helpers import run_engine
    from wannier90_gb300 import synth
    for W, texp in CASES:
        p = synth.make_problem(kind="sc", a=4.0, mp=(2, 2, 2), num_wann=W, rmax=1, eps=0.3, seed=2)
        M, A = synth.to_math_m(p.m), synth.to_math_u(p.a)
        ctl = O.WannControl(num_iter=5)
        out = run_engine(p.real_lattice, p.kpoints, M, A, ctl, W, extra={"gpu_tensor": 1, "gpu_tensor_exp": texp})
        assert out["ierr"] == 0, out["err"]
        km = O.kmesh_get(p.real_lattice, p.kpoints)
        U0, M0 = O.overlap_project(M, A, km["nnlist"])
        rr = O.wann_main(M0, U0, km, ctl)
        assert abs(out["log"][1][3] - rr.iters[0].spread.om_tot) < 1e-9 * abs(rr.iters[0].spread.om_tot)
