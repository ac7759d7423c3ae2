"""wann_check_unitarity (src/wannierise.F90:2594-2661): the reference stops with
'wann_check_unitarity: unitariety of final U violated' when max |U U^H - I| or
|U^H U - I| of the final U exceeds eps5 (1e-5).  The engine checks the final U on the
device (k_unitarity) and returns the same failure as ierr 1 with that message.  The
failure is driven from the input side: the projected U0 of a small problem scaled by
1.001, which the rotations U <- U dU keep non-unitary by 2e-3 (well above 1e-5); the
same U0 unscaled passes.  Both the FP64 path and the tensor path (which rebuilds U as
U0 R at the end of the solve) are covered."""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests.engine_helpers import run_engine
from wannier90_gb300 import synth

pytestmark = pytest.mark.gpu


def _projected(W=8, mp=(3, 3, 3), seed=3):
    p = synth.make_problem(kind="sc", a=4.0, mp=mp, num_wann=W, rmax=1, eps=0.3, seed=seed)
    M, A = synth.to_math_m(p.m), synth.to_math_u(p.a)
    km = O.kmesh_get(p.real_lattice, p.kpoints, 36)
    U0, M0 = O.overlap_project(M, A, km["nnlist"])
    return p, M0, U0


@pytest.mark.parametrize("tensor", [0, 1], ids=["fp64", "tensor"])
def test_non_unitary_start_fails_the_final_check(tensor):
    p, M0, U0 = _projected()
    ctl = O.WannControl(num_iter=3)
    # the projected overlaps and rotation handed to wannierise as they are (no projection)
    ok = run_engine(p.real_lattice, p.kpoints, M0, U0, ctl, U0.shape[1], project=False,
                    extra={"gpu_tensor": tensor})
    assert ok["ierr"] == 0, ok["err"]
    bad = run_engine(p.real_lattice, p.kpoints, M0, U0 * 1.001, ctl, U0.shape[1], project=False,
                     extra={"gpu_tensor": tensor})
    assert bad["ierr"] == 1
    assert "unitariety of final U violated" in bad["err"], bad["err"]
    # the solve itself ran: its spreads are finite
    assert np.all(np.isfinite(bad["log"][:, 3]))
