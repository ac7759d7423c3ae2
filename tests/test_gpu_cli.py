"""`python -m wannier90_gb300 seed` on files written in Wannier90's formats (GPU)."""
import numpy as np
import pytest

from oracle import w90_oracle as O
from wannier90_gb300 import __main__ as cli
from wannier90_gb300 import synth, w90io

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["tensor", "fp64"])
def test_cli_seed_files_to_chk(tmp_path, precision):
    p = synth.make_problem(kind="sc", a=5.0, mp=(3, 3, 3), num_wann=4, rmax=1, eps=0.2, seed=7)
    seed = str(tmp_path / "tb")
    w90io.write_win(seed + ".win", p.real_lattice, p.kpoints, p.mp_grid, 4, num_iter=30, iprint=0)
    w90io.write_mmn(seed + ".mmn", p.m, p.nnlist, p.nncell)
    w90io.write_amn(seed + ".amn", p.a)
    assert cli.run(seed, precision) == 0
    chk = w90io.read_chk(seed + ".chk")
    km = O.kmesh_get(p.real_lattice, p.kpoints)
    M = synth.to_math_m(w90io.read_mmn(seed + ".mmn", p.nnlist, p.nncell))
    A = synth.to_math_u(w90io.read_amn(seed + ".amn"))
    U0, M0 = O.overlap_project(M, A, km["nnlist"])
    r = O.wann_main(M0, U0, km, O.WannControl(num_iter=30))
    np.testing.assert_allclose(chk["centres"], r.centres, atol=1e-6)
    np.testing.assert_allclose(chk["spreads"], r.spreads, atol=1e-6)
    # near the minimum the gauge is only fixed to ~sqrt(per-step roundoff): 1e-7 for the
    # FP64 path, up to a few 1e-6 for the tensor path (M update sliced to 2^-49 of the scales)
    np.testing.assert_allclose(synth.to_math_u(chk["u"]), r.U, atol=1e-7 if precision == "fp64" else 5e-6)
