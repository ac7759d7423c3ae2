"""The two largest synthetic workloads against the oracle at full size.

* fcc 10x10x10 (1000 k), nntot 8, num_wann 32, run to convergence (conv_tol 1e-10 A^2 over
  5 iterations): the engine's converged state on both paths against the oracle's own
  converged run (tests/golden/fcc10_w32_conv.npz, made by tests/golden/make_converged.py).
  The 32 WFs span all orbitals of the tight-binding model, so Omega_I = 0 and the minimum
  is Omega = 0 with every WF on an orbital site.  The minimisation is chaotic: the oracle
  from M0 perturbed by 1e-15 (also in the fixture) stops after 1958 iterations at
  Omega = 7.6e-8 A^2 instead of 1535 iterations at 1.18e-7 -- where a run meets the
  1e-10 window near Omega = 0 depends on its path -- while its centres agree with the
  unperturbed run's to 6e-8 A and its spreads to 2.3e-8 A^2.  So the test holds the
  engine to the same minimum: at the configured window, converged, with Omega within 1e-8
  of the functional's scale (the projected U's spread, 1.2e4 A^2) of the oracle's; then,
  run to a 100x tighter window (a run that stops higher up, as the tensor path's first run
  does at 1.5e-6 A^2, has not yet brought its centres as close), every centre within 1e-6
  A of an oracle centre (matched as sets, modulo lattice vectors) and the spreads within
  1e-6 A^2.  Iteration counts are reported, not compared.
* sc 8x8x8 (512 k), nntot 6, num_wann 128, gauge noise 0.5: every iteration's Omega parts
  and centres against the oracle's (tests/golden/sc8_w128_window.npz) over the stable
  window -- the iterations over which the oracle agrees with itself to a tenth of the
  test's bounds (1e-9 relative, 1e-7 A) when M0 is perturbed by 1e-13 (22 iterations).
  That one perturbation stands for rounding renewed at every update: the tensor path's M
  update is exact to 2^-49 of the scales, and the FP64 path sums in another order than
  the oracle at every step (a 1e-15 perturbation of M0 alone would allow 26 iterations,
  and the FP64 engine is 3e-8 off by iteration 24).  Beyond the window the oracle's own
  runs part (1e-5 relative by iteration 33, 3e-2 by 36, three different Omega after 40
  iterations), so no implementation can be held to them there.  The 128 WFs span all
  orbitals, so Omega_I = 0 (to 1e-11) and is compared in absolute terms.
"""
import os

import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G
from tests.engine_helpers import run_engine
from wannier90_gb300 import synth

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated (tests/golden/make_converged.py)" % name)
    return np.load(path)


def _problem(name):
    p = synth.make_problem(**synth.CONFIGS[name], seed=0)
    return p, synth.to_math_m(p.m), synth.to_math_u(p.a)


def _match_centres(a, b, lattice):
    """Largest distance between the centres a[i] and their partners in b (one-to-one,
    greedy by distance), distances taken modulo lattice translations."""
    worst, _, d = G.match_centres(a, b, lattice)
    return worst, d


@pytest.mark.parametrize("tensor", [1, 0], ids=["tensor", "fp64"])
def test_fcc10_w32_converges_to_the_oracle_minimum(tensor):
    z = _load("fcc10_w32_conv.npz")
    p, M, A = _problem("fcc10_w32")
    om_ref, om_p15 = float(z["omega"][3]), float(z["p15_omega"][3])
    om0 = float(z["spread_log"][0])           # the functional's scale: Omega of the projected U
    assert bool(z["converged"]) and bool(z["p15_converged"])
    path = "tensor" if tensor else "fp64"
    # the configured run (conv_tol 1e-10 A^2 over 5 iterations)
    ctl = O.WannControl(num_iter=20000, conv_tol=1e-10, conv_window=5)
    out = run_engine(p.real_lattice, p.kpoints, M, A, ctl, p.num_wann, extra={"gpu_tensor": tensor})
    assert out["ierr"] == 0, out["err"]
    om, niter = float(out["omega"][3]), int(out["log"][-1][0])
    worst, _ = _match_centres(out["centres"].T, z["centres"], p.real_lattice)    # (W, 3) both
    msg = ("engine (%s) Omega %.6e after %d iterations, centres %.3e A from the oracle's; oracle %.6e after %d; "
           "oracle from M0 + 1e-15 noise %.6e after %d" % (path, om, niter, worst, om_ref, int(z["niter"]), om_p15,
                                                          int(z["p15_niter"])))
    print(msg)
    assert niter < 20000, "not converged: " + msg
    # Omega -> 0 at this minimum, so its relative difference is not defined; 1e-8 of the
    # functional's scale (the spread it started from) is
    assert abs(om - om_ref) <= 1e-8 * om0, "different minimum (Omega): " + msg
    # The same minimum, to the centre bound: where a run meets the window near Omega = 0
    # depends on its path (the oracle's own runs stop at 1.2e-7 and 7.6e-8), and a run that
    # stops higher has not yet brought its centres as close.  Run on with a 100x tighter
    # window, then every centre and spread against the oracle's.
    ctl2 = O.WannControl(num_iter=20000, conv_tol=1e-12, conv_window=5)
    out2 = run_engine(p.real_lattice, p.kpoints, M, A, ctl2, p.num_wann, extra={"gpu_tensor": tensor})
    assert out2["ierr"] == 0, out2["err"]
    om2, niter2 = float(out2["omega"][3]), int(out2["log"][-1][0])
    worst2, _ = _match_centres(out2["centres"].T, z["centres"], p.real_lattice)
    msg2 = "window 1e-12: Omega %.6e after %d iterations, centres %.3e A from the oracle's; %s" % (
        om2, niter2, worst2, msg)
    print(msg2)
    assert niter2 < 20000, "not converged: " + msg2
    assert abs(om2 - om_ref) <= 1e-8 * om0, "different minimum (Omega): " + msg2
    assert worst2 <= 1e-6, "different minimum (centres): " + msg2
    np.testing.assert_allclose(np.sort(out2["spreads"]), np.sort(z["spreads"]), rtol=0, atol=1e-6, err_msg=msg2)


def _stable_window(z, tag, rel_tol=1e-9, cen_tol=1e-7):
    base, pert = z["omega_log"][:, 3], z[tag + "omega_log"][:, 3]
    dcen = np.abs(z["centres_log"] - z[tag + "centres_log"]).max(axis=(1, 2))
    bad = np.nonzero((np.abs(pert - base) > rel_tol * np.abs(base)) | (dcen > cen_tol))[0]
    return int(bad[0]) if len(bad) else len(base)


@pytest.mark.parametrize("tensor", [1, 0], ids=["tensor", "fp64"])
def test_sc8_w128_stable_window(tensor):
    z = _load("sc8_w128_window.npz")
    p, M, A = _problem("sc8_w128")
    n = len(z["omega_log"]) - 1
    ctl = O.WannControl(num_iter=n, conv_tol=1e-10, conv_window=-1)
    out = run_engine(p.real_lattice, p.kpoints, M, A, ctl, p.num_wann, extra={"gpu_tensor": tensor})
    assert out["ierr"] == 0, out["err"]
    window = _stable_window(z, "p13_")
    assert window >= 20, window
    log = out["log"][: window + 1]
    ref = z["omega_log"][: window + 1]
    # Omega_total, Omega_D, Omega_OD (log columns 3, 4, 5) and Omega_I = total - D - OD (= 0)
    np.testing.assert_allclose(log[:, 3], ref[:, 3], rtol=1e-8, atol=0)
    np.testing.assert_array_less(np.abs(log[:, 3] - log[:, 4] - log[:, 5] - ref[:, 0]), 1e-8 * ref[:, 3])
    np.testing.assert_allclose(log[:, 4], ref[:, 1], rtol=1e-6, atol=2e-8 * ref[0, 3])
    np.testing.assert_allclose(log[:, 5], ref[:, 2], rtol=1e-8, atol=2e-8 * ref[0, 3])
    cen = out["log_centres"][: window + 1, :3, :].transpose(0, 2, 1)    # [iter][W][3]
    np.testing.assert_allclose(cen, z["centres_log"][: window + 1], rtol=0, atol=1e-6)
