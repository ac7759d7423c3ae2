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
  engine to the same minimum: Omega within 1e-8 relative or five times the oracle's
  run-to-run difference of the stopping value (whichever is larger), every centre within
  1e-6 A of an oracle centre (matched as sets, modulo lattice vectors), the spreads within
  1e-6 A^2; the iteration count is reported, not compared.
* sc 8x8x8 (512 k), nntot 6, num_wann 128, gauge noise 0.5: every iteration's Omega parts
  and centres against the oracle's (tests/golden/sc8_w128_window.npz) over the stable
  window -- the iterations over which the oracle agrees with itself to a tenth of the
  test's bounds (1e-9 relative, 1e-7 A) when M0 is perturbed by 1e-15 (FP64 path: 26
  iterations) or 1e-13 (tensor path, whose M update is exact to 2^-49 of the scales: 22
  iterations).  Beyond it the oracle's own runs part (1e-5 relative by iteration 33, 3e-2
  by 36, three different Omega after 40 iterations), so no implementation can be held to
  them there.
"""
import os

import numpy as np
import pytest

from oracle import w90_oracle as O
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
    inv = np.linalg.inv(lattice)
    d = np.zeros((len(a), len(b)))
    for i in range(len(a)):
        f = (b - a[i]) @ inv
        f -= np.round(f)
        d[i] = np.linalg.norm(f @ lattice, axis=1)
    used_a, used_b, worst = set(), set(), 0.0
    for flat in np.argsort(d, axis=None):
        i, j = divmod(int(flat), len(b))
        if i in used_a or j in used_b:
            continue
        used_a.add(i)
        used_b.add(j)
        worst = max(worst, d[i, j])
    return worst, d


@pytest.mark.parametrize("tensor", [1, 0], ids=["tensor", "fp64"])
def test_fcc10_w32_converges_to_the_oracle_minimum(tensor):
    z = _load("fcc10_w32_conv.npz")
    p, M, A = _problem("fcc10_w32")
    ctl = O.WannControl(num_iter=20000, conv_tol=1e-10, conv_window=5)
    out = run_engine(p.real_lattice, p.kpoints, M, A, ctl, p.num_wann, extra={"gpu_tensor": tensor})
    assert out["ierr"] == 0, out["err"]
    om_ref, om_p15 = z["omega"][3], z["p15_omega"][3]
    om = out["omega"][3]
    niter = int(out["log"][-1][0])
    worst, _ = _match_centres(out["centres"], z["centres"], p.real_lattice)
    msg = ("engine (%s) Omega %.6e after %d iterations; oracle %.6e after %d; oracle from M0 + 1e-15 "
           "noise %.6e after %d; largest centre distance to the oracle's %.3e A"
           % ("tensor" if tensor else "fp64", om, niter, om_ref, int(z["niter"]), om_p15, int(z["p15_niter"]),
              worst))
    print(msg)
    assert bool(z["converged"]) and bool(z["p15_converged"])
    assert int(out["log"][-1][0]) < 20000, "not converged: " + msg
    tol = max(1e-8 * abs(om_ref), 5.0 * abs(om_ref - om_p15))
    assert abs(om - om_ref) <= tol, "different minimum (Omega): " + msg
    assert worst <= 1e-6, "different minimum (centres): " + msg
    np.testing.assert_allclose(np.sort(out["spreads"]), np.sort(z["spreads"]), rtol=0, atol=1e-6, err_msg=msg)


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
    window = _stable_window(z, "p13_" if tensor else "p15_")
    assert window >= 20, window
    log = out["log"][: window + 1]
    ref = z["omega_log"][: window + 1]
    # Omega_total, Omega_D, Omega_OD (log columns 3, 4, 5) and Omega_I = total - D - OD
    np.testing.assert_allclose(log[:, 3], ref[:, 3], rtol=1e-8, atol=0)
    np.testing.assert_allclose(log[:, 3] - log[:, 4] - log[:, 5], ref[:, 0], rtol=1e-8, atol=0)
    np.testing.assert_allclose(log[:, 4], ref[:, 1], rtol=1e-6, atol=2e-8 * ref[0, 3])
    np.testing.assert_allclose(log[:, 5], ref[:, 2], rtol=1e-8, atol=2e-8 * ref[0, 3])
    cen = out["log_centres"][: window + 1, :3, :].transpose(0, 2, 1)    # [iter][W][3]
    np.testing.assert_allclose(cen, z["centres_log"][: window + 1], rtol=0, atol=1e-6)
