"""The oracle against the reference's own regression outputs (parity pin of the oracle).

Inputs and expected values are the reference test suite's (test-suite/tests/testw90_example02,
_example01, _example05, _basic1, the preconditioned _precond_1 / _precond_2, the
selective-localisation _example26, the disentanglement cases and the guiding-centre
checkpoint), packed by tests/golden/make_fixtures.py.  Every printed
<-- CONV spread (10 decimals) must match to 2e-10 A^2 (RMS gradient to 1e-3 relative above a 1e-6 roundoff floor), final centres to 1e-6 A (printed to
6 decimals), spreads to 1e-7 A^2 and the b-vector / weight table to 1e-6.
"""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G


@pytest.mark.parametrize("name", G.CASES)
def test_oracle_reproduces_reference_trajectory(name):
    d = G.load(name)
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    # b-vectors and weights in the reference's order (benchmark table)
    tab = d["bvec_table"]
    assert km["nntot"] == len(tab)
    np.testing.assert_allclose(km["bk"][0], tab[:, :3], atol=1e-6)
    np.testing.assert_allclose(km["wb"], tab[:, 3], atol=1e-6)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"])
    r = O.wann_main(M0, U0, km, G.control(d), precond=G.precond_tables(d))
    rec = {0: r.initial}
    rec.update({it.iter: it for it in r.iters})
    for it, delta, rms, spread in d["conv"]:
        got = rec[int(it)]
        assert abs(got.spread.om_tot - spread) < 2e-10, (it, got.spread.om_tot, spread)
        # the gradient norm near the minimum is a small difference of O(1) terms whose
        # roundoff floor (different BLAS, summation order) is ~1e-6
        assert abs(got.rms_grad - rms) < 1e-6 + 1e-3 * rms
    fin = d["centres_final"]
    np.testing.assert_allclose(r.centres.T, fin[:, :3], atol=1.01e-6)
    np.testing.assert_allclose(r.spreads, fin[:, 3], atol=1.01e-8)
    om = d["omega_final"]
    got = [r.spread.om_i, r.spread.om_d, r.spread.om_od, r.spread.om_tot]
    np.testing.assert_allclose(got, om, atol=1.01e-9)


def test_oracle_guiding_centres_reach_reference_checkpoint():
    """testpostw90_gaas_shc (spinor GaAs, 16 isolated bands, guiding_centres = T,
    1000 iterations): the final centres and spreads of the shipped checkpoint."""
    d = G.load("gaas_guide")
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(d["knobs"]["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"])
    ctl, rguide = G.guiding(d)
    r = O.wann_main(M0, U0, km, ctl, rguide=rguide)
    fin = d["centres_final"]
    np.testing.assert_allclose(r.centres.T, fin[:, :3], atol=2e-6)
    np.testing.assert_allclose(r.spreads, fin[:, 3], atol=5e-6)
    assert abs(r.spread.om_tot - d["omega_final_total"][0]) < 1e-6


@pytest.mark.parametrize("name", G.DIS_CASES)
def test_oracle_disentanglement_reproduces_reference(name):
    """testw90_example03 (silicon) / _example04 (copper): 12 bands, 8 / 7 WFs;
    testw90_basic2: 8 -> 4 with lower window bounds; testw90_gaas_disentanglement_issue192:
    12 -> 8, mixing ratio 1.  Every printed '<-- DIS' line (Omega_I before and after the
    step, 8 decimals), the final Omega_I, and the wannierise trajectory that follows: each
    printed spread within 2e-10 A^2 where the trajectory is stable at that level, else within
    ten times the spread that a 1e-14 perturbation of M0 causes in the oracle itself (the
    GaAs case's middle iterations move by 1e-5 A^2 under it), and the final state."""
    d = G.load(name)
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U0, M0, Uo, omi, recs = O.dis_main(M, d["amn"], d["eig"], km, int(kn["num_wann"]), G.dis_control(d))
    assert len(recs) == len(d["dis"])
    for r, (it, prev, cur, delta) in zip(recs, d["dis"]):
        assert r.iter == int(it)
        assert abs(r.omega_i_prev - prev) < 1e-8 and abs(r.omega_i - cur) < 1e-8
    assert abs(omi - d["omega_i_final"][0]) < 1e-8
    r = O.wann_main(M0, U0, km, G.control(d))
    rec = {0: r.initial}
    rec.update({it.iter: it for it in r.iters})
    sens = G.conv_sensitivity(M0, U0, km, G.control(d))
    for it, delta, rms, spread in d["conv"]:
        tol = G.conv_tolerance(sens, it, spread)
        assert abs(rec[int(it)].spread.om_tot - spread) < tol, (int(it), rec[int(it)].spread.om_tot, spread, tol)
    np.testing.assert_allclose(r.centres.T, d["centres_final"][:, :3], atol=1.01e-6)
    np.testing.assert_allclose([r.spread.om_i, r.spread.om_tot], d["omega_final"][[0, 3]], atol=1.01e-9)


def test_oracle_selective_localisation_reproduces_reference():
    """testw90_example26 (GaAs, 4 WFs, 4x4x4 k, 100 iterations): selective localisation
    of WF 1 (slwf_num = 1) with its centre constrained (slwf_constrain = T,
    slwf_lambda = 1).  Every printed spread within 2e-10 A^2 where the trajectory is
    stable at that level, else within ten times the spread that a 1e-14 perturbation of
    M0 causes in the oracle itself; the RMS gradient likewise; the printed Omega_IOD
    (Omega_IOD + Omega_nu) and Omega_D of every '<-- SPRD' line; the final centres, spreads
    and the Omega IOD_C / D / Rest / Penalty / Total_C block (the non-objective WFs' parts
    to their roundoff sensitivity)."""
    d = G.load("slwf26")
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    tab = d["bvec_table"]
    np.testing.assert_allclose(km["bk"][0], tab[:, :3], atol=1e-6)
    np.testing.assert_allclose(km["wb"], tab[:, 3], atol=1e-6)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"])
    ctl, sl = G.slwf(d)
    r = O.wann_main(M0, U0, km, ctl, slwf=sl)
    sens, gsens = G.conv_sensitivity(M0, U0, km, ctl, runs=3, slwf=sl, grad=True)
    recs = [r.initial] + r.iters
    assert len(recs) == len(d["conv"]) == len(d["sprd"])
    for got, (it, delta, rms, spread), (iod, od, tot) in zip(recs, d["conv"], d["sprd"]):
        assert got.iter == int(it)
        tol = G.conv_tolerance(sens, it, spread, span=3)
        assert abs(got.spread.om_tot - spread) < tol, (it, got.spread.om_tot, spread, tol)
        assert abs(got.rms_grad - rms) < G.grad_tolerance(gsens, it, rms), (it, got.rms_grad, rms)
        # SPRD lines carry 7 decimals
        assert abs(got.spread.om_iod + got.spread.om_nu - iod) < 6e-8 + tol
        assert abs(got.spread.om_d - od) < 6e-8 + tol
    fin = d["centres_final"]
    s = sl.num
    # the objective WF is pinned; the others are outside the functional (their gauge is
    # free), so where the run stops them depends on roundoff: a 1e-14 perturbation of M0
    # moves their spreads and centres by up to 2e-6 in the oracle itself
    np.testing.assert_allclose(r.centres.T[:s], fin[:s, :3], rtol=0, atol=1.01e-6)
    np.testing.assert_allclose(r.spreads[:s], fin[:s, 3], rtol=0, atol=1.01e-8)
    np.testing.assert_allclose(r.centres.T[s:], fin[s:, :3], rtol=0, atol=2e-5)
    np.testing.assert_allclose(r.spreads[s:], fin[s:, 3], rtol=0, atol=2e-5)
    iod_c, om_d, rest, penalty, total_c = d["omega_final_slwf"]
    sp = r.spread
    assert abs(sp.om_iod + sp.om_nu - iod_c) < 1.01e-9
    assert abs(sp.om_d - om_d) < 1.01e-9
    assert abs(r.spreads.sum() + sp.om_tot - rest) < 6e-5
    rnr0n2 = ((r.centres[:, :sl.num] - sl.centres[:, :sl.num]) ** 2).sum()     # :829-836
    assert abs(rnr0n2 - penalty) < 1.01e-9
    assert abs(sp.om_tot - total_c) < 1.01e-9


def test_oracle_site_symmetry_reproduces_reference():
    """testw90_example21_As_sp (GaAs sp3, 4 WFs, 64 k of which 10 irreducible, 24
    symmetries, site_symmetry = T, symmetrize_eps = 1e-9): the symmetry-adapted initial
    U, the symmetrised gradient (sitesym_symmetrize_gradient modes 1 and 2) and the
    rotations of the reducible k from the irreducible ones.  Every printed spread within
    2e-10 A^2, the final centres/spreads and Omega terms to the printed decimals; the
    run differs from the plain one from its initial state on."""
    d = G.load("sitesym21")
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    tab = d["bvec_table"]
    np.testing.assert_allclose(km["bk"][0], tab[:, :3], atol=1e-6)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    sym = G.sitesym(d)
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"], sitesym=sym)
    r = O.wann_main(M0, U0, km, G.control(d), sitesym=sym)
    recs = [r.initial] + r.iters
    assert len(recs) == len(d["conv"])
    for got, (it, delta, rms, spread) in zip(recs, d["conv"]):
        assert got.iter == int(it)
        assert abs(got.spread.om_tot - spread) < 2e-10, (it, got.spread.om_tot, spread)
        assert abs(got.rms_grad - rms) < 1e-6 + 1e-3 * rms
    fin = d["centres_final"]
    np.testing.assert_allclose(r.centres.T, fin[:, :3], rtol=0, atol=1.01e-6)
    np.testing.assert_allclose(r.spreads, fin[:, 3], rtol=0, atol=1.01e-8)
    sp = r.spread
    np.testing.assert_allclose([sp.om_i, sp.om_d, sp.om_od, sp.om_tot], d["omega_final"], rtol=0, atol=1.01e-9)
    # the symmetry-adapted mode is what reproduces the printed run
    U0p, M0p = O.overlap_project(M, d["amn"], km["nnlist"])
    plain = O.wann_main(M0p, U0p, km, O.WannControl(**{**G.control(d).__dict__, "num_iter": 3}))
    assert abs(plain.iters[2].spread.om_tot - d["conv"][3][3]) > 1e-6


def test_oracle_symmetry_adapted_disentanglement_reproduces_reference():
    """testw90_disentanglement_sawfs (H3S, 20 bands -> 12 WFs, 8 k of which 3
    irreducible, 48 symmetries, outer window only, site_symmetry = T): the symmetry-adapted
    U_opt, the symmetrised Z matrices, the constrained extraction at the irreducible k
    (sitesym_dis_extract_symmetry), the symmetric initial U, then the symmetric
    wannierisation.  Every '<-- DIS' line (8 decimals) within 1e-8, the printed
    '<-- CONV' spreads within 2e-10 A^2, the final Omega terms and centres."""
    d = G.load("sitesym_dis")
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    np.testing.assert_allclose(km["wb"], d["bvec_table"][:, 3], atol=1e-6)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    sym = G.sitesym(d)
    U0, M0, Uo, omi, recs = O.dis_main(M, d["amn"], d["eig"], km, int(kn["num_wann"]), G.dis_control(d),
                                       sitesym=sym)
    assert len(recs) == len(d["dis"])
    for r, (it, prev, cur, delta) in zip(recs, d["dis"]):
        assert r.iter == int(it)
        assert abs(r.omega_i_prev - prev) < 1e-8 and abs(r.omega_i - cur) < 1e-8, (r.iter, r, prev, cur)
    assert abs(omi - d["omega_i_final"][0]) < 1e-8
    r = O.wann_main(M0, U0, km, G.control(d), sitesym=sym)
    rec = {0: r.initial}
    rec.update({x.iter: x for x in r.iters})
    for it, delta, rms, spread in d["conv"]:
        assert abs(rec[int(it)].spread.om_tot - spread) < 2e-10, (int(it), rec[int(it)].spread.om_tot, spread)
    sp = r.spread
    np.testing.assert_allclose([sp.om_i, sp.om_d, sp.om_od, sp.om_tot], d["omega_final"], rtol=0, atol=1.01e-9)
    np.testing.assert_allclose(r.centres.T, d["centres_final"][:, :3], rtol=0, atol=1.01e-6)


def test_oracle_restart_from_checkpoint_reproduces_reference():
    """testw90_example02_restart (lead, restart = wannierise): wann_main continued from the
    U and M of the checkpoint the test ships; every printed spread within 2e-10 A^2, the
    final Omega terms and centres."""
    d = G.load("restart02")
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(d["knobs"]["search_shells"]))
    np.testing.assert_allclose(km["wb"], d["bvec_table"][:, 3], atol=1e-6)
    r = O.wann_main(d["m"], d["u"], km, G.control(d))
    recs = [r.initial] + r.iters
    assert len(recs) == len(d["conv"])
    for got, (it, delta, rms, spread) in zip(recs, d["conv"]):
        assert got.iter == int(it) and abs(got.spread.om_tot - spread) < 2e-10
    sp = r.spread
    np.testing.assert_allclose([sp.om_i, sp.om_d, sp.om_od, sp.om_tot], d["omega_final"], rtol=0, atol=1.01e-9)
    np.testing.assert_allclose(r.centres.T, d["centres_final"][:, :3], rtol=0, atol=1.01e-6)
