"""Parity of the GPU disentanglement (cdisentangle: dis_main + setup_m_loc) with the
oracle and with the reference's own outputs, through the C ABI.

Quantities compared are the ones that do not depend on the gauge freedom of the
eigen-solvers: the Omega_I record of every iteration, the final Omega_I, the rotated
overlaps M0 = U^H U_opt^H M U_opt' U' (U = polar(U_opt^H A) absorbs any unitary mixing
of U_opt's columns, so M0 and U_opt U depend only on the optimal subspace), and U_opt U.
Tolerances: Omega_I 1e-10 relative against the oracle and 1e-8 absolute against the
reference's printed 8 decimals; M0 and U_opt U 1e-9 absolute (the eigenvalue gaps at the
selection cut are 1e-2 or larger, so eigenvector roundoff stays at 1e-13).
"""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G
from tests.engine_dis import entangled_windows, run_dis
from wannier90_gb300 import synth

pytestmark = pytest.mark.gpu


def _check_dis(out, recs, omi, U0, M0, Uo, rel=1e-10):
    assert out["ierr"] == 0, out["err"]
    log = out["dis_log"]
    assert len(log) == len(recs), (len(log), len(recs))
    for row, r in zip(log, recs):
        assert int(row[0]) == r.iter
        assert abs(row[1] - r.omega_i_prev) <= rel * abs(r.omega_i_prev), (r.iter, row[1], r.omega_i_prev)
        assert abs(row[2] - r.omega_i) <= rel * abs(r.omega_i), (r.iter, row[2], r.omega_i)
    assert abs(out["dis_info"]["omega_invariant"] - omi) <= rel * abs(omi)
    np.testing.assert_allclose(out["M0"], M0, atol=1e-9)
    np.testing.assert_allclose(out["Uopt"] @ out["U0"], Uo @ U0, atol=1e-9)
    # U is unitary and U_opt has orthonormal columns
    W = U0.shape[1]
    for k in range(len(U0)):
        np.testing.assert_allclose(out["U0"][k].conj().T @ out["U0"][k], np.eye(W), atol=1e-12)
        np.testing.assert_allclose(out["Uopt"][k].conj().T @ out["Uopt"][k], np.eye(W), atol=1e-12)


@pytest.mark.parametrize("tensor", [0, 1], ids=["fp64", "tensor"])
@pytest.mark.parametrize("name", G.DIS_CASES)
def test_disentangle_golden(name, tensor):
    """testw90_example03 (silicon, 12 bands -> 8 WFs), _example04 (copper, 12 -> 7),
    testw90_basic2 (8 -> 4, lower window bounds), testw90_gaas_disentanglement_issue192
    (12 -> 8, mixing ratio 1): every '<-- DIS' line, the final Omega_I, then wann_main on
    the disentangled overlaps against the printed '<-- CONV' lines and final centres."""
    d = G.load(name)
    kn = d["knobs"]
    ss = int(kn["search_shells"])
    W = int(kn["num_wann"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], ss)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    dc = G.dis_control(d)
    ctl = G.control(d)
    out = run_dis(d["real_lattice"], d["kpt_latt"], M, d["amn"], d["eig"], W, dc, ss, wann_ctl=ctl,
                  extra={"gpu_tensor": tensor})
    U0, M0, Uo, omi, recs = O.dis_main(M, d["amn"], d["eig"], km, W, dc)
    _check_dis(out, recs, omi, U0, M0, Uo)
    # the reference's printed DIS lines (8 decimals) and final Omega_I
    for row, (it, prev, cur, delta) in zip(out["dis_log"], d["dis"]):
        assert int(row[0]) == int(it)
        assert abs(row[1] - prev) < 1e-8 and abs(row[2] - cur) < 1e-8
    assert abs(out["dis_info"]["omega_invariant"] - d["omega_i_final"][0]) < 1e-8
    # wann_main on the top-left num_wann x num_wann blocks of m_local: each printed spread
    # within 2e-10 A^2 where the trajectory is stable at that level, else within ten times
    # the oracle's own sensitivity to a 1e-14 perturbation of M0 (the GaAs case's middle
    # iterations move by 1e-5 A^2 under it).  The tensor path rounds every product at
    # ~2^-49 of its scales on every iteration, a perturbation renewed at each step: 2e-9,
    # and twenty times the largest change over four 1e-13 perturbations.  The final centres:
    # the printed 6 decimals plus three times the oracle's own spread of them over runs
    # perturbed as the path rounds (the tensor path: 1e-13 at every M update; the GaAs
    # case's centres move by up to 4e-7 A under it)
    assert out["wann_ierr"] == 0, out["wann_err"]
    by_iter = {int(row[0]): row for row in out["log"]}
    sens = G.conv_sensitivity(M0, U0, km, ctl, noise=1e-13 if tensor else 1e-14, runs=4 if tensor else 2)
    for it, delta, rms, spread in d["conv"]:
        tol = G.conv_tolerance(sens, it, spread, floor=2e-9 if tensor else 2e-10, factor=20.0 if tensor else 10.0)
        assert abs(by_iter[int(it)][3] - spread) < tol, (int(it), by_iter[int(it)][3], spread, tol)
    _, csens = G.conv_sensitivity(M0, U0, km, ctl, noise=1e-13 if tensor else 1e-14, runs=4 if tensor else 2,
                                  centres=True, per_update=bool(tensor))
    ctol = 1.01e-6 + 3.0 * csens
    assert np.all(np.abs(out["centres"].T - d["centres_final"][:, :3]) <= ctol[:, None]), \
        (out["centres"].T, d["centres_final"][:, :3], ctol)
    np.testing.assert_allclose(out["omega"][[0, 3]], d["omega_final"][[0, 3]], atol=1.01e-9)
    # wann_main wrote only the top-left blocks: the rest of m_local is the raw overlaps
    nb = M.shape[2]
    mask = np.ones((nb, nb), dtype=bool)
    mask[:W, :W] = False
    np.testing.assert_array_equal(out["m_after_wann"][:, :, mask], M[:, :, mask])
    r = O.wann_main(M0, U0, km, ctl)
    assert np.all(np.abs(out["centres"] - np.asarray(r.centres)) <= 1e-6 + 3.0 * csens[None, :])


@pytest.mark.parametrize("case", [
    dict(kind="sc", mp=(4, 4, 4), num_bands=12, num_wann=8, frozen=True, seed=1),
    dict(kind="fcc", mp=(4, 4, 4), num_bands=20, num_wann=16, frozen=False, seed=2),
    dict(kind="bcc", mp=(3, 3, 3), num_bands=40, num_wann=24, frozen=True, seed=3),
    dict(kind="sc", mp=(2, 2, 3), num_bands=64, num_wann=40, frozen=True, seed=4),
], ids=["sc4_12to8_frozen", "fcc4_20to16_outer", "bcc3_40to24_frozen", "sc_64to40_frozen"])
def test_disentangle_synthetic(case):
    """Seeded entangled tight-binding problems: windows that cut bands off at the bottom
    at some k-points (nfirstwin > 0), a varying number of window and frozen states per k,
    and the largest band count the engine takes (64)."""
    c = dict(case)
    frozen = c.pop("frozen")
    p = synth.make_entangled_problem(a=5.0, rmax=2, eps=0.3, **c)
    eig = np.ascontiguousarray(p.eig.T)
    W = p.num_wann
    w = entangled_windows(eig, W)
    dc = O.DisControl(num_iter=200, mix_ratio=0.5, conv_tol=1e-10, conv_window=3,
                      win_min=w["win_min"], win_max=w["win_max"])
    if frozen:
        dc.froz_max = w["froz_max"]
        dc.frozen_states = True
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    km = O.kmesh_get(p.real_lattice, p.kpoints, 36)
    out = run_dis(p.real_lattice, p.kpoints, M, A, eig, W, dc)
    U0, M0, Uo, omi, recs = O.dis_main(M, A, eig, km, W, dc)
    _check_dis(out, recs, omi, U0, M0, Uo)
    win = O.dis_windows(eig, W, dc)
    assert (win["nfirstwin"] > 0).any() and (win["nfirstwin"] == 0).any()
    if frozen:
        assert (win["ndimfroz"] > 0).any()


def test_disentangle_mix_and_window_options():
    """dis_mix_ratio < 1 with a short dis_conv_window (converges at a clean crossing of
    the tolerance: delta falls by 2% per iteration there), and dis_num_iter reached before
    convergence (the record stops at dis_num_iter, converged = False).  Windows are set:
    with every band kept the orbital subspace of the model gives Omega_I = 0 and delta is
    roundoff over roundoff."""
    p = synth.make_entangled_problem(kind="sc", mp=(3, 3, 3), num_bands=14, num_wann=9, seed=7)
    eig = np.ascontiguousarray(p.eig.T)
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    km = O.kmesh_get(p.real_lattice, p.kpoints, 36)
    w = entangled_windows(eig, p.num_wann)
    win = dict(win_min=w["win_min"], win_max=w["win_max"])
    for dc in (O.DisControl(num_iter=400, mix_ratio=0.3, conv_tol=1e-5, conv_window=2, **win),
               O.DisControl(num_iter=4, mix_ratio=0.7, conv_tol=1e-14, conv_window=3, **win)):
        out = run_dis(p.real_lattice, p.kpoints, M, A, eig, p.num_wann, dc)
        U0, M0, Uo, omi, recs = O.dis_main(M, A, eig, km, p.num_wann, dc)
        _check_dis(out, recs, omi, U0, M0, Uo)
        assert out["dis_info"]["iterations"] == len(recs)
        tail = recs[-dc.conv_window:]
        conv = len(recs) >= dc.conv_window and all(abs(r.delta) < dc.conv_tol for r in tail)
        assert out["dis_info"]["converged"] == conv


def test_project_overlap_after_disentangle_is_noop():
    """w90_project_overlap does nothing once disentanglement ran
    (src/library_interface.F90:449-459)."""
    from wannier90_gb300 import library as w90
    p = synth.make_entangled_problem(kind="sc", mp=(2, 2, 2), num_bands=10, num_wann=6, seed=9)
    eig = np.ascontiguousarray(p.eig.T)
    out = run_dis(p.real_lattice, p.kpoints, synth.to_math_m(p.m), synth.to_math_u(p.a), eig, p.num_wann,
                  O.DisControl())
    assert out["ierr"] == 0, out["err"]
    c = out["handle"]
    u_before = np.array(c._keep["u"], copy=True)
    m_before = np.array(c._keep["m"], copy=True)
    assert w90.w90_project_overlap(c) == 0
    np.testing.assert_array_equal(c._keep["u"], u_before)
    np.testing.assert_array_equal(c._keep["m"], m_before)


def test_device_entry_equals_host_entry():
    """w90g_disentangle_device + w90g_wannierise_device on device buffers give the host
    path's results bit for bit (same kernels, same order), and the profiled form too."""
    import torch

    from wannier90_gb300 import library as w90
    p = synth.make_entangled_problem(kind="fcc", mp=(3, 3, 3), num_bands=16, num_wann=10, seed=11)
    eig = np.ascontiguousarray(p.eig.T)
    w = entangled_windows(eig, p.num_wann)
    dc = O.DisControl(num_iter=80, win_min=w["win_min"], win_max=w["win_max"], froz_max=w["froz_max"],
                      frozen_states=True)
    ctl = O.WannControl(num_iter=40, conv_window=-1)
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    host = run_dis(p.real_lattice, p.kpoints, M, A, eig, p.num_wann, dc, wann_ctl=ctl)
    assert host["ierr"] == 0 and host["wann_ierr"] == 0
    from tests.engine_dis import dis_options
    for profiled in (False, True):
        c = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=p.num_wann, num_bands=p.num_bands,
                      iprint=0, num_iter=40, conv_window=-1, **dis_options(dc))
        dm = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
        da = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
        du = torch.zeros(2 * p.num_wann ** 2 * len(p.kpoints), dtype=torch.float64, device="cuda")
        de = torch.from_numpy(np.ascontiguousarray(p.eig.reshape(-1, order="F"))).cuda()
        if profiled:
            ierr, prof = w90.w90_profile_dis_device(c, dm.data_ptr(), da.data_ptr(), du.data_ptr(), de.data_ptr())
            assert prof["k_dis_step"][1] == len(host["dis_log"]) and prof["k_dis_rotate"][1] == 1
            assert all(ms >= 0.0 for ms, _ in prof.values())
        else:
            ierr = w90.w90_disentangle_device(c, dm.data_ptr(), da.data_ptr(), du.data_ptr(), de.data_ptr())
        assert ierr == 0, c.last_error()
        np.testing.assert_array_equal(w90.w90_get_dis_log(c, 100)[:, :4], host["dis_log"][:, :4])
        u = du.cpu().numpy().view(np.complex128).reshape((p.num_wann, p.num_wann, -1), order="F")
        np.testing.assert_array_equal(synth.to_math_u(u), host["U0"])
        assert w90.w90_wannierise_device(c, dm.data_ptr(), du.data_ptr()) == 0, c.last_error()
        m = dm.cpu().numpy().view(np.complex128).reshape(p.m.shape, order="F")
        np.testing.assert_array_equal(synth.to_math_m(m), host["m_after_wann"])
        np.testing.assert_array_equal(w90.w90_get_centres(c, p.num_wann), host["centres"])
        assert w90.w90_kernel_launches(c) > 0


def test_entangled_problems_in_batched_and_served_forms():
    """After w90g_disentangle_device, the (nb x nb)-block overlaps go through the batched
    and the served forms like isolated ones (top-left num_wann blocks): each member's
    result is bitwise the stand-alone w90g_wannierise_device result."""
    import torch

    from tests.engine_dis import dis_options
    from wannier90_gb300 import library as w90
    cases = [dict(kind="sc", mp=(3, 3, 3), num_bands=12, num_wann=8, seed=21, tensor=1),
             dict(kind="fcc", mp=(3, 3, 3), num_bands=16, num_wann=10, seed=22, tensor=0),
             dict(kind="sc", mp=(2, 2, 3), num_bands=20, num_wann=13, seed=23, tensor=1)]
    handles, ms, us, alone = [], [], [], []
    for c in cases:
        c = dict(c)
        tensor = c.pop("tensor")
        p = synth.make_entangled_problem(eps=0.3, **c)
        eig = np.ascontiguousarray(p.eig.T)
        w = entangled_windows(eig, p.num_wann)
        dc = O.DisControl(num_iter=40, win_min=w["win_min"], win_max=w["win_max"], froz_max=w["froz_max"],
                          frozen_states=True)
        h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=p.num_wann,
                      num_bands=p.num_bands, iprint=0, num_iter=12, conv_window=-1, gpu_tensor=tensor,
                      **dis_options(dc))
        dm = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
        da = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
        du = torch.zeros(2 * p.num_wann ** 2 * len(p.kpoints), dtype=torch.float64, device="cuda")
        de = torch.from_numpy(np.ascontiguousarray(p.eig.reshape(-1, order="F"))).cuda()
        assert w90.w90_disentangle_device(h, dm.data_ptr(), da.data_ptr(), du.data_ptr(), de.data_ptr()) == 0
        m1, u1 = dm.clone(), du.clone()
        assert w90.w90_wannierise_device(h, m1.data_ptr(), u1.data_ptr()) == 0, h.last_error()
        torch.cuda.synchronize()
        alone.append((m1.cpu().numpy(), u1.cpu().numpy(), w90.w90_get_log(h, 13).copy()))
        handles.append(h)
        ms.append(dm)
        us.append(du)
    # batched
    mb = [m.clone() for m in ms]
    ub = [u.clone() for u in us]
    ierr = w90.w90_wannierise_batch_device(handles, [m.data_ptr() for m in mb], [u.data_ptr() for u in ub])
    torch.cuda.synchronize()
    assert ierr == [0] * len(cases), [h.last_error() for h in handles]
    for i, h in enumerate(handles):
        np.testing.assert_array_equal(w90.w90_get_log(h, 13)[:, :8], alone[i][2][:, :8])
        np.testing.assert_array_equal(mb[i].cpu().numpy(), alone[i][0])
        np.testing.assert_array_equal(ub[i].cpu().numpy(), alone[i][1])
    # served
    srv = w90.Server(8e9, max_active=2)
    ms2 = [m.clone() for m in ms]
    us2 = [u.clone() for u in us]
    for i, h in enumerate(handles):
        assert srv.submit(h, ms2[i].data_ptr(), us2[i].data_ptr(), tag=i) == 0, h.last_error()
    srv.drain()
    done = srv.poll()
    assert sorted(d[0] for d in done) == list(range(len(cases))) and all(d[1] == 0 for d in done)
    torch.cuda.synchronize()
    for i in range(len(cases)):
        np.testing.assert_array_equal(ms2[i].cpu().numpy(), alone[i][0])
        np.testing.assert_array_equal(us2[i].cpu().numpy(), alone[i][1])
    srv.close()
