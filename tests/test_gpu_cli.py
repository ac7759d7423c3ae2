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


@pytest.mark.parametrize("name", ["silicon_dis"])
def test_cli_entangled_seed_files(tmp_path, name):
    """Entangled bands through the file flow: .win (dis_* keywords) / .mmn / .amn / .eig ->
    cdisentangle + cwannierise -> a disentangled .chk; against the reference's printed
    final Omega_I and centres."""
    from tests import golden_cases as G
    d = G.load(name)
    kn = d["knobs"]
    ss = int(kn["search_shells"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], ss)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    dc = G.dis_control(d)
    ctl = G.control(d)
    nb, nw, K = int(d["num_bands"]), int(kn["num_wann"]), len(d["kpt_latt"])
    seed = str(tmp_path / name)
    kw = dict(num_iter=ctl.num_iter, conv_tol=ctl.conv_tol, trial_step=ctl.trial_step, search_shells=ss,
              iprint=0, dis_num_iter=dc.num_iter, dis_mix_ratio=dc.mix_ratio, dis_conv_tol=dc.conv_tol,
              dis_conv_window=dc.conv_window, dis_win_max=dc.win_max, dis_froz_max=dc.froz_max)
    w90io.write_win(seed + ".win", d["real_lattice"], d["kpt_latt"], d["mp_grid"], nw, num_bands=nb, **kw)
    w90io.write_mmn(seed + ".mmn", synth.from_math_m(M), km["nnlist"], km["nncell"])
    w90io.write_amn(seed + ".amn", synth.from_math_u(d["amn"]))
    w90io.write_eig(seed + ".eig", np.asfortranarray(d["eig"].T))
    assert cli.run(seed, "fp64") == 0
    chk = w90io.read_chk(seed + ".chk")
    assert chk["have_disentangled"] and chk["num_bands"] == nb and chk["num_wann"] == nw
    assert abs(chk["omega_invariant"] - d["omega_i_final"][0]) < 1e-8
    win = O.dis_windows(d["eig"], nw, dc)
    np.testing.assert_array_equal(chk["ndimwin"], win["ndimwin"])
    for k in range(K):
        f, n = win["nfirstwin"][k], win["ndimwin"][k]
        assert chk["lwindow"][f:f + n, k].all() and chk["lwindow"][:, k].sum() == n
    np.testing.assert_allclose(chk["centres"].T, d["centres_final"][:, :3], atol=1.01e-6)
    uo = synth.to_math_u(chk["u_opt"])
    for k in range(K):
        np.testing.assert_allclose(uo[k].conj().T @ uo[k], np.eye(nw), atol=1e-12)


def test_cli_restart_wannierise(tmp_path, capfd):
    """testw90_example02_restart: restart = wannierise continues wann_main from the
    checkpoint (here the shipped one's U and M written as a .chk) -- no .mmn / .amn are
    read; every printed spread within 2e-10 A^2 of the reference's."""
    from tests import golden_cases as G
    d = G.load("restart02")
    kn = d["knobs"]
    seed = str(tmp_path / "lead")
    w90io.write_win(seed + ".win", d["real_lattice"], d["kpt_latt"], d["mp_grid"], int(kn["num_wann"]),
                    num_iter=int(kn["num_iter"]), search_shells=int(kn["search_shells"]), iprint=1,
                    restart="wannierise")
    W, K = int(kn["num_wann"]), len(d["kpt_latt"])
    w90io.write_chk(seed + ".chk", num_bands=W, lattice=d["real_lattice"], kpts=d["kpt_latt"], mp_grid=d["mp_grid"],
                    nntot=int(d["nntot"]), num_wann=W, u=np.asfortranarray(d["u"].transpose(1, 2, 0)),
                    m=np.asfortranarray(d["m"].transpose(2, 3, 1, 0)), centres=np.zeros((3, W)), spreads=np.zeros(W))
    capfd.readouterr()
    assert cli.run(seed, "fp64") == 0
    text = capfd.readouterr().out.splitlines()
    conv = {int(l.split()[0]): float(l.split()[3]) for l in text
            if l.rstrip().endswith("<-- CONV") and not l.strip().startswith(("+", "|"))}
    for it, delta, rms, spread in d["conv"]:
        assert abs(conv[int(it)] - spread) < 2e-10, int(it)
    chk = w90io.read_chk(seed + ".chk")
    np.testing.assert_allclose(chk["centres"].T, d["centres_final"][:, :3], atol=1.01e-6)


def test_cli_restart_after_disentanglement(tmp_path):
    """An entangled run checkpoints the disentangled subspace; restart = wannierise from
    that checkpoint continues wann_main on its num_wann x num_wann overlaps and keeps
    U_opt, the windows and Omega_I.  Run 0 wannierisation iterations after the
    disentanglement, then restart for the full count: the same trajectory as the one-shot
    run (the controller starts from the same state), so the same final centres."""
    from tests import golden_cases as G
    d = G.load("silicon_dis")
    kn = d["knobs"]
    ss = int(kn["search_shells"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], ss)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    dc = G.dis_control(d)
    ctl = G.control(d)
    nb, nw = int(d["num_bands"]), int(kn["num_wann"])

    def files(seed, num_iter, **extra):
        kw = dict(num_iter=num_iter, conv_tol=ctl.conv_tol, trial_step=ctl.trial_step, search_shells=ss,
                  iprint=0, dis_num_iter=dc.num_iter, dis_mix_ratio=dc.mix_ratio, dis_conv_tol=dc.conv_tol,
                  dis_conv_window=dc.conv_window, dis_win_max=dc.win_max, dis_froz_max=dc.froz_max, **extra)
        w90io.write_win(seed + ".win", d["real_lattice"], d["kpt_latt"], d["mp_grid"], nw, num_bands=nb, **kw)

    one = str(tmp_path / "one")
    files(one, ctl.num_iter)
    w90io.write_mmn(one + ".mmn", synth.from_math_m(M), km["nnlist"], km["nncell"])
    w90io.write_amn(one + ".amn", synth.from_math_u(d["amn"]))
    w90io.write_eig(one + ".eig", np.asfortranarray(d["eig"].T))
    assert cli.run(one, "fp64") == 0
    ref = w90io.read_chk(one + ".chk")
    two = str(tmp_path / "two")
    files(two, 0)
    for ext in (".mmn", ".amn", ".eig"):
        with open(one + ext) as a, open(two + ext, "w") as b:
            b.write(a.read())
    assert cli.run(two, "fp64") == 0
    mid = w90io.read_chk(two + ".chk")
    assert mid["have_disentangled"]
    files(two, ctl.num_iter, restart="wannierise")
    assert cli.run(two, "fp64") == 0
    end = w90io.read_chk(two + ".chk")
    assert end["have_disentangled"] and end["num_bands"] == nb
    assert end["omega_invariant"] == ref["omega_invariant"]
    np.testing.assert_array_equal(end["ndimwin"], ref["ndimwin"])
    np.testing.assert_array_equal(end["lwindow"], ref["lwindow"])
    np.testing.assert_array_equal(end["u_opt"], ref["u_opt"])
    np.testing.assert_allclose(end["centres"], ref["centres"], atol=1e-8)
    np.testing.assert_allclose(end["spreads"], ref["spreads"], atol=1e-8)
