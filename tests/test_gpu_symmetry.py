"""Symmetry-adapted mode (site_symmetry = T) on the GPU engine, through the C ABI, against
the oracle and the reference's testw90_example21_As_sp (GaAs sp3, 64 k of which 10
irreducible, 24 symmetries).  The oracle reproduces that run's printed spreads to
5e-11 A^2 and the trajectory is stable at that level, so the engine is held to 2e-10
A^2 on every printed line (the tensor path to 2e-9), to the oracle's symmetry-adapted
initial U and M to 1e-10, and to the printed final state."""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G
from wannier90_gb300 import library as w90
from wannier90_gb300 import synth

pytestmark = pytest.mark.gpu


def _run(d, tensor, project_only=False):
    kn = d["knobs"]
    ss = int(kn["search_shells"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], ss)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    A = np.ascontiguousarray(d["amn"])
    ctl = G.control(d)
    c = w90.setup(kpoints=d["kpt_latt"], unit_cell_cart=d["real_lattice"], num_wann=4, num_iter=ctl.num_iter,
                  search_shells=ss, iprint=0, gpu_tensor=tensor, site_symmetry=True,
                  symmetrize_eps=float(kn["symmetrize_eps"]))
    assert w90.w90_set_sitesym(c, G.dmn_dict(d)) == 0, c.last_error()
    m = np.array(synth.from_math_m(M), order="F", copy=True)
    u = np.array(synth.from_math_u(A), order="F", copy=True)
    w90.w90_set_m_local(c, m)
    w90.w90_set_u_matrix(c, u)
    w90.w90_set_u_opt(c, np.asfortranarray(np.broadcast_to(np.eye(4, dtype=np.complex128)[:, :, None],
                                                           (4, 4, len(d["kpt_latt"]))).copy()))
    w90.check(c, w90.w90_project_overlap(c), "project_overlap")
    out = dict(U0=synth.to_math_u(u).copy(), M0=synth.to_math_m(m).copy(), km=km, M=M, A=A, ctl=ctl)
    if project_only:
        return out
    out["ierr"] = w90.w90_wannierise(c)
    out["err"] = c.last_error()
    out["log"] = w90.w90_get_log(c, ctl.num_iter + 1)
    out["centres"] = w90.w90_get_centres(c, 4)
    out["spreads"] = w90.w90_get_spreads(c, 4)
    out["omega"] = w90.w90_get_omega(c)
    out["U"] = synth.to_math_u(u)
    return out


def test_symmetry_adapted_projection():
    """cproject_overlap with site_symmetry: the Loewdin U made symmetry-adapted
    (symmetrize_ukirr at the irreducible k, d U D^+ over the stars) and M rotated by it."""
    d = G.load("sitesym21")
    out = _run(d, 0, project_only=True)
    sym = G.sitesym(d)
    U0, M0 = O.overlap_project(out["M"], out["A"], out["km"]["nnlist"], sitesym=sym)
    np.testing.assert_allclose(out["U0"], U0, atol=1e-10)
    np.testing.assert_allclose(out["M0"], M0, atol=1e-10)
    # the symmetry condition itself: U(R k) = d U(k) D^+ on every star
    for ir in range(sym.nkirr):
        ik = sym.ir2ik[ir]
        for isym in range(sym.nsym):
            k2 = sym.kptsym[isym, ir]
            want = sym.d_band[ir, isym] @ out["U0"][ik] @ sym.d_wann[ir, isym].conj().T
            if isym == 0 or k2 == ik:
                continue
            np.testing.assert_allclose(out["U0"][k2], want, atol=1e-9)


@pytest.mark.parametrize("tensor", [0, 1], ids=["fp64", "tensor"])
def test_symmetry_adapted_golden_example21(tensor):
    d = G.load("sitesym21")
    out = _run(d, tensor)
    assert out["ierr"] == 0, out["err"]
    sym = G.sitesym(d)
    U0, M0 = O.overlap_project(out["M"], out["A"], out["km"]["nnlist"], sitesym=sym)
    r = O.wann_main(M0, U0, out["km"], out["ctl"], sitesym=sym)
    log = out["log"]
    assert len(log) == len(d["conv"]) == len(r.iters) + 1
    tol = 2e-9 if tensor else 2e-10
    # the RMS gradient near the minimum moves with the state at the 1e-6 level: the
    # oracle's own value at iteration 20 (1.7e-6 printed) spreads over 1.7e-6 .. 4.2e-6
    # when every M update carries 1e-13 relative noise, the tensor path's rounding level
    _, gsens = G.conv_sensitivity(M0, U0, out["km"], out["ctl"], noise=1e-13 if tensor else 1e-15,
                                  runs=4 if tensor else 2, grad=True, sitesym=sym, per_update=True)
    for row, x, (it, delta, rms, spread) in zip(log, [r.initial] + r.iters, d["conv"]):
        assert int(row[0]) == int(it) == x.iter
        assert abs(row[3] - x.spread.om_tot) < tol, (int(it), row[3], x.spread.om_tot)
        assert abs(row[3] - spread) < tol + 6e-11, (int(it), row[3], spread)
        assert abs(row[2] - rms) < G.grad_tolerance(gsens, it, rms, factor=3.0), (int(it), row[2], rms)
    fin = d["centres_final"]
    np.testing.assert_allclose(out["centres"].T, fin[:, :3], rtol=0, atol=1.01e-6)
    np.testing.assert_allclose(out["spreads"], fin[:, 3], rtol=0, atol=2e-8)
    np.testing.assert_allclose(out["omega"], d["omega_final"], rtol=0, atol=2e-9 if tensor else 1.01e-9)
    # the run stays on the symmetric manifold: U(R k) = d U(k) D^+ still holds at the end
    for ir in range(sym.nkirr):
        ik = sym.ir2ik[ir]
        for isym in range(1, sym.nsym):
            k2 = sym.kptsym[isym, ir]
            if k2 == ik:
                continue
            want = sym.d_band[ir, isym] @ out["U"][ik] @ sym.d_wann[ir, isym].conj().T
            np.testing.assert_allclose(out["U"][k2], want, atol=1e-8)


def test_symmetry_adapted_cli(tmp_path, capfd):
    """The file flow: site_symmetry / symmetrize_eps in the .win and the seed's .dmn."""
    from wannier90_gb300 import __main__ as cli
    from wannier90_gb300 import w90io
    d = G.load("sitesym21")
    kn = d["knobs"]
    ss = int(kn["search_shells"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], ss)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    seed = str(tmp_path / "GaAs")
    w90io.write_win(seed + ".win", d["real_lattice"], d["kpt_latt"], d["mp_grid"], 4, search_shells=ss, iprint=1,
                    site_symmetry=".true.", symmetrize_eps="1d-9")
    w90io.write_mmn(seed + ".mmn", synth.from_math_m(M), km["nnlist"], km["nncell"])
    w90io.write_amn(seed + ".amn", synth.from_math_u(d["amn"]))
    G.write_dmn(seed + ".dmn", d)
    capfd.readouterr()
    assert cli.run(seed, "fp64") == 0
    text = capfd.readouterr().out.splitlines()
    conv = {int(l.split()[0]): float(l.split()[3]) for l in text
            if l.rstrip().endswith("<-- CONV") and not l.strip().startswith(("+", "|"))}
    for it, delta, rms, spread in d["conv"]:
        assert abs(conv[int(it)] - spread) < 2.6e-10, int(it)
    chk = w90io.read_chk(seed + ".chk")
    np.testing.assert_allclose(chk["centres"].T, d["centres_final"][:, :3], atol=1.01e-6)


def test_symmetry_adapted_disentanglement_golden():
    """testw90_disentanglement_sawfs through the C ABI: site_symmetry = T with the .dmn
    data, cdisentangle (symmetry-adapted), then cwannierise.  Every '<-- DIS' line (8
    decimals) within 1e-8, the final Omega_I, the printed '<-- CONV' spreads within
    2e-10 A^2 and the final Omega terms."""
    from tests.engine_dis import run_dis
    d = G.load("sitesym_dis")
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    out = run_dis(d["real_lattice"], d["kpt_latt"], M, np.ascontiguousarray(d["amn"]), d["eig"], int(kn["num_wann"]),
                  G.dis_control(d), int(kn["search_shells"]), wann_ctl=G.control(d),
                  extra={"site_symmetry": True, "symmetrize_eps": float(kn["symmetrize_eps"])},
                  before=lambda c: w90.w90_set_sitesym(c, G.dmn_dict(d)))
    assert out["ierr"] == 0 and out["wann_ierr"] == 0, (out["err"], out.get("wann_err"))
    for row, (it, prev, cur, delta) in zip(out["dis_log"], d["dis"]):
        assert int(row[0]) == int(it)
        assert abs(row[1] - prev) < 1e-8 and abs(row[2] - cur) < 1e-8, (int(it), row, prev, cur)
    assert abs(out["dis_info"]["omega_invariant"] - d["omega_i_final"][0]) < 1e-8
    by_iter = {int(r[0]): r for r in out["log"]}
    for it, delta, rms, spread in d["conv"]:
        assert abs(by_iter[int(it)][3] - spread) < 2e-10, (int(it), by_iter[int(it)][3], spread)
    np.testing.assert_allclose(out["omega"], d["omega_final"], rtol=0, atol=2e-9)


def test_symmetry_adapted_restart_cli(tmp_path, capfd):
    """restart = wannierise with site_symmetry = T: the .dmn is read before the restart
    branch (sitesym_read precedes it in the reference's program), and wann_main continues
    from the checkpoint in the symmetry-adapted mode: every spread of the restarted run
    against the oracle's symmetry-adapted wann_main from the same U and M."""
    from wannier90_gb300 import __main__ as cli
    from wannier90_gb300 import w90io
    d = G.load("sitesym21")
    kn = d["knobs"]
    ss = int(kn["search_shells"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], ss)
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    seed = str(tmp_path / "GaAs")
    first = 12
    w90io.write_win(seed + ".win", d["real_lattice"], d["kpt_latt"], d["mp_grid"], 4, search_shells=ss, iprint=0,
                    site_symmetry=".true.", symmetrize_eps="1d-9", num_iter=first)
    w90io.write_mmn(seed + ".mmn", synth.from_math_m(M), km["nnlist"], km["nncell"])
    w90io.write_amn(seed + ".amn", synth.from_math_u(d["amn"]))
    G.write_dmn(seed + ".dmn", d)
    assert cli.run(seed, "fp64") == 0
    chk = w90io.read_chk(seed + ".chk")
    more = 20
    w90io.write_win(seed + ".win", d["real_lattice"], d["kpt_latt"], d["mp_grid"], 4, search_shells=ss, iprint=1,
                    site_symmetry=".true.", symmetrize_eps="1d-9", num_iter=more, restart="wannierise")
    capfd.readouterr()
    assert cli.run(seed, "fp64") == 0
    text = capfd.readouterr().out.splitlines()
    conv = {int(l.split()[0]): float(l.split()[3]) for l in text
            if l.rstrip().endswith("<-- CONV") and not l.strip().startswith(("+", "|"))}
    r = O.wann_main(synth.to_math_m(chk["m"]), synth.to_math_u(chk["u"]), km, O.WannControl(num_iter=more),
                    sitesym=G.sitesym(d))
    for rec in r.iters:
        assert abs(conv[rec.iter] - rec.spread.om_tot) < 1e-9, rec.iter
    end = w90io.read_chk(seed + ".chk")
    np.testing.assert_allclose(end["centres"], r.centres, atol=1e-6)
