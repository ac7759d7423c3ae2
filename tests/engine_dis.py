"""Drive the disentanglement step through the C ABI the way a Wannier90 library caller
does (w90_disentangle, then optionally w90_wannierise on the same handle)."""
import numpy as np

from wannier90_gb300 import library as w90
from wannier90_gb300 import synth
from wannier90_gb300.synth import entangled_windows  # noqa: F401  (re-exported for the tests)


def dis_options(dc):
    """cinput_setopt keywords of an oracle DisControl (only what differs from the defaults
    is set, like a .win file)."""
    o = dict(dis_num_iter=int(dc.num_iter), dis_mix_ratio=float(dc.mix_ratio),
             dis_conv_tol=float(dc.conv_tol), dis_conv_window=int(dc.conv_window))
    if dc.win_min > -1e299:
        o["dis_win_min"] = float(dc.win_min)
    if dc.win_max < 1e299:
        o["dis_win_max"] = float(dc.win_max)
    if dc.frozen_states:
        o["dis_froz_max"] = float(dc.froz_max)
        if dc.froz_min > -1e299:
            o["dis_froz_min"] = float(dc.froz_min)
    return o


def run_dis(real_lattice, kpoints, M_raw, A, eig, num_wann, dc, search_shells=36, wann_ctl=None, extra=None,
            before=None):
    """M_raw[k,b,nb,nb], A[k,nb,W], eig[k,nb] (math layout) -> dict of results (math layout).
    before(handle): called after cinput_setopt (e.g. to pass the symmetry data); returns
    an ierr that must be 0."""
    K, nb, W = A.shape
    opts = dict(iprint=0, search_shells=int(search_shells))
    opts.update(dis_options(dc))
    if wann_ctl is not None:
        opts.update(num_iter=int(wann_ctl.num_iter), num_cg_steps=int(wann_ctl.num_cg_steps),
                    conv_tol=float(wann_ctl.conv_tol), conv_window=int(wann_ctl.conv_window))
        if wann_ctl.lfixstep:
            opts["fixed_step"] = float(wann_ctl.fixed_step)
        else:
            opts["trial_step"] = float(wann_ctl.trial_step)
    opts.update(extra or {})
    c = w90.setup(kpoints=kpoints, unit_cell_cart=real_lattice, num_wann=num_wann, num_bands=nb, **opts)
    if before is not None:
        assert before(c) == 0, c.last_error()
    m = np.array(synth.from_math_m(M_raw), order="F", copy=True)
    uopt = np.array(synth.from_math_u(A), order="F", copy=True)
    u = np.zeros((W, W, K), dtype=np.complex128, order="F")
    e = np.asfortranarray(np.asarray(eig, dtype=np.float64).T)
    w90.w90_set_m_local(c, m)
    w90.w90_set_u_matrix(c, u)
    w90.w90_set_u_opt(c, uopt)
    w90.w90_set_eigval(c, e)
    out = {"ierr": w90.w90_disentangle(c), "handle": c}
    out["err"] = c.last_error()
    out["dis_log"] = w90.w90_get_dis_log(c, int(dc.num_iter) + 1)
    out["dis_info"] = w90.w90_get_dis_info(c)
    out["U0"] = synth.to_math_u(u).copy()
    out["Uopt"] = synth.to_math_u(uopt).copy()
    out["M0"] = synth.to_math_m(m)[:, :, :W, :W].copy()
    out["m_raw_after"] = synth.to_math_m(m).copy()
    if wann_ctl is not None and out["ierr"] == 0:
        out["wann_ierr"] = w90.w90_wannierise(c)
        out["wann_err"] = c.last_error()
        out["U"] = synth.to_math_u(u).copy()
        out["M"] = synth.to_math_m(m)[:, :, :W, :W].copy()
        out["m_after_wann"] = synth.to_math_m(m).copy()
        out["log"] = w90.w90_get_log(c, int(wann_ctl.num_iter) + 1)
        out["centres"] = w90.w90_get_centres(c, num_wann)
        out["spreads"] = w90.w90_get_spreads(c, num_wann)
        out["omega"] = w90.w90_get_omega(c)
    return out
