"""Drive the engine through its C ABI the way a Wannier90 library caller does."""
import numpy as np

from wannier90_gb300 import library as w90
from wannier90_gb300 import synth


def run_engine(real_lattice, kpoints, M_raw, A, ctl, num_wann, search_shells=36, project=True,
               iprint=0, extra=None):
    """M_raw[k,b,m,n], A[k,m,n] (math layout) -> dict of engine results (math layout)."""
    opts = dict(num_iter=int(ctl.num_iter), num_cg_steps=int(ctl.num_cg_steps),
                conv_tol=float(ctl.conv_tol), conv_window=int(ctl.conv_window), iprint=iprint,
                search_shells=int(search_shells))
    if ctl.lfixstep:
        opts["fixed_step"] = float(ctl.fixed_step)
    else:
        opts["trial_step"] = float(ctl.trial_step)
    opts.update(extra or {})
    c = w90.setup(kpoints=kpoints, unit_cell_cart=real_lattice, num_wann=num_wann, **opts)
    K = len(kpoints)
    # fresh Fortran-ordered copies: the engine updates them in place
    m = np.array(synth.from_math_m(M_raw), order="F", copy=True)
    u = np.array(synth.from_math_u(A), order="F", copy=True)
    uopt = np.asfortranarray(np.broadcast_to(np.eye(num_wann, dtype=np.complex128)[:, :, None],
                                             (num_wann, num_wann, K)).copy())
    w90.w90_set_m_local(c, m)
    w90.w90_set_u_matrix(c, u)
    w90.w90_set_u_opt(c, uopt)
    out = {}
    if project:
        w90.check(c, w90.w90_project_overlap(c), "project_overlap")
        out["U0"] = synth.to_math_u(u).copy()
        out["M0"] = synth.to_math_m(m).copy()
    ierr = w90.w90_wannierise(c)
    out["ierr"] = ierr
    out["err"] = c.last_error()
    out["U"] = synth.to_math_u(u)
    out["M"] = synth.to_math_m(m)
    out["log"] = w90.w90_get_log(c, int(ctl.num_iter) + 1)
    out["log_centres"] = w90.w90_get_log_centres(c, int(ctl.num_iter) + 1, num_wann)
    out["centres"] = w90.w90_get_centres(c, num_wann)
    out["spreads"] = w90.w90_get_spreads(c, num_wann)
    out["omega"] = w90.w90_get_omega(c)
    out["launches"] = w90.w90_kernel_launches(c)
    out["handle"] = c
    return out
