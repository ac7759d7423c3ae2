"""``python -m wannier90_gb300 seedname``: the wannier90.x flow (src/wannier_prog.F90).

Reads ``seedname.win``, builds the k-mesh, reads ``seedname.mmn`` / ``seedname.amn``.
Isolated bands (num_bands = num_wann): the projections are read into u_matrix
(src/wannier_prog.F90:523-529) and the Loewdin projection runs.  Entangled bands
(num_bands > num_wann): ``seedname.eig`` is read too, the projections go into u_opt
and the disentanglement (dis_main + setup_m_loc) runs with the ``dis_*`` keywords of
the .win.  With site_symmetry = T, ``seedname.dmn`` supplies the symmetry data; with
restart = wannierise the run continues from ``seedname.chk`` instead.  Then
wann_main runs on the GPU, the wannierise section of the .wout is printed
when iprint > 0, and ``seedname.chk`` is written (src/wannier_prog.F90:256-275), with
Omega_I, lwindow, ndimwin and U_opt after a disentanglement.
Options: ``--precision tensor|fp64`` (default tensor).
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from . import library as w90
from . import w90io


def run(seedname, precision="tensor"):
    lattice, kpts, opts = w90io.win_system(seedname + ".win")
    nw = int(opts.pop("num_wann"))
    nb = int(opts.pop("num_bands", nw))
    mp = opts.pop("mp_grid", None)
    # the seed files hold the bands left after exclusion; the list goes to the checkpoint
    exclude = opts.pop("exclude_bands", [])
    restart = opts.pop("restart", None)
    if restart is not None and restart != "wannierise":
        raise SystemExit("restart = %s: only restart = wannierise is supported" % restart)
    opts.setdefault("iprint", 1)
    opts["gpu_tensor"] = 1 if precision == "tensor" else 0
    K = len(kpts)
    if restart == "wannierise":
        return _restart_wannierise(seedname, nb, nw, lattice, kpts, mp, exclude, opts)
    c = w90.setup(kpoints=kpts, unit_cell_cart=lattice, num_wann=nw, num_bands=nb, mp_grid=mp, **opts)
    if opts.get("site_symmetry"):
        # sitesym_read after the input (src/wannier_prog.F90:174-177)
        w90.check(c, w90.w90_set_sitesym(c, w90io.read_dmn(seedname + ".dmn", nw)), "sitesym_read")
    nnkp = w90.w90_get_nnkp(c, K) - 1
    gkpb = np.transpose(w90.w90_get_gkpb(c, K), (1, 2, 0))
    m = w90io.read_mmn(seedname + ".mmn", nnkp, gkpb)
    a = w90io.read_amn(seedname + ".amn")
    dis = None
    if nb > nw:
        eig = w90io.read_eig(seedname + ".eig", nb, K)
        u = np.zeros((nw, nw, K), dtype=np.complex128, order="F")
        uopt = np.asfortranarray(a[:, :nw, :].copy())
        w90.w90_set_eigval(c, eig)
        w90.w90_set_m_local(c, m)
        w90.w90_set_u_matrix(c, u)
        w90.w90_set_u_opt(c, uopt)
        w90.check(c, w90.w90_disentangle(c), "w90_disentangle")
        ndim, nfirst = w90.w90_get_dis_windows(c, K)
        lwindow = np.zeros((nb, K), dtype=bool, order="F")
        for k in range(K):
            lwindow[nfirst[k]:nfirst[k] + ndim[k], k] = True
        dis = dict(omega_invariant=w90.w90_get_dis_info(c)["omega_invariant"], lwindow=lwindow, ndimwin=ndim,
                   u_opt=uopt)
        # the 'postdis' checkpoint (src/wannier_prog.F90:264-266): U_opt, windows and the
        # rotated num_wann x num_wann overlaps, from which restart = wannierise continues
        w90io.write_chk(seedname + ".chk", num_bands=nb, lattice=lattice, kpts=kpts,
                        mp_grid=mp if mp is not None else (0, 0, 0), nntot=w90.w90_get_nn(c), num_wann=nw,
                        u=u, m=np.asfortranarray(m[:nw, :nw]), centres=np.zeros((3, nw)),
                        spreads=np.zeros(nw), dis=dis, exclude_bands=exclude, checkpoint="postdis")
    else:
        u = np.asfortranarray(a[:, :nw, :].copy())
        uopt = np.asfortranarray(np.broadcast_to(np.eye(nb, nw, dtype=np.complex128)[:, :, None],
                                                 (nb, nw, K)).copy())
        w90.w90_set_m_local(c, m)
        w90.w90_set_u_matrix(c, u)
        w90.w90_set_u_opt(c, uopt)
        w90.check(c, w90.w90_project_overlap(c), "w90_project_overlap")
    ierr = w90.w90_wannierise(c)
    w90.check(c, ierr, "w90_wannierise")
    centres = w90.w90_get_centres(c, nw)
    spreads = w90.w90_get_spreads(c, nw)
    w90io.write_chk(seedname + ".chk", num_bands=nb, lattice=lattice, kpts=kpts,
                    mp_grid=mp if mp is not None else (0, 0, 0), nntot=w90.w90_get_nn(c), num_wann=nw,
                    u=u, m=np.asfortranarray(m[:nw, :nw]), centres=centres, spreads=spreads, dis=dis,
                    exclude_bands=exclude)
    return ierr


def _restart_wannierise(seedname, nb, nw, lattice, kpts, mp, exclude, opts):
    """restart = wannierise: wann_main continues from the U and M of seedname.chk (the
    reference reads the checkpoint instead of the overlaps and the projections,
    src/wannier_prog.F90:204-235).  The symmetry data are read first, as sitesym_read
    comes before the restart branch (src/wannier_prog.F90:174-177).  A checkpoint
    written after a disentanglement ('postdis', or a finished entangled run) holds the
    num_wann x num_wann overlaps of the optimal subspace: wann_main runs on them, and its
    U_opt, windows and Omega_I go into the new checkpoint unchanged."""
    chk = w90io.read_chk(seedname + ".chk")
    K = len(kpts)
    if chk["num_wann"] != nw or chk["num_kpts"] != K:
        raise SystemExit("restart: %s.chk does not match the .win (num_wann / k-points)" % seedname)
    dis = None
    if chk.get("have_disentangled"):
        if chk["num_bands"] != nb:
            raise SystemExit("restart: %s.chk does not match the .win (num_bands)" % seedname)
        dis = dict(omega_invariant=chk["omega_invariant"], lwindow=chk["lwindow"], ndimwin=chk["ndimwin"],
                   u_opt=chk["u_opt"])
    # the overlaps of the checkpoint are num_wann x num_wann blocks
    c = w90.setup(kpoints=kpts, unit_cell_cart=lattice, num_wann=nw, num_bands=nw, mp_grid=mp, **opts)
    if opts.get("site_symmetry"):
        w90.check(c, w90.w90_set_sitesym(c, w90io.read_dmn(seedname + ".dmn", nw)), "sitesym_read")
    u = np.asfortranarray(chk["u"].astype(np.complex128))
    m = np.asfortranarray(chk["m"].astype(np.complex128))
    uopt = np.asfortranarray(np.broadcast_to(np.eye(nw, dtype=np.complex128)[:, :, None], (nw, nw, K)).copy())
    w90.w90_set_m_local(c, m)
    w90.w90_set_u_matrix(c, u)
    w90.w90_set_u_opt(c, uopt)
    ierr = w90.w90_wannierise(c)
    w90.check(c, ierr, "w90_wannierise")
    w90io.write_chk(seedname + ".chk", num_bands=nb, lattice=lattice, kpts=kpts,
                    mp_grid=mp if mp is not None else (0, 0, 0), nntot=w90.w90_get_nn(c), num_wann=nw, u=u, m=m,
                    centres=w90.w90_get_centres(c, nw), spreads=w90.w90_get_spreads(c, nw), dis=dis,
                    exclude_bands=exclude)
    return ierr


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m wannier90_gb300")
    ap.add_argument("seedname")
    ap.add_argument("--precision", default="tensor", choices=["tensor", "fp64"])
    a = ap.parse_args(argv)
    return run(a.seedname, a.precision)


if __name__ == "__main__":
    sys.exit(main())
