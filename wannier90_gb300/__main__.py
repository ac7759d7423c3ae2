"""``python -m wannier90_gb300 seedname``: the wannier90.x flow for isolated bands.

Reads ``seedname.win``, builds the k-mesh, reads ``seedname.mmn`` / ``seedname.amn``
(the projections are read into u_matrix, src/wannier_prog.F90:523-529), runs the
Loewdin projection and wann_main on the GPU, prints the wannierise section of the
.wout when iprint > 0, and writes ``seedname.chk`` (src/wannier_prog.F90:256-275).
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
    if nb != nw:
        raise SystemExit("disentanglement (num_bands > num_wann) is not supported by the GPU engine")
    mp = opts.pop("mp_grid", None)
    opts.setdefault("iprint", 1)
    opts["gpu_tensor"] = 1 if precision == "tensor" else 0
    c = w90.setup(kpoints=kpts, unit_cell_cart=lattice, num_wann=nw, num_bands=nb, mp_grid=mp, **opts)
    K = len(kpts)
    nnkp = w90.w90_get_nnkp(c, K) - 1
    gkpb = np.transpose(w90.w90_get_gkpb(c, K), (1, 2, 0))
    m = w90io.read_mmn(seedname + ".mmn", nnkp, gkpb)
    a = w90io.read_amn(seedname + ".amn")
    u = np.asfortranarray(a[:, :nw, :].copy())
    uopt = np.asfortranarray(np.broadcast_to(np.eye(nb, nw, dtype=np.complex128)[:, :, None], (nb, nw, K)).copy())
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
                    u=u, m=m, centres=centres, spreads=spreads)
    return ierr


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m wannier90_gb300")
    ap.add_argument("seedname")
    ap.add_argument("--precision", default="tensor", choices=["tensor", "fp64"])
    a = ap.parse_args(argv)
    return run(a.seedname, a.precision)


if __name__ == "__main__":
    sys.exit(main())
