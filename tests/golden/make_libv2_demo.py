"""Oracle fixture of the C++ library-mode flow on GaAs (test infrastructure).

The reference's libv2 C++ demo (test-suite/libv2-demo/libc-gas-mix-serial) drives the
library as a DFT code would: wannier_setup (cset_option_* for the system, cinput_setopt,
cinput_reader for the keywords of its gaas.win, cget_nn / cget_nnkp), then wannier_run
(cset_eigval / cset_m_local / cset_u_opt / cset_u_matrix, cdisentangle, cwannierise,
cget_centres / cget_spreads).  Its inputs (12 bands -> 8 WFs, fcc, 4x4x4 k, nntot 8) are
the ones of testw90_gaas_disentanglement_issue192, already packed in
tests/golden/gaas192_dis.npz.  Its .win keywords are DEMO_KEYWORDS below.

This script runs the oracle's dis_main and wann_main with those keywords and stores the
final state in tests/golden/libv2_gaas.npz: centres (num_wann, 3), spreads, Omega parts,
the disentanglement's iteration count and final Omega_I, the wannierisation's iteration
count and its spread at every iteration.

    python tests/golden/make_libv2_demo.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the demo's gaas.win (keywords of the library run; the system comes through cset_option)
DEMO_KEYWORDS = dict(conv_tol="1.e-13", conv_window=3, dis_froz_max="14.0d0", dis_mix_ratio="1.d0",
                     dis_num_iter=1200, fixed_step="50.d0", dis_win_max="24.0d0", num_iter=1000,
                     exclude_bands="1-5", iprint=1)


def fnum(x):
    return float(str(x).lower().replace("d", "e"))


def main():
    from oracle import w90_oracle as O
    from tests import golden_cases as G
    d = G.load("gaas192_dis")
    kn = d["knobs"]
    nw = int(kn["num_wann"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"])
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    dc = O.DisControl(num_iter=int(DEMO_KEYWORDS["dis_num_iter"]), mix_ratio=fnum(DEMO_KEYWORDS["dis_mix_ratio"]),
                      win_max=fnum(DEMO_KEYWORDS["dis_win_max"]), froz_max=fnum(DEMO_KEYWORDS["dis_froz_max"]),
                      frozen_states=True)
    U0, M0, _, _, recs = O.dis_main(M, d["amn"], d["eig"], km, nw, dc)
    ctl = O.WannControl(num_iter=int(DEMO_KEYWORDS["num_iter"]), conv_tol=fnum(DEMO_KEYWORDS["conv_tol"]),
                        conv_window=int(DEMO_KEYWORDS["conv_window"]),
                        fixed_step=fnum(DEMO_KEYWORDS["fixed_step"]), lfixstep=True)
    r = O.wann_main(M0, U0, km, ctl)
    s = r.spread
    np.savez_compressed(os.path.join(HERE, "libv2_gaas.npz"),
                        centres=np.asarray(r.centres).T.copy(), spreads=np.asarray(r.spreads).copy(),
                        omega=np.array([s.om_i, s.om_d, s.om_od, s.om_tot]),
                        dis_iterations=np.int64(len(recs)), dis_omega_i=np.float64(recs[-1].omega_i),
                        niter=np.int64(r.niter), converged=np.bool_(r.converged),
                        spread_log=np.array([x.spread.om_tot for x in [r.initial] + r.iters]),
                        keywords=np.array(sorted("%s = %s" % kv for kv in DEMO_KEYWORDS.items())))
    print("dis iterations %d, wann iterations %d (converged %s), Omega %.10f"
          % (len(recs), r.niter, r.converged, s.om_tot))


if __name__ == "__main__":
    main()
