"""Oracle fixtures of the two largest synthetic workloads (test infrastructure).

* ``fcc10_w32_conv.npz`` -- the 1000-k fcc problem with 32 Wannier functions (fcc
  a = 6 A, 10x10x10 k, nntot 8, hopping range 3 cells, gauge noise 0.3, seed 0) run by
  the oracle's ``wann_main`` to convergence (conv_tol 1e-10 A^2 over a 5-iteration
  window, src/wannierise.F90:1076-1164), once from the Loewdin-projected M0/U0 and once
  from M0 with a seeded relative perturbation of 1e-15.  Stored per run: the iteration
  count, the final Omega parts, centres and spreads, and the spread at every iteration.
  The perturbed run shows how far roundoff alone moves the converged state and the
  iteration count of this chaotic minimisation.
* ``sc8_w128_window.npz`` -- the 512-k simple-cubic problem with 128 Wannier functions
  (a = 5 A, 8x8x8 k, nntot 6, gauge noise 0.5, seed 0) for ``NITER_SC8`` iterations,
  unperturbed and with 1e-15 and 1e-13 relative perturbations of M0: spreads, Omega
  parts and centres at every iteration, from which the tests read the stable window
  (the iterations over which the oracle agrees with itself under that noise).

The problems come from the seeded tight-binding generator with the oracle's own k-mesh
(no GPU, no compiled code).  Runs take about an hour (fcc10_w32) on one core each; they
run in parallel processes.

    python tests/golden/make_converged.py            # both fixtures
    python tests/golden/make_converged.py fcc10_w32  # one of them
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

# one BLAS thread per process (set before numpy loads OpenBLAS; the workers inherit it)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
os.environ.setdefault("OMP_NUM_THREADS", "1")

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NITER_SC8 = 40


def oracle_kmesh(real_lattice, kpoints, search_shells):
    """kmesh_tables-shaped tables from the oracle's kmesh_get."""
    from oracle import w90_oracle as O
    km = O.kmesh_get(real_lattice, kpoints, search_shells)
    return km["nntot"], km["nnlist"], km["nncell"], km["bk"]


def perturbed(M0, rel, seed=1234):
    if rel <= 0:
        return M0
    rng = np.random.Generator(np.random.PCG64(seed))
    noise = rng.standard_normal(M0.shape) + 1j * rng.standard_normal(M0.shape)
    return M0 + rel * np.abs(M0) * noise


def problem(name):
    from oracle import w90_oracle as O
    from wannier90_gb300 import synth
    p = synth.make_problem(**synth.CONFIGS[name], seed=0, kmesh=oracle_kmesh)
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    km = O.kmesh_get(p.real_lattice, p.kpoints)
    U0, M0 = O.overlap_project(M, A, km["nnlist"])
    return km, U0, M0


def run(job):
    name, rel, num_iter, conv_window = job
    from oracle import w90_oracle as O
    t0 = time.time()
    km, U0, M0 = problem(name)
    ctl = O.WannControl(num_iter=num_iter, num_cg_steps=5, conv_tol=1e-10, conv_window=conv_window)
    r = O.wann_main(perturbed(M0, rel), U0, km, ctl)
    recs = [r.initial] + r.iters
    s = r.spread
    out = dict(niter=np.int64(r.niter if r.niter else len(r.iters)), converged=np.bool_(r.converged),
               omega=np.array([s.om_i, s.om_d, s.om_od, s.om_tot]),
               centres=np.asarray(r.centres).T.copy(), spreads=np.asarray(r.spreads).copy(),
               spread_log=np.array([x.spread.om_tot for x in recs]),
               seconds=np.float64(time.time() - t0))
    if conv_window < 0:   # fixed-length run: keep every iteration's parts and centres
        out["omega_log"] = np.array([[x.spread.om_i, x.spread.om_d, x.spread.om_od, x.spread.om_tot]
                                     for x in recs])
        out["centres_log"] = np.array([np.asarray(x.centres).T for x in recs])
    print("%s rel=%g: %d iterations, Omega %.10f, %.0f s" % (name, rel, len(recs) - 1, s.om_tot,
                                                             time.time() - t0), flush=True)
    return job, out


def main(names):
    jobs = []
    if "fcc10_w32" in names:
        jobs += [("fcc10_w32", 0.0, 20000, 5), ("fcc10_w32", 1e-15, 20000, 5)]
    if "sc8_w128" in names:
        jobs += [("sc8_w128", rel, NITER_SC8, -1) for rel in (0.0, 1e-15, 1e-13)]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        results = pool.map(run, jobs)
    by = {}
    for (name, rel, _, _), out in results:
        tag = {0.0: "", 1e-15: "p15_", 1e-13: "p13_"}[rel]
        for k, v in out.items():
            by.setdefault(name, {})[tag + k] = v
    if "fcc10_w32" in by:
        np.savez_compressed(os.path.join(HERE, "fcc10_w32_conv.npz"), **by["fcc10_w32"])
    if "sc8_w128" in by:
        np.savez_compressed(os.path.join(HERE, "sc8_w128_window.npz"), **by["sc8_w128"])


if __name__ == "__main__":
    main(sys.argv[1:] or ["fcc10_w32", "sc8_w128"])
