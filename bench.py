"""Benchmark: converged MLWF solves/s on one GB300 (replicas over N GPUs).

Workload (default ``fcc10_w32``): seeded tight-binding problem, fcc a = 6 A, 10x10x10
k-mesh (1000 k), nntot = 8, num_wann = 32, hopping range 3 cells, gauge noise 0.3,
run to convergence (conv_tol = 1e-10 A^2 over conv_window = 5).  One *step* is one
full wann_main solve starting from the Loewdin-projected M^(0), U^(0).

value : solves/s with M^(0), U^(0) resident in HBM (device-pointer entry point);
        M (131 MB) plus the solver state exceed the 129 MB L2, so no flush is needed.
e2e   : solves/s through the reference-named C ABI (cwannierise) with host buffers:
        per step H2D of M and U, D2H of the rotated M and final U.
roofline: dominant kernel, timed live with CUDA events on its launch stream
        (profiling pass of the engine), algorithmic FLOPs per launch.
cpu_baseline: the NumPy oracle (CPU restatement of wann_main) on the host cores, one
        process per core over the same problem, a bounded number of iterations,
        converted to solves/s with the GPU's iteration count per solve.

``--impl reference`` times that CPU restatement alone (the reference wannier90.x is
Fortran and cannot be built in this image), printing the same metric.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "converged MLWF solves/s"
try:
    MEASURED = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
except Exception:
    MEASURED = {}
WORKLOADS = {
    "fcc10_w32": dict(cfg="fcc10_w32", conv_tol=1e-10, conv_window=5, num_iter=20000),
    "sc4_w8": dict(cfg="sc4_w8", conv_tol=1e-10, conv_window=-1, num_iter=200),
    # 256 independent problems, W ~ U{4,8,...,64}, k-mesh ~ U{3^3,4^3,6^3,8^3}, sc a ~ U[3,7] A,
    # nntot 6, 300 iterations each, solved together
    "batch256": dict(cfg=None, conv_tol=1e-10, conv_window=-1, num_iter=300, nprob=256),
    # precision stress: sc 8^3 (512 k), nntot 6, num_wann 128, gauge noise 0.5, 200
    # iterations; tensor-core products against the FP64 engine, per-iteration errors
    "sc8_w128": dict(cfg="sc8_w128", conv_tol=1e-10, conv_window=-1, num_iter=200, precision_report=True),
    # serving stream: Poisson arrivals (200 req/s), W log-uniform [8,96], k-mesh
    # U{4^3,6^3,8^3,10^3,12^3}, sc/fcc 50/50, gauge noise U[0.1,0.5], each run to
    # convergence (1e-10 A^2 over 5 iterations); admission by a 150 GB HBM budget.
    # One step = the first `njobs` arrivals of the seeded stream, end to end.
    "serve": dict(cfg=None, conv_tol=1e-10, conv_window=5, num_iter=20000, serve=True, rate=200.0, njobs=24,
                  budget=150e9, slots=64),
    # entangled bands: fcc a = 6 A, 8x8x8 k-mesh (512 k), nntot 8, 48 orbitals -> 32 WFs,
    # the 16 other orbitals raised by 8 (energy units of the model) so their bands overlap
    # the top of the target manifold; outer window ~40 of 48 bands (lowest band cut at
    # some k), frozen window up to 17 states; dis_main (dis_num_iter 200, dis_conv_tol
    # 1e-10, window 3, mixing 0.5) + setup_m_loc, then wann_main to convergence (1e-10 A^2
    # over 5 iterations).  One step = the whole library run (cdisentangle + cwannierise).
    # seed-file input of config 2: the fcc 10^3, W = 32 overlaps as a formatted .mmn
    # (8.2 M records, 303 MB), parsed into the device-resident M the engine solves on.
    "seedio_fcc10_w32": dict(cfg="fcc10_w32", seedio=True),
    "dis_fcc8_b48w32": dict(cfg=None, dis=True, problem=dict(kind="fcc", a=6.0, mp=(8, 8, 8), num_bands=48,
                                                               num_wann=32, rmax=2, eps=0.3, offset=8.0),
                            dis_num_iter=200, dis_conv_tol=1e-10, dis_conv_window=3, dis_mix_ratio=0.5,
                            conv_tol=1e-10, conv_window=5, num_iter=20000),
}


def batch_params(i):
    """Shape of problem i of the batched workload (seeded by its index)."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(1000003 * (i + 1)))
    W = int(rng.choice(np.arange(4, 65, 4)))
    n = int(rng.choice([3, 4, 6, 8]))
    a = float(rng.uniform(3.0, 7.0))
    return dict(kind="sc", a=a, mp=(n, n, n), num_wann=W, rmax=2, eps=0.3)


def serve_params(i, wmax=96, nmax=12):
    """Shape of request i of the serving stream (seeded by its arrival index)."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(7919 * (i + 1)))
    W = int(round(math.exp(rng.uniform(math.log(8.0), math.log(wmax)))))
    n = int(rng.choice([x for x in (4, 6, 8, 10, 12) if x <= nmax]))
    kind = "sc" if rng.random() < 0.5 else "fcc"
    eps = float(rng.uniform(0.1, 0.5))
    return dict(kind=kind, a=5.0 if kind == "sc" else 6.0, mp=(n, n, n), num_wann=W, rmax=2, eps=eps)


def _gen_serve_problem(args):
    i, wmax, nmax = args
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    from wannier90_gb300 import synth
    return i, synth.make_problem(**serve_params(i, wmax, nmax), seed=i)


def _gen_batch_problem(i):
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    from wannier90_gb300 import synth
    p = synth.make_problem(**batch_params(i), seed=i)
    return i, p


def replica_rate(ms_local, steps, world, dist=None, device="cuda"):
    """Replicas: every rank times its own `steps` solves; the job's time is the slowest
    rank's (max over ranks) and the whole-job rate counts every rank's solves.
    Returns (ms per step, solves/s of the job)."""
    ms = ms_local
    if dist is not None:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / steps
    return ms_per_step, world * 1e3 / ms_per_step


def _env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


# ----------------------------------------------------------------------------------
# CPU restatement timing (oracle) -- used by the cpu_baseline leg and --impl reference
# ----------------------------------------------------------------------------------
def _oracle_kmesh(real_lattice, kpoints, search_shells):
    """The k-mesh tables of the oracle's kmesh_get in the generator's layout."""
    from oracle import w90_oracle as O
    km = O.kmesh_get(real_lattice, kpoints, search_shells)
    return km["nntot"], km["nnlist"], km["nncell"], km["bk"]


def oracle_iterations(workload):
    """Iterations per converged solve of the oracle's own wann_main on this workload: the
    committed fixture of the oracle run to convergence (tests/golden/make_converged.py);
    fixed-length workloads run their num_iter."""
    wl = WORKLOADS[workload]
    if wl.get("conv_window", -1) <= 1:
        return wl["num_iter"]
    import numpy as np
    path = os.path.join(ROOT, "tests", "golden", workload + "_conv.npz")
    if not os.path.exists(path):
        return None
    return int(np.load(path)["niter"])


def bench_config(workload, wl, K=None, B=None, W=None, world=1):
    """The config object of both arms' lines (identical keys and values for one workload)."""
    from wannier90_gb300 import synth
    c = synth.CONFIGS[wl["cfg"]]
    K = K or c["mp"][0] * c["mp"][1] * c["mp"][2]
    B = B or {"sc": 6, "fcc": 8, "bcc": 12}[c["kind"]]
    W = W or c["num_wann"]
    return {"workload": workload, "lattice": c["kind"], "a_angstrom": c["a"],
            "kmesh": "%dx%dx%d" % tuple(c["mp"]), "num_kpts": K, "nntot": B, "num_wann": W,
            "conv_tol": wl["conv_tol"], "conv_window": wl["conv_window"], "num_iter_cap": wl["num_iter"],
            "seed": 0, "l2": ("inputs larger than L2 (M = %d MiB)" if W * W * K * B * 16 > 129e6 else
                              "inputs smaller than L2 (M = %d MiB), not flushed") % (W * W * K * B * 16 >> 20),
            "parallelism": "replicas" if world > 1 else "single"}


def _cpu_worker(args):
    wl, seed, iters = args
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    import numpy as np  # noqa: F401

    from oracle import w90_oracle as O
    from wannier90_gb300 import synth

    # the problem is built on the oracle's k-mesh: nothing of the engine's library is loaded
    p = synth.make_problem(**synth.CONFIGS[wl["cfg"]], seed=seed, kmesh=_oracle_kmesh)
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    km = O.kmesh_get(p.real_lattice, p.kpoints)
    U0, M0 = O.overlap_project(M, A, km["nnlist"])
    ctl = O.WannControl(num_iter=iters, conv_tol=wl["conv_tol"], conv_window=-1)
    t = time.perf_counter()
    r = O.wann_main(M0, U0, km, ctl, record=False)
    dt = time.perf_counter() - t
    return dt / max(r.niter, 1)


def _cpu_dis_worker(args):
    """Seconds per dis_extract iteration and per wann_main iteration of the oracle on one
    core (entangled workload)."""
    wl, iters = args
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    import numpy as np

    from oracle import w90_oracle as O
    from wannier90_gb300 import synth

    p = synth.make_entangled_problem(**wl["problem"], seed=0)
    eig = np.ascontiguousarray(p.eig.T)
    w = synth.entangled_windows(eig, p.num_wann)
    km = O.kmesh_get(p.real_lattice, p.kpoints)
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    dc = O.DisControl(num_iter=iters, mix_ratio=wl["dis_mix_ratio"], conv_tol=0.0, conv_window=wl["dis_conv_window"],
                      win_min=w["win_min"], win_max=w["win_max"], froz_max=w["froz_max"], frozen_states=True)
    t = time.perf_counter()
    U0, M0, _, _, recs = O.dis_main(M, A, eig, km, p.num_wann, dc)
    t_dis = (time.perf_counter() - t) / max(len(recs), 1)
    t = time.perf_counter()
    r = O.wann_main(M0, U0, km, O.WannControl(num_iter=iters, conv_window=-1), record=False)
    t_wann = (time.perf_counter() - t) / max(r.niter, 1)
    return t_dis, t_wann


def cpu_dis_seconds(wl, iters, procs):
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        per = pool.map(_cpu_dis_worker, [(wl, iters)] * procs)
    return statistics.mean(x[0] for x in per), statistics.mean(x[1] for x in per)


def cpu_seconds_per_iteration(wl, iters, procs):
    ctx = mp.get_context("spawn")
    env_old = os.environ.get("OPENBLAS_NUM_THREADS")
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    try:
        with ctx.Pool(procs) as pool:
            per = pool.map(_cpu_worker, [(wl, 0, iters)] * procs)
    finally:
        if env_old is None:
            os.environ.pop("OPENBLAS_NUM_THREADS", None)
        else:
            os.environ["OPENBLAS_NUM_THREADS"] = env_old
    return statistics.mean(per)


# ----------------------------------------------------------------------------------
# clocks sampling during the timed region
# ----------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------------
def run_reference_arm(args, wl):
    rank, _, world = _env_rank()
    if rank != 0:
        return 0
    if wl.get("dis"):
        return run_reference_arm_dis(args, wl)
    if wl.get("seedio"):
        return run_reference_arm_seedio(args, wl)
    procs = os.cpu_count() or 1
    iters = args.cpu_iters
    spi = cpu_seconds_per_iteration(wl, iters, procs)
    niter = args.assume_iters or oracle_iterations(args.workload)
    if niter is None:
        print(json.dumps({"impl": "reference", "unavailable": "no converged oracle fixture for %s "
                          "(tests/golden/make_converged.py)" % args.workload}))
        return 0
    # each step: a bounded sample (iters iterations on every core); solves/s extrapolated
    t_steps = []
    for _ in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        s = cpu_seconds_per_iteration(wl, max(2, iters // 2), procs)
        t_steps.append(time.perf_counter() - t0)
        spi = 0.5 * (spi + s)
    value = procs / (spi * niter)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(t_steps[args.warmup:]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded tight-binding generator)",
        "config": bench_config(args.workload, wl, world=world),
        "note": "CPU restatement of wann_main (NumPy/LAPACK), not wannier90.x: no Fortran compiler in the image",
        "iterations_per_solve": niter,
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": procs, "kind": "port",
                         "sample": "%d iterations per core of the %s solve (1 process per core, 1 BLAS thread), "
                                   "solves/s = cores / (s_per_iter * %d iterations per solve; the oracle's own "
                                   "converged count)" % (iters, args.workload, niter)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_reference_arm_seedio(args, wl):
    """The reference reads the .mmn record by record on one core; its stand-in is the host
    reader restricted to one thread on the same file."""
    import tempfile

    from wannier90_gb300 import synth, w90io
    p = synth.make_problem(**synth.CONFIGS[wl["cfg"]], seed=0)
    tmp = tempfile.mkdtemp(prefix="w90g_seed_")
    path = os.path.join(tmp, "fcc10_w32.mmn")
    w90io.write_mmn(path, p.m, p.nnlist, p.nncell)
    size = os.path.getsize(path)
    ts = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        w90io.read_mmn(path, p.nnlist, p.nncell, nthreads=1)
        if i >= args.warmup:
            ts.append(time.perf_counter() - t0)
    os.remove(path)
    os.rmdir(tmp)
    value = size / statistics.mean(ts) / 1e6
    print(json.dumps({
        "impl": "reference", "metric": "seed .mmn parsed into device overlaps", "value": value, "unit": "MB/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(ts),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "text->f64",
        "data": "synthetic (config-2 overlaps written as a formatted .mmn)",
        "config": {"workload": args.workload, "note": "host reader on one thread (overlap_read is a serial "
                   "record-by-record read); wannier90.x cannot be built here"},
        "cpu_baseline": {"value": value, "unit": "MB/s", "cores": 1, "kind": "port", "sample": "the whole file"},
        "e2e": {"value": value, "unit": "MB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def run_reference_arm_dis(args, wl):
    """CPU restatement of the entangled workload: dis_extract and wann_main iterations timed
    on every core, solves/s extrapolated with the GPU arm's iteration counts."""
    procs = os.cpu_count() or 1
    n_dis, n_wann = KNOWN_ITERS[args.workload]
    t_steps, vals = [], []
    for _ in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        t_dis, t_wann = cpu_dis_seconds(wl, args.cpu_iters, procs)
        t_steps.append(time.perf_counter() - t0)
        vals.append(procs / (t_dis * n_dis + t_wann * n_wann))
    value = statistics.mean(vals[args.warmup:])
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(t_steps[args.warmup:]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded entangled tight-binding generator)",
        "config": {"workload": args.workload, "note": "CPU restatement of dis_main + wann_main (NumPy/LAPACK), "
                   "not wannier90.x: no Fortran compiler in the image"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": procs, "kind": "port",
                         "sample": "%d dis_extract + %d wann_main iterations per core (1 process per core, 1 BLAS "
                                   "thread); solves/s = cores / (s_per_dis_iter * %d + s_per_wann_iter * %d)"
                                   % (args.cpu_iters, args.cpu_iters, n_dis, n_wann)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _dis_flops(p, w):
    """Algorithmic FP64 FLOPs of one k_dis_z launch: per (k,b) C_b = M_w(k,b) U_opt(k+b)
    (n x W x n') and the upper triangle of C_b C_b^H over the window (n(n+1)/2 x W), per k
    tr(U^H Z U) (n x n x W); 8 real FLOPs per complex multiply-add."""
    import numpy as np
    eig = np.ascontiguousarray(p.eig.T)                      # ascending per k
    inwin = (eig >= w["win_min"]) & (eig <= w["win_max"])
    n = inwin.sum(axis=1)                                    # window states per k
    W = p.num_wann
    z = 0.0
    for k in range(len(n)):
        for b in range(p.nntot):
            k2 = p.nnlist[k, b]
            z += 8.0 * (n[k] * W * n[k2] + n[k] * (n[k] + 1) / 2 * W)
        z += 8.0 * n[k] * n[k] * W
    return z


def run_dis(args, wl):
    """Entangled workload: cdisentangle + cwannierise on one problem.  value = solves/s with
    the inputs resident in HBM (device entry points); e2e through cdisentangle /
    cwannierise with host buffers."""
    import ctypes as C

    import numpy as np
    import torch

    from wannier90_gb300 import library as w90
    from wannier90_gb300 import synth

    torch.cuda.set_device(0)
    p = synth.make_entangled_problem(**wl["problem"], seed=0)
    nb, W, K, B = p.num_bands, p.num_wann, len(p.kpoints), p.nntot
    eig = np.ascontiguousarray(p.eig.T)
    w = synth.entangled_windows(eig, W)
    opts = dict(num_iter=wl["num_iter"], conv_tol=wl["conv_tol"], conv_window=wl["conv_window"], iprint=0,
                gpu_tensor=1 if args.precision == "tensor" else 0, dis_num_iter=wl["dis_num_iter"],
                dis_conv_tol=wl["dis_conv_tol"], dis_conv_window=wl["dis_conv_window"],
                dis_mix_ratio=wl["dis_mix_ratio"], dis_win_min=w["win_min"], dis_win_max=w["win_max"],
                dis_froz_max=w["froz_max"])
    h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_bands=nb, **opts)
    stream = torch.cuda.Stream()
    w90.w90_set_stream(h, stream.cuda_stream)
    m0 = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
    a0 = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
    e0 = torch.from_numpy(np.ascontiguousarray(p.eig.reshape(-1, order="F"))).cuda()
    m_w, a_w = torch.empty_like(m0), torch.empty_like(a0)
    u_w = torch.zeros(2 * W * W * K, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    if args.profile_case > 0:
        # one disentanglement capped at profile_case iterations, no wannierisation (ncu)
        hp = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_bands=nb,
                       **dict(opts, dis_num_iter=args.profile_case))
        m_w.copy_(m0)
        a_w.copy_(a0)
        w90.check(hp, w90.w90_disentangle_device(hp, m_w.data_ptr(), a_w.data_ptr(), u_w.data_ptr(), e0.data_ptr()),
                  "profile case")
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": args.profile_case, "workload": args.workload,
                          "omega_invariant": w90.w90_get_dis_info(hp)["omega_invariant"]}))
        return 0

    def device_step():
        with torch.cuda.stream(stream):
            m_w.copy_(m0)
            a_w.copy_(a0)
        w90.check(h, w90.w90_disentangle_device(h, m_w.data_ptr(), a_w.data_ptr(), u_w.data_ptr(), e0.data_ptr()),
                  "disentangle")
        w90.check(h, w90.w90_wannierise_device(h, m_w.data_ptr(), u_w.data_ptr()), "wannierise")

    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()
    n_dis = len(w90.w90_get_dis_log(h, wl["dis_num_iter"] + 1))
    n_wann = int(w90.w90_get_log(h, wl["num_iter"] + 1)[-1][0])
    launches_per_step = w90.w90_kernel_launches(h)   # last disentanglement + last wannierisation
    clocks = ClockSampler(0)
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        device_step()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_per_step = ev0.elapsed_time(ev1) / args.steps
    value = 1e3 / ms_per_step
    info = w90.w90_get_dis_info(h)
    omega = w90.w90_get_omega(h)

    # e2e: the library calls with host buffers (pageable NumPy arrays, as a Fortran or
    # C++ caller passes them), copies inside the calls
    m_h = np.empty_like(p.m)
    a_h = np.empty_like(p.a)
    u_h = np.zeros((W, W, K), dtype=np.complex128, order="F")
    e_h = np.asfortranarray(p.eig)
    w90.w90_set_m_local(h, m_h)
    w90.w90_set_u_opt(h, a_h)
    w90.w90_set_u_matrix(h, u_h)
    w90.w90_set_eigval(h, e_h)
    e2e_t = []
    for _ in range(max(1, args.e2e_steps)):
        m_h[...] = p.m
        a_h[...] = p.a
        t0 = time.perf_counter()
        w90.check(h, w90.w90_disentangle(h), "disentangle")
        w90.check(h, w90.w90_wannierise(h), "wannierise")
        e2e_t.append(time.perf_counter() - t0)
    e2e_value = 1.0 / statistics.mean(e2e_t)
    h2d = p.m.nbytes + p.a.nbytes + p.eig.nbytes + 2 * W * W * B * K * 16 + W * W * K * 16
    d2h = p.a.nbytes + W * W * K * 16 + 2 * W * W * B * K * 16 + W * W * K * 16

    # per-kernel device times of the disentanglement (CUDA events around every launch)
    with torch.cuda.stream(stream):
        m_w.copy_(m0)
        a_w.copy_(a0)
    torch.cuda.synchronize()
    ierr, prof = w90.w90_profile_dis_device(h, m_w.data_ptr(), a_w.data_ptr(), u_w.data_ptr(), e0.data_ptr())
    w90.check(h, ierr, "profile")
    tot = sum(v[0] for v in prof.values())
    per_kernel = {k: {"ms_total": v[0], "launches": v[1], "ms_avg": v[0] / v[1] if v[1] else None,
                      "share": v[0] / tot if tot else None} for k, v in prof.items()}
    # wall split of one step between the two library calls (device entry points)
    with torch.cuda.stream(stream):
        m_w.copy_(m0)
        a_w.copy_(a0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    w90.check(h, w90.w90_disentangle_device(h, m_w.data_ptr(), a_w.data_ptr(), u_w.data_ptr(), e0.data_ptr()),
              "disentangle")
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    w90.check(h, w90.w90_wannierise_device(h, m_w.data_ptr(), u_w.data_ptr()), "wannierise")
    torch.cuda.synchronize()
    phase_s = {"disentangle": t1 - t0, "wannierise": time.perf_counter() - t1}
    fp64_peak = lib_fp64_peak()
    zf = _dis_flops(p, w)
    dom = max(per_kernel, key=lambda k: per_kernel[k]["ms_total"])
    zavg = per_kernel["k_dis_z"]["ms_avg"]
    achieved = zf / (zavg * 1e-3) / 1e12
    roof = {"bound": "fp64", "kernel": "k_dis_z", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": achieved / fp64_peak if fp64_peak > 0 else None, "traffic": None,
            "peak_source": "FP64 FMA probe measured in this run (MEASURED_PEAKS.json has no FP64 figure)",
            "algorithmic_flops_per_launch": zf, "dominant_dis_kernel": dom,
            "dis_ms_total": tot, "per_kernel": per_kernel, "phase_seconds": phase_s,
            "note": "k_dis_z is the dominant kernel of the disentanglement; the wannierisation phase "
                    "runs the kernels of the isolated-band workloads (see fcc10_w32)"}
    cpu = None
    if not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        t_dis, t_wann = cpu_dis_seconds(wl, args.cpu_iters, procs)
        cpu = {"value": procs / (t_dis * n_dis + t_wann * n_wann), "unit": "solves/s", "cores": procs,
               "kind": "port",
               "sample": "%d dis_extract + %d wann_main iterations per core on %d cores (1 process per core, "
                         "1 BLAS thread); %.3f s/dis iter, %.3f s/wann iter; solves/s = cores / (s/dis iter * %d "
                         "+ s/wann iter * %d)" % (args.cpu_iters, args.cpu_iters, procs, t_dis, t_wann, n_dis,
                                                  n_wann)}
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded entangled tight-binding generator)",
        "config": {"workload": args.workload, "lattice": "fcc", "num_kpts": K, "nntot": B, "num_bands": nb,
                   "num_wann": W, "dis_iterations": n_dis, "dis_converged": info["converged"],
                   "dis_max_jacobi_sweeps": info["max_sweeps"], "offset": wl["problem"]["offset"],
                   "omega_invariant": info["omega_invariant"], "wannierise_iterations": n_wann,
                   "omega_total": float(omega[3]), "windows": w,
                   "precision": "disentanglement fp64; wannierise " + args.precision,
                   "l2": "inputs larger than L2 (M = %d MB)" % (p.m.nbytes >> 20)},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches_per_step) * args.steps,
        "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def run_seedio(args, wl):
    """Seed-file workload: one step = the .mmn of config 2 read from the page cache into
    device memory.  value: MB/s of text converted by the parse kernels (text resident in
    HBM); e2e: MB/s of the whole call (file read into pinned memory, copy, kernels);
    cpu_baseline: the host reader (all cores) on the same file."""
    import tempfile

    import numpy as np
    import torch

    from wannier90_gb300 import synth, w90io

    torch.cuda.set_device(0)
    p = synth.make_problem(**synth.CONFIGS[wl["cfg"]], seed=0)
    tmp = tempfile.mkdtemp(prefix="w90g_seed_")
    path = os.path.join(tmp, "fcc10_w32.mmn")
    w90io.write_mmn(path, p.m, p.nnlist, p.nncell)
    size = os.path.getsize(path)
    nb, _, B, K = p.m.shape
    nrec = nb * nb * B * K
    dm = torch.empty(2 * p.m.size, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    timing = np.zeros(3)

    def step():
        t0 = time.perf_counter()
        used, nl = w90io.read_mmn_device(path, p.nnlist, p.nncell, dm.data_ptr(), stream.cuda_stream, timing)
        torch.cuda.synchronize()
        if not used:
            raise RuntimeError("the device parser handed the file to the host reader")
        return time.perf_counter() - t0, timing.copy(), nl

    for _ in range(args.warmup):
        step()
    host_ref = w90io.read_mmn(path, p.nnlist, p.nncell)
    got = dm.cpu().numpy().view(np.complex128).reshape(p.m.shape, order="F")
    if not np.array_equal(got, host_ref):
        raise RuntimeError("device parse differs from the host reader")
    clocks = ClockSampler(0)
    clocks.start()
    res = [step() for _ in range(args.steps)]
    clk = clocks.stop()
    wall = statistics.mean(r[0] for r in res)
    k_vals = statistics.mean(r[1][0] for r in res)
    k_all = statistics.mean(r[1][1] for r in res)
    h2d = statistics.mean(r[1][2] for r in res)
    launches = res[-1][2]
    # host reader, all cores
    t_cpu = []
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        w90io.read_mmn(path, p.nnlist, p.nncell)
        t_cpu.append(time.perf_counter() - t0)
    cpu_s = statistics.mean(t_cpu)
    # k_mmn_values: reads the text of the value records (all but the block headers) and
    # two record offsets, writes 16 B per record
    head_bytes = 0
    with open(path, "rb") as f:
        f.readline()
        f.readline()
        first = f.readline()
    head_bytes = len(first) * B * K
    alg = (size - head_bytes) + nrec * (16 + 16)
    achieved = alg / (k_vals * 1e-3) / 1e9
    peak = float(MEASURED.get("hbm_gbs", 6800.0))
    line = {
        "metric": "seed .mmn parsed into device overlaps", "value": size / (k_all * 1e-3) / 1e6, "unit": "MB/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "text->f64",
        "data": "synthetic (config-2 overlaps written as a formatted .mmn)",
        "config": {"workload": args.workload, "file_MB": size / 1e6, "records": nrec, "num_kpts": K, "nntot": B,
                   "num_bands": nb, "l2": "text (303 MB) larger than L2",
                   "value_basis": "text bytes / device time of all parse kernels (text resident in HBM)",
                   "h2d_ms": h2d},
        "e2e": {"value": size / wall / 1e6, "unit": "MB/s", "h2d_bytes_per_step": size, "d2h_bytes_per_step": 4 * B * K},
        "gpu_launches": int(launches) * args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_mmn_values", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "peak_source": "hbm_gbs of MEASURED_PEAKS.json, of measured" if "hbm_gbs" in MEASURED
                     else "6.8 TB/s, of fallback",
                     "algorithmic_bytes_per_launch": alg, "ms_per_launch": k_vals},
        "cpu_baseline": {"value": size / cpu_s / 1e6, "unit": "MB/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": "the host reader (w90g_read_mmn: record index + from_chars on all cores) on the "
                                   "same file; the reference reads it record by record on one core"},
        "clocks": clk,
    }
    print(json.dumps(line))
    os.remove(path)
    os.rmdir(tmp)
    return 0


def lib_fp64_peak():
    from wannier90_gb300._native import lib
    return lib().w90g_measure_fp64_peak()


def run_batch(args, wl):
    """Batched workload (256 independent problems, 300 iterations each): all problems solved
    together, grouped by kernel configuration, one captured iteration graph per group, the
    groups concurrently on their own streams.  One step = one batch solve of every problem.
    The mixed-precision arm takes each width's configuration from the autotuner; the FP64
    arm solves the same problems with every product on the FP64 pipe.  Both arms run the
    same 300 iterations per problem (iteration-matched by construction).  Warm-up steps
    solve a 16-problem prefix (three times per arm); the timed steps solve all problems."""
    import numpy as np
    import torch

    from wannier90_gb300 import autotune
    from wannier90_gb300 import library as w90

    torch.cuda.set_device(0)
    n = args.batch_size or wl["nprob"]
    procs = min(os.cpu_count() or 1, 16)
    with mp.get_context("spawn").Pool(procs) as pool:
        probs = [p for _, p in sorted(pool.map(_gen_batch_problem, range(n)))]
    ws = [p.num_wann for p in probs]
    tune = autotune.table(ws)
    m0s = [torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda() for p in probs]
    u0s = [torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda() for p in probs]

    def make_arm(mixed):
        handles = []
        for i, p in enumerate(probs):
            opts = autotune.options(p.num_wann) if mixed else dict(gpu_tensor=0)
            h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=p.num_wann,
                          num_iter=wl["num_iter"], conv_window=-1, iprint=0, **opts)
            handles.append(h)
        return handles

    # Loewdin projection once (the FP64 path), shared by both arms
    hproj = make_arm(False)
    for h, m, u in zip(hproj, m0s, u0s):
        w90.check(h, w90.w90_project_overlap_device(h, m.data_ptr(), u.data_ptr()), "projection")
    torch.cuda.synchronize()
    mw = [torch.empty_like(m) for m in m0s]
    uw = [torch.empty_like(u) for u in u0s]

    def step(handles, count):
        for a, b in zip(mw[:count], m0s[:count]):
            a.copy_(b)
        for a, b in zip(uw[:count], u0s[:count]):
            a.copy_(b)
        torch.cuda.synchronize()
        t = time.perf_counter()
        ierr = w90.w90_wannierise_batch_device(handles[:count], [x.data_ptr() for x in mw[:count]],
                                               [x.data_ptr() for x in uw[:count]])
        torch.cuda.synchronize()
        if any(e > 0 for e in ierr):
            raise RuntimeError("batch failed: %s" % [h.last_error() for h in handles if h.last_error()])
        return time.perf_counter() - t

    arms = {}
    clk = None
    for name in (["mixed", "fp64"] if args.precision == "tensor" else ["fp64"]):
        hs = make_arm(name == "mixed")
        for _ in range(args.warmup):
            step(hs, min(16, n))
        clocks = ClockSampler(0)
        clocks.start()
        ts = [step(hs, n) for _ in range(args.steps)]
        c = clocks.stop()
        clk = clk or c
        finals = np.array([w90.w90_get_log(h, wl["num_iter"] + 1)[-1][3] for h in hs])
        arms[name] = {"seconds": ts, "t_step": statistics.mean(ts), "handles": hs, "final": finals, "clocks": c}
    main_arm = arms.get("mixed", arms["fp64"])
    t_step = main_arm["t_step"]
    hs = main_arm["handles"]
    # e2e (mixed arm): host buffers, H2D of every problem's M and U, D2H of the results
    mh = [x.cpu().pin_memory() for x in m0s]
    uh = [x.cpu().pin_memory() for x in u0s]
    torch.cuda.synchronize()
    t = time.perf_counter()
    for a, b in zip(mw, mh):
        a.copy_(b, non_blocking=True)
    for a, b in zip(uw, uh):
        a.copy_(b, non_blocking=True)
    torch.cuda.synchronize()
    w90.w90_wannierise_batch_device(hs, [x.data_ptr() for x in mw], [x.data_ptr() for x in uw])
    for a, b in zip(mh, mw):
        a.copy_(b, non_blocking=True)
    for a, b in zip(uh, uw):
        a.copy_(b, non_blocking=True)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t
    nbytes = sum(x.numel() * 8 for x in m0s) + sum(x.numel() * 8 for x in u0s)
    choice = {str(k): v["choice"] for k, v in tune.items()}
    line = {
        "metric": METRIC, "value": n / t_step, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded tight-binding generator)",
        "config": {"workload": args.workload, "problems": n, "iterations_each": wl["num_iter"],
                   "num_wann": "U{4,...,64}", "kmesh": "U{3^3,4^3,6^3,8^3}", "lattice": "sc a~U[3,7]",
                   "warmup_problems": min(16, n), "total_state_MB": nbytes >> 20, "l2": "inputs larger than L2"},
        "autotune": {"choice_by_num_wann": choice,
                     "times_s": {str(k): v["times"] for k, v in tune.items()}},
        "e2e": {"value": n / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
        "gpu_launches": None, "roofline": None, "cpu_baseline": None, "clocks": clk,
        "widths": {"min": min(ws), "max": max(ws), "mean": float(np.mean(ws))},
    }
    if "mixed" in arms and "fp64" in arms:
        f64 = arms["fp64"]
        fm, ff = arms["mixed"]["final"], f64["final"]
        rel = np.abs(fm - ff) / np.maximum(np.abs(ff), 1e-300)
        worst = int(np.argmax(rel))
        # the problems are chaotic minimisations run for a fixed 300 iterations: the two
        # arms' final spreads differ by where each trajectory has got to, not by roundoff
        line["fp64_gpu"] = {"value": n / f64["t_step"], "unit": "solves/s", "ms_per_step": 1e3 * f64["t_step"],
                            "mixed_over_fp64": f64["t_step"] / t_step,
                            "final_spread_rel_diff": {
                                "median": float(np.median(rel)), "p90": float(np.percentile(rel, 90)),
                                "max": float(rel.max()),
                                "worst": {"problem": worst, "num_wann": probs[worst].num_wann,
                                          "num_kpts": len(probs[worst].kpoints), "mixed": float(fm[worst]),
                                          "fp64": float(ff[worst])},
                                "mixed_lower": int(np.sum(fm < ff)), "fp64_lower": int(np.sum(ff < fm))},
                            "clocks": f64["clocks"]}
    print(json.dumps(line, default=float))
    return 0


def run_serve(args, wl):
    """Serving workload: the first njobs requests of a seeded Poisson stream are submitted
    at their arrival times to the continuous-batching server (w90g_server_*) and run to
    convergence; one step = the whole stream.  value = solves/s over the makespan
    (first arrival to last completion); latency = completion - arrival per request."""
    import numpy as np
    import torch

    from wannier90_gb300 import library as w90

    torch.cuda.set_device(0)
    n = args.serve_jobs or wl["njobs"]
    rate = args.serve_rate or wl["rate"]
    arr = np.cumsum(np.random.Generator(np.random.PCG64(0)).exponential(1.0 / rate, n))
    arr -= arr[0]
    procs = min(os.cpu_count() or 1, 16)
    with mp.get_context("spawn").Pool(procs) as pool:
        probs = [p for _, p in sorted(pool.map(_gen_serve_problem, [(i, args.serve_wmax, args.serve_nmax)
                                                                   for i in range(n)]))]
    tensor = 1 if args.precision == "tensor" else 0
    handles, m0s, u0s = [], [], []
    for p in probs:
        h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=p.num_wann,
                      num_iter=wl["num_iter"], conv_tol=wl["conv_tol"], conv_window=wl["conv_window"], iprint=0,
                      gpu_tensor=tensor)
        m = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
        u = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
        w90.check(h, w90.w90_project_overlap_device(h, m.data_ptr(), u.data_ptr()), "projection")
        handles.append(h)
        m0s.append(m)
        u0s.append(u)
    torch.cuda.synchronize()
    mw = [torch.empty_like(m) for m in m0s]
    uw = [torch.empty_like(u) for u in u0s]
    srv = w90.Server(wl["budget"], max_active=wl["slots"], chunk_iters=8)

    def step():
        for a, b in zip(mw, m0s):
            a.copy_(b)
        for a, b in zip(uw, u0s):
            a.copy_(b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(n):
            dt = arr[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            rc = srv.submit(handles[i], mw[i].data_ptr(), uw[i].data_ptr(), i)
            if rc:
                raise RuntimeError("submit %d: %s" % (i, handles[i].last_error()))
        srv.drain()
        done = srv.poll(n)
        if len(done) != n or any(d[1] > 0 for d in done):
            raise RuntimeError("serve failed: %s" % [(d[0], handles[d[0]].last_error()) for d in done if d[1]])
        lat = np.array([d[4] - d[2] for d in sorted(done)])
        span = max(d[4] for d in done) - min(d[2] for d in done)
        return span, lat

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(0)
    clocks.start()
    res = [step() for _ in range(args.steps)]
    clk = clocks.stop()
    span = statistics.mean(r[0] for r in res)
    lat = np.concatenate([r[1] for r in res])
    stats = srv.stats()
    srv.close()
    iters = [int(w90.w90_get_log(h, wl["num_iter"] + 1)[-1][0]) for h in handles]
    nbytes = sum(x.numel() * 8 for x in m0s) + sum(x.numel() * 8 for x in u0s)
    line = {
        "metric": METRIC + " + p50/p99 latency", "value": n / span, "unit": "solves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * span, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded tight-binding generator)",
        "config": {"workload": args.workload, "precision": args.precision, "requests": n, "rate_per_s": rate,
                   "num_wann": "round(logU[8,%d])" % args.serve_wmax,
                   "kmesh": "U{%s}" % ",".join("%d^3" % x for x in (4, 6, 8, 10, 12) if x <= args.serve_nmax),
                   "lattice": "sc a=5 / fcc a=6, 50/50", "conv": "1e-10 A^2 over 5 iterations",
                   "hbm_budget_GB": wl["budget"] / 1e9, "slots": wl["slots"], "l2": "inputs larger than L2"},
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "max": float(lat.max())},
        "server": stats, "iterations": {"min": min(iters), "median": int(np.median(iters)), "max": max(iters)},
        "widths": sorted(p.num_wann for p in probs), "kpts": sorted(len(p.kpoints) for p in probs),
        "e2e": None, "gpu_launches": None, "roofline": None, "cpu_baseline": None, "clocks": clk,
        "state_MB": nbytes >> 20,
    }
    print(json.dumps(line))
    return 0


def run_precision(args, wl):
    """Precision report: the same 200 iterations with every product on the FP64 pipe
    (the plain FP64 engine, reference of this report) and with the tensor-core products,
    plus the FP64 engine on an input perturbed by 1e-15 (relative), which shows how fast
    roundoff-level differences grow along this trajectory.  Errors of Omega_I, Omega_D,
    Omega_OD, Omega and of every centre are reported per iteration."""
    import numpy as np
    import torch

    from wannier90_gb300 import library as w90
    from wannier90_gb300 import synth

    torch.cuda.set_device(0)
    n_it = args.precision_iters or wl["num_iter"]
    p = synth.make_problem(**synth.CONFIGS[wl["cfg"]], seed=0)
    W, K, B = p.num_wann, len(p.kpoints), p.nntot
    opts = dict(num_iter=n_it, conv_tol=wl["conv_tol"], conv_window=-1, iprint=0)
    h0 = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, gpu_tensor=0, **opts)
    m0 = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
    u0 = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
    w90.check(h0, w90.w90_project_overlap_device(h0, m0.data_ptr(), u0.data_ptr()), "projection")
    torch.cuda.synchronize()
    rng = np.random.Generator(np.random.PCG64(12345))
    noise = torch.from_numpy(1.0 + 1e-15 * rng.standard_normal(m0.numel())).cuda()

    def run(tensor, perturb=False):
        h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, gpu_tensor=tensor, **opts)
        m, u = m0.clone(), u0.clone()
        if perturb:
            m.mul_(noise)
        torch.cuda.synchronize()
        t = time.perf_counter()
        w90.check(h, w90.w90_wannierise_device(h, m.data_ptr(), u.data_ptr()), "wannierise")
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        log = w90.w90_get_log(h, n_it + 1)
        cen = w90.w90_get_log_centres(h, n_it + 1, W)
        return log, cen, dt

    clocks = ClockSampler(0)
    clocks.start()
    ref, ref_c, t_ref = run(0)
    ten, ten_c, t_ten = run(1)
    clk = clocks.stop()
    per, per_c, _ = run(0, perturb=True)

    def errors(log, cen):
        n = min(len(log), len(ref))
        om = lambda L: np.stack([L[:n, 3] - L[:n, 4] - L[:n, 5], L[:n, 4], L[:n, 5], L[:n, 3]], axis=1)
        d = np.abs(om(log) - om(ref))
        rel = d[:, 3] / np.abs(ref[:n, 3])
        dc = np.abs(cen[:n, :3, :] - ref_c[:n, :3, :]).max(axis=(1, 2))
        return d, rel, dc

    d_t, rel_t, dc_t = errors(ten, ten_c)
    d_p, rel_p, dc_p = errors(per, per_c)
    marks = [i for i in (0, 1, 2, 3, 5, 10, 20, 30, 50, 100, 150, 200) if i < len(rel_t)]

    def first_over(rel, dc, tol_rel=1e-8, tol_c=1e-6):
        bad = np.nonzero((rel > tol_rel) | (dc > tol_c))[0]
        return int(bad[0]) if len(bad) else len(rel)

    # stable window: iterations over which roundoff-level input noise (1e-15) moves the
    # FP64 engine's own trajectory by less than 1e-11 relative (1e-9 A for centres)
    window = first_over(rel_p, dc_p, 1e-11, 1e-9)
    line = {
        "metric": "per-iteration error of the tensor-core engine against the FP64 engine",
        "value": float(rel_t[:window].max()) if window else 0.0,
        "unit": "max |dOmega|/Omega over the stable window",
        "stable_window": window,
        "max_centre_error_A_in_window": float(dc_t[:window].max()) if window else 0.0,
        "max_error_in_window": {"dOmega_I": float(d_t[:window, 0].max()) if window else 0.0,
                                "dOmega_D": float(d_t[:window, 1].max()) if window else 0.0,
                                "dOmega_OD": float(d_t[:window, 2].max()) if window else 0.0},
        "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": False, "dtype": "f64 (FP64 engine) / fp16-sliced (tensor)",
        "data": "synthetic (seeded tight-binding generator)",
        "config": {"workload": args.workload, "lattice": "sc a=5", "kmesh": "8^3", "nntot": B, "num_wann": W,
                   "eps": 0.5, "iterations": n_it},
        "ms_per_iteration": {"fp64": 1e3 * t_ref / n_it, "tensor": 1e3 * t_ten / n_it,
                             "speedup": t_ref / t_ten},
        "first_iteration_over_1e-8_or_1e-6A": {"tensor_vs_fp64": first_over(rel_t, dc_t),
                                               "fp64_vs_fp64_input_1e-15": first_over(rel_p, dc_p)},
        "per_iteration": {str(i): {"tensor": {"dOmega_I": d_t[i, 0], "dOmega_D": d_t[i, 1], "dOmega_OD": d_t[i, 2],
                                              "dOmega_rel": rel_t[i], "dcentre_A": dc_t[i]},
                                   "fp64_input_1e-15": {"dOmega_rel": rel_p[i], "dcentre_A": dc_p[i]}}
                          for i in marks},
        "final_spread": {"fp64": float(ref[-1, 3]), "tensor": float(ten[-1, 3])},
        "clocks": clk,
    }
    print(json.dumps(line, default=float))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="fcc10_w32", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-iters", type=int, default=4)
    ap.add_argument("--assume-iters", type=int, default=0,
                    help="iterations per solve for the reference arm (0: the oracle's converged count)")
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="timed solves of the plain FP64 GPU path reported beside the tensor path")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-iters", type=int, default=6)
    ap.add_argument("--e2e-steps", type=int, default=0, help="solves of the e2e leg (0: --steps)")
    ap.add_argument("--batch-size", type=int, default=0, help="problems in the batched workload (default 256)")
    ap.add_argument("--serve-jobs", type=int, default=0, help="requests of the serving stream (default 24)")
    ap.add_argument("--serve-rate", type=float, default=0.0, help="arrival rate of the serving stream (200/s)")
    ap.add_argument("--serve-wmax", type=int, default=96, help="largest num_wann of the serving stream")
    ap.add_argument("--serve-nmax", type=int, default=12, help="largest k-mesh edge of the serving stream")
    ap.add_argument("--precision-iters", type=int, default=0, help="iterations of the precision report (200)")
    ap.add_argument("--profile-case", type=int, default=0,
                    help="run one solve capped at this many iterations and exit (small case for ncu)")
    ap.add_argument("--precision", default="tensor", choices=["tensor", "fp64"],
                    help="tensor: M update and exp on tcgen05 tensor cores (exact FP16 slicing, FP64-accurate); "
                         "fp64: every product on the FP64 pipe")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference_arm(args, wl)

    if wl.get("dis"):
        return run_dis(args, wl)
    if wl.get("seedio"):
        return run_seedio(args, wl)
    if wl.get("nprob"):
        return run_batch(args, wl)
    if wl.get("serve"):
        return run_serve(args, wl)
    if wl.get("precision_report"):
        return run_precision(args, wl)
    rank, local_rank, world = _env_rank()
    import numpy as np
    import torch

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from wannier90_gb300 import library as w90
    from wannier90_gb300 import synth
    from wannier90_gb300._native import lib

    # problem (replicas: every rank solves its own copy of the same seeded problem)
    p = synth.make_problem(**synth.CONFIGS[wl["cfg"]], seed=0)
    W, K, B = p.num_wann, len(p.kpoints), p.nntot
    opts = dict(num_iter=wl["num_iter"], conv_tol=wl["conv_tol"], conv_window=wl["conv_window"], iprint=0,
                gpu_tensor=1 if args.precision == "tensor" else 0)
    h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, **opts)
    stream = torch.cuda.Stream()
    w90.w90_set_stream(h, stream.cuda_stream)
    # Loewdin projection on the device -> resident M0, U0
    m_dev = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
    u_dev = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
    torch.cuda.synchronize()
    w90.check(h, w90.w90_project_overlap_device(h, m_dev.data_ptr(), u_dev.data_ptr()), "project")
    torch.cuda.synchronize()
    m0, u0 = m_dev.clone(), u_dev.clone()
    m_work, u_work = torch.empty_like(m0), torch.empty_like(u0)

    if args.profile_case > 0:
        hp = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W,
                       **dict(opts, num_iter=args.profile_case))
        w90.check(hp, w90.w90_wannierise_device(hp, m0.clone().data_ptr(), u0.clone().data_ptr()), "profile case")
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": args.profile_case, "workload": args.workload,
                          "spread": float(w90.w90_get_log(hp, args.profile_case + 1)[-1][3])}))
        return 0

    def device_step():
        with torch.cuda.stream(stream):
            m_work.copy_(m0)
            u_work.copy_(u0)
        ierr = w90.w90_wannierise_device(h, m_work.data_ptr(), u_work.data_ptr())
        if ierr > 0:
            raise RuntimeError(h.last_error())

    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()
    log = w90.w90_get_log(h, wl["num_iter"] + 1)
    niter = int(log[-1][0])
    launches = w90.w90_kernel_launches(h)
    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for i in range(args.steps):
        device_step()
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    ms_per_step, value = replica_rate(evs[0].elapsed_time(evs[-1]), args.steps, world, dist, "cuda")
    lat_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]

    # the plain FP64 GPU path on the same problem (the metric compares the two)
    fp64 = None
    if args.precision == "tensor" and args.fp64_steps > 0:
        h64 = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, **dict(opts, gpu_tensor=0))
        w90.w90_set_stream(h64, stream.cuda_stream)

        def fp64_step():
            with torch.cuda.stream(stream):
                m_work.copy_(m0)
                u_work.copy_(u0)
            ierr = w90.w90_wannierise_device(h64, m_work.data_ptr(), u_work.data_ptr())
            if ierr > 0:
                raise RuntimeError(h64.last_error())

        fp64_step()
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(args.fp64_steps + 1)]
        e[0].record(stream)
        for i in range(args.fp64_steps):
            fp64_step()
            e[i + 1].record(stream)
        torch.cuda.synchronize()
        ms64, v64 = replica_rate(e[0].elapsed_time(e[-1]), args.fp64_steps, world, dist, "cuda")
        n64 = int(w90.w90_get_log(h64, wl["num_iter"] + 1)[-1][0])
        fp64 = {"value": v64, "unit": "solves/s", "ms_per_step": ms64, "steps": args.fp64_steps,
                "iterations_per_solve": n64, "ms_per_iteration": ms64 / n64,
                "mixed_over_fp64": value / v64,
                "mixed_over_fp64_per_iteration": (ms64 / n64) / (ms_per_step / niter)}

    # e2e through the reference-named C ABI with host buffers (pinned)
    m_host0 = torch.from_numpy(m0.cpu().numpy()).pin_memory()
    u_host0 = torch.from_numpy(u0.cpu().numpy()).pin_memory()
    m_host = torch.empty_like(m_host0).pin_memory()
    u_host = torch.empty_like(u_host0).pin_memory()
    L = lib()
    import ctypes as C
    uopt = np.asfortranarray(np.broadcast_to(np.eye(W, dtype=np.complex128)[:, :, None], (W, W, K)).copy())
    L.cset_u_opt(h.handle, uopt.ctypes.data)
    L.cset_m_local(h.handle, C.c_void_p(m_host.data_ptr()))
    L.cset_u_matrix(h.handle, C.c_void_p(u_host.data_ptr()))

    def e2e_step():
        m_host.copy_(m_host0)
        u_host.copy_(u_host0)
        ierr = C.c_int(0)
        t0 = time.perf_counter()
        L.cwannierise(h.handle, C.byref(ierr))
        dt = time.perf_counter() - t0
        if ierr.value > 0:
            raise RuntimeError(h.last_error())
        return dt

    e2e_t = [e2e_step() for _ in range(max(1, args.e2e_steps or args.steps))]
    e2e_value = world / statistics.mean(e2e_t)
    bytes_m = W * W * B * K * 16
    bytes_u = W * W * K * 16

    # roofline of the dominant kernel (profiling pass, CUDA events on the launch stream)
    nkind = 9
    msk = (C.c_double * nkind)()
    cnt = (C.c_int * nkind)()
    with torch.cuda.stream(stream):
        m_work.copy_(m0)
        u_work.copy_(u0)
    torch.cuda.synchronize()
    ierr = L.w90g_profile_device(h.handle, C.c_void_p(m_work.data_ptr()), C.c_void_p(u_work.data_ptr()),
                                 args.profile_iters, msk, cnt)
    names = [L.w90g_profile_kernel_name(i).decode() for i in range(nkind)]
    per_kernel = {n: {"ms_total": msk[i], "launches": cnt[i],
                      "ms_avg": (msk[i] / cnt[i]) if cnt[i] else None} for i, n in enumerate(names)}
    exp_products = L.w90g_profile_exp_products(h.handle)
    fp64_peak = L.w90g_measure_fp64_peak()
    tot = sum(v["ms_total"] for v in per_kernel.values())
    for v in per_kernel.values():
        v["share"] = v["ms_total"] / tot if tot else None
    dom = max(("k_m_update", "k_exp_u", "k_grad"), key=lambda n: per_kernel[n]["ms_total"])
    avg = per_kernel[dom]["ms_avg"]
    useful_mupdate = 2 * 8.0 * W ** 3 * K * B          # two complex W^3 GEMMs per (k,b)
    wp = next(x for x in (8, 16, 32, 64, 128) if W <= x) if W <= 128 else 0
    # FP16 MMA work of one exact-sliced complex product on a 128-row tile (the dense FP16
    # and BF16 tensor rates are the same):
    # 28 digit pairs of (128 x 2WP x 2WP)
    tile_flops = 28 * 2.0 * 128 * (2 * wp) * (2 * wp)
    peak = float(MEASURED.get("bf16_tflops", 1900.0))
    peak_src = ("bf16_tflops of MEASURED_PEAKS.json (burst), of measured" if "bf16_tflops" in MEASURED
                else "1.9 PFLOP/s bf16 burst, of fallback")
    hbm_peak = float(MEASURED.get("hbm_gbs", 6800.0))
    if args.precision == "tensor" and dom in ("k_m_update", "k_exp_u"):
        if dom == "k_m_update":
            issued = tile_flops * 2 * K * -(-(B * wp) // 128)
            algo = useful_mupdate
            algo_bytes = 16.0 * K * W * W * (2 * B + 3)
            kname = "k_oz_mupdate (tcgen05, steps 1+2)"
        else:
            cnt_exp = max(per_kernel["k_exp_u"]["launches"], 1)
            prods = exp_products / cnt_exp / K           # products per matrix per launch
            issued = tile_flops * prods * K
            algo = prods * K * 8.0 * W ** 3
            algo_bytes = 16.0 * K * W * W * 3
            kname = "k_oz_exp (tcgen05)"
        sec = avg * 1e-3
        achieved = algo / sec / 1e12
        traffic = NCU_TRAFFIC.get((args.workload, dom))
        roof = {"bound": "tensor", "kernel": kname, "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                "peak_source": peak_src,
                "algorithmic_flops_per_launch": algo,
                "algorithmic_flops_note": "complex FP64-equivalent products (8 W^3 real FLOP each): "
                                          "2 per (k,b) for the M update, the exp chain's products for exp",
                "issued_mma": {"flops_per_launch": issued, "tflops": issued / sec / 1e12,
                               "frac": issued / sec / 1e12 / peak,
                               "note": "FP16 MMA FLOP actually issued: 28 digit pairs x 128 x 2WP x 2WP per tile"},
                "hbm": {"algorithmic_bytes_per_launch": algo_bytes, "gbs": algo_bytes / sec / 1e9,
                        "peak_gbs": hbm_peak, "frac": algo_bytes / sec / 1e9 / hbm_peak},
                "fp64_pipe": {"tflops": achieved, "fp64_pipe_peak_tflops": fp64_peak,
                              "ratio": achieved / fp64_peak if fp64_peak > 0 else None}}
    else:
        if dom == "k_exp_u":
            cnt_exp = max(per_kernel["k_exp_u"]["launches"], 1)
            flops = exp_products / cnt_exp * 8.0 * W ** 3
        elif dom == "k_grad":
            flops = 16.0 * K * B * W * W
        else:
            flops = useful_mupdate
        achieved = flops / (avg * 1e-3) / 1e12
        roof = {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak if fp64_peak > 0 else None,
                "traffic": NCU_TRAFFIC.get((args.workload + ":fp64", dom)),
                "peak_source": "FP64 FMA probe measured in this run (MEASURED_PEAKS.json has no FP64 figure)",
                "algorithmic_flops_per_launch": flops}
    roof["per_kernel"] = per_kernel
    roof["profiled_iterations"] = args.profile_iters

    # CPU baseline (oracle on host cores, bounded sample)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        procs = os.cpu_count() or 1
        spi = cpu_seconds_per_iteration(wl, args.cpu_iters, procs)
        # the CPU restatement's own iterations per converged solve (as the reference arm)
        cpu_niter = oracle_iterations(args.workload) or niter
        cpu = {"value": procs / (spi * cpu_niter), "unit": "solves/s", "cores": procs, "kind": "port",
               "sample": "%d iterations of the %s solve on each of %d cores (1 process per core, 1 BLAS "
                         "thread); solves/s = cores / (%.3f s/iter * %d iter/solve, the oracle's own converged "
                         "count)" % (args.cpu_iters, args.workload, procs, spi, cpu_niter)}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded tight-binding generator)",
            "config": bench_config(args.workload, wl, K, B, W, world),
            "iterations_per_solve": niter,
            "precision": ("tensor: M(k,b) = U^H M0 U (7x7-bit digits) and exp(sD), U dU (56-bit "
                          "digits) on tcgen05 FP16 MMAs with exact slicing (FP64-accurate); "
                          "gradient, Im ln M_nn, spread and controller on the FP64 pipe"
                          if args.precision == "tensor" else "fp64"),
            "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                           "max": float(max(lat_ms)), "note": "per converged solve, device-resident inputs"},
            "fp64_gpu": fp64,
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": bytes_m + bytes_u,
                    "d2h_bytes_per_step": bytes_m + bytes_u, "steps": len(e2e_t)},
            "gpu_launches": int(launches) * args.steps,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


# iterations per solve of the entangled workload as measured by the GPU arm (FP64 engine):
# (dis_main iterations, wann_main iterations)
KNOWN_ITERS = {"dis_fcc8_b48w32": (200, 3053)}

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the dominant
# kernel, from the committed ncu captures under profiles/ (name of the summary beside each)
NCU_TRAFFIC = {
    # profiles/k_oz_mupdate2_fcc10_w32.md: steps 1 + 2 of one M update
    ("fcc10_w32", "k_m_update"): 678.3e6,
    # profiles/k_oz_exp_fcc10_w32.md: one trial-step exp launch
    ("fcc10_w32", "k_exp_u"): 131.9e6,
}

if __name__ == "__main__":
    sys.exit(main())
