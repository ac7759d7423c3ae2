"""Autotuner keyed on num_wann: picks the kernel configuration of the iteration per width.

Candidates (engine options of the handle):

* ``fp64``    -- every product on the FP64 pipe (gpu_tensor = 0);
* ``tensor``  -- the tcgen05 M update and exp(sD) (gpu_tensor = 1), for num_wann <= 32 with
                 the pipelined warp-specialised M update (persistent, one CTA per SM, a ring
                 of 28 KB K-step stages; gpu_mupdate_pipe = 1);
* ``tensor_cta`` -- num_wann <= 32 only: the M update with one CTA per group and the whole
                 K extent of a tile staged at once (gpu_mupdate_pipe = 0);
* ``tensor_fp64exp`` -- the tcgen05 M update with exp(sD) and U dU on the FP64 pipe
                 (gpu_tensor_exp = 0), which wins for the smallest widths where a W x W
                 product fills little of a 128-row MMA tile;
* ``tensor_smemexp`` -- 16 < num_wann <= 32: the tensor exp with its six FP64 matrices in
                 shared memory, one CTA per SM (gpu_exp_smem = 1), instead of in L2 with two
                 CTAs per SM.

The padded tile width (8 / 16 / 32 / 64 / 128) follows from num_wann.  For each width the
tuner times a few iterations of a seeded tight-binding probe (sc lattice, 4x4x4 k-mesh,
nntot 6) in every candidate on the current GPU and keeps the fastest; all candidates
give the same minimum (the tensor ones bitwise the same M update).  Results are cached
per process; :func:`table` also writes them to a JSON file.  The batched and served forms
ask :func:`options` per problem.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import library as w90
from . import synth

_CACHE: dict[int, dict] = {}

CANDIDATES = {
    "fp64": dict(gpu_tensor=0),
    "tensor": dict(gpu_tensor=1, gpu_tensor_exp=1, gpu_mupdate_pipe=1),
    "tensor_cta": dict(gpu_tensor=1, gpu_tensor_exp=1, gpu_mupdate_pipe=0),
    "tensor_fp64exp": dict(gpu_tensor=1, gpu_tensor_exp=0, gpu_mupdate_pipe=1),
    "tensor_smemexp": dict(gpu_tensor=1, gpu_tensor_exp=1, gpu_mupdate_pipe=1, gpu_exp_smem=1),
}


def candidates_for(num_wann: int):
    if num_wann > 128:
        return ["fp64"]
    names = ["fp64", "tensor", "tensor_fp64exp"]
    if num_wann <= 32:
        names.append("tensor_cta")
    if 16 < num_wann <= 32:
        names.append("tensor_smemexp")
    return names


def _time_variant(p, opts: dict, iters: int) -> float:
    import torch

    W = p.num_wann
    h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_iter=iters,
                  iprint=0, **opts)
    m0 = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
    u0 = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
    w90.check(h, w90.w90_project_overlap_device(h, m0.data_ptr(), u0.data_ptr()), "autotune projection")
    best = float("inf")
    for _ in range(3):
        m, u = m0.clone(), u0.clone()
        torch.cuda.synchronize()
        t = time.perf_counter()
        w90.check(h, w90.w90_wannierise_device(h, m.data_ptr(), u.data_ptr()), "autotune run")
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t)
    return best


def tune(num_wann: int, iters: int = 12, mp=(4, 4, 4)) -> dict:
    """Time every candidate for this width; returns {'choice': name, 'options': {...},
    'tensor': 0/1, 'times': {name: seconds}}."""
    W = int(num_wann)
    if W in _CACHE:
        return _CACHE[W]
    names = candidates_for(W)
    times = {}
    if len(names) == 1:
        times = {names[0]: None}
        best = names[0]
    else:
        p = synth.make_problem(kind="sc", a=5.0, mp=mp, num_wann=W, rmax=1, eps=0.3, seed=12345)
        for n in names:
            times[n] = _time_variant(p, CANDIDATES[n], iters)
        best = min(names, key=lambda n: times[n])
    res = {"choice": best, "options": dict(CANDIDATES[best]), "tensor": CANDIDATES[best].get("gpu_tensor", 0),
           "times": times}
    _CACHE[W] = res
    return res


def options(num_wann: int) -> dict:
    """Engine options of the fastest candidate for this width."""
    return dict(tune(num_wann)["options"])


def choose_tensor(num_wann: int) -> int:
    return tune(num_wann)["tensor"]


def table(widths, path: str | None = None) -> dict:
    out = {int(w): tune(int(w)) for w in sorted(set(int(x) for x in widths))}
    if path:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
    return out
