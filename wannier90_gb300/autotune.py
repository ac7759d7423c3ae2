"""Autotuner keyed on num_wann: picks the M-update variant for each width.

Variants: the tensor-core M update at padded tile width 8 / 16 / 32 / 64 / 128 and the
FP64 shared-/global-memory kernels.  For each W the tuner times a few iterations of a
seeded tight-binding probe (sc lattice, 4x4x4 k-mesh, nntot 6) in both variants on the
current GPU and keeps the faster.  Results are cached per process and, optionally, in a
JSON file.  The batched and served forms ask :func:`choose_tensor` per problem.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import library as w90
from . import synth

_CACHE: dict[int, dict] = {}


def _time_variant(p, tensor: int, iters: int) -> float:
    import torch

    W = p.num_wann
    h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_iter=iters,
                  iprint=0, gpu_tensor=tensor)
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
    """Time both variants for this width; returns {'tensor': 0/1, 't_fp64': s, 't_tensor': s}."""
    W = int(num_wann)
    if W in _CACHE:
        return _CACHE[W]
    if W > 128:
        res = {"tensor": 0, "t_fp64": None, "t_tensor": None, "reason": "W > 128: FP64 kernels only"}
    else:
        p = synth.make_problem(kind="sc", a=5.0, mp=mp, num_wann=W, rmax=1, eps=0.3, seed=12345)
        t0 = _time_variant(p, 0, iters)
        t1 = _time_variant(p, 1, iters)
        res = {"tensor": int(t1 < t0), "t_fp64": t0, "t_tensor": t1}
    _CACHE[W] = res
    return res


def choose_tensor(num_wann: int) -> int:
    return tune(num_wann)["tensor"]


def table(widths, path: str | None = None) -> dict:
    out = {int(w): tune(int(w)) for w in sorted(set(int(x) for x in widths))}
    if path:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
    return out
