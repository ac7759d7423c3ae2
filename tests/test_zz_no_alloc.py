"""The allocation-free Loewdin projection against the allocating one.

w90g_project_overlap_noalloc serves callers that cannot call cudaMalloc (their device
memory belongs to another allocator); it keeps its scratch in a file-scope device array.
This file runs last so that a failure here leaves every other test already run; it must
pass alone in a fresh process too (the first call performs the per-device set-up).
"""
import ctypes as C

import numpy as np
import pytest

from wannier90_gb300 import library as w90
from wannier90_gb300 import synth
from wannier90_gb300._native import lib


def _nnkp(h, K):
    nnkp = w90.w90_get_nnkp(h, K)            # (K, B) Fortran order = [b][k] in memory
    return np.asfortranarray(nnkp, dtype=np.int32)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [dict(kind="sc", a=5.0, mp=(4, 4, 4), num_wann=8, rmax=2, eps=0.3),
                                 dict(kind="fcc", a=6.0, mp=(3, 3, 3), num_wann=32, rmax=1, eps=0.4)])
def test_noalloc_projection_matches_allocating_entry_point_twice(cfg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = lib()
    p = synth.make_problem(**cfg, seed=3)
    W, K, B = p.num_wann, len(p.kpoints), p.nntot
    h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, iprint=0)
    m_in = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
    u_in = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
    # existing (allocating) entry point
    m_ref, u_ref = m_in.clone(), u_in.clone()
    torch.cuda.synchronize()
    assert w90.w90_project_overlap_device(h, m_ref.data_ptr(), u_ref.data_ptr()) == 0, h.last_error()
    torch.cuda.synchronize()
    nnkp = _nnkp(h, K)
    for _ in range(2):
        m, u = m_in.clone(), u_in.clone()
        torch.cuda.synchronize()
        rc = L.w90g_project_overlap_noalloc(W, K, B, nnkp.ctypes.data_as(C.POINTER(C.c_int)),
                                            C.c_void_p(m.data_ptr()), C.c_void_p(u.data_ptr()), None)
        assert rc == 0
        torch.cuda.synchronize()
        np.testing.assert_allclose(u.cpu().numpy(), u_ref.cpu().numpy(), atol=1e-11, rtol=0)
        np.testing.assert_allclose(m.cpu().numpy(), m_ref.cpu().numpy(), atol=1e-11, rtol=0)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = lib()
    nnkp = np.ones(8, dtype=np.int32)
    dummy = C.c_void_p(16)      # never dereferenced: the size check comes first
    ip = nnkp.ctypes.data_as(C.POINTER(C.c_int))
    assert L.w90g_project_overlap_noalloc(33, 1, 8, ip, dummy, dummy, None) == 5
    assert L.w90g_project_overlap_noalloc(8, 4097, 1, ip, dummy, dummy, None) == 5
    assert L.w90g_project_overlap_noalloc(8, 1000, 9, ip, dummy, dummy, None) == 5
    # an nnkp entry that names no k-point would be a gather index outside U on the GPU
    for bad in (0, 3, -1):
        table = np.ones(8, dtype=np.int32)
        table[5] = bad
        tp = table.ctypes.data_as(C.POINTER(C.c_int))
        assert L.w90g_project_overlap_noalloc(8, 2, 4, tp, dummy, dummy, None) == 5
