"""Batched form: uneven problems solved together give exactly their stand-alone results."""
import numpy as np
import pytest

from oracle import w90_oracle as O
from wannier90_gb300 import library as w90
from wannier90_gb300 import synth

pytestmark = pytest.mark.gpu

SHAPES = [  # (W, mp, tensor)
    (4, (3, 3, 3), 1), (8, (2, 2, 2), 1), (13, (3, 3, 3), 1), (20, (2, 2, 2), 1),
    (33, (2, 2, 2), 1), (8, (3, 3, 3), 0), (6, (4, 4, 4), 1),
]


def _problem(i, W, mp):
    return synth.make_problem(kind="sc", a=3.0 + 0.5 * i, mp=mp, num_wann=W, rmax=1, eps=0.3, seed=100 + i)


def _device(p):
    torch = pytest.importorskip("torch")
    m = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
    u = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
    return m, u


def test_batch_members_equal_standalone_runs():
    torch = pytest.importorskip("torch")
    probs, handles, ms, us, alone = [], [], [], [], []
    for i, (W, mp, tensor) in enumerate(SHAPES):
        p = _problem(i, W, mp)
        h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_iter=15, iprint=0,
                      gpu_tensor=tensor)
        m, u = _device(p)
        assert w90.w90_project_overlap_device(h, m.data_ptr(), u.data_ptr()) == 0, h.last_error()
        torch.cuda.synchronize()
        # stand-alone solve on copies
        m1, u1 = m.clone(), u.clone()
        assert w90.w90_wannierise_device(h, m1.data_ptr(), u1.data_ptr()) == 0, h.last_error()
        torch.cuda.synchronize()
        alone.append((m1.cpu().numpy(), u1.cpu().numpy(), w90.w90_get_log(h, 16).copy()))
        probs.append(p)
        handles.append(h)
        ms.append(m)
        us.append(u)
    ierr = w90.w90_wannierise_batch_device(handles, [m.data_ptr() for m in ms], [u.data_ptr() for u in us])
    torch.cuda.synchronize()
    assert ierr == [0] * len(SHAPES), [h.last_error() for h in handles]
    for i, h in enumerate(handles):
        m_a, u_a, log_a = alone[i]
        log_b = w90.w90_get_log(h, 16)
        assert log_b.shape == log_a.shape, (i, log_b.shape)
        np.testing.assert_array_equal(log_b[:, :8], log_a[:, :8])   # same trajectory, bit for bit
        np.testing.assert_array_equal(ms[i].cpu().numpy(), m_a)
        np.testing.assert_array_equal(us[i].cpu().numpy(), u_a)


def test_batch_member_matches_oracle():
    torch = pytest.importorskip("torch")
    handles, ms, us, probs = [], [], [], []
    for i, (W, mp, tensor) in enumerate(SHAPES[:4]):
        p = _problem(i, W, mp)
        h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_iter=6, iprint=0,
                      gpu_tensor=tensor)
        m, u = _device(p)
        assert w90.w90_project_overlap_device(h, m.data_ptr(), u.data_ptr()) == 0
        handles.append(h)
        ms.append(m)
        us.append(u)
        probs.append(p)
    torch.cuda.synchronize()
    assert w90.w90_wannierise_batch_device(handles, [m.data_ptr() for m in ms], [u.data_ptr() for u in us]) == [0] * 4
    for p, h in zip(probs, handles):
        km = O.kmesh_get(p.real_lattice, p.kpoints)
        U0, M0 = O.overlap_project(synth.to_math_m(p.m), synth.to_math_u(p.a), km["nnlist"])
        r = O.wann_main(M0, U0, km, O.WannControl(num_iter=6))
        log = w90.w90_get_log(h, 7)
        for row, it in zip(log[:3], [r.initial] + r.iters[:2]):
            assert abs(row[3] - it.spread.om_tot) <= 1e-8 * abs(it.spread.om_tot) + 2e-10
