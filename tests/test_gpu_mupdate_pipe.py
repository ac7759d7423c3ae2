"""The pipelined M-update kernel (num_wann <= 32, k_mupdate2.cu) against the
one-CTA-per-group kernel: the same digit arithmetic on a different schedule, so every
iteration's spread, U and M must agree bit for bit -- stand-alone, batched with uneven
widths, and for widths that leave partial 128-row tiles and padded columns."""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests.engine_helpers import run_engine
from wannier90_gb300 import library as w90
from wannier90_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,W,mp", [("sc", 1, (3, 3, 3)), ("sc", 5, (3, 3, 3)), ("fcc", 8, (3, 3, 3)),
                                       ("sc", 13, (2, 2, 3)), ("fcc", 16, (3, 3, 3)), ("sc", 20, (2, 2, 2)),
                                       ("fcc", 32, (3, 3, 3)), ("bcc", 27, (2, 2, 2))])
def test_pipelined_equals_classic_bitwise(kind, W, mp):
    p = synth.make_problem(kind=kind, a=5.0, mp=mp, num_wann=W, rmax=1, eps=0.3, seed=11)
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    ctl = O.WannControl(num_iter=25)
    a = run_engine(p.real_lattice, p.kpoints, M, A, ctl, W, extra={"gpu_tensor": 1, "gpu_mupdate_pipe": 0})
    b = run_engine(p.real_lattice, p.kpoints, M, A, ctl, W, extra={"gpu_tensor": 1, "gpu_mupdate_pipe": 1})
    assert a["ierr"] == 0 and b["ierr"] == 0, (a["err"], b["err"])
    np.testing.assert_array_equal(b["log"][:, :8], a["log"][:, :8])
    np.testing.assert_array_equal(b["U"], a["U"])
    np.testing.assert_array_equal(b["M"], a["M"])


def test_pipelined_batch_uneven_widths_equals_standalone():
    torch = pytest.importorskip("torch")
    shapes = [(4, (3, 3, 3)), (7, (2, 2, 2)), (12, (3, 3, 3)), (16, (2, 2, 3)), (24, (2, 2, 2)), (32, (2, 2, 2))]
    hs, ms, us, alone = [], [], [], []
    for i, (W, mp) in enumerate(shapes):
        p = synth.make_problem(kind="sc", a=4.0 + 0.3 * i, mp=mp, num_wann=W, rmax=1, eps=0.3, seed=40 + i)
        h = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=W, num_iter=30, iprint=0,
                      gpu_tensor=1)
        m = torch.from_numpy(p.m.reshape(-1, order="F").view(np.float64).copy()).cuda()
        u = torch.from_numpy(p.a.reshape(-1, order="F").view(np.float64).copy()).cuda()
        assert w90.w90_project_overlap_device(h, m.data_ptr(), u.data_ptr()) == 0, h.last_error()
        m1, u1 = m.clone(), u.clone()
        torch.cuda.synchronize()
        assert w90.w90_wannierise_device(h, m1.data_ptr(), u1.data_ptr()) == 0, h.last_error()
        torch.cuda.synchronize()
        alone.append((m1.cpu().numpy(), u1.cpu().numpy(), w90.w90_get_log(h, 31).copy()))
        hs.append(h)
        ms.append(m)
        us.append(u)
    torch.cuda.synchronize()
    ierr = w90.w90_wannierise_batch_device(hs, [x.data_ptr() for x in ms], [x.data_ptr() for x in us])
    torch.cuda.synchronize()
    assert all(e == 0 for e in ierr), [h.last_error() for h in hs]
    for i, h in enumerate(hs):
        np.testing.assert_array_equal(w90.w90_get_log(h, 31)[:, :8], alone[i][2][:, :8])
        np.testing.assert_array_equal(ms[i].cpu().numpy(), alone[i][0])
        np.testing.assert_array_equal(us[i].cpu().numpy(), alone[i][1])


@pytest.mark.parametrize("W", [20, 32])
def test_exp_matrices_in_shared_memory_bitwise(W):
    """The tensor exp with its FP64 matrices in shared memory (gpu_exp_smem = 1) is the same
    arithmetic as with them in L2: bitwise the same trajectory."""
    p = synth.make_problem(kind="fcc", a=5.0, mp=(3, 3, 3), num_wann=W, rmax=1, eps=0.3, seed=13)
    M = synth.to_math_m(p.m)
    A = synth.to_math_u(p.a)
    ctl = O.WannControl(num_iter=20)
    a = run_engine(p.real_lattice, p.kpoints, M, A, ctl, W, extra={"gpu_tensor": 1, "gpu_exp_smem": 0})
    b = run_engine(p.real_lattice, p.kpoints, M, A, ctl, W, extra={"gpu_tensor": 1, "gpu_exp_smem": 1})
    assert a["ierr"] == 0 and b["ierr"] == 0, (a["err"], b["err"])
    np.testing.assert_array_equal(b["log"][:, :8], a["log"][:, :8])
    np.testing.assert_array_equal(b["U"], a["U"])
    np.testing.assert_array_equal(b["M"], a["M"])
