"""Host-side checks of the disentanglement entry (no GPU needed): the dis_* keywords of
cinput_setopt and the window errors of dis_windows, which cdisentangle reports before it
touches the device, with the same messages as the oracle (src/disentangle.F90:851-1171,
src/readwrite.F90:651-682, src/wannier90_readwrite.F90:824-854)."""
import numpy as np
import pytest

from oracle import w90_oracle as O
from wannier90_gb300 import library as w90


def _handle(nb=6, W=4, **opts):
    c = w90.w90_create()
    kp = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])
    w90.w90_set_option(c, "kpoints", kp)
    w90.w90_set_option(c, "num_kpts", 2)
    w90.w90_set_option(c, "num_wann", W)
    w90.w90_set_option(c, "num_bands", nb)
    w90.w90_set_option(c, "unit_cell_cart", np.eye(3) * 4.0)
    w90.w90_set_option(c, "iprint", 0)
    for k, v in opts.items():
        w90.w90_set_option(c, k, v)
    return c, w90.w90_input_setopt(c)


@pytest.mark.parametrize("opts,msg", [
    (dict(dis_mix_ratio=0.0), "dis_mix_ratio must be greater than 0.0"),
    (dict(dis_mix_ratio=1.5), "dis_mix_ratio must be greater than 0.0"),
    (dict(dis_num_iter=-1), "dis_num_iter must be positive"),
    (dict(dis_conv_tol=-1e-3), "dis_conv_tol must be positive"),
    (dict(dis_conv_window=-2), "dis_conv_window must be positive"),
    (dict(dis_win_min=5.0, dis_win_max=1.0), "check disentanglement windows"),
    (dict(dis_froz_min=1.0), "found dis_froz_min but not dis_froz_max"),
    (dict(dis_froz_min=3.0, dis_froz_max=1.0), "check disentanglement frozen windows"),
])
def test_dis_keyword_errors(opts, msg):
    c, ierr = _handle(**opts)
    assert ierr == 5
    assert msg in c.last_error()


def test_num_bands_below_num_wann():
    c, ierr = _handle(nb=3, W=4)
    assert ierr == 5 and "num_bands must be greater than or equal to num_wann" in c.last_error()


def _call(c, nb, W, K, eig):
    m = np.zeros((nb, nb, w90.w90_get_nn(c), K), dtype=np.complex128, order="F")
    a = np.zeros((nb, W, K), dtype=np.complex128, order="F")
    u = np.zeros((W, W, K), dtype=np.complex128, order="F")
    w90.w90_set_m_local(c, m)
    w90.w90_set_u_matrix(c, u)
    w90.w90_set_u_opt(c, a)
    w90.w90_set_eigval(c, np.asfortranarray(eig.T))
    return w90.w90_disentangle(c)


EIG = np.array([[-3.0, -1.0, 0.0, 1.0, 2.0, 6.0], [-2.5, -1.5, 0.5, 1.5, 2.5, 7.0]])


@pytest.mark.parametrize("opts,msg", [
    (dict(dis_win_min=-0.5, dis_win_max=1.2), "fewer states than number of target WFs"),
    (dict(dis_win_min=100.0, dis_win_max=200.0), "outer energy window contains no eigenvalues"),
    (dict(dis_froz_max=2.2), "More states in the frozen window than target WFs"),
])
def test_dis_window_errors_match_oracle(opts, msg):
    c, ierr = _handle(**opts)
    assert ierr == 0
    assert _call(c, 6, 4, 2, EIG) == 1
    assert msg in c.last_error()
    dc = O.DisControl(win_min=opts.get("dis_win_min", -1e300), win_max=opts.get("dis_win_max", 1e300),
                      froz_max=opts.get("dis_froz_max", 1e300), frozen_states="dis_froz_max" in opts)
    with pytest.raises(RuntimeError, match=msg):
        O.dis_windows(EIG, 4, dc)


def test_dis_band_limit_and_missing_pointers():
    c, ierr = _handle(nb=65, W=4)
    assert ierr == 0
    eig = np.tile(np.linspace(-5, 5, 65), (2, 1))
    assert _call(c, 65, 4, 2, eig) == 5
    assert "num_bands <= 64" in c.last_error()
    c, ierr = _handle()
    assert w90.w90_disentangle(c) == 1
    assert "m_matrix_local not associated" in c.last_error()
