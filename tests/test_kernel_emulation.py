"""The symmetry-adapted kernels (wannier90_gb300/csrc/k_sitesym.cu) and the FP64
iteration (k_fp64.cu) executed on the CPU.

tests/emu/ compiles the kernel sources with g++ against a host stand-in for
<cuda_runtime.h>: each CTA runs as 256 host threads (or fibers) with a barrier for
__syncthreads -- these kernels use block-level synchronisation only.  k_sitesym.cu is
compiled unchanged; k_fp64.cu gets two mechanical edits (dynamic shared memory, the
%globaltimer read).  The results are compared with the oracle's restatement of
src/sitesym.F90 and src/wannierise.F90 on the reference's example21 data (GaAs, 64 k, 10
irreducible, 24 symmetries), together with the host tables the C ABI builds
(sym_tables.cpp, compiled into the same harness).  The tensor-core kernels stay GPU-only.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "wannier90_gb300", "csrc")


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("emu") / "emu_sym.so")
    subprocess.run([gxx, "-std=c++20", "-O1", "-pthread", "-shared", "-fPIC", "-D__CUDACC__",
                    "-I" + os.path.join(HERE, "emu"), "-I" + CSRC, os.path.join(HERE, "emu", "emu_sym.cpp"),
                    os.path.join(CSRC, "sym_tables.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    head = [C.c_int] * 4 + [ip, ip, ip, dp, dp]
    lib.emu_sym_grad.argtypes = head + [dp, dp, dp]
    lib.emu_sym_dir.argtypes = head + [dp, dp, C.c_double, C.c_double]
    lib.emu_sym_u.argtypes = head + [C.c_double, dp, ip, C.c_int, C.c_int]
    for f in (lib.emu_sym_grad, lib.emu_sym_dir, lib.emu_sym_u):
        f.restype = C.c_int
    return lib


def _sym_args(d):
    """(nsym, nkirr, ik2ir, ir2ik, kptsym, d_wann, d_band) in the C ABI's Fortran layouts."""
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    kpt = i32(d["kptsym"].T)                                        # (nsym, nkirr) Fortran
    dw = np.ascontiguousarray(d["d_matrix_wann"].transpose(0, 1, 3, 2))   # (i, j, isym, ir) Fortran
    db = np.ascontiguousarray(d["d_matrix_band"].transpose(0, 1, 3, 2))
    return kpt.shape[1], kpt.shape[0], i32(d["ik2ir"]), i32(d["ir2ik"]), kpt, dw, db


def _ptr(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def _blocks(X):
    """[k, m, n] complex -> the kernels' column-major blocks (a writable copy)."""
    return np.ascontiguousarray(X.transpose(0, 2, 1)).astype(np.complex128)


def _unblocks(B):
    return np.ascontiguousarray(B.transpose(0, 2, 1))


def _call(lib, fn, d, W, K, *rest):
    nsym, nkirr, ik2ir, ir2ik, kpt, dw, db = _sym_args(d)
    args = [W, K, nsym, nkirr, _ptr(ik2ir, C.c_int), _ptr(ir2ik, C.c_int), _ptr(kpt, C.c_int),
            _ptr(dw.view(np.float64)), _ptr(db.view(np.float64))]
    return getattr(lib, fn)(*args, *rest)


def _random_kmat(K, W, seed, anti=False):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((K, W, W)) + 1j * rng.standard_normal((K, W, W))
    return X - np.conj(np.swapaxes(X, 1, 2)) if anti else X


def test_k_sym_grad_matches_oracle(emu):
    d = G.load("sitesym21")
    sym = G.sitesym(d)
    K, W = 64, 4
    Gm = _random_kmat(K, W, 1, anti=True)
    Dp = _random_kmat(K, W, 2, anti=True)
    gb, db_ = _blocks(Gm), _blocks(Dp)
    gpart = np.full(K * 2, 7.0)
    assert _call(emu, "emu_sym_grad", d, W, K, _ptr(gb.view(np.float64)), _ptr(db_.view(np.float64)),
                 _ptr(gpart)) == 0
    want = O.sitesym_symmetrize_gradient(O.sitesym_symmetrize_gradient(Gm, sym, 1), sym, 2)
    got = _unblocks(gb)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())
    # the CG partials: |G|^2 and Re<G, D_prev> over the whole mesh (zero off the irreducible k)
    g2 = gpart[0::2].sum()
    gd = gpart[1::2].sum()
    assert abs(g2 - float(np.vdot(want, want).real)) < 1e-11 * g2
    assert abs(gd - float(np.vdot(want, Dp).real)) < 1e-11 * max(1.0, abs(gd))
    irr = np.array([sym.irreducible(k) for k in range(K)])
    assert np.all(gpart[0::2][~irr] == 0) and np.all(gpart[1::2][~irr] == 0)


def test_k_sym_dir_matches_rotation(emu):
    d = G.load("sitesym21")
    sym = G.sitesym(d)
    K, W = 64, 4
    Gm = O.sitesym_symmetrize_gradient(O.sitesym_symmetrize_gradient(_random_kmat(K, W, 3, anti=True), sym, 1),
                                       sym, 2)
    Dp = _random_kmat(K, W, 4, anti=True)
    cg, cd = -1.0, 0.37
    gb, dbk = _blocks(Gm), _blocks(Dp)
    assert _call(emu, "emu_sym_dir", d, W, K, _ptr(gb.view(np.float64)), _ptr(dbk.view(np.float64)), cg, cd) == 0
    want = cg * Gm + cd * Dp
    done = np.zeros(K, dtype=bool)
    for ir in range(sym.nkirr):
        ik = sym.ir2ik[ir]
        done[ik] = True
        for isym in range(1, sym.nsym):
            k2 = sym.kptsym[isym, ir]
            if done[k2]:
                continue
            done[k2] = True
            Dm = sym.d_wann[ir, isym]
            want[k2] = Dm @ want[ik] @ Dm.conj().T
    np.testing.assert_allclose(_unblocks(dbk), want, rtol=0, atol=1e-13)


def test_k_sym_u_matches_oracle(emu):
    """The symmetry-adapted initial U from the Loewdin U of example21 (and from a Loewdin
    U pushed off the symmetric manifold, which takes several passes of the fixed point)."""
    d = G.load("sitesym21")
    sym = G.sitesym(d)
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(d["knobs"]["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U_l, _ = O.overlap_project(M, d["amn"], km["nnlist"])
    rng = np.random.default_rng(9)
    for U0, eps in ((U_l, 1e-9), (U_l @ np.linalg.qr(np.eye(4) + 0.05 * rng.standard_normal((4, 4)))[0], 1e-9)):
        sym.eps = eps
        want = O.sitesym_symmetrize_u_matrix(U0, sym)
        ub = _blocks(U0)
        status = np.zeros(sym.nkirr, dtype=np.int32)
        assert _call(emu, "emu_sym_u", d, 4, 64, eps, _ptr(ub.view(np.float64)), _ptr(status, C.c_int), 256, -1) == 0
        assert np.all(status == 0), status
        np.testing.assert_allclose(_unblocks(ub), want, rtol=0, atol=1e-10)


def test_k_sym_u_reports_no_convergence(emu):
    """symmetrize_eps below what 100 passes reach: status 1 (the engine's ierr -1).  One
    CTA (the Gamma point, whose little group is the whole group) on 32 emulated threads:
    100 passes of the fixed point take minutes at 256."""
    d = G.load("sitesym21")
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(d["knobs"]["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U_l, _ = O.overlap_project(M, d["amn"], km["nnlist"])
    ub = _blocks(U_l)
    nkirr = len(d["ir2ik"])
    status = np.full(nkirr, -7, dtype=np.int32)
    assert _call(emu, "emu_sym_u", d, 4, 64, 0.0, _ptr(ub.view(np.float64)), _ptr(status, C.c_int), 32, 0) == 0
    assert status[0] == 1


# ---------------------------------------------------------------------------
# the whole FP64 iteration with site symmetry (tests/emu/emu_iter.cpp)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def emu_iter(tmp_path_factory):
    """k_fp64.cu + k_sitesym.cu under the fiber emulation.  The copy of k_fp64.cu gets the
    two mechanical edits the host build needs: dynamic shared memory from emu_dyn_smem()
    and the %globaltimer read as 0."""
    import re
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    tmp = tmp_path_factory.mktemp("emu_iter")
    src = open(os.path.join(CSRC, "k_fp64.cu")).read()
    src, n_smem = re.subn(r"extern __shared__ double2 smem\[\];", "double2* smem = emu_dyn_smem<double2>();", src)
    src, n_timer = re.subn(r'asm volatile\("mov\.u64 %0, %%globaltimer;" : "=l"\((\w+)\)\);', r"\1 = 0;", src)
    assert n_smem >= 1 and n_timer == 2
    (tmp / "k_fp64_emu.cu").write_text(src)
    out = str(tmp / "emu_iter.so")
    subprocess.run([gxx, "-std=c++20", "-O1", "-shared", "-fPIC", "-D__CUDACC__", "-DEMU_FIBERS", "-I" + str(tmp),
                    "-I" + os.path.join(HERE, "emu"), "-I" + CSRC, os.path.join(HERE, "emu", "emu_iter.cpp"),
                    os.path.join(CSRC, "sym_tables.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    lib.emu_wann_main.argtypes = [C.c_int, C.c_int, C.c_int, ip, dp, dp, C.c_double, dp, dp, C.c_int, C.c_int,
                                  C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, ip, ip, ip, dp, dp, C.c_double,
                                  C.c_int, C.c_double, dp, dp, dp, ip]
    lib.emu_wann_main.restype = C.c_int
    return lib


def test_emulated_iteration_with_site_symmetry(emu_iter):
    """example21 through the engine's launch order on the emulated kernels: the Loewdin
    projection with the symmetry-adapted U (k_lowdin, k_sym_u, k_m_update), the initial
    spread, then four iterations (k_grad, k_sym_grad, k_ctrl_search, k_sym_dir, k_exp_u
    reading the rotated directions, k_m_update, the spread passes, the controller).  Every
    spread and RMS gradient against the oracle's symmetry-adapted run (1e-12) and the
    reference's printed lines (2e-10 A^2)."""
    d = G.load("sitesym21")
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(d["knobs"]["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    K, B, W, niter = len(d["kpt_latt"]), km["nntot"], 4, 4
    nsym, nkirr, ik2ir, ir2ik, kpt, dw, db = _sym_args(d)
    Mb = np.ascontiguousarray(M.transpose(0, 1, 3, 2)).astype(np.complex128)
    Ab = np.ascontiguousarray(d["amn"].transpose(0, 2, 1)).astype(np.complex128)
    nn = np.ascontiguousarray(km["nnlist"], dtype=np.int32)
    bk = np.ascontiguousarray(km["bk"], dtype=np.float64)
    wb = np.ascontiguousarray(km["wb"], dtype=np.float64)
    log = np.zeros((niter + 1) * 10)
    U = np.zeros(K * W * W, dtype=np.complex128)
    status = np.zeros(2, dtype=np.int32)
    rows = emu_iter.emu_wann_main(W, K, B, _ptr(nn, C.c_int), _ptr(bk), _ptr(wb), km["wbtot"],
                                  _ptr(Mb.view(np.float64)), _ptr(Ab.view(np.float64)), niter, 5, -1, 1e-10, 2.0, nsym,
                                  nkirr, _ptr(ik2ir, C.c_int), _ptr(ir2ik, C.c_int), _ptr(kpt, C.c_int),
                                  _ptr(dw.view(np.float64)), _ptr(db.view(np.float64)),
                                  float(d["knobs"]["symmetrize_eps"]), 0, 0.0, None, _ptr(log),
                                  _ptr(U.view(np.float64)), _ptr(status, C.c_int))
    assert rows == niter + 1 and status[0] == 0 and status[1] == 0
    log = log.reshape(-1, 10)[:rows]
    sym = G.sitesym(d)
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"], sitesym=sym)
    r = O.wann_main(M0, U0, km, O.WannControl(num_iter=niter), sitesym=sym)
    for row, x, printed in zip(log, [r.initial] + r.iters, d["conv"]):
        assert int(row[0]) == x.iter == int(printed[0])
        assert abs(row[3] - x.spread.om_tot) < 1e-12, (x.iter, row[3], x.spread.om_tot)
        assert abs(row[2] - x.rms_grad) <= 1e-10 * max(1.0, x.rms_grad)
        assert abs(row[3] - printed[3]) < 2e-10
    np.testing.assert_allclose(_unblocks(U.reshape(K, W, W)), r.U, atol=1e-12)


# ---------------------------------------------------------------------------
# the symmetry-adapted disentanglement (tests/emu/emu_dis.cpp)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def emu_dis(tmp_path_factory):
    """The kernel part of dis.cu (everything before dis_run) under the fiber emulation; the
    copy reads its dynamic shared memory from emu_dyn_smem()."""
    import re
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    tmp = tmp_path_factory.mktemp("emu_dis")
    src = open(os.path.join(CSRC, "dis.cu")).read()
    src = src[:src.index("int dis_run(")] + "}  // namespace w90g\n"
    src, n_smem = re.subn(r"extern __shared__ double2 (\w+)\[\];", r"double2* \1 = emu_dyn_smem<double2>();", src)
    assert n_smem == 2
    (tmp / "dis_emu.cu").write_text(src)
    out = str(tmp / "emu_dis.so")
    subprocess.run([gxx, "-std=c++20", "-O1", "-shared", "-fPIC", "-D__CUDACC__", "-DEMU_FIBERS", "-I" + str(tmp),
                    "-I" + os.path.join(HERE, "emu"), "-I" + CSRC, os.path.join(HERE, "emu", "emu_dis.cpp"),
                    os.path.join(CSRC, "sym_tables.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    lib.emu_dis_sym.argtypes = ([C.c_int] * 4 + [ip, dp, C.c_double, dp, dp, dp, C.c_int, C.c_double, C.c_double,
                                C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, ip, ip, ip, dp, dp, C.c_double,
                                C.c_int, dp, dp, dp, dp, ip])
    lib.emu_dis_sym.restype = C.c_int
    return lib


def test_emulated_symmetry_adapted_disentanglement(emu_dis):
    """testw90_disentanglement_sawfs (H3S, 20 -> 12, 3 irreducible of 8 k, 48 symmetries)
    through dis_run's symmetry-adapted launch order on the emulated kernels (k_dis_project,
    k_dis_sym_u, k_dis_z, k_dis_sym_z, k_dis_sym_step, k_dis_findu, k_dis_rotate): the
    first two iterations' Omega_I(i-1), Omega_I(i) against the oracle (1e-10) and the
    printed lines (1e-8), U_opt U0 and M0 against the oracle (1e-9; U_opt and U0 alone
    are fixed only up to a rotation that cancels there).  32 emulated threads per CTA:
    the kernels take any power-of-two block size, and the nested fixed points of the
    constrained extraction take minutes at 256."""
    d = G.load("sitesym_dis")
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    nb, W, K, B = int(d["num_bands"]), int(kn["num_wann"]), len(d["kpt_latt"]), km["nntot"]
    dc = G.dis_control(d)
    dc.num_iter = 2
    nsym, nkirr, ik2ir, ir2ik, kpt, dw, db = _sym_args(d)
    Mf = np.ascontiguousarray(M.transpose(0, 1, 3, 2)).astype(np.complex128)
    Af = np.ascontiguousarray(d["amn"].transpose(0, 2, 1)).astype(np.complex128)
    eig = np.ascontiguousarray(d["eig"])
    nn = np.ascontiguousarray(km["nnlist"], dtype=np.int32)
    wb = np.ascontiguousarray(km["wb"])
    log = np.zeros(3 * dc.num_iter)
    U0 = np.zeros(K * W * W, dtype=np.complex128)
    M0 = np.zeros(K * B * W * W, dtype=np.complex128)
    Uo = np.zeros(K * nb * W, dtype=np.complex128)
    status = np.zeros(1, dtype=np.int32)
    rows = emu_dis.emu_dis_sym(nb, W, K, B, _ptr(nn, C.c_int), _ptr(wb), km["wbtot"], _ptr(eig),
                               _ptr(Mf.view(np.float64)), _ptr(Af.view(np.float64)), dc.num_iter, dc.mix_ratio,
                               dc.conv_tol, dc.conv_window, dc.win_min, dc.win_max, nsym, nkirr, _ptr(ik2ir, C.c_int),
                               _ptr(ir2ik, C.c_int), _ptr(kpt, C.c_int), _ptr(dw.view(np.float64)),
                               _ptr(db.view(np.float64)), float(kn["symmetrize_eps"]), 32, _ptr(log),
                               _ptr(U0.view(np.float64)), _ptr(M0.view(np.float64)), _ptr(Uo.view(np.float64)),
                               _ptr(status, C.c_int))
    assert rows == 2 and status[0] == 0
    U0o, M0o, Uoo, omi, recs = O.dis_main(M, d["amn"], d["eig"], km, W, dc, sitesym=G.sitesym(d))
    for row, r, printed in zip(log.reshape(-1, 3), recs, d["dis"]):
        assert abs(row[1] - r.omega_i_prev) < 1e-10 and abs(row[2] - r.omega_i) < 1e-10
        assert abs(row[1] - printed[1]) < 1e-8 and abs(row[2] - printed[2]) < 1e-8
    U0e = U0.reshape(K, W, W).transpose(0, 2, 1)
    Uoe = Uo.reshape(K, W, nb).transpose(0, 2, 1)
    for k in range(K):
        np.testing.assert_allclose(Uoe[k] @ U0e[k], Uoo[k] @ U0o[k], atol=1e-9)
    np.testing.assert_allclose(M0.reshape(K, B, W, W).transpose(0, 1, 3, 2), M0o, atol=1e-9)


@pytest.mark.parametrize("name", G.DIS_CASES)
def test_emulated_disentanglement_with_frozen_states(emu_dis, name):
    """The reference's disentanglement cases (silicon, copper, basic2, GaAs issue 192: 64 k,
    outer and frozen windows) through dis_run's plain launch order on the emulated kernels
    (k_dis_project, k_dis_froz, k_dis_z, k_dis_step, k_dis_gauge, k_dis_findu,
    k_dis_rotate): every Omega_I line against the oracle (1e-10) and the printed lines
    (1e-8), U_opt U and M0 against the oracle (1e-9).  32 emulated threads per CTA."""
    d = G.load(name)
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    nb, W, K, B = int(d["num_bands"]), int(kn["num_wann"]), len(d["kpt_latt"]), km["nntot"]
    dc = G.dis_control(d)
    lib = emu_dis
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    lib.emu_dis_plain.argtypes = ([C.c_int] * 4 + [ip, dp, C.c_double, dp, dp, dp, C.c_int, C.c_double, C.c_double,
                                  C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int, dp, dp, dp,
                                  dp, ip])
    lib.emu_dis_plain.restype = C.c_int
    Mf = np.ascontiguousarray(M.transpose(0, 1, 3, 2)).astype(np.complex128)
    Af = np.ascontiguousarray(d["amn"].transpose(0, 2, 1)).astype(np.complex128)
    eig = np.ascontiguousarray(d["eig"])
    nn = np.ascontiguousarray(km["nnlist"], dtype=np.int32)
    wb = np.ascontiguousarray(km["wb"])
    log = np.zeros(3 * dc.num_iter)
    U0 = np.zeros(K * W * W, dtype=np.complex128)
    M0 = np.zeros(K * B * W * W, dtype=np.complex128)
    Uo = np.zeros(K * nb * W, dtype=np.complex128)
    status = np.zeros(1, dtype=np.int32)
    rows = lib.emu_dis_plain(nb, W, K, B, _ptr(nn, C.c_int), _ptr(wb), km["wbtot"], _ptr(eig),
                             _ptr(Mf.view(np.float64)), _ptr(Af.view(np.float64)), dc.num_iter, dc.mix_ratio,
                             dc.conv_tol, dc.conv_window, dc.win_min, dc.win_max, int(dc.frozen_states), dc.froz_min,
                             dc.froz_max, 32, _ptr(log), _ptr(U0.view(np.float64)), _ptr(M0.view(np.float64)),
                             _ptr(Uo.view(np.float64)), _ptr(status, C.c_int))
    assert status[0] == 0
    U0o, M0o, Uoo, omi, recs = O.dis_main(M, d["amn"], d["eig"], km, W, dc)
    assert rows == len(recs) == len(d["dis"])
    for row, r, printed in zip(log.reshape(-1, 3), recs, d["dis"]):
        assert abs(row[1] - r.omega_i_prev) < 1e-10 and abs(row[2] - r.omega_i) < 1e-10
        assert abs(row[1] - printed[1]) < 1e-8 and abs(row[2] - printed[2]) < 1e-8
    U0e = U0.reshape(K, W, W).transpose(0, 2, 1)
    Uoe = Uo.reshape(K, W, nb).transpose(0, 2, 1)
    for k in range(K):
        np.testing.assert_allclose(Uoe[k] @ U0e[k], Uoo[k] @ U0o[k], atol=1e-9)
    np.testing.assert_allclose(M0.reshape(K, B, W, W).transpose(0, 1, 3, 2), M0o, atol=1e-9)


def test_emulated_iteration_with_selective_localisation(emu_iter):
    """testw90_example26 (GaAs, slwf_num = 1 with its centre constrained, lambda = 1) through
    the engine's launch order on the emulated FP64 kernels: the SLWF spread passes and the
    factored SLWF gradient.  Every spread, O_IOD and Omega_nu against the oracle (1e-9
    relative) and the printed lines of the first iterations (2e-10 A^2, 1.2e-9 from the third on,
    where the printed run itself is sensitive at 1e-10)."""
    d = G.load("slwf26")
    kn = d["knobs"]
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(kn["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    K, B, W, niter = len(d["kpt_latt"]), km["nntot"], 4, 3
    ctl, sl = G.slwf(d)
    Mb = np.ascontiguousarray(M.transpose(0, 1, 3, 2)).astype(np.complex128)
    Ab = np.ascontiguousarray(d["amn"].transpose(0, 2, 1)).astype(np.complex128)
    nn = np.ascontiguousarray(km["nnlist"], dtype=np.int32)
    bk = np.ascontiguousarray(km["bk"], dtype=np.float64)
    wb = np.ascontiguousarray(km["wb"], dtype=np.float64)
    cen = np.ascontiguousarray(sl.centres, dtype=np.float64)       # [3][W] Cartesian
    log = np.zeros((niter + 1) * 10)
    U = np.zeros(K * W * W, dtype=np.complex128)
    status = np.zeros(2, dtype=np.int32)
    z = np.zeros(1, dtype=np.int32)
    rows = emu_iter.emu_wann_main(W, K, B, _ptr(nn, C.c_int), _ptr(bk), _ptr(wb), km["wbtot"],
                                  _ptr(Mb.view(np.float64)), _ptr(Ab.view(np.float64)), niter, ctl.num_cg_steps,
                                  ctl.conv_window, ctl.conv_tol, ctl.trial_step, 0, 0, _ptr(z, C.c_int),
                                  _ptr(z, C.c_int), _ptr(z, C.c_int), None, None, 0.0, sl.num, sl.lam, _ptr(cen),
                                  _ptr(log), _ptr(U.view(np.float64)), _ptr(status, C.c_int))
    assert rows == niter + 1 and status[1] == 0
    log = log.reshape(-1, 10)[:rows]
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"])
    r = O.wann_main(M0, U0, km, O.WannControl(num_iter=niter), slwf=sl)
    for row, x, printed in zip(log, [r.initial] + r.iters, d["conv"]):
        sp = x.spread
        # summation order differs from the oracle's and the run amplifies roundoff (a 1e-16
        # perturbation of M0 moves it by 1e-10 from the third iteration): 1e-9 relative to
        # each term, as on the GPU
        for got, want in ((row[3], sp.om_tot), (row[5], sp.om_iod + sp.om_nu), (row[9], sp.om_nu), (row[4], sp.om_d)):
            assert abs(got - want) <= 1e-9 * max(1.0, abs(want), abs(sp.om_iod)) + 1e-11, (x.iter, got, want)
        assert abs(row[3] - printed[3]) < 2e-10 + 1e-9 * (x.iter >= 3)
