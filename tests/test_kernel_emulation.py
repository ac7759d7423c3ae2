"""The symmetry-adapted kernels (wannier90_gb300/csrc/k_sitesym.cu) executed on the CPU.

tests/emu/ compiles the kernel source unchanged with g++ against a host stand-in for
<cuda_runtime.h>: each CTA runs as 256 host threads with a barrier for __syncthreads
(these kernels use block-level synchronisation only).  The results are compared with
the oracle's restatement of src/sitesym.F90 on the reference's example21 symmetry data
(GaAs, 64 k, 10 irreducible, 24 symmetries), together with the host tables the C ABI
builds (sym_tables.cpp, compiled into the same harness).
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
