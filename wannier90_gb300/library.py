"""Python mirror of Wannier90's library interface for the wannierisation path.

The reference exposes ``w90_library`` (src/library_interface.F90) to Python through
f90wrap (wrap/Makefile.serial:52-71): a ``lib_common_type`` object plus module
functions ``w90_set_option``, ``w90_input_setopt``, ``w90_get_nn``, ``w90_get_nnkp``,
``w90_set_m_local``, ``w90_set_u_matrix``, ``w90_set_u_opt``, ``w90_set_eigval``,
``w90_disentangle``, ``w90_project_overlap``, ``w90_wannierise``, ``w90_get_centres``,
``w90_get_spreads``.  This module provides the
same names and argument meaning on top of the engine's C ABI
(include/wannier90_gb300.h).  Arrays are NumPy arrays in Fortran order, exactly the
reference's shapes:

    m_matrix  complex128 (num_bands, num_bands, nntot, num_kpts)
    u_matrix  complex128 (num_wann, num_wann, num_kpts)
    u_opt     complex128 (num_bands, num_wann, num_kpts)

Status: functions return ``ierr`` like the Fortran library (0 ok, >0 error, <0 warning).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import lib


class W90Error(RuntimeError):
    def __init__(self, ierr, msg):
        super().__init__("ierr=%d: %s" % (ierr, msg))
        self.ierr = ierr


def _cplx(a, shape=None):
    a = np.asarray(a)
    if a.dtype != np.complex128 or not a.flags.f_contiguous:
        raise TypeError("expected a Fortran-ordered complex128 array")
    if shape is not None and a.shape != tuple(shape):
        raise ValueError("array shape %s, expected %s" % (a.shape, tuple(shape)))
    return a


class LibCommon:
    """Counterpart of ``lib_common_type`` (src/library_interface.F90:27-99)."""

    def __init__(self):
        self._L = lib()
        self._h = self._L.w90_create()
        self._keep = {}      # arrays whose pointers the library holds
        self.num_wann = self.num_bands = self.num_kpts = 0
        self.nntot = 0

    def __del__(self):
        try:
            if self._h:
                self._L.w90_delete(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def last_error(self):
        return self._L.w90g_last_error(self._h).decode()


def w90_create():
    return LibCommon()


def w90_set_option(common: LibCommon, keyword: str, value):
    """w90_set_option (src/library_interface.F90:667-808): int, bool, real, 1-D int,
    2-D real (kpoints: shape (num_kpts, 3); unit_cell_cart: rows a_1..a_3 in Angstrom)."""
    L, h, key = common._L, common._h, keyword.encode()
    if isinstance(value, (bool, np.bool_)):
        L.cset_option_int(h, key, int(bool(value)))
    elif isinstance(value, (int, np.integer)):
        L.cset_option_int(h, key, int(value))
    elif isinstance(value, (float, np.floating)):
        L.cset_option_float(h, key, float(value))
    else:
        a = np.asarray(value)
        if a.dtype.kind in "iu":
            a = np.ascontiguousarray(a, dtype=np.int32).reshape(-1)
            if a.size == 3 and keyword.lower() == "mp_grid":
                L.cset_option_int3(h, key, a.ctypes.data_as(C.POINTER(C.c_int)))
            else:
                L.cset_option_intx(h, key, a.ctypes.data_as(C.POINTER(C.c_int)), a.size)
        else:
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.ndim == 1:
                a = a.reshape(1, -1)
            if a.shape == (3, 3) and keyword.lower() == "unit_cell_cart":
                L.cset_option_float33(h, key, a.ctypes.data_as(C.POINTER(C.c_double)))
            else:
                L.cset_option_floatxy(h, key, a.ctypes.data_as(C.POINTER(C.c_double)),
                                      a.shape[0], a.shape[1])


def w90_input_setopt(common: LibCommon, seedname: str = "wannier", comm: int = 0) -> int:
    """w90_input_setopt (src/library_interface.F90:161-292): process options, build the k-mesh."""
    ierr = C.c_int(0)
    common._L.cinput_setopt(common._h, seedname.encode(), C.byref(ierr), int(comm))
    if ierr.value == 0:
        nn = C.c_int(0)
        common._L.cget_nn(common._h, C.byref(nn))
        common.nntot = nn.value
    return ierr.value


def w90_input_reader(common: LibCommon) -> int:
    """w90_input_reader (src/library_interface.F90:294-360): the remaining keywords of
    seedname.win after w90_input_setopt (seedname as given there)."""
    ierr = C.c_int(0)
    common._L.cinput_reader(common._h, C.byref(ierr))
    if ierr.value == 0:
        nn = C.c_int(0)
        common._L.cget_nn(common._h, C.byref(nn))
        common.nntot = nn.value
    return ierr.value


def w90_input_reader_special(common: LibCommon, seedname: str) -> int:
    """The whole input, system included, from seedname.win (cinput_reader_special)."""
    ierr = C.c_int(0)
    common._L.cinput_reader_special(common._h, seedname.encode(), C.byref(ierr))
    if ierr.value == 0:
        nn = C.c_int(0)
        common._L.cget_nn(common._h, C.byref(nn))
        common.nntot = nn.value
    return ierr.value


def w90_set_kpoint_distribution(common: LibCommon, dist):
    """set_kpoint_distribution (src/wannier_prog.F90:798-820): only all-zero (one rank)
    is accepted; anything else makes the next work call return 5."""
    d = np.ascontiguousarray(dist, dtype=np.int32)
    common._keep["dist"] = d
    common._L.cset_kpoint_distribution(common._h, d.ctypes.data_as(C.POINTER(C.c_int)))


def w90_set_parallel_comms(common: LibCommon, comm: int):
    common._L.cset_parallel_comms(common._h, int(comm))


def w90_set_a_matrix(common: LibCommon, a):
    """The projections A (num_bands, num_wann, num_kpts): filled by w90_overlaps, the start
    of w90_project_overlap (isolated) / w90_disentangle (entangled)."""
    common._keep["a"] = _cplx(a)
    common._L.cset_a_matrix(common._h, common._keep["a"].ctypes.data)


def w90_overlaps(common: LibCommon) -> int:
    """overlaps (src/wannier_prog.F90:478-537): seedname.mmn into m, seedname.amn into
    the projections."""
    ierr = C.c_int(0)
    common._L.coverlaps(common._h, C.byref(ierr))
    return ierr.value


def w90_write_chkpt(common: LibCommon, label: str = "postwann") -> int:
    """write_chkpt (src/wannier_prog.F90:575-700): seedname.chk; returns 0, or 1 with
    the message in last_error()."""
    common._L.cchkpt(common._h, label.encode())
    return 1 if common.last_error() else 0


def w90_get_nn(common: LibCommon) -> int:
    nn = C.c_int(0)
    common._L.cget_nn(common._h, C.byref(nn))
    return nn.value


def w90_get_nnkp(common: LibCommon, num_kpts: int) -> np.ndarray:
    """nnlist as (num_kpts, nntot) int32, 1-based (w90_get_nnkp)."""
    B = w90_get_nn(common)
    out = np.zeros((num_kpts, B), dtype=np.int32, order="F")
    common._L.cget_nnkp(common._h, out.ctypes.data_as(C.POINTER(C.c_int)))
    return out


def w90_get_gkpb(common: LibCommon, num_kpts: int) -> np.ndarray:
    """nncell as (3, num_kpts, nntot) int32 (w90_get_gkpb)."""
    B = w90_get_nn(common)
    out = np.zeros((3, num_kpts, B), dtype=np.int32, order="F")
    common._L.cget_gkpb(common._h, out.ctypes.data_as(C.POINTER(C.c_int)))
    return out


def w90_set_m_local(common: LibCommon, m):
    common._keep["m"] = _cplx(m)
    common._L.cset_m_local(common._h, common._keep["m"].ctypes.data)


def w90_set_u_matrix(common: LibCommon, u):
    common._keep["u"] = _cplx(u)
    common._L.cset_u_matrix(common._h, common._keep["u"].ctypes.data)


def w90_set_u_opt(common: LibCommon, u_opt):
    common._keep["u_opt"] = _cplx(u_opt)
    common._L.cset_u_opt(common._h, common._keep["u_opt"].ctypes.data)


def w90_set_eigval(common: LibCommon, eigval):
    e = np.asarray(eigval, dtype=np.float64)
    if not e.flags.f_contiguous:
        raise TypeError("expected a Fortran-ordered float64 array")
    common._keep["eig"] = e
    common._L.cset_eigval(common._h, e.ctypes.data)


def w90_project_overlap(common: LibCommon) -> int:
    """Loewdin initialisation (src/library_interface.F90:422-462) on the GPU."""
    ierr = C.c_int(0)
    common._L.cproject_overlap(common._h, C.byref(ierr))
    return ierr.value


def w90_disentangle(common: LibCommon) -> int:
    """dis_main + setup_m_loc (src/library_interface.F90:362-420) on the GPU.  Reads
    m_local (raw overlaps), u_opt (projections) and eigval; writes u_opt (optimal
    subspace), u_matrix (internal_find_u) and the top-left num_wann x num_wann of every
    m_local block."""
    ierr = C.c_int(0)
    common._L.cdisentangle(common._h, C.byref(ierr))
    return ierr.value


def w90_disentangle_device(common: LibCommon, m_ptr: int, u_opt_ptr: int, u_ptr: int, eig_ptr: int) -> int:
    """w90_disentangle with m_local, u_opt, u_matrix and eigval resident in device memory."""
    ierr = C.c_int(0)
    common._L.w90g_disentangle_device(common._h, C.c_void_p(m_ptr), C.c_void_p(u_opt_ptr), C.c_void_p(u_ptr),
                                      C.c_void_p(eig_ptr), C.byref(ierr))
    return ierr.value


def w90_profile_dis_device(common: LibCommon, m_ptr: int, u_opt_ptr: int, u_ptr: int, eig_ptr: int):
    """Disentanglement on device buffers with per-kernel CUDA-event timing:
    (ierr, {kernel: (ms_total, launches)})."""
    L = common._L
    names = []
    while L.w90g_dis_kernel_name(len(names)):
        names.append(L.w90g_dis_kernel_name(len(names)).decode())
    ms = np.zeros(len(names), dtype=np.float64)
    counts = np.zeros(len(names), dtype=np.int32)
    ierr = L.w90g_profile_dis_device(common._h, C.c_void_p(m_ptr), C.c_void_p(u_opt_ptr), C.c_void_p(u_ptr),
                                     C.c_void_p(eig_ptr), ms.ctypes.data_as(C.POINTER(C.c_double)),
                                     counts.ctypes.data_as(C.POINTER(C.c_int)))
    return ierr, {nm: (float(ms[i]), int(counts[i])) for i, nm in enumerate(names)}


def w90_get_dis_log(common: LibCommon, max_rows: int) -> np.ndarray:
    """Omega_I iteration record of the last w90_disentangle: columns iter,
    Omega_I(i-1), Omega_I(i), delta (frac.), seconds."""
    out = np.zeros((max_rows, 5), dtype=np.float64)
    n = common._L.w90g_get_dis_log(common._h, out.ctypes.data_as(C.POINTER(C.c_double)), max_rows)
    return out[:n]


def w90_set_sitesym(common: LibCommon, dmn: dict) -> int:
    """The symmetry data of the symmetry-adapted mode (sitesym_read's content; see
    w90io.read_dmn for the keys).  Returns the ierr."""
    i32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.int32).reshape(-1, order="F"))
    c128 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.complex128).reshape(-1, order="F"))
    ik2ir, ir2ik, kptsym = i32(dmn["ik2ir"]), i32(dmn["ir2ik"]), i32(dmn["kptsym"])
    dw, db = c128(dmn["d_matrix_wann"]), c128(dmn["d_matrix_band"])
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    return common._L.w90g_set_sitesym(common._h, int(dmn["num_bands"]), int(dmn["nsymmetry"]), int(dmn["nkptirr"]),
                                      int(dmn["num_kpts"]), ip(ik2ir), ip(ir2ik), ip(kptsym), dp(dw), dp(db))


def w90_get_dis_windows(common: LibCommon, num_kpts: int):
    """(ndimwin[nk], nfirstwin[nk] 0-based) of the last w90_disentangle's outer window."""
    nd = np.zeros(num_kpts, dtype=np.int32)
    nf = np.zeros(num_kpts, dtype=np.int32)
    common._L.w90g_get_dis_windows(common._h, nd.ctypes.data_as(C.POINTER(C.c_int)),
                                   nf.ctypes.data_as(C.POINTER(C.c_int)))
    return nd, nf


def w90_get_dis_info(common: LibCommon) -> dict:
    """Final Omega_I (omega%invariant), convergence flag, iteration count and the most
    Jacobi sweeps one Z eigenproblem took."""
    out = np.zeros(4, dtype=np.float64)
    common._L.w90g_get_dis_info(common._h, out.ctypes.data_as(C.POINTER(C.c_double)))
    return {"omega_invariant": float(out[0]), "converged": bool(out[1]), "iterations": int(out[2]),
            "max_sweeps": int(out[3])}


def w90_wannierise(common: LibCommon) -> int:
    """wann_main (src/library_interface.F90:464-530) on the GPU; U and M updated in place."""
    ierr = C.c_int(0)
    common._L.cwannierise(common._h, C.byref(ierr))
    return ierr.value


def w90_wannierise_device(common: LibCommon, m_ptr: int, u_ptr: int) -> int:
    """wann_main with M and U already resident in device memory (raw CUDA pointers)."""
    ierr = C.c_int(0)
    common._L.w90g_wannierise_device(common._h, C.c_void_p(m_ptr), C.c_void_p(u_ptr), C.byref(ierr))
    return ierr.value


def w90_project_overlap_device(common: LibCommon, m_ptr: int, u_ptr: int) -> int:
    ierr = C.c_int(0)
    common._L.w90g_project_overlap_device(common._h, C.c_void_p(m_ptr), C.c_void_p(u_ptr), C.byref(ierr))
    return ierr.value


def w90_wannierise_batch_device(commons, m_ptrs, u_ptrs):
    """Solve several problems (one LibCommon each) together on the GPU; device buffers.
    Returns the list of per-problem ierr."""
    n = len(commons)
    L = commons[0]._L
    hs = (C.c_void_p * n)(*[c._h for c in commons])
    ms = (C.c_void_p * n)(*[C.c_void_p(p) for p in m_ptrs])
    us = (C.c_void_p * n)(*[C.c_void_p(p) for p in u_ptrs])
    ierr = (C.c_int * n)()
    L.w90g_wannierise_batch_device(hs, n, ms, us, ierr)
    return list(ierr)


class Server:
    """Serving loop (continuous batching) over the C ABI's w90g_server_*: jobs are
    admitted first-in first-out by an HBM budget and a slot count, run concurrently on
    the GPU until they converge, and are collected with :meth:`poll`."""

    def __init__(self, hbm_budget_bytes: float, max_active: int = 32, chunk_iters: int = 8):
        self._L = lib()
        self._s = self._L.w90g_server_create(float(hbm_budget_bytes), int(max_active), int(chunk_iters))
        if not self._s:
            raise W90Error(2, "w90g_server_create failed")
        self._keep = {}

    def submit(self, common: LibCommon, m_ptr: int, u_ptr: int, tag: int) -> int:
        """Queue a solve of ``common`` on device buffers (projected M0 / U0, updated in place)."""
        self._keep[int(tag)] = common
        return self._L.w90g_server_submit(self._s, common.handle, C.c_void_p(m_ptr), C.c_void_p(u_ptr),
                                          C.c_longlong(int(tag)))

    def poll(self, max_jobs: int = 1024):
        """Completed jobs: list of (tag, ierr, t_submit, t_admit, t_done) on the server clock."""
        tags = (C.c_longlong * max_jobs)()
        ierr = (C.c_int * max_jobs)()
        ts, ta, td = ((C.c_double * max_jobs)() for _ in range(3))
        n = self._L.w90g_server_poll(self._s, tags, ierr, ts, ta, td, max_jobs)
        out = [(int(tags[i]), int(ierr[i]), ts[i], ta[i], td[i]) for i in range(n)]
        for t in out:
            self._keep.pop(t[0], None)
        return out

    def pending(self) -> int:
        return int(self._L.w90g_server_pending(self._s))

    def drain(self):
        self._L.w90g_server_drain(self._s)

    def now(self) -> float:
        return float(self._L.w90g_server_now(self._s))

    def stats(self) -> dict:
        out = np.zeros(4, dtype=np.float64)
        self._L.w90g_server_stats(self._s, out.ctypes.data_as(C.POINTER(C.c_double)))
        return {"peak_active": int(out[0]), "peak_bytes": float(out[1]), "jobs_done": int(out[2]),
                "iterations_done": int(out[3])}

    def close(self):
        if self._s:
            self._L.w90g_server_delete(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def w90_get_centres(common: LibCommon, num_wann: int) -> np.ndarray:
    """Wannier centres as (3, num_wann) (Fortran layout, Angstrom)."""
    out = np.zeros((3, num_wann), dtype=np.float64, order="F")
    common._L.cget_centres(common._h, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def w90_get_spreads(common: LibCommon, num_wann: int) -> np.ndarray:
    out = np.zeros(num_wann, dtype=np.float64)
    common._L.cget_spreads(common._h, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def w90_get_omega(common: LibCommon) -> np.ndarray:
    """(Omega_I, Omega_D, Omega_OD, Omega_total)."""
    out = np.zeros(4, dtype=np.float64)
    common._L.cget_omega(common._h, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def w90_get_log(common: LibCommon, max_rows: int) -> np.ndarray:
    """Per-iteration record: columns iter, dOmega, rms_grad, Omega, Omega_D, Omega_OD,
    lquad, alphamin, device time (ns), Omega_nu.  With selective localisation Omega_OD
    holds Omega_IOD + Omega_nu (the reference's printed O_IOD) and Omega_nu the centre
    constraint's term; Omega_nu is 0 otherwise."""
    out = np.zeros((max_rows, 10), dtype=np.float64)
    n = common._L.w90g_get_log(common._h, out.ctypes.data_as(C.POINTER(C.c_double)), max_rows)
    return out[:n]


def w90_get_log_centres(common: LibCommon, max_rows: int, num_wann: int) -> np.ndarray:
    out = np.zeros((max_rows, 4 * num_wann), dtype=np.float64)
    n = common._L.w90g_get_log_centres(common._h, out.ctypes.data_as(C.POINTER(C.c_double)), max_rows)
    return out[:n].reshape(n, 4, num_wann)


def ws_vectors(real_lattice, mp_grid, ws_search_size=(2, 2, 2), ws_distance_tol=1.0e-5):
    """Wigner-Seitz points of the Born-von Karman supercell (host): (irvec[n,3], ndegen[n])."""
    L = lib()
    a = np.ascontiguousarray(real_lattice, dtype=np.float64)
    mp = np.ascontiguousarray(mp_grid, dtype=np.int32)
    ss = np.ascontiguousarray(np.broadcast_to(ws_search_size, (3,)), dtype=np.int32)
    args = (a.ctypes.data_as(C.POINTER(C.c_double)), mp.ctypes.data_as(C.POINTER(C.c_int)),
            ss.ctypes.data_as(C.POINTER(C.c_int)), float(ws_distance_tol))
    n = L.w90g_ws_vectors(*args, None, None, 0)
    if n < 0:
        raise W90Error(1, "hamiltonian_wigner_seitz: error in finding Wigner-Seitz points")
    irvec = np.zeros((n, 3), dtype=np.int32)
    ndegen = np.zeros(n, dtype=np.int32)
    L.w90g_ws_vectors(*args, irvec.ctypes.data_as(C.POINTER(C.c_int)),
                      ndegen.ctypes.data_as(C.POINTER(C.c_int)), n)
    return irvec, ndegen


def w90_set_stream(common: LibCommon, cuda_stream: int):
    common._L.w90g_set_stream(common._h, C.c_void_p(cuda_stream))


def w90_kernel_launches(common: LibCommon) -> int:
    return int(common._L.w90g_kernel_launches(common._h))


def check(common: LibCommon, ierr: int, what: str):
    if ierr > 0:
        raise W90Error(ierr, "%s: %s" % (what, common.last_error()))
    return ierr


def setup(*, kpoints, unit_cell_cart, num_wann, num_bands=None, mp_grid=None, seedname="wannier",
          **options) -> LibCommon:
    """wannier_setup-style helper (test-suite/libv2-demo/*/wannier.cc:5-34)."""
    c = w90_create()
    kp = np.asarray(kpoints, dtype=np.float64)
    w90_set_option(c, "kpoints", kp)
    w90_set_option(c, "num_kpts", int(kp.shape[0]))
    w90_set_option(c, "num_wann", int(num_wann))
    w90_set_option(c, "num_bands", int(num_bands or num_wann))
    w90_set_option(c, "unit_cell_cart", np.asarray(unit_cell_cart, dtype=np.float64))
    if mp_grid is not None:
        w90_set_option(c, "mp_grid", np.asarray(mp_grid, dtype=np.int32))
    for k, v in options.items():
        w90_set_option(c, k, v)
    check(c, w90_input_setopt(c, seedname), "w90_input_setopt")
    c.num_wann = int(num_wann)
    c.num_bands = int(num_bands or num_wann)
    c.num_kpts = int(kp.shape[0])
    return c
