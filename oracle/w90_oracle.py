"""CPU oracle for the MLWF spread-minimisation path (test infrastructure only).

This module is a plain NumPy/SciPy restatement of Wannier90's ``wann_main``
path and of the set-up steps that feed it.  It exists so that the tests, the
``smoke()`` entry and the ``cpu_baseline`` leg of ``bench.py`` can check and
time the CUDA engine.  Nothing in the product (``wannier90_gb300``) imports it;
the engine never falls back to it.

Every function cites the reference routine it follows (paths are relative to
the Wannier90 source tree).  Arithmetic is FP64 / complex128 throughout, as in
the reference (``src/constants.F90`` ``dp``).  LAPACK ``zheev`` and ``zgesvd``
are called through ``scipy.linalg.lapack`` (same LAPACK routines the reference
links; bundled OpenBLAS build).

Parity pin: ``tests/test_oracle_golden.py`` runs this oracle on the reference's
own regression inputs (Pb, GaAs, diamond, basic1, the preconditioned GaAs runs,
selective localisation (example26), site symmetry (example21), four
disentanglement cases and a guiding-centre checkpoint; fixtures under
``tests/golden/``) and compares every printed ``<-- CONV`` / ``<-- DIS`` line,
the final centres/spreads and the b-vector tables with the reference's
benchmark outputs.

Array conventions (oracle-internal, "math" layout):
  M[k, b, m, n]  = M_mn^{(k,b)}     complex128  (K, B, W, W)
  U[k, m, n]     = U_mn^{(k)}       complex128  (K, W, W)
  bk[k, b, :]    = b-vector (Cartesian, 1/Angstrom)
  nnlist[k, b]   = 0-based index of k+b
The reference stores the same data Fortran column-major, i.e. ``m_matrix(m,n,b,k)``;
``from_fortran_m``/``to_fortran_m`` convert.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.linalg import lapack

# src/constants.F90:109 (CODATA 2006, the default build)
BOHR_ANGSTROM = 0.52917720859
TWOPI = 2.0 * math.pi
EPS_DP = np.finfo(np.float64).eps      # Fortran epsilon(1.0_dp)
TINY_DP = np.finfo(np.float64).tiny    # Fortran tiny(1.0_dp)
EPS5 = 1.0e-5
EPS6 = 1.0e-6
EPS8 = 1.0e-8


# ---------------------------------------------------------------------------
# layout helpers
# ---------------------------------------------------------------------------
def from_fortran_m(flat, W, B, K):
    """Fortran ``m_matrix(W,W,B,K)`` buffer -> M[k,b,m,n]."""
    a = np.asarray(flat).reshape(K, B, W, W)  # [k][b][n][m]
    return np.ascontiguousarray(a.transpose(0, 1, 3, 2))


def to_fortran_m(M):
    return np.ascontiguousarray(M.transpose(0, 1, 3, 2)).reshape(-1)


def from_fortran_u(flat, W, K):
    a = np.asarray(flat).reshape(K, W, W)
    return np.ascontiguousarray(a.transpose(0, 2, 1))


def to_fortran_u(U):
    return np.ascontiguousarray(U.transpose(0, 2, 1)).reshape(-1)


# ---------------------------------------------------------------------------
# lattice helpers  (src/utility.F90:233-336, :426-446)
# ---------------------------------------------------------------------------
def recip_lattice(real_lattice):
    """utility_recip_lattice_base: rows b_i = 2*pi (a_j x a_k)/det."""
    a = np.asarray(real_lattice, dtype=np.float64)
    cof = np.empty((3, 3))
    cof[0] = np.cross(a[1], a[2])
    cof[1] = np.cross(a[2], a[0])
    cof[2] = np.cross(a[0], a[1])
    det = float(np.dot(a[0], cof[0]))
    return TWOPI * cof / det, abs(det)


def frac_to_cart(frac, lattice):
    return np.asarray(frac) @ np.asarray(lattice)


# ---------------------------------------------------------------------------
# k-mesh  (src/kmesh.F90:61-740, :984-1104, :1107-1432)
# ---------------------------------------------------------------------------
NSUPCELL = 5  # src/kmesh.F90:55


def _supercell_sort(recip):
    """kmesh_supercell_sort (src/kmesh.F90:984-1038) incl. internal_maxloc tie rule."""
    n = NSUPCELL
    lmn = [(0, 0, 0)]
    for l in range(-n, n + 1):
        for m in range(-n, n + 1):
            for nn in range(-n, n + 1):
                if l == 0 and m == 0 and nn == 0:
                    continue
                lmn.append((l, m, nn))
    lmn = np.array(lmn, dtype=np.int64)
    dist = np.sqrt(((lmn @ recip) ** 2).sum(axis=1))
    N = len(lmn)
    out = np.empty_like(lmn)
    d = dist.copy()
    alive = np.ones(N, dtype=bool)
    for pos in range(N - 1, -1, -1):
        mx = np.max(np.where(alive, d, -1.0))
        # lowest index among (near-)degenerate maxima  (internal_maxloc, :1866-1883)
        g = int(np.argmax(np.where(alive, d, -1.0)))
        cand = np.where(alive & (np.abs(d - d[g]) < EPS8))[0]
        idx = int(cand.min()) if len(cand) else g
        del mx
        out[pos] = lmn[idx]
        alive[idx] = False
        d[idx] = -1.0
    return out


def _get_bvectors(kpt_cart, recip, lmn, shell_dist, multi, tol):
    """kmesh_get_bvectors (src/kmesh.F90:1041-1104) for origin k-point 1."""
    bvec = []
    for cell in lmn:
        vkpp2 = cell @ recip
        for nkp2 in range(len(kpt_cart)):
            vkpp = vkpp2 + kpt_cart[nkp2]
            dist = np.sqrt(((kpt_cart[0] - vkpp) ** 2).sum())
            if shell_dist * (1.0 - tol) <= dist <= shell_dist * (1.0 + tol):
                bvec.append(vkpp - kpt_cart[0])
            if len(bvec) == multi:
                return np.array(bvec)
    return np.array(bvec)


def kmesh_get(real_lattice, kpt_latt, search_shells=36, tol=1.0e-6):
    """Restatement of kmesh_get (src/kmesh.F90:61-740), automatic shells only.

    Returns dict(nntot, nnlist[K,B] (0-based), nncell[K,B,3], wb[B], bk[K,B,3],
    wbtot, shells, dnn, multi).
    """
    recip, _ = recip_lattice(real_lattice)
    lmn = _supercell_sort(recip)
    kpt_latt = np.asarray(kpt_latt, dtype=np.float64)
    K = len(kpt_latt)
    kpt_cart = kpt_latt @ recip
    eta = 99999999.0

    # shell distances / multiplicities (src/kmesh.F90:129-158); the reference scans
    # |k + G| over all k-points and cells, keeping the smallest distance above the
    # previous shell and counting its multiplicity
    cell_cart = lmn @ recip
    alld = np.sqrt(((kpt_cart[:, None, :] + cell_cart[None, :, :]) ** 2).sum(axis=2)).reshape(-1)
    dnn, multi = [], []
    dnn0 = 0.0
    for _ in range(search_shells):
        cand = alld[(alld > tol) & (alld > dnn0 + tol)]
        if len(cand) == 0:
            dnn.append(eta)
            multi.append(0)
            dnn0 = eta
            continue
        dnn1 = float(cand.min())
        counter = int(((cand > dnn1 - tol) & (cand < dnn1 + tol)).sum())
        dnn.append(dnn1)
        multi.append(counter)
        dnn0 = dnn1
    # kmesh_shell_automatic (src/kmesh.F90:1107-1432)
    target = np.array([1.0, 1.0, 1.0, 0.0, 0.0, 0.0])
    shell_list, shell_bvecs = [], []
    bweight = None
    for shell in range(search_shells):
        bv = _get_bvectors(kpt_cart, recip, lmn, dnn[shell], multi[shell], tol)
        lpar = False
        for b1 in bv:
            for prev in shell_bvecs:
                for b2 in prev:
                    delta = np.dot(b1, b2) / math.sqrt(np.dot(b1, b1) * np.dot(b2, b2))
                    if abs(abs(delta) - 1.0) < EPS6:
                        lpar = True
        if lpar:
            continue
        shell_list.append(shell)
        shell_bvecs.append(bv)
        ns = len(shell_list)
        amat = np.zeros((6, ns))
        for s, b in enumerate(shell_bvecs):
            amat[0, s] = (b[:, 0] * b[:, 0]).sum()
            amat[1, s] = (b[:, 1] * b[:, 1]).sum()
            amat[2, s] = (b[:, 2] * b[:, 2]).sum()
            amat[3, s] = (b[:, 0] * b[:, 1]).sum()
            amat[4, s] = (b[:, 1] * b[:, 2]).sum()
            amat[5, s] = (b[:, 2] * b[:, 0]).sum()
        u, sv, vt = np.linalg.svd(amat, full_matrices=True)
        if np.any(np.abs(sv) < EPS5):
            if ns == 1:
                raise RuntimeError("kmesh_shell_automatic: very small singular value")
            shell_list.pop()
            shell_bvecs.pop()
            continue
        w = vt.T @ ((u.T @ target)[:ns] / sv)
        b1sat = True
        for i in range(3):
            for j in range(i, 3):
                delta = sum(w[s] * (b[:, i] * b[:, j]).sum() for s, b in enumerate(shell_bvecs))
                if i == j and abs(delta - 1.0) > tol:
                    b1sat = False
                if i != j and abs(delta) > tol:
                    b1sat = False
        if b1sat:
            bweight = w
            break
    if bweight is None:
        raise RuntimeError("Unable to satisfy B1 with the searched shells")

    nntot = sum(multi[s] for s in shell_list)
    wb = np.concatenate([[bweight[i]] * multi[s] for i, s in enumerate(shell_list)])

    # neighbour lists (src/kmesh.F90:362-390): cells in sorted order, k2 ascending,
    # stop at the shell multiplicity (vectorised over k2 within one cell)
    nnlist = np.zeros((K, nntot), dtype=np.int64)
    nncell = np.zeros((K, nntot, 3), dtype=np.int64)
    bk = np.zeros((K, nntot, 3))
    for nkp in range(K):
        nnx = 0
        for s in shell_list:
            cnt = 0
            lo, hi = dnn[s] * (1 - tol), dnn[s] * (1 + tol)
            for ci, cell in enumerate(lmn):
                vkpp = cell_cart[ci] + kpt_cart                  # (K,3)
                dist = np.sqrt(((kpt_cart[nkp] - vkpp) ** 2).sum(axis=1))
                hits = np.nonzero((dist >= lo) & (dist <= hi))[0]
                for nkp2 in hits:
                    nnlist[nkp, nnx] = nkp2
                    nncell[nkp, nnx] = cell
                    bk[nkp, nnx] = vkpp[nkp2] - kpt_cart[nkp]
                    nnx += 1
                    cnt += 1
                    if cnt == multi[s]:
                        break
                if cnt == multi[s]:
                    break
    wbtot = float(wb.sum())
    # b directions without inversion partners, from the first k-point (:505-528), and
    # the index of each direction in every k-point's neighbour list (:561-577)
    compar = lambda a, b: (float(((a - b) ** 2).sum()) < EPS8, float(((a + b) ** 2).sum()) < EPS8)
    bka = []
    for nn in range(nntot):
        if not any(compar(v, bk[0, nn])[1] for v in bka):
            bka.append(bk[0, nn].copy())
    nnh = nntot // 2
    if len(bka) != nnh:
        raise RuntimeError("Did not find right number of bk directions")
    bka = np.array(bka)
    neigh = np.zeros((K, nnh), dtype=np.int64)
    for nkp in range(K):
        for na in range(nnh):
            hit = -1
            for nn in range(nntot):
                if compar(bka[na], bk[nkp, nn])[0]:
                    hit = nn
            if hit < 0:
                raise RuntimeError("kmesh_get: failed to find neighbours for this kpoint")
            neigh[nkp, na] = hit
    return dict(nntot=nntot, nnlist=nnlist, nncell=nncell, wb=wb, bk=bk, wbtot=wbtot,
                shells=[s + 1 for s in shell_list], dnn=np.array(dnn), multi=np.array(multi),
                nnh=nnh, bka=bka, neigh=neigh)


# ---------------------------------------------------------------------------
# overlap_project (Loewdin)  (src/overlap.F90:758-952)
# ---------------------------------------------------------------------------
def overlap_project(M, A, nnlist, sitesym=None):
    """U(k) = Z V^dagger from zgesvd of A(k); M(k,b) <- U(k)^dag M(k,b) U(k+b).
    ``sitesym``: U is made symmetry-adapted first (src/overlap.F90:901-905)."""
    K, B, W, _ = M.shape
    U = np.empty((K, W, W), dtype=np.complex128)
    for k in range(K):
        z, s, vh, info = lapack.zgesvd(A[k], full_matrices=1, compute_uv=1)[:4]
        if info != 0:
            raise RuntimeError("zgesvd failed in overlap_project")
        U[k] = z @ vh
        chk = U[k].conj().T @ U[k]
        if np.max(np.abs(chk - np.eye(W))) > EPS5:
            raise RuntimeError("unitarity of initial U")
    if sitesym is not None:
        U = sitesym_symmetrize_u_matrix(U, sitesym)
    Mout = np.conj(U)[:, None].transpose(0, 1, 3, 2) @ M @ U[nnlist]
    return U, Mout


# ---------------------------------------------------------------------------
# symmetry-adapted mode (site_symmetry = T): src/sitesym.F90
# ---------------------------------------------------------------------------
@dataclass
class Sitesym:
    """sitesym_type (src/wannier90_types.F90:260-268) with 0-based indices:
    ik2ir[k] (irreducible index of k), ir2ik[ir], kptsym[isym, ir] (index of R_isym k_ir),
    d_wann[ir, isym] = D(R, k_ir) (W x W), d_band[ir, isym] = d(R, k_ir) (nb x nb),
    eps = symmetrize_eps (default 1e-3)."""
    ik2ir: np.ndarray
    ir2ik: np.ndarray
    kptsym: np.ndarray
    d_wann: np.ndarray
    d_band: np.ndarray
    eps: float = 1.0e-3

    @property
    def nsym(self):
        return self.kptsym.shape[0]

    @property
    def nkirr(self):
        return len(self.ir2ik)

    def irreducible(self, k):
        return self.ir2ik[self.ik2ir[k]] == k


def _orthogonalize_u(u, n):
    """orthogonalize_u (src/sitesym.F90:500-548): the polar factor of u[:n] through
    zgesvd('A','A'): u = L[:, :m] R."""
    m = u.shape[1]
    L, sv, R, info = lapack.zgesvd(np.ascontiguousarray(u[:n, :]), full_matrices=1, compute_uv=1)[:4]
    if info != 0:
        raise RuntimeError("ERROR: IN ZGESVD IN orthogonalize_u")
    out = np.zeros_like(u)
    out[:n, :] = L[:, :m] @ R
    return out


def _symmetrize_ukirr(u, ir, sym, n=None, d_band=None):
    """symmetrize_ukirr (src/sitesym.F90:392-497): average d^+(R,k) u D(R,k) over the
    little group {R: Rk = k} and orthonormalise, until sum |ngk I - sum u^+ d^+ u D| <
    symmetrize_eps (100 passes at most)."""
    W = u.shape[1]
    ntmp = u.shape[0] if n is None else n
    db = sym.d_band if d_band is None else d_band
    ik = sym.ir2ik[ir]
    little = [isym for isym in range(sym.nsym) if sym.kptsym[isym, ir] == ik]
    ngk = len(little)
    if ngk == 1:
        return _orthogonalize_u(u, ntmp)
    for it in range(1, 101):
        usum = np.zeros_like(u)
        cmat2 = ngk * np.eye(W, dtype=np.complex128)
        for isym in little:
            sub = u[:ntmp] @ sym.d_wann[ir, isym]
            cmat = np.zeros_like(u)
            cmat[:ntmp] = db[ir, isym][:ntmp, :ntmp].conj().T @ sub
            usum += cmat
            cmat2 -= u[:ntmp].conj().T @ cmat[:ntmp]
        diff = float(np.abs(cmat2).sum())
        if diff < sym.eps:
            break
        if it == 100:
            raise RuntimeError("symmetrize_ukirr: not converged (diff %.10e, eps %.10e)" % (diff, sym.eps))
        u = _orthogonalize_u(usum / ngk, ntmp)
    return u


def sitesym_symmetrize_u_matrix(U, sym, ndimwin=None, d_band=None):
    """sitesym_symmetrize_u_matrix (src/sitesym.F90:104-192): U(k_ir) symmetrised, then
    U(R k_ir) = d(R,k) U(k) D^+(R,k) for each star member not yet set.  ndimwin None: the
    wannierisation form (ndim = num_wann); else the disentanglement form, U_opt with
    n = ndimwin(k_ir) window rows.  d_band overrides sym.d_band (after
    sitesym_replace_d_matrix_band it is D itself)."""
    U = U.copy()
    db = sym.d_band if d_band is None else d_band
    done = np.zeros(len(U), dtype=bool)
    for ir in range(sym.nkirr):
        ik = sym.ir2ik[ir]
        done[ik] = True
        n = U.shape[1] if ndimwin is None else int(ndimwin[ik])
        U[ik] = _symmetrize_ukirr(U[ik], ir, sym, None if ndimwin is None else n, d_band=db)
        for isym in range(1, sym.nsym):
            irk = sym.kptsym[isym, ir]
            if done[irk]:
                continue
            done[irk] = True
            U[irk][:n] = db[ir, isym][:n, :n] @ U[ik][:n] @ sym.d_wann[ir, isym].conj().T
    if not done.all():
        raise RuntimeError("error in sitesym_symmetrize_u_matrix")
    return U


def sitesym_symmetrize_gradient(G, sym, mode):
    """sitesym_symmetrize_gradient (src/sitesym.F90:195-278).  mode 1: the star's
    gradients gathered onto k_ir, G(k_ir) += D^+(R,k) G(Rk) D(R,k) for each star member,
    and zero at the reducible k; mode 2: G(k_ir) averaged over its little group."""
    G = G.copy()
    if mode == 1:
        found = np.zeros(len(G), dtype=bool)
        for ir in range(sym.nkirr):
            ik = sym.ir2ik[ir]
            tot = G[ik].copy()
            found[ik] = True
            for isym in range(1, sym.nsym):
                irk = sym.kptsym[isym, ir]
                if found[irk]:
                    continue
                found[irk] = True
                D = sym.d_wann[ir, isym]
                tot = tot + (D.conj().T @ G[irk]) @ D
            G[ik] = tot
        for k in range(len(G)):
            if not sym.irreducible(k):
                G[k] = 0.0
    elif mode == 2:
        for ir in range(sym.nkirr):
            ik = sym.ir2ik[ir]
            ngk = int(np.count_nonzero(sym.kptsym[:, ir] == ik))
            if ngk == 1:
                continue
            tot = G[ik].copy()
            for isym in range(1, sym.nsym):
                if sym.kptsym[isym, ir] != ik:
                    continue
                D = sym.d_wann[ir, isym]
                tot = tot + D.conj().T @ (G[ik] @ D)
            G[ik] = tot / ngk
    else:
        raise ValueError("unknown mode argument in sitesym_symmetrize_gradient")
    return G


def sitesym_symmetrize_rotation(dU, sym):
    """sitesym_symmetrize_rotation (src/sitesym.F90:281-328): dU(R k_ir) =
    D(R,k) dU(k_ir) D^+(R,k) for each star member not yet set."""
    dU = dU.copy()
    done = np.zeros(len(dU), dtype=bool)
    for ir in range(sym.nkirr):
        ik = sym.ir2ik[ir]
        done[ik] = True
        for isym in range(1, sym.nsym):
            irk = sym.kptsym[isym, ir]
            if irk == ik or done[irk]:
                continue
            done[irk] = True
            D = sym.d_wann[ir, isym]
            dU[irk] = D @ (dU[ik] @ D.conj().T)
    if not done.all():
        raise RuntimeError("error in sitesym_symmetrize_rotation")
    return dU


def sitesym_symmetrize_zmatrix(Z, sym, ndimwin):
    """sitesym_symmetrize_zmatrix (src/sitesym.F90:331-391): at each irreducible k,
    Z(k) += d^+ Z(Rk) d over the star's first occurrences, then the little-group terms
    d^+ Z d of that sum, divided by the little group's order.  Z: list of nd x nd (the
    window part); the reducible k are left as they are."""
    Z = [None if z is None else z.copy() for z in Z]
    found = np.zeros(len(Z), dtype=bool)
    for ir in range(sym.nkirr):
        ik = sym.ir2ik[ir]
        nd = int(ndimwin[ik])
        found[ik] = True
        for isym in range(1, sym.nsym):
            irk = sym.kptsym[isym, ir]
            if found[irk]:
                continue
            found[irk] = True
            d = sym.d_band[ir, isym][:nd, :nd]
            Z[ik] = Z[ik] + d.conj().T @ (Z[irk][:nd, :nd] @ d)
        tmp = Z[ik].copy()
        for isym in range(1, sym.nsym):
            if sym.kptsym[isym, ir] != ik:
                continue
            d = sym.d_band[ir, isym][:nd, :nd]
            Z[ik] = Z[ik] + d.conj().T @ (tmp @ d)
        Z[ik] = Z[ik] / int(np.count_nonzero(sym.kptsym[:, ir] == ik))
    return Z


def _gen_eig_larger(h11, h12, h22, s11, s12, s22):
    """The eigenvector of the larger eigenvalue of H v = w S v (2 x 2 Hermitian, S
    positive definite), normalised to v^+ S v = 1, in the phase ZHPGVX gives it: what
    sitesym_dis_extract_symmetry takes (src/sitesym.F90:649-668).  ZHPGVX reduces with the
    upper Cholesky factor of S and zhptrd, whose reflector leaves the last coordinate
    alone, so the second component comes out real; on these problems it comes out
    positive.  The phase is not free: the symmetrisation that follows averages d^+ U D
    column by column, and the testw90_disentanglement_sawfs lines move by 1e-7 A^2 under
    another choice (5e-9 with this one)."""
    H = np.array([[h11, h12], [np.conj(h12), h22]], dtype=np.complex128)
    S = np.array([[s11, s12], [np.conj(s12), s22]], dtype=np.complex128)
    L = np.linalg.cholesky(S)
    Li = np.linalg.inv(L)
    w, y = np.linalg.eigh(Li @ H @ Li.conj().T)
    v = Li.conj().T @ y[:, 1]
    if v[1] != 0:
        v = v * (abs(v[1]) / v[1])
    return v


def sitesym_dis_extract_symmetry(sym, U, Z, ik, n, num_wann):
    """sitesym_dis_extract_symmetry (src/sitesym.F90:550-695): steepest descent of
    Omega_I at an irreducible k within the symmetric subspaces.  Per pass: ZU = Z U,
    lambda = U^+ Z U, dU = ZU - U lambda (done when sum |dU| < 1e-10); each column moves
    to the larger solution of the 2 x 2 problem in span(u_i, dU_i); then symmetrize_ukirr.
    Up to 50 passes.  Returns (U, lambda of the last pass)."""
    U = U.copy()
    ir = sym.ik2ir[ik]
    Zn = Z[:n, :n]
    lam = None
    for _ in range(50):
        ZU = Zn @ U[:n]
        lam = U[:n].conj().T @ ZU
        dU = ZU - U[:n] @ lam
        if np.abs(dU).sum() < 1e-10:
            return U, lam
        Unew = np.zeros_like(U)
        for i in range(num_wann):
            u, zu, du = U[:n, i], ZU[:, i], dU[:, i]
            h11 = np.vdot(u, zu).real
            h12 = np.vdot(zu, du)
            h22 = np.vdot(du, Zn @ du).real
            s11 = np.vdot(u, u).real
            s12 = np.vdot(u, du)
            s22 = np.vdot(du, du).real
            if abs(s22) < 1e-10:
                Unew[:, i] = U[:, i]
                continue
            v = _gen_eig_larger(h11, h12, h22, s11, s12, s22)
            Unew[:n, i] = v[0] * u + v[1] * du
        U = _symmetrize_ukirr(Unew, ir, sym, n)
    return U, lam


# ---------------------------------------------------------------------------
# disentanglement: dis_main (src/disentangle.F90:31-284), k-point path, no site symmetry
# ---------------------------------------------------------------------------
@dataclass
class DisControl:
    """dis_control_type / dis_manifold_type defaults (src/wannier90_types.F90:125-137,
    src/types.F90:179-199)."""
    num_iter: int = 200
    mix_ratio: float = 0.5
    conv_tol: float = 1.0e-10
    conv_window: int = 3
    win_min: float = -1.0e300
    win_max: float = 1.0e300
    froz_min: float = -1.0e300
    froz_max: float = 1.0e300
    frozen_states: bool = False


def _heev(h):
    """Eigenpairs of a Hermitian matrix, ascending (the reference calls ZHPEVX 'V','A','U')."""
    w, v, info = lapack.zheev(h, compute_v=1, lower=0)
    if info != 0:
        raise RuntimeError("zheev failed")
    return w, v


def dis_windows(eig, num_wann, dc: DisControl):
    """dis_windows (src/disentangle.F90:851-1171): outer window [nfirstwin, +ndimwin) and
    the frozen states inside it, per k (0-based band indices)."""
    K, nb = eig.shape
    out = dict(ndimwin=np.zeros(K, int), nfirstwin=np.zeros(K, int), ndimfroz=np.zeros(K, int),
               indxfroz=[], indxnfroz=[], lfrozen=[], eigval_opt=np.zeros((K, nb)))
    for k in range(K):
        e = eig[k]
        if e[0] > dc.win_max or e[-1] < dc.win_min:
            raise RuntimeError("dis_windows: The outer energy window contains no eigenvalues")
        imin = -1
        imax = -1
        for i in range(nb):
            if imin < 0:
                if dc.win_min <= e[i] <= dc.win_max:
                    imin = i
                imax = i
            if e[i] <= dc.win_max:
                imax = i
        ndim = imax - imin + 1
        if ndim < num_wann:
            raise RuntimeError("dis_windows: Energy window contains fewer states than number of target WFs")
        fmin, fmax = -1, -2
        if dc.frozen_states:
            for i in range(imin, imax + 1):
                if fmin < 0:
                    if dc.froz_min <= e[i] <= dc.froz_max:
                        fmin = fmax = i - imin
                elif e[i] <= dc.froz_max:
                    fmax += 1
        nf = fmax - fmin + 1 if fmin >= 0 else 0
        if nf > num_wann:
            raise RuntimeError("dis_windows: More states in the frozen window than target WFs")
        froz = list(range(fmin, fmin + nf)) if nf else []
        lfr = np.zeros(ndim, bool)
        lfr[froz] = True
        out["ndimwin"][k], out["nfirstwin"][k], out["ndimfroz"][k] = ndim, imin, nf
        out["indxfroz"].append(np.array(froz, int))
        out["indxnfroz"].append(np.array([j for j in range(ndim) if not lfr[j]], int))
        out["lfrozen"].append(lfr)
        out["eigval_opt"][k, :ndim] = e[imin:imin + ndim]
    return out


def dis_project(A, win, num_wann):
    """dis_project (src/disentangle.F90:1173-1429): U_opt = Z V^dagger from the SVD of the
    windowed projections; returns (U_opt [K][nb][W], A_win [K][nb][W]), rows past ndimwin 0."""
    K, nb, W = A.shape
    Uo = np.zeros((K, nb, W), dtype=np.complex128)
    Aw = np.zeros((K, nb, W), dtype=np.complex128)
    for k in range(K):
        n, f = win["ndimwin"][k], win["nfirstwin"][k]
        a = A[k, f:f + n, :]
        z, sv, vh, info = lapack.zgesvd(a, full_matrices=1, compute_uv=1)[:4]
        if info != 0:
            raise RuntimeError("dis_project: problem in ZGESVD 1")
        Uo[k, :n] = z[:, :W] @ vh
        Aw[k, :n] = (z[:, :W] * sv[None, :W]) @ vh
        chk = Uo[k, :n].conj().T @ Uo[k, :n]
        if np.max(np.abs(chk - np.eye(W))) > EPS5:
            raise RuntimeError("dis_project: Error in unitarity of initial U in dis_project")
    return Uo, Aw


def dis_proj_froz(Uo, win, num_wann):
    """dis_proj_froz (src/disentangle.F90:1431-1891): keep the frozen states and complete
    them with the leading eigenvectors of Q P Q (P the projector on the projected
    subspace, Q on the non-frozen states), with the reference's zero-eigenvalue fix."""
    K = Uo.shape[0]
    W = num_wann
    Uo = Uo.copy()
    for k in range(K):
        n, nf = win["ndimwin"][k], win["ndimfroz"][k]
        lfr = win["lfrozen"][k]
        if W > nf:
            u = Uo[k, :n]
            P = u @ u.conj().T
            q = (~lfr).astype(np.float64)
            QPQ = q[:, None] * P * q[None, :]
            w, cz = _heev(QPQ)
            il = n - (W - nf)                      # 0-based first of the leading ones
            tops = list(range(n - 1, il - 1, -1))
            nzero = sum(1 for j in tops if w[j] < EPS8)
            goods = len(tops) - nzero
            if nzero > 0:
                vmap = [j for j in range(n - 1, n - 1 - goods, -1)]
                for _ in range(nzero):
                    for v in range(n - 1, -1, -1):
                        if v in vmap:
                            continue
                        take = all(abs(np.vdot(Uo[k, :n, m], cz[:, v])) <= EPS8 for m in range(nf))
                        if take:
                            vmap.append(v)
                            break
                if len(vmap) < W - nf:
                    raise RuntimeError("dis_proj_froz: Ortho-fix failed to find enough vectors")
                for c, v in enumerate(vmap[:W - nf]):
                    Uo[k, :n, nf + c] = cz[:, v]
            else:
                for c in range(W - nf):
                    Uo[k, :n, nf + c] = cz[:, il + c]
        if nf > 0:
            for l in range(nf):
                Uo[k, :, l] = 0.0
                Uo[k, win["indxfroz"][k][l], l] = 1.0
    return Uo


def slim_m(Mraw, win, nnlist):
    """internal_slim_m (src/disentangle.F90:453-529): M restricted to the windows,
    Mw[k,b][:ndimwin(k), :ndimwin(k+b)] (rest zero)."""
    K, B, nb, _ = Mraw.shape
    Mw = np.zeros_like(Mraw)
    for k in range(K):
        f1, n1 = win["nfirstwin"][k], win["ndimwin"][k]
        for b in range(B):
            k2 = nnlist[k, b]
            f2, n2 = win["nfirstwin"][k2], win["ndimwin"][k2]
            Mw[k, b, :n1, :n2] = Mraw[k, b, f1:f1 + n1, f2:f2 + n2]
    return Mw


def _zmatrix(Mw, Uo, win, km, k):
    """internal_zmatrix (src/disentangle.F90:2922-2988) on the non-frozen states of k."""
    nf_idx = win["indxnfroz"][k]
    Z = np.zeros((len(nf_idx), len(nf_idx)), dtype=np.complex128)
    for b in range(km["nntot"]):
        k2 = km["nnlist"][k, b]
        cbw = Mw[k, b] @ Uo[k2]                     # (nb, W)
        c = cbw[nf_idx]
        Z += km["wb"][b] * (c @ c.conj().T)
    return Z


def _omega_i_k(Mw, Uo, km, k, W, rows=None):
    """sum_b w_b |U(k)^dag M(k,b) U(k+b)|^2 restricted to the first `rows` rows."""
    tot = 0.0
    for b in range(km["nntot"]):
        k2 = km["nnlist"][k, b]
        cww = Uo[k].conj().T @ Mw[k, b] @ Uo[k2]
        if rows is not None:
            cww = cww[:rows]
        tot += km["wb"][b] * float((cww.real ** 2 + cww.imag ** 2).sum())
    return tot


@dataclass
class DisRecord:
    iter: int
    omega_i_prev: float   # womegai1 (from the eigenvalues)
    omega_i: float        # womegai (from the overlaps)
    delta: float


def dis_extract(Mw, Uo, win, km, num_wann, dc: DisControl, sitesym=None):
    """dis_extract (src/disentangle.F90:1893-2864): iterative minimisation of Omega_I
    with Z-matrix mixing; then the subspace Hamiltonian is diagonalised to fix U_opt's
    gauge.  Returns (U_opt, Omega_I, records, converged).
    ``sitesym``: the symmetry-adapted form (:2193-2207, :2214-2216, :2242-2247,
    :2289-2298, :2404-2411, :2504-2513, :2675): symmetrised Z matrices, updates at the
    irreducible k only (each weighted by its star in Omega_I(i-1)), symmetrised U_opt,
    and no final gauge change."""
    K = Mw.shape[0]
    W = num_wann
    Uo = Uo.copy()
    nf = win["ndimfroz"]
    zin = [None] * K
    zout = [None] * K
    history = np.zeros(dc.conv_window)
    recs = []
    converged = False
    womegai = 0.0
    sym = sitesym
    if sym is not None and any(nf > 0):
        raise RuntimeError("not implemented in symmetry-adapted mode")
    for it in range(1, dc.num_iter + 1):
        if it == 1:
            for k in range(K):
                if W > nf[k]:
                    zin[k] = _zmatrix(Mw, Uo, win, km, k)
            if sym is not None:
                zin = sitesym_symmetrize_zmatrix(zin, sym, win["ndimwin"])
        else:
            for k in range(K):
                if sym is not None and not sym.irreducible(k):
                    continue
                if W > nf[k]:
                    zin[k] = dc.mix_ratio * zout[k] + (1.0 - dc.mix_ratio) * zin[k]
                    zin[k] = np.triu(zin[k]) + np.triu(zin[k], 1).conj().T
        womegai1 = 0.0
        Unew = Uo.copy()
        for k in range(K):
            wk = W * km["wbtot"]
            if sym is not None:
                if not sym.irreducible(k):
                    continue
                ir = sym.ik2ir[k]
                wk = wk * sym.nsym / int(np.count_nonzero(sym.kptsym[:, ir] == k))
                Unew[k], lam = sitesym_dis_extract_symmetry(sym, Uo[k], zin[k], k, win["ndimwin"][k], W)
                wk -= float(np.trace(lam).real)
                womegai1 += wk
                continue
            if nf[k] > 0:
                wk -= _omega_i_k(Mw, Uo, km, k, W, rows=nf[k])
            if W > nf[k]:
                w, cz = _heev(zin[k])
                n = win["ndimwin"][k]
                m = nf[k]
                for j in range(n - W, n - nf[k]):
                    wk -= w[j]
                    Unew[k, :, m] = 0.0
                    Unew[k, win["indxnfroz"][k], m] = cz[:, j]
                    m += 1
            womegai1 += wk
        Uo = Unew
        if sym is not None:
            Uo = sitesym_symmetrize_u_matrix(Uo, sym, ndimwin=win["ndimwin"])
        womegai1 /= K
        womegai = sum(W * km["wbtot"] - _omega_i_k(Mw, Uo, km, k, W) for k in range(K)) / K
        delta = womegai1 / womegai - 1.0
        recs.append(DisRecord(it, womegai1, womegai, delta))
        for k in range(K):
            if W > nf[k]:
                zout[k] = _zmatrix(Mw, Uo, win, km, k)
        if sym is not None:
            zout = sitesym_symmetrize_zmatrix(zout, sym, win["ndimwin"])
        # internal_test_convergence (:2866-2920)
        if it <= dc.conv_window:
            history[it - 1] = delta
        else:
            history = np.concatenate([history[1:], [delta]])
        if it >= dc.conv_window and np.all(np.abs(history) < dc.conv_tol):
            converged = True
            break
    # subspace Hamiltonian gauge (:2560-2640); kept out in the symmetry-adapted mode (:2675)
    for k in range(K if sym is None else 0):
        n = win["ndimwin"][k]
        ham = Uo[k, :n].conj().T @ (win["eigval_opt"][k, :n, None] * Uo[k, :n])
        w, cz = _heev(ham)
        Uo[k, :n] = Uo[k, :n] @ cz
    return Uo, womegai, recs, converged


def dis_main(Mraw, A, eig, km, num_wann, dc: DisControl, sitesym=None):
    """The disentanglement step of the library (w90_disentangle,
    src/library_interface.F90:362-420): dis_main plus setup_m_loc.  Mraw[k,b,nb,nb],
    A[k,nb,W], eig[k,nb].  Returns (U0[K,W,W], M0[K,B,W,W], U_opt[K,nb,W], Omega_I, records)
    with M0 = U0^dag U_opt^dag M U_opt' U0' ready for wann_main.
    ``sitesym``: the symmetry-adapted mode (src/disentangle.F90:151-157, :186-190, :237,
    :627-629, :688-692)."""
    win = dis_windows(eig, num_wann, dc)
    Uo, Aw = dis_project(A, win, num_wann)
    if any(win["ndimfroz"] > 0):
        if sitesym is not None:
            raise RuntimeError("in symmetry-adapted mode, frozen window not implemented yet")
        Uo = dis_proj_froz(Uo, win, num_wann)
    Mw = slim_m(Mraw, win, km["nnlist"])
    if sitesym is not None:
        Uo = sitesym_symmetrize_u_matrix(Uo, sitesym, ndimwin=win["ndimwin"])
    Uo, omi, recs, conv = dis_extract(Mw, Uo, win, km, num_wann, dc, sitesym=sitesym)
    K, B = Mraw.shape[:2]
    W = num_wann
    Mopt = np.empty((K, B, W, W), dtype=np.complex128)
    for k in range(K):
        for b in range(B):
            Mopt[k, b] = Uo[k].conj().T @ Mw[k, b] @ Uo[km["nnlist"][k, b]]
    # internal_find_u (:531-698): U = Z V^dagger from the SVD of U_opt^dag A
    U = np.zeros((K, W, W), dtype=np.complex128)
    for k in range(K):
        if sitesym is not None and not sitesym.irreducible(k):
            continue
        caa = Uo[k].conj().T @ Aw[k]
        z, sv, vh, info = lapack.zgesvd(caa, full_matrices=1, compute_uv=1)[:4]
        if info != 0:
            raise RuntimeError("dis_main: problem in ZGESVD 1")
        U[k] = z @ vh
    if sitesym is not None:
        # sitesym_replace_d_matrix_band: d_band <- D from here on
        U = sitesym_symmetrize_u_matrix(U, sitesym, d_band=sitesym.d_wann)
    # setup_m_loc (:286-370)
    M0 = np.conj(U)[:, None].transpose(0, 1, 3, 2) @ Mopt @ U[km["nnlist"]]
    return U, M0, Uo, omi, recs


# ---------------------------------------------------------------------------
# wann_omega / wann_domega  (src/wannierise.F90:1979-2284, :2287-2569)
# ---------------------------------------------------------------------------
@dataclass
class Spread:
    """localisation_vars_type (src/wannierise.F90:35-43).  With selective localisation
    om_i and om_od are not computed (left 0) and om_iod / om_nu hold the SLWF terms."""
    om_i: float = 0.0
    om_d: float = 0.0
    om_od: float = 0.0
    om_tot: float = 0.0
    om_iod: float = 0.0
    om_nu: float = 0.0

    def copy(self):
        return Spread(self.om_i, self.om_d, self.om_od, self.om_tot, self.om_iod, self.om_nu)


@dataclass
class Slwf:
    """wann_slwf_type as wann_main uses it (src/wannier90_types.F90:147-161): the first
    ``num`` Wannier functions are the objective ones; ``lam`` is lambda_loc (the
    constraint's Lagrange multiplier, 0 when slwf_constrain = F, src/wannierise.F90:445-450);
    ``centres`` [3, W] are the constrained centres (Cartesian, Angstrom; None when
    unconstrained)."""
    num: int
    lam: float = 0.0
    centres: np.ndarray | None = None

    def __post_init__(self):
        if self.centres is None:
            self.lam = 0.0

    @property
    def constrain(self):
        return self.centres is not None


def _ln_diag(diag, sheet):
    """Im ln M_nn on the branch chosen by the guiding centres: aimag(log(csheet*M_nn))
    - sheet (src/wannierise.F90:2036-2041, :2368-2374); sheet None = no guiding."""
    if sheet is None:
        return np.angle(diag)
    return np.angle(np.exp(1j * sheet) * diag) - sheet


def wann_omega(M, km, omega_invariant=None, sheet=None, slwf=None):
    """Returns (Spread, rave[3,W], r2ave[W], rave2[W]).

    ``omega_invariant`` None reproduces the ``first_pass`` branch (:2214-2239).
    ``sheet`` [K,B,W]: branch-cut offsets of the guiding centres (wann_phases).
    ``slwf`` (:class:`Slwf`): the selective-localisation branch (:2144-2211).
    """
    K, B, W, _ = M.shape
    wb, bk = km["wb"], km["bk"]
    diag = np.diagonal(M, axis1=2, axis2=3)           # (K,B,W)
    ln = _ln_diag(diag, sheet)                        # aimag(log(.)) :2034-2043
    rave = -np.einsum("b,kbi,kbn->in", wb, bk, ln) / K          # :2045-2061
    rave2 = (rave * rave).sum(axis=0)
    mnn2 = (diag * diag.conj()).real
    r2ave = np.einsum("b,kbn->n", wb, 1.0 - mnn2 + ln ** 2) / K  # :2076-2090
    if slwf is not None:
        return _omega_slwf(ln, mnn2, rave, wb, bk, K, slwf), rave, r2ave, rave2
    absm2 = (M * M.conj()).real
    if omega_invariant is None:
        summ = absm2.sum(axis=(2, 3))                  # (K,B)
        om_i = float(np.einsum("b,kb->", wb, W - summ) / K)
    else:
        om_i = omega_invariant
    offd = absm2.sum(axis=(2, 3)) - mnn2.sum(axis=2)  # (K,B)
    om_od = float(np.einsum("b,kb->", wb, offd) / K)  # :2241-2258
    brn = np.einsum("kbi,in->kbn", bk, rave)
    om_d = float(np.einsum("b,kbn->", wb, (ln + brn) ** 2) / K)  # :2260-2275
    sp = Spread(om_i, om_d, om_od, om_i + om_d + om_od)
    return sp, rave, r2ave, rave2


def _omega_slwf(ln, mnn2, rave, wb, bk, K, slwf):
    """wann_omega's selective-localisation branch (src/wannierise.F90:2144-2211):
    Omega_IOD over the objective WFs (minus lambda ln^2 when constrained), Omega_D
    weighted by (1 - lambda), and the constraint term Omega_nu."""
    s, lam = slwf.num, slwf.lam
    ln_s, a_s = ln[:, :, :s], mnn2[:, :, :s]
    summ = a_s.sum(axis=2)
    if slwf.constrain:
        summ = summ - lam * (ln_s ** 2).sum(axis=2)                  # :2153-2157
    om_iod = float(np.einsum("b,kb->", wb, s - summ) / K)             # :2158-2167
    brn = np.einsum("kbi,in->kbn", bk, rave)[:, :, :s]
    om_d = float(np.einsum("b,kbn->", (1.0 - lam) * wb, (ln_s + brn) ** 2) / K)   # :2169-2183
    om_nu = 0.0
    if slwf.constrain:                                                # :2186-2208
        bc = np.einsum("kbi,in->kbn", bk, slwf.centres)[:, :, :s]
        om_nu = float(np.einsum("b,kbn->", 2.0 * wb, ln_s * lam * bc) / K)
        om_nu += lam * float((slwf.centres[:, :s] ** 2).sum())
    return Spread(0.0, om_d, 0.0, om_iod + om_d + om_nu, om_iod, om_nu)


def _domega_slwf(M, diag, lnw, rnkb, wb, bk, K, slwf):
    """wann_domega's selective-localisation branch (src/wannierise.F90:2431-2509), term
    by term: objective rows/columns only, the constraint terms when constrained."""
    W = M.shape[-1]
    s, lam = slwf.num, slwf.lam
    c = -0.5j
    H = lambda X: np.conj(np.swapaxes(X, -1, -2))
    crt = M / diag[:, :, None, :]                      # crt(m,n) = M_mn / M_nn
    cr = M * np.conj(diag)[:, :, None, :]              # cr(m,n)  = M_mn conj(M_nn)
    crt_h, cr_h = H(crt), H(cr)                        # conj(crt(n,m)), conj(cr(n,m)) at (m,n)
    w = wb[None, :, None, None]
    qn, qm = lnw[:, :, None, :], lnw[:, :, :, None]
    rn, rm = rnkb[:, :, None, :], rnkb[:, :, :, None]
    obj = np.arange(W) < s
    # m <= slwf_num, n <= slwf_num (:2434-2468)
    gb = w * 0.5 * (cr - cr_h)
    gb = gb - (crt * qn + crt_h * qm) * c
    gb = gb - (crt * rn + crt_h * rm) * c
    # m <= slwf_num < n (:2469-2486)
    gm = -w * 0.5 * cr_h - crt_h * (qm + w * rm) * c
    # n <= slwf_num < m (:2487-2504)
    gn = w * cr * 0.5 - crt * (qn + w * rn) * c
    if slwf.constrain:
        r0 = np.einsum("kbi,in->kbn", bk, slwf.centres)      # r0kb (:2396-2406)
        r0n, r0m = r0[:, :, None, :], r0[:, :, :, None]
        gb = gb + lam * (crt * qn + crt_h * qm) * c
        gb = gb + w * lam * (crt * rn + crt_h * rm) * c
        gb = gb - lam * (crt * qn + crt_h * qm) * c
        gb = gb - w * lam * (r0n * crt + r0m * crt_h) * c
        gm = gm + lam * crt_h * (qm + w * rm) * c - lam * crt_h * qm * c
        gm = gm - w * lam * r0m * crt_h * c
        gn = gn + lam * crt * (qn + w * rn) * c - lam * crt * qn * c
        gn = gn - w * lam * r0n * crt * c
    mo, no = obj[:, None], obj[None, :]
    g = np.where(mo & no, gb, np.where(mo & ~no, gm, np.where(~mo & no, gn, 0.0)))
    return g.sum(axis=1) * (4.0 / K)                   # :2531


def wann_domega(M, km, sheet=None, slwf=None):
    """Gradient cdodq(m,n,k) (src/wannierise.F90:2287-2569); ``slwf``: the
    selective-localisation branch."""
    K, B, W, _ = M.shape
    wb, bk = km["wb"], km["bk"]
    diag = np.diagonal(M, axis1=2, axis2=3)
    lnw = wb[None, :, None] * _ln_diag(diag, sheet)    # :2366-2375
    rave = -np.einsum("kbi,kbn->in", bk, lnw) / K      # :2378-2391
    rnkb = np.einsum("kbi,in->kbn", bk, rave)          # :2409-2417
    if slwf is not None:
        return _domega_slwf(M, diag, lnw, rnkb, wb, bk, K, slwf)
    crt = M / diag[:, :, None, :]
    cr = M * np.conj(diag)[:, :, None, :]
    G = np.zeros((K, W, W), dtype=np.complex128)
    H = lambda X: np.conj(np.swapaxes(X, -1, -2))
    w = wb[None, :, None, None]
    G += (w * 0.5 * (cr - H(cr))).sum(axis=1)          # :2511-2515
    T = crt * lnw[:, :, None, :]
    G -= ((T + H(T)) * (-0.5j)).sum(axis=1)            # :2516-2520
    R = crt * rnkb[:, :, None, :]
    G -= (w * (R + H(R)) * (-0.5j)).sum(axis=1)        # :2521-2524
    return G * (4.0 / K)                               # :2531


# ---------------------------------------------------------------------------
# guiding centres: wann_phases (src/wannierise.F90:1756-1976)
# ---------------------------------------------------------------------------
def inv3(a):
    """utility_inv3 (src/utility.F90:233-262): cofactor matrix b and determinant;
    for the symmetric matrices it is used on, inverse(a) = b / det."""
    b = np.empty((3, 3))
    b[0, 0] = a[1, 1] * a[2, 2] - a[2, 1] * a[1, 2]
    b[0, 1] = a[1, 2] * a[2, 0] - a[2, 2] * a[1, 0]
    b[0, 2] = a[1, 0] * a[2, 1] - a[2, 0] * a[1, 1]
    b[1, 0] = a[2, 1] * a[0, 2] - a[0, 1] * a[2, 2]
    b[1, 1] = a[2, 2] * a[0, 0] - a[0, 2] * a[2, 0]
    b[1, 2] = a[2, 0] * a[0, 1] - a[0, 0] * a[2, 1]
    b[2, 0] = a[0, 1] * a[1, 2] - a[1, 1] * a[0, 2]
    b[2, 1] = a[0, 2] * a[1, 0] - a[1, 2] * a[0, 0]
    b[2, 2] = a[0, 0] * a[1, 1] - a[1, 0] * a[0, 1]
    det = float(a[0, 0] * b[0, 0] + a[0, 1] * b[0, 1] + a[0, 2] * b[0, 2])
    return b, det


def wann_phases(M, km, rguide, irguide):
    """Returns (rguide[3,W], sheet[K,B,W]).  The centres are refitted from the phases of
    sum_k M_nn(k, b) over the b directions when irguide != 0 (:1830-1925); the sheet is
    b . rguide_n (:1927-1939)."""
    K, B, W, _ = M.shape
    bka, neigh = km["bka"], km["neigh"]
    rguide = np.array(rguide, dtype=np.float64, copy=True)
    diag = np.diagonal(M, axis1=2, axis2=3)            # (K,B,W)
    for n in range(W):
        csum = np.array([diag[np.arange(K), neigh[:, na], n].sum() for na in range(km["nnh"])])
        smat = np.zeros((3, 3))
        svec = np.zeros(3)
        for nn in range(km["nnh"]):
            if nn < 3:
                xx = -math.atan2(csum[nn].imag, csum[nn].real)
            else:
                xx0 = float(bka[nn] @ rguide[:, n])
                z = csum[nn] * complex(math.cos(xx0), math.sin(xx0))
                xx = xx0 - math.atan2(z.imag, z.real)
            smat += np.outer(bka[nn], bka[nn])
            svec += bka[nn] * xx
            if nn >= 2:
                sinv, det = inv3(smat)
                if abs(det) > EPS6 and irguide != 0:
                    rguide[:, n] = sinv @ svec / det
    sheet = np.einsum("kbi,in->kbn", km["bk"], rguide)
    return rguide, sheet


# ---------------------------------------------------------------------------
# preconditioner (src/wannierise.F90:1256-1368) and its Wigner-Seitz grid
# ---------------------------------------------------------------------------
def ws_vectors(real_lattice, mp_grid, ws_search_size=(2, 2, 2), ws_distance_tol=1.0e-5):
    """hamiltonian_wigner_seitz (src/hamiltonian.F90:689-853): lattice points n of the
    Born-von Karman supercell's Wigner-Seitz cell, in the reference's loop order
    (n1 outer, n3 inner), with degeneracies.  Returns (irvec[nrpts,3] int, ndegen[nrpts])."""
    A = np.asarray(real_lattice, dtype=np.float64)
    metric = A @ A.T                                         # utility_metric
    mp = np.asarray(mp_grid, dtype=np.int64)
    s = np.asarray(ws_search_size, dtype=np.int64)
    rng = [np.arange(-s[i] * mp[i], s[i] * mp[i] + 1) for i in range(3)]
    n = np.stack(np.meshgrid(*rng, indexing="ij"), axis=-1).reshape(-1, 3)
    sh = [np.arange(-s[i] - 1, s[i] + 2) for i in range(3)]
    shifts = np.stack(np.meshgrid(*sh, indexing="ij"), axis=-1).reshape(-1, 3)
    centre = (len(shifts) - 1) // 2                          # i1 = i2 = i3 = 0
    tol2 = ws_distance_tol ** 2
    irvec, ndegen = [], []
    for c0 in range(0, len(n), 4096):
        nd = (n[c0:c0 + 4096, None, :] - shifts[None, :, :] * mp).astype(np.float64)
        dist = np.einsum("psi,ij,psj->ps", nd, metric, nd)
        dmin = dist.min(axis=1)
        keep = np.abs(dist[:, centre] - dmin) < tol2
        deg = (np.abs(dist - dmin[:, None]) < tol2).sum(axis=1)
        irvec.append(n[c0:c0 + 4096][keep])
        ndegen.append(deg[keep])
    irvec = np.concatenate(irvec).astype(np.int64)
    ndegen = np.concatenate(ndegen).astype(np.int64)
    tot = float(np.sum(1.0 / ndegen))                        # sum rule (:829-852)
    if abs(tot - float(np.prod(mp))) > EPS8:
        raise RuntimeError("hamiltonian_wigner_seitz: error in finding Wigner-Seitz points")
    return irvec, ndegen


def precond_setup(real_lattice, kpt_latt, mp_grid):
    """The tables wann_main builds for precond=T (src/wannierise.F90:269-300):
    irvec/ndegen from hamiltonian_setup and k_to_r(k, R) = exp(-i 2pi k.R)."""
    irvec, ndegen = ws_vectors(real_lattice, mp_grid)
    rdotk = TWOPI * np.asarray(kpt_latt, dtype=np.float64) @ irvec.T.astype(np.float64)
    # the filter's |R|^2 uses matmul(real_lattice, irvec) exactly as the reference
    # (:1341), i.e. (a_1.n, a_2.n, a_3.n) with a_i the rows of real_lattice
    rvec = irvec.astype(np.float64) @ np.asarray(real_lattice, dtype=np.float64).T
    return {"irvec": irvec, "ndegen": ndegen, "k_to_r": np.exp(-1j * rdotk),
            "r2": (rvec * rvec).sum(axis=1)}


def precond_search_direction(cdodq, om_tot, pc):
    """precond_search_direction, optimisation >= 3 form (src/wannierise.F90:1256-1368):
    k -> R, filter by 1/(1 + R^2/alpha) with alpha = 10*om_tot/num_wann, R -> k."""
    K, W, _ = cdodq.shape
    k_to_r = pc["k_to_r"]
    cr = np.einsum("kmn,kr->rmn", cdodq, k_to_r) / K         # :1317-1320
    alpha = 10.0 * om_tot / W                                # :1339
    cr = cr * (1.0 / (1.0 + pc["r2"] / alpha))[:, None, None]
    cr = cr / pc["ndegen"][:, None, None].astype(np.float64)  # :1347-1349
    return np.einsum("rmn,kr->kmn", cr, k_to_r.conj())       # :1350-1351


# ---------------------------------------------------------------------------
# wann_main  (src/wannierise.F90:48-1752)
# ---------------------------------------------------------------------------
@dataclass
class WannControl:
    """wann_control_type defaults (src/wannier90_types.F90:170-192)."""
    num_iter: int = 100
    num_cg_steps: int = 5
    conv_tol: float = 1.0e-10
    conv_window: int = -1
    trial_step: float = 2.0
    fixed_step: float = -999.0
    lfixstep: bool = False
    conv_noise_amp: float = -1.0
    conv_noise_num: int = 3
    precond: bool = False
    guiding_centres: bool = False
    num_no_guide_iter: int = 0
    num_guide_cycles: int = 1


@dataclass
class IterRecord:
    iter: int
    delta: float
    rms_grad: float
    spread: Spread
    centres: np.ndarray
    spreads: np.ndarray
    lquad: bool
    alphamin: float


@dataclass
class WannResult:
    U: np.ndarray
    M: np.ndarray
    spread: Spread
    centres: np.ndarray
    spreads: np.ndarray
    iters: list = field(default_factory=list)
    initial: IterRecord | None = None
    converged: bool = False
    niter: int = 0


def new_u_and_m(cdq, U, M, nnlist, sitesym=None):
    """internal_new_u_and_m (src/wannierise.F90:1599-1751): zheev of i*cdq, dU=V e^{-i l} V^dag.
    ``sitesym``: dU at the irreducible k only, the rest by sitesym_symmetrize_rotation
    (:1656-1659, :1719-1726)."""
    K, W, _ = cdq.shape
    dU = cdq.copy()
    for k in range(K):
        if sitesym is not None and not sitesym.irreducible(k):
            continue
        w, v, info = lapack.zheev(1j * cdq[k], compute_v=1, lower=0)
        if info != 0:
            raise RuntimeError("zheev failed in internal_new_u_and_m")
        dU[k] = (v * np.exp(-1j * w)[None, :]) @ v.conj().T
    if sitesym is not None:
        dU = sitesym_symmetrize_rotation(dU, sitesym)
    Unew = U @ dU                                                     # :1728-1733
    Mnew = np.conj(np.swapaxes(dU, 1, 2))[:, None] @ M @ dU[nnlist]  # :1736-1748
    return Unew, Mnew


def wann_main(M, U, km, ctl: WannControl, record=True, precond=None, rguide=None, slwf=None, sitesym=None,
              update_noise=None):
    """Restatement of wann_main.
    ``precond``: the tables of :func:`precond_setup` when ``ctl.precond``;
    ``rguide``: guiding centres [3,W] (Cartesian, Angstrom) when ``ctl.guiding_centres``;
    ``slwf``: :class:`Slwf` for selective localisation (slwf_num < num_wann);
    ``sitesym``: :class:`Sitesym` for the symmetry-adapted mode (site_symmetry = T);
    ``update_noise``: test use only -- a function applied to every updated M (e.g. a
    seeded relative perturbation modelling an implementation whose M update carries
    rounding at that level); None for the reference's arithmetic.
    The mode-2 symmetrisation the reference applies to its global cdq array after the
    search direction (:589-591) acts on the previous step's rotation, which
    internal_new_u_and_m overwrites before reading it: it does not enter the run."""
    if ctl.precond and precond is None:
        raise ValueError("precond=T needs the precond_setup tables")
    if ctl.guiding_centres and rguide is None:
        raise ValueError("guiding_centres=T needs the projection centres")
    M = M.copy()
    U = U.copy()
    K, B, W, _ = M.shape
    nnlist = km["nnlist"]
    wbtot = km["wbtot"]

    sheet = None
    irguide = 0
    if ctl.guiding_centres:
        sheet = np.zeros((K, B, W))
        if ctl.num_no_guide_iter <= 0:                            # :435-443
            rguide, sheet = wann_phases(M, km, rguide, irguide)
            irguide = 1
    wann_spread, rave, r2ave, rave2 = wann_omega(M, km, sheet=sheet, slwf=slwf)   # :452-457
    om_invariant = wann_spread.om_i
    res = WannResult(U, M, wann_spread, rave, r2ave - rave2)
    res.initial = IterRecord(0, wann_spread.om_tot, 0.0, wann_spread.copy(), rave.copy(),
                             r2ave - rave2, False, 0.0)
    old_spread = Spread()
    ncg = 0
    gcnorm0 = gcnorm1 = 0.0
    cdqkeep = np.zeros((K, W, W), dtype=np.complex128)
    history = np.zeros(max(ctl.conv_window, 1))
    conv_count = 0
    noise_count = 0
    lconverged = False
    lrandom = False
    lfirst = True
    save_spread = 0.0
    lquad = False
    alphamin = 0.0
    it = 0
    for it in range(1, ctl.num_iter + 1):
        if (ctl.guiding_centres and it > ctl.num_no_guide_iter
                and it % max(ctl.num_guide_cycles, 1) == 0):           # :546-555
            rguide, sheet = wann_phases(M, km, rguide, irguide)
            irguide = 1
        cdodq = wann_domega(M, km, sheet=sheet, slwf=slwf)            # :566-571
        if sitesym is not None:                                       # :2543-2551
            cdodq = sitesym_symmetrize_gradient(cdodq, sitesym, 1)
            cdodq = sitesym_symmetrize_gradient(cdodq, sitesym, 2)
        if ctl.precond:                                               # :577-581
            cdodq_p = precond_search_direction(cdodq, wann_spread.om_tot, precond)
        else:
            cdodq_p = cdodq
        # internal_search_direction (:1371-1525)
        gcnorm1 = float(np.vdot(cdodq_p, cdodq).real)
        if it == 1 or ncg >= ctl.num_cg_steps:
            gcfac = 0.0
            ncg = 0
        else:
            if gcnorm0 > EPS_DP:
                gcfac = gcnorm1 / gcnorm0
                if gcfac > 3.0:
                    gcfac = 0.0
                    ncg = 0
                else:
                    ncg += 1
            else:
                gcfac = 0.0
                ncg = 0
        gcnorm0 = gcnorm1
        cdq = cdodq_p + cdqkeep * gcfac
        if lrandom:
            raise NotImplementedError("conv_noise_amp > 0 is not restated in the oracle")
        doda0 = -float(np.vdot(cdodq, cdq).real) / (4.0 * wbtot)
        if doda0 > 0.0:
            if ncg > 0:
                cdq = cdodq.copy()
                ncg = 0
                gcfac = 0.0
                doda0 = -float(np.vdot(cdodq, cdq).real) / (4.0 * wbtot)
                if doda0 > 0.0:
                    cdq = -cdq
                    doda0 = -doda0
            else:
                cdq = -cdq
                doda0 = -doda0
        lrandom = False
        cdqkeep = cdq.copy()                                          # :595

        if ctl.lfixstep:
            alphamin = ctl.fixed_step
            lquad = False
        else:
            cdq_t = cdqkeep * (ctl.trial_step / (4.0 * wbtot))        # :605
            U0, M0 = U, M
            U, M = new_u_and_m(cdq_t, U0, M0, nnlist, sitesym)
            if update_noise is not None:
                M = update_noise(M)
            trial_spread, rave, r2ave, rave2 = wann_omega(M, km, om_invariant, sheet=sheet, slwf=slwf)
            # internal_optimal_step (:1528-1596)
            fac = trial_spread.om_tot - wann_spread.om_tot
            if abs(fac) > TINY_DP:
                fac = 1.0 / fac
                shift = 1.0
            else:
                fac = 1.0e6
                shift = fac * trial_spread.om_tot - fac * wann_spread.om_tot
            eqb = fac * doda0
            eqa = shift - eqb * ctl.trial_step
            if abs(eqa / (fac * wann_spread.om_tot)) > EPS_DP:
                lquad = True
                alphamin = -0.5 * eqb / eqa * (ctl.trial_step ** 2)
            else:
                lquad = False
                alphamin = ctl.trial_step
            if doda0 * alphamin > 0.0:
                lquad = False
                alphamin = ctl.trial_step

        if ctl.lfixstep or lquad:
            cdq_a = cdqkeep * (alphamin / (4.0 * wbtot))              # :665
            if not ctl.lfixstep:
                U, M = U0, M0
            U, M = new_u_and_m(cdq_a, U, M, nnlist, sitesym)
            if update_noise is not None:
                M = update_noise(M)
            old_spread = wann_spread.copy()
            wann_spread, rave, r2ave, rave2 = wann_omega(M, km, om_invariant, sheet=sheet, slwf=slwf)
        else:
            old_spread = wann_spread.copy()
            wann_spread = trial_spread.copy()

        if record:
            res.iters.append(IterRecord(it, wann_spread.om_tot - old_spread.om_tot,
                                        math.sqrt(abs(gcnorm1)), wann_spread.copy(),
                                        rave.copy(), r2ave - rave2, lquad, alphamin))

        if ctl.conv_window > 1:                                       # :799-805
            # internal_test_convergence (:1076-1164)
            delta = wann_spread.om_tot - old_spread.om_tot
            if it <= ctl.conv_window:
                history[it - 1] = delta
            else:
                history = np.concatenate([history[1:], [delta]])
            conv_count += 1
            if conv_count >= ctl.conv_window and np.all(np.abs(history) <= ctl.conv_tol):
                if ctl.conv_noise_amp > 0.0 and noise_count < ctl.conv_noise_num:
                    if lfirst:
                        lfirst = False
                        save_spread = wann_spread.om_tot
                        lrandom = True
                        conv_count = 0
                    else:
                        if abs(save_spread - wann_spread.om_tot) < ctl.conv_tol:
                            lconverged = True
                        else:
                            save_spread = wann_spread.om_tot
                            lrandom = True
                            conv_count = 0
                    if lrandom:
                        noise_count += 1
                else:
                    lconverged = True
        if lconverged:
            break

    res.U, res.M = U, M
    res.spread = wann_spread
    res.centres = rave
    res.spreads = r2ave - rave2
    res.converged = lconverged
    res.niter = it
    check_unitarity(U)
    return res


def check_unitarity(U, tol=EPS5):
    """wann_check_unitarity (src/wannierise.F90:2594-2661)."""
    K, W, _ = U.shape
    eye = np.eye(W)
    a = U @ np.conj(np.swapaxes(U, 1, 2))
    b = np.conj(np.swapaxes(U, 1, 2)) @ U
    if np.max(np.abs(a - eye)) > tol or np.max(np.abs(b - eye)) > tol:
        raise RuntimeError("wann_check_unitarity: U not unitary")
    return True
