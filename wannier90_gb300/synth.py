"""Seeded tight-binding Wannierisation problems (synthetic stand-ins for DFT inputs).

A problem is what Wannier90 reads from ``.win/.mmn/.amn`` for an isolated group of
bands: the lattice, a Monkhorst-Pack k-mesh, overlaps M_mn(k,b) and projections
A_mn(k).  They are generated from a random tight-binding model:

* W orbitals at uniform random fractional positions tau (Cartesian tau = tau_frac . A);
* hoppings H(R) for all integer R with |R|_inf <= rmax, complex Gaussian entries
  (re, im ~ N(0,1)/sqrt 2) scaled by exp(-|R_cart| / (0.7 a)); H(-R) = H(R)^dagger,
  H(0) = (X + X^dagger)/2;
* Bloch Hamiltonian H(k) = sum_R H(R) e^{2 pi i k.R} (periodic gauge, H(k+G) = H(k)),
  eigenvectors C(k) (all W bands kept);
* M_mn(k,b) = sum_a conj(C_am(k)) C_an(k+b) e^{-i b.tau_a}, with k+b folded into the mesh;
* A(k) = C(k)^dagger exp(eps X_k), X_k a seeded anti-Hermitian matrix (entries N(0,1)),
  independent per k: the orbital basis rotated by a random unitary.

The b-vectors come from the engine's own k-mesh construction (``cinput_setopt``), so
the overlaps are laid out exactly as the engine (and Wannier90) index them.
Arrays returned are Fortran-ordered like the reference's library arguments:
``m`` (W, W, B, K), ``a`` (W, W, K) complex128.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import library as w90


@dataclass
class TBProblem:
    real_lattice: np.ndarray   # (3,3) rows a_i, Angstrom
    kpoints: np.ndarray        # (K,3) fractional
    mp_grid: tuple
    num_wann: int
    nntot: int
    nnlist: np.ndarray         # (K,B) 0-based
    nncell: np.ndarray         # (K,B,3)
    bk: np.ndarray             # (K,B,3) Cartesian
    m: np.ndarray              # (W,W,B,K) F-order complex128, raw overlaps
    a: np.ndarray              # (W,W,K)   F-order complex128, projections
    tau: np.ndarray            # (W,3) Cartesian orbital positions
    seed: int


def lattice(kind: str, a: float) -> np.ndarray:
    if kind == "sc":
        return np.eye(3) * a
    if kind == "fcc":
        return 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])
    if kind == "bcc":
        return 0.5 * a * np.array([[-1.0, 1.0, 1.0], [1.0, -1.0, 1.0], [1.0, 1.0, -1.0]])
    raise ValueError(kind)


def mp_kpoints(n1, n2, n3) -> np.ndarray:
    """Gamma-centred Monkhorst-Pack grid, last index fastest (utility/kmesh.pl order)."""
    g = np.array([[i / n1, j / n2, k / n3] for i in range(n1) for j in range(n2) for k in range(n3)])
    return g


def kmesh_tables(real_lattice, kpoints, search_shells=36):
    """nnlist / nncell / bk from the engine's k-mesh (CPU-only library calls)."""
    K = len(kpoints)
    c = w90.setup(kpoints=kpoints, unit_cell_cart=real_lattice, num_wann=1, iprint=0,
                  search_shells=search_shells)
    B = w90.w90_get_nn(c)
    nnkp = w90.w90_get_nnkp(c, K)          # (K,B) 1-based
    gkpb = w90.w90_get_gkpb(c, K)          # (3,K,B)
    nnlist = np.asarray(nnkp, dtype=np.int64) - 1
    nncell = np.transpose(gkpb, (1, 2, 0)).astype(np.int64)
    a = np.asarray(real_lattice, dtype=np.float64)
    recip = 2 * math.pi * np.linalg.inv(a).T
    bfrac = kpoints[nnlist] + nncell - kpoints[:, None, :]
    bk = bfrac @ recip
    return B, nnlist, nncell, bk


def _tb_bands(rng, kind, a, mp, norb, rmax, onsite=None):
    """Random tight-binding model with `norb` orbitals: lattice, k-points, orbital
    positions, band energies E[k, m] (ascending) and eigenvectors C[k, :, m].  `onsite`
    (length norb) is added to the diagonal of H(R = 0)."""
    A = lattice(kind, a)
    kp = mp_kpoints(*mp)
    K = len(kp)
    tau_frac = rng.random((norb, 3))
    tau = tau_frac @ A
    # hoppings
    rng_R = np.arange(-rmax, rmax + 1)
    Rs = np.array([[i, j, k] for i in rng_R for j in rng_R for k in rng_R], dtype=np.float64)
    nR = len(Rs)
    half = [r for r in range(nR) if tuple(Rs[r]) > (0.0, 0.0, 0.0)]
    HR = np.zeros((nR, norb, norb), dtype=np.complex128)
    idx = {tuple(r): i for i, r in enumerate(Rs)}
    for r in half:
        x = (rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb))) / math.sqrt(2.0)
        Rc = Rs[r] @ A
        x *= math.exp(-np.linalg.norm(Rc) / (0.7 * a))
        HR[r] = x
        HR[idx[tuple(-Rs[r])]] = x.conj().T
    x0 = (rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb))) / math.sqrt(2.0)
    HR[idx[(0.0, 0.0, 0.0)]] = 0.5 * (x0 + x0.conj().T)
    if onsite is not None:
        HR[idx[(0.0, 0.0, 0.0)]] += np.diag(np.asarray(onsite, dtype=np.float64))
    # Bloch Hamiltonians and eigenvectors
    ph = np.exp(2j * math.pi * (kp @ Rs.T))                      # (K, nR)
    Hk = (ph @ HR.reshape(nR, norb * norb)).reshape(K, norb, norb)
    Hk = 0.5 * (Hk + np.conj(np.swapaxes(Hk, 1, 2)))
    Ek, Ck = np.linalg.eigh(Hk)                                    # columns = bands
    return A, kp, tau, Ek, Ck


def _tb_overlaps(A, kp, tau, Ck, search_shells, kmesh=None):
    """M_mn(k,b) = sum_a conj(C_am(k)) C_an(k+b) e^{-i b.tau_a} on the engine's k-mesh
    (or on the tables ``kmesh(real_lattice, kpoints, search_shells)`` returns, a
    (B, nnlist, nncell, bk) tuple in kmesh_tables' layout)."""
    B, nnlist, nncell, bk = (kmesh or kmesh_tables)(A, kp, search_shells)
    phase = np.exp(-1j * np.einsum("kbi,ai->kba", bk, tau))        # (K,B,norb)
    Ckp = Ck[nnlist]                                               # (K,B,norb,norb)
    M = np.conj(Ck)[:, None].transpose(0, 1, 3, 2) @ (phase[..., None] * Ckp)   # [k,b,m,n]
    return B, nnlist, nncell, bk, M


def _random_unitaries(rng, K, W, eps):
    """exp(eps X_k), X_k seeded anti-Hermitian with N(0,1) entries."""
    Xk = rng.standard_normal((K, W, W)) + 1j * rng.standard_normal((K, W, W))
    Xk = 0.5 * (Xk - np.conj(np.swapaxes(Xk, 1, 2)))
    ev, V = np.linalg.eigh(1j * eps * Xk)                          # exp(eps X) = V e^{-i ev} V^H
    return (V * np.exp(-1j * ev)[:, None, :]) @ np.conj(np.swapaxes(V, 1, 2))


def make_problem(kind="sc", a=5.0, mp=(4, 4, 4), num_wann=8, rmax=2, eps=0.3, seed=0,
                 search_shells=36, kmesh=None) -> TBProblem:
    """``kmesh``: optional k-mesh builder with kmesh_tables' signature and result; by
    default the engine's own (which loads the C library)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    W = int(num_wann)
    A, kp, tau, _, Ck = _tb_bands(rng, kind, a, mp, W, rmax)
    K = len(kp)
    B, nnlist, nncell, bk, M = _tb_overlaps(A, kp, tau, Ck, search_shells, kmesh)
    # projections
    Ek = _random_unitaries(rng, K, W, eps)
    Amat = np.conj(np.swapaxes(Ck, 1, 2)) @ Ek                     # [k,m,n]
    m = np.asfortranarray(M.transpose(2, 3, 1, 0))
    af = np.asfortranarray(Amat.transpose(1, 2, 0))
    return TBProblem(A, kp, tuple(mp), W, B, nnlist, nncell, bk, m, af, tau, seed)


@dataclass
class EntangledProblem:
    """Input of the disentanglement step: num_bands > num_wann bands per k-point."""
    real_lattice: np.ndarray
    kpoints: np.ndarray
    mp_grid: tuple
    num_bands: int
    num_wann: int
    nntot: int
    nnlist: np.ndarray
    nncell: np.ndarray
    bk: np.ndarray
    m: np.ndarray              # (nb,nb,B,K) F-order complex128, raw overlaps
    a: np.ndarray              # (nb,W,K)    F-order complex128, projections
    eig: np.ndarray            # (nb,K)      F-order float64, band energies (ascending)
    tau: np.ndarray
    seed: int


def make_entangled_problem(kind="sc", a=5.0, mp=(4, 4, 4), num_bands=12, num_wann=8, rmax=2, eps=0.3,
                           seed=0, search_shells=36, offset=0.0) -> EntangledProblem:
    """Tight-binding model with num_bands orbitals, all bands kept; the trial orbitals are
    the first num_wann orbitals rotated by a seeded random unitary per k, so
    A_mn(k) = sum_{a < num_wann} conj(C_am(k)) (exp(eps X_k))_an.  `offset` raises the
    on-site energy of the other num_bands - num_wann orbitals, which then form bands
    above the target manifold that overlap it only partly (offset 0: fully mixed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nb, W = int(num_bands), int(num_wann)
    onsite = np.concatenate([np.zeros(W), np.full(nb - W, float(offset))]) if offset else None
    A, kp, tau, Ek, Ck = _tb_bands(rng, kind, a, mp, nb, rmax, onsite)
    K = len(kp)
    B, nnlist, nncell, bk, M = _tb_overlaps(A, kp, tau, Ck, search_shells)
    G = np.zeros((K, nb, W), dtype=np.complex128)
    G[:, :W, :] = _random_unitaries(rng, K, W, eps)
    Amat = np.conj(np.swapaxes(Ck, 1, 2)) @ G                      # [k,m,n]
    return EntangledProblem(A, kp, tuple(mp), nb, W, B, nnlist, nncell, bk,
                            np.asfortranarray(M.transpose(2, 3, 1, 0)),
                            np.asfortranarray(Amat.transpose(1, 2, 0)),
                            np.asfortranarray(Ek.T), tau, seed)


def entangled_windows(eig, W):
    """Outer and frozen windows for an entangled problem (eig[k, nb]): the outer window
    drops the lowest band at some k-points (nfirstwin > 0), keeps >= W + 1 states
    everywhere and about half of the bands above W on average; the frozen window holds
    at most W // 2 + 1 states."""
    nb = eig.shape[1]
    return dict(win_min=float(eig[:, 1].min()),
                win_max=float(max(eig[:, W].max(), np.median(eig[:, (W + nb) // 2]))),
                froz_max=float(eig[:, W // 2].min()))


# the workloads of the benchmark configurations (sizes as named in the suite)
CONFIGS = {
    "sc4_w8": dict(kind="sc", a=5.0, mp=(4, 4, 4), num_wann=8, rmax=2, eps=0.3),
    "fcc10_w32": dict(kind="fcc", a=6.0, mp=(10, 10, 10), num_wann=32, rmax=3, eps=0.3),
    "sc8_w128": dict(kind="sc", a=5.0, mp=(8, 8, 8), num_wann=128, rmax=2, eps=0.5),
}


def to_math_m(m):
    """(W,W,B,K) Fortran array -> M[k,b,m,n]."""
    return np.ascontiguousarray(np.asarray(m).transpose(3, 2, 0, 1))


def to_math_u(u):
    return np.ascontiguousarray(np.asarray(u).transpose(2, 0, 1))


def from_math_m(M):
    return np.asfortranarray(np.asarray(M).transpose(2, 3, 1, 0))


def from_math_u(U):
    return np.asfortranarray(np.asarray(U).transpose(1, 2, 0))
