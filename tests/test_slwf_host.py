"""Selective localisation: the algebra the GPU kernels use, checked on the CPU.

k_grad forms the gradient as G = (4/K)(P - P^H), P_mn = sum_b M_mn(k,b) alpha_n(k,b), with
one coefficient per column: every term of the reference's expression is X - X^H of one
(k,b) block.  With selective localisation (slwf_num = s < num_wann) the reference's
term-by-term expression (src/wannierise.F90:2431-2509) factors the same way, with two
coefficient variants per objective index j < s -- one for partners inside the objective
block, one for partners outside it -- and zero coefficients for j >= s:

    X_j = wb ln_j + (b.r_j)(1 - wb lambda) + wb lambda (b.c_j)      (both indices objective)
    Y_j = wb ln_j + wb (b.r_j)(1 - lambda) + wb lambda (b.c_j)      (partner not objective)

k_omega_p1 and k_omega_p2 form Omega_IOD + Omega_nu from per-index sums over the objective WFs and
scale Omega_D by (1 - lambda).  This file restates both in NumPy exactly as the kernels
arrange them and compares with the oracle's direct restatement.
"""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G


def kernel_gradient(M, km, slwf):
    """The factored gradient, coefficient by coefficient as k_grad computes it:
    P_mn = sum_b M_mn alpha^{v(m)}_n, then G = (4/K)(P - P^H)."""
    K, B, W, _ = M.shape
    wb, bk = km["wb"], km["bk"]
    diag = np.diagonal(M, axis1=2, axis2=3)
    ln = np.angle(diag)
    rave = -np.einsum("b,kbi,kbn->in", wb, bk, ln) / K       # the spread pass's rave
    s = slwf.num if slwf is not None else W
    lam = slwf.lam if slwf is not None else 0.0
    P_ = np.zeros((K, W, W), dtype=np.complex128)
    for k in range(K):
        for b in range(B):
            w = wb[b]
            brn = bk[k, b] @ rave
            alpha = np.zeros((2, W), dtype=np.complex128)
            for j in range(W):
                d = diag[k, b, j]
                inv = 1.0 / (d.real ** 2 + d.imag ** 2)
                if slwf is None:
                    qs = (w * (ln[k, b, j] + brn[j]),) * 2
                elif j < s:
                    r0 = bk[k, b] @ slwf.centres[:, j] if slwf.constrain else 0.0
                    qs = (w * ln[k, b, j] + brn[j] * (1.0 - w * lam) + w * lam * r0,
                          w * ln[k, b, j] + w * brn[j] * (1.0 - lam) + w * lam * r0)
                else:
                    continue
                for v, q in enumerate(qs):
                    alpha[v, j] = complex(0.5 * w * d.real + 0.5 * q * inv * d.imag,
                                          -0.5 * w * d.imag + 0.5 * q * inv * d.real)
            Mb = M[k, b]
            for m in range(W):
                P_[k, m, :] += Mb[m, :] * alpha[0 if m < s else 1, :]
    fac = 4.0 / K
    Ph = np.conj(np.swapaxes(P_, 1, 2))
    return (P_.real - Ph.real) * fac + 1j * ((P_.imag - Ph.imag) * fac)


def kernel_spread(M, km, slwf):
    """Omega terms as k_omega_p1 and k_omega_p2 arrange them (per-index chunk sums, then totals)."""
    K, B, W, _ = M.shape
    wb, bk = km["wb"], km["bk"]
    diag = np.diagonal(M, axis1=2, axis2=3)
    ln, a = np.angle(diag), np.abs(diag) ** 2
    rave = -np.einsum("b,kbi,kbn->in", wb, bk, ln) / K
    s, lam = slwf.num, slwf.lam
    bc = np.einsum("kbi,in->kbn", bk, slwf.centres) if slwf.constrain else np.zeros_like(ln)
    # pass 1: sum over (k,b) and n < s of wb (1 - |M_nn|^2 + lambda ln^2) + 2 wb lambda ln (b.c_n)
    iodnu = 0.0
    for n in range(s):
        w = wb[None, :]
        iodnu += float(np.sum(w * (1.0 - a[:, :, n] + lam * ln[:, :, n] ** 2)
                              + 2.0 * w * ln[:, :, n] * lam * bc[:, :, n]))
    # pass 2: sum wb (ln + b.r)^2 over n < s
    brn = np.einsum("kbi,in->kbn", bk, rave)
    dd = float(np.einsum("b,kbn->", wb, (ln + brn)[:, :, :s] ** 2))
    nu0 = lam * float((slwf.centres[:, :s] ** 2).sum()) if slwf.constrain else 0.0
    om_od = iodnu / K + nu0          # the reference prints this sum as O_IOD
    om_d = (1.0 - lam) * dd / K
    return om_od, om_d, om_od + om_d


def _case():
    d = G.load("slwf26")
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(d["knobs"]["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"])
    # a generic gauge: one oracle step along a random anti-Hermitian direction
    rng = np.random.default_rng(5)
    K, B, W, _ = M0.shape
    X = rng.standard_normal((K, W, W)) + 1j * rng.standard_normal((K, W, W))
    X = 0.2 * (X - np.conj(np.swapaxes(X, 1, 2)))
    _, M1 = O.new_u_and_m(X, U0, M0, km["nnlist"])
    return d, km, M1


SLWF_FORMS = [(1, 1.0, True), (2, 0.5, True), (3, 0.0, False), (2, 0.0, False), (3, 2.5, True)]


@pytest.mark.parametrize("s,lam,constrain", SLWF_FORMS)
def test_factored_gradient_equals_reference_terms(s, lam, constrain):
    d, km, M = _case()
    W = M.shape[-1]
    rng = np.random.default_rng(s)
    cen = rng.uniform(-2, 2, (3, W)) if constrain else None
    sl = O.Slwf(s, lam, cen)
    ref = O.wann_domega(M, km, slwf=sl)
    got = kernel_gradient(M, km, sl)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    # exactly anti-Hermitian, as the reference's X - X^H terms are
    assert np.array_equal(got, -np.conj(np.swapaxes(got, 1, 2)))
    # the objective block is non-zero, the non-objective block is exactly zero
    assert np.all(got[:, s:, s:] == 0)
    assert np.abs(got[:, :s, :s]).max() > 0


def test_factored_gradient_without_slwf_is_the_plain_form():
    d, km, M = _case()
    np.testing.assert_allclose(kernel_gradient(M, km, None), O.wann_domega(M, km), rtol=0, atol=1e-13)


@pytest.mark.parametrize("s,lam,constrain", SLWF_FORMS)
def test_spread_passes_equal_reference_terms(s, lam, constrain):
    d, km, M = _case()
    W = M.shape[-1]
    rng = np.random.default_rng(s)
    cen = rng.uniform(-2, 2, (3, W)) if constrain else None
    sl = O.Slwf(s, lam, cen)
    sp = O.wann_omega(M, km, slwf=sl)[0]
    om_od, om_d, om_tot = kernel_spread(M, km, sl)
    assert abs(om_od - (sp.om_iod + sp.om_nu)) < 1e-12
    assert abs(om_d - sp.om_d) < 1e-12
    assert abs(om_tot - sp.om_tot) < 1e-12


def test_gradient_is_the_derivative_of_the_functional_for_one_objective_wf():
    """slwf_num = 1: the objective block is the diagonal element, where the reference's
    b.r term (unweighted in the objective block) sums to zero over +-b pairs; the gradient
    is then exactly the derivative of Omega_tot along an anti-Hermitian direction."""
    import scipy.linalg as sla
    d, km, M = _case()
    K, B, W, _ = M.shape
    sl = O.Slwf(1, 0.7, np.random.default_rng(3).uniform(-1, 1, (3, W)))
    Gr = O.wann_domega(M, km, slwf=sl)
    rng = np.random.default_rng(11)
    X = rng.standard_normal((K, W, W)) + 1j * rng.standard_normal((K, W, W))
    X = X - np.conj(np.swapaxes(X, 1, 2))

    def om(t):
        dU = np.array([sla.expm(t * X[k]) for k in range(K)])
        Mn = np.conj(np.swapaxes(dU, 1, 2))[:, None] @ M @ dU[km["nnlist"]]
        return O.wann_omega(Mn, km, slwf=sl)[0].om_tot

    h = 1e-5
    fd = (om(h) - om(-h)) / (2 * h)
    assert abs(fd + np.vdot(Gr, X).real) < 1e-7 * max(1.0, abs(fd))


# ---------------------------------------------------------------------------
# host side of the C library: the slwf_* keywords of cinput_setopt (no GPU needed)
# (src/wannier90_readwrite.F90:757-802, :1660-1708)
# ---------------------------------------------------------------------------
def _handle(**opts):
    from wannier90_gb300 import library as w90
    d = G.load("slwf26")
    c = w90.w90_create()
    w90.w90_set_option(c, "kpoints", d["kpt_latt"])
    w90.w90_set_option(c, "num_wann", 4)
    w90.w90_set_option(c, "unit_cell_cart", d["real_lattice"])
    w90.w90_set_option(c, "search_shells", 12)
    w90.w90_set_option(c, "iprint", 0)
    for k, v in opts.items():
        w90.w90_set_option(c, k, v)
    return c, w90.w90_input_setopt(c)


@pytest.mark.parametrize("opts,msg", [
    (dict(slwf_num=0), "slwf_num must be an integer between 1 and num_wann"),
    (dict(slwf_num=5), "slwf_num must be an integer between 1 and num_wann"),
    (dict(slwf_num=2, slwf_lambda=-0.5), "slwf_lambda  must be positive"),
    (dict(slwf_num=2, slwf_constrain=True), "neither <slwf_centre> block  nor <projection_block>"),
    (dict(slwf_num=2, slwf_constrain=True, slwf_centres_frac=np.zeros((2, 3))), "num_wann x 3"),
])
def test_slwf_keyword_errors(opts, msg):
    c, ierr = _handle(**opts)
    assert ierr == 5
    assert msg in c.last_error()


@pytest.mark.parametrize("opts", [
    dict(slwf_num=4),                                        # = num_wann: the plain functional
    dict(slwf_num=4, slwf_constrain=True),                   # constraint ignored without selection
    dict(slwf_num=1),
    dict(slwf_num=1, slwf_constrain=True, slwf_centres_frac=np.full((4, 3), 0.25)),
    dict(slwf_num=3, slwf_constrain=True, guiding_centres_frac=np.zeros((4, 3)), slwf_lambda=0.0),
])
def test_slwf_keywords_accepted(opts):
    c, ierr = _handle(**opts)
    assert ierr == 0, c.last_error()


def test_win_slwf_keywords_and_centres(tmp_path):
    """.win keywords, the <slwf_centres> block over the projection sites (the default
    constrained centres), a trailing per-centre lambda read and ignored."""
    from wannier90_gb300 import w90io
    d = G.load("slwf26")
    f = str(tmp_path / "s.win")
    w90io.write_win(f, d["real_lattice"], d["kpt_latt"], (4, 4, 4), 4, slwf_num=2, slwf_constrain=".true.",
                    slwf_lambda=0.75)
    with open(f, "a") as fh:
        fh.write("begin projections\nf= 0.125, 0.125, 0.125: s\nf=0.125,0.125,-.375:s\n"
                 "f= -.375, 0.125, 0.125: s\nf= 0.125, -.375, 0.125: s\nend projections\n")
        fh.write("begin slwf_centres\n 2  0.25 0.25 0.25  1.0\nend slwf_centres\n")
    _, _, o = w90io.win_system(f)
    assert o["slwf_num"] == 2 and o["slwf_constrain"] == 1 and o["slwf_lambda"] == 0.75
    np.testing.assert_allclose(o["slwf_centres_frac"],
                               [[0.125, 0.125, 0.125], [0.25, 0.25, 0.25], [-0.375, 0.125, 0.125],
                                [0.125, -0.375, 0.125]])
