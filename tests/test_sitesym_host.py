"""Symmetry-adapted mode (site_symmetry = T), host side and the kernels' arrangement,
without a GPU.

* the .dmn reader against the fixture's arrays (a file written in the reference's
  list-directed layout, src/sitesym.F90:698-765);
* w90g_set_sitesym's checks: the reference's count messages, index ranges, stars that
  must cover the mesh -- no index that reaches the GPU kernels can be out of range;
* the arrangement k_sitesym.cu uses, restated in NumPy: the search direction formed at
  the irreducible k and rotated onto the star before the exponential (exp(s D X D^+) =
  D exp(s X) D^+) reproduces the oracle's trajectory, where the reference rotates dU.
"""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G
from wannier90_gb300 import library as w90
from wannier90_gb300 import w90io


def _handle(d, **opts):
    kn = d["knobs"]
    c = w90.w90_create()
    w90.w90_set_option(c, "kpoints", d["kpt_latt"])
    w90.w90_set_option(c, "num_wann", int(kn["num_wann"]))
    w90.w90_set_option(c, "unit_cell_cart", d["real_lattice"])
    w90.w90_set_option(c, "search_shells", int(kn["search_shells"]))
    w90.w90_set_option(c, "iprint", 0)
    for k, v in opts.items():
        w90.w90_set_option(c, k, v)
    return c, w90.w90_input_setopt(c)


def test_read_dmn_matches_fixture(tmp_path):
    d = G.load("sitesym21")
    f = str(tmp_path / "s.dmn")
    G.write_dmn(f, d)
    r = w90io.read_dmn(f, 4)
    assert (r["num_bands"], r["nsymmetry"], r["nkptirr"], r["num_kpts"]) == (4, 24, 10, 64)
    np.testing.assert_array_equal(r["ik2ir"], d["ik2ir"])
    np.testing.assert_array_equal(r["ir2ik"], d["ir2ik"])
    np.testing.assert_array_equal(r["kptsym"], d["kptsym"])
    np.testing.assert_allclose(r["d_matrix_wann"], d["d_matrix_wann"].transpose(2, 3, 1, 0), atol=1e-10)
    np.testing.assert_allclose(r["d_matrix_band"], d["d_matrix_band"].transpose(2, 3, 1, 0), atol=1e-10)


def test_set_sitesym_accepts_the_reference_data():
    d = G.load("sitesym21")
    c, ierr = _handle(d, site_symmetry=True, symmetrize_eps=1e-9)
    assert ierr == 0, c.last_error()
    assert w90.w90_set_sitesym(c, G.dmn_dict(d)) == 0, c.last_error()


def _bad(d, key, fn):
    x = G.dmn_dict(d)
    x[key] = fn(x[key])
    return x


@pytest.mark.parametrize("mutate,code,msg", [
    (lambda d: {**G.dmn_dict(d), "num_bands": 5}, 6, "Number of bands is not correct (sitesym_read)"),
    (lambda d: {**G.dmn_dict(d), "num_kpts": 63}, 6, "Number of k-points is not correct (sitesym_read)"),
    (lambda d: _bad(d, "kptsym", lambda a: np.where(a == 17, 65, a)), 6, "kptsym out of range"),
    (lambda d: _bad(d, "kptsym", lambda a: np.where(a == 17, 0, a)), 6, "kptsym out of range"),
    (lambda d: _bad(d, "ik2ir", lambda a: np.where(a == 3, 11, a)), 6, "ik2ir out of range"),
    (lambda d: _bad(d, "ir2ik", lambda a: np.where(a == 28, 27, a)), 6, "ik2ir and ir2ik disagree"),
    # a k-point that no star reaches
    (lambda d: _bad(d, "kptsym", lambda a: np.where(a == 64, 2, a)), 1, "error in sitesym_symmetrize_rotation"),
])
def test_set_sitesym_errors(mutate, code, msg):
    d = G.load("sitesym21")
    c, ierr = _handle(d, site_symmetry=True)
    assert ierr == 0
    assert w90.w90_set_sitesym(c, mutate(d)) == code
    assert msg in c.last_error()


def test_site_symmetry_needs_its_data():
    d = G.load("sitesym21")
    # entangled bands are accepted; the data must then carry num_bands bands
    c, ierr = _handle(d, site_symmetry=True, num_bands=6)
    assert ierr == 0, c.last_error()
    assert w90.w90_set_sitesym(c, G.dmn_dict(d)) == 6
    assert "Number of bands is not correct" in c.last_error()
    # site_symmetry = T without w90g_set_sitesym: the projection stops before the device
    c, ierr = _handle(d, site_symmetry=True)
    assert ierr == 0
    K = len(d["kpt_latt"])
    m = np.zeros((4, 4, 8, K), dtype=np.complex128, order="F")
    u = np.zeros((4, 4, K), dtype=np.complex128, order="F")
    w90.w90_set_m_local(c, m)
    w90.w90_set_u_matrix(c, u)
    assert w90.w90_project_overlap(c) == 6
    assert "w90g_set_sitesym" in c.last_error()


def test_rotated_direction_reproduces_the_rotated_rotation():
    """k_sym_dir rotates the search direction onto the star and the exp kernels then
    exponentiate every k; the reference exponentiates at the irreducible k and rotates
    dU.  Same trajectory to roundoff over the whole example21 run."""
    d = G.load("sitesym21")
    sym = G.sitesym(d)
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"], int(d["knobs"]["search_shells"]))
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    U0, M0 = O.overlap_project(M, d["amn"], km["nnlist"], sitesym=sym)
    ctl = G.control(d)
    ref = O.wann_main(M0, U0, km, ctl, sitesym=sym)
    orig = O.new_u_and_m

    def rotated_direction(cdq, U, M, nnlist, sitesym=None):
        X = cdq.copy()
        done = np.zeros(len(X), dtype=bool)
        for ir in range(sitesym.nkirr):
            ik = sitesym.ir2ik[ir]
            done[ik] = True
            for isym in range(1, sitesym.nsym):
                irk = sitesym.kptsym[isym, ir]
                if done[irk]:
                    continue
                done[irk] = True
                D = sitesym.d_wann[ir, isym]
                X[irk] = D @ (X[ik] @ D.conj().T)
        return orig(X, U, M, nnlist)

    try:
        O.new_u_and_m = rotated_direction
        got = O.wann_main(M0, U0, km, ctl, sitesym=sym)
    finally:
        O.new_u_and_m = orig
    for a, b in zip([ref.initial] + ref.iters, [got.initial] + got.iters):
        assert abs(a.spread.om_tot - b.spread.om_tot) < 1e-12
    np.testing.assert_allclose(got.U, ref.U, atol=1e-10)
