"""Host side of the preconditioner: the Wigner-Seitz grid of the C library against the
oracle's restatement of hamiltonian_wigner_seitz (src/hamiltonian.F90:689-853)."""
import numpy as np
import pytest

from oracle import w90_oracle as O
from tests import golden_cases as G
from wannier90_gb300 import library as w90

LATTICES = {
    "gaas_fcc": G.load("precond1")["real_lattice"],
    "sc": np.eye(3) * 5.0,
    "hex": np.array([[3.0, 0.0, 0.0], [-1.5, 3.0 * np.sqrt(3) / 2, 0.0], [0.0, 0.0, 5.0]]),
    "triclinic": np.array([[4.0, 0.3, 0.1], [0.7, 5.0, -0.2], [0.4, -0.6, 6.0]]),
}


@pytest.mark.parametrize("name", sorted(LATTICES))
@pytest.mark.parametrize("mp", [(2, 2, 2), (4, 4, 4), (3, 2, 5), (1, 1, 6)])
def test_ws_vectors_match_oracle(name, mp):
    a = LATTICES[name]
    irvec, ndegen = w90.ws_vectors(a, mp)
    ref_irvec, ref_ndegen = O.ws_vectors(a, mp)
    np.testing.assert_array_equal(irvec, ref_irvec)
    np.testing.assert_array_equal(ndegen, ref_ndegen)
    assert abs(np.sum(1.0 / ndegen) - np.prod(mp)) < 1e-9


def test_precond_needs_mp_grid():
    d = G.load("precond1")
    c = w90.w90_create()
    w90.w90_set_option(c, "kpoints", d["kpt_latt"])
    w90.w90_set_option(c, "num_wann", 4)
    w90.w90_set_option(c, "unit_cell_cart", d["real_lattice"])
    w90.w90_set_option(c, "precond", True)
    assert w90.w90_input_setopt(c) == 5
    assert "mp_grid" in c.last_error()
