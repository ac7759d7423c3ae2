"""Wannier90 file formats (no GPU): .win/.mmn/.amn/.eig round trips, the reference's own
.mmn/.amn read through the k-mesh tables, and the unformatted .chk layout."""
import os
import struct

import numpy as np
import pytest

from tests import golden_cases as G
from wannier90_gb300 import library as w90
from wannier90_gb300 import synth, w90io

from tests.conftest import reference_root

# the reference's own example02 (lead) inputs, read from the Wannier90 source tree named
# by W90_REFERENCE; skipped without it
REF = os.path.join(reference_root() or "", "test-suite", "tests", "testw90_example02")


def _small():
    return synth.make_problem(kind="fcc", a=6.0, mp=(3, 3, 3), num_wann=5, rmax=1, eps=0.3, seed=4)


def test_mmn_amn_eig_roundtrip(tmp_path):
    p = _small()
    f = str(tmp_path / "x")
    w90io.write_mmn(f + ".mmn", p.m, p.nnlist, p.nncell)
    w90io.write_amn(f + ".amn", p.a)
    eig = np.asfortranarray(np.arange(5 * 27, dtype=float).reshape(5, 27, order="F") * 0.1)
    w90io.write_eig(f + ".eig", eig)
    m = w90io.read_mmn(f + ".mmn", p.nnlist, p.nncell)
    a = w90io.read_amn(f + ".amn")
    np.testing.assert_allclose(m, p.m, atol=1e-11)
    np.testing.assert_allclose(a, p.a, atol=1e-11)
    np.testing.assert_allclose(w90io.read_eig(f + ".eig", 5, 27), eig, atol=1e-11)


def test_win_roundtrip(tmp_path):
    p = _small()
    f = str(tmp_path / "x.win")
    w90io.write_win(f, p.real_lattice, p.kpoints, p.mp_grid, 5, num_iter=40, conv_tol="1d-9", precond=".false.")
    lat, kp, opts = w90io.win_system(f)
    np.testing.assert_allclose(lat, p.real_lattice, atol=1e-12)
    np.testing.assert_allclose(kp, p.kpoints, atol=1e-12)
    assert opts["num_wann"] == 5 and opts["num_iter"] == 40 and abs(opts["conv_tol"] - 1e-9) < 1e-24
    assert opts["precond"] == 0 and list(opts["mp_grid"]) == [3, 3, 3]


@pytest.mark.skipif(reference_root() is None, reason="W90_REFERENCE (Wannier90 source tree) not set")
def test_reads_reference_inputs():
    d = G.load("pb")
    lat, kp, opts = w90io.win_system(os.path.join(REF, "lead.win"))
    np.testing.assert_allclose(lat, d["real_lattice"], atol=1e-12)
    c = w90.setup(kpoints=kp, unit_cell_cart=lat, num_wann=4, iprint=0, search_shells=12)
    K = len(kp)
    nnkp = w90.w90_get_nnkp(c, K) - 1
    gkpb = np.transpose(w90.w90_get_gkpb(c, K), (1, 2, 0))
    m = w90io.read_mmn(os.path.join(REF, "lead.mmn"), nnkp, gkpb)
    M = G.assemble_m(d, nnkp, gkpb)           # independent parser of the same file
    np.testing.assert_array_equal(synth.to_math_m(m), M)
    a = w90io.read_amn(os.path.join(REF, "lead.amn"))
    np.testing.assert_array_equal(a.transpose(2, 0, 1), d["amn"])


def test_chk_layout(tmp_path):
    p = _small()
    u = np.asfortranarray(np.broadcast_to(np.eye(5, dtype=complex)[:, :, None], (5, 5, 27)).copy())
    cen = np.asfortranarray(np.arange(15, dtype=float).reshape(3, 5))
    f = str(tmp_path / "x.chk")
    w90io.write_chk(f, num_bands=5, lattice=p.real_lattice, kpts=p.kpoints, mp_grid=(3, 3, 3), nntot=p.nntot,
                    num_wann=5, u=u, m=p.m, centres=cen, spreads=np.ones(5))
    r = w90io.read_chk(f)
    assert r["num_bands"] == 5 and r["num_kpts"] == 27 and r["nntot"] == p.nntot and r["num_wann"] == 5
    assert r["checkpoint"] == "postwann"
    np.testing.assert_allclose(r["real_lattice"], p.real_lattice)
    np.testing.assert_allclose(r["recip_lattice"] @ p.real_lattice.T, 2 * np.pi * np.eye(3), atol=1e-12)
    np.testing.assert_array_equal(r["m"], p.m)
    np.testing.assert_array_equal(r["u"], u)
    np.testing.assert_array_equal(r["centres"], cen)
    # first record: 4-byte marker 33, 33-byte header, marker 33 (Fortran sequential)
    raw = open(f, "rb").read(41)
    assert struct.unpack("<i", raw[:4])[0] == 33 and struct.unpack("<i", raw[37:41])[0] == 33


def test_chk_disentangled_records(tmp_path):
    """have_disentangled = T adds omega_invariant, lwindow(nb,nk), ndimwin(nk) and
    u_matrix_opt(nb,nw,nk) before U (src/wannier90_readwrite.F90:2356-2363)."""
    p = _small()
    nb, nw, nk = 8, 5, 27
    rng = np.random.default_rng(3)
    u = np.asfortranarray(np.broadcast_to(np.eye(nw, dtype=complex)[:, :, None], (nw, nw, nk)).copy())
    uopt = np.asfortranarray(rng.standard_normal((nb, nw, nk)) + 1j * rng.standard_normal((nb, nw, nk)))
    ndim = rng.integers(nw, nb + 1, nk).astype(np.int32)
    lwin = np.zeros((nb, nk), dtype=bool, order="F")
    for k in range(nk):
        lwin[:ndim[k], k] = True
    cen = np.asfortranarray(np.arange(3 * nw, dtype=float).reshape(3, nw))
    f = str(tmp_path / "d.chk")
    w90io.write_chk(f, num_bands=nb, lattice=p.real_lattice, kpts=p.kpoints, mp_grid=(3, 3, 3), nntot=p.nntot,
                    num_wann=nw, u=u, m=p.m, centres=cen, spreads=np.ones(nw),
                    dis=dict(omega_invariant=12.5, lwindow=lwin, ndimwin=ndim, u_opt=uopt))
    r = w90io.read_chk(f)
    assert r["have_disentangled"] and r["omega_invariant"] == 12.5
    np.testing.assert_array_equal(r["lwindow"], lwin)
    np.testing.assert_array_equal(r["ndimwin"], ndim)
    np.testing.assert_array_equal(r["u_opt"], uopt)
    np.testing.assert_array_equal(r["u"], u)
    np.testing.assert_array_equal(r["m"], p.m)


def test_win_dis_keywords(tmp_path):
    p = _small()
    f = str(tmp_path / "w.win")
    w90io.write_win(f, p.real_lattice, p.kpoints, (3, 3, 3), 4, num_bands=9, dis_win_max=17.0,
                    dis_froz_max=6.4, dis_num_iter=120, dis_mix_ratio=1.0, dis_conv_tol=1e-10, dis_conv_window=3)
    _, _, o = w90io.win_system(f)
    assert o["num_bands"] == 9 and o["dis_num_iter"] == 120 and o["dis_conv_window"] == 3
    assert o["dis_win_max"] == 17.0 and o["dis_froz_max"] == 6.4 and o["dis_mix_ratio"] == 1.0
    assert o["dis_conv_tol"] == 1e-10 and "dis_win_min" not in o


def _fortranish(path):
    """Rewrite a seed file the way other writers format it: 'D' exponents, commas, a blank
    record every few records, trailing items after the values."""
    lines = open(path).read().split("\n")
    out = lines[:2]
    for i, l in enumerate(lines[2:]):
        p = l.split()
        if len(p) == 2:
            out.append(("  %.14E, %.14E   trailing" % (float(p[0]), float(p[1]))).replace("E", "D"))
        else:
            out.append(l)
        if i % 7 == 3:
            out.append("   ")
    open(path, "w").write("\n".join(out))


@pytest.mark.parametrize("threads", [1, 3, 0])
def test_native_readers_match_record_reader(tmp_path, threads):
    """The parallel native .mmn/.amn/.eig readers against the record-by-record checker,
    bit for bit, on plain files and on files with D exponents, commas, blank records and
    trailing items; any thread count gives the same arrays."""
    from tests import seed_reference as R
    p = _small()
    f = str(tmp_path / "s")
    w90io.write_mmn(f + ".mmn", p.m, p.nnlist, p.nncell)
    w90io.write_amn(f + ".amn", p.a)
    eig = np.asfortranarray(np.sort(np.random.default_rng(2).standard_normal((5, 27)), axis=0))
    w90io.write_eig(f + ".eig", eig)
    for variant in (False, True):
        if variant:
            _fortranish(f + ".mmn")
        m = w90io.read_mmn(f + ".mmn", p.nnlist, p.nncell, nthreads=threads)
        np.testing.assert_array_equal(m, R.read_mmn(f + ".mmn", p.nnlist, p.nncell))
    np.testing.assert_array_equal(w90io.read_amn(f + ".amn", nthreads=threads), R.read_amn(f + ".amn"))
    np.testing.assert_array_equal(w90io.read_eig(f + ".eig", 5, 27), R.read_eig(f + ".eig", 5, 27))


def test_native_reader_errors_and_duplicates(tmp_path):
    """overlap_read's checks: neighbour count, a block whose (k2, G) is no neighbour, a
    truncated file; when two blocks name the same neighbour slot the later one wins, as in
    a sequential read; the .eig band/k order check."""
    from tests import seed_reference as R
    p = _small()
    f = str(tmp_path / "e")
    w90io.write_mmn(f + ".mmn", p.m, p.nnlist, p.nncell)
    with pytest.raises(ValueError, match="number of k-points|nearest neighbours"):
        w90io.read_mmn(f + ".mmn", p.nnlist[:, :-1], p.nncell[:, :-1])
    bad = np.array(p.nncell)
    bad[0, :, 0] += 7
    with pytest.raises(ValueError, match="Neighbour not found"):
        w90io.read_mmn(f + ".mmn", p.nnlist, bad)
    txt = open(f + ".mmn").read().split("\n")
    open(f + "_t.mmn", "w").write("\n".join(txt[: len(txt) // 2]))
    with pytest.raises(ValueError, match="Problem reading"):
        w90io.read_mmn(f + "_t.mmn", p.nnlist, p.nncell)
    # block 1 relabelled as block 0's (k, k2, G): slot of block 0 takes block 1's values
    nb = p.m.shape[0]
    per = 1 + nb * nb
    dup = list(txt)
    dup[2 + per] = txt[2]
    open(f + "_d.mmn", "w").write("\n".join(dup))
    m = w90io.read_mmn(f + "_d.mmn", p.nnlist, p.nncell, nthreads=4)
    np.testing.assert_array_equal(m, R.read_mmn(f + "_d.mmn", p.nnlist, p.nncell))
    k0, k1 = 0, 0
    b0, b1 = 0, 1
    np.testing.assert_allclose(m[:, :, b0, k0], p.m[:, :, b1, k1], atol=1e-12)
    assert not m[:, :, b1, k1].any()
    w90io.write_eig(f + ".eig", np.zeros((5, 27)))
    t = open(f + ".eig").read().split("\n")
    t[3], t[4] = t[4], t[3]
    open(f + ".eig", "w").write("\n".join(t))
    with pytest.raises(ValueError, match="mismatch"):
        w90io.read_eig(f + ".eig", 5, 27)


def test_exclude_bands_range_vector(tmp_path):
    """exclude_bands ranges as the .win writes them; the CLI keeps them for the checkpoint."""
    assert w90io.parse_range_vector("1-5") == [1, 2, 3, 4, 5]
    assert w90io.parse_range_vector("1-3, 7 9-10") == [1, 2, 3, 7, 9, 10]
    with pytest.raises(ValueError):
        w90io.parse_range_vector("5-1")
    p = _small()
    f = str(tmp_path / "x.win")
    w90io.write_win(f, p.real_lattice, p.kpoints, (3, 3, 3), 4, exclude_bands="1-5")
    _, _, o = w90io.win_system(f)
    assert o["exclude_bands"] == [1, 2, 3, 4, 5]
