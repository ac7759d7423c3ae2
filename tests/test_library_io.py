"""Library-mode input and file entry points on the host (no GPU): cinput_reader /
cinput_reader_special (.win keywords), coverlaps (.mmn/.amn into the caller's buffers),
cchkpt (.chk) against the records of the reference's shipped checkpoint, and
cset_kpoint_distribution."""
import ctypes as C
import os
import struct

import numpy as np
import pytest

from tests import golden_cases as G
from wannier90_gb300 import library as w90
from wannier90_gb300 import synth, w90io


def _records(path):
    out = []
    with open(path, "rb") as f:
        while True:
            h = f.read(4)
            if not h:
                return out
            (n,) = struct.unpack("<i", h)
            out.append(f.read(n))
            assert struct.unpack("<i", f.read(4))[0] == n


def _win(path, lattice, kpts, mp, nw, **kw):
    w90io.write_win(path, lattice, kpts, mp, nw, **kw)


def _small():
    return synth.make_problem(kind="fcc", a=6.0, mp=(3, 3, 3), num_wann=5, rmax=1, eps=0.3, seed=4)


def test_input_reader_special_matches_setopt(tmp_path):
    p = _small()
    seed = str(tmp_path / "x")
    _win(seed + ".win", p.real_lattice, p.kpoints, p.mp_grid, 5, num_iter=7, search_shells=12, iprint=0)
    a = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=5, iprint=0)
    b = w90.w90_create()
    assert w90.w90_input_reader_special(b, seed) == 0, b.last_error()
    K = len(p.kpoints)
    assert w90.w90_get_nn(b) == w90.w90_get_nn(a)
    np.testing.assert_array_equal(w90.w90_get_nnkp(b, K), w90.w90_get_nnkp(a, K))
    np.testing.assert_array_equal(w90.w90_get_gkpb(b, K), w90.w90_get_gkpb(a, K))


def test_input_reader_keywords_and_errors(tmp_path):
    p = _small()
    seed = str(tmp_path / "x")

    def handle():
        return w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=5, seedname=seed, iprint=0)

    def write(text):
        with open(seed + ".win", "w") as f:
            f.write(text)

    # keywords the engine uses, comments, ':' and blank separators, Fortran reals, ranges
    write("! comment\nnum_iter : 50\nconv_tol = 1.d-12 # trailing\nconv_window 4\nexclude_bands : 1-3, 7\n"
          "dis_mix_ratio = 0.5\nwrite_hr = .true.\nbands_plot = false\n")
    c = handle()
    assert w90.w90_input_reader(c) == 0, c.last_error()
    # the setup is redone with the .win's keywords: an invalid one is reported as setopt does
    write("dis_mix_ratio = 2.0\n")
    c = handle()
    assert w90.w90_input_reader(c) == 5
    assert "dis_mix_ratio" in c.last_error()
    write("fixed_step = 1.0\ntrial_step = 2.0\n")
    c = handle()
    assert w90.w90_input_reader(c) == 5 and "fixed_step and trial_step" in c.last_error()
    write("num_iter = 5\nnot_a_keyword = 1\n")
    c = handle()
    assert w90.w90_input_reader(c) == 5 and "Unrecognised keyword" in c.last_error()
    write("num_iter = 5\nnum_iter = 6\n")
    c = handle()
    assert w90.w90_input_reader(c) == 5 and "more than once" in c.last_error()
    write("num_wann = 6\n")
    c = handle()
    assert w90.w90_input_reader(c) == 5 and "num_wann" in c.last_error()
    write("num_iter = abc\n")
    c = handle()
    assert w90.w90_input_reader(c) == 5
    write("begin projections\nf=0,0,0:s\n")
    c = handle()
    assert w90.w90_input_reader(c) == 5 and "Ending tag" in c.last_error()
    os.remove(seed + ".win")
    c = handle()
    assert w90.w90_input_reader(c) == 6
    # options set after cinput_setopt and not consumed: the reader refuses (setopt first)
    write("num_iter = 5\n")
    c = handle()
    w90.w90_set_option(c, "num_iter", 3)
    assert w90.w90_input_reader(c) == 1


def test_overlaps_reads_seed_files_into_caller_buffers(tmp_path):
    p = _small()
    seed = str(tmp_path / "x")
    w90io.write_mmn(seed + ".mmn", p.m, p.nnlist, p.nncell)
    w90io.write_amn(seed + ".amn", p.a)
    c = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=5, seedname=seed, iprint=0)
    K, B = len(p.kpoints), c.nntot
    assert w90.w90_overlaps(c) == 1 and "not associated" in c.last_error()
    m = np.zeros((5, 5, B, K), dtype=np.complex128, order="F")
    u = np.zeros((5, 5, K), dtype=np.complex128, order="F")
    w90.w90_set_m_local(c, m)
    w90.w90_set_u_matrix(c, u)
    assert w90.w90_overlaps(c) == 0, c.last_error()
    np.testing.assert_allclose(c._keep["m"], p.m, atol=1e-11)
    np.testing.assert_allclose(c._keep["u"], p.a, atol=1e-11)
    # with cset_a_matrix the projections go there instead
    a = np.zeros((5, 5, K), dtype=np.complex128, order="F")
    w90.w90_set_a_matrix(c, a)
    assert w90.w90_overlaps(c) == 0
    np.testing.assert_allclose(c._keep["a"], p.a, atol=1e-11)


def test_kpoint_distribution_single_rank_only(tmp_path):
    p = _small()
    seed = str(tmp_path / "x")
    w90io.write_mmn(seed + ".mmn", p.m, p.nnlist, p.nncell)
    w90io.write_amn(seed + ".amn", p.a)
    c = w90.setup(kpoints=p.kpoints, unit_cell_cart=p.real_lattice, num_wann=5, seedname=seed, iprint=0)
    K, B = len(p.kpoints), c.nntot
    w90.w90_set_m_local(c, np.zeros((5, 5, B, K), dtype=np.complex128, order="F"))
    w90.w90_set_u_matrix(c, np.zeros((5, 5, K), dtype=np.complex128, order="F"))
    w90.w90_set_u_opt(c, np.zeros((5, 5, K), dtype=np.complex128, order="F"))
    w90.w90_set_parallel_comms(c, 0)
    w90.w90_set_kpoint_distribution(c, np.zeros(K, dtype=np.int32))
    assert w90.w90_overlaps(c) == 0, c.last_error()
    dist = np.zeros(K, dtype=np.int32)
    dist[K // 2:] = 1
    w90.w90_set_kpoint_distribution(c, dist)
    assert w90.w90_overlaps(c) == 5 and "single-GPU" in c.last_error()
    # the host-side check comes before any GPU work
    assert w90.w90_project_overlap(c) == 5
    assert w90.w90_wannierise(c) == 5


@pytest.mark.parametrize("writer", ["cchkpt", "python"])
def test_chk_records_match_reference_checkpoint(tmp_path, writer):
    """testw90_example02_restart's lead.chk.fmt (the formatted image of a wannier90.x .chk,
    src/wannier90_readwrite.F90:2336-2366): the checkpoint written from the same state
    holds the same records in the same order -- header, num_bands, exclude list, the real
    and reciprocal lattice records, k-points, nntot, num_wann, label, have_disentangled,
    U, M, centres, spreads."""
    d = G.load("restart02")
    W, K, B = 4, len(d["kpt_latt"]), int(d["nntot"])
    u = np.asfortranarray(d["u"].transpose(1, 2, 0))
    m = np.asfortranarray(d["m"].transpose(2, 3, 1, 0))
    cen, spr = d["chk_centres"], d["chk_spreads"]
    seed = str(tmp_path / "lead")
    if writer == "python":
        w90io.write_chk(seed + ".chk", num_bands=W, lattice=d["real_lattice"], kpts=d["kpt_latt"],
                        mp_grid=d["mp_grid"], nntot=B, num_wann=W, u=u, m=m, centres=cen.T, spreads=spr,
                        checkpoint=str(d["chk_label"]), header=str(d["chk_header"]))
    else:
        c = w90.setup(kpoints=d["kpt_latt"], unit_cell_cart=d["real_lattice"], num_wann=W, mp_grid=d["mp_grid"],
                      seedname=seed, iprint=0)
        w90.w90_set_m_local(c, m.copy(order="F"))
        w90.w90_set_u_matrix(c, u.copy(order="F"))
        w90.w90_set_u_opt(c, np.asfortranarray(np.broadcast_to(np.eye(W, dtype=np.complex128)[:, :, None],
                                                                (W, W, K)).copy()))
        assert w90.w90_write_chkpt(c, str(d["chk_label"])) == 0, c.last_error()
    r = _records(seed + ".chk")
    assert len(r) == 17
    if writer == "python":
        assert r[0].decode() == str(d["chk_header"])[:33].ljust(33)
    else:
        assert len(r[0]) == 33 and r[0].decode().startswith("written on ")
    assert struct.unpack("<i", r[1])[0] == int(d["chk_num_bands"])
    assert struct.unpack("<i", r[2])[0] == len(d["chk_exclude"]) and r[3] == b""
    np.testing.assert_allclose(np.frombuffer(r[4], "<f8"), d["chk_lattice9"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(np.frombuffer(r[5], "<f8"), d["chk_recip9"], rtol=1e-15, atol=2e-16)
    assert struct.unpack("<i", r[6])[0] == K
    np.testing.assert_array_equal(np.frombuffer(r[7], "<i4"), d["chk_mp_grid"])
    np.testing.assert_array_equal(np.frombuffer(r[8], "<f8").reshape(K, 3), d["kpt_latt"])
    assert struct.unpack("<i", r[9])[0] == B and struct.unpack("<i", r[10])[0] == W
    assert r[11].decode().strip() == str(d["chk_label"]) and len(r[11]) == 20
    assert struct.unpack("<i", r[12])[0] == int(d["chk_have_dis"]) == 0
    np.testing.assert_array_equal(np.frombuffer(r[13], "<c16"), u.reshape(-1, order="F"))
    np.testing.assert_array_equal(np.frombuffer(r[14], "<c16"), m.reshape(-1, order="F"))
    if writer == "python":
        np.testing.assert_array_equal(np.frombuffer(r[15], "<f8").reshape(W, 3), cen)
        np.testing.assert_array_equal(np.frombuffer(r[16], "<f8"), spr)
    else:
        assert len(r[15]) == 8 * 3 * W and len(r[16]) == 8 * W
    # and the reader takes it back
    chk = w90io.read_chk(seed + ".chk")
    np.testing.assert_array_equal(chk["u"], u)
    np.testing.assert_array_equal(chk["m"], m)
