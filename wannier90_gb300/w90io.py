"""Wannier90 file formats used around the wannierisation path.

Readers: ``.win`` (keywords and blocks; src/readwrite.F90 tokenizer conventions),
``.mmn`` / ``.amn`` (src/overlap.F90:234-366), ``.eig``; writers for the same (used
to export synthetic problems that the reference ``wannier90.x`` can read) and the
unformatted checkpoint ``.chk`` (src/wannier90_readwrite.F90:2278-2373).

Arrays follow the library layouts (Fortran order):
  m   complex128 (num_bands, num_bands, nntot, num_kpts)
  a   complex128 (num_bands, num_proj, num_kpts)
  u   complex128 (num_wann, num_wann, num_kpts)
  eig float64    (num_bands, num_kpts)
"""
from __future__ import annotations

import datetime
import math
import re
import struct

import numpy as np

# src/constants.F90:109 (CODATA 2006, the default build)
BOHR_ANGSTROM = 0.52917720859


# --------------------------------------------------------------------------------
# .win
# --------------------------------------------------------------------------------
def _strip(line):
    for c in "!#":
        if c in line:
            line = line[: line.index(c)]
    return line.strip()


def read_win(path):
    """Return (keywords: dict[str, str], blocks: dict[str, list[str]]), keys lower-case."""
    lines = [_strip(l) for l in open(path)]
    lines = [l for l in lines if l]
    kw, blocks = {}, {}
    i = 0
    while i < len(lines):
        low = lines[i].lower()
        if low.startswith("begin"):
            name = low.split()[1]
            body = []
            i += 1
            while i < len(lines) and not lines[i].lower().startswith("end"):
                body.append(lines[i])
                i += 1
            blocks[name] = body
        else:
            m = re.match(r"([A-Za-z_0-9]+)\s*[=:\s]\s*(.*)", lines[i])
            if m:
                kw[m.group(1).lower()] = m.group(2).strip()
        i += 1
    return kw, blocks


def _fnum(s):
    return float(s.lower().replace("d", "e"))


def _flag(s):
    return s.strip().lower().lstrip(".").startswith("t")


def parse_range_vector(text):
    """A .win range list ("1-5, 7 9-10") as the sorted 1-based integers it names
    (w90_readwrite_get_range_vector, src/readwrite.F90)."""
    out = []
    for tok in re.split(r"[\s,]+", text.strip()):
        if not tok:
            continue
        if "-" in tok[1:]:
            a, b = tok.split("-", 1)
            lo, hi = int(a), int(b)
            if hi < lo:
                raise ValueError("range %s is decreasing" % tok)
            out.extend(range(lo, hi + 1))
        else:
            out.append(int(tok))
    return sorted(set(out))


def win_system(path):
    """Lattice (rows a_i, Angstrom), k-points (fractional), mp_grid and the wannierise
    keywords of a .win file, as library options."""
    kw, blocks = read_win(path)
    cell = blocks["unit_cell_cart"]
    scale = 1.0
    if cell[0].lower().startswith(("bohr", "ang")):
        scale = BOHR_ANGSTROM if cell[0].lower().startswith("bohr") else 1.0
        cell = cell[1:]
    lattice = np.array([[_fnum(x) for x in r.split()[:3]] for r in cell]) * scale
    kpts = np.array([[_fnum(x) for x in r.split()[:3]] for r in blocks["kpoints"]])
    opts = {}
    ints = ("num_wann", "num_bands", "num_iter", "num_cg_steps", "conv_window", "search_shells",
            "iprint", "num_print_cycles", "conv_noise_num", "dis_num_iter", "dis_conv_window",
            "dis_spheres_num", "slwf_num")
    reals = ("conv_tol", "trial_step", "fixed_step", "conv_noise_amp", "kmesh_tol", "dis_win_min",
             "dis_win_max", "dis_froz_min", "dis_froz_max", "dis_mix_ratio", "dis_conv_tol", "slwf_lambda",
             "symmetrize_eps")
    bools = ("precond", "guiding_centres", "gamma_only", "slwf_constrain", "site_symmetry")
    for k in ints:
        if k in kw:
            opts[k] = int(kw[k].split()[0])
    for k in reals:
        if k in kw:
            opts[k] = _fnum(kw[k].split()[0])
    for k in bools:
        if k in kw:
            opts[k] = int(_flag(kw[k]))
    if "mp_grid" in kw:
        opts["mp_grid"] = np.array([int(x) for x in re.split(r"[\s,]+", kw["mp_grid"])[:3]], dtype=np.int32)
    for k in ("num_no_guide_iter", "num_guide_cycles", "optimisation"):
        if k in kw:
            opts[k] = int(kw[k].split()[0])
    if "exclude_bands" in kw:
        opts["exclude_bands"] = parse_range_vector(kw["exclude_bands"])
    if "restart" in kw:
        opts["restart"] = kw["restart"].split()[0].lower()
    if opts.get("guiding_centres") and "projections" in blocks:
        spin = _flag(kw.get("spinors", "f"))
        opts["guiding_centres_frac"] = projection_sites(blocks, lattice, spin)
    if opts.get("slwf_constrain") and ("projections" in blocks or "slwf_centres" in blocks):
        opts["slwf_centres_frac"] = slwf_centres(blocks, lattice, int(opts.get("num_wann", 0)),
                                                 _flag(kw.get("spinors", "f")))
    return lattice, kpts, opts


def slwf_centres(blocks, lattice, num_wann, spinors=False):
    """Constrained centres (num_wann x 3, fractional) as w90_readwrite_get_centre_constraints
    forms them (src/readwrite.F90:3266-3357): the projection sites, then each
    <slwf_centres> row 'index x y z [lambda]' replacing its WF's centre (a per-centre
    lambda is read and ignored, as there)."""
    cen = np.zeros((num_wann, 3))
    if "projections" in blocks:
        sites = projection_sites(blocks, lattice, spinors)
        n = min(num_wann, len(sites))
        cen[:n] = sites[:n]
    for row in blocks.get("slwf_centres", []):
        p = row.split()
        if len(p) > 5:
            raise ValueError("Didn't expect anything else after Lagrange multiplier")
        cen[int(p[0]) - 1] = [_fnum(x) for x in p[1:4]]
    return cen


_NORB = {"s": 1, "p": 3, "d": 5, "f": 7, "sp": 2, "sp2": 3, "sp3": 4, "sp3d": 5, "sp3d2": 6,
         "l=0": 1, "l=1": 3, "l=2": 5, "l=3": 7, "l=-1": 2, "l=-2": 3, "l=-3": 4, "l=-4": 5, "l=-5": 6}


def projection_sites(blocks, lattice, spinors):
    """Fractional sites of the projections in the order w90_readwrite_get_projections
    builds them (src/readwrite.F90:3536-3960): per line, per atom of the species (or the
    explicit site), per orbital, per spin.  Handles 'Element:orbitals' and
    'f=x,y,z:orbitals' / 'c=x,y,z:orbitals' with orbitals separated by ';'."""
    atoms = []
    if "atoms_frac" in blocks:
        atoms = [(r.split()[0], np.array([_fnum(x) for x in r.split()[1:4]])) for r in blocks["atoms_frac"]]
    elif "atoms_cart" in blocks:
        rows = blocks["atoms_cart"]
        scale = 1.0
        if rows[0].lower().startswith(("bohr", "ang")):
            scale = BOHR_ANGSTROM if rows[0].lower().startswith("bohr") else 1.0
            rows = rows[1:]
        inv = np.linalg.inv(np.asarray(lattice))
        atoms = [(r.split()[0], np.array([_fnum(x) for x in r.split()[1:4]]) * scale @ inv) for r in rows]
    sites = []
    for line in blocks["projections"]:
        parts = [x.strip() for x in line.replace(" ", "").split(":")]
        if len(parts) < 2:
            continue
        where, orbs = parts[0], parts[1]
        norb = sum(_NORB[o.lower().split(",")[0]] for o in orbs.split(";") if o)
        nspin = 2 if spinors else 1
        if where.lower().startswith(("f=", "c=")):
            v = np.array([_fnum(x) for x in where[2:].split(",")])
            frac = v if where.lower().startswith("f=") else v @ np.linalg.inv(np.asarray(lattice))
            sites += [frac] * (norb * nspin)
        else:
            for name, frac in atoms:
                if name.lower() == where.lower():
                    sites += [frac] * (norb * nspin)
    return np.array(sites, dtype=np.float64)


def write_win(path, lattice, kpts, mp_grid, num_wann, num_bands=None, **keywords):
    with open(path, "w") as f:
        f.write("num_wann = %d\n" % num_wann)
        f.write("num_bands = %d\n" % (num_bands or num_wann))
        for k, v in keywords.items():
            f.write("%s = %s\n" % (k, v))
        f.write("mp_grid : %d %d %d\n" % tuple(mp_grid))
        f.write("begin unit_cell_cart\nang\n")
        for r in lattice:
            f.write("  %.12f %.12f %.12f\n" % tuple(r))
        f.write("end unit_cell_cart\nbegin kpoints\n")
        for k in kpts:
            f.write("  %.12f %.12f %.12f\n" % tuple(k))
        f.write("end kpoints\n")


# --------------------------------------------------------------------------------
# .mmn / .amn / .eig   (src/overlap.F90:234-366)
# --------------------------------------------------------------------------------
def _header(path):
    with open(path) as f:
        f.readline()
        return [int(x) for x in f.readline().split()[:3]]


def _check(rc, err):
    if rc:
        raise ValueError(err.value.decode())


def read_mmn(path, nnlist, nncell, nthreads=0):
    """Overlaps placed at (k, nn) by matching each block's (k2, G) with the k-mesh tables,
    as overlap_read does.  nnlist (K,B) 0-based, nncell (K,B,3).  Parsed in parallel by the
    native reader (w90g_read_mmn)."""
    import ctypes as C

    from ._native import lib
    nnlist = np.ascontiguousarray(nnlist, dtype=np.int32)
    nncell = np.ascontiguousarray(nncell, dtype=np.int32)
    nb, nk, nntot = _header(path)
    if nnlist.shape != (nk, nntot):
        raise ValueError(".mmn has not the right number of k-points / nearest neighbours")
    m = np.zeros((nb, nb, nntot, nk), dtype=np.complex128, order="F")
    err = C.create_string_buffer(512)
    _check(lib().w90g_read_mmn(path.encode(), nb, nk, nntot, nnlist.ctypes.data_as(C.POINTER(C.c_int)),
                               nncell.ctypes.data_as(C.POINTER(C.c_int)), m.ctypes.data, nthreads, err, 512), err)
    return m


def write_mmn(path, m, nnlist, nncell, comment="written by wannier90_gb300"):
    nb, _, nntot, nk = m.shape
    with open(path, "w") as f:
        f.write(comment[:60] + "\n")
        f.write("%12d%12d%12d\n" % (nb, nk, nntot))
        for k in range(nk):
            for b in range(nntot):
                g = nncell[k, b]
                f.write("%5d%5d%5d%5d%5d\n" % (k + 1, nnlist[k, b] + 1, g[0], g[1], g[2]))
                blk = m[:, :, b, k].reshape(-1, order="F")
                for z in blk:
                    f.write("%18.12f%18.12f\n" % (z.real, z.imag))


def read_mmn_device(path, nnlist, nncell, d_m, stream=0, timing=None):
    """.mmn parsed on the GPU into the device buffer at address d_m (complex128,
    (nb, nb, nntot, nk) column-major; e.g. a torch tensor's data_ptr()).  Returns
    (used_gpu, kernels launched); `timing` (a float64 array of 3) receives the ms of the
    value-conversion kernel, of all parse kernels and of the text copy."""
    import ctypes as C

    from ._native import lib
    nnlist = np.ascontiguousarray(nnlist, dtype=np.int32)
    nncell = np.ascontiguousarray(nncell, dtype=np.int32)
    nb, nk, nntot = _header(path)
    if nnlist.shape != (nk, nntot):
        raise ValueError(".mmn has not the right number of k-points / nearest neighbours")
    err = C.create_string_buffer(512)
    used = C.c_int(0)
    nl = C.c_longlong(0)
    _check(lib().w90g_read_mmn_device(path.encode(), nb, nk, nntot, nnlist.ctypes.data_as(C.POINTER(C.c_int)),
                                      nncell.ctypes.data_as(C.POINTER(C.c_int)), C.c_void_p(d_m),
                                      C.c_void_p(stream), C.byref(used), C.byref(nl),
                                      None if timing is None else timing.ctypes.data_as(C.POINTER(C.c_double)),
                                      err, 512), err)
    return bool(used.value), int(nl.value)


def read_amn(path, nthreads=0):
    """Projections A(m, n, k), parsed in parallel by the native reader (w90g_read_amn)."""
    import ctypes as C

    from ._native import lib
    nb, nk, npj = _header(path)
    a = np.zeros((nb, npj, nk), dtype=np.complex128, order="F")
    err = C.create_string_buffer(512)
    _check(lib().w90g_read_amn(path.encode(), nb, npj, nk, a.ctypes.data, nthreads, err, 512), err)
    return a


def write_amn(path, a, comment="written by wannier90_gb300"):
    nb, npj, nk = a.shape
    with open(path, "w") as f:
        f.write(comment[:60] + "\n")
        f.write("%12d%12d%12d\n" % (nb, nk, npj))
        for k in range(nk):
            for n in range(npj):
                for mm in range(nb):
                    z = a[mm, n, k]
                    f.write("%5d%5d%5d%18.12f%18.12f\n" % (mm + 1, n + 1, k + 1, z.real, z.imag))


def read_dmn(path, num_wann):
    """A .dmn file as sitesym_read reads it (src/sitesym.F90:698-765): the counts
    (num_bands, nsymmetry, nkptirr, num_kpts), then list-directed ik2ir(num_kpts),
    ir2ik(nkptirr), kptsym(nsymmetry, nkptirr) (1-based), d_matrix_wann(num_wann,
    num_wann, nsymmetry, nkptirr) and d_matrix_band(num_bands, num_bands, nsymmetry,
    nkptirr) with complex values written '(re, im)'.  Arrays are returned with those
    Fortran shapes and index order."""
    with open(path) as f:
        f.readline()
        nb, nsym, nkirr, nk = (int(x) for x in f.readline().split()[:4])
        rest = f.read()
    first = rest.find("(")
    ints = np.array(rest[:first if first >= 0 else len(rest)].replace(",", " ").split(), dtype=np.int64)
    want = nk + nkirr + nsym * nkirr
    if len(ints) < want:
        raise ValueError("%s: expected %d integers before the matrices, found %d" % (path, want, len(ints)))
    vals = re.findall(r"\(\s*([^,\s]+)\s*,\s*([^)\s]+)\s*\)", rest[first:] if first >= 0 else "")
    z = np.array([_fnum(a) + 1j * _fnum(b) for a, b in vals], dtype=np.complex128)
    nw2 = num_wann * num_wann * nsym * nkirr
    nb2 = nb * nb * nsym * nkirr
    if len(z) < nw2 + nb2:
        raise ValueError("%s: expected %d complex values, found %d" % (path, nw2 + nb2, len(z)))
    return dict(num_bands=nb, nsymmetry=nsym, nkptirr=nkirr, num_kpts=nk,
                ik2ir=ints[:nk], ir2ik=ints[nk:nk + nkirr],
                kptsym=ints[nk + nkirr:want].reshape((nsym, nkirr), order="F"),
                d_matrix_wann=z[:nw2].reshape((num_wann, num_wann, nsym, nkirr), order="F"),
                d_matrix_band=z[nw2:nw2 + nb2].reshape((nb, nb, nsym, nkirr), order="F"))


def read_eig(path, num_bands, num_kpts):
    """Band energies eig(n, k) with the reference's band/k-point order check."""
    import ctypes as C

    from ._native import lib
    e = np.zeros((num_bands, num_kpts), order="F")
    err = C.create_string_buffer(512)
    _check(lib().w90g_read_eig(path.encode(), num_bands, num_kpts, e.ctypes.data, err, 512), err)
    return e


def write_eig(path, eig):
    nb, nk = eig.shape
    with open(path, "w") as f:
        for k in range(nk):
            for n in range(nb):
                f.write("%5d%5d%18.12f\n" % (n + 1, k + 1, eig[n, k]))


# --------------------------------------------------------------------------------
# .chk  (unformatted sequential records, 4-byte record markers as gfortran writes them;
# src/wannier90_readwrite.F90:2336-2366)
# --------------------------------------------------------------------------------
def _rec(f, payload: bytes):
    n = struct.pack("<i", len(payload))
    f.write(n + payload + n)


def recip_lattice(lattice):
    a = np.asarray(lattice, dtype=np.float64)
    cof = np.stack([np.cross(a[1], a[2]), np.cross(a[2], a[0]), np.cross(a[0], a[1])])
    return 2.0 * math.pi * cof / float(np.dot(a[0], cof[0]))


def write_chk(path, *, num_bands, lattice, kpts, mp_grid, nntot, num_wann, u, m, centres, spreads,
              exclude_bands=(), checkpoint="postwann", header=None, dis=None):
    """centres (3, num_wann) Angstrom; u (nw,nw,nk); m (nw,nw,nntot,nk).  dis: None, or
    for a disentangled run dict(omega_invariant, lwindow (nb,nk) bool, ndimwin (nk),
    u_opt (nb,nw,nk))."""
    if header is None:
        now = datetime.datetime.now()
        header = "written on " + now.strftime("%d%b%Y") + " at " + now.strftime("%H:%M:%S")
    header = header.ljust(33)[:33]
    lat = np.asarray(lattice, dtype=np.float64)
    with open(path, "wb") as f:
        _rec(f, header.encode())
        _rec(f, struct.pack("<i", num_bands))
        _rec(f, struct.pack("<i", len(exclude_bands)))
        _rec(f, np.asarray(exclude_bands, dtype="<i4").tobytes())
        _rec(f, np.asarray(lat, dtype="<f8").reshape(-1, order="F").tobytes())      # real_lattice(i,j) i fastest
        _rec(f, np.asarray(recip_lattice(lat), dtype="<f8").reshape(-1, order="F").tobytes())
        _rec(f, struct.pack("<i", len(kpts)))
        _rec(f, np.asarray(mp_grid, dtype="<i4").tobytes())
        _rec(f, np.asarray(kpts, dtype="<f8").reshape(-1).tobytes())                # kpt_latt(3, nk)
        _rec(f, struct.pack("<i", nntot))
        _rec(f, struct.pack("<i", num_wann))
        _rec(f, checkpoint.ljust(20)[:20].encode())
        _rec(f, struct.pack("<i", 1 if dis is not None else 0))                     # have_disentangled
        if dis is not None:
            _rec(f, struct.pack("<d", float(dis["omega_invariant"])))
            _rec(f, np.asarray(dis["lwindow"], dtype="<i4").reshape(-1, order="F").tobytes())
            _rec(f, np.asarray(dis["ndimwin"], dtype="<i4").tobytes())
            _rec(f, np.asarray(dis["u_opt"], dtype="<c16").reshape(-1, order="F").tobytes())
        _rec(f, np.asarray(u, dtype="<c16").reshape(-1, order="F").tobytes())
        _rec(f, np.asarray(m, dtype="<c16").reshape(-1, order="F").tobytes())
        _rec(f, np.asarray(centres, dtype="<f8").reshape(-1, order="F").tobytes())
        _rec(f, np.asarray(spreads, dtype="<f8").tobytes())


def read_chk(path):
    """Parse a .chk written by write_chk or by wannier90.x."""
    recs = []
    with open(path, "rb") as f:
        while True:
            h = f.read(4)
            if not h:
                break
            (n,) = struct.unpack("<i", h)
            recs.append(f.read(n))
            f.read(4)
    i = 0
    out = {"header": recs[0].decode(errors="replace")}
    out["num_bands"] = struct.unpack("<i", recs[1])[0]
    nex = struct.unpack("<i", recs[2])[0]
    out["exclude_bands"] = np.frombuffer(recs[3], "<i4").copy()
    i = 4
    out["real_lattice"] = np.frombuffer(recs[i], "<f8").reshape(3, 3, order="F").copy(); i += 1
    out["recip_lattice"] = np.frombuffer(recs[i], "<f8").reshape(3, 3, order="F").copy(); i += 1
    nk = struct.unpack("<i", recs[i])[0]; i += 1
    out["mp_grid"] = np.frombuffer(recs[i], "<i4").copy(); i += 1
    out["kpts"] = np.frombuffer(recs[i], "<f8").reshape(nk, 3).copy(); i += 1
    nntot = struct.unpack("<i", recs[i])[0]; i += 1
    nw = struct.unpack("<i", recs[i])[0]; i += 1
    out["checkpoint"] = recs[i].decode().strip(); i += 1
    have_dis = struct.unpack("<i", recs[i])[0]; i += 1
    out["have_disentangled"] = bool(have_dis)
    if have_dis:
        nb = out["num_bands"]
        out["omega_invariant"] = struct.unpack("<d", recs[i])[0]; i += 1
        out["lwindow"] = np.frombuffer(recs[i], "<i4").reshape(nb, nk, order="F").astype(bool); i += 1
        out["ndimwin"] = np.frombuffer(recs[i], "<i4").copy(); i += 1
        out["u_opt"] = np.frombuffer(recs[i], "<c16").reshape(nb, nw, nk, order="F").copy(); i += 1
    out["u"] = np.frombuffer(recs[i], "<c16").reshape(nw, nw, nk, order="F").copy(); i += 1
    out["m"] = np.frombuffer(recs[i], "<c16").reshape(nw, nw, nntot, nk, order="F").copy(); i += 1
    out["centres"] = np.frombuffer(recs[i], "<f8").reshape(3, nw, order="F").copy(); i += 1
    out["spreads"] = np.frombuffer(recs[i], "<f8").copy()
    out.update(num_kpts=nk, nntot=nntot, num_wann=nw, num_exclude=nex)
    return out
