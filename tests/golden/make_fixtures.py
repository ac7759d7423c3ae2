"""Build the golden fixtures under tests/golden/ from Wannier90's regression inputs.

Run once in a checkout that has the Wannier90 source tree:

    python tests/golden/make_fixtures.py /path/to/wannier90

For each isolated-band ``wann_main`` regression case of the reference test suite
(test-suite/tests/testw90_example02 Pb, testw90_example01 GaAs,
testw90_example05 diamond, testw90_basic1, and the preconditioned GaAs runs
testw90_precond_1 / _2) it stores, in one ``.npz``:

* the inputs exactly as the reference reads them: lattice (Angstrom), k-points,
  the raw ``.mmn`` blocks with their ``(k, k2, G)`` headers, the raw ``.amn``;
* the wannierise keywords of the ``.win`` file;
* the golden outputs parsed from the reference's ``benchmark.out`` file: every
  ``<-- CONV`` line (iteration, delta, RMS gradient, spread), the initial and
  final centres/spreads, the final Omega_I/Omega_D/Omega_OD/Omega_total and the
  b-vector/weight table.

The disentanglement cases (testw90_example03 silicon, _example04 copper: num_bands >
num_wann with outer and frozen energy windows) also store the .eig eigenvalues and every
printed '<-- DIS' line.

The selective-localisation case (testw90_example26: GaAs, slwf_num = 1 with a constrained
centre) also stores the constrained centres and every '<-- SPRD' line (Omega_IOD, Omega_D).

The site-symmetry cases (testw90_example21_As_sp: GaAs sp3; testw90_disentanglement_sawfs:
H3S, entangled) also store the symmetry data of their .dmn files (k-point stars and the D
matrices).

The restart case (testw90_example02_restart: restart = wannierise) stores the U and M of
the checkpoint the test ships and the run's printed lines.

The guiding-centre case (testpostw90_gaas_shc: spinor GaAs, 16 isolated bands,
guiding_centres = T) has no printed wannierise trajectory; its expected values are the
final centres and spreads of the checkpoint shipped with that test.

The parser here is deliberately independent of the package's own file readers.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

BOHR_ANGSTROM = 0.52917720859  # src/constants.F90:109 (CODATA 2006 default)

CASES = {
    "pb": ("test-suite/tests/testw90_example02", "lead"),
    "gaas": ("test-suite/tests/testw90_example01", "gaas"),
    "diamond": ("test-suite/tests/testw90_example05", "diamond"),
    "basic1": ("test-suite/tests/testw90_basic1", "wannier"),
    "precond1": ("test-suite/tests/testw90_precond_1", "gaas1"),
    "precond2": ("test-suite/tests/testw90_precond_2", "gaas2"),
}


def _strip(line):
    for c in "!#":
        if c in line:
            line = line[: line.index(c)]
    return line.strip()


def parse_win(path):
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
            while not lines[i].lower().startswith("end"):
                body.append(lines[i])
                i += 1
            blocks[name] = body
        else:
            m = re.match(r"([A-Za-z_0-9]+)\s*[=:\s]\s*(.*)", lines[i])
            if m:
                kw[m.group(1).lower()] = m.group(2).strip()
        i += 1
    cell = blocks["unit_cell_cart"]
    scale = 1.0
    if cell[0].lower().startswith(("bohr", "ang")):
        scale = BOHR_ANGSTROM if cell[0].lower().startswith("bohr") else 1.0
        cell = cell[1:]
    real_lattice = np.array([[float(x) for x in r.split()[:3]] for r in cell]) * scale
    kpts = np.array([[float(x) for x in r.split()[:3]] for r in blocks["kpoints"]])
    return kw, real_lattice, kpts


def parse_mmn(path):
    with open(path) as f:
        f.readline()
        nb, nk, nntot = (int(x) for x in f.readline().split())
        heads = np.zeros((nk * nntot, 5), dtype=np.int64)
        blocks = np.zeros((nk * nntot, nb, nb), dtype=np.complex128)  # [ncount][m][n]
        for c in range(nk * nntot):
            heads[c] = [int(x) for x in f.readline().split()]
            for n in range(nb):
                for m in range(nb):
                    re_, im_ = (float(x) for x in f.readline().split())
                    blocks[c, m, n] = re_ + 1j * im_
    return nb, nk, nntot, heads, blocks


def parse_amn(path):
    with open(path) as f:
        f.readline()
        nb, nk, npj = (int(x) for x in f.readline().split())
        A = np.zeros((nk, nb, npj), dtype=np.complex128)
        for _ in range(nb * npj * nk):
            p = f.readline().split()
            m, n, k = int(p[0]), int(p[1]), int(p[2])
            A[k - 1, m - 1, n - 1] = float(p[3]) + 1j * float(p[4])
    return A


def parse_benchmark(path):
    txt = open(path).read().splitlines()
    conv = []
    for l in txt:
        if l.rstrip().endswith("<-- CONV") and not l.strip().startswith(("+", "|")):
            p = l.split()
            conv.append([int(p[0]), float(p[1]), float(p[2]), float(p[3])])
    conv = np.array(conv)

    def centres_after(tag):
        idx = next(i for i, l in enumerate(txt) if l.strip() == tag)
        out = []
        for l in txt[idx + 1:]:
            if "WF centre and spread" in l:
                m = re.search(r"\(\s*([-\d.]+),\s*([-\d.]+),\s*([-\d.]+)\s*\)\s+([-\d.]+)", l)
                out.append([float(m.group(i)) for i in range(1, 5)])
            elif out:
                break
        return np.array(out)

    final = centres_after("Final State")
    initial = centres_after("Initial State")
    om = {}
    for l in txt:
        for key, tag in (("om_i", "Omega I"), ("om_d", "Omega D"), ("om_od", "Omega OD"),
                         ("om_tot", "Omega Total")):
            if tag + " " in l and "=" in l:
                om[key] = float(l.split("=")[-1])
    bvec = []
    in_tab = False
    for l in txt:
        if "b_k Vectors" in l:
            in_tab = True
            continue
        if in_tab:
            p = l.replace("|", " ").split()
            if len(p) == 5 and p[0].isdigit():
                bvec.append([float(x) for x in p[1:]])
            elif bvec and l.strip().startswith("+"):
                break
    return conv, initial, final, om, np.array(bvec)


def projection_sites(blocks, real_lattice, spinors):
    """Sites of the projections, in the order of w90_readwrite_get_projections
    (src/readwrite.F90:3536-3960): per line, per atom of the species, per orbital, per
    spin.  Only the 'Element:orbital' form with atoms_frac is handled."""
    norb = {"s": 1, "p": 3, "d": 5, "f": 7, "sp": 2, "sp2": 3, "sp3": 4, "sp3d": 5, "sp3d2": 6}
    atoms = [(l.split()[0], [float(x) for x in l.split()[1:4]]) for l in blocks["atoms_frac"]]
    sites = []
    for line in blocks["projections"]:
        el, orbs = [x.strip() for x in line.split(":")[:2]]
        n = sum(norb[o.strip().lower()] for o in orbs.split(";"))
        for name, frac in atoms:
            if name.lower() == el.lower():
                sites += [frac] * (n * (2 if spinors else 1))
    return np.array(sites)


def parse_chk_fmt_tail(lines, num_wann):
    """Final centres (Angstrom) and spreads: the last 2*num_wann lines of a formatted
    .chk (src/wannier90_readwrite.F90:2336-2366, written by w90chk2chk -u2f)."""
    cen = np.array([[float(x) for x in l.split()] for l in lines[-2 * num_wann:-num_wann]])
    spr = np.array([float(l.split()[0]) for l in lines[-num_wann:]])
    return cen, spr


def build_guiding(ref_root, out_dir):
    """testpostw90_gaas_shc: GaAs, spinor isolated bands (16), 4x4x4 k, guiding
    centres, conv_window 40.  Expected values: the final centres and spreads of the
    checkpoint the test ships (GaAs.chk.fmt.bz2)."""
    import bz2
    d = os.path.join(ref_root, "test-suite/tests/testpostw90_gaas_shc")
    lines = [_strip(l) for l in open(os.path.join(d, "GaAs.win"))]
    blocks, i = {}, 0
    lines = [l for l in lines if l]
    while i < len(lines):
        if lines[i].lower().startswith("begin"):
            name = lines[i].lower().split()[1]
            body = []
            i += 1
            while not lines[i].lower().startswith("end"):
                body.append(lines[i])
                i += 1
            blocks[name] = body
        i += 1
    kw, real_lattice, kpts = parse_win(os.path.join(d, "GaAs.win"))
    tmp = os.path.join(out_dir, "_tmp_gaas")
    os.makedirs(tmp, exist_ok=True)
    for ext in ("mmn", "amn"):
        with bz2.open(os.path.join(d, "GaAs.%s.bz2" % ext), "rb") as f, open(os.path.join(tmp, "GaAs." + ext), "wb") as g:
            g.write(f.read())
    nb, nk, nntot, heads, blk = parse_mmn(os.path.join(tmp, "GaAs.mmn"))
    A = parse_amn(os.path.join(tmp, "GaAs.amn"))
    for ext in ("mmn", "amn"):
        os.remove(os.path.join(tmp, "GaAs." + ext))
    os.rmdir(tmp)
    chk = bz2.open(os.path.join(d, "GaAs.chk.fmt.bz2"), "rt").read().splitlines()
    W = int(kw["num_wann"])
    cen, spr = parse_chk_fmt_tail(chk, W)
    spinors = kw.get("spinors", "f").strip(".").lower().startswith("t")
    sites = projection_sites(blocks, real_lattice, spinors)
    knobs = dict(num_wann=W, num_iter=int(kw.get("num_iter", 100)), num_cg_steps=int(kw.get("num_cg_steps", 5)),
                 conv_tol=float(kw.get("conv_tol", "1e-10").replace("d", "e")),
                 conv_window=int(kw.get("conv_window", -1)), trial_step=float(kw.get("trial_step", 2.0)),
                 search_shells=int(kw.get("search_shells", 36)), precond=0, optimisation=3,
                 guiding_centres=1, num_no_guide_iter=int(kw.get("num_no_guide_iter", 0)),
                 num_guide_cycles=int(kw.get("num_guide_cycles", 1)))
    np.savez_compressed(
        os.path.join(out_dir, "gaas_guide.npz"),
        real_lattice=real_lattice, kpt_latt=kpts, mp_grid=np.array([int(x) for x in kw["mp_grid"].split()[:3]]),
        num_bands=nb, num_kpts=nk, nntot=nntot, mmn_heads=heads, mmn_blocks=blk, amn=A,
        knobs=np.array([knobs[k] for k in sorted(knobs)], dtype=np.float64), knob_names=np.array(sorted(knobs)),
        proj_site_frac=sites, centres_final=np.concatenate([cen, spr[:, None]], axis=1),
        omega_final_total=np.array([spr.sum()]))
    print("gaas_guide", nb, nk, nntot, sites.shape, spr.sum())


DIS_CASES = {
    "silicon_dis": ("test-suite/tests/testw90_example03", "silicon"),
    "copper_dis": ("test-suite/tests/testw90_example04", "copper"),
    # 8 bands -> 4 WFs, outer window with a lower bound, frozen window with both bounds
    "basic2_dis": ("test-suite/tests/testw90_basic2", "wannier"),
    # 12 -> 8 (bands 1-5 excluded upstream), mixing ratio 1, conv_window 3
    "gaas192_dis": ("test-suite/tests/testw90_gaas_disentanglement_issue192", "gaas"),
}


def parse_eig(path, nb, nk):
    eig = np.zeros((nk, nb))
    for line in open(path):
        p = line.split()
        if len(p) >= 3:
            eig[int(p[1]) - 1, int(p[0]) - 1] = float(p[2])
    return eig


def parse_dis_lines(path):
    """Every '<-- DIS' iteration line: iter, Omega_I(i-1), Omega_I(i), delta."""
    out = []
    for l in open(path):
        if l.rstrip().endswith("<-- DIS") and not l.strip().startswith(("+", "|")):
            p = l.split()
            out.append([int(p[0]), float(p[1]), float(p[2]), float(p[3])])
        if "Final Omega_I" in l:
            final = float(l.split()[2])
    return np.array(out), final


def build_dis(ref_root, out_dir):
    """Disentanglement cases (num_bands > num_wann, outer and frozen windows): inputs,
    the printed disentanglement iterations and the wannierise trajectory that follows."""
    import bz2
    for name, (sub, seed) in DIS_CASES.items():
        d = os.path.join(ref_root, sub)
        kw, real_lattice, kpts = parse_win(os.path.join(d, seed + ".win"))
        mmn = os.path.join(d, seed + ".mmn")
        if not os.path.exists(mmn):
            tmp = os.path.join(out_dir, "_tmp_" + name)
            os.makedirs(tmp, exist_ok=True)
            with bz2.open(mmn + ".bz2", "rb") as f, open(os.path.join(tmp, seed + ".mmn"), "wb") as g:
                g.write(f.read())
            nb, nk, nntot, heads, blocks = parse_mmn(os.path.join(tmp, seed + ".mmn"))
            os.remove(os.path.join(tmp, seed + ".mmn"))
            os.rmdir(tmp)
        else:
            nb, nk, nntot, heads, blocks = parse_mmn(mmn)
        A = parse_amn(os.path.join(d, seed + ".amn"))
        eig = parse_eig(os.path.join(d, seed + ".eig"), nb, nk)
        bench = os.path.join(d, "benchmark.out.default.inp=%s.win" % seed)
        conv, initial, final, om, bvec = parse_benchmark(bench)
        dis, omi_final = parse_dis_lines(bench)
        num = lambda k, default: float(kw.get(k, str(default)).replace("d", "e").replace("D", "e"))
        knobs = dict(num_wann=int(kw["num_wann"]), num_bands=int(kw["num_bands"]),
                     num_iter=int(kw.get("num_iter", 100)), num_cg_steps=int(kw.get("num_cg_steps", 5)),
                     conv_tol=num("conv_tol", 1e-10), conv_window=int(kw.get("conv_window", -1)),
                     trial_step=num("trial_step", 2.0), search_shells=int(kw.get("search_shells", 36)),
                     dis_num_iter=int(kw.get("dis_num_iter", 200)), dis_mix_ratio=num("dis_mix_ratio", 0.5),
                     dis_conv_tol=num("dis_conv_tol", 1e-10), dis_conv_window=int(kw.get("dis_conv_window", 3)),
                     dis_win_min=num("dis_win_min", -1e300), dis_win_max=num("dis_win_max", 1e300),
                     dis_froz_min=num("dis_froz_min", -1e300), dis_froz_max=num("dis_froz_max", 1e300),
                     frozen_states=int("dis_froz_max" in kw))
        np.savez_compressed(
            os.path.join(out_dir, name + ".npz"),
            real_lattice=real_lattice, kpt_latt=kpts, mp_grid=np.array([int(x) for x in kw["mp_grid"].split()[:3]]),
            num_bands=nb, num_kpts=nk, nntot=nntot, mmn_heads=heads, mmn_blocks=blocks, amn=A, eig=eig,
            knobs=np.array([knobs[k] for k in sorted(knobs)], dtype=np.float64), knob_names=np.array(sorted(knobs)),
            dis=dis, omega_i_final=np.array([omi_final]), conv=conv, centres_final=final,
            omega_final=np.array([om["om_i"], om["om_d"], om["om_od"], om["om_tot"]]), bvec_table=bvec)
        print(name, nb, nk, nntot, dis.shape, omi_final, conv.shape, om)


def parse_sprd(path):
    """Every '<-- SPRD' line as {key: value} (O_D, O_OD / O_IOD, O_TOT)."""
    out = []
    for l in open(path):
        if l.rstrip().endswith("<-- SPRD"):
            out.append({k: float(v) for k, v in re.findall(r"(O_[A-Z]+)=\s*([-\d.Ee+]+)", l)})
    return out


def build_slwf(ref_root, out_dir):
    """testw90_example26: GaAs, 4 isolated bands, 4x4x4 k, selective localisation of
    one WF (slwf_num = 1) with its centre constrained (slwf_constrain = T, slwf_lambda = 1)
    to the <slwf_centres> site; the other constrained centres default to the projection
    sites (src/readwrite.F90:3266-3357)."""
    d = os.path.join(ref_root, "test-suite/tests/testw90_example26")
    win = os.path.join(d, "gaas.win")
    kw, real_lattice, kpts = parse_win(win)
    lines = [l for l in (_strip(x) for x in open(win)) if l]
    blocks, i = {}, 0
    while i < len(lines):
        if lines[i].lower().startswith("begin"):
            name = lines[i].lower().split()[1]
            body = []
            i += 1
            while not lines[i].lower().startswith("end"):
                body.append(lines[i])
                i += 1
            blocks[name] = body
        i += 1
    W = int(kw["num_wann"])
    sites = []
    for line in blocks["projections"]:                 # 'f= x, y, z: orbital' lines
        xyz = line.split(":")[0].split("=")[1]
        sites.append([float(x) for x in xyz.replace(",", " ").split()])
    cfrac = np.array(sites, dtype=np.float64)
    for line in blocks["slwf_centres"]:
        p = line.split()
        cfrac[int(p[0]) - 1] = [float(x) for x in p[1:4]]
    nb, nk, nntot, heads, blocks_m = parse_mmn(os.path.join(d, "gaas.mmn"))
    A = parse_amn(os.path.join(d, "gaas.amn"))
    bench = os.path.join(d, "benchmark.out.default.inp=gaas.win")
    conv, initial, final, om, bvec = parse_benchmark(bench)
    sprd = parse_sprd(bench)
    txt = open(bench).read()
    fin = {key: float(re.search(tag + r"\s*=\s*([-\d.]+)", txt).group(1))
           for key, tag in (("iod_c", "Omega IOD_C"), ("d", r"Omega D  "), ("rest", "Omega Rest"),
                            ("penalty", "Penalty func"), ("total_c", "Omega Total_C"))}
    tf = lambda v: float(str(v).strip(".").lower().startswith("t"))
    knobs = dict(num_wann=W, num_iter=int(kw.get("num_iter", 100)), num_cg_steps=int(kw.get("num_cg_steps", 5)),
                 conv_tol=float(kw.get("conv_tol", "1e-10").replace("d", "e")),
                 conv_window=int(kw.get("conv_window", -1)), trial_step=float(kw.get("trial_step", 2.0)),
                 search_shells=int(kw.get("search_shells", 36)), slwf_num=int(kw["slwf_num"]),
                 slwf_constrain=tf(kw.get("slwf_constrain", "f")), slwf_lambda=float(kw.get("slwf_lambda", 1.0)))
    np.savez_compressed(
        os.path.join(out_dir, "slwf26.npz"),
        real_lattice=real_lattice, kpt_latt=kpts, mp_grid=np.array([int(x) for x in kw["mp_grid"].split()[:3]]),
        num_bands=nb, num_kpts=nk, nntot=nntot, mmn_heads=heads, mmn_blocks=blocks_m, amn=A,
        knobs=np.array([knobs[k] for k in sorted(knobs)], dtype=np.float64), knob_names=np.array(sorted(knobs)),
        slwf_centres_frac=cfrac, proj_site_frac=np.array(sites, dtype=np.float64), conv=conv, centres_initial=initial, centres_final=final,
        sprd=np.array([[x.get("O_IOD", np.nan), x.get("O_D", np.nan), x.get("O_TOT", np.nan)] for x in sprd]),
        omega_final_slwf=np.array([fin["iod_c"], fin["d"], fin["rest"], fin["penalty"], fin["total_c"]]),
        bvec_table=bvec)
    print("slwf26", nb, nk, nntot, conv.shape, len(sprd), fin)


def parse_dmn(path, nw):
    """A .dmn file as sitesym_read reads it (src/sitesym.F90:698-765): list-directed
    integers ik2ir(nk), ir2ik(nkirr), kptsym(nsym, nkirr), then the complex
    d_matrix_wann(nw, nw, nsym, nkirr) and d_matrix_band(nb, nb, nsym, nkirr), all
    Fortran order.  Returned 1-based as in the file; the matrices as [ir, isym, i, j]."""
    lines = open(path).read().splitlines()
    nb, nsym, nkirr, nk = (int(x) for x in lines[1].split())
    ints, cplx = [], []
    for l in lines[2:]:
        l = l.strip()
        if not l:
            continue
        if l.startswith("("):
            re_, im_ = l.strip("()").split(",")
            cplx.append(float(re_) + 1j * float(im_))
        else:
            ints += [int(x) for x in l.split()]
    ik2ir = np.array(ints[:nk])
    ir2ik = np.array(ints[nk:nk + nkirr])
    kptsym = np.array(ints[nk + nkirr:nk + nkirr + nsym * nkirr]).reshape(nkirr, nsym).T
    cw = np.array(cplx[:nw * nw * nsym * nkirr]).reshape(nkirr, nsym, nw, nw).transpose(0, 1, 3, 2)
    cb = np.array(cplx[nw * nw * nsym * nkirr:]).reshape(nkirr, nsym, nb, nb).transpose(0, 1, 3, 2)
    return nb, nsym, nkirr, nk, ik2ir, ir2ik, kptsym, cw, cb


def build_sitesym(ref_root, out_dir):
    """testw90_example21_As_sp: GaAs, 4 isolated bands (sp3 on As), 4x4x4 k, symmetry-
    adapted mode (site_symmetry = T, symmetrize_eps = 1e-9) with the test's .dmn."""
    d = os.path.join(ref_root, "test-suite/tests/testw90_example21_As_sp")
    kw, real_lattice, kpts = parse_win(os.path.join(d, "GaAs.win"))
    W = int(kw["num_wann"])
    nb, nk, nntot, heads, blocks = parse_mmn(os.path.join(d, "GaAs.mmn"))
    A = parse_amn(os.path.join(d, "GaAs.amn"))
    dnb, nsym, nkirr, dnk, ik2ir, ir2ik, kptsym, dw, db = parse_dmn(os.path.join(d, "GaAs.dmn"), W)
    assert dnb == nb and dnk == nk
    bench = os.path.join(d, "benchmark.out.default.inp=GaAs.win")
    conv, initial, final, om, bvec = parse_benchmark(bench)
    num = lambda k, default: float(kw.get(k, str(default)).replace("d", "e").replace("D", "e"))
    knobs = dict(num_wann=W, num_iter=int(kw.get("num_iter", 100)), num_cg_steps=int(kw.get("num_cg_steps", 5)),
                 conv_tol=num("conv_tol", 1e-10), conv_window=int(kw.get("conv_window", -1)),
                 trial_step=num("trial_step", 2.0), search_shells=int(kw.get("search_shells", 36)),
                 symmetrize_eps=num("symmetrize_eps", 1e-3))
    np.savez_compressed(
        os.path.join(out_dir, "sitesym21.npz"),
        real_lattice=real_lattice, kpt_latt=kpts, mp_grid=np.array([int(x) for x in kw["mp_grid"].split()[:3]]),
        num_bands=nb, num_kpts=nk, nntot=nntot, mmn_heads=heads, mmn_blocks=blocks, amn=A,
        knobs=np.array([knobs[k] for k in sorted(knobs)], dtype=np.float64), knob_names=np.array(sorted(knobs)),
        ik2ir=ik2ir, ir2ik=ir2ik, kptsym=kptsym, d_matrix_wann=dw, d_matrix_band=db,
        conv=conv, centres_initial=initial, centres_final=final,
        omega_final=np.array([om["om_i"], om["om_d"], om["om_od"], om["om_tot"]]), bvec_table=bvec)
    print("sitesym21", nb, nk, nntot, nsym, nkirr, conv.shape, om)


def build_sitesym_dis(ref_root, out_dir):
    """testw90_disentanglement_sawfs: H3S, 20 bands -> 12 WFs, 2x2x2 k (3 irreducible, 48
    symmetries), outer window only, site_symmetry = T (symmetrize_eps = 1e-8), ten
    disentanglement and ten wannierisation iterations."""
    d = os.path.join(ref_root, "test-suite/tests/testw90_disentanglement_sawfs")
    kw, real_lattice, kpts = parse_win(os.path.join(d, "H3S.win"))
    W = int(kw["num_wann"])
    nb, nk, nntot, heads, blocks = parse_mmn(os.path.join(d, "H3S.mmn"))
    A = parse_amn(os.path.join(d, "H3S.amn"))
    eig = parse_eig(os.path.join(d, "H3S.eig"), nb, nk)
    dnb, nsym, nkirr, dnk, ik2ir, ir2ik, kptsym, dw, db = parse_dmn(os.path.join(d, "H3S.dmn"), W)
    assert dnb == nb and dnk == nk
    bench = os.path.join(d, "benchmark.out.default.inp=H3S.win")
    conv, initial, final, om, bvec = parse_benchmark(bench)
    dis, omi_final = parse_dis_lines(bench)
    num = lambda k, default: float(kw.get(k, str(default)).replace("d", "e").replace("D", "e"))
    knobs = dict(num_wann=W, num_bands=nb, num_iter=int(kw.get("num_iter", 100)),
                 num_cg_steps=int(kw.get("num_cg_steps", 5)), conv_tol=num("conv_tol", 1e-10),
                 conv_window=int(kw.get("conv_window", -1)), trial_step=num("trial_step", 2.0),
                 search_shells=int(kw.get("search_shells", 36)), dis_num_iter=int(kw.get("dis_num_iter", 200)),
                 dis_mix_ratio=num("dis_mix_ratio", 0.5), dis_conv_tol=num("dis_conv_tol", 1e-10),
                 dis_conv_window=int(kw.get("dis_conv_window", 3)), dis_win_min=num("dis_win_min", -1e300),
                 dis_win_max=num("dis_win_max", 1e300), dis_froz_min=num("dis_froz_min", -1e300),
                 dis_froz_max=num("dis_froz_max", 1e300), frozen_states=int("dis_froz_max" in kw),
                 symmetrize_eps=num("symmetrize_eps", 1e-3))
    np.savez_compressed(
        os.path.join(out_dir, "sitesym_dis.npz"),
        real_lattice=real_lattice, kpt_latt=kpts, mp_grid=np.array([int(x) for x in kw["mp_grid"].split()[:3]]),
        num_bands=nb, num_kpts=nk, nntot=nntot, mmn_heads=heads, mmn_blocks=blocks, amn=A, eig=eig,
        knobs=np.array([knobs[k] for k in sorted(knobs)], dtype=np.float64), knob_names=np.array(sorted(knobs)),
        ik2ir=ik2ir, ir2ik=ir2ik, kptsym=kptsym, d_matrix_wann=dw, d_matrix_band=db,
        dis=dis, omega_i_final=np.array([omi_final]), conv=conv, centres_final=final,
        omega_final=np.array([om["om_i"], om["om_d"], om["om_od"], om["om_tot"]]), bvec_table=bvec)
    print("sitesym_dis", nb, nk, nntot, nsym, nkirr, dis.shape, omi_final, conv.shape, om)


def parse_chk_fmt(lines):
    """A formatted checkpoint (w90chk2chk -u2f of the .chk, src/wannier90_readwrite.F90:
    2336-2366) without disentanglement: (num_wann, nntot, num_kpts, u[k,m,n], m[k,b,m,n])."""
    i = 1
    nb = int(lines[i]); i += 1
    nex = int(lines[i]); i += 1 + (1 if nex > 0 else 0)
    i += 2                                        # real and reciprocal lattice
    nk = int(lines[i]); i += 1
    i += 1 + nk                                   # mp_grid, k-points
    nntot = int(lines[i]); i += 1
    W = int(lines[i]); i += 1
    i += 1                                        # checkpoint
    assert int(lines[i]) == 0, "disentangled checkpoints are not handled here"
    i += 1
    vals = np.array([[float(x) for x in l.split()] for l in lines[i:i + W * W * nk + W * W * nntot * nk]])
    z = vals[:, 0] + 1j * vals[:, 1]
    u = z[:W * W * nk].reshape(nk, W, W).transpose(0, 2, 1)                  # (m,n,k) Fortran
    m = z[W * W * nk:].reshape(nk, nntot, W, W).transpose(0, 1, 3, 2)        # (m,n,b,k) Fortran
    return W, nntot, nk, np.ascontiguousarray(u), np.ascontiguousarray(m)


def parse_chk_fmt_records(lines, W, nntot, nk):
    """The records of a formatted checkpoint other than u and m, in file order: header,
    num_bands, exclude_bands, the real and reciprocal lattice as the nine numbers of their
    records, mp_grid, the checkpoint label, have_disentangled, centres and spreads
    (src/wannier90_readwrite.F90:2336-2366)."""
    i = 0
    header = lines[i]; i += 1
    nb = int(lines[i]); i += 1
    nex = int(lines[i]); i += 1
    exclude = np.array([int(x) for x in lines[i].split()], dtype=np.int64) if nex > 0 else np.zeros(0, np.int64)
    i += 1 if nex > 0 else 0
    lat9 = np.array([float(x) for x in lines[i].split()]); i += 1
    rec9 = np.array([float(x) for x in lines[i].split()]); i += 1
    i += 1                                        # num_kpts
    mp = np.array([int(x) for x in lines[i].split()]); i += 1
    i += nk + 2                                   # k-points, nntot, num_wann
    label = lines[i].strip(); i += 1
    have_dis = int(lines[i]); i += 1
    i += W * W * nk + W * W * nntot * nk
    cen = np.array([[float(x) for x in l.split()] for l in lines[i:i + W]]); i += W
    spr = np.array([float(l.split()[0]) for l in lines[i:i + W]])
    return dict(chk_header=header, chk_num_bands=nb, chk_exclude=exclude, chk_lattice9=lat9, chk_recip9=rec9,
                chk_mp_grid=mp, chk_label=label, chk_have_dis=have_dis, chk_centres=cen, chk_spreads=spr)


def build_restart(ref_root, out_dir):
    """testw90_example02_restart: lead, restart = wannierise from the converged checkpoint
    the test ships (lead.chk.fmt.bz2), 20 more iterations."""
    import bz2
    d = os.path.join(ref_root, "test-suite/tests/testw90_example02_restart")
    kw, real_lattice, kpts = parse_win(os.path.join(d, "lead.win"))
    lines = bz2.open(os.path.join(d, "lead.chk.fmt.bz2"), "rt").read().splitlines()
    W, nntot, nk, u, m = parse_chk_fmt(lines)
    bench = os.path.join(d, "benchmark.out.default.inp=lead.win")
    conv, initial, final, om, bvec = parse_benchmark(bench)
    knobs = dict(num_wann=W, num_iter=int(kw.get("num_iter", 100)), num_cg_steps=int(kw.get("num_cg_steps", 5)),
                 conv_tol=float(kw.get("conv_tol", "1e-10").replace("d", "e")),
                 conv_window=int(kw.get("conv_window", -1)), trial_step=float(kw.get("trial_step", 2.0)),
                 search_shells=int(kw.get("search_shells", 36)))
    np.savez_compressed(
        os.path.join(out_dir, "restart02.npz"),
        real_lattice=real_lattice, kpt_latt=kpts, mp_grid=np.array([int(x) for x in kw["mp_grid"].split()[:3]]),
        num_kpts=nk, nntot=nntot, u=u, m=m,
        knobs=np.array([knobs[k] for k in sorted(knobs)], dtype=np.float64), knob_names=np.array(sorted(knobs)),
        conv=conv, centres_final=final, omega_final=np.array([om["om_i"], om["om_d"], om["om_od"], om["om_tot"]]),
        bvec_table=bvec, **parse_chk_fmt_records(lines, W, nntot, nk))
    print("restart02", W, nntot, nk, conv.shape, om)


def build(ref_root, out_dir):
    for name, (sub, seed) in CASES.items():
        d = os.path.join(ref_root, sub)
        kw, real_lattice, kpts = parse_win(os.path.join(d, seed + ".win"))
        nb, nk, nntot, heads, blocks = parse_mmn(os.path.join(d, seed + ".mmn"))
        A = parse_amn(os.path.join(d, seed + ".amn"))
        bench = os.path.join(d, "benchmark.out.default.inp=%s.win" % seed)
        conv, initial, final, om, bvec = parse_benchmark(bench)
        knobs = dict(num_wann=int(kw["num_wann"]), num_iter=int(kw.get("num_iter", 100)),
                     num_cg_steps=int(kw.get("num_cg_steps", 5)),
                     conv_tol=float(kw.get("conv_tol", "1e-10").replace("d", "e")),
                     conv_window=int(kw.get("conv_window", -1)),
                     trial_step=float(kw.get("trial_step", 2.0)),
                     search_shells=int(kw.get("search_shells", 36)),
                     precond=int(kw.get("precond", "f").strip(".").lower().startswith("t")),
                     optimisation=int(kw.get("optimisation", 3)))
        np.savez_compressed(
            os.path.join(out_dir, name + ".npz"),
            real_lattice=real_lattice, kpt_latt=kpts,
            mp_grid=np.array([int(x) for x in kw["mp_grid"].split()[:3]]),
            num_bands=nb, num_kpts=nk, nntot=nntot,
            mmn_heads=heads, mmn_blocks=blocks, amn=A,
            knobs=np.array([knobs[k] for k in sorted(knobs)], dtype=np.float64),
            knob_names=np.array(sorted(knobs)),
            conv=conv, centres_initial=initial, centres_final=final,
            omega_final=np.array([om["om_i"], om["om_d"], om["om_od"], om["om_tot"]]),
            bvec_table=bvec)
        print(name, nb, nk, nntot, conv.shape, final.shape, om)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("W90_REFERENCE")
    if not root or not os.path.isdir(root):
        raise SystemExit("usage: make_fixtures.py <Wannier90 source tree> (or set W90_REFERENCE)")
    build(root, os.path.dirname(os.path.abspath(__file__)))
    build_guiding(root, os.path.dirname(os.path.abspath(__file__)))
    build_dis(root, os.path.dirname(os.path.abspath(__file__)))
    build_slwf(root, os.path.dirname(os.path.abspath(__file__)))
    build_sitesym(root, os.path.dirname(os.path.abspath(__file__)))
    build_sitesym_dis(root, os.path.dirname(os.path.abspath(__file__)))
    build_restart(root, os.path.dirname(os.path.abspath(__file__)))
