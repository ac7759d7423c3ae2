"""Helpers that turn the golden fixtures (tests/golden/*.npz) into engine/oracle inputs."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["pb", "gaas", "diamond", "basic1", "precond1", "precond2"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    d["knobs"] = dict(zip([str(x) for x in z["knob_names"]], z["knobs"]))
    return d


def assemble_m(d, nnlist, nncell):
    """Place the .mmn blocks at (k, nn) by matching (k2, G) against the k-mesh tables,
    as overlap_read does (src/overlap.F90:270-300).  Returns M[k,b,m,n]."""
    K = int(d["num_kpts"])
    B = nnlist.shape[1]
    W = int(d["num_bands"])
    M = np.zeros((K, B, W, W), dtype=np.complex128)
    filled = np.zeros((K, B), dtype=bool)
    for h, blk in zip(d["mmn_heads"], d["mmn_blocks"]):
        k, k2 = int(h[0]) - 1, int(h[1]) - 1
        hit = [b for b in range(B) if nnlist[k, b] == k2 and tuple(nncell[k, b]) == tuple(h[2:])]
        assert len(hit) == 1, (h, hit)
        M[k, hit[0]] = blk
        filled[k, hit[0]] = True
    assert filled.all()
    return M


def control(d):
    from oracle import w90_oracle as O
    kn = d["knobs"]
    return O.WannControl(num_iter=int(kn["num_iter"]), num_cg_steps=int(kn["num_cg_steps"]),
                         conv_tol=float(kn["conv_tol"]), conv_window=int(kn["conv_window"]),
                         trial_step=float(kn["trial_step"]), precond=bool(kn.get("precond", 0)))


def precond_tables(d):
    """irvec / ndegen / k_to_r of a preconditioned case (None otherwise)."""
    from oracle import w90_oracle as O
    if not d["knobs"].get("precond", 0):
        return None
    return O.precond_setup(d["real_lattice"], d["kpt_latt"], d["mp_grid"])


def guiding(d):
    """(WannControl, rguide[3,W] Cartesian) of the guiding-centre case."""
    from oracle import w90_oracle as O
    kn = d["knobs"]
    ctl = O.WannControl(num_iter=int(kn["num_iter"]), num_cg_steps=int(kn["num_cg_steps"]),
                        conv_tol=float(kn["conv_tol"]), conv_window=int(kn["conv_window"]),
                        trial_step=float(kn["trial_step"]), guiding_centres=True,
                        num_no_guide_iter=int(kn["num_no_guide_iter"]), num_guide_cycles=int(kn["num_guide_cycles"]))
    return ctl, (d["proj_site_frac"] @ d["real_lattice"]).T


def slwf(d):
    """(WannControl, Slwf) of the selective-localisation case: constrained centres in
    Cartesian Angstrom (utility_frac_to_cart of the fractional sites)."""
    from oracle import w90_oracle as O
    kn = d["knobs"]
    ctl = O.WannControl(num_iter=int(kn["num_iter"]), num_cg_steps=int(kn["num_cg_steps"]),
                        conv_tol=float(kn["conv_tol"]), conv_window=int(kn["conv_window"]),
                        trial_step=float(kn["trial_step"]))
    cen = (d["slwf_centres_frac"] @ d["real_lattice"]).T if kn["slwf_constrain"] else None
    return ctl, O.Slwf(int(kn["slwf_num"]), float(kn["slwf_lambda"]), cen)


def sitesym(d):
    """Sitesym (0-based) of the site-symmetry case, from its .dmn data."""
    from oracle import w90_oracle as O
    return O.Sitesym(d["ik2ir"] - 1, d["ir2ik"] - 1, d["kptsym"] - 1, d["d_matrix_wann"], d["d_matrix_band"],
                     float(d["knobs"]["symmetrize_eps"]))


DIS_CASES = ["silicon_dis", "copper_dis", "basic2_dis", "gaas192_dis"]


def dis_control(d):
    """DisControl of a disentanglement case."""
    from oracle import w90_oracle as O
    kn = d["knobs"]
    return O.DisControl(num_iter=int(kn["dis_num_iter"]), mix_ratio=float(kn["dis_mix_ratio"]),
                        conv_tol=float(kn["dis_conv_tol"]), conv_window=int(kn["dis_conv_window"]),
                        win_min=float(kn["dis_win_min"]), win_max=float(kn["dis_win_max"]),
                        froz_min=float(kn["dis_froz_min"]), froz_max=float(kn["dis_froz_max"]),
                        frozen_states=bool(kn["frozen_states"]))


def conv_sensitivity(M0, U0, km, ctl, noise=1e-14, runs=2, slwf=None, grad=False, centres=False, sitesym=None,
                     per_update=False):
    """Per iteration, the largest change of the oracle's own wann_main spread when M0 is
    perturbed by `noise` (relative, seeded): the part of a printed trajectory that no FP64
    implementation can reproduce more closely.  per_update=True perturbs every updated M
    instead (the model of the tensor path, whose M update carries ~1e-13 relative rounding
    at every iteration).  grad=True also returns the same for the RMS gradient column;
    centres=True also returns the largest change of any final centre coordinate (per WF,
    A)."""
    import numpy as np

    from oracle import w90_oracle as O
    base = O.wann_main(M0, U0, km, ctl, slwf=slwf, sitesym=sitesym)
    ref = {x.iter: x.spread.om_tot for x in [base.initial] + base.iters}
    gref = {x.iter: x.rms_grad for x in [base.initial] + base.iters}
    sens = {i: 0.0 for i in ref}
    gsens = {i: 0.0 for i in ref}
    csens = np.zeros(np.asarray(base.centres).shape[1])
    rng = np.random.default_rng(2024)
    for _ in range(runs):
        if per_update:
            def perturb(M):
                return M * (1 + noise * rng.standard_normal(M.shape))
            r = O.wann_main(M0, U0, km, ctl, slwf=slwf, sitesym=sitesym, update_noise=perturb)
        else:
            r = O.wann_main(M0 * (1 + noise * rng.standard_normal(M0.shape)), U0, km, ctl, slwf=slwf,
                            sitesym=sitesym)
        for x in [r.initial] + r.iters:
            if x.iter in sens:
                sens[x.iter] = max(sens[x.iter], abs(x.spread.om_tot - ref[x.iter]))
                gsens[x.iter] = max(gsens[x.iter], abs(x.rms_grad - gref[x.iter]))
        csens = np.maximum(csens, np.abs(np.asarray(r.centres) - np.asarray(base.centres)).max(axis=0))
    out = (sens,)
    if grad:
        out += (gsens,)
    if centres:
        out += (csens,)
    return out if len(out) > 1 else sens


def match_centres(a, b, lattice):
    """One-to-one partners of the centres a[i] among b[j] (greedy by distance, distances
    modulo lattice translations): (largest distance, [(i, j), ...], distance matrix).  WF
    labels are arbitrary: two runs that end at the same minimum may order the WFs
    differently."""
    import numpy as np
    inv = np.linalg.inv(lattice)
    d = np.zeros((len(a), len(b)))
    for i in range(len(a)):
        f = (b - a[i]) @ inv
        f -= np.round(f)
        d[i] = np.linalg.norm(f @ lattice, axis=1)
    used_a, used_b, pairs, worst = set(), set(), [], 0.0
    for flat in np.argsort(d, axis=None):
        i, j = divmod(int(flat), len(b))
        if i in used_a or j in used_b:
            continue
        used_a.add(i)
        used_b.add(j)
        pairs.append((i, j))
        worst = max(worst, d[i, j])
    return worst, sorted(pairs), d


def conv_tolerance(sens, it, spread, floor=2e-10, factor=10.0, span=0):
    """2e-10 A^2 where the trajectory is insensitive at that level, else `factor` times the
    measured sensitivity (at least the metric's 1e-8 relative).  span > 0 takes the
    sensitivity as the largest over iterations it-span..it+span: a few perturbed runs
    sample it, and a sample can dip at one iteration of a segment that is sensitive."""
    it = int(it)
    s = max(sens.get(j, 0.0) for j in range(it - span, it + span + 1))
    return floor if s < 0.1 * floor else max(factor * s, 1e-8 * abs(spread))


def grad_tolerance(gsens, it, rms, factor=10.0):
    """The printed RMS gradient: 1e-6 + 1e-3 relative (its roundoff floor near a minimum),
    or `factor` times its measured sensitivity where that is larger (a converged SLWF run,
    whose non-objective gauge is free, moves it by up to 1e-4 under a 1e-14 perturbation)."""
    return max(1e-6 + 1e-3 * rms, factor * gsens.get(int(it), 0.0))


def write_dmn(path, d):
    """The fixture's symmetry data in the .dmn layout (10 integers a line, one complex
    '(re, im)' a line, blank lines between the records)."""
    ik2ir, ir2ik, kptsym = d["ik2ir"], d["ir2ik"], d["kptsym"]
    dw = d["d_matrix_wann"].transpose(2, 3, 1, 0)      # [ir, isym, i, j] -> (i, j, isym, ir)
    db = d["d_matrix_band"].transpose(2, 3, 1, 0)
    nsym, nkirr = kptsym.shape
    nb = db.shape[0]

    def ints(v):
        v = list(v)
        return "\n".join("".join("%9d" % x for x in v[i:i + 10]) for i in range(0, len(v), 10)) + "\n \n"

    with open(path, "w") as f:
        f.write(" Created by the test\n")
        f.write("%9d%9d%9d%9d\n \n" % (nb, nsym, nkirr, len(ik2ir)))
        f.write(ints(ik2ir))
        f.write(ints(ir2ik))
        for ir in range(nkirr):
            f.write(ints(kptsym[:, ir]))
        for arr in (dw, db):
            for z in arr.reshape(-1, order="F"):
                f.write(" (%17.10E,%17.10E)\n" % (z.real, z.imag))


def dmn_dict(d):
    """The site-symmetry fixture as w90io.read_dmn returns a .dmn file (Fortran shapes)."""
    nsym, nkirr = d["kptsym"].shape
    return dict(num_bands=d["d_matrix_band"].shape[-1], nsymmetry=nsym, nkptirr=nkirr, num_kpts=len(d["ik2ir"]),
                ik2ir=d["ik2ir"].copy(),
                ir2ik=d["ir2ik"].copy(), kptsym=d["kptsym"].copy(),
                d_matrix_wann=d["d_matrix_wann"].transpose(2, 3, 1, 0).copy(),
                d_matrix_band=d["d_matrix_band"].transpose(2, 3, 1, 0).copy())
