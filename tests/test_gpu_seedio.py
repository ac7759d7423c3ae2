"""The GPU .mmn parser (w90g_read_mmn_device) against the host reader, bit for bit: on a
plain file of a k-mesh problem, on a file whose numbers carry exponents and signs the
device fast path converts, and on files it hands to the host reader (blank records, more
digits than the fast path takes)."""
import numpy as np
import pytest

from wannier90_gb300 import synth, w90io

pytestmark = pytest.mark.gpu


def _device_read(path, p):
    import torch
    nb, _, B, K = p.m.shape
    d = torch.zeros(2 * nb * nb * B * K, dtype=torch.float64, device="cuda")
    used, launches = w90io.read_mmn_device(path, p.nnlist, p.nncell, d.data_ptr())
    torch.cuda.synchronize()
    m = d.cpu().numpy().view(np.complex128).reshape(p.m.shape, order="F")
    return m, used, launches


def _rewrite(path, fmt, blank_every=0):
    lines = open(path).read().split("\n")
    out = lines[:2]
    for i, l in enumerate(lines[2:]):
        q = l.split()
        out.append(fmt(float(q[0]), float(q[1])) if len(q) == 2 else l)
        if blank_every and i % blank_every == blank_every - 1:
            out.append("")
    open(path, "w").write("\n".join(out))


def test_device_mmn_plain_and_exponent_forms(tmp_path):
    p = synth.make_problem(kind="fcc", a=6.0, mp=(4, 4, 4), num_wann=12, rmax=2, eps=0.3, seed=3)
    f = str(tmp_path / "a.mmn")
    w90io.write_mmn(f, p.m, p.nnlist, p.nncell)
    host = w90io.read_mmn(f, p.nnlist, p.nncell)
    m, used, launches = _device_read(f, p)
    assert used and launches >= 5
    np.testing.assert_array_equal(m, host)
    # exponent forms, explicit '+', Fortran 'D', leading '.', negative zero: still the fast path
    forms = [lambda a, b: "%.12E %.12E" % (a, b), lambda a, b: "%+.13e,%+.13e" % (a, b),
             lambda a, b: ("%.12E %.12E" % (a, b)).replace("E", "D"),
             lambda a, b: ("%.10f %.10f" % (a, b)).replace("0.", ".", 1)]
    for i, fmt in enumerate(forms):
        g = str(tmp_path / ("e%d.mmn" % i))
        w90io.write_mmn(g, p.m, p.nnlist, p.nncell)
        _rewrite(g, fmt)
        m, used, _ = _device_read(g, p)
        assert used, i
        np.testing.assert_array_equal(m, w90io.read_mmn(g, p.nnlist, p.nncell))


def test_device_mmn_hands_unusual_files_to_the_host_reader(tmp_path):
    p = synth.make_problem(kind="sc", a=5.0, mp=(3, 3, 3), num_wann=6, rmax=1, eps=0.3, seed=4)
    cases = {"blank": (lambda a, b: "%18.12f%18.12f" % (a, b), 5),
             "digits": (lambda a, b: "%.20f %.20f" % (a, b), 0),
             "farexp": (lambda a, b: "%.6E %.6E" % (a * 1e-30, b * 1e30), 0)}
    for name, (fmt, blank) in cases.items():
        g = str(tmp_path / (name + ".mmn"))
        w90io.write_mmn(g, p.m, p.nnlist, p.nncell)
        _rewrite(g, fmt, blank)
        m, used, _ = _device_read(g, p)
        assert not used, name
        np.testing.assert_array_equal(m, w90io.read_mmn(g, p.nnlist, p.nncell))
    # errors carry overlap_read's messages on the device path too
    g = str(tmp_path / "x.mmn")
    w90io.write_mmn(g, p.m, p.nnlist, p.nncell)
    bad = np.array(p.nncell)
    bad[2, :, 1] += 5
    import torch
    d = torch.zeros(2 * p.m.size, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="Neighbour not found"):
        w90io.read_mmn_device(g, p.nnlist, bad, d.data_ptr())
