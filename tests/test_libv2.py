"""C and C++ callers of the library mode against include/wannier90_gb300.h.

* The reference's own C++ demo (test-suite/libv2-demo/libc-gas-mix-serial: wannier.cc,
  demo.cc) compiles and links against this library with its `#include "wannier90.hh"`
  changed to `#include "wannier90_gb300.h"` and nothing else (needs the Wannier90 source
  tree through W90_REFERENCE; demo.cc includes <ISO_Fortran_binding.h> without using it,
  so an empty stand-in is put on its include path).
* tests/libv2/gaas_driver.cc, a caller written against the header the same way, compiles
  and links here, and on a GPU runs the demo's GaAs case (12 bands -> 8 WFs, the demo's
  .win keywords: fixed_step 50, conv_tol 1e-13 over 3 iterations, frozen window) to the
  oracle's final centres and spreads (tests/golden/libv2_gaas.npz).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.conftest import reference_root
from wannier90_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.dirname(B.lib_path())


def _link(objs, out):
    cmd = ["g++", "-o", out, *objs, "-L" + LIBDIR, "-lw90gb300", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _compile(src, obj, extra_inc=()):
    cmd = ["g++", "-std=c++17", "-Wall", "-pedantic", "-O1", "-I" + INC, *("-I" + d for d in extra_inc),
           "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.fixture(scope="module")
def library():
    B.build()
    return B.lib_path()


@pytest.mark.skipif(reference_root() is None, reason="W90_REFERENCE (Wannier90 source tree) not set")
def test_reference_cpp_demo_builds_against_header(tmp_path, library):
    demo = os.path.join(reference_root(), "test-suite", "libv2-demo", "libc-gas-mix-serial")
    src = open(os.path.join(demo, "wannier.cc")).read()
    assert '#include "wannier90.hh"' in src
    (tmp_path / "wannier.cc").write_text(src.replace('#include "wannier90.hh"', '#include "wannier90_gb300.h"'))
    shutil.copy(os.path.join(demo, "wannier.hh"), tmp_path / "wannier.hh")
    shutil.copy(os.path.join(demo, "demo.cc"), tmp_path / "demo.cc")
    stub = tmp_path / "stub"
    stub.mkdir()
    (stub / "ISO_Fortran_binding.h").write_text("/* not used by demo.cc */\n")
    _compile(str(tmp_path / "wannier.cc"), str(tmp_path / "wannier.o"))
    _compile(str(tmp_path / "demo.cc"), str(tmp_path / "demo.o"), [str(stub), str(tmp_path)])
    _link([str(tmp_path / "wannier.o"), str(tmp_path / "demo.o")], str(tmp_path / "demo"))
    assert os.path.exists(tmp_path / "demo")


def _driver(tmp_path):
    _compile(os.path.join(ROOT, "tests", "libv2", "gaas_driver.cc"), str(tmp_path / "driver.o"))
    exe = str(tmp_path / "gaas_driver")
    _link([str(tmp_path / "driver.o")], exe)
    return exe


def test_cpp_driver_builds_against_header(tmp_path, library):
    assert os.path.exists(_driver(tmp_path))


@pytest.mark.gpu
def test_cpp_library_flow_gaas(tmp_path, library):
    from oracle import w90_oracle as O
    from tests import golden_cases as G
    from tests.golden.make_libv2_demo import DEMO_KEYWORDS
    from wannier90_gb300 import synth, w90io
    d = G.load("gaas192_dis")
    ref = np.load(os.path.join(ROOT, "tests", "golden", "libv2_gaas.npz"))
    nb, nw = int(d["num_bands"]), int(d["knobs"]["num_wann"])
    km = O.kmesh_get(d["real_lattice"], d["kpt_latt"])
    M = G.assemble_m(d, km["nnlist"], km["nncell"])
    seed = str(tmp_path / "gaas")
    w90io.write_mmn(seed + ".mmn", synth.from_math_m(M), km["nnlist"], km["nncell"])
    w90io.write_amn(seed + ".amn", synth.from_math_u(d["amn"]))
    w90io.write_eig(seed + ".eig", np.asfortranarray(d["eig"].T))
    with open(seed + ".win", "w") as f:
        for k, v in DEMO_KEYWORDS.items():
            f.write("%-17s = %s\n" % (k, v))
    exe = _driver(tmp_path)
    args = [exe, seed, str(nb), str(nw), *map(str, d["mp_grid"]), *("%.16g" % x for x in d["real_lattice"].ravel())]
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    assert lines[-1].split()[:1] == ["ierr"] and int(lines[-1].split()[1]) == 0
    vals = np.array([[float(x) for x in l.split()] for l in lines[-1 - nw:-1]])
    np.testing.assert_allclose(vals[:, :3], ref["centres"], atol=1e-6)
    np.testing.assert_allclose(vals[:, 3], ref["spreads"], atol=1e-6)
