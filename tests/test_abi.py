"""The C-ABI library loads and exports every entry point include/*.h declares (no GPU needed)."""
import os
import re

from wannier90_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(inc, f)).read()
        # only the extern "C" block (before the C++ helper section)
        c_part = txt.split("#ifdef __cplusplus\n}")[0]
        c_part = re.sub(r"/\*.*?\*/", "", c_part, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([a-z_0-9]+)\s*\(", c_part, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    L = _native.lib()
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    bound = {s[0] for s in _native.SIGNATURES}
    assert names == bound, (names ^ bound)


def test_fortran_shim_binds_every_declared_symbol():
    """include/wannier90_gb300.F90 (the iso_c_binding module for Fortran hosts) has an
    interface block for every entry point of the C header, under its C name, and the
    w90_library module keeps the reference's procedure names for the wannierisation path
    (src/library_interface.F90:101-136)."""
    txt = open(os.path.join(ROOT, "include", "wannier90_gb300.F90")).read()
    bound = set(re.findall(r'bind\(c, name="([a-z_0-9]+)"\)', txt))
    assert _declared() <= bound, _declared() - bound
    for name in ("w90_set_option", "w90_input_setopt", "w90_input_reader", "w90_get_nn", "w90_get_nnkp",
                 "w90_get_gkpb", "w90_set_m_local", "w90_set_u_matrix", "w90_set_u_opt", "w90_set_eigval",
                 "w90_disentangle", "w90_project_overlap", "w90_wannierise", "w90_get_centres", "w90_get_spreads",
                 "w90_create_kmesh"):
        assert re.search(r"subroutine %s\b" % name, txt) or re.search(r"interface %s\b" % name, txt), name
