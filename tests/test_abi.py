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
