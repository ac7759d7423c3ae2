"""ctypes binding of the in-tree CUDA library ``lib/libw90gb300.so``.

The library is the product: every compute entry point of this package goes through
it.  If it is missing, importing :func:`lib` raises -- there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_LIB = None

_c_double_p = C.POINTER(C.c_double)
_c_int_p = C.POINTER(C.c_int)

# (name, restype, argtypes) of every symbol declared in include/wannier90_gb300.h
SIGNATURES = [
    ("w90_create", C.c_void_p, []),
    ("w90_delete", None, [C.c_void_p]),
    ("cset_option_int", None, [C.c_void_p, C.c_char_p, C.c_int]),
    ("cset_option_int3", None, [C.c_void_p, C.c_char_p, _c_int_p]),
    ("cset_option_intx", None, [C.c_void_p, C.c_char_p, _c_int_p, C.c_int]),
    ("cset_option_float", None, [C.c_void_p, C.c_char_p, C.c_double]),
    ("cset_option_float33", None, [C.c_void_p, C.c_char_p, _c_double_p]),
    ("cset_option_floatxy", None, [C.c_void_p, C.c_char_p, _c_double_p, C.c_int, C.c_int]),
    ("cinput_setopt", None, [C.c_void_p, C.c_char_p, _c_int_p, C.c_int]),
    ("cinput_reader", None, [C.c_void_p, _c_int_p]),
    ("cinput_reader_special", None, [C.c_void_p, C.c_char_p, _c_int_p]),
    ("cset_a_matrix", None, [C.c_void_p, C.c_void_p]),
    ("cset_kpoint_distribution", None, [C.c_void_p, _c_int_p]),
    ("cset_parallel_comms", None, [C.c_void_p, C.c_int]),
    ("coverlaps", None, [C.c_void_p, _c_int_p]),
    ("cchkpt", None, [C.c_void_p, C.c_char_p]),
    ("cset_eigval", None, [C.c_void_p, C.c_void_p]),
    ("cset_m_local", None, [C.c_void_p, C.c_void_p]),
    ("cset_u_matrix", None, [C.c_void_p, C.c_void_p]),
    ("cset_u_opt", None, [C.c_void_p, C.c_void_p]),
    ("cwannierise", None, [C.c_void_p, _c_int_p]),
    ("cdisentangle", None, [C.c_void_p, _c_int_p]),
    ("cget_nn", None, [C.c_void_p, _c_int_p]),
    ("cget_nnkp", None, [C.c_void_p, _c_int_p]),
    ("cget_centres", None, [C.c_void_p, _c_double_p]),
    ("cget_spreads", None, [C.c_void_p, _c_double_p]),
    ("cproject_overlap", None, [C.c_void_p, _c_int_p]),
    ("cget_omega", None, [C.c_void_p, _c_double_p]),
    ("cget_gkpb", None, [C.c_void_p, _c_int_p]),
    ("w90g_last_error", C.c_char_p, [C.c_void_p]),
    ("w90g_get_log", C.c_int, [C.c_void_p, _c_double_p, C.c_int]),
    ("w90g_get_log_centres", C.c_int, [C.c_void_p, _c_double_p, C.c_int]),
    ("w90g_get_dis_log", C.c_int, [C.c_void_p, _c_double_p, C.c_int]),
    ("w90g_get_dis_info", None, [C.c_void_p, _c_double_p]),
    ("w90g_get_dis_windows", None, [C.c_void_p, _c_int_p, _c_int_p]),
    ("w90g_set_sitesym", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _c_int_p, _c_int_p, _c_int_p,
                                   _c_double_p, _c_double_p]),
    ("w90g_read_mmn", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, _c_int_p, _c_int_p, C.c_void_p, C.c_int,
                                C.c_char_p, C.c_int]),
    ("w90g_read_amn", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_char_p, C.c_int]),
    ("w90g_read_eig", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_char_p, C.c_int]),
    ("w90g_read_mmn_device", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, _c_int_p, _c_int_p, C.c_void_p,
                                       C.c_void_p, _c_int_p, C.POINTER(C.c_longlong), _c_double_p, C.c_char_p,
                                       C.c_int]),
    ("w90g_disentangle_device", None, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _c_int_p]),
    ("w90g_profile_dis_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _c_double_p, _c_int_p]),
    ("w90g_dis_kernel_name", C.c_char_p, [C.c_int]),
    ("w90g_wannierise_device", None, [C.c_void_p, C.c_void_p, C.c_void_p, _c_int_p]),
    ("w90g_project_overlap_device", None, [C.c_void_p, C.c_void_p, C.c_void_p, _c_int_p]),
    ("w90g_set_stream", None, [C.c_void_p, C.c_void_p]),
    ("w90g_wannierise_batch_device", None,
     [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _c_int_p]),
    ("w90g_kernel_launches", C.c_longlong, [C.c_void_p]),
    ("w90g_profile_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, _c_double_p, _c_int_p]),
    ("w90g_profile_kernel_name", C.c_char_p, [C.c_int]),
    ("w90g_profile_exp_products", C.c_double, [C.c_void_p]),
    ("w90g_measure_fp64_peak", C.c_double, []),
    ("w90g_server_create", C.c_void_p, [C.c_double, C.c_int, C.c_int]),
    ("w90g_server_submit", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]),
    ("w90g_server_poll", C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), _c_int_p, _c_double_p, _c_double_p,
                                   _c_double_p, C.c_int]),
    ("w90g_server_pending", C.c_int, [C.c_void_p]),
    ("w90g_server_drain", None, [C.c_void_p]),
    ("w90g_server_stats", None, [C.c_void_p, _c_double_p]),
    ("w90g_server_now", C.c_double, [C.c_void_p]),
    ("w90g_server_delete", None, [C.c_void_p]),
    ("w90g_ws_vectors", C.c_int, [_c_double_p, _c_int_p, _c_int_p, C.c_double, _c_int_p, _c_int_p, C.c_int]),
    ("w90g_project_overlap_noalloc", C.c_int,
     [C.c_int, C.c_int, C.c_int, _c_int_p, C.c_void_p, C.c_void_p, C.c_void_p]),
]


def lib_path():
    """The in-tree library; W90G_LIBRARY names another build of it (the test of the
    kernels' bounded-wait path loads one compiled with a tiny spin limit)."""
    return os.environ.get("W90G_LIBRARY") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib",
                                                           "libw90gb300.so")


def lib():
    """Load (once) and return the native library; raise if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(
            "wannier90_gb300 native library not found at %s; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)" % path)
    L = C.CDLL(path)
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L
