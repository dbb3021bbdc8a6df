"""ctypes binding of libspherocyl's C ABI (include/spherocyl.h).

The shared library is built in-tree (``spherocyls_gb300/build.py``).  There is no
fallback: importing the package works without it, but the first call that needs
the library raises if it has not been built.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(PKG, "lib", "libspherocyl.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_llp = ctypes.POINTER(ctypes.c_longlong)
_vp = ctypes.c_void_p

SC_OK = 0
SC_E_ARG = 1
SC_E_IO = 2
SC_E_NAN = 3
SC_E_OVERFLOW = 4
SC_E_NOCONV = 5
SC_E_TIMEOUT = 6
SC_E_CUDA = 7
SC_E_STATE = 8
SC_E_NOMEM = 9

PREC = {"fp64": 0, "mixed": 1}
STRESS = {"compat": 0, "virial": 1}
PASS = {"auto": 0, "list": 1, "tile": 2}


class ScOptions(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int),
        ("stress_mode", ctypes.c_int),
        ("device", ctypes.c_int),
        ("max_nbrs", ctypes.c_int),
        ("use_graphs", ctypes.c_int),
        ("block", ctypes.c_int),
        ("profile", ctypes.c_int),
        ("contact_model", ctypes.c_int),
        ("stage_inputs", ctypes.c_int),
        ("cg_max_probes", ctypes.c_int),
        ("pass_kind", ctypes.c_int),
        ("tile_target", ctypes.c_int),
        ("persist_steps", ctypes.c_int),
    ]


class ScGenOptions(ctypes.Structure):
    _fields_ = [
        ("layout", ctypes.c_int),
        ("angle_mode", ctypes.c_int),
        ("angle_min", ctypes.c_double),
        ("angle_max", ctypes.c_double),
        ("shear_angles", ctypes.c_int),
        ("min_sep", ctypes.c_double),
        ("max_overlap", ctypes.c_double),
        ("a_sigma", ctypes.c_double),
    ]


# (name, restype, argtypes) of every entry point declared in include/spherocyl.h
SIGNATURES = [
    ("sc_version", ctypes.c_char_p, []),
    ("sc_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("sc_default_options", None, [ctypes.POINTER(ScOptions)]),
    ("sc_create", ctypes.c_int, [ctypes.POINTER(ScOptions), ctypes.c_int, _ip, _dp, _dp, _dp, _dp,
                                 _dp, _dp, _dp, ctypes.POINTER(_vp)]),
    ("sc_destroy", ctypes.c_int, [_vp]),
    ("sc_last_error", ctypes.c_char_p, [_vp]),
    ("sc_set_stream", ctypes.c_int, [_vp, _vp]),
    ("sc_synchronize", ctypes.c_int, [_vp]),
    ("sc_set_strain_rate", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    ("sc_set_resize_rate", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    ("sc_set_step", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    ("sc_set_gamma", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    ("sc_set_total_gamma", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    ("sc_find_neighbors", ctypes.c_int, [_vp]),
    ("sc_calc_forces", ctypes.c_int, [_vp]),
    ("sc_calc_se", ctypes.c_int, [_vp, _dp]),
    ("sc_strain_steps", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    ("sc_resize_steps", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]),
    ("sc_pure_strain_steps", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    ("sc_strain_to_gamma", ctypes.c_int, [_vp, ctypes.c_double, ctypes.POINTER(ctypes.c_long)]),
    ("sc_trim_memory", ctypes.c_int, [ctypes.c_int]),
    ("sc_gd_minimize", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, _ip, _dp]),
    ("sc_cg_minimize", ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _ip]),
    ("sc_fire_minimize", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, _ip, _dp, _ip]),
    ("sc_fire_iterations", ctypes.c_int, [_vp, _ip]),
    ("sc_affine_scale", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    ("sc_quasistatic_compress", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp,
                                               _ip]),
    ("sc_find_jam", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _ip]),
    ("sc_autotune", ctypes.c_int, [_vp, ctypes.c_int, _dp, _ip]),
    ("sc_get_options", ctypes.c_int, [_vp, ctypes.c_void_p]),
    ("sc_flip_shear", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sc_rotate_shear", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sc_create_rect", ctypes.c_int, [ctypes.POINTER(ScOptions), ctypes.c_int, _ip, _dp, _dp,
                                      _dp, _dp, _dp, _dp, _dp, _dp,
                                      ctypes.POINTER(ctypes.c_void_p)]),
    ("sc_get_state", ctypes.c_int, [_vp, _dp, _dp, _dp]),
    ("sc_get_forces", ctypes.c_int, [_vp, _dp, _dp, _dp]),
    ("sc_get_box", ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    ("sc_get_pairs", ctypes.c_int, [_vp, ctypes.c_int, _ip, ctypes.c_long,
                                    ctypes.POINTER(ctypes.c_long)]),
    ("sc_get_counters", ctypes.c_int, [_vp, _llp]),
    ("sc_get_pass_times", ctypes.c_int, [_vp, _dp]),
    ("sc_generate_packing", ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                           ctypes.c_double, _dp, _dp, _dp, _dp, _dp, _dp]),
    ("sc_default_gen_options", None, [_vp]),
    ("sc_generate_config", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                          _dp, _dp, _dp, _dp, _dp, _dp]),
    ("sc_generate_packing_device", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_uint64,
                                                  ctypes.c_double, _dp, _dp, _dp, _dp, _dp, _dp]),
    ("sc_generate_config_rect", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_uint64, _dp, _dp, _dp,
                                               _dp, _dp, _dp, _dp]),
    ("sc_read_positions", ctypes.c_int, [ctypes.c_char_p, _ip, _dp, _dp, _dp, _dp, _dp, _dp]),
    ("sc_save_positions", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]),
    ("sc_write_positions", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                          _dp, _dp, _dp, _dp]),
    ("sc_run_strain", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_ulong, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_ulong)]),
    ("sc_run_resize", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_ulong, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_ulong)]),
    ("sc_run_pure_strain", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_ulong,
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_ulong)]),
    ("sc_run_minimize", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int, _ip]),
    ("sc_run_find_jam", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_int, _ip, _dp]),
    ("sc_run_y_compress", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int, _ip, _dp]),
    ("sc_run_qs_compress", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_int, _ip]),
    ("sc_forces_noalloc", ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                         _vp]),
    ("sc_noalloc_last_error", ctypes.c_char_p, []),
]

_LIB = None


class ScError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def lib() -> ctypes.CDLL:
    """Load libspherocyl (raises when it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(
                f"libspherocyl is not built ({LIBPATH} missing); run "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIBPATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, handle=None) -> None:
    if status != SC_OK:
        msg = lib().sc_last_error(handle)
        raise ScError(status, msg.decode() if msg else "")
