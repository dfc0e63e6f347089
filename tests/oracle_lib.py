"""ctypes access to the CPU oracle's per-kernel entry points
(oracle/tea_oracle.h), for the kernel-level parity tests.  Test
infrastructure only."""
import ctypes as C

import numpy as np

from tests.oracle_run import ORACLE_LIB, build_oracle

_lib = None
_D = C.POINTER(C.c_double)

FIELD = {"density": 1, "energy0": 2, "energy1": 3, "u": 4, "p": 5, "sd": 6, "r": 7, "u0": 8,
         "w": 9, "z": 10, "kx": 11, "ky": 12, "mi": 13, "cp": 14, "bfp": 15, "volume": 16,
         "rtemp": 17, "utemp": 18, "r_store": 19}


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        l = C.CDLL(ORACLE_LIB)
        l.ora_parse_deck.argtypes = [C.c_char_p, C.c_void_p, C.c_char_p, C.c_int]
        l.ora_chunk_new.restype = C.c_void_p
        l.ora_chunk_new.argtypes = [C.c_void_p]
        l.ora_chunk_free.argtypes = [C.c_void_p]
        l.ora_start.argtypes = [C.c_void_p, C.c_void_p]
        l.ora_get_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        l.ora_set_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        l.ora_common_init.argtypes = [C.c_void_p, C.c_double, _D, _D]
        for n in ("ora_calc_residual", "ora_ppcg_store_r", "ora_ppcg_update_z", "ora_finalise"):
            getattr(l, n).argtypes = [C.c_void_p]
        for n in ("ora_cg_init", "ora_cg_calc_w", "ora_ppcg_calc_rrn", "ora_ppcg_calc_zrnorm",
                  "ora_jacobi_solve"):
            getattr(l, n).argtypes = [C.c_void_p]
            getattr(l, n).restype = C.c_double
        l.ora_calc_2norm.argtypes = [C.c_void_p, C.c_int]
        l.ora_calc_2norm.restype = C.c_double
        l.ora_cg_calc_ur.argtypes = [C.c_void_p, C.c_double]
        l.ora_cg_calc_ur.restype = C.c_double
        l.ora_cg_calc_p.argtypes = [C.c_void_p, C.c_double]
        l.ora_ppcg_calc_p.argtypes = [C.c_void_p, C.c_double]
        l.ora_cheby_init.argtypes = [C.c_void_p, _D, _D, C.c_int, C.c_double]
        l.ora_cheby_iterate.argtypes = [C.c_void_p, C.c_int]
        l.ora_ppcg_init_constants.argtypes = [C.c_void_p, _D, _D, C.c_int]
        l.ora_ppcg_init.argtypes = [C.c_void_p, C.c_int]
        l.ora_ppcg_init.restype = C.c_double
        l.ora_ppcg_init_sd_new.argtypes = [C.c_void_p, C.c_double]
        l.ora_ppcg_inner.argtypes = [C.c_void_p, C.c_int]
        l.ora_field_summary.argtypes = [C.c_void_p, _D, _D, _D, _D]
        l.ora_update_halo.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int]
        _lib = l
    return _lib


class OracleChunk:
    def __init__(self, deck_text):
        l = lib()
        self.cfg = C.create_string_buffer(1 << 16)
        err = C.create_string_buffer(256)
        rc = l.ora_parse_deck(deck_text.encode(), self.cfg, err, 256)
        assert rc == 0, err.value
        self.h = C.c_void_p(l.ora_chunk_new(self.cfg))
        self.res = C.create_string_buffer(4096)
        l.ora_start(self.h, self.res)

    def __del__(self):
        try:
            lib().ora_chunk_free(self.h)
        except Exception:
            pass

    def field(self, name, shape):
        a = np.empty(shape, dtype=np.float64)
        lib().ora_get_field(self.h, FIELD[name], a.ctypes.data)
        return a

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        lib().ora_set_field(self.h, FIELD[name], a.ctypes.data)

    def __getattr__(self, name):
        f = getattr(lib(), "ora_" + name)
        return lambda *a: f(self.h, *a)
