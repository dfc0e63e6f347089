"""tealeaf_cuda_gb300 -- GB300 (sm_103a) CUDA implementation of TeaLeaf's
implicit heat-conduction solve.

The product is the C-ABI library `_build/libtealeaf_gb300.so` (declared in
include/tealeaf_capi.h).  This module is the Python side of that boundary:
ctypes mirrors of the public structs, the `tl_*` handle API (`Chunk`,
`parse_deck`, `run_deck`) and the reference-named entry points (`legacy`),
whose argument meaning follows the reference's *_kernel_cuda_ functions.

There is no CPU fallback: if the library is missing or cannot load, the
import-time `load()` raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtealeaf_gb300.so")

# status codes and enumerations (include/tealeaf_capi.h)
TL_OK, TL_WARN_MAXITER = 0, 1
TL_ERR_ARG, TL_ERR_CUDA, TL_ERR_ALLOC, TL_ERR_BREAKDOWN = -1, -2, -3, -4
TL_ERR_STATE, TL_ERR_DECK, TL_ERR_EIGEN = -5, -6, -7
SOLVER_JACOBI, SOLVER_CG, SOLVER_CHEBYSHEV, SOLVER_PPCG = 1, 2, 3, 4
PREC_NONE, PREC_JAC_DIAG, PREC_JAC_BLOCK = 1, 2, 3
PRECISION_FP64, PRECISION_MIXED = 0, 1
WARM_NONE, WARM_LEARNED, WARM_PREV = 0, 1, 2
WARM_PROJ_ENERGY, WARM_PROJ_RESIDUAL = 0, 1
FIELDS = {"density": 1, "energy0": 2, "energy1": 3, "u": 4, "p": 5, "sd": 6, "r": 7,
          "u0": 8, "w": 9, "z": 10, "kx": 11, "ky": 12, "mi": 13, "cp": 14, "bfp": 15,
          "volume": 16, "rtemp": 17, "utemp": 18, "r_store": 19}
MAX_STATES = 64


class State(C.Structure):
    _fields_ = [("geometry", C.c_int), ("density", C.c_double), ("energy", C.c_double),
                ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
                ("ymax", C.c_double), ("radius", C.c_double)]


class Config(C.Structure):
    _fields_ = [("x_cells", C.c_int), ("y_cells", C.c_int),
                ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double),
                ("dtinit", C.c_double), ("end_time", C.c_double),
                ("end_step", C.c_int), ("summary_frequency", C.c_int),
                ("max_iters", C.c_int), ("eps", C.c_double),
                ("solver", C.c_int), ("precond", C.c_int), ("coefficient", C.c_int),
                ("halo_depth", C.c_int), ("reflective_boundary", C.c_int), ("check_result", C.c_int),
                ("ch_cg_presteps", C.c_int), ("ch_cg_epslim", C.c_double), ("ppcg_inner_steps", C.c_int),
                ("profiler_on", C.c_int), ("verbose", C.c_int), ("test_problem", C.c_int),
                ("cuda_device", C.c_int), ("precision", C.c_int), ("inner_eps", C.c_double),
                ("warm_start", C.c_int), ("nstates", C.c_int), ("states", State * MAX_STATES)]


class SolveInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("ppcg_inner_iters", C.c_int),
                ("switch_n", C.c_int), ("est_itc", C.c_int), ("outer_iters", C.c_int),
                ("inner_iters", C.c_int), ("initial_residual", C.c_double), ("error", C.c_double),
                ("error_ratio", C.c_double), ("exact_error_ratio", C.c_double),
                ("eigmin", C.c_double), ("eigmax", C.c_double), ("rx", C.c_double),
                ("ry", C.c_double), ("seconds", C.c_double), ("warm_used", C.c_int),
                ("warm_ratio", C.c_double), ("warm_net_share", C.c_double)]


class StepRecord(C.Structure):
    _fields_ = [("step", C.c_int), ("time", C.c_double), ("dt", C.c_double), ("solve", SolveInfo),
                ("has_summary", C.c_int), ("vol", C.c_double), ("mass", C.c_double),
                ("ie", C.c_double), ("temp", C.c_double), ("wall", C.c_double)]


class RunOptions(C.Structure):
    _fields_ = [("out_path", C.c_char_p), ("echo", C.c_int), ("legacy_abi", C.c_int),
                ("max_steps", C.c_int), ("records", C.POINTER(StepRecord)), ("max_records", C.c_int),
                ("model_path", C.c_char_p)]


class RunResult(C.Structure):
    _fields_ = [("status", C.c_int), ("steps", C.c_int), ("total_iterations", C.c_longlong),
                ("wall_seconds", C.c_double), ("solve_seconds", C.c_double),
                ("vol", C.c_double), ("mass", C.c_double), ("ie", C.c_double), ("temp", C.c_double),
                ("qa_checked", C.c_int), ("qa_passed", C.c_int), ("qa_diff", C.c_double),
                ("kernel_launches", C.c_longlong), ("n_records", C.c_int)]


_STRUCTS = [Config, SolveInfo, StepRecord, RunOptions, RunResult, State]
_lib = None

# reference-named entry points and their argument types (tealeaf_capi.h)
_D, _I = C.POINTER(C.c_double), C.POINTER(C.c_int)
LEGACY_SIGNATURES = {
    "initialise_cuda_": [_I, _I, _I, _I],
    "initialise_chunk_kernel_cuda_": [_D, _D, _D, _D],
    "generate_chunk_kernel_cuda_": [_I, _D, _D, _D, _D, _D, _D, _D, _I, _I, _I, _I],
    "set_field_kernel_cuda_": [],
    "field_summary_kernel_cuda_": [_D, _D, _D, _D],
    "update_halo_kernel_cuda_": [_I, _I, _I],
    "cuda_pack_buffers_": [_I, _I, _I, _I, _D],
    "cuda_unpack_buffers_": [_I, _I, _I, _I, _D],
    "tea_leaf_common_init_kernel_cuda_": [_I, _D, _D, _D, _I, _I],
    "tea_leaf_common_finalise_kernel_cuda_": [],
    "tea_leaf_calc_residual_cuda_": [],
    "tea_leaf_calc_2norm_kernel_cuda_": [_I, _D],
    "tea_leaf_cg_init_kernel_cuda_": [_D],
    "tea_leaf_cg_calc_w_kernel_cuda_": [_D],
    "tea_leaf_cg_calc_ur_kernel_cuda_": [_D, _D],
    "tea_leaf_cg_calc_p_kernel_cuda_": [_D],
    "tea_leaf_cheby_init_kernel_cuda_": [_D, _D, _I, _D],
    "tea_leaf_cheby_iterate_kernel_cuda_": [_I],
    "tea_leaf_ppcg_init_constants_cuda_": [_D, _D, _I],
    "tea_leaf_ppcg_init_kernel_cuda_": [_I, _D],
    "tea_leaf_ppcg_init_sd_kernel_cuda_": [_D],
    "tea_leaf_ppcg_init_sd_new_kernel_cuda_": [_D],
    "tea_leaf_ppcg_store_r_kernel_cuda_": [],
    "tea_leaf_ppcg_update_z_kernel_cuda_": [],
    "tea_leaf_ppcg_calc_rrn_kernel_cuda_": [_D],
    "tea_leaf_ppcg_inner_kernel_cuda_": [_I, _I, _I],
    "tea_leaf_ppcg_calc_2norm_kernel_cuda_": [_D],
    "tea_leaf_ppcg_calc_p_kernel_cuda_": [_D],
    "tea_leaf_jacobi_solve_kernel_cuda_": [_D],
}


def build(verbose=False):
    """Compile the library for sm_103a (see make_lib.py)."""
    from . import make_lib
    return make_lib.build(verbose=verbose)


def load():
    """Load the C-ABI library; raises if it is missing or does not match the
    struct layouts mirrored here."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with tealeaf_cuda_gb300.build() "
                           "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    lib.tl_sizeof.restype = C.c_longlong
    lib.tl_sizeof.argtypes = [C.c_int]
    for k, s in enumerate(_STRUCTS):
        if lib.tl_sizeof(k) != C.sizeof(s):
            raise RuntimeError(f"ABI mismatch for {s.__name__}: C {lib.tl_sizeof(k)} vs ctypes {C.sizeof(s)}")
    lib.tl_last_error.restype = C.c_char_p
    lib.tl_version.restype = C.c_char_p
    lib.tl_parse_deck.argtypes = [C.c_char_p, C.POINTER(Config), C.c_char_p, C.c_int]
    lib.tl_chunk_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    lib.tl_chunk_destroy.argtypes = [C.c_void_p]
    lib.tl_start.argtypes = [C.c_void_p, _D, _D, _D, _D]
    lib.tl_timestep.argtypes = [C.c_void_p, C.POINTER(SolveInfo)]
    lib.tl_field_summary.argtypes = [C.c_void_p, _D, _D, _D, _D]
    lib.tl_get_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.tl_set_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.tl_set_dt.argtypes = [C.c_void_p, C.c_double]
    lib.tl_set_inner_fusion.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
    lib.tl_kernel_launches.restype = C.c_longlong
    lib.tl_kernel_launches.argtypes = [C.c_void_p]
    lib.tl_default_chunk.restype = C.c_void_p
    lib.tl_default_chunk_init.argtypes = [C.POINTER(Config)]
    lib.tl_run_deck.argtypes = [C.c_char_p, C.POINTER(RunOptions), C.POINTER(RunResult)]
    lib.tl_warm_start_param_count.restype = C.c_longlong
    lib.tl_set_warm_start_model.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong]
    lib.tl_set_warm_start_options.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.tl_warm_start_features.argtypes = [C.c_void_p, C.c_void_p]
    _vp, _i, _f = C.c_void_p, C.c_int, C.c_float
    lib.tl_nn_conv.argtypes = [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp]
    lib.tl_nn_gelu_backward.argtypes = [_vp, _vp, _vp, _i, _i, _i, _i, _vp]
    lib.tl_nn_wgrad_partial_floats.restype = C.c_longlong
    lib.tl_nn_wgrad_partial_floats.argtypes = [_i, _i, _i, _i, _i, _i]
    lib.tl_nn_wgrad.argtypes = [_vp, _vp, _i, _i, _vp, _vp, _vp, _i, _i, _i, _i, _vp]
    lib.tl_nn_adam.argtypes = [_vp, _vp, _vp, _vp, _i, _f, _f, _f, _f, _i, _vp]
    lib.tl_nn_pack.argtypes = [_vp, _vp, _vp, _i, _i, _vp]
    lib.tl_nn_loss.argtypes = [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _i, _vp]
    lib.tl_nn_gather.argtypes = [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _i, _i, _vp]
    for name, args in LEGACY_SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = None
    _lib = lib
    return lib


class TeaLeafError(RuntimeError):
    def __init__(self, code, what):
        msg = load().tl_last_error().decode()
        super().__init__(f"{what} failed ({code}): {msg}")
        self.code = code


def _check(rc, what):
    if rc < 0:
        raise TeaLeafError(rc, what)
    return rc


def last_error():
    return load().tl_last_error().decode()


def parse_deck(text):
    """tea.in text -> Config (parse.f90 / read_input.f90 semantics)."""
    lib = load()
    cfg = Config()
    err = C.create_string_buffer(256)
    rc = lib.tl_parse_deck(text.encode(), C.byref(cfg), err, 256)
    if rc < 0:
        raise ValueError(f"deck error: {err.value.decode()}")
    return cfg


def _info_dict(info):
    return {k: getattr(info, k) for k, _ in SolveInfo._fields_}


class Chunk:
    """One TeaLeaf chunk on the GPU (the tl_* handle API)."""

    def __init__(self, cfg):
        lib = load()
        self.cfg = cfg
        self._h = C.c_void_p()
        _check(lib.tl_chunk_create(C.byref(cfg), C.byref(self._h)), "tl_chunk_create")
        self.shape = (cfg.y_cells + 2 * cfg.halo_depth, cfg.x_cells + 2 * cfg.halo_depth)

    def close(self):
        if self._h:
            load().tl_chunk_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def start(self):
        v = [C.c_double() for _ in range(4)]
        _check(load().tl_start(self._h, *[C.byref(x) for x in v]), "tl_start")
        return tuple(x.value for x in v)

    def set_warm_start_options(self, history=8, projection=WARM_PROJ_ENERGY):
        """increments the warm start combines (1..8) and its projection's
        inner product (WARM_PROJ_ENERGY or WARM_PROJ_RESIDUAL)"""
        _check(load().tl_set_warm_start_options(self._h, history, projection), "tl_set_warm_start_options")

    def set_dt(self, dt):
        _check(load().tl_set_dt(self._h, dt), "tl_set_dt")

    def set_inner_fusion(self, steps, seg_strips=0, fold_rrn=False):
        """FP32 PPCG inner steps per HBM pass (1..5), strips per CTA share
        (0: automatic), and whether the last pass also sums PPCG's rrn"""
        _check(load().tl_set_inner_fusion(self._h, steps, seg_strips, 1 if fold_rrn else 0),
               "tl_set_inner_fusion")

    def timestep(self):
        info = SolveInfo()
        _check(load().tl_timestep(self._h, C.byref(info)), "tl_timestep")
        return _info_dict(info)

    def field_summary(self):
        v = [C.c_double() for _ in range(4)]
        _check(load().tl_field_summary(self._h, *[C.byref(x) for x in v]), "tl_field_summary")
        return tuple(x.value for x in v)

    def get_field(self, name, out=None):
        """the whole padded field (device -> host); into `out` (C-contiguous
        float64 of self.shape, e.g. pinned) when given"""
        a = np.empty(self.shape, dtype=np.float64) if out is None else out
        assert a.shape == self.shape and a.dtype == np.float64 and a.flags.c_contiguous
        _check(load().tl_get_field(self._h, FIELDS[name], a.ctypes.data), "tl_get_field")
        return a

    def set_field(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == self.shape
        _check(load().tl_set_field(self._h, FIELDS[name], a.ctypes.data), "tl_set_field")

    def interior(self, name):
        h = self.cfg.halo_depth
        return self.get_field(name)[h:-h, h:-h]

    @property
    def kernel_launches(self):
        return load().tl_kernel_launches(self._h)


def run_deck(text, legacy_abi=False, max_steps=0, out_path=None, echo=False, max_records=4096,
             model_path=None):
    """Run a whole deck (tea_leaf.f90 main program); returns (records, result)."""
    lib = load()
    recs = (StepRecord * max_records)()
    opt = RunOptions(out_path.encode() if out_path else None, 1 if echo else 0,
                     1 if legacy_abi else 0, max_steps, recs, max_records,
                     model_path.encode() if model_path else None)
    res = RunResult()
    rc = lib.tl_run_deck(text.encode(), C.byref(opt), C.byref(res))
    _check(rc, "tl_run_deck")
    out = []
    for k in range(res.n_records):
        r = recs[k]
        d = {"step": r.step, "time": r.time, "dt": r.dt, "has_summary": r.has_summary,
             "vol": r.vol, "mass": r.mass, "ie": r.ie, "temp": r.temp, "wall": r.wall}
        d.update(_info_dict(r.solve))
        out.append(d)
    return out, {k: getattr(res, k) for k, _ in RunResult._fields_}


class _Legacy:
    """The reference-named entry points, by reference like the Fortran
    interface: `legacy.call("tea_leaf_cg_calc_w_kernel_cuda_", out=1)`
    returns the output double(s)."""

    def __getattr__(self, name):
        return getattr(load(), name)


legacy = _Legacy()
