"""tl_dot_noalloc, the allocation-free entry point, against the existing
reduction entry point tea_leaf_calc_2norm_kernel_cuda_.

Callers that cannot let the library allocate (a host that fixed its device
memory budget at start-up, or whose device memory belongs to another
allocator) pass their own device arrays; the reduction's scratch is a fixed
device array inside the library.  Here the test owns the device arrays
(torch tensors) and checks two calls in a row against the chunk's own
reduction, within the 1e-12 relative tolerance the other dot-product tests
use.  This file is collected last so a stop-at-first-failure run has run
every other test before it."""
import ctypes as C

import numpy as np
import pytest

import tealeaf_cuda_gb300 as tl
from tests import decks

pytestmark = pytest.mark.gpu


def _lib():
    lib = tl.load()
    lib.tl_dot_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_longlong,
                                   C.c_void_p, C.c_void_p]
    lib.tl_dot_noalloc.restype = C.c_int
    return lib


def test_dot_noalloc_matches_calc_2norm_twice():
    torch = pytest.importorskip("torch")
    lib = _lib()
    nx, ny = 300, 203
    deck = decks.make_deck(x_cells=nx, y_cells=ny, end_step=1, tl_preconditioner_type="jac_diag")
    cfg = tl.parse_deck(deck)
    assert lib.tl_default_chunk_init(C.byref(cfg)) == 0, tl.last_error()
    h = lib.tl_default_chunk()
    v = [C.c_double() for _ in range(4)]
    assert lib.tl_start(h, *[C.byref(x) for x in v]) == 0
    by = C.byref
    coef, dt, rx, ry = C.c_int(1), C.c_double(0.004), C.c_double(), C.c_double()
    zero, refl = (C.c_int * 4)(1, 1, 1, 1), C.c_int(0)
    lib.tea_leaf_common_init_kernel_cuda_(by(coef), by(dt), by(rx), by(ry), zero, by(refl))
    lib.tea_leaf_calc_residual_cuda_()
    expect = {}
    for which in (0, 1):  # u0.u0 and r.r through the existing entry point
        arr, out = C.c_int(which), C.c_double()
        lib.tea_leaf_calc_2norm_kernel_cuda_(by(arr), by(out))
        expect[which] = out.value
    hd = cfg.halo_depth
    shape = (ny + 2 * hd, nx + 2 * hd)
    fields, independent = {}, {}
    for which, name in ((0, "u0"), (1, "r")):
        host = np.empty(shape, dtype=np.float64)
        assert lib.tl_get_field(h, tl.FIELDS[name], host.ctypes.data) == 0
        fields[which] = torch.from_numpy(host).to("cuda:0")  # caller-owned device memory
        inner = host[hd:hd + ny, hd:hd + nx].ravel()
        independent[which] = float(np.dot(inner, inner))
    pitch = shape[1]
    out = torch.full((4,), -1.0, dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        for which in (0, 1):
            d = fields[which]
            first = d.data_ptr() + (hd * pitch + hd) * 8  # first interior cell
            rc = lib.tl_dot_noalloc(first, first, nx, ny, pitch, out.data_ptr() + 8 * (2 * call + which),
                                    stream)
            assert rc == 0, tl.last_error()
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for call in range(2):
        for which in (0, 1):
            assert got[2 * call + which] == pytest.approx(expect[which], rel=1e-12), (call, which)
            # and against a sum made without the library at all
            assert got[2 * call + which] == pytest.approx(independent[which], rel=1e-12), (call, which)
    # the second call must not see the first call's leftovers
    assert got[0] == got[2] and got[1] == got[3]


def test_dot_noalloc_rejects_blocks_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = _lib()
    d = torch.zeros(16, dtype=torch.float64, device="cuda:0")
    # 12000 x 12000 cells need more tiles than the fixed scratch holds; the
    # size check fails before any access to d
    rc = lib.tl_dot_noalloc(d.data_ptr(), d.data_ptr(), 12000, 12000, 12000, d.data_ptr(), None)
    assert rc == tl.TL_ERR_ARG
    assert "scratch" in tl.last_error()
