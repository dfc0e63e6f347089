"""Field copies between the host and the chunk (tl_set_field / tl_get_field):
the reference layout ((x_cells + 2 halo) x (y_cells + 2 halo), x fastest) on
the host, the padded, re-pitched layout on the device.  Pageable host arrays
go through a device staging buffer; page-locked (mapped) ones are read or
written by the re-pitching kernel directly.  Both routes must give the same
bits, on grids whose rows need re-pitching and on one whose rows do not."""
import numpy as np
import pytest

import tealeaf_cuda_gb300 as tl
from tests import decks

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx", [100, 126, 37])
def test_field_round_trip_pageable_and_pinned(nx):
    torch = pytest.importorskip("torch")
    cfg = tl.parse_deck(decks.make_deck(x_cells=nx, y_cells=23, end_step=1))
    rng = np.random.default_rng(nx)
    with tl.Chunk(cfg) as ch:
        ch.start()
        a = rng.normal(size=ch.shape)
        ch.set_field("u", a)  # pageable: staged copy
        got = ch.get_field("u")
        assert np.array_equal(got, a)
        pin = torch.empty(ch.shape, dtype=torch.float64, pin_memory=True).numpy()
        pin[...] = rng.normal(size=ch.shape)
        ch.set_field("p", pin)  # page-locked: the kernel reads it directly
        out = torch.zeros(ch.shape, dtype=torch.float64, pin_memory=True).numpy()
        ch.get_field("p", out=out)  # and writes it directly
        assert np.array_equal(out, pin)
        assert np.array_equal(ch.get_field("p"), pin)  # pageable read of the same field
        assert np.array_equal(ch.get_field("u"), a)    # the other field untouched
