"""The allocation-free cell order, idpd_cell_order_noalloc, through the C ABI.

Some callers cannot allocate device memory: a host MD code whose memory pool
owns the whole device budget, or a step loop that must not pay the
device-wide synchronisation of cudaMalloc / cudaFree. This entry point serves
them from one static scratch array of the library. These tests hand it
device buffers owned by the caller (torch here) and check its output against
the engine's own idpd_cell_order at its default tuning (cell reach 1, skin
0), which is integer work and must agree bit for bit: two calls in a row on
the same buffers, then the same on a smaller grid (the scratch keeps the
larger grid's counts, which the next call must not see). The file runs last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import mdpd_params, mixed_system
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.engine import Engine, last_error, load

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

IDPD_OK = 0
IDPD_ERR_CAPACITY = 2
MAX_ROWS = 1 << 20


def _noalloc(pos_d, n, box, cell_d, perm_d):
    L = load()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.idpd_cell_order_noalloc(
        C.c_void_p(pos_d.data_ptr() if pos_d is not None else 0), n,
        np.ascontiguousarray(box, np.float64),
        C.c_void_p(cell_d.data_ptr() if cell_d is not None else 0),
        C.c_void_p(perm_d.data_ptr() if perm_d is not None else 0), C.c_void_p(stream))
    return rc


def _engine_order(box, st):
    e = Engine()
    e.set_params(mdpd_params(box))
    e.upload(st)
    return e.cell_order()


def _systems():
    """The larger grid first (13 x 12 x 14 cells), then a smaller one (9 x 10 x 11)."""
    box1, st1, _ = mixed_system()
    st2 = configs.liquid((13.5, 12.0, 14.7), 3.0, seed=5)
    return [(np.array([13.5, 12.0, 14.7]), st2), (np.asarray(box1, np.float64), st1)]


def test_noalloc_cell_order_matches_cell_order_on_two_calls():
    for box, st in _systems():
        cell_ref, perm_ref = _engine_order(box, st)
        n = len(st["pos"])
        pos_d = torch.from_numpy(st["pos"]).to("cuda")
        cell_d = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        perm_d = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        for call in range(2):  # two calls in a row on the same buffers
            rc = _noalloc(pos_d, n, box, cell_d, perm_d)
            assert rc == IDPD_OK, last_error()
            torch.cuda.synchronize()
            cell = cell_d.cpu().numpy().view(np.uint32)
            perm = perm_d.cpu().numpy().view(np.uint32)
            assert np.array_equal(cell, cell_ref), f"call {call}"
            assert np.array_equal(perm, perm_ref), f"call {call}"


def test_noalloc_grid_is_the_default_tuning_grid_only():
    # reach 2 gives idpd_cell_order twice the cells per axis; the
    # allocation-free call keeps floor(box) cells per axis
    box = np.array([13.5, 12.0, 14.7])
    st = configs.liquid(box, 3.0, seed=5)
    n = len(st["pos"])
    e = Engine()
    e.set_params(mdpd_params(box))
    e.upload(st)
    e.set_tuning(2, 0.0)
    cell2, _ = e.cell_order()
    e.close()
    pos_d = torch.from_numpy(st["pos"]).to("cuda")
    cell_d = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    perm_d = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    assert _noalloc(pos_d, n, box, cell_d, perm_d) == IDPD_OK, last_error()
    torch.cuda.synchronize()
    cell1 = cell_d.cpu().numpy().view(np.uint32)
    nc1 = np.floor(box).astype(np.int64)
    inv_cs = nc1 / box  # cell index = trunc(x * (nc / box)), clamped to the grid
    c1 = np.clip((st["pos"] * inv_cs).astype(np.int64), 0, nc1 - 1)
    assert np.array_equal(cell1, (c1[:, 2] * nc1[1] + c1[:, 1]) * nc1[0] + c1[:, 0])
    assert cell2.max() >= np.prod(nc1)  # the reach-2 grid has 8x the cells


def test_noalloc_rejects_sizes_beyond_its_scratch():
    # Too many cells: rejected before any device work (n = 0, no arrays).
    rc = _noalloc(None, 0, np.array([100.0, 100.0, 100.0]), None, None)
    assert rc == IDPD_ERR_CAPACITY
    assert "cells" in last_error()
    # Too many rows, with real buffers of that size.
    n = MAX_ROWS + 1
    pos_d = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    cell_d = torch.zeros((n,), dtype=torch.int32, device="cuda")
    perm_d = torch.zeros((n,), dtype=torch.int32, device="cuda")
    rc = _noalloc(pos_d, n, np.array([10.0, 10.0, 10.0]), cell_d, perm_d)
    assert rc == IDPD_ERR_CAPACITY
    assert "rows" in last_error()
    torch.cuda.synchronize()
