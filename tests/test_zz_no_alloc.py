"""femmd_bin_cells_noalloc: cell binning for callers that cannot allocate.

Some callers of this library cannot call cudaMalloc at the point where they
need particles binned: a simulation loop being captured into a CUDA graph, or
a host framework that owns all device memory through its own pool.  The
entry point takes device pointers for the positions and both outputs and
keeps its working memory in a fixed-size array that lives in the library.

This test calls it through the C ABI on caller-owned device buffers and
compares its output with the context's own binning (femmd_build_neighbor_list
then femmd_get_cells), which must agree exactly (integer cell lists).  It runs
two systems back to back and then the first one again, so a call that
inherited the previous call's working memory would be caught.  The file is
named so that pytest collects it last.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import femmd_old_gb300 as F
from femmd_old_gb300 import _lib
from femmd_old_gb300 import scene as S

pytestmark = pytest.mark.gpu


def context_cells(sc):
    s = F.System(0)
    sc.replay(s)
    s.build_nn()
    st, ids = s.cells()
    box = s.get_box()
    return s.positions(), (box["x"], box["y"]), s.grid(), st, ids


def noalloc_cells(torch, pos, box, grid):
    lib = _lib.load()
    n = pos.shape[0]
    ncx, ncy = grid
    d_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    d_start = torch.full((ncx * ncy + 1,), -7, dtype=torch.int32, device="cuda")
    d_ids = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.femmd_bin_cells_noalloc(C.c_void_p(d_pos.data_ptr()), n, box[0], box[1], ncx, ncy,
                                     C.c_void_p(d_start.data_ptr()), C.c_void_p(d_ids.data_ptr()), None)
    torch.cuda.synchronize()
    assert st == 0, _lib.STATUS.get(st, st)
    return d_start.cpu().numpy(), d_ids.cpu().numpy()[:n]


def test_noalloc_binning_matches_context_binning_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    a = context_cells(S.suspension(n_side=4, rings=4, T=0.3))
    b = context_cells(S.lj_fluid(n_side=40, seed_pos=5, seed_vel=6))
    for pos, box, grid, st, ids in (a, b, a):
        got_st, got_ids = noalloc_cells(torch, pos, box, grid)
        assert np.array_equal(got_st, st)
        assert np.array_equal(got_ids, ids)


def header_limit(name):
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "femmd.h")
    m = re.search(r"#define\s+" + name + r"\s+\(?([0-9]+)\s*<<\s*([0-9]+)\)?", open(hdr).read())
    return int(m.group(1)) << int(m.group(2))


def test_noalloc_rejects_sizes_beyond_its_maximum():
    lib = _lib.load()
    too_many = header_limit("FEMMD_NOALLOC_MAX_PARTICLES")
    # no device work is issued for a rejected call, so null device pointers are fine here
    st = lib.femmd_bin_cells_noalloc(None, too_many + 1, 10.0, 10.0, 3, 3, C.c_void_p(1), C.c_void_p(1), None)
    assert _lib.STATUS[st] == "CAPACITY_OVERFLOW"
    side = int(header_limit("FEMMD_NOALLOC_MAX_CELLS") ** 0.5) + 1
    st = lib.femmd_bin_cells_noalloc(None, 0, 10.0, 10.0, side, side, C.c_void_p(1), None, None)
    assert _lib.STATUS[st] == "CAPACITY_OVERFLOW"
