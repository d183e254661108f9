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


def test_noalloc_binning_matches_the_oracle():
    """The same binning against the oracle's cells (the reference's CPU
    updateCellsCPU restated) at the same positions, not only against the
    context's own GPU binning."""
    torch = pytest.importorskip("torch")
    from oracle import Oracle
    for sc in (S.suspension(n_side=4, rings=4, T=0.3), S.lj_fluid(n_side=40, seed_pos=7, seed_vel=8)):
        pos, box, grid, _, _ = context_cells(sc)
        o = Oracle(image_mode=1, log_mode=1)
        sc.replay(o)
        o.set_positions_array(pos)
        o.build_nn()
        ost, oids = o.cells()
        got_st, got_ids = noalloc_cells(torch, pos, box, grid)
        assert np.array_equal(got_st, ost)
        assert np.array_equal(got_ids, oids)


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


def call(lib, d_pos, n, box, grid, d_start, d_ids, stream):
    return lib.femmd_bin_cells_noalloc(C.c_void_p(d_pos.data_ptr()) if d_pos is not None else None, n, box[0],
                                       box[1], grid[0], grid[1], C.c_void_p(d_start.data_ptr()),
                                       C.c_void_p(d_ids.data_ptr()) if d_ids is not None else None,
                                       C.c_void_p(stream) if stream else None)


def test_noalloc_with_no_particles_gives_empty_cells():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    d_start = torch.full((5 * 4 + 1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert call(lib, None, 0, (10.0, 8.0), (5, 4), d_start, None, 0) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_start.cpu().numpy(), np.zeros(21, np.int32))


def test_noalloc_on_a_side_stream():
    """The work goes to the caller's stream: synchronising that stream alone
    is enough to read the result."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    pos, box, grid, st, ids = context_cells(S.lj_fluid(n_side=30, seed_pos=11, seed_vel=12))
    n = pos.shape[0]
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        d_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
        d_start = torch.full((grid[0] * grid[1] + 1,), -7, dtype=torch.int32, device="cuda")
        d_ids = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        assert call(lib, d_pos, n, box, grid, d_start, d_ids, side.cuda_stream) == 0
    side.synchronize()
    assert np.array_equal(d_start.cpu().numpy(), st)
    assert np.array_equal(d_ids.cpu().numpy(), ids)


def test_noalloc_captured_into_a_graph_and_replayed_on_two_systems():
    """A warm call, then one call captured into a CUDA graph on a torch
    stream; the graph is replayed on two systems of the same size and box
    (positions copied into the captured buffer before each replay), and each
    replay equals the context's binning of that system."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    a = context_cells(S.lj_fluid(n_side=32, seed_pos=21, seed_vel=22))
    b = context_cells(S.lj_fluid(n_side=32, seed_pos=23, seed_vel=24))
    assert a[1] == b[1] and tuple(a[2]) == tuple(b[2])
    pos, box, grid = a[0], a[1], a[2]
    n = pos.shape[0]
    d_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    d_start = torch.zeros((grid[0] * grid[1] + 1,), dtype=torch.int32, device="cuda")
    d_ids = torch.zeros((n,), dtype=torch.int32, device="cuda")
    cap = torch.cuda.Stream()
    with torch.cuda.stream(cap):
        assert call(lib, d_pos, n, box, grid, d_start, d_ids, cap.cuda_stream) == 0
    cap.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=cap):
        st = call(lib, d_pos, n, box, grid, d_start, d_ids, torch.cuda.current_stream().cuda_stream)
    assert st == 0
    for pos_k, _, _, st_k, ids_k in (b, a, b):
        d_start.fill_(-7)
        d_ids.fill_(-7)
        d_pos.copy_(torch.from_numpy(np.ascontiguousarray(pos_k, np.float32)))
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(d_start.cpu().numpy(), st_k)
        assert np.array_equal(d_ids.cpu().numpy(), ids_k)
