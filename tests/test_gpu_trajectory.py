"""Trajectory frames written during runs (femmd_set_trajectory): the reference's
dump, xyz and vtk layouts, frames at the step counts that are multiples of
'every', bit-identical results with and without frames, and no duplicate
frames when a run is repeated after a list overflow.  Frame values are
printed with %f (6 decimals): compared within 5e-7 of the state a separate
run reaches at that step."""
import os

import numpy as np
import pytest

import femmd_old_gb300 as F
from femmd_old_gb300 import scene as S

pytestmark = pytest.mark.gpu


def system(sc):
    s = F.System(0)
    sc.replay(s)
    return s


def read_dump(path):
    frames = []
    with open(path) as f:
        lines = f.read().split("\n")
    k = 0
    while k < len(lines) and lines[k].startswith("ITEM: TIMESTEP"):
        step = int(lines[k + 1])
        n = int(lines[k + 3])
        rows = np.array([[float(x) for x in lines[k + 9 + j].split()] for j in range(n)])
        frames.append((step, rows))
        k += 9 + n
    return frames


def state_at(sc, runs):
    s = system(sc)
    for n in runs:
        s.run(n)
    p, v, a = s.get_state()
    return p, v


def test_frames_are_the_states_and_change_nothing(tmp_path):
    sc = S.suspension(n_side=3, rings=3, T=0.3, center_jitter=0.3)
    path = str(tmp_path / "traj.dump")
    s = system(sc)
    s.set_trajectory(path, 25, 0)
    s.run(120)
    assert s.flush_trajectory() == 4
    plain = system(sc)
    plain.run(120)
    for x, y in zip(s.get_state(), plain.get_state()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    frames = read_dump(path)
    assert [f[0] for f in frames] == [25, 50, 75, 100]
    for step, rows in frames:
        p, v = state_at(sc, [step])
        assert np.abs(rows[:, 2:4] - p).max() <= 5e-7
        assert np.abs(rows[:, 5:7] - v).max() <= 5e-7


def test_frames_across_runs_and_slot_reuse(tmp_path):
    sc = S.lj_fluid(n_side=24)
    path = str(tmp_path / "traj.dump")
    s = system(sc)
    s.set_trajectory(path, 10, 0)
    s.run(35)
    s.run(200)  # frames 40 .. 230: more than the pinned slots
    n = s.flush_trajectory()
    steps = [f[0] for f in read_dump(path)]
    assert steps == list(range(10, 231, 10)) and n == len(steps)


def test_no_duplicate_frames_after_overflow(tmp_path):
    sc = S.lj_fluid(n_side=24)
    path = str(tmp_path / "traj.dump")
    s = system(sc)
    s.run(0)
    s.set_neighbor_capacity(2)
    s.set_trajectory(path, 20, 0)
    s.run(100)
    assert s.neighbor_capacity() > 2
    assert s.flush_trajectory() == 5
    steps = [f[0] for f in read_dump(path)]
    assert steps == [20, 40, 60, 80, 100]
    plain = system(sc)
    plain.run(0)
    plain.run(100)
    for x, y in zip(s.get_state(), plain.get_state()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_xyz_and_vtk_layouts(tmp_path):
    sc = S.suspension(n_side=2, rings=3, T=0.3)
    s = system(sc)
    xyz = str(tmp_path / "traj.xyz")
    s.set_trajectory(xyz, 10, 1)
    s.run(20)
    s.flush_trajectory()
    lines = open(xyz).read().split("\n")
    n = s.N
    assert int(lines[0]) == n and lines[2].startswith("A\t") and int(lines[n + 2]) == n
    base = str(tmp_path / "frame")
    s.set_trajectory(base, 10, 2)
    s.run(20)
    s.flush_trajectory()
    files = sorted(f for f in os.listdir(tmp_path) if f.startswith("frame"))
    assert files == ["frame000000030.vtk", "frame000000040.vtk"]
    text = open(os.path.join(tmp_path, files[-1])).read()
    nt = s.counts()["triangles"]
    assert f"POINTS {n} FLOAT" in text and f"CELLS {nt} {4 * nt}" in text and "VECTORS Velocity FLOAT" in text


def test_frames_and_averaging_leave_area_spring_runs_unchanged(tmp_path):
    """With area springs (positions moved inside every force pass), a run
    with trajectory frames and one with property averaging end bit for bit
    where the plain run ends: the split step adds no second force pass."""
    base = S.suspension(n_side=3, rings=6, bonds="boundary", T=0.6, center_jitter=0.3, phi=0.5)
    calls = []
    for n, a in base.calls:
        calls.append((n, a))
        if n == "set_elastomer_bonds":
            calls.append(("set_kArea", (0.3,)))
    sc = S.Scene(calls=calls, meta=dict(base.meta))
    plain = system(sc)
    plain.run(0)
    plain.run(120)
    framed = system(sc)
    framed.run(0)
    framed.set_trajectory(str(tmp_path / "a.dump"), 25, 0)
    framed.run(120)
    assert framed.flush_trajectory() == 4
    averaged = system(sc)
    averaged.set_property_averaging(True, 40, 0)
    averaged.run(0)
    averaged.run(120)
    for other in (framed, averaged):
        for x, y in zip(other.get_state(), plain.get_state()):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    # evaluating the properties moves nothing either, and the run continues
    # as if it had not been called
    before = plain.positions().copy()
    plain.properties()
    assert np.array_equal(plain.positions().view(np.uint32), before.view(np.uint32))
    plain.run(30)
    averaged.run(30)
    assert np.array_equal(plain.positions().view(np.uint32), averaged.positions().view(np.uint32))
