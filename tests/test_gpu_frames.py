"""The reference's file writers (md3dsystem.cpp:232-522) through
femmd_save_frame and femmd_set_trajectory, byte for byte against the files
the reference itself wrote for the same scenes (tests/golden/frames, made by
tests/golden/make_golden.py): xyz, VTF, cluster VTF, legacy VTK, VTK XML
ascii and VTK XML with raw appended arrays, at the start and after runs,
with disks across the periodic boundary (unfolded), type letters, radii, the
bond list and the set_scale radius.  The scenes run with the FEA forces off,
so the states are bit-exact with the reference's (checked first); the files
must then be identical."""
import os

import numpy as np
import pytest

import golden_io as G
import femmd_old_gb300 as F

pytestmark = pytest.mark.gpu


class InDir:
    """A System whose frames go to one folder (the scene names files only)."""

    def __init__(self, s, folder):
        self._s, self._dir = s, folder

    def __getattr__(self, name):
        return getattr(self._s, name)

    def save_frame(self, name, fmt, append):
        self._s.save_frame(os.path.join(self._dir, name), fmt, append)


def replay(sc, folder):
    s = F.System()
    s.set_image_mode(0)  # the reference's float image arithmetic
    sc.replay(InDir(s, folder))
    return s


@pytest.mark.parametrize("name", G.frame_names())
def test_saved_frames_match_reference_files(name, tmp_path):
    sc, ref, files = G.load_frames(name)
    s = replay(sc, str(tmp_path))
    rs = [d for t, d in ref if t == "state"]
    gs = [d for t, d in s.dumps if t == "state"]
    assert len(rs) == len(gs)
    for a, b in zip(rs, gs):
        for f in ("pos", "vel"):
            assert np.array_equal(G.bits(a[f]), G.bits(b[f])), f
    got = sorted(os.listdir(tmp_path))
    assert got == sorted(files)
    for fname, want in files.items():
        have = (tmp_path / fname).read_bytes()
        if have != want:
            k = next(i for i in range(min(len(have), len(want)) + 1) if have[i:i + 1] != want[i:i + 1])
            pytest.fail(f"{fname}: first difference at byte {k}: {have[max(0, k - 40):k + 40]!r} "
                        f"vs {want[max(0, k - 40):k + 40]!r}")


def test_trajectory_frames_match_reference_files(tmp_path):
    """The same layouts written by the trajectory thread during runs: frames
    at steps 40 and 100 of the disks scene equal the reference's saves there."""
    sc, _, files = G.load_frames("elastomers")
    calls = [c for c in sc.calls if c[0] not in ("save_frame", "run", "dump_state")]
    runs = [c[1][0] for c in sc.calls if c[0] == "run"]
    assert runs == [40, 60]
    for fmt, fname in ((F.System.FRAME_VTF, "f.vtf"), (F.System.FRAME_CLUSTER_VTF, "c.vtf"),
                       (F.System.FRAME_XYZ, "f.xyz")):
        s = F.System()
        s.set_image_mode(0)
        for n, a in calls:
            getattr(s, n)(*a)
        path = str(tmp_path / f"traj_{fname}")
        s.set_trajectory(path, 20, fmt)
        s.run(40)
        s.run(60)
        assert s.flush_trajectory() == 5
        # reference frames: steps 0, 40, 100; trajectory frames: 20, 40, 60, 80, 100
        want = files[fname].decode()
        have = open(path).read()
        ref_blocks = _frames(want, fmt)
        got_blocks = _frames(have, fmt)
        assert len(ref_blocks) == 3 and len(got_blocks) == 5
        assert got_blocks[1] == ref_blocks[1] and got_blocks[4] == ref_blocks[2]
        if fmt != F.System.FRAME_XYZ:
            # the structure block comes with the first frame
            assert have.split("timestep\n")[0] == want.split("timestep\n")[0]


def _frames(text, fmt):
    if fmt == F.System.FRAME_XYZ:
        lines = text.split("\n")
        out, k = [], 0
        while k < len(lines) and lines[k]:
            n = int(lines[k])
            out.append("\n".join(lines[k:k + 2 + n]))
            k += 2 + n
        return out
    return text.split("timestep\n")[1:]


def test_writer_arguments_are_checked(tmp_path):
    """Layouts outside 0..6 and files that cannot be opened come back as
    errors with a message, from the one-shot save and from the trajectory."""
    sc, _, _ = G.load_frames("mixed")
    s = F.System()
    for n, a in sc.calls:
        if n not in ("save_frame", "run", "dump_state"):
            getattr(s, n)(*a)
    for bad in (-1, 7):
        with pytest.raises(F.FemmdError):
            s.save_frame(str(tmp_path / "x"), bad)
        with pytest.raises(F.FemmdError):
            s.set_trajectory(str(tmp_path / "t"), 10, bad)
    with pytest.raises(F.FemmdError, match="cannot open"):
        s.save_frame(str(tmp_path / "no_such_dir" / "f.vtf"), F.System.FRAME_VTF)
    with pytest.raises(F.FemmdError, match="cannot"):
        s.set_trajectory(str(tmp_path / "no_such_dir" / "t.xyz"), 10, F.System.FRAME_XYZ)
    # a per-frame layout into a missing folder fails at the frame, reported by the flush
    s.set_trajectory(str(tmp_path / "no_such_dir" / "v"), 5, F.System.FRAME_VTU)
    s.run(10)
    with pytest.raises(F.FemmdError, match="cannot open"):
        s.flush_trajectory()
    s.set_trajectory(None, 0)
    # append = 0 starts a file anew; append = 1 adds a frame after it
    p = tmp_path / "two.vtf"
    s.save_frame(str(p), F.System.FRAME_VTF, 0)
    one = p.read_text()
    s.save_frame(str(p), F.System.FRAME_VTF, 1)
    two = p.read_text()
    assert two.startswith(one) and two.count("timestep\n") == 2 and one.count("timestep\n") == 1
    s.save_frame(str(p), F.System.FRAME_VTF, 0)
    assert p.read_text() == one
