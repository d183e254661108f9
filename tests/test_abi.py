"""C ABI of libfemmd.so without a GPU: the library loads, exports every entry
point include/femmd.h declares, and its host-side setup (the reference's
System.* calls) produces the reference's setup arrays bit for bit."""
import os
import re

import numpy as np
import pytest

import golden_io as G
import femmd_old_gb300 as F
from femmd_old_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COMPUTE_CALLS = {"build_nn", "calc_forces", "run", "dump_nn", "dump_state", "do_step"}


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "femmd.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(femmd_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers them all
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_version_and_errors_without_gpu():
    s = F.System()
    assert b"sm_103a" in s._L.femmd_version()
    with pytest.raises(F.FemmdError) as e:
        s.add_particle(1, 1, 0, 0, 1, 1, 0)  # before init
    assert "NOT_READY" in str(e.value)
    s.init(10, 10)
    with pytest.raises(F.FemmdError):
        s.set_numTypes(0)
    with pytest.raises(F.FemmdError):
        s.create_bond(0, 1)  # no particles
    with pytest.raises(F.FemmdError):
        s.run(5)  # no init_neighbor_list
    s.set_gravity(1.0)  # calcGravityForces is on the path
    s.set_gravity(0.0)
    s.set_kArea(1.0)  # calcAreaForcesCPU is on the path
    s.set_kArea(0.0)


def test_elastomer_constraints_and_bad_meshes():
    s = F.System()
    s.init(40, 40)
    v = np.array([[0, 0], [1, 0], [0, 1]], np.float32)
    s.add_particle(20, 20, 0, 0, 1, 1, 0)
    with pytest.raises(F.FemmdError):  # elastomers must come first
        s.add_elastomer(v, np.array([[1, 2, 3]]), 5, 5, 0, 0, 1, 1, True)
    s2 = F.System()
    s2.init(40, 40)
    with pytest.raises(F.FemmdError):  # 1-based indices
        s2.add_elastomer(v, np.array([[0, 1, 2]]), 5, 5, 0, 0, 1, 1, True)
    s2.add_elastomer(v, np.array([[1, 2, 3]]), 5, 5, 0, 0, 1, 1, True)
    with pytest.raises(F.FemmdError):  # same mesh for every elastomer
        s2.add_elastomer(np.vstack([v, [[1, 1]]]), np.array([[1, 2, 3], [2, 4, 3]]), 9, 9, 0, 0, 1, 1, True)


@pytest.mark.parametrize("name", G.names())
def test_host_setup_matches_reference_bitwise(name):
    sc, ref = G.load(name)
    s = F.System()
    sc.replay(s, stop_at=COMPUTE_CALLS)
    setup = [d for t, d in ref if t == "setup"][0]
    got = s.setup_arrays()
    bad = [k for k in setup if not np.array_equal(G.bits(setup[k]), G.bits(got[k]))]
    assert not bad, bad


def test_info_matches_reference_fields():
    sc, ref = G.load("susp_all")
    s = F.System()
    sc.replay(s, stop_at=COMPUTE_CALLS)
    info = s.info()
    setup = [d for t, d in ref if t == "setup"][0]
    assert info["N"] == setup["mass"].size
    assert info["nbonds"] == 2 * setup["bonds"].shape[0]  # bondList.size(), interface.cpp:575
    assert info["ntrigs"] == setup["tris"].shape[0]
    assert info["nelastomers"] == 9


def test_argument_limits_without_gpu():
    """Host-side checks at the limits, before any GPU work: type count in
    [1, 32] (five tag bits in the list entries), averaging windows, cell
    factor in [1, 8], a negative skin."""
    s = F.System()
    s.init(10, 10)
    s.set_numTypes(32)
    with pytest.raises(F.FemmdError) as e:
        s.set_numTypes(33)
    assert "INVALID_ARG" in str(e.value)
    s.set_numTypes(1)
    with pytest.raises(F.FemmdError):
        s.set_property_averaging(True, 0, 10)
    with pytest.raises(F.FemmdError):
        s.set_property_averaging(True, 10, -1)
    s.set_property_averaging(False)  # off needs no window
    for bad in (0.5, 9.0):
        with pytest.raises(F.FemmdError):
            s.set_cell_factor(bad)
    s.set_cell_factor(2.0)
    with pytest.raises(F.FemmdError):
        s.set_skin(-0.1)
