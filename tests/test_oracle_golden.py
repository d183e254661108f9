"""The oracle (oracle/femmd_oracle.c) against golden vectors produced by the
reference itself (tests/golden/make_golden.py).  In reference mode (float
minimum image, C library logf) every dumped array must match bit for bit:
setup arrays (masses, bonds, triangle inverses), cell and neighbour lists in
the reference's order, forces, energies and trajectory snapshots."""
import numpy as np
import pytest

import golden_io as G
from oracle import Oracle


@pytest.mark.parametrize("name", G.names())
def test_oracle_matches_reference_bitwise(name):
    sc, ref = G.load(name)
    o = Oracle(image_mode=0, log_mode=0)
    sc.replay(o)
    bad = G.diff_report(ref, o.dumps)
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("name", G.frame_names())
def test_oracle_matches_reference_on_writer_scenes(name):
    """The scenes of the writer fixtures (FEA off, edge bonds) step bit for
    bit as the reference's, so their frames can be compared byte for byte."""
    sc, ref, _ = G.load_frames(name)
    o = Oracle(image_mode=0, log_mode=0)
    sc.replay(o)
    bad = G.diff_report(ref, o.dumps)
    assert not bad, "\n".join(bad)


def test_writer_fixtures_hold_every_layout():
    """Scene streams with frame saves round-trip, and the reference's raw VTK
    XML frames have the appended arrays their offsets announce."""
    assert set(G.frame_names()) == {"elastomers", "mixed"}
    sc, _, files = G.load_frames("elastomers")
    assert sc.to_bytes() == type(sc).from_bytes(sc.to_bytes()).to_bytes()
    assert ("set_scale", (0.8,)) in sc.calls
    exts = {n.split(".")[-1] for n in files}
    assert exts == {"xyz", "vtf", "vtk", "vtu"}
    for n, b in files.items():
        if not n.startswith("b"):
            continue
        head, raw = b.split(b"\t_", 1)
        txt = head.decode()
        npts = int(txt.split('NumberOfPoints="')[1].split('"')[0])
        ncell = int(txt.split('NumberOfCells="')[1].split('"')[0])
        offs = [int(x.split('"')[0]) for x in txt.split('offset="')[1:]]
        sizes = [4 * npts, 12 * npts, 12 * ncell, 4 * ncell, ncell]
        assert offs == list(np.cumsum([0] + [s + 4 for s in sizes[:-1]]))
        for o, size in zip(offs, sizes):
            assert int.from_bytes(raw[o:o + 4], "little") == size
        assert raw[offs[-1] + 4:offs[-1] + 4 + ncell] == bytes([5]) * ncell
        assert raw[offs[-1] + 4 + ncell:] == b"\n\t</AppendedData>\n</VTKFile>"


def test_golden_cases_cover_edge_cases():
    names = set(G.names())
    for required in ("lj_xy", "lj_multitype", "lj_xpbc", "lj_nopbc", "tiny_box", "susp_all", "susp_boundary",
                     "susp_refdisk", "susp_crossing", "susp_mixed", "lj_nopbc_walls", "susp_xpbc_gravity",
                     "susp_area", "susp_area_xpbc"):
        assert required in names


def test_tiny_box_has_duplicate_neighbours():
    # two cells per axis: the reference's wrapped 3x3 stencil counts some pairs twice
    sc, ref = G.load("tiny_box")
    nn = [d for t, d in ref if t == "nn"][0]
    st, lst = nn["nbr_start"], nn["nbr_list"]
    dup = any(len(set(lst[st[i]:st[i + 1]])) < st[i + 1] - st[i] for i in range(len(st) - 1))
    assert dup


def test_crossing_case_crosses_the_boundary():
    sc, ref = G.load("susp_crossing")
    states = [d for t, d in ref if t == "state"]
    x0, x1 = states[0]["pos"], states[-1]["pos"]
    # some vertices wrapped from near L to near 0 in x (or y)
    assert ((x0[:, 0] > 15) & (x1[:, 0] < 5)).any() or ((x0[:, 1] > 15) & (x1[:, 1] < 5)).any()


def test_area_case_exercises_the_area_springs():
    # the same scene without area springs ends elsewhere, and a disk crosses
    # the periodic boundary during the runs
    import femmd_old_gb300.scene as S
    sc, ref = G.load("susp_area")
    off = S.Scene(calls=[(n, (0.0,) if n == "set_kArea" else a) for n, a in sc.calls], meta=sc.meta)
    o = Oracle(image_mode=0, log_mode=0)
    off.replay(o)
    states = [d for t, d in ref if t == "state"]
    assert np.abs(o.positions() - states[-1]["pos"]).max() > 1e-3
    x0, x1 = states[0]["pos"], states[-1]["pos"]
    assert ((x0[:, 0] > 18) & (x1[:, 0] < 5)).any() or ((x0[:, 1] > 18) & (x1[:, 1] < 5)).any()


def test_own_log_accuracy():
    from oracle import logf_own
    xs = np.concatenate([np.linspace(0.2, 5.0, 20001), np.geomspace(1e-30, 1e30, 2001),
                         1.0 + np.linspace(-1e-3, 1e-3, 2001)]).astype(np.float32)
    got = np.array([logf_own(float(x)) for x in xs], np.float64)
    ref = np.log(xs.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    err = np.abs(got - ref) / np.maximum(ulp, np.finfo(np.float32).tiny)
    assert err.max() <= 2.0, err.max()


# ------------------------------------------- the Green-strain / linear-C law

def _green_dumps():
    sc, ref = G.load("green/susp_cpu1")
    return sc, ref, [d for t, d in ref if t == "state"]


def test_green_law_cpu1_matches_reference_bitwise():
    """The reference's own CPU Green-strain / linear-C law
    (Interactions::calcFeaForcesCPU1, interactions.cpp:411-530), called alone
    after zeroStuff at positions the reference's run deformed: the oracle's
    restatement of it (its double-precision force sums included) reproduces
    every dumped array bit for bit -- positions, forces and the FEA energy."""
    sc, ref, _ = _green_dumps()
    assert sum(n == "fea_cpu1" for n, _ in sc.calls) == 2
    o = Oracle(image_mode=0, log_mode=0)
    sc.replay(o)
    bad = G.diff_report(ref, o.dumps)
    assert not bad, "\n".join(bad)


def test_green_law_float_restatement_within_rounding_of_cpu1():
    """The float restatement of the same law (the reference's GPU kernel
    computeFeaForcesGPU, interactionsCuda.cu:312-451, which the product's
    tri_green follows bit for bit) against the reference's CPU twin at the
    same positions: every nodal force within 1e-6 of the largest FEA force
    (the CPU twin sums the nodal force terms in double, the kernel in float;
    measured 1.9e-7), the energy within 1e-6 relative (measured equal).  The
    disks are apart (no pair inside the WCA cutoff, so the full force pass
    is the FEA pass) and some straddle the periodic edges."""
    sc, ref, states = _green_dumps()
    o = Oracle(image_mode=0, log_mode=0, fea_law=1)
    first = next(k for k, (n, _) in enumerate(sc.calls) if n == "run")
    for n, a in sc.calls[:first]:
        if n.startswith("dump"):
            continue
        getattr(o, n)(*a)
    crossed = False
    for k in (0, 2):
        pos, cpu1 = states[k]["pos"], states[k + 1]
        o.set_positions_array(pos)
        o.fea_only()
        f = o.forces().astype(np.float64)
        g = cpu1["force"].astype(np.float64)
        scale = np.abs(g).max()
        assert scale > 1.0
        assert np.abs(f - g).max() <= 1e-6 * scale, np.abs(f - g).max() / scale
        u, uref = float(o.scalars()[0]), float(cpu1["scalars"][0])
        assert abs(u - uref) <= 1e-6 * abs(uref)
        o.build_nn()
        o.calc_forces()
        assert np.array_equal(G.bits(o.forces()), G.bits(f.astype(np.float32)))
        crossed = crossed or (np.abs(np.diff(pos[:37, 0])).max() > 15.0)
    assert crossed  # the first disk straddles x = 0
