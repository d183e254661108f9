"""GPU parity of the femmd2D timestep (libfemmd.so, sm_103a) against the
reference and the oracle.

Tolerances (stated here, used below):
  * cell sets, neighbour lists (in the reference's order), setup arrays:
    bit-exact against the reference's own output (golden fixtures);
  * LJ-only trajectories in reference image mode: bit-exact against the
    reference (positions, velocities, accelerations, forces, step and rebuild
    counters) over the fixture's 250 steps;
  * everything in either image mode, FEA included: bit-exact against the
    oracle run with the same image mode and the own-log (the only arithmetic
    difference from the reference is logf -> own log, within 2 ulp);
  * forces vs the FP64 restatement: |f_i - f64_i| <= 1e-5 * C_i per particle
    and ||f - f64|| <= 1e-5 * ||C|| over the system, where C_i is the
    condition scale of particle i's float force: the sum over its bond,
    triangle and pair contributions of the magnitudes of the operands of each
    float expression (oracle.forces_f64).  A result that cancels to ~0 (a
    rigidly moving triangle, a pair at the LJ force zero) is judged against
    the size of what cancelled, which is what float32 arithmetic can resolve;
  * U and W (FP64 reductions on the GPU) vs FP64: within 1e-5 of their
    condition scales.
"""
import numpy as np
import pytest

import golden_io as G
import femmd_old_gb300 as F
from femmd_old_gb300 import scene as S
from oracle import Oracle

pytestmark = pytest.mark.gpu

FEA_CASES = {"susp_all", "susp_boundary", "susp_refdisk", "susp_crossing", "susp_mixed", "susp_xpbc_gravity",
             "susp_area", "susp_area_xpbc"}
F_IMAGE_REFERENCE = 0
F_IMAGE_EXACT = 1
STATE_FIELDS = ("pos", "vel", "acc", "force")


def product(image_mode, **kw):
    s = F.System()
    s.set_image_mode(image_mode)
    for k, v in kw.items():
        getattr(s, k)(v)
    return s


def state_diffs(ref, got, fields=STATE_FIELDS, counters=True):
    bad = []
    rs = [d for t, d in ref if t == "state"]
    gs = [d for t, d in got if t == "state"]
    assert len(rs) == len(gs)
    for k, (a, b) in enumerate(zip(rs, gs)):
        for f in fields:
            if not np.array_equal(G.bits(a[f]), G.bits(b[f])):
                d = np.abs(a[f].astype(np.float64) - b[f].astype(np.float64))
                bad.append(f"state{k}.{f}: max|d|={d.max():.3e} n={int((d > 0).sum())}")
        if counters:
            for f in ("steps", "total_updates"):
                if int(a[f]) != int(b[f]):
                    bad.append(f"state{k}.{f}: {a[f]} vs {b[f]}")
    return bad


def nn_diffs(ref, got):
    bad = []
    rn = [d for t, d in ref if t == "nn"]
    gn = [d for t, d in got if t == "nn"]
    assert len(rn) == len(gn)
    for k, (a, b) in enumerate(zip(rn, gn)):
        if tuple(a["grid"]) != tuple(b["grid"]):
            bad.append(f"nn{k}.grid {a['grid']} vs {b['grid']}")
        for f in ("cell_start", "cell_ids", "nbr_start", "nbr_list"):
            if not np.array_equal(a[f], b[f]):
                bad.append(f"nn{k}.{f} differs")
    return bad


# ------------------------------------------------------------ golden parity

@pytest.mark.parametrize("name", G.names())
def test_reference_mode_matches_golden(name):
    sc, ref = G.load(name)
    s = product(F_IMAGE_REFERENCE)
    sc.replay(s)
    got = s.dumps
    # setup and neighbour structures: bit-exact against the reference itself
    assert not G.diff_report([d for d in ref if d[0] == "setup"], [d for d in got if d[0] == "setup"])
    assert not nn_diffs(ref, got)
    if name in FEA_CASES:
        # FEA uses the own log: bit-exact against the oracle with the own log ...
        o = Oracle(image_mode=0, log_mode=1)
        sc.replay(o)
        bad = state_diffs(o.dumps, got)
        assert not bad, bad
        # ... and at the first force dump (same positions) close to the reference
        a = [d for t, d in ref if t == "state"][0]["force"].astype(np.float64)
        b = [d for t, d in got if t == "state"][0]["force"].astype(np.float64)
        assert np.abs(a - b).max() <= 1e-5 * max(1.0, np.abs(a).max())
    else:
        bad = state_diffs(ref, got)
        assert not bad, bad


@pytest.mark.parametrize("name", G.names())
def test_exact_mode_matches_oracle(name):
    sc, _ = G.load(name)
    s = product(F_IMAGE_EXACT)
    sc.replay(s)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    assert not nn_diffs(o.dumps, s.dumps)
    bad = state_diffs(o.dumps, s.dumps)
    assert not bad, bad


@pytest.mark.parametrize("law,kmode", [(1, 1), (1, 0), (0, 1)])
def test_alternate_laws_match_oracle(law, kmode):
    """Green-strain / linear-C law of the reference GPU kernel and k = E/r0
    bonds (interactionsCuda.cu:238, 312-451): restated, checked against the
    oracle bit for bit (the reference's GPU path cannot run here)."""
    sc = S.suspension(n_side=3, rings=3, bonds="all", T=0.3, center_jitter=0.3)
    sc.add("build_nn").add("calc_forces").add("dump_state").add("run", 150).add("dump_state")
    s = product(F_IMAGE_EXACT, set_fea_law=law, set_bond_k_mode=kmode)
    sc.replay(s)
    o = Oracle(image_mode=1, log_mode=1, fea_law=law, bond_k_mode=kmode)
    sc.replay(o)
    bad = state_diffs(o.dumps, s.dumps)
    assert not bad, bad


def with_area(sc, k, pbc=None, gravity=None):
    """The scene with area springs of stiffness k (and optionally another box
    kind and gravity) set before the elastomers are added."""
    calls = []
    for n, a in sc.calls:
        if n == "PBC" and pbc is not None:
            a = (pbc,)
        calls.append((n, a))
        if n == "set_elastomer_bonds":
            calls.append(("set_kArea", (k,)))
            if gravity:
                calls.append(("set_gravity", (gravity,)))
    return S.Scene(calls=calls, meta=dict(sc.meta))


@pytest.mark.parametrize("pbc", [2, 1, 0])
def test_area_springs_match_oracle(pbc):
    """Area springs (calcAreaForcesCPU, interactions.cpp:696-750) in each box
    kind, on 127-vertex disks: the vertices move triangle after triangle
    inside every force pass, the walls and bonds see the positions from before
    that pass and the pairs those after it.  Bit-exact against the oracle's
    serial loop in both image modes."""
    base = S.suspension(n_side=3, rings=6, bonds="boundary", T=0.6, center_jitter=0.3, phi=0.5)
    sc = with_area(base, 0.3, pbc=pbc, gravity=0.5 if pbc == 1 else None)
    sc.add("build_nn").add("calc_forces").add("dump_state")
    sc.add("run", 120).add("dump_state").add("run", 80).add("dump_state")
    for mode in (F_IMAGE_EXACT, F_IMAGE_REFERENCE):
        s = product(mode)
        sc.replay(s)
        o = Oracle(image_mode=mode, log_mode=1)
        sc.replay(o)
        bad = state_diffs(o.dumps, s.dumps)
        assert not bad, (mode, bad)
    # the springs act: without them the run ends elsewhere
    s0 = product(F_IMAGE_EXACT)
    with_area(base, 0.0, pbc=pbc, gravity=0.5 if pbc == 1 else None).replay(s0)
    s0.run(200)
    assert np.abs(s0.positions() - s.positions()).max() > 1e-4


def test_area_springs_outside_the_batch_and_adjoint():
    """The batched kernel and the adjoint do not implement the area springs:
    both refuse such a system instead of ignoring them."""
    sc = with_area(S.suspension(n_side=2, rings=3, bonds="boundary", T=0.2), 0.3)
    s = F.System()
    sc.replay(s)
    b = F.Batch()
    b.add(s)
    with pytest.raises(F.FemmdError) as e:
        b.run(5)
    assert "UNSUPPORTED" in str(e.value)
    with pytest.raises(F.FemmdError) as e:
        s.adjoint_forward(10, 5)
    assert "UNSUPPORTED" in str(e.value)
    s.set_kArea(0.0)  # off again: the system runs in the batch
    b.run(5)
    # trajectory frames and property averaging are not done by the batched
    # kernel either: refused, not silently skipped
    s.set_property_averaging(True, 10, 0)
    with pytest.raises(F.FemmdError) as e:
        b.run(5)
    assert "UNSUPPORTED" in str(e.value)
    s.set_property_averaging(False)
    b.run(5)


# ------------------------------------------------------------- FP64 checks

def fp64_check(s, o, tol=1e-5):
    s.build_nn()
    s.calc_forces()
    f = s.forces().astype(np.float64)
    e = s.energies()
    o.set_positions_array(s.positions())
    o.build_nn()
    f64, cond, ui, tot = o.forces_f64()
    err = np.linalg.norm(f - f64, axis=1)
    worst = float((err / np.maximum(cond, 1e-30)).max())
    assert worst <= tol, worst
    assert np.linalg.norm(f - f64) <= tol * np.linalg.norm(cond)
    assert abs(e[0] - tot[0]) <= tol * tot[2], (e[0], tot[0], tot[2])
    assert abs(e[1] - tot[1]) <= tol * max(tot[3], 1e-30), (e[1], tot[1])
    return worst


@pytest.mark.parametrize("name", G.names())
def test_forces_within_1e5_of_fp64(name):
    sc, _ = G.load(name)
    s = product(F_IMAGE_EXACT)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(s, stop_at={"dump_setup"})
    sc.replay(o, stop_at={"dump_setup"})
    s.run(120)  # thermalised positions, lists from a rebuild in the run
    # the FP64 restatement evaluates forces at fixed positions; area springs,
    # which move the positions inside the force pass, are switched off for it
    # (their arithmetic is checked bit for bit against the oracle above)
    s.set_kArea(0.0)
    o.set_kArea(0.0)
    fp64_check(s, o)


def test_cfg1_lj_fluid_1000_steps_bitwise_and_fp64():
    """Benchmark config 1 (N=4096, rho=0.8, rc=2.5, skin 0.3, dt=0.005): 1000
    steps bit-exact against the oracle, forces within 1e-5 of FP64 after them,
    momentum conserved and energy drift small."""
    sc = S.lj_fluid()
    s = product(F_IMAGE_EXACT)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(s)
    sc.replay(o)
    s.run(1000)
    o.run(1000)
    for a, b in ((s.positions(), o.positions()), (s.velocities(), o.velocities()),
                 (s.accelerations(), o.accelerations())):
        assert np.array_equal(G.bits(a), G.bits(b))
    assert s.total_updates() == o.total_updates()
    obs = s.step_observables()
    assert obs.shape == (1000, 6)
    etot = obs[:, 0] + 0.5 * obs[:, 2]
    assert abs(etot[-1] - etot[0]) / abs(etot[0]) < 2e-3
    p = (s.velocities().astype(np.float64) * s.masses()[:, None]).sum(0)
    assert np.abs(p).max() < 1e-2
    fp64_check(s, o)


def test_cfg2_suspension_bitwise():
    """Benchmark config 2 at 8x8 disks (64 x 127 vertices): 400 steps
    bit-exact against the oracle (neo-Hookean FEA, boundary bonds, WCA)."""
    sc = S.suspension(n_side=8)
    s = product(F_IMAGE_EXACT)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(s)
    sc.replay(o)
    s.run(400)
    o.run(400)
    assert np.array_equal(G.bits(s.positions()), G.bits(o.positions()))
    assert np.array_equal(G.bits(s.velocities()), G.bits(o.velocities()))
    fp64_check(s, o)


# ---------------------------------------------------------- full-size checks

def test_cfg3_large_mixed_properties():
    """Benchmark config 3 at full size (4096 disks = 520,192 vertices plus
    1,000,000 solvent): the first neighbour list equals the oracle's as sets,
    forces within 1e-5 of FP64, momentum conserved over 100 steps and two runs
    from the same state bit-identical (deterministic reductions)."""
    sc = S.large_mixed()
    s = product(F_IMAGE_EXACT)
    sc.replay(s)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    s.build_nn()
    o.build_nn()
    st, lst = s.neighbors()
    ost, olst = o.neighbors()
    assert np.array_equal(st, ost) and np.array_equal(lst, olst)
    s.calc_forces()
    o.calc_forces()
    assert np.array_equal(G.bits(s.forces()), G.bits(o.forces()))
    fp64_check(s, o)
    p0, v0, _ = s.get_state()
    s.run(100)
    pa, va, _ = s.get_state()
    m = s.masses().astype(np.float64)[:, None]
    assert np.abs((va * m).sum(0) - (v0 * m).sum(0)).max() < 1e-2 * np.abs(v0 * m).sum()
    s.set_state(p0, v0)
    s.run(100)
    pb, vb, _ = s.get_state()
    assert np.array_equal(G.bits(pa), G.bits(pb)) and np.array_equal(G.bits(va), G.bits(vb))


# ------------------------------------------------------------- edge cases

def test_overflowing_capacity_is_grown_and_run_repeated():
    sc = S.lj_fluid(n_side=24)
    a = product(F_IMAGE_EXACT)
    sc.replay(a)
    a.run(300)
    b = product(F_IMAGE_EXACT)
    sc.replay(b)
    b.set_neighbor_capacity(3)
    b.run(300)
    assert b.neighbor_capacity() > 3
    assert np.array_equal(G.bits(a.positions()), G.bits(b.positions()))


@pytest.mark.parametrize("cap", [16, 17, 18, 19])
def test_list_groups_at_every_capacity_remainder(cap):
    """The lists are stored in groups of four entries: a capacity is rounded
    up to a multiple of 4, and lists ending anywhere inside a group (counts
    of every remainder, some beyond a small capacity) read back in the
    reference's order, with the same trajectory as the default capacity."""
    sc, ref = G.load("susp_mixed")
    s = product(F_IMAGE_REFERENCE)
    first = next(k for k, (n, _) in enumerate(sc.calls) if n == "dump_setup")
    for n, a in sc.calls[:first]:
        getattr(s, n)(*a)
    s.set_neighbor_capacity(cap)
    assert s.neighbor_capacity() % 4 == 0 and s.neighbor_capacity() >= cap
    for n, a in sc.calls[first:]:
        getattr(s, n)(*a)
    assert not nn_diffs(ref, s.dumps)
    start, nbr = s.neighbors()
    counts = np.diff(start)
    assert set(np.unique(counts % 4)) == {0, 1, 2, 3}
    o = Oracle(image_mode=0, log_mode=1)
    sc.replay(o)
    assert not state_diffs(o.dumps, s.dumps)


def test_graph_and_direct_launches_agree():
    sc = S.suspension(n_side=4, rings=4)
    a = product(F_IMAGE_EXACT)
    sc.replay(a)
    a.run(257)
    b = product(F_IMAGE_EXACT)
    sc.replay(b)
    b.set_profiling(True)
    b.run(257)
    assert b.profile()["force_launches"] == 258
    assert np.array_equal(G.bits(a.positions()), G.bits(b.positions()))
    assert np.array_equal(G.bits(a.velocities()), G.bits(b.velocities()))


def test_do_step_matches_oracle():
    sc = S.lj_fluid(n_side=20)
    s = product(F_IMAGE_REFERENCE)
    o = Oracle(image_mode=0, log_mode=1)
    sc.replay(s)
    sc.replay(o)
    s.run(10)
    o.run(10)
    for _ in range(30):
        s.do_step()
        o.do_step()
    assert np.array_equal(G.bits(s.positions()), G.bits(o.positions()))
    assert s.steps() == o.steps() == 40


def test_repeated_runs_follow_the_reference_run_semantics():
    # each run() starts with a forced rebuild and a fresh force pass
    sc = S.lj_fluid(n_side=20)
    s = product(F_IMAGE_REFERENCE)
    o = Oracle(image_mode=0, log_mode=1)
    sc.replay(s)
    sc.replay(o)
    for n in (1, 0, 7, 64, 33):
        s.run(n)
        o.run(n)
        assert np.array_equal(G.bits(s.positions()), G.bits(o.positions()))
        assert np.array_equal(G.bits(s.accelerations()), G.bits(o.accelerations()))
        assert s.total_updates() == o.total_updates()


def test_step_observables_and_energies():
    sc = S.lj_fluid(n_side=16)
    s = product(F_IMAGE_EXACT)
    sc.replay(s)
    s.run(50)
    obs = s.step_observables()
    e = s.energies()
    assert obs.shape == (50, 6)
    assert obs[-1, 0] == e[0] and obs[-1, 2] == e[2]
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    o.run(50)
    sc32 = o.scalars()
    assert abs(obs[-1, 3] - sc32[4]) == 0.0  # max v^2 is order-independent
    assert abs(obs[-1, 2] - sc32[3]) <= 1e-5 * abs(sc32[3])


def test_nonfinite_forces_are_reported():
    s = F.System()
    s.init(10, 10)
    s.set_pair_potential([1.0], [2.5], [0.0])
    s.add_particle(5, 5, 0, 0, 1, 1, 0)
    s.add_particle(5, 5, 0, 0, 1, 1, 0)  # coincident: r = 0
    s.init_neighbor_list()
    with pytest.raises(F.FemmdError) as e:
        s.run(2)
    assert "NONFINITE" in str(e.value)


def test_empty_system_runs():
    s = F.System()
    s.init(10, 10)
    s.init_neighbor_list()
    s.run(5)
    assert s.steps() == 5 and s.N == 0
