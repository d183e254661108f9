"""GPU checks of the fast force mode (femmd_set_force_mode(FEMMD_FORCE_FAST)).

The fast mode keeps the neighbour and cell SETS and the force accuracy of the
reference-exact mode, but sums with fused multiply-adds and the hardware
reciprocal and stores the free particles in cell order on the device.
Tolerances (stated here, used below):
  * cell sets: identical to the oracle's (the getter lists ids ascending in a
    cell, the reference's format), bit for bit;
  * neighbour sets: every particle's list equals the oracle's as a set, at the
    same positions (the order inside a row is the fast walk's own);
  * forces vs the FP64 restatement: |f_i - f64_i| <= 1e-5 * C_i per particle
    and ||f - f64|| <= 1e-5 * ||C|| (C_i the condition scale of particle i's
    float force, oracle.forces_f64), U and W within 1e-5 of their condition
    scales -- the same bar as the reference-exact mode;
  * trajectories: benchmark config 1 (N = 4096 LJ fluid) against the
    reference-exact run from the same start: positions within 1e-4 sigma
    after 50 steps and 1e-2 sigma after 200 steps (the LJ fluid is chaotic:
    float-rounding differences grow by e^(lambda t)), and over 1000 steps the
    total-energy drift of both runs below 2e-3 of |E| and within 1e-3 of |E|
    of each other, the mean potential energy within 1 % and momentum
    conserved;
  * runs are deterministic: two runs from one state are bit-identical.
"""
import numpy as np
import pytest

import golden_io as G
import femmd_old_gb300 as F
from femmd_old_gb300 import scene as S
from oracle import Oracle

from test_gpu_parity import fp64_check

pytestmark = pytest.mark.gpu

FAST = 1
EXACT_IMAGE = 1


def fast_system(**kw):
    s = F.System()
    s.set_force_mode(FAST)
    for k, v in kw.items():
        getattr(s, k)(v)
    return s


def min_image(d, L):
    return d - L * np.round(d / L)


def rows_as_sets_equal(st_a, la, st_b, lb):
    """Per-row equality of two CSR neighbour lists as sets (multiplicity kept)."""
    if not np.array_equal(st_a, st_b):
        return False
    rows = np.repeat(np.arange(len(st_a) - 1), np.diff(st_a))
    ka = np.lexsort((la, rows))
    kb = np.lexsort((lb, rows))
    return np.array_equal(la[ka], lb[kb])


def test_mode_is_selectable_and_reported():
    s = F.System()
    assert s.force_mode() == 0
    s.set_force_mode(FAST)
    assert s.force_mode() == FAST
    with pytest.raises(F.FemmdError):
        s.set_force_mode(7)


@pytest.mark.parametrize("name", G.names())
def test_fast_sets_and_forces_on_golden_scenes(name):
    """On every reference-run scene: after a fast run(120) the cell and
    neighbour sets equal the oracle's at the same positions and the forces
    are within 1e-5 of FP64."""
    sc, _ = G.load(name)
    s = fast_system()
    sc.replay(s, stop_at={"dump_setup"})
    o = Oracle(image_mode=EXACT_IMAGE, log_mode=1)
    sc.replay(o, stop_at={"dump_setup"})
    s.run(120)
    s.set_kArea(0.0)
    o.set_kArea(0.0)
    o.set_positions_array(s.positions())
    s.build_nn()
    o.build_nn()
    cs, ci = s.cells()
    ocs, oci = o.cells()
    assert np.array_equal(cs, ocs) and np.array_equal(ci, oci)
    st, lst = s.neighbors()
    ost, olst = o.neighbors()
    assert rows_as_sets_equal(st, lst, ost, olst)
    fp64_check(s, o)


def test_fast_config2_suspension_forces():
    """Benchmark config 2 at 8x8 disks: neo-Hookean FEA, boundary bonds and WCA
    between disks in fast mode, forces within 1e-5 of FP64 after 300 steps."""
    sc = S.suspension(n_side=8)
    s = fast_system()
    sc.replay(s)
    o = Oracle(image_mode=EXACT_IMAGE, log_mode=1)
    sc.replay(o)
    s.run(300)
    fp64_check(s, o)


def test_fast_config1_trajectory_against_reference_exact():
    """Config 1 (4096 LJ atoms): the fast run against the reference-exact run
    from the same start -- pointwise close while the chaos has not amplified
    the rounding differences, and the same energy drift and mean potential
    energy over 1000 steps."""
    sc = S.lj_fluid()
    L = sc.meta["L"]
    a = F.System()
    a.set_image_mode(EXACT_IMAGE)
    sc.replay(a)
    b = fast_system()
    sc.replay(b)
    for steps, tol in ((50, 1e-4), (150, 1e-2)):
        a.run(steps)
        b.run(steps)
        d = np.abs(min_image(a.positions().astype(np.float64) - b.positions().astype(np.float64), L)).max()
        assert d <= tol, (steps, d)
    a.run(800)
    b.run(800)
    ea, eb = a.step_observables(), b.step_observables()
    ta = ea[:, 0] + 0.5 * ea[:, 2]
    tb = eb[:, 0] + 0.5 * eb[:, 2]
    scale = abs(ta[0])
    assert abs(ta[-1] - ta[0]) / scale < 2e-3
    assert abs(tb[-1] - tb[0]) / scale < 2e-3
    assert abs((tb[-1] - tb[0]) - (ta[-1] - ta[0])) / scale < 1e-3
    assert abs(ea[:, 0].mean() - eb[:, 0].mean()) <= 1e-2 * abs(ea[:, 0].mean())
    p = (b.velocities().astype(np.float64) * b.masses()[:, None]).sum(0)
    assert np.abs(p).max() < 1e-2
    o = Oracle(image_mode=EXACT_IMAGE, log_mode=1)
    sc.replay(o)
    fp64_check(b, o)


def test_fast_runs_are_deterministic_and_state_round_trips():
    """Two fast runs from the same state are bit-identical, and set_state /
    get_state keep the particle ids although the device stores the free
    particles in cell order (the storage order after a rebuild depends on
    the positions and ids only, not on the order before)."""
    sc = S.large_mixed(n_side=6, n_solvent=20000)
    s = fast_system()
    sc.replay(s)
    s.run(0)
    p0, v0, _ = s.get_state()
    s.run(60)
    pa, va, aa = s.get_state()
    assert np.array_equal(G.bits(s.positions()), G.bits(pa))
    s.set_state(p0, v0)
    s.run(60)
    pb, vb, ab = s.get_state()
    assert np.array_equal(G.bits(pa), G.bits(pb)) and np.array_equal(G.bits(va), G.bits(vb))
    assert np.array_equal(G.bits(aa), G.bits(ab))
    t = fast_system()
    sc.replay(t)
    t.set_state(p0, v0)
    t.run(60)
    assert np.array_equal(G.bits(pa), G.bits(t.positions()))
    assert np.array_equal(s.masses(), t.masses())


def test_fast_overflow_rollback_and_do_step():
    """A list capacity too small is grown and the run repeated from its start
    (storage order included): the same result as the default capacity.
    do_step continues a fast run like the fused steps do."""
    sc = S.lj_fluid(n_side=24)
    a = fast_system()
    sc.replay(a)
    a.run(300)
    b = fast_system()
    sc.replay(b)
    b.set_neighbor_capacity(3)
    b.run(300)
    assert b.neighbor_capacity() > 3
    assert np.array_equal(G.bits(a.positions()), G.bits(b.positions()))
    for _ in range(5):
        a.do_step()
    assert a.steps() == 305
    o = Oracle(image_mode=EXACT_IMAGE, log_mode=1)
    sc.replay(o)
    fp64_check(a, o)


def test_fast_mode_switches_both_ways():
    """Switching modes keeps the state: reference-exact -> fast -> reference-exact."""
    sc = S.lj_fluid(n_side=20)
    s = F.System()
    s.set_image_mode(EXACT_IMAGE)
    sc.replay(s)
    s.run(40)
    p1 = s.positions()
    s.set_force_mode(FAST)
    assert np.array_equal(G.bits(s.positions()), G.bits(p1))
    s.run(40)
    p2 = s.positions()
    s.set_force_mode(0)
    assert np.array_equal(G.bits(s.positions()), G.bits(p2))
    s.run(40)
    assert s.steps() == 120


def test_fast_trajectory_frames_keep_ids(tmp_path):
    """Frames written during a fast run list the particles by id: the last
    frame of run(20) (every 10 steps) holds the final positions."""
    sc = S.lj_fluid(n_side=12)
    s = fast_system()
    sc.replay(s)
    path = str(tmp_path / "f.xyz")
    s.set_trajectory(path, 10, 1)
    s.run(20)
    s.flush_trajectory()
    n = s.N
    body = [ln for ln in open(path).read().splitlines() if ln.startswith("A\t")]
    assert len(body) == 2 * n
    xy = np.array([[float(v) for v in ln.split()[1:3]] for ln in body[-n:]])
    assert np.allclose(xy, s.positions().astype(np.float64), atol=1e-4)


def test_fast_mode_outside_batch_and_adjoint():
    sc = S.suspension(n_side=2, rings=3, bonds="boundary", T=0.2)
    s = fast_system()
    sc.replay(s)
    b = F.Batch()
    b.add(s)
    with pytest.raises(F.FemmdError) as e:
        b.run(5)
    assert "UNSUPPORTED" in str(e.value)
    with pytest.raises(F.FemmdError) as e:
        s.adjoint_forward(10, 5)
    assert "UNSUPPORTED" in str(e.value)


def test_fast_lj_1m_full_size_sets_and_forces():
    """The 1M-atom LJ fluid of the benchmark (1000 x 1000 lattice, rho 0.8,
    rc 2.5, skin 0.3): after a fast run(20) the neighbour sets equal the
    oracle's, the forces are within 1e-5 of FP64 and momentum is conserved."""
    sc = S.lj_fluid(n_side=1000)
    s = fast_system()
    sc.replay(s)
    p0 = (s.velocities().astype(np.float64)).sum(0)
    s.run(20)
    o = Oracle(image_mode=EXACT_IMAGE, log_mode=1)
    sc.replay(o)
    o.set_positions_array(s.positions())
    s.build_nn()
    o.build_nn()
    st, lst = s.neighbors()
    ost, olst = o.neighbors()
    assert rows_as_sets_equal(st, lst, ost, olst)
    fp64_check(s, o)
    p1 = (s.velocities().astype(np.float64)).sum(0)
    assert np.abs(p1 - p0).max() < 1e-2


def lj_fluid_sigma(n_side, sigma, density):
    """The LJ fluid scene with every particle's sigma set to 'sigma' (one
    kind: sigma by type, not 1, so the pair loops scale 1/r^2 by sigma^2)."""
    sc = S.lj_fluid(n_side=n_side, density=density)
    sc.calls = [(n, a[:5] + (np.full_like(a[5], sigma),) + a[6:]) if n == "add_particles" else (n, a)
                for n, a in sc.calls]
    return sc


@pytest.mark.parametrize("n_side", [64, 120, 10, "sigma"])
def test_small_system_run_matches_the_step_kernels(n_side):
    """Small fast-mode systems advance a run's steps and rebuilds in one
    cooperative launch (k_fsmall): config 1 (64^2 = 4096 LJ atoms), 120^2 =
    14,400 atoms (113 step blocks, near the 128 the run takes), and 10^2 atoms
    in a box of 3 x 3 cells, where no step block has a window and every
    rebuild is handed back to the rebuild kernels.  The same run with every
    kernel launched on its own (profiling mode: k_fstep_p and the rebuild
    kernels) gives bit-identical positions, velocities and accelerations and
    the same rebuilds; the per-step energies agree within 1e-9 of |U| (exact
    fixed-point sums of per-block float partial sums that differ).  "sigma":
    48^2 atoms of sigma 1.2 at the same packing (the kernels' sigma != 1
    form)."""
    sc = lj_fluid_sigma(48, 1.2, 0.8 / 1.44) if n_side == "sigma" else S.lj_fluid(n_side=n_side)
    a = fast_system()
    sc.replay(a)
    a.run(0)
    a.run(300)
    b = fast_system()
    sc.replay(b)
    b.set_profiling(True)
    b.run(0)
    b.run(300)
    for x, y in ((a.positions(), b.positions()), (a.velocities(), b.velocities()),
                 (a.accelerations(), b.accelerations())):
        assert np.array_equal(G.bits(x), G.bits(y))
    assert a.total_updates() == b.total_updates() and a.steps() == b.steps() == 300
    oa, ob = a.step_observables(), b.step_observables()
    assert oa.shape == ob.shape == (300, 6)
    assert np.array_equal(oa[:, 3:], ob[:, 3:])  # max v^2, dispHi, rebuilt: exact
    assert np.abs(oa[:, :3] - ob[:, :3]).max() <= 1e-9 * np.abs(oa[:, 0]).max()


def test_small_run_exchange_timeout_is_reported_and_recovered():
    """A grid-wide exchange of the small-system run that never completes (block
    0 withholds its first record: femmd_test_expire_next_exchange) gives up
    after its bounded wait; run() returns FEMMD_TIMEOUT, and the context stays
    usable: the same run from the same state then matches a fresh system bit
    for bit."""
    sc = S.lj_fluid(n_side=24)
    s = fast_system()
    sc.replay(s)
    s.run(0)
    p0, v0, _ = s.get_state()
    s.test_expire_next_exchange()
    with pytest.raises(F.FemmdError) as err:
        s.run(50)
    assert err.value.status == 5  # FEMMD_TIMEOUT
    s.set_state(p0, v0)
    s.run(50)
    t = fast_system()
    sc.replay(t)
    t.run(0)
    t.set_state(p0, v0)
    t.run(50)
    assert np.array_equal(G.bits(s.positions()), G.bits(t.positions()))
    assert np.array_equal(G.bits(s.velocities()), G.bits(t.velocities()))
