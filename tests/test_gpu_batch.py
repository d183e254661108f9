"""Batched replicas (femmd_batch_*): one persistent launch advancing many
systems of uneven size.  Every replica must end bit-identical to the same
system run alone through System.run (positions, velocities, accelerations,
step and rebuild counters), whatever the launch shape, including when a
replica's neighbour list overflows and the batch rolls back and repeats."""
import numpy as np
import pytest

import golden_io as G
import femmd_old_gb300 as F
from femmd_old_gb300 import scene as S

pytestmark = pytest.mark.gpu


def replicas(n=7, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = [300, 700, 1800, 2600, 4100, 900, 1400][:n]
    return [S.mixed_replica(int(sz), float(rng.uniform(0.6, 0.85)), float(rng.uniform(0.1, 1.5)), seed=100 + k)
            for k, sz in enumerate(sizes)]


def alone(sc, steps_list):
    s = F.System(0)
    sc.replay(s)
    for n in steps_list:
        s.run(n)
    return s


def same(a, b):
    pa, va, aa = a.get_state()
    pb, vb, ab = b.get_state()
    return (np.array_equal(G.bits(pa), G.bits(pb)) and np.array_equal(G.bits(va), G.bits(vb))
            and np.array_equal(G.bits(aa), G.bits(ab)) and a.steps() == b.steps()
            and a.total_updates() == b.total_updates())


@pytest.mark.parametrize("launch", [(512, 2), (128, 4), (1024, 1)])
def test_batch_matches_replicas_run_alone(launch):
    scs = replicas()
    b = F.Batch(0)
    systems = []
    for sc in scs:
        s = F.System(0)
        sc.replay(s)
        systems.append(s)
        b.add(s)
    b.set_launch(*launch)
    b.run(60)
    b.run(0)
    b.run(41)
    for sc, s in zip(scs, systems):
        assert same(s, alone(sc, [60, 0, 41]))


def test_batch_autotune_keeps_results():
    scs = replicas(5, seed=1)
    b = F.Batch(0)
    systems = []
    for sc in scs:
        s = F.System(0)
        sc.replay(s)
        systems.append(s)
        b.add(s)
    cfg = b.autotune(5)
    assert cfg["threads"] in (128, 256, 512, 1024)
    b.run(50)
    for sc, s in zip(scs, systems):
        assert same(s, alone(sc, [50]))


def test_batch_overflow_rolls_back_and_repeats():
    scs = replicas(4, seed=2)
    b = F.Batch(0)
    systems = []
    for k, sc in enumerate(scs):
        s = F.System(0)
        sc.replay(s)
        if k == 2:
            s.set_neighbor_capacity(2)
        systems.append(s)
        b.add(s)
    b.run(40)
    assert systems[2].neighbor_capacity() > 2
    for sc, s in zip(scs, systems):
        assert same(s, alone(sc, [40]))


def test_batch_rejects_mixed_variants():
    a = F.System(0)
    S.mixed_replica(500, 0.7, 1.0, seed=7).replay(a)
    c = F.System(0)
    S.lj_fluid(n_side=16).replay(c)  # one type: a different kernel variant
    b = F.Batch(0)
    b.add(a)
    b.add(c)
    with pytest.raises(F.FemmdError):
        b.run(5)


def test_batch_walls_gravity_and_moving_walls():
    """XPBC replicas: the reference's harmonic walls under gravity and the
    moving compression wall, each bit-identical to running alone."""
    import golden_io as G
    base, _ = G.load("susp_xpbc_gravity")
    calls = []
    for name, args in base.calls:
        if name == "dump_setup":
            break
        calls.append((name, args))
    scs = []
    for g in (0.5, 2.0, 3.5):
        sc = S.Scene(calls=[(n, (g,) if n == "set_gravity" else a) for n, a in calls])
        scs.append(sc)
    scs.append(S.compression(n_side=3, steps=60))
    scs.append(S.compression(n_side=2, steps=60, seeds=(3, 14, 15, 11)))
    b = F.Batch(0)
    systems = []
    for sc in scs:
        s = F.System(0)
        sc.replay(s)
        systems.append(s)
        b.add(s)
    b.run(60)
    b.run(37)
    for sc, s in zip(scs, systems):
        assert same(s, alone(sc, [60, 37]))


def test_batch_autotune_lists_applies_the_choice():
    """Opt-in cadence/cell tuning: afterwards every replica runs exactly like
    the same system set up alone with the chosen skin and cell factor."""
    scs = replicas(4, seed=4)
    b = F.Batch(0)
    systems = []
    for sc in scs:
        s = F.System(0)
        sc.replay(s)
        systems.append(s)
        b.add(s)
    b.run(10)
    r = b.autotune_lists(15, skins=(0.3, 0.5), factors=(1.0, 1.25))
    assert r["skin"] in (0.3, 0.5) and r["cell_factor"] in (1.0, 1.25)
    b.run(40)
    for sc, s in zip(scs, systems):
        a = F.System(0)
        sc.replay(a)
        a.run(10)
        a.set_skin(r["skin"])
        a.set_cell_factor(r["cell_factor"])
        a.init_neighbor_list()
        a.run(40)
        assert same(s, a)


def test_tuned_lists_keep_the_trajectory():
    """The tuner's other skin and cell size change only the rounding: the
    lists still hold every pair inside the cutoff, so a replica run with skin
    0.5 and cells 1.25x larger (another list order, so other roundings of the
    force sums) stays within 1e-3 sigma of the default run after 30 steps
    (before the chaos of the dense disks amplifies the rounding) and its
    total energy within 1e-4 of |E|."""
    sc = replicas(1, seed=5)[0]
    runs = []
    for skin, factor in ((None, None), (0.5, 1.25)):
        s = F.System(0)
        sc.replay(s)
        if skin is not None:
            s.set_skin(skin)
            s.set_cell_factor(factor)
            s.init_neighbor_list()
        s.run(0)
        s.run(30)
        runs.append(s)
    a, t = runs
    box = a.get_box()
    L = np.array([box["x"], box["y"]])
    d = a.positions().astype(np.float64) - t.positions().astype(np.float64)
    d -= L * np.round(d / L)
    assert np.abs(d).max() <= 1e-3
    ea, et = a.energies(), t.energies()
    tot_a, tot_t = ea[0] + 0.5 * ea[2], et[0] + 0.5 * et[2]
    assert abs(tot_a - tot_t) <= 1e-4 * abs(tot_a)


@pytest.mark.parametrize("sizes,launch", [((8000, 600, 900, 1200, 700, 500), (1024, 1)),
                                          ((6000, 5000, 700, 800), (512, 2)),
                                          ((7000, 6500, 6000, 900, 400, 300), (256, 4))])
def test_large_replicas_on_cta_pairs_match_alone(sizes, launch):
    """Replicas heavier than a CTA's average share run on a pair of CTAs (a
    thread-block cluster of two, particles split between them): still bit
    for bit the replica run alone, split or not."""
    rng = np.random.Generator(np.random.PCG64(11))
    scs = [S.mixed_replica(int(sz), float(rng.uniform(0.6, 0.85)), float(rng.uniform(0.1, 1.5)), seed=300 + k)
           for k, sz in enumerate(sizes)]
    for split in (True, False):
        b = F.Batch(0)
        systems = []
        for sc in scs:
            s = F.System(0)
            sc.replay(s)
            systems.append(s)
            b.add(s)
        b.set_launch(*launch)
        b.set_split(split)
        b.run(60)
        b.run(0)
        b.run(41)
        for sc, s in zip(scs, systems):
            assert same(s, alone(sc, [60, 0, 41])), (split, s.N)


def test_batched_replicas_match_the_oracle_directly():
    """Three replicas of the ensemble's kind (LJ solvent plus hex-ring disks,
    uneven sizes), advanced together by the batched kernel through run(60)
    then run(41), against the oracle (the reference's CPU path restated, the
    same exact image mode and log) running each replica alone: positions,
    velocities, accelerations bit-identical, and the same rebuild count."""
    from oracle import Oracle
    scs = replicas(3, seed=2)
    b = F.Batch(0)
    systems = []
    for sc in scs:
        s = F.System(0)
        sc.replay(s)
        systems.append(s)
        b.add(s)
    b.run(60)
    b.run(41)
    for sc, s in zip(scs, systems):
        o = Oracle(image_mode=1, log_mode=1)
        sc.replay(o)
        o.run(60)
        o.run(41)
        for a, c in ((s.positions(), o.positions()), (s.velocities(), o.velocities()),
                     (s.accelerations(), o.accelerations())):
            assert np.array_equal(G.bits(a), G.bits(c))
        assert s.total_updates() == o.total_updates()
