"""Observables of Properties::evaluate (femmd_get_properties) against the
oracle's FP64 restatement on the same float state: uKinetic, uPotential,
uTotal, temperature, virial, feaVirial, pressure, clusterUKinetic,
clusterVirial, molPressure.  Tolerance: relative 1e-4, with absolute floors
of 1e-5 times the condition scale (sum of term magnitudes, from the oracle)
for the virials and pressures -- the GPU's forces are float, the oracle's
double, and a virial can cancel to a tiny fraction of its terms -- and 1e-6
times (|uKinetic| + |uPotential| + 1) for the energies."""
import numpy as np
import pytest

import golden_io as G
import femmd_old_gb300 as F
from femmd_old_gb300 import scene as S
from oracle import Oracle

pytestmark = pytest.mark.gpu


def compare(sc, steps):
    s = F.System(0)
    sc.replay(s)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    s.run(0)
    s.run(steps)
    o.run(0)
    o.run(steps)
    o.build_nn()
    g = s.properties()
    r = o.properties(scales=True)
    V = r.pop("V", None)
    sc_v, sc_f, sc_c = r.pop("virialScale"), r.pop("feaVirialScale"), r.pop("clusterVirialScale")
    area = sc.calls[0][1][0] * sc.calls[0][1][1]  # init(Lx, Ly)
    escale = abs(r["uKinetic"]) + abs(r["uPotential"]) + 1.0
    floors = {"virial": sc_v, "feaVirial": sc_f, "clusterVirial": sc_c,
              "pressure": 0.5 * (sc_v + sc_f) / area, "molPressure": 0.5 * sc_c / area}
    for k in r:
        floor = 1e-5 * floors[k] if k in floors else 1e-6 * escale
        assert abs(g[k] - r[k]) <= max(1e-4 * abs(r[k]), floor), (k, g[k], r[k], floor)
    return g, r


def test_properties_dense_suspension():
    # disks in contact: LJ virial and cluster virial act
    sc = S.suspension(n_side=4, phi=0.62, center_jitter=0.3, T=0.3)
    g, r = compare(sc, 150)
    assert r["virial"] != 0 and r["clusterVirial"] != 0 and r["feaVirial"] != 0


def test_properties_disks_across_the_boundary():
    # the golden crossing scene: disks moving across the periodic edges, so
    # clusters are unfolded (a disk created across an edge gets rest lengths
    # of about L from the reference's bond setup and blows up, in the
    # reference and here alike)
    sc, _ = G.load("susp_crossing")
    calls = []
    for name, args in sc.calls:
        if name == "dump_setup":
            break
        calls.append((name, args))
    sc.calls = calls
    compare(sc, 300)


def test_properties_mixed_solvent():
    # free particles are left out of the cluster virial on both sides
    compare(S.mixed_replica(3000, 0.75, 1.0, seed=3), 60)


# ------------------------------------------------------------- averaging
#
# femmd_set_property_averaging (Properties::compute after every step) against
# the per-step values of femmd_get_properties fed through the oracle's
# restatement of the reference's window logic (oracle.PropertyAverages).
# The device sums m v^2 as float block sums in fixed point, the per-step
# evaluation in FP64, so the kinetic terms differ by ~1e-7 relative: averages
# within 1e-6 of the largest per-step magnitude of that property, variances
# within 1e-5 of its square; counters exact.

def _per_step_reference(sc, segments, step_avg, step_equi):
    """The per-step values of a system stepped with do_step, each segment
    started by run(0) as a run() call starts (forced rebuild, forces)."""
    from oracle import PropertyAverages
    b = F.System(0)
    sc.replay(b)
    b.run(0)
    acc = PropertyAverages(F.System.PROPERTY_NAMES, step_avg, step_equi)
    mags = dict.fromkeys(F.System.PROPERTY_NAMES, 0.0)
    n = 0
    for seg in segments:
        b.run(0)
        for _ in range(seg):
            b.do_step()
            n += 1
            v = b.properties()
            for k in mags:
                mags[k] = max(mags[k], abs(v[k]))
            acc.compute(n, v)
    return acc, mags, b


def _check(got, acc, mags):
    assert got["windows"] == acc.windows and got["last_step"] == acc.last_step and got["count"] == acc.count
    for k in acc.names:
        m = mags[k] + 1e-300
        assert abs(got["avg"][k] - acc.avg[k]) <= 1e-6 * m, (k, got["avg"][k], acc.avg[k])
        assert abs(got["stdv"][k] ** 2 - acc.stdv[k] ** 2) <= 1e-5 * m * m, (k, got["stdv"][k], acc.stdv[k])


def test_property_averages_match_per_step_evaluation():
    sc = S.suspension(n_side=3, phi=0.62, center_jitter=0.3, T=0.3)
    acc, mags, b = _per_step_reference(sc, (57, 43), 20, 30)
    a = F.System(0)
    sc.replay(a)
    a.set_property_averaging(True, 20, 30)
    a.run(0)
    a.run(57)   # windows close at steps 40 and 60 (past 30, multiples of 20),
    a.run(43)   # 80 and 100, across run() calls as in the reference
    got = a.average_properties()
    assert acc.windows == 4 and acc.last_step == 100
    _check(got, acc, mags)
    for k in ("virial", "feaVirial", "clusterVirial", "pressure"):
        assert acc.stdv[k] > 0 and got["stdv"][k] > 0
    # averaging splits each step (LAST, properties, drift) with the fused
    # step's arithmetic: the trajectory is unchanged bit for bit
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    plain = F.System(0)
    sc.replay(plain)
    plain.run(0)
    plain.run(57)
    plain.run(43)
    for x, y in zip(a.get_state(), plain.get_state()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_property_averaging_survives_a_repeated_run():
    # a run repeated after a list overflow restores the sums from its start
    sc = S.lj_fluid(n_side=24)
    acc, mags, _ = _per_step_reference(sc, (60,), 10, 0)
    a = F.System(0)
    sc.replay(a)
    a.set_property_averaging(True, 10, 0)
    a.run(0)
    a.set_neighbor_capacity(2)
    a.run(60)
    assert a.neighbor_capacity() > 2
    _check(a.average_properties(), acc, mags)


def test_property_averaging_with_do_step_and_frames(tmp_path):
    # do_step and trajectory frames end steps on their own paths; the open
    # window's count and the last step's values follow them
    sc = S.suspension(n_side=2, rings=3, T=0.3)
    acc, mags, _ = _per_step_reference(sc, (35,), 1000, 10000)
    a = F.System(0)
    sc.replay(a)
    a.set_property_averaging(True)
    a.set_trajectory(str(tmp_path / "t.dump"), 7, 0)
    a.run(0)
    a.run(30)
    for _ in range(5):
        a.do_step()
    got = a.average_properties()
    assert got["count"] == 35 and got["windows"] == 0
    last = a.properties()
    for k in acc.names:
        assert abs(got["val"][k] - last[k]) <= 1e-6 * (mags[k] + 1e-300), k


# ------------------------------------------------------------- cluster props

def _ranges(sc):
    off, out = 0, []
    for name, args in sc.calls:
        if name == "add_elastomer":
            n = len(args[0]) // 2 if np.ndim(args[0]) == 1 else len(args[0])
            out.append((off, n))
            off += n
    return out


@pytest.mark.parametrize("case", ["dense", "crossing"])
def test_cluster_centres_and_centroids(case):
    """femmd_get_clusters against the oracle's FP64 restatement on the same
    float state: centres of mass and centroids within 1e-6 of the box, centre
    velocities within 1e-6 of the largest vertex speed."""
    from oracle import cluster_props
    if case == "dense":
        sc = S.suspension(n_side=3, phi=0.62, center_jitter=0.3, T=0.3)
        steps = 200
    else:
        sc, _ = G.load("susp_crossing")
        sc.calls = sc.calls[:[n for n, _ in sc.calls].index("dump_setup")]
        steps = 300
    s = F.System(0)
    sc.replay(s)
    s.run(0)
    s.run(steps)
    got = s.clusters()
    Lx, Ly = sc.calls[0][1]
    ref = cluster_props(s.positions(), s.velocities(), s.masses(), _ranges(sc), Lx, Ly)
    L = np.array([Lx, Ly])
    assert np.abs(got["cm"] - ref["cm"]).max() <= 1e-6 * L.max()
    vmax = np.abs(s.velocities()).max()
    assert np.abs(got["cm_vel"] - ref["cm_vel"]).max() <= 1e-6 * vmax
    d = got["centroid"] - ref["centroid"]
    d -= L * np.round(d / L)
    assert np.abs(d).max() <= 1e-6 * L.max()
    if case == "crossing":
        # a disk straddles the edge: its centre lies within a radius of it
        # and the unfold moved it, the centroid sits inside the box
        assert ((got["centroid"] >= 0) & (got["centroid"] <= L)).all()
