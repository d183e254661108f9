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
