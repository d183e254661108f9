"""Observables of Properties::evaluate (femmd_get_properties) against the
oracle's FP64 restatement on the same float state: uKinetic, uPotential,
uTotal, temperature, virial, feaVirial, pressure, clusterUKinetic,
clusterVirial, molPressure.  Tolerance: relative 1e-4, with absolute floors
of 1e-4 times the largest virial-type magnitude for the virials and pressures
(float forces against double; the virials sum terms of both signs) and 1e-6
times (|uKinetic| + |uPotential| + 1) for the energies (a potential energy
that cancels to ~0 is float noise)."""
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
    r = o.properties()
    vscale = max(abs(r["virial"]), abs(r["feaVirial"]), abs(r["clusterVirial"]), 1e-12)
    escale = abs(r["uKinetic"]) + abs(r["uPotential"]) + 1.0
    for k in r:
        floor = 1e-4 * vscale if ("irial" in k or "ressure" in k) else 1e-6 * escale
        assert abs(g[k] - r[k]) <= max(1e-4 * abs(r[k]), floor), (k, g[k], r[k])
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
