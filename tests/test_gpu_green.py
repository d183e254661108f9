"""GPU parity of the Green-strain / linear-C triangle law (tri_green, the
reference's GPU kernel computeFeaForcesGPU, interactionsCuda.cu:312-451)
against the reference's own CPU twin of that law,
Interactions::calcFeaForcesCPU1 (interactions.cpp:411-530), run by the
reference itself (tests/golden/green/susp_cpu1.npz).

Tolerances: at the positions the reference dumped, the product's forces are
bit-identical to the oracle's float restatement of the kernel, and within
1e-6 of the largest FEA force of the reference's CPU twin (which sums the
nodal force terms in double); both force modes.
"""
import numpy as np
import pytest

import golden_io as G
import femmd_old_gb300 as F
from oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1])
def test_green_law_against_reference_cpu_twin(mode):
    sc, ref = G.load("green/susp_cpu1")
    states = [d for t, d in ref if t == "state"]
    first = next(k for k, (n, _) in enumerate(sc.calls) if n == "run")
    s = F.System()
    s.set_force_mode(mode)
    s.set_image_mode(0)
    s.set_fea_law(1)
    o = Oracle(image_mode=0, log_mode=0, fea_law=1)
    for n, a in sc.calls[:first]:
        if n.startswith("dump"):
            continue
        getattr(s, n)(*a)
        getattr(o, n)(*a)
    for k in (0, 2):
        pos, vel, cpu1 = states[k]["pos"], states[k]["vel"], states[k + 1]
        s.set_state(pos, vel)
        s.build_nn()
        s.calc_forces()
        f = s.forces()
        o.set_positions_array(pos)
        o.build_nn()
        o.calc_forces()
        assert np.array_equal(G.bits(f), G.bits(o.forces()))
        g = cpu1["force"].astype(np.float64)
        assert np.abs(f.astype(np.float64) - g).max() <= 1e-6 * np.abs(g).max()
        assert abs(s.energies()[0] - float(cpu1["scalars"][0])) <= 1e-6 * abs(float(cpu1["scalars"][0]))
