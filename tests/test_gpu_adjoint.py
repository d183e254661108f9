"""Differentiable compression on the GPU (benchmark config 5): moving harmonic
top wall, per-disk E and nu, and the adjoint (femmd_adjoint_*).

Tolerances (stated here, used below):
  * forward with walls and per-disk materials: bit-exact against the oracle
    (same kernels' arithmetic, exact image, own log), wall forces equal;
    forces within 1e-5 of the FP64 restatement's condition scales;
  * GPU adjoint (FP32 forward and adjoint) against the FP64 adjoint taken
    along the same float trajectory (the oracle's float run, bit-identical
    to the GPU's, differentiated in double): relative error <= 1e-4 for dJ/dE
    and dJ/dnu (vectors over the disks), dJ/dlog eps, dJ/dlog sigma and the
    initial position and velocity gradients (norm of the difference over the
    norm);
  * GPU adjoint against the fully FP64 run (FP64 trajectory + FP64 adjoint):
    relative <= 2e-3.  The float trajectory itself leaves the double one by
    a few 1e-4 in the velocities over 100-200 steps of these stiff contacts,
    and the FP64 gradients along the two trajectories differ by as much, so
    no float forward can be closer;
  * GPU adjoint against central differences of the GPU forward in log sigma
    (h = 1e-3): relative 1e-2 (FP32 forward noise); along one random
    direction of each other input (log eps, E, nu, initial positions and
    velocities): 1e-2 of the directional derivative plus 4e-6 |J|, the
    spread of two FP32 forward runs of the dense compression;
  * the torch.autograd.Function wrapper gives the same gradients as the C ABI.
"""
import numpy as np
import pytest
import torch

import femmd_old_gb300 as F
from femmd_old_gb300 import scene as S
from oracle import Oracle
from adjoint_torch import CompressionRun, build

pytestmark = pytest.mark.gpu


KEYS = ("E", "nu", "log_eps", "log_sigma", "x0", "v0")


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def gpu_system(sc):
    s = F.System(0)
    sc.replay(s)
    return s


def test_compression_forward_bitwise_vs_oracle():
    sc = S.compression(n_side=4)
    s = gpu_system(sc)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    for n in (0, 37, 50):
        s.run(n)
        o.run(n)
        p, v, a = s.get_state()
        assert np.array_equal(p.view(np.uint32), o.positions().view(np.uint32))
        assert np.array_equal(v.view(np.uint32), o.velocities().view(np.uint32))
        assert np.array_equal(a.view(np.uint32), o.accelerations().view(np.uint32))
        assert s.wall_forces() == o.wall_forces()
    assert s.wall_forces()[0] > 0  # the top wall is pushing


def test_compression_forces_vs_fp64():
    sc = S.compression(n_side=4)
    s = gpu_system(sc)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    s.run(0)
    s.run(60)
    o.run(0)
    o.run(60)
    s.calc_forces()
    f = s.forces().astype(np.float64)
    o.build_nn()
    f64, cond, ui, tot = o.forces_f64()
    err = np.linalg.norm(f - f64, axis=1)
    assert (err / np.maximum(cond, 1e-30)).max() <= 1e-5


def fp64_reference(sc, steps, every, xseed=None, vseed=None):
    """(J, gradients) of the fully FP64 run, and the FP64 gradients along the
    float trajectory of the same run(every) segments."""
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    o.d_init()
    J = o.d_forward(0, steps)
    g = o.d_backward(0, 1.0, 1.0, xseed=xseed, vseed=vseed)
    of = Oracle(image_mode=1, log_mode=1)
    sc.replay(of)
    traj = of.float_trajectory(steps, every)
    of.d_init()
    of.d_set_traj(traj)
    gf = of.d_backward(0, 1.0, 1.0, xseed=xseed, vseed=vseed)
    return J, g, gf


@pytest.fixture(scope="module")
def config5():
    sc = S.compression()  # 64 disks, 200 steps, checkpoint every 20
    s = gpu_system(sc)
    s.adjoint_forward(200, 20)
    ws, fe = s.adjoint_observable()
    state = s.get_state()
    g = s.adjoint_backward()
    J64, g64, gf = fp64_reference(sc, 200, 20)
    return sc, s, ws + fe, state, g, J64, g64, gf


def test_adjoint_observable_matches_fp64(config5):
    sc, s, J, state, g, J64, g64, gf = config5
    assert abs(J - J64) <= 1e-4 * abs(J64), (J, J64)


@pytest.mark.parametrize("key", KEYS)
def test_adjoint_matches_fp64_adjoint_on_float_trajectory(config5, key):
    sc, s, J, state, g, J64, g64, gf = config5
    r = rel(g[key], gf[key])
    assert r <= 1e-4, (key, r)


@pytest.mark.parametrize("key", KEYS)
def test_adjoint_matches_fully_fp64_run(config5, key):
    sc, s, J, state, g, J64, g64, gf = config5
    r = rel(g[key], g64[key])
    assert r <= 2e-3, (key, r)


def test_adjoint_restores_final_state(config5):
    sc, s, J, state, g, J64, g64, gf = config5
    p, v, a = s.get_state()
    for x, y in zip((p, v, a), state):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    assert s.steps() == 200


def test_adjoint_seeds_vs_fp64():
    # denser than config 5 so that the disks press on each other (the LJ
    # terms and their eps/sigma derivatives act)
    sc = S.compression(n_side=4, steps=100, phi=0.62, strain=0.05, center_jitter=0.3, T=0.02)
    s = gpu_system(sc)
    n = s.N
    rng = np.random.default_rng(3)
    xs = rng.normal(size=(n, 2)).astype(np.float32)
    vs = rng.normal(size=(n, 2)).astype(np.float32)
    s.adjoint_forward(100, 20)
    g = s.adjoint_backward(1.0, 1.0, xbar_final=xs, vbar_final=vs)
    J64, g64, gf = fp64_reference(sc, 100, 20, xseed=xs.astype(np.float64), vseed=vs.astype(np.float64))
    assert abs(g64["log_eps"]) > 0
    for key in KEYS:
        assert rel(g[key], gf[key]) <= 1e-4, key
        assert rel(g[key], g64[key]) <= 2e-3, key


def test_adjoint_vs_gpu_finite_differences():
    sc = S.compression(n_side=4, steps=100)
    E = sc.meta["E"]
    nu = sc.meta["nu"]

    def J(log_sigma):
        s = build(sc, E, nu, 0.0, log_sigma)
        s.adjoint_forward(100, 20)
        ws, fe = s.adjoint_observable()
        return ws + fe

    s = build(sc, E, nu, 0.0, 0.0)
    s.adjoint_forward(100, 20)
    g = s.adjoint_backward()
    h = 1e-3
    fd = (J(h) - J(-h)) / (2 * h)
    assert abs(fd - g["log_sigma"]) <= 1e-2 * abs(g["log_sigma"]), (fd, g["log_sigma"])


@pytest.mark.parametrize("key", ["log_eps", "E", "nu", "x0", "v0"])
def test_adjoint_directional_finite_differences(key):
    # the dense compression, where the disks press on each other: central
    # differences of the GPU forward along one random direction of each input
    # against the adjoint's directional derivative. E moves by exp(+-h d) per
    # disk, nu and the initial state by +-h d; the initial state is rounded to
    # float before the run, so the prediction uses the rounded difference.
    # h per input keeps the FP64 run's own central-difference error below
    # 4e-3 of the derivative (E 2e-4, nu 1e-4, x0 2e-3, v0 4e-3, log eps 3e-4)
    # while the step's change of J is large against the FP32 forward's noise:
    # two float runs of these stiff contacts land a few 1e-6 of J apart
    # (J ~ 2e3), which bounds the check from below by 4e-6 |J|.
    sc = S.compression(n_side=4, steps=100, phi=0.62, strain=0.05, center_jitter=0.3, T=0.02)
    E0 = np.asarray(sc.meta["E"], np.float64)
    nu0 = np.asarray(sc.meta["nu"], np.float64)
    b = build(sc, E0, nu0, 0.0, 0.0)
    x0, v0 = b.positions(), b.velocities()

    def run(E=E0, nu=nu0, le=0.0, x=x0, v=v0):
        s = build(sc, E, nu, le, 0.0)
        s.set_positions_array(x)
        s.set_velocities_array(v)
        s.adjoint_forward(100, 20)
        return s

    def J(**kw):
        ws, fe = run(**kw).adjoint_observable()
        return ws + fe

    s0 = run()
    ws0, fe0 = s0.adjoint_observable()
    g = s0.adjoint_backward()
    rng = np.random.default_rng(11)
    h = {"log_eps": 3e-2, "E": 1e-2, "nu": 1e-3, "x0": 1e-3, "v0": 3e-2}[key]
    if key == "log_eps":
        d = J(le=h) - J(le=-h)
        pred = g["log_eps"] * 2 * h
    elif key == "E":
        u = rng.choice([-1.0, 1.0], size=E0.shape)
        d = J(E=E0 * np.exp(h * u)) - J(E=E0 * np.exp(-h * u))
        pred = float(np.dot(g["E"], E0 * (np.exp(h * u) - np.exp(-h * u))))
    elif key == "nu":
        u = rng.choice([-1.0, 1.0], size=nu0.shape)
        d = J(nu=nu0 + h * u) - J(nu=nu0 - h * u)
        pred = float(np.dot(g["nu"], 2 * h * u))
    else:
        z = x0 if key == "x0" else v0
        u = rng.normal(size=z.shape)
        zp = (z + h * u).astype(np.float32)
        zm = (z - h * u).astype(np.float32)
        d = J(**{key[0]: zp}) - J(**{key[0]: zm})
        pred = float((np.asarray(g[key], np.float64) * (zp.astype(np.float64) - zm)).sum())
    assert abs(pred) > 25 * 4e-6 * abs(ws0 + fe0), (key, pred)
    assert abs(d - pred) <= 1e-2 * abs(pred) + 4e-6 * abs(ws0 + fe0), (key, d, pred)


def test_torch_autograd_function():
    sc = S.compression(n_side=4, steps=60)
    s = gpu_system(sc)
    x0 = torch.tensor(s.positions(), dtype=torch.float64, requires_grad=True)
    v0 = torch.tensor(s.velocities(), dtype=torch.float64, requires_grad=True)
    E = torch.tensor(sc.meta["E"], dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(sc.meta["nu"], dtype=torch.float64, requires_grad=True)
    le = torch.zeros((), dtype=torch.float64, requires_grad=True)
    ls = torch.zeros((), dtype=torch.float64, requires_grad=True)
    cx = torch.from_numpy(np.random.default_rng(5).normal(size=(s.N, 2)).astype(np.float32))
    J = CompressionRun.apply(x0, v0, E, nu, le, ls, sc, 60, 20, cx)
    (2.0 * J).backward()
    # the same through the C ABI
    s2 = build(sc, sc.meta["E"], sc.meta["nu"], 0.0, 0.0)
    s2.adjoint_forward(60, 20)
    r = s2.adjoint_backward(2.0, 2.0, xbar_final=2.0 * cx.numpy())
    assert np.allclose(x0.grad.numpy(), r["x0"], rtol=1e-6, atol=1e-6)
    assert np.allclose(v0.grad.numpy(), r["v0"], rtol=1e-6, atol=1e-6)
    assert np.allclose(E.grad.numpy(), r["E"], rtol=1e-9)
    assert np.allclose(nu.grad.numpy(), r["nu"], rtol=1e-9)
    assert abs(float(ls.grad) - r["log_sigma"]) <= 1e-9 * abs(r["log_sigma"])


def test_adjoint_rejects_green_law():
    sc = S.compression(n_side=2, steps=20)
    s = F.System(0)
    s.set_fea_law(1)
    sc.replay(s)
    with pytest.raises(F.FemmdError):
        s.adjoint_forward(20, 10)
