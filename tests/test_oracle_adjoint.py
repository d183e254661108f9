"""The oracle's FP64 trajectory and its hand-written adjoint (the reference
gradient for the GPU adjoint) against central finite differences of the same
FP64 forward, on a small compression scene (4 hex-ring disks, moving top
wall, per-disk E and nu).  Tolerance: relative 1e-4.  Steps: h = 1e-4 for
the parameters (E, nu, log eps, log sigma); h = 1e-6 along random
unit-scale directions of the initial positions and velocities, where the
contact-rich dynamics curves J strongly enough that h = 1e-4 differences are
off by a few percent (they converge to the adjoint value as h shrinks).  Also the float oracle's wall
and per-disk material forces against its FP64 restatement (1e-5 of the
condition scales, as the GPU checks)."""
import numpy as np
import pytest

from femmd_old_gb300 import scene as S
from oracle import Oracle

STEPS = 40
H = 1e-4


def scene():
    # denser than the benchmark case so that disks touch and every term acts
    return S.compression(n_side=2, phi=0.66, steps=STEPS, T=0.05, strain=0.15, center_jitter=0.2)


@pytest.fixture(scope="module")
def setup():
    sc = scene()
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    o.d_init()
    x0, v0 = o.d_get_state()
    ne = o.n_elastomers()
    E0 = np.array([float(np.float32(e)) for e in sc.meta["E"][:ne]])
    nu0 = np.array([float(np.float32(v)) for v in sc.meta["nu"][:ne]])
    rng = np.random.default_rng(7)
    xs, vs = rng.normal(size=x0.shape), rng.normal(size=v0.shape)
    o.d_forward(0, STEPS)
    g = o.d_backward(0, 1.0, 1.0, xseed=xs, vseed=vs)
    return o, x0, v0, E0, nu0, xs, vs, g


def J(o, x0, v0, E0, nu0, xs, vs, x=None, v=None, E=None, nu=None, se=1.0, ss=1.0):
    o.d_init()
    E = E0 if E is None else E
    nu = nu0 if nu is None else nu
    for e in range(len(E)):
        o.d_set_material(e, E[e], nu[e])
    o.d_set_scales(se, ss)
    o.d_set_state(x0 if x is None else x, v0 if v is None else v)
    j = o.d_forward(0, STEPS)
    xN, vN = o.d_get_state()
    return j + float((xs * xN).sum() + (vs * vN).sum())


def close(fd, ad, tol=1e-4):
    assert abs(fd - ad) <= tol * max(abs(fd), abs(ad), 1e-9), (fd, ad)


def test_fp64_adjoint_scales(setup):
    o, x0, v0, E0, nu0, xs, vs, g = setup
    args = (o, x0, v0, E0, nu0, xs, vs)
    assert abs(g["log_eps"]) > 0 and abs(g["log_sigma"]) > 0
    close((J(*args, se=np.exp(H)) - J(*args, se=np.exp(-H))) / (2 * H), g["log_eps"])
    close((J(*args, ss=np.exp(H)) - J(*args, ss=np.exp(-H))) / (2 * H), g["log_sigma"])


@pytest.mark.parametrize("e", [0, 3])
def test_fp64_adjoint_materials(setup, e):
    o, x0, v0, E0, nu0, xs, vs, g = setup
    args = (o, x0, v0, E0, nu0, xs, vs)
    Ep, Em = E0.copy(), E0.copy()
    Ep[e] += H
    Em[e] -= H
    close((J(*args, E=Ep) - J(*args, E=Em)) / (2 * H), g["E"][e])
    Np, Nm = nu0.copy(), nu0.copy()
    Np[e] += H
    Nm[e] -= H
    close((J(*args, nu=Np) - J(*args, nu=Nm)) / (2 * H), g["nu"][e])


@pytest.mark.parametrize("seed", [1, 2])
def test_fp64_adjoint_initial_state(setup, seed):
    o, x0, v0, E0, nu0, xs, vs, g = setup
    args = (o, x0, v0, E0, nu0, xs, vs)
    d = np.random.default_rng(seed).normal(size=x0.shape)
    h = 1e-6
    close((J(*args, x=x0 + h * d) - J(*args, x=x0 - h * d)) / (2 * h), float((g["x0"] * d).sum()))
    close((J(*args, v=v0 + h * d) - J(*args, v=v0 - h * d)) / (2 * h), float((g["v0"] * d).sum()))


def test_float_wall_and_material_forces_vs_fp64():
    sc = S.compression(n_side=3, phi=0.6, T=0.05, center_jitter=0.3)
    o = Oracle(image_mode=1, log_mode=1)
    sc.replay(o)
    o.run(0)
    o.run(60)
    o.build_nn()
    o.calc_forces()
    f = o.forces().astype(np.float64)
    f64, cond, ui, tot = o.forces_f64()
    err = np.linalg.norm(f - f64, axis=1)
    assert (err / np.maximum(cond, 1e-30)).max() <= 1e-5
    top, bottom = o.wall_forces()
    assert top > 0 or bottom > 0  # the walls act
