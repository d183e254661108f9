"""Generate the golden fixtures of the femmd2D timestep from the reference itself.

Each case is a seeded scene (femmd_old_gb300.scene) replayed by the reference's
own C++ classes, compiled from the reference sources (oracle/Makefile target
``ref`` -> oracle/_ref/ref_harness).  The harness dumps setup arrays, cell and
neighbour sets, forces, energies and trajectory snapshots; this script stores
the scene command stream and every dump in tests/golden/<case>.npz.

Run where the reference checkout exists, naming its source and mesh
directories:
    FEMMD_REF_SRC=<checkout>/femmd2D/src FEMMD_REF_MESHES=<checkout>/femmd2D/meshes \
        python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from femmd_old_gb300 import scene as S  # noqa: E402
import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
# the reference's meshes directory (femmd2D/meshes of its checkout), needed
# by the case that uses the reference's own disk mesh
MESHES = os.environ.get("FEMMD_REF_MESHES", "")


def probes(sc: S.Scene, runs=(50, 200)) -> S.Scene:
    sc.add("dump_setup").add("build_nn").add("dump_nn").add("calc_forces").add("dump_state")
    for n in runs:
        sc.add("run", n).add("dump_state")
    sc.add("dump_nn")
    return sc


def case_lj_xy():
    return probes(S.lj_fluid(n_side=16, seed_pos=11, seed_vel=12))


def case_lj_multitype():
    """Two types, per-particle sigma, asymmetric epsilon/cutoff tables."""
    n_side, rho = 14, 0.7
    n = n_side * n_side
    L = math.sqrt(n / rho)
    a = L / n_side
    rng = np.random.Generator(np.random.PCG64(21))
    ij = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy"), -1).reshape(-1, 2)
    pos = (ij + 0.5) * a + rng.uniform(-0.08, 0.08, size=(n, 2))
    typ = (rng.uniform(size=n) < 0.4).astype(np.int32)
    sig = np.where(typ == 1, 0.9, 1.05)
    m = np.where(typ == 1, 0.8, 1.2)
    vel = rng.normal(0, 0.8, size=(n, 2))
    sc = S.Scene(meta=dict(workload="lj_multitype"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.004).add("set_numTypes", 2)
    sc.add("set_pair_potential", [1.0, 0.7, 0.7, 1.3], [2.5, 1.8, 1.8, S.WCA_RC],
           [S.lj_shift(2.5), S.lj_shift(1.8), S.lj_shift(1.8), 1.0])
    sc.add("set_skin", 0.35)
    sc.add("add_particles", pos[:, 0], pos[:, 1], vel[:, 0], vel[:, 1], m, sig, typ)
    sc.add("init_neighbor_list")
    return probes(sc)


def _slab(pbc, seed):
    n_side = 12
    L = 16.0
    rng = np.random.Generator(np.random.PCG64(seed))
    ij = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy"), -1).reshape(-1, 2)
    pos = 2.0 + (ij + 0.5) * (12.0 / n_side) + rng.uniform(-0.05, 0.05, size=(n_side * n_side, 2))
    vel = rng.normal(0, 0.3, size=pos.shape)
    sc = S.Scene(meta=dict(workload=f"slab_pbc{pbc}"))
    sc.add("init", L, L).add("PBC", pbc).add("set_dt", 0.003).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [2.5], [S.lj_shift(2.5)])
    sc.add("set_skin", 0.3)
    n = pos.shape[0]
    sc.add("add_particles", pos[:, 0], pos[:, 1], vel[:, 0], vel[:, 1], np.ones(n), np.ones(n),
           np.zeros(n, np.int32))
    sc.add("init_neighbor_list")
    return probes(sc, runs=(20, 40))


def case_lj_xpbc():
    return _slab(1, 31)


def case_lj_nopbc():
    return _slab(0, 32)


def case_lj_nopbc_walls():
    """NOPBC box filled to the edges, velocities pointing outward: particles
    enter the contact range of the reference's LJ walls on every side."""
    n_side = 12
    L = 14.0
    rng = np.random.Generator(np.random.PCG64(33))
    ij = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy"), -1).reshape(-1, 2)
    pos = 0.9 + ij * ((L - 1.8) / (n_side - 1)) + rng.uniform(-0.05, 0.05, size=(n_side * n_side, 2))
    vel = (pos - L / 2) * 0.4 + rng.normal(0, 0.2, size=pos.shape)
    sc = S.Scene(meta=dict(workload="nopbc_walls"))
    sc.add("init", L, L).add("PBC", 0).add("set_dt", 0.002).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [2.5], [S.lj_shift(2.5)])
    sc.add("set_skin", 0.3)
    n = pos.shape[0]
    sc.add("add_particles", pos[:, 0], pos[:, 1], vel[:, 0], vel[:, 1], np.ones(n), np.ones(n),
           np.zeros(n, np.int32))
    sc.add("init_neighbor_list")
    return probes(sc, runs=(60, 120))


def case_susp_xpbc_gravity():
    """XPBC suspension under gravity: disks settle onto the reference's
    harmonic bottom wall (kWall = 10); one starts at the top wall."""
    verts, tris = S.hex_disk_mesh(2.5, 3, jitter=0.02, seed=71)
    nv = verts.shape[0]
    L = 22.0
    sc = S.Scene(meta=dict(workload="susp_xpbc_gravity"))
    sc.add("init", L, L).add("PBC", 1).add("set_dt", 0.002).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [S.WCA_RC], [1.0]).add("set_skin", 0.3)
    sc.add("set_kBond", 80.0).add("set_youngs_modulus", 40.0).add("set_poisson_ratio", 0.3)
    sc.add("set_elastomer_bonds", 1).add("set_gravity", 2.0)
    for c in [(5.0, 3.2), (12.0, 3.4), (18.5, 9.0), (8.0, 18.9)]:
        sc.add("add_elastomer", verts, tris, c[0], c[1], 0, 0, 1.0, float(nv), True)
    sc.add("init_neighbor_list")
    # the reference's per-cell capacity heuristic (nn.cpp:214-220) is too
    # small once the disks settle onto the wall; raise it as its C++ allows
    sc.add("set_capacity", 64, 256)
    rng = np.random.Generator(np.random.PCG64(72))
    sc.add("set_velocities_array", rng.normal(0, 0.2, size=(4 * nv, 2)).astype(np.float32))
    return probes(sc, runs=(150, 300))


def case_tiny_box():
    """Box of two cells per axis: the 3x3 stencil visits cells twice and the
    reference's list holds duplicates (applyCellBC always wraps)."""
    n_side = 6
    L = 6.0
    rng = np.random.Generator(np.random.PCG64(41))
    ij = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy"), -1).reshape(-1, 2)
    pos = (ij + 0.5) * (L / n_side) + rng.uniform(-0.05, 0.05, size=(36, 2))
    vel = rng.normal(0, 0.5, size=pos.shape)
    sc = S.Scene(meta=dict(workload="tiny_box"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.002).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [2.5], [S.lj_shift(2.5)])
    sc.add("set_skin", 0.3)
    sc.add("add_particles", pos[:, 0], pos[:, 1], vel[:, 0], vel[:, 1], np.ones(36), np.ones(36),
           np.zeros(36, np.int32))
    sc.add("init_neighbor_list")
    return probes(sc, runs=(30,))


def case_susp_all():
    return probes(S.suspension(n_side=3, rings=3, bonds="all", T=0.5, center_jitter=0.3), runs=(100, 300))


def case_susp_boundary():
    return probes(S.suspension(n_side=3, rings=3, bonds="boundary", T=0.5, center_jitter=0.3, seeds=(13, 14, 15)),
                  runs=(100, 300))


def case_susp_refdisk():
    if not MESHES:
        raise SystemExit("set FEMMD_REF_MESHES to the meshes directory of the reference checkout (femmd2D/meshes)")
    v, t = S.load_mesh(os.path.join(MESHES, "diskVertices.txt"), os.path.join(MESHES, "diskTriangles.txt"))
    sc = S.suspension(n_side=3, radius=4.0, mesh=(v * 8.0, t), bonds="all", T=0.3, center_jitter=0.2, phi=0.4)
    return probes(sc, runs=(100, 200))


def case_susp_crossing():
    """Disks drifting across the periodic boundary: FEA unwrap and
    minimum-image bond paths.  Rest lengths come from unwrapped positions."""
    verts, tris = S.hex_disk_mesh(3.0, 3, jitter=0.02, seed=51)
    nv = verts.shape[0]
    L = 20.0
    sc = S.Scene(meta=dict(workload="susp_crossing"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.002).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [S.WCA_RC], [1.0]).add("set_skin", 0.3)
    sc.add("set_kBond", 80.0).add("set_youngs_modulus", 40.0).add("set_poisson_ratio", 0.3)
    sc.add("set_elastomer_bonds", 1)
    centers = [(16.8, 10.0), (10.0, 16.8), (4.0, 4.0)]
    for c in centers:
        sc.add("add_elastomer", verts, tris, c[0], c[1], 0, 0, 1.0, float(nv), True)
    sc.add("init_neighbor_list")
    vel = np.zeros((3 * nv, 2), np.float32)
    vel[:nv, 0] = 6.0
    vel[nv:2 * nv, 1] = 6.0
    vel[2 * nv:, :] = -6.0
    sc.add("set_velocities_array", vel)
    return probes(sc, runs=(200, 300))


def case_susp_mixed():
    """Elastomers first, then free LJ particles of a second type."""
    verts, tris = S.hex_disk_mesh(3.0, 3, jitter=0.02, seed=61)
    nv = verts.shape[0]
    L = 24.0
    rng = np.random.Generator(np.random.PCG64(62))
    sc = S.Scene(meta=dict(workload="susp_mixed"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.003).add("set_numTypes", 2)
    sc.add("set_pair_potential", [1.0, 1.0, 1.0, 1.0], [2.5, S.WCA_RC, S.WCA_RC, S.WCA_RC],
           [S.lj_shift(2.5), 1.0, 1.0, 1.0])
    sc.add("set_skin", 0.3).add("set_kBond", 100.0).add("set_youngs_modulus", 50.0)
    for c in [(6.0, 6.0), (18.0, 6.0), (6.0, 18.0), (18.0, 18.0)]:
        sc.add("add_elastomer", verts, tris, c[0], c[1], 1, 0, 1.0, float(nv), True)
    centers = np.array([(6.0, 6.0), (18.0, 6.0), (6.0, 18.0), (18.0, 18.0)])
    g = (np.stack(np.meshgrid(np.arange(20), np.arange(20), indexing="xy"), -1).reshape(-1, 2) + 0.5) * (L / 20)
    d = g[:, None, :] - centers[None]
    d -= L * np.round(d / L)
    keep = ((d ** 2).sum(-1) > 4.2 ** 2).all(1)
    p = g[keep] + rng.uniform(-0.05, 0.05, size=(int(keep.sum()), 2))
    n = p.shape[0]
    v = rng.normal(0, 1.0, size=(n, 2))
    sc.add("add_particles", p[:, 0], p[:, 1], v[:, 0], v[:, 1], np.ones(n), np.ones(n), np.zeros(n, np.int32))
    sc.add("init_neighbor_list")
    return probes(sc, runs=(100, 200))


def case_susp_area():
    """Area springs (kArea > 0): disks drifting across the periodic boundary
    in a solvent of a second type, deformed by random velocities; the
    positions move triangle after triangle inside every force pass."""
    verts, tris = S.hex_disk_mesh(3.0, 3, jitter=0.02, seed=81)
    nv = verts.shape[0]
    L = 24.0
    rng = np.random.Generator(np.random.PCG64(82))
    sc = S.Scene(meta=dict(workload="susp_area"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.002).add("set_numTypes", 2)
    sc.add("set_pair_potential", [1.0, 1.0, 1.0, 1.0], [2.5, S.WCA_RC, S.WCA_RC, S.WCA_RC],
           [S.lj_shift(2.5), 1.0, 1.0, 1.0])
    sc.add("set_skin", 0.3).add("set_kBond", 80.0).add("set_youngs_modulus", 40.0)
    sc.add("set_poisson_ratio", 0.3).add("set_elastomer_bonds", 1).add("set_kArea", 0.4)
    centers = np.array([(20.8, 12.0), (12.0, 20.8), (5.0, 5.0)])
    for c in centers:
        sc.add("add_elastomer", verts, tris, c[0], c[1], 1, 0, 1.0, float(nv), True)
    g = (np.stack(np.meshgrid(np.arange(18), np.arange(18), indexing="xy"), -1).reshape(-1, 2) + 0.5) * (L / 18)
    d = g[:, None, :] - centers[None]
    d -= L * np.round(d / L)
    keep = ((d ** 2).sum(-1) > 4.3 ** 2).all(1)
    p = g[keep] + rng.uniform(-0.05, 0.05, size=(int(keep.sum()), 2))
    n = p.shape[0]
    v = rng.normal(0, 1.0, size=(n, 2))
    sc.add("add_particles", p[:, 0], p[:, 1], v[:, 0], v[:, 1], np.ones(n), np.ones(n), np.zeros(n, np.int32))
    sc.add("init_neighbor_list")
    vel = np.zeros((3 * nv + n, 2), np.float32)
    vel[:3 * nv] = rng.normal(0, 1.5, size=(3 * nv, 2))
    vel[:nv, 0] += 5.0
    vel[nv:2 * nv, 1] += 5.0
    vel[3 * nv:] = v
    sc.add("set_velocities_array", vel)
    return probes(sc, runs=(100, 250))


def case_susp_area_xpbc():
    """Area springs in an XPBC box under gravity: the reference's fixed
    top/bottom walls and gravity act on the positions from before the area
    pass, the pairs on those after it."""
    verts, tris = S.hex_disk_mesh(2.5, 3, jitter=0.02, seed=91)
    nv = verts.shape[0]
    L = 22.0
    sc = S.Scene(meta=dict(workload="susp_area_xpbc"))
    sc.add("init", L, L).add("PBC", 1).add("set_dt", 0.002).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [S.WCA_RC], [1.0]).add("set_skin", 0.3)
    sc.add("set_kBond", 80.0).add("set_youngs_modulus", 40.0).add("set_poisson_ratio", 0.3)
    sc.add("set_elastomer_bonds", 1).add("set_gravity", 2.0).add("set_kArea", 0.5)
    for c in [(5.0, 3.2), (12.0, 3.4), (18.5, 9.0), (8.0, 18.9)]:
        sc.add("add_elastomer", verts, tris, c[0], c[1], 0, 0, 1.0, float(nv), True)
    sc.add("init_neighbor_list")
    sc.add("set_capacity", 64, 256)
    rng = np.random.Generator(np.random.PCG64(92))
    sc.add("set_velocities_array", rng.normal(0, 0.6, size=(4 * nv, 2)).astype(np.float32))
    return probes(sc, runs=(150, 300))


CASES = {k[5:]: v for k, v in globals().items() if k.startswith("case_")}


# ------------------------------------------------------- writer fixtures
# The reference's file writers (md3dsystem.cpp:232-522) run on scenes with the
# FEA forces off (E = 0, the disks held by edge bonds), whose runs are bit-exact
# with the reference, so every frame can be compared byte for byte.  The
# legacy dump (layout 0) is left out: the reference lists only the first NC
# particles in it.  Fixtures go to tests/golden/frames/<case>.npz.

def _saves(sc: S.Scene, first: bool, vtk: bool):
    a = 0 if first else 1
    sc.add("save_frame", "f.xyz", 1, a).add("save_frame", "f.vtf", 3, a).add("save_frame", "c.vtf", 4, a)
    if vtk:
        sc.add("save_frame", "v", 2, 0).add("save_frame", "x", 5, 0).add("save_frame", "b", 6, 0)
    return sc


def frames_elastomers():
    """Disks only (the VTK writers read unfolded positions, which the
    reference holds for elastomer vertices alone), held by bonds on every
    mesh edge, drifting across the periodic boundary; every layout at the
    start and after two runs."""
    verts, tris = S.hex_disk_mesh(3.0, 3, jitter=0.02, seed=111)
    nv = verts.shape[0]
    L = 20.0
    rng = np.random.Generator(np.random.PCG64(112))
    sc = S.Scene(meta=dict(workload="frames_elastomers"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.002).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [S.WCA_RC], [1.0]).add("set_skin", 0.3)
    sc.add("set_kBond", 80.0).add("set_youngs_modulus", 0.0).add("set_elastomer_bonds", 0)
    for c in [(16.6, 10.0), (10.0, 16.6), (4.0, 4.0)]:
        sc.add("add_elastomer", verts, tris, c[0], c[1], 0, 0, 1.0, float(nv), True)
    sc.add("init_neighbor_list")
    vel = rng.normal(0, 0.3, size=(3 * nv, 2))
    vel[:nv, 0] += 6.0
    vel[nv:2 * nv, 1] += 6.0
    vel[2 * nv:] -= 6.0
    sc.add("set_velocities_array", vel.astype(np.float32))
    sc.add("set_scale", 0.8)
    _saves(sc, True, True)
    for n in (40, 60):
        sc.add("run", n).add("dump_state")
        _saves(sc, False, True)
    return sc


def frames_mixed():
    """Disks of type 1 among free particles of type 0 (sigma 0.9) with bonds
    between free neighbours: the VTF structure block (type letters, radii,
    bond list, box) and one cluster VTF atom per disk."""
    verts, tris = S.hex_disk_mesh(2.5, 2, jitter=0.02, seed=121)
    nv = verts.shape[0]
    L = 16.0
    rng = np.random.Generator(np.random.PCG64(122))
    sc = S.Scene(meta=dict(workload="frames_mixed"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.002).add("set_numTypes", 2)
    sc.add("set_pair_potential", [1.0, 1.0, 1.0, 1.0], [2.5, S.WCA_RC, S.WCA_RC, S.WCA_RC],
           [S.lj_shift(2.5), 1.0, 1.0, 1.0])
    sc.add("set_skin", 0.3).add("set_kBond", 60.0).add("set_youngs_modulus", 0.0).add("set_elastomer_bonds", 0)
    centers = np.array([(4.0, 4.0), (12.0, 4.0), (4.0, 12.0), (12.0, 12.0)])
    for c in centers:
        sc.add("add_elastomer", verts, tris, float(c[0]), float(c[1]), 1, 0, 1.0, float(nv), True)
    g = (np.stack(np.meshgrid(np.arange(12), np.arange(12), indexing="xy"), -1).reshape(-1, 2) + 0.5) * (L / 12)
    d = g[:, None, :] - centers[None]
    d -= L * np.round(d / L)
    keep = ((d ** 2).sum(-1) > 3.6 ** 2).all(1)
    p = g[keep] + rng.uniform(-0.05, 0.05, size=(int(keep.sum()), 2))
    n = p.shape[0]
    v = rng.normal(0, 0.8, size=(n, 2))
    sc.add("add_particles", p[:, 0], p[:, 1], v[:, 0], v[:, 1], np.ones(n), np.full(n, 0.9), np.zeros(n, np.int32))
    base = 4 * nv
    for k in range(0, n - 1, 5):
        sc.add("create_bond", base + k, base + k + 1)
    sc.add("init_neighbor_list")
    _saves(sc, True, False)
    for n_ in (50, 50):
        sc.add("run", n_).add("dump_state")
        _saves(sc, False, False)
    return sc


FRAME_CASES = {k[7:]: v for k, v in globals().items() if k.startswith("frames_")}


def green_susp_cpu1():
    """The reference's CPU Green-strain / linear-C law
    (Interactions::calcFeaForcesCPU1, interactions.cpp:411-530), called alone
    after zeroStuff at positions the reference's own run (neo-Hookean, no
    bonds) deformed: six hex-ring disks, apart from each other (no pair
    inside the WCA cutoff), three across the periodic edges."""
    verts, tris = S.hex_disk_mesh(3.0, 3, jitter=0.03, seed=81)
    nv = verts.shape[0]
    L = 30.0
    sc = S.Scene(meta=dict(workload="green_cpu1"))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", 0.002).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [S.WCA_RC], [1.0]).add("set_skin", 0.3)
    sc.add("set_kBond", 0.0).add("set_youngs_modulus", 45.0).add("set_poisson_ratio", 0.3)
    sc.add("set_elastomer_bonds", 2)
    centers = [(0.4, 7.0), (15.0, 0.2), (29.6, 29.5), (8.0, 20.0), (21.0, 12.0), (14.5, 23.0)]
    for c in centers:
        sc.add("add_elastomer", verts, tris, c[0], c[1], 0, 0, 1.0, float(nv), True)
    sc.add("init_neighbor_list")
    rng = np.random.Generator(np.random.PCG64(82))
    sc.add("set_velocities_array", rng.normal(0, 0.6, size=(len(centers) * nv, 2)).astype(np.float32))
    sc.add("dump_setup")
    for n in (60, 90):
        sc.add("run", n).add("dump_state").add("fea_cpu1").add("dump_state")
    return sc


GREEN_CASES = {k[6:]: v for k, v in globals().items() if k.startswith("green_")}


def save_frames(name: str, sc: S.Scene, dumps, files):
    blob = {"scene": np.frombuffer(sc.to_bytes(), np.uint8)}
    for k, (tag, d) in enumerate(dumps):
        for key, val in d.items():
            blob[f"d{k:02d}_{tag}_{key}"] = np.asarray(val)
    blob["frame_names"] = np.array(sorted(files), dtype="U64")
    for k, fname in enumerate(sorted(files)):
        blob[f"frame{k:03d}"] = np.frombuffer(files[fname], np.uint8)
    os.makedirs(os.path.join(OUT, "frames"), exist_ok=True)
    np.savez_compressed(os.path.join(OUT, "frames", f"{name}.npz"), **blob)


def save(name: str, sc: S.Scene, dumps):
    blob = {"scene": np.frombuffer(sc.to_bytes(), np.uint8)}
    for k, (tag, d) in enumerate(dumps):
        for key, val in d.items():
            blob[f"d{k:02d}_{tag}_{key}"] = np.asarray(val)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **blob)


def main(names=None):
    if O.build_reference() is None:
        raise SystemExit("reference sources not found: set FEMMD_REF_SRC to the checkout's femmd2D/src")
    for name, fn in CASES.items():
        if names and name not in names:
            continue
        sc = fn()
        dumps = O.run_reference(sc)
        save(name, sc, dumps)
        print(f"{name}: {len(dumps)} dumps, {os.path.getsize(os.path.join(OUT, name + '.npz'))} bytes")
    for name, fn in GREEN_CASES.items():
        if names and "green_" + name not in names:
            continue
        sc = fn()
        dumps = O.run_reference(sc)
        os.makedirs(os.path.join(OUT, "green"), exist_ok=True)
        save(os.path.join("green", name), sc, dumps)
        print(f"green {name}: {len(dumps)} dumps")
    for name, fn in FRAME_CASES.items():
        if names and "frames_" + name not in names:
            continue
        sc = fn()
        files = {}
        dumps = O.run_reference(sc, files=files)
        save_frames(name, sc, dumps, files)
        print(f"frames {name}: {len(files)} files, {os.path.getsize(os.path.join(OUT, 'frames', name + '.npz'))} bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
