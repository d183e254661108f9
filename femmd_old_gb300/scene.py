"""Scenes: replayable lists of setup/run calls, and the seeded synthetic
workloads of the femmd2D timestep benchmarks.

A scene is the sequence of calls a reference script makes on its ``System``
object (femmd2D/src/interface.cpp:656-696: ``init``, ``PBC``, ``set_dt``,
``set_pair_potential``, ``set_kBond``, ``set_youngs_modulus``,
``add_elastomer``, ``add_particle``, ``init_neighbor_list``, ``run`` ...), plus
the C++-only knobs the reference exposes on its classes (``set_skin`` =
``NeighborList::setSkin`` femmd2D/src/nn.h:64, ``set_poisson_ratio`` =
``Interactions::nu`` femmd2D/src/interactions.h:22).  ``Scene.replay(target)``
calls the same-named methods on any target (``femmd_old_gb300.System`` or a
checker), and ``Scene.to_bytes()`` writes the little-endian command stream
understood by the reference harness.

All workloads are synthetic and seeded (numpy PCG64); no dataset is involved.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

# command opcodes of the serialized scene stream
OP = dict(END=0, INIT=1, PBC=2, DT=3, NUMTYPES=4, PAIR=5, KBOND=6, YOUNG=7, NU=8, SKIN=9,
          ELASTOMER=10, PARTICLE=11, BOND=12, INITNN=13, CAPACITY=14, RUN=15, STEP=16,
          BUILDNN=17, FORCES=18, ELASTOMER_BONDS=19, DUMP_STATE=20, DUMP_NN=21, DUMP_SETUP=22,
          SETVEL=23, GRAVITY=24, KAREA=25, SAVE=26, SCALE=27, FEA_CPU1=28)

WCA_RC = 2.0 ** (1.0 / 6.0)


def lj_shift(rc: float) -> float:
    """uShift making the truncated LJ potential vanish at rc: -4(rc^-12 - rc^-6)."""
    return -4.0 * (rc ** -12 - rc ** -6)


@dataclass
class Scene:
    calls: list = field(default_factory=list)
    meta: dict = field(default_factory=dict)

    def add(self, name, *args):
        self.calls.append((name, args))
        return self

    def replay(self, target, stop_at=None):
        for name, args in self.calls:
            if stop_at is not None and name in stop_at:
                break
            getattr(target, name)(*args)
        return target

    # --------------------------------------------------------- serialization
    def to_bytes(self) -> bytes:
        out = bytearray()
        w = out.extend
        for name, a in self.calls:
            if name == "init":
                w(struct.pack("<idd", OP["INIT"], a[0], a[1]))
            elif name == "PBC":
                w(struct.pack("<ii", OP["PBC"], int(a[0])))
            elif name == "set_dt":
                w(struct.pack("<id", OP["DT"], a[0]))
            elif name == "set_numTypes":
                w(struct.pack("<ii", OP["NUMTYPES"], int(a[0])))
            elif name == "set_pair_potential":
                e, r, u = (np.asarray(x, np.float64).ravel() for x in a)
                w(struct.pack("<ii", OP["PAIR"], e.size))
                w(e.tobytes()); w(r.tobytes()); w(u.tobytes())
            elif name == "set_kBond":
                w(struct.pack("<id", OP["KBOND"], a[0]))
            elif name == "set_gravity":
                w(struct.pack("<id", OP["GRAVITY"], a[0]))
            elif name == "set_kArea":
                w(struct.pack("<id", OP["KAREA"], a[0]))
            elif name == "set_youngs_modulus":
                w(struct.pack("<id", OP["YOUNG"], a[0]))
            elif name == "set_poisson_ratio":
                w(struct.pack("<id", OP["NU"], a[0]))
            elif name == "set_skin":
                w(struct.pack("<id", OP["SKIN"], a[0]))
            elif name == "set_elastomer_bonds":
                w(struct.pack("<ii", OP["ELASTOMER_BONDS"], int(a[0])))
            elif name == "add_elastomer":
                v = np.ascontiguousarray(a[0], np.float32).ravel()
                t = np.ascontiguousarray(a[1], np.int32).ravel()
                x, y, typ, g, sig, mass, exc = a[2:9]
                w(struct.pack("<iii", OP["ELASTOMER"], v.size // 2, t.size // 3))
                w(v.tobytes()); w(t.tobytes())
                w(struct.pack("<ddiiddi", x, y, int(typ), int(g), sig, mass, int(bool(exc))))
            elif name == "add_particle":
                w(struct.pack("<iddddddi", OP["PARTICLE"], *[float(v) for v in a[:6]], int(a[6])))
            elif name == "create_bond":
                w(struct.pack("<iii", OP["BOND"], int(a[0]), int(a[1])))
            elif name == "add_particles":
                # bulk form of add_particle: (x, y, vx, vy, m, sig, typ) columns
                cols = [np.asarray(c) for c in a]
                for k in range(cols[0].size):
                    w(struct.pack("<iddddddi", OP["PARTICLE"], *[float(c[k]) for c in cols[:6]], int(cols[6][k])))
            elif name == "set_velocities_array":
                v = np.ascontiguousarray(a[0], np.float32).ravel()
                w(struct.pack("<i", OP["SETVEL"]))
                w(v.tobytes())
            elif name == "init_neighbor_list":
                w(struct.pack("<i", OP["INITNN"]))
            elif name == "set_capacity":
                w(struct.pack("<iii", OP["CAPACITY"], int(a[0]), int(a[1])))
            elif name == "run":
                w(struct.pack("<ii", OP["RUN"], int(a[0])))
            elif name == "do_step":
                w(struct.pack("<i", OP["STEP"]))
            elif name == "build_nn":
                w(struct.pack("<i", OP["BUILDNN"]))
            elif name == "calc_forces":
                w(struct.pack("<i", OP["FORCES"]))
            elif name == "fea_cpu1":
                w(struct.pack("<i", OP["FEA_CPU1"]))
            elif name == "dump_state":
                w(struct.pack("<i", OP["DUMP_STATE"]))
            elif name == "dump_nn":
                w(struct.pack("<i", OP["DUMP_NN"]))
            elif name == "dump_setup":
                w(struct.pack("<i", OP["DUMP_SETUP"]))
            elif name == "save_frame":
                # (file name, layout, append): the name is relative to where the frames go
                nm = str(a[0]).encode()
                w(struct.pack("<iiii", OP["SAVE"], int(a[1]), int(a[2]), len(nm)))
                w(nm)
            elif name == "set_scale":
                w(struct.pack("<id", OP["SCALE"], a[0]))
            elif name in ("allocate_cuda", "DEV", "set_fea_law", "set_bond_k_mode", "set_image_mode"):
                continue
            else:
                raise ValueError(f"scene call {name!r} has no command encoding")
        w(struct.pack("<i", OP["END"]))
        return bytes(out)

    @staticmethod
    def from_bytes(buf: bytes) -> "Scene":
        sc = Scene()
        off = 0

        def take(fmt):
            nonlocal off
            vals = struct.unpack_from("<" + fmt, buf, off)
            off += struct.calcsize("<" + fmt)
            return vals

        def take_arr(dtype, n):
            nonlocal off
            arr = np.frombuffer(buf, dtype=dtype, count=n, offset=off).copy()
            off += arr.nbytes
            return arr

        inv = {v: k for k, v in OP.items()}
        pend_particles = []

        def flush():
            if pend_particles:
                cols = list(zip(*pend_particles))
                sc.add("add_particles", *[np.array(c, dtype=np.float64 if i < 6 else np.int32)
                                          for i, c in enumerate(cols)])
                pend_particles.clear()

        while True:
            (op,) = take("i")
            name = inv[op]
            if name != "PARTICLE":
                flush()
            if name == "END":
                break
            if name == "INIT":
                sc.add("init", *take("dd"))
            elif name == "PBC":
                sc.add("PBC", *take("i"))
            elif name == "DT":
                sc.add("set_dt", *take("d"))
            elif name == "NUMTYPES":
                sc.add("set_numTypes", *take("i"))
            elif name == "PAIR":
                (n2,) = take("i")
                sc.add("set_pair_potential", take_arr(np.float64, n2), take_arr(np.float64, n2),
                       take_arr(np.float64, n2))
            elif name == "KBOND":
                sc.add("set_kBond", *take("d"))
            elif name == "GRAVITY":
                sc.add("set_gravity", *take("d"))
            elif name == "KAREA":
                sc.add("set_kArea", *take("d"))
            elif name == "YOUNG":
                sc.add("set_youngs_modulus", *take("d"))
            elif name == "NU":
                sc.add("set_poisson_ratio", *take("d"))
            elif name == "SKIN":
                sc.add("set_skin", *take("d"))
            elif name == "ELASTOMER_BONDS":
                sc.add("set_elastomer_bonds", *take("i"))
            elif name == "ELASTOMER":
                nv, nt = take("ii")
                v = take_arr(np.float32, 2 * nv)
                t = take_arr(np.int32, 3 * nt)
                x, y, typ, g, sig, mass, exc = take("ddiiddi")
                sc.add("add_elastomer", v, t, x, y, typ, g, sig, mass, bool(exc))
            elif name == "PARTICLE":
                pend_particles.append(take("ddddddi"))
            elif name == "BOND":
                sc.add("create_bond", *take("ii"))
            elif name == "SAVE":
                layout, append, n = take("iii")
                nm = bytes(take_arr(np.uint8, n)).decode()
                sc.add("save_frame", nm, layout, append)
            elif name == "SCALE":
                sc.add("set_scale", *take("d"))
            elif name == "SETVEL":
                n = sum(len(a[0]) for nm, a in sc.calls if nm == "add_particles") + \
                    sum(len(a[0]) // 2 for nm, a in sc.calls if nm == "add_elastomer") + \
                    sum(1 for nm, a in sc.calls if nm == "add_particle")
                sc.add("set_velocities_array", take_arr(np.float32, 2 * n).reshape(-1, 2))
            elif name == "INITNN":
                sc.add("init_neighbor_list")
            elif name == "CAPACITY":
                sc.add("set_capacity", *take("ii"))
            elif name == "RUN":
                sc.add("run", *take("i"))
            elif name == "STEP":
                sc.add("do_step")
            elif name == "BUILDNN":
                sc.add("build_nn")
            elif name == "FORCES":
                sc.add("calc_forces")
            elif name == "FEA_CPU1":
                sc.add("fea_cpu1")
            elif name == "DUMP_STATE":
                sc.add("dump_state")
            elif name == "DUMP_NN":
                sc.add("dump_nn")
            elif name == "DUMP_SETUP":
                sc.add("dump_setup")
        return sc


# ------------------------------------------------------------------- meshes

def hex_disk_mesh(radius: float = 5.0, rings: int = 6, jitter: float = 0.0, seed: int | None = None):
    """Structured hexagonal-ring disk: 1 + sum_{k=1..rings} 6k vertices,
    6 rings^2 counter-clockwise triangles.  Returns (vertices float32 [nv,2],
    triangles int32 [nt,3] 1-based, boundary-edge mask per triangle edge).

    Ring k holds 6k vertices on the hexagon of 'radius' k*h (h = radius/rings)
    projected to the circle, so the outer ring is a circle of the given radius.
    Interior vertices get uniform jitter in [-jitter, jitter] per axis.
    """
    h = radius / rings
    verts = [(0.0, 0.0)]
    ring_start = [0]
    for k in range(1, rings + 1):
        ring_start.append(len(verts))
        for s in range(6):
            a0 = math.pi / 3 * s
            a1 = math.pi / 3 * (s + 1)
            for j in range(k):
                # point on the hexagon side, then radial projection to radius k*h
                px = (1 - j / k) * math.cos(a0) + (j / k) * math.cos(a1)
                py = (1 - j / k) * math.sin(a0) + (j / k) * math.sin(a1)
                ang = math.atan2(py, px)
                verts.append((k * h * math.cos(ang), k * h * math.sin(ang)))

    def vid(k, i):  # vertex i (mod 6k) of ring k
        if k == 0:
            return 0
        return ring_start[k] + (i % (6 * k))

    tris = []
    for k in range(1, rings + 1):
        for s in range(6):
            for j in range(k):
                # outer ring index along side s: i = s*k + j ; inner ring: s*(k-1) + j
                o0 = vid(k, s * k + j)
                o1 = vid(k, s * k + j + 1)
                i0 = vid(k - 1, s * (k - 1) + j)
                tris.append((o0, o1, i0))
                if j < k - 1:
                    i1 = vid(k - 1, s * (k - 1) + j + 1)
                    tris.append((i0, o1, i1))
    v = np.array(verts, dtype=np.float64)
    t = np.array(tris, dtype=np.int64)
    # orient counter-clockwise
    e1 = v[t[:, 1]] - v[t[:, 0]]
    e2 = v[t[:, 2]] - v[t[:, 0]]
    cw = (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]) < 0
    t[cw] = t[cw][:, [0, 2, 1]]
    if jitter > 0:
        rng = np.random.Generator(np.random.PCG64(seed))
        interior = np.arange(v.shape[0]) < ring_start[rings]
        v[interior] += rng.uniform(-jitter, jitter, size=(int(interior.sum()), 2))
    return v.astype(np.float32), (t + 1).astype(np.int32)


def load_mesh(vertices_path: str, triangles_path: str):
    """Whitespace mesh files as in femmd2D/meshes (read_file,
    femmd2D/src/interface.cpp:135-195): 'x y' per line, 1-based 'i j k'."""
    v = np.loadtxt(vertices_path, dtype=np.float64).astype(np.float32).reshape(-1, 2)
    t = np.loadtxt(triangles_path, dtype=np.int64).astype(np.int32).reshape(-1, 3)
    return v, t


def boundary_edges(tris1: np.ndarray) -> set:
    """Undirected edges (0-based, sorted pairs) that belong to one triangle."""
    from collections import Counter
    c = Counter()
    for a, b, d in (tris1 - 1):
        for e in ((a, b), (a, d), (b, d)):
            c[tuple(sorted((int(e[0]), int(e[1]))))] += 1
    return {e for e, n in c.items() if n == 1}


# --------------------------------------------------------------- workloads

def _mb_velocities(rng, n, T, mass=None):
    """Maxwell-Boltzmann velocities with zero net momentum, rescaled so the
    kinetic energy per particle, 0.5 sum m v^2 / n, equals T exactly (2D, kB=1)."""
    m = np.ones(n) if mass is None else np.asarray(mass, np.float64)
    v = rng.normal(0.0, 1.0, size=(n, 2)) * np.sqrt(T / m)[:, None]
    v -= (m[:, None] * v).sum(0) / m.sum()
    ke = 0.5 * (m * (v ** 2).sum(1)).sum() / n
    if ke > 0:
        v *= math.sqrt(T / ke)
    return v


def lj_fluid(n_side: int = 64, density: float = 0.8, jitter: float = 0.1, T: float = 1.0,
             rc: float = 2.5, skin: float = 0.3, dt: float = 0.005, seed_pos: int = 1, seed_vel: int = 2) -> Scene:
    """Plain 2D LJ fluid on a jittered square lattice (benchmark config 1 at
    n_side=64: N=4096, rho=0.8, rc=2.5, skin 0.3, dt=0.005, XYPBC)."""
    n = n_side * n_side
    L = math.sqrt(n / density)
    a = L / n_side
    rp = np.random.Generator(np.random.PCG64(seed_pos))
    rv = np.random.Generator(np.random.PCG64(seed_vel))
    ij = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy"), -1).reshape(-1, 2)
    pos = (ij + 0.5) * a + rp.uniform(-jitter, jitter, size=(n, 2))
    vel = _mb_velocities(rv, n, T)
    sc = Scene(meta=dict(workload="lj_fluid", N=n, L=L, steps=1000))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", dt).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [rc], [lj_shift(rc)])
    sc.add("set_skin", skin)
    sc.add("add_particles", pos[:, 0], pos[:, 1], vel[:, 0], vel[:, 1], np.ones(n), np.ones(n),
           np.zeros(n, np.int32))
    sc.add("init_neighbor_list")
    return sc


def suspension(n_side: int = 16, radius: float = 5.0, rings: int = 6, phi: float = 0.5, E: float = 50.0,
               nu: float = 0.3, kbond: float = 100.0, T: float = 0.1, dt: float = 0.002, skin: float = 0.3,
               bonds: str = "boundary", mesh=None, center_jitter: float = 0.5,
               seeds=(3, 4, 5)) -> Scene:
    """Elastomer suspension (benchmark config 2 at n_side=16: 256 hex-ring
    disks of radius 5 with 127 vertices, E=50, nu=0.3, boundary bonds k=100,
    WCA between disks, area fraction 0.5, T=0.1, dt=0.002)."""
    nd = n_side * n_side
    L = math.sqrt(nd * math.pi * radius ** 2 / phi)
    if mesh is None:
        verts, tris = hex_disk_mesh(radius, rings, jitter=0.02, seed=seeds[0])
    else:
        verts, tris = mesh
    nv = verts.shape[0]
    rp = np.random.Generator(np.random.PCG64(seeds[1]))
    rv = np.random.Generator(np.random.PCG64(seeds[2]))
    a = L / n_side
    sc = Scene(meta=dict(workload="suspension", N=nd * nv, L=L, n_disks=nd, steps=5000))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", dt).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [WCA_RC], [1.0])
    sc.add("set_skin", skin)
    sc.add("set_kBond", kbond).add("set_youngs_modulus", E).add("set_poisson_ratio", nu)
    sc.add("set_elastomer_bonds", {"all": 0, "boundary": 1, "none": 2}[bonds])
    centers = []
    for iy in range(n_side):
        for ix in range(n_side):
            c = (np.array([ix, iy]) + 0.5) * a + rp.uniform(-center_jitter, center_jitter, size=2)
            centers.append(c)
            sc.add("add_elastomer", verts, tris, float(c[0]), float(c[1]), 0, 0, 1.0, float(nv), True)
    sc.meta["centers"] = np.array(centers)
    sc.add("init_neighbor_list")
    vel = _mb_velocities(rv, nd * nv, T)
    sc.add("set_velocities_array", vel.astype(np.float32))
    return sc


def compression(n_side: int = 8, radius: float = 5.0, rings: int = 6, phi: float = 0.5, kbond: float = 100.0,
                T: float = 0.01, dt: float = 0.002, skin: float = 0.3, wall_k: float = 100.0, strain: float = 0.02,
                steps: int = 200, E_range=(20.0, 80.0), nu_range=(0.2, 0.45), mesh=None, center_jitter: float = 0.5,
                seeds=(3, 4, 5, 10)) -> Scene:
    """Differentiable compression (benchmark config 5 at n_side=8): 64 hex-ring
    disks as the suspension, periodic in x, a fixed harmonic wall at y = 0 and
    a harmonic top wall (k_w = 100) that starts at y = L and moves down by
    strain * L over 'steps' steps; per-disk E ~ U(20, 80), nu ~ U(0.2, 0.45)
    (seed 10); dt = 0.002.  The default strain, 2 % of L in 200 steps, moves
    the wall at 5 sigma/tau, about the disks' elastic wave speed; at 10 % in
    200 steps (25 sigma/tau) the top row of disks inverts (det F <= 0) within
    about 100 steps in float and in double alike."""
    nd = n_side * n_side
    L = math.sqrt(nd * math.pi * radius ** 2 / phi)
    if mesh is None:
        verts, tris = hex_disk_mesh(radius, rings, jitter=0.02, seed=seeds[0])
    else:
        verts, tris = mesh
    nv = verts.shape[0]
    rp = np.random.Generator(np.random.PCG64(seeds[1]))
    rv = np.random.Generator(np.random.PCG64(seeds[2]))
    rm = np.random.Generator(np.random.PCG64(seeds[3]))
    a = L / n_side
    v_wall = strain * L / (steps * dt)
    Es = rm.uniform(*E_range, size=nd)
    nus = rm.uniform(*nu_range, size=nd)
    sc = Scene(meta=dict(workload="compression", N=nd * nv, L=L, n_disks=nd, steps=steps, wall_k=wall_k,
                         wall_v=v_wall, E=Es, nu=nus))
    sc.add("init", L, L).add("PBC", 1).add("set_dt", dt).add("set_numTypes", 1)
    sc.add("set_pair_potential", [1.0], [WCA_RC], [1.0])
    sc.add("set_skin", skin)
    sc.add("set_kBond", kbond).add("set_youngs_modulus", float(np.mean(E_range))).add("set_poisson_ratio", 0.3)
    sc.add("set_elastomer_bonds", 1)
    for iy in range(n_side):
        for ix in range(n_side):
            c = (np.array([ix, iy]) + 0.5) * a + rp.uniform(-center_jitter, center_jitter, size=2)
            sc.add("add_elastomer", verts, tris, float(c[0]), float(c[1]), 0, 0, 1.0, float(nv), True)
    for e in range(nd):
        sc.add("set_elastomer_material", e, float(Es[e]), float(nus[e]))
    sc.add("set_moving_wall", wall_k, L, v_wall)
    sc.add("init_neighbor_list")
    vel = _mb_velocities(rv, nd * nv, T)
    sc.add("set_velocities_array", vel.astype(np.float32))
    return sc


def large_mixed(n_side: int = 64, n_solvent: int = 1_000_000, radius: float = 5.0, rings: int = 6,
                E: float = 50.0, nu: float = 0.3, kbond: float = 100.0, T: float = 1.0, dt: float = 0.005,
                skin: float = 0.3, density: float = 0.8, center_jitter: float = 2.0,
                seeds=(3, 6, 7, 5)) -> Scene:
    """Large mixed system (benchmark config 3 at defaults: 4096 hex-ring disks
    on a 64x64 lattice plus 1,000,000 LJ solvent particles, two types:
    solvent-solvent LJ rc=2.5, every pair involving a vertex WCA)."""
    nd = n_side * n_side
    L = math.sqrt(n_solvent / density + nd * math.pi * radius ** 2)
    verts, tris = hex_disk_mesh(radius, rings, jitter=0.02, seed=seeds[0])
    nv = verts.shape[0]
    rp = np.random.Generator(np.random.PCG64(seeds[1]))
    rs = np.random.Generator(np.random.PCG64(seeds[2]))
    rv = np.random.Generator(np.random.PCG64(seeds[3]))
    a = L / n_side
    gx, gy = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="xy")
    centers = (np.stack([gx.ravel(), gy.ravel()], 1) + 0.5) * a + rp.uniform(-center_jitter, center_jitter,
                                                                           size=(nd, 2))
    # solvent lattice: enough sites that n_solvent survive the rejection
    excl_r = radius + 1.0
    avail = L * L - nd * math.pi * excl_r ** 2
    m = int(math.ceil(L / math.sqrt(avail / (n_solvent * 1.02))))
    sp = L / m
    sx, sy = np.meshgrid(np.arange(m), np.arange(m), indexing="xy")
    sites = (np.stack([sx.ravel(), sy.ravel()], 1) + 0.5) * sp
    sites += rs.uniform(-0.1, 0.1, size=sites.shape)
    # reject sites within excl_r of any disk centre (periodic), via a coarse grid
    keep = np.ones(sites.shape[0], bool)
    cell = a
    ci = np.floor(sites / cell).astype(np.int64) % n_side
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            nb = ((ci[:, 1] + dy) % n_side) * n_side + ((ci[:, 0] + dx) % n_side)
            d = sites - centers[nb]
            d -= L * np.round(d / L)
            keep &= (d ** 2).sum(1) >= excl_r ** 2
    sites = sites[keep]
    if sites.shape[0] < n_solvent:
        raise RuntimeError("solvent lattice too sparse")
    sites = sites[:n_solvent]
    sites = np.mod(sites, L)
    n_tot = nd * nv + n_solvent
    vel = _mb_velocities(rv, n_tot, T)
    sc = Scene(meta=dict(workload="large_mixed", N=n_tot, L=L, n_disks=nd, n_solvent=n_solvent, steps=1000))
    rc = 2.5
    sc.add("init", L, L).add("PBC", 2).add("set_dt", dt).add("set_numTypes", 2)
    sc.add("set_pair_potential", [1.0, 1.0, 1.0, 1.0], [rc, WCA_RC, WCA_RC, WCA_RC],
           [lj_shift(rc), 1.0, 1.0, 1.0])
    sc.add("set_skin", skin)
    sc.add("set_kBond", kbond).add("set_youngs_modulus", E).add("set_poisson_ratio", nu)
    sc.add("set_elastomer_bonds", 1)
    for c in centers:
        sc.add("add_elastomer", verts, tris, float(c[0]), float(c[1]), 1, 0, 1.0, float(nv), True)
    sc.add("add_particles", sites[:, 0], sites[:, 1], np.zeros(n_solvent), np.zeros(n_solvent),
           np.ones(n_solvent), np.ones(n_solvent), np.zeros(n_solvent, np.int32))
    sc.add("init_neighbor_list")
    sc.add("set_velocities_array", vel.astype(np.float32))
    return sc


def mixed_replica(n_total: int, density: float, T: float, seed: int, radius: float = 5.0, rings: int = 6,
                  E: float = 50.0, nu: float = 0.3, kbond: float = 100.0, dt: float = 0.005, skin: float = 0.3,
                  mesh=None) -> Scene:
    """One replica of the batched ensemble: 90 % LJ solvent by count plus
    floor(0.1 n_total / 127) hex-ring disks, two types as the large mixed
    system (solvent-solvent LJ rc = 2.5, pairs with a vertex WCA)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if mesh is None:
        verts, tris = hex_disk_mesh(radius, rings, jitter=0.02, seed=3)
    else:
        verts, tris = mesh
    nv = verts.shape[0]
    nd = int(0.1 * n_total // nv)
    n_solv = n_total - nd * nv
    L = math.sqrt(n_solv / density + nd * math.pi * radius ** 2)
    centers = np.zeros((0, 2))
    if nd:
        side = int(math.ceil(math.sqrt(nd)))
        a = L / side
        gx, gy = np.meshgrid(np.arange(side), np.arange(side), indexing="xy")
        lat = (np.stack([gx.ravel(), gy.ravel()], 1) + 0.5) * a
        centers = lat[rng.permutation(lat.shape[0])[:nd]] + rng.uniform(-0.5, 0.5, size=(nd, 2))
    excl_r = radius + 1.0
    avail = L * L - nd * math.pi * excl_r ** 2
    m = int(math.ceil(L / math.sqrt(max(avail, 1e-9) / (n_solv * 1.05))))
    while True:
        sp = L / m
        sx, sy = np.meshgrid(np.arange(m), np.arange(m), indexing="xy")
        sites = (np.stack([sx.ravel(), sy.ravel()], 1) + 0.5) * sp + rng.uniform(-0.05 * sp, 0.05 * sp,
                                                                                 size=(m * m, 2))
        keep = np.ones(sites.shape[0], bool)
        for c in centers:
            d = sites - c
            d -= L * np.round(d / L)
            keep &= (d ** 2).sum(1) >= excl_r ** 2
        if keep.sum() >= n_solv:
            break
        m += 1
    sites = np.mod(sites[keep][:n_solv], L)
    vel = _mb_velocities(rng, n_total, T)
    sc = Scene(meta=dict(workload="mixed_replica", N=n_total, L=L, n_disks=nd))
    sc.add("init", L, L).add("PBC", 2).add("set_dt", dt).add("set_numTypes", 2)
    sc.add("set_pair_potential", [1.0, 1.0, 1.0, 1.0], [2.5, WCA_RC, WCA_RC, WCA_RC], [lj_shift(2.5), 1.0, 1.0, 1.0])
    sc.add("set_skin", skin)
    sc.add("set_kBond", kbond).add("set_youngs_modulus", E).add("set_poisson_ratio", nu)
    sc.add("set_elastomer_bonds", 1)
    for c in centers:
        sc.add("add_elastomer", verts, tris, float(c[0]), float(c[1]), 1, 0, 1.0, float(nv), True)
    sc.add("add_particles", sites[:, 0], sites[:, 1], np.zeros(n_solv), np.zeros(n_solv), np.ones(n_solv),
           np.ones(n_solv), np.zeros(n_solv, np.int32))
    sc.add("init_neighbor_list")
    sc.add("set_velocities_array", vel.astype(np.float32))
    return sc


def batched_ensemble(n_replicas: int = 512, n_min: int = 500, n_max: int = 20000, seeds=(8, 9)):
    """Benchmark config 4: replica sizes log-uniform in [n_min, n_max] (seed 8),
    density U(0.6, 0.85) and temperature U(0.1, 1.5) (seed 9)."""
    rs = np.random.Generator(np.random.PCG64(seeds[0]))
    rp = np.random.Generator(np.random.PCG64(seeds[1]))
    sizes = np.rint(np.exp(rs.uniform(math.log(n_min), math.log(n_max), size=n_replicas))).astype(int)
    dens = rp.uniform(0.6, 0.85, size=n_replicas)
    temps = rp.uniform(0.1, 1.5, size=n_replicas)
    mesh = hex_disk_mesh(5.0, 6, jitter=0.02, seed=3)
    return [mixed_replica(int(sizes[r]), float(dens[r]), float(temps[r]), seed=1000 + r, mesh=mesh)
            for r in range(n_replicas)]
