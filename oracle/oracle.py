"""TEST INFRASTRUCTURE: Python face of the oracle (oracle/femmd_oracle.c) and
of the compiled reference harness (oracle/_ref/ref_harness).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may
import this module; the product never does.

``Oracle`` exposes the same method names as ``femmd_old_gb300.System`` (the
names of the reference's script surface, femmd2D/src/interface.cpp:656-696),
so a ``Scene`` replays onto either.  ``run_reference(scene)`` runs the
reference itself (compiled from its own sources, only where the reference
checkout exists) and parses what it dumps.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")

_lib = None


def build(quiet: bool = True) -> str:
    """Compile the C restatement (make -C oracle); returns the library path."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def build_reference() -> str | None:
    """Compile the reference harness from the reference sources named by
    FEMMD_REF_SRC (the checkout's femmd2D/src), when they exist."""
    src = os.environ.get("FEMMD_REF_SRC")
    if not src or not os.path.isdir(src):
        return None
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF_SRC={src}", "-j8"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "femmd_oracle.c")
        if not os.path.exists(LIB_PATH) or (os.path.exists(src) and os.path.getmtime(src) > os.path.getmtime(LIB_PATH)):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        fp, ip, dp = C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_double)
        sig = {
            "orc_create": (P, []), "orc_destroy": (None, [P]), "orc_init": (None, [P, C.c_double, C.c_double]),
            "orc_set_box": (None, [P, C.c_double, C.c_double]), "orc_set_pbc": (None, [P, C.c_int]),
            "orc_set_dt": (None, [P, C.c_double]), "orc_set_num_types": (None, [P, C.c_int]),
            "orc_set_pair_potential": (C.c_int, [P, dp, dp, dp, C.c_int]),
            "orc_set_kbond": (None, [P, C.c_double]), "orc_set_youngs_modulus": (None, [P, C.c_double]),
            "orc_set_nu": (None, [P, C.c_double]), "orc_set_skin": (None, [P, C.c_double]),
            "orc_set_threads": (None, [P, C.c_int]), "orc_set_elastomer_bonds": (None, [P, C.c_int]),
            "orc_set_modes": (None, [P, C.c_int, C.c_int, C.c_int, C.c_int]),
            "orc_add_particle": (C.c_int, [P] + [C.c_double] * 6 + [C.c_int]),
            "orc_add_particles": (C.c_int, [P, C.c_int, dp, dp, dp, dp, dp, dp, ip]),
            "orc_add_elastomer": (C.c_int, [P, fp, C.c_int, ip, C.c_int, C.c_double, C.c_double, C.c_int,
                                            C.c_int, C.c_double, C.c_double, C.c_int]),
            "orc_create_bond": (C.c_int, [P, C.c_int, C.c_int]),
            "orc_init_neighbor_list": (C.c_int, [P]), "orc_build_nn": (None, [P]),
            "orc_update_nn": (None, [P, C.c_int]), "orc_zero_stuff": (None, [P]),
            "orc_calc_forces": (None, [P]), "orc_run": (None, [P, C.c_int]), "orc_do_step": (None, [P]),
            "orc_fea_cpu1": (None, [P]), "orc_fea_only": (None, [P]),
            "orc_forces_f64": (None, [P, dp, dp, dp, dp, dp]),
            "orc_n": (C.c_int, [P]), "orc_nref": (C.c_int, [P]), "orc_nbonds": (C.c_int, [P]), "orc_ntri": (C.c_int, [P]),
            "orc_steps": (C.c_int, [P]), "orc_total_updates": (C.c_int, [P]), "orc_ncells": (C.c_int, [P]),
            "orc_grid": (None, [P, ip, ip]), "orc_nbr_total": (C.c_longlong, [P]),
            "orc_scalars": (None, [P, fp]),
            "orc_get_pos": (None, [P, fp]), "orc_get_vel": (None, [P, fp]), "orc_get_acc": (None, [P, fp]),
            "orc_get_force": (None, [P, fp]), "orc_get_refpos": (None, [P, fp]), "orc_get_mass": (None, [P, fp]),
            "orc_get_excl": (None, [P, ip]), "orc_get_bonds": (None, [P, ip, fp]),
            "orc_get_tris": (None, [P, ip, fp, fp]), "orc_get_cells": (None, [P, ip, ip]),
            "orc_get_nbrs": (None, [P, ip, ip]), "orc_set_pos": (None, [P, fp]), "orc_set_vel": (None, [P, fp]),
            "orc_logf_own": (C.c_float, [C.c_float]),
            "orc_set_elastomer_material": (C.c_int, [P, C.c_int, C.c_double, C.c_double]),
            "orc_set_moving_wall": (None, [P, C.c_double, C.c_double, C.c_double]),
            "orc_wall_forces": (None, [P, dp, dp]),
            "orc_set_gravity": (None, [P, C.c_double]), "orc_set_karea": (None, [P, C.c_double]), "orc_ncl": (C.c_int, [P]), "orc_d_init": (None, [P]), "orc_properties": (None, [P, dp]), "orc_d_set_material": (None, [C.c_int, C.c_double, C.c_double]),
            "orc_d_set_scales": (None, [C.c_double, C.c_double]), "orc_d_set_state": (None, [dp, dp]),
            "orc_d_get_state": (None, [dp, dp]), "orc_d_set_traj": (None, [dp, C.c_int]),
            "orc_d_forward": (C.c_double, [P, C.c_int, C.c_int, C.c_double, C.c_double]),
            "orc_d_backward": (None, [P, C.c_int, C.c_double, C.c_double, dp, dp, dp, dp, dp, dp, dp, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def cluster_props(pos, vel, mass, ranges, Lx, Ly):
    """FeaElements::calcClusterProps (src/feaElements.cpp:199-204) in FP64 on
    float positions: unfoldPos (:86-150) -- a cluster wider than half the box
    has its vertices beyond L/2 moved down by L, and all moved up by L again
    when their mean is negative -- then the mass-weighted centre and
    velocity; updateClustersCentroid (:162-197) -- L (atan2(-<sin>, -<cos>)
    + pi) / (2 pi) of the angles 2 pi x / L -- with each axis on its own sums
    (the reference reuses the x sums for y)."""
    pos = np.asarray(pos, np.float32)
    out = {"cm": [], "cm_vel": [], "centroid": []}
    L = (np.float32(Lx), np.float32(Ly))
    for off, n in ranges:
        p, v, m = pos[off:off + n], np.asarray(vel[off:off + n], np.float64), np.asarray(mass[off:off + n], np.float64)
        u = p.astype(np.float64)
        for a in range(2):
            if p[:, a].max() - p[:, a].min() > L[a] / np.float32(2):
                u[:, a] = np.where(p[:, a] > L[a] / np.float32(2), u[:, a] - float(L[a]), u[:, a])
                if u[:, a].sum() / n < 0:
                    u[:, a] += float(L[a])
        M = m.sum()
        out["cm"].append((m[:, None] * u).sum(0) / M)
        out["cm_vel"].append((m[:, None] * v).sum(0) / M)
        c = []
        for a in range(2):
            t = 2.0 * np.pi * p[:, a].astype(np.float64) / float(L[a])
            c.append(float(L[a]) * (np.arctan2(-np.sin(t).mean(), -np.cos(t).mean()) + np.pi) / (2.0 * np.pi))
        out["centroid"].append(c)
    return {k: np.array(v) for k, v in out.items()}


class PropertyAverages:
    """Properties::compute (src/properties.cpp:85-95) with Prop
    (src/properties.h:5-13), for values given per step: accumulate(1) adds
    val and val^2 and counts the step; at steps past step_equi that are
    multiples of step_avg, accumulate(2) sets avgval = sum / n and
    stdv = sqrt(max(sum2 / n - avgval^2, 0)), then accumulate(0) clears the
    sums and the count.  (evalClusterRdf, also called there, is out of
    scope.)"""

    def __init__(self, names, step_avg=1000, step_equi=10000):
        self.names, self.step_avg, self.step_equi = tuple(names), step_avg, step_equi
        self.count, self.windows, self.last_step = 0, 0, 0
        self.sum = dict.fromkeys(self.names, 0.0)
        self.sum2 = dict.fromkeys(self.names, 0.0)
        self.avg = dict.fromkeys(self.names, 0.0)
        self.stdv = dict.fromkeys(self.names, 0.0)

    def compute(self, step, vals):
        self.count += 1
        for k in self.names:
            self.sum[k] += vals[k]
            self.sum2[k] += vals[k] * vals[k]
        if step > self.step_equi and step % self.step_avg == 0:
            for k in self.names:
                a = self.sum[k] / self.count
                self.avg[k] = a
                self.stdv[k] = max(self.sum2[k] / self.count - a * a, 0.0) ** 0.5
                self.sum[k] = self.sum2[k] = 0.0
            self.count = 0
            self.windows += 1
            self.last_step = step


class Oracle:
    """CPU restatement of the reference timestep with the System method names.

    Modes: image_mode 0 = reference float arithmetic, 1 = exact-image
    differences; log_mode 0 = C library logf (as the reference), 1 = own log
    (as the CUDA kernels); fea_law 0 = neo-Hookean (reference CPU default),
    1 = Green strain with linear C (reference GPU kernel); bond_k_mode 0 =
    kBond (reference CPU), 1 = E/r0 (reference GPU kernel)."""

    def __init__(self, image_mode=0, log_mode=0, fea_law=0, bond_k_mode=0, threads=1):
        self.L = lib()
        self.h = self.L.orc_create()
        self.modes = [fea_law, bond_k_mode, image_mode, log_mode]
        self.L.orc_set_modes(self.h, *self.modes)
        self.L.orc_set_threads(self.h, threads)

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    # ----------------------------------------------------- setup (System.*)
    def init(self, Lx, Ly):
        self.L.orc_init(self.h, Lx, Ly)

    def PBC(self, p):
        self.L.orc_set_pbc(self.h, int(p))

    def DEV(self, d):
        pass

    def set_box(self, Lx, Ly):
        self.L.orc_set_box(self.h, Lx, Ly)

    def set_dt(self, dt):
        self.L.orc_set_dt(self.h, dt)

    def set_numTypes(self, n):
        self.L.orc_set_num_types(self.h, int(n))

    def set_pair_potential(self, eps, rc, us):
        e, r, u = (np.ascontiguousarray(x, np.float64).ravel() for x in (eps, rc, us))
        if self.L.orc_set_pair_potential(self.h, _ptr(e, C.c_double), _ptr(r, C.c_double), _ptr(u, C.c_double), e.size):
            raise ValueError("pair table smaller than numTypes^2")

    def set_kBond(self, k):
        self.L.orc_set_kbond(self.h, k)

    def set_youngs_modulus(self, E):
        self.L.orc_set_youngs_modulus(self.h, E)

    def set_poisson_ratio(self, nu):
        self.L.orc_set_nu(self.h, nu)

    def set_skin(self, s):
        self.L.orc_set_skin(self.h, s)

    def set_gravity(self, g):
        self.L.orc_set_gravity(self.h, float(g))

    def set_kArea(self, k):
        self.L.orc_set_karea(self.h, float(k))

    # File writers are outside the restated timestep: the product's frames are
    # compared with the files the reference itself wrote.
    def save_frame(self, name, fmt, append):
        pass

    def set_scale(self, scale):
        pass

    def set_elastomer_material(self, e, E, nu):
        if self.L.orc_set_elastomer_material(self.h, int(e), float(E), float(nu)):
            raise ValueError(f"no elastomer {e}")

    def set_moving_wall(self, k, y0, v):
        self.L.orc_set_moving_wall(self.h, float(k), float(y0), float(v))

    PROPERTY_NAMES = ("uKinetic", "uPotential", "uTotal", "temperature", "virial", "feaVirial", "pressure",
                      "clusterUKinetic", "clusterVirial", "molPressure")

    def properties(self, scales=False):
        out = np.zeros(13)
        self.L.orc_properties(self.h, _ptr(out, C.c_double))
        d = dict(zip(self.PROPERTY_NAMES, out[:10].tolist()))
        if scales:
            d.update(virialScale=out[10], feaVirialScale=out[11], clusterVirialScale=out[12])
        return d

    def n_elastomers(self):
        return self.L.orc_ncl(self.h)

    # ---- FP64 trajectory and adjoint (one engine per process)
    def d_init(self):
        self.L.orc_d_init(self.h)

    def d_set_material(self, e, E, nu):
        self.L.orc_d_set_material(int(e), float(E), float(nu))

    def d_set_scales(self, eps_scale, sig_scale):
        self.L.orc_d_set_scales(float(eps_scale), float(sig_scale))

    def d_set_state(self, x, v):
        x = np.ascontiguousarray(x, np.float64).ravel()
        v = np.ascontiguousarray(v, np.float64).ravel()
        self.L.orc_d_set_state(_ptr(x, C.c_double), _ptr(v, C.c_double))

    def d_get_state(self):
        n = self.N
        x = np.zeros(2 * n)
        v = np.zeros(2 * n)
        self.L.orc_d_get_state(_ptr(x, C.c_double), _ptr(v, C.c_double))
        return x.reshape(n, 2), v.reshape(n, 2)

    def d_set_traj(self, traj):
        t = np.ascontiguousarray(traj, np.float64)
        self.L.orc_d_set_traj(_ptr(t, C.c_double), t.shape[0] - 1)

    def float_trajectory(self, steps, every):
        """Positions of every step of a float run done as run(every) segments
        (run(0) then do_step, which is what run(k) does)."""
        traj = [self.positions().astype(np.float64)]
        done = 0
        while done < steps:
            k = min(every, steps - done)
            self.run(0)
            for _ in range(k):
                self.do_step()
                traj.append(self.positions().astype(np.float64))
            done += k
        return np.stack(traj)

    def d_forward(self, n0, steps, c_wall=1.0, c_fea=1.0):
        return self.L.orc_d_forward(self.h, int(n0), int(steps), float(c_wall), float(c_fea))

    def d_backward(self, n0, c_wall=1.0, c_fea=1.0, xseed=None, vseed=None):
        n = self.N
        ne = max(1, self.n_elastomers())
        gx, gv = np.zeros(2 * n), np.zeros(2 * n)
        gE, gnu = np.zeros(ne), np.zeros(ne)
        ge, gs = np.zeros(1), np.zeros(1)
        sx = None if xseed is None else np.ascontiguousarray(xseed, np.float64).ravel()
        sv = None if vseed is None else np.ascontiguousarray(vseed, np.float64).ravel()
        self.L.orc_d_backward(self.h, int(n0), float(c_wall), float(c_fea),
                              None if sx is None else _ptr(sx, C.c_double), None if sv is None else _ptr(sv, C.c_double),
                              *[_ptr(a, C.c_double) for a in (gx, gv, gE, gnu, ge, gs)])
        return dict(x0=gx.reshape(n, 2), v0=gv.reshape(n, 2), E=gE, nu=gnu, log_eps=float(ge[0]),
                    log_sigma=float(gs[0]))

    def wall_forces(self):
        t, b = C.c_double(), C.c_double()
        self.L.orc_wall_forces(self.h, C.byref(t), C.byref(b))
        return t.value, b.value

    def set_elastomer_bonds(self, mode):
        self.L.orc_set_elastomer_bonds(self.h, int(mode))

    def set_capacity(self, ppc, nbr):
        pass

    def add_particle(self, x, y, vx, vy, m, sig, typ):
        self.L.orc_add_particle(self.h, x, y, vx, vy, m, sig, int(typ))

    def add_particles(self, x, y, vx, vy, m, sig, typ):
        cols = [np.ascontiguousarray(c, np.float64) for c in (x, y, vx, vy, m, sig)]
        t = np.ascontiguousarray(typ, np.int32)
        self.L.orc_add_particles(self.h, t.size, *[_ptr(c, C.c_double) for c in cols], _ptr(t, C.c_int))

    def add_elastomer(self, verts, tris, x, y, typ, g, sig, mass, exclude):
        v = np.ascontiguousarray(verts, np.float32).ravel()
        t = np.ascontiguousarray(tris, np.int32).ravel()
        rc = self.L.orc_add_elastomer(self.h, _ptr(v, C.c_float), v.size // 2, _ptr(t, C.c_int), t.size // 3,
                                      x, y, int(typ), int(g), sig, mass, int(bool(exclude)))
        if rc:
            raise ValueError("elastomers must share one mesh and precede free particles")

    def create_bond(self, i, j):
        self.L.orc_create_bond(self.h, int(i), int(j))

    def set_velocities_array(self, v):
        v = np.ascontiguousarray(v, np.float32).ravel()
        self.L.orc_set_vel(self.h, _ptr(v, C.c_float))

    def set_positions_array(self, p):
        p = np.ascontiguousarray(p, np.float32).ravel()
        self.L.orc_set_pos(self.h, _ptr(p, C.c_float))

    def allocate_cuda(self):
        pass

    def init_neighbor_list(self):
        if self.L.orc_init_neighbor_list(self.h):
            raise ValueError("box smaller than one neighbour cell")

    # ------------------------------------------------------------- running
    def run(self, n):
        self.L.orc_run(self.h, int(n))

    def do_step(self):
        self.L.orc_do_step(self.h)

    def build_nn(self):
        self.L.orc_build_nn(self.h)

    def calc_forces(self):
        self.L.orc_zero_stuff(self.h)
        self.L.orc_calc_forces(self.h)

    def fea_cpu1(self):
        """zeroStuff, then Interactions::calcFeaForcesCPU1 alone (the
        reference's CPU Green-strain / linear-C law, with its double-precision
        force sums)."""
        self.L.orc_fea_cpu1(self.h)

    def fea_only(self):
        """zeroStuff, then the FEA forces alone by the oracle's law in use."""
        self.L.orc_fea_only(self.h)

    # ---------------------------------------- dumps (same records as the harness)
    dumps: list

    def dump_state(self):
        self.__dict__.setdefault("dumps", []).append(("state", dict(
            pos=self.positions(), vel=self.velocities(), acc=self.accelerations(), force=self.forces(),
            scalars=self.scalars(), steps=self.steps(), total_updates=self.total_updates())))

    def dump_nn(self):
        st, ids = self.cells()
        nst, lst = self.neighbors()
        self.__dict__.setdefault("dumps", []).append(("nn", dict(
            grid=self.grid(), cell_start=st, cell_ids=ids, nbr_start=nst, nbr_list=lst)))

    def dump_setup(self):
        self.__dict__.setdefault("dumps", []).append(("setup", self.setup_arrays()))

    # ------------------------------------------------------------- getters
    @property
    def N(self):
        return self.L.orc_n(self.h)

    def _get2(self, fn):
        o = np.empty((self.N, 2), np.float32)
        fn(self.h, _ptr(o, C.c_float))
        return o

    def positions(self):
        return self._get2(self.L.orc_get_pos)

    def velocities(self):
        return self._get2(self.L.orc_get_vel)

    def accelerations(self):
        return self._get2(self.L.orc_get_acc)

    def forces(self):
        return self._get2(self.L.orc_get_force)

    def masses(self):
        o = np.empty(self.N, np.float32)
        self.L.orc_get_mass(self.h, _ptr(o, C.c_float))
        return o

    def scalars(self):
        """potEnergy, virial, feaVirial, kinEneSum, vvMax, dispHi (float32)."""
        o = np.empty(6, np.float32)
        self.L.orc_scalars(self.h, _ptr(o, C.c_float))
        return o

    def steps(self):
        return self.L.orc_steps(self.h)

    def total_updates(self):
        return self.L.orc_total_updates(self.h)

    def grid(self):
        a, b = C.c_int(), C.c_int()
        self.L.orc_grid(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def cells(self):
        nc = self.L.orc_ncells(self.h)
        st = np.empty(nc + 1, np.int32)
        ids = np.empty(self.N, np.int32)
        self.L.orc_get_cells(self.h, _ptr(st, C.c_int), _ptr(ids, C.c_int))
        return st, ids

    def neighbors(self):
        tot = self.L.orc_nbr_total(self.h)
        st = np.empty(self.N + 1, np.int32)
        lst = np.empty(max(int(tot), 1), np.int32)
        self.L.orc_get_nbrs(self.h, _ptr(st, C.c_int), _ptr(lst, C.c_int))
        return st, lst[:tot]

    def setup_arrays(self):
        nb, nt = self.L.orc_nbonds(self.h), self.L.orc_ntri(self.h)
        ij = np.empty((max(nb, 1), 2), np.int32)
        r0 = np.empty(max(nb, 1), np.float32)
        self.L.orc_get_bonds(self.h, _ptr(ij, C.c_int), _ptr(r0, C.c_float))
        t = np.empty((max(nt, 1), 3), np.int32)
        xm = np.empty((max(nt, 1), 9), np.float32)
        vol = np.empty(max(nt, 1), np.float32)
        self.L.orc_get_tris(self.h, _ptr(t, C.c_int), _ptr(xm, C.c_float), _ptr(vol, C.c_float))
        excl = np.empty(self.N, np.int32)
        self.L.orc_get_excl(self.h, _ptr(excl, C.c_int))
        ref = self._get2(self.L.orc_get_refpos)
        return dict(mass=self.masses(), excl=excl, bonds=ij[:nb], r0=r0[:nb], tris=t[:nt], xm=xm[:nt],
                    refVol=vol[:nt], refPos=ref[:self.L.orc_nref(self.h)])

    def forces_f64(self):
        """FP64 forces on the current list: (f [N,2], scale [N], u_i [N],
        (U, W, sum|u|, sum|w|))."""
        n = self.N
        fx, fy, sc, ui = (np.empty(n, np.float64) for _ in range(4))
        out = np.empty(4, np.float64)
        self.L.orc_forces_f64(self.h, *[_ptr(a, C.c_double) for a in (fx, fy, sc, ui, out)])
        return np.stack([fx, fy], 1), sc, ui, out


def logf_own(x: float) -> float:
    return lib().orc_logf_own(float(x))


# ------------------------------------------------------ reference harness

def run_reference(scene, timeout=600, files=None):
    """Replay a scene on the compiled reference; returns the list of dumps
    (('state'|'nn'|'setup', dict)) in the order the scene requested them.
    With a dict 'files', the frames the scene saved (save_frame) are added to
    it as {file name: bytes}."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError("reference harness not built (make -C oracle ref)")
    with tempfile.TemporaryDirectory() as d:
        cin, cout = os.path.join(d, "cmd.bin"), os.path.join(d, "out.bin")
        with open(cin, "wb") as f:
            f.write(scene.to_bytes())
        r = subprocess.run([REF_BIN, cin, cout], capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("reference harness failed: " + r.stderr[-2000:])
        buf = open(cout, "rb").read()
        if files is not None:
            for name in sorted(os.listdir(d)):
                if name not in ("cmd.bin", "out.bin"):
                    with open(os.path.join(d, name), "rb") as f:
                        files[name] = f.read()
    return parse_dumps(buf)


def parse_dumps(buf: bytes):
    off = 0
    out = []

    def i32():
        nonlocal off
        (v,) = struct.unpack_from("<i", buf, off)
        off += 4
        return v

    def arr(dt, n):
        nonlocal off
        a = np.frombuffer(buf, dtype=dt, count=n, offset=off).copy()
        off += a.nbytes
        return a

    while True:
        tag = i32()
        if tag == 0:
            break
        if tag == 20:
            n = i32()
            d = dict(pos=arr(np.float32, 2 * n).reshape(n, 2), vel=arr(np.float32, 2 * n).reshape(n, 2),
                     acc=arr(np.float32, 2 * n).reshape(n, 2), force=arr(np.float32, 2 * n).reshape(n, 2),
                     scalars=arr(np.float32, 6))
            d["steps"] = i32()
            d["total_updates"] = i32()
            out.append(("state", d))
        elif tag == 21:
            ncx, ncy = i32(), i32()
            st = arr(np.int32, ncx * ncy + 1)
            ids = arr(np.int32, int(st[-1]))
            # every particle sits in one cell, so the occupancy total is N
            n = int(st[-1])
            nst = arr(np.int32, n + 1)
            lst = arr(np.int32, int(nst[-1]))
            out.append(("nn", dict(grid=(ncx, ncy), cell_start=st, cell_ids=ids, nbr_start=nst, nbr_list=lst)))
        elif tag == 22:
            n = i32()
            mass = arr(np.float32, n)
            excl = arr(np.int32, n)
            nb = i32()
            bonds = arr(np.int32, 2 * nb).reshape(nb, 2)
            r0 = arr(np.float32, nb)
            nt = i32()
            tris = arr(np.int32, 3 * nt).reshape(nt, 3)
            xm = arr(np.float32, 9 * nt).reshape(nt, 9)
            vol = arr(np.float32, nt)
            nref = i32()
            ref = arr(np.float32, 2 * nref).reshape(nref, 2)
            out.append(("setup", dict(mass=mass, excl=excl, bonds=bonds, r0=r0, tris=tris, xm=xm, refVol=vol,
                                      refPos=ref)))
        else:
            raise ValueError(f"bad dump tag {tag}")
    return out
