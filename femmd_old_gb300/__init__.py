"""femmd_old_gb300 -- GB300-native femmd2D timestep.

``System`` mirrors the reference's script object (femmd2D/src/interface.cpp:
656-696): the same method names, argument meaning and call order
(``init``, ``PBC``, ``set_dt``, ``set_pair_potential``, ``set_kBond``,
``set_youngs_modulus``, ``add_elastomer``, ``add_particle``,
``allocate_cuda``, ``init_neighbor_list``, ``run``, ``info``, ...), plus the
C++-only knobs of the reference classes and the getters the C ABI adds.
Every call goes through libfemmd.so (include/femmd.h); failures raise
``FemmdError`` with the library's status and message.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FemmdError

__all__ = ["System", "Batch", "FemmdError", "read_file", "FILECONTENT", "DEV", "PBCTYPE", "lib"]

DEV = {"CPU": 0, "GPU": 1}
PBCTYPE = {"NOPBC": 0, "XPBC": 1, "XYPBC": 2}
FILECONTENT = {"INT": 0, "FLOAT": 1, "TEXT": 2}


def lib():
    return _lib.load()


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def read_file(name: str, kind: int):
    """read_file(name, FILECONTENT.FLOAT|INT|TEXT) of the reference
    (femmd2D/src/interface.cpp:135-195): whitespace-separated numbers as a
    float32 or int32 array, or the text."""
    with open(name) as fh:
        txt = fh.read()
    if kind == FILECONTENT["TEXT"]:
        return txt
    return np.array(txt.split(), dtype=np.float32 if kind == FILECONTENT["FLOAT"] else np.int32)


class System:
    """One simulated system on one GPU (a femmd_ctx)."""

    def __init__(self, device: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        self._check(self._L.femmd_create(int(device), C.byref(h)), None)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.femmd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, h=0):
        if st != 0:
            msg = self._L.femmd_last_error(self._h if h == 0 else h)
            raise FemmdError(st, msg.decode() if msg else "")

    def _call(self, name, *args):
        self._check(getattr(self._L, name)(self._h, *args))

    # ------------------------------------------------ System.* (reference)
    def init(self, Lx, Ly):
        self._call("femmd_init", float(Lx), float(Ly))

    def reset(self):
        self._call("femmd_reset")

    def set_box(self, Lx, Ly):
        self._call("femmd_set_box", float(Lx), float(Ly))

    def get_box(self):
        a, b = C.c_double(), C.c_double()
        self._call("femmd_get_box", C.byref(a), C.byref(b))
        return {"x": a.value, "y": b.value}

    def PBC(self, p):
        self._call("femmd_set_pbc", int(p))

    def DEV(self, d):
        self._call("femmd_set_dev", int(d))

    def set_dt(self, dt):
        self._call("femmd_set_dt", float(dt))

    def get_dt(self):
        v = C.c_double()
        self._call("femmd_get_dt", C.byref(v))
        return v.value

    def useNN(self, x):
        # the reference's System.useNN sets dt (femmd2D/src/interface.cpp:429-434)
        self.set_dt(x)

    def set_numTypes(self, n):
        self._call("femmd_set_num_types", int(n))

    def set_pair_potential(self, eps, rc, ushift):
        e, r, u = (np.ascontiguousarray(x, np.float64).ravel() for x in (eps, rc, ushift))
        self._call("femmd_set_pair_potential", _d(e), _d(r), _d(u), int(e.size))

    def set_kBond(self, k):
        self._call("femmd_set_kbond", float(k))

    def set_youngs_modulus(self, E):
        self._call("femmd_set_youngs_modulus", float(E))

    def set_gravity(self, g):
        self._call("femmd_set_gravity", float(g))

    def set_kArea(self, k):
        self._call("femmd_set_karea", float(k))

    def add_particle(self, x, y, vx, vy, m, sig, typ):
        self._call("femmd_add_particle", float(x), float(y), float(vx), float(vy), float(m), float(sig), int(typ))

    def add_elastomer(self, verts, tris, x, y, typ, g, sig, mass, exclude):
        v = np.ascontiguousarray(verts, np.float32).ravel()
        t = np.ascontiguousarray(tris, np.int32).ravel()
        self._call("femmd_add_elastomer", _f(v), int(v.size // 2), _i(t), int(t.size // 3), float(x), float(y),
                   int(typ), int(g), float(sig), float(mass), int(bool(exclude)))

    def set_velocities(self, v0, seed=0):
        self._call("femmd_set_velocities", float(v0), C.c_uint64(int(seed)))

    def allocate_cuda(self):
        self._call("femmd_allocate_cuda")

    def init_neighbor_list(self):
        self._call("femmd_init_neighbor_list")

    def run(self, n):
        self._call("femmd_run", int(n))

    def info(self):
        o = np.zeros(9)
        self._check(self._L.femmd_info(self._h, _d(o)))
        return {"N": int(o[0]), "nelastomers": int(o[1]), "nbonds": int(o[2]), "ntrigs": int(o[3]), "dt": o[4],
                "kBonds": o[5], "kArea": o[6], "E": o[7], "box": self.get_box()}

    # ------------------------------------------- C++-only knobs / c_* calls
    def set_poisson_ratio(self, nu):
        self._call("femmd_set_poisson_ratio", float(nu))

    def set_elastomer_material(self, e, E, nu):
        self._call("femmd_set_elastomer_material", int(e), float(E), float(nu))

    def set_moving_wall(self, k, y0, v):
        self._call("femmd_set_moving_wall", float(k), float(y0), float(v))

    def wall_forces(self):
        t, b = C.c_double(), C.c_double()
        self._call("femmd_get_wall_forces", C.byref(t), C.byref(b))
        return t.value, b.value

    # layouts of femmd_set_trajectory / femmd_save_frame
    FRAME_DUMP, FRAME_XYZ, FRAME_VTK, FRAME_VTF, FRAME_CLUSTER_VTF, FRAME_VTU, FRAME_VTU_BIN = range(7)

    def set_trajectory(self, path, every, fmt=0):
        """Frames every 'every' steps of run(), in layout fmt (FRAME_*)."""
        self._call("femmd_set_trajectory", None if path is None else str(path).encode(), int(every), int(fmt))

    def flush_trajectory(self):
        n = C.c_longlong()
        self._call("femmd_flush_trajectory", C.byref(n))
        return n.value

    def save_frame(self, path, fmt, append=0):
        """The current state written now in layout fmt; append 0 starts the file anew."""
        self._call("femmd_save_frame", str(path).encode(), int(fmt), int(append))

    # the reference's writers by their script names (interface.cpp:664-668)
    def save_vtk(self, name):
        self.save_frame(name, self.FRAME_VTK)

    def save_vtf(self, name, flag):
        self.save_frame(name, self.FRAME_VTF, flag)

    def save_cluster_vtf(self, name, flag):
        self.save_frame(name, self.FRAME_CLUSTER_VTF, flag)

    def save_cluster_xyz(self, name, flag):
        self.save_frame(name, self.FRAME_DUMP, flag)

    def save_xyz(self, name, flag):
        self.save_frame(name, self.FRAME_XYZ, flag)

    def save_vtk_xml(self, name, binary=False):
        self.save_frame(name, self.FRAME_VTU_BIN if binary else self.FRAME_VTU)

    def set_scale(self, scale):
        self._call("femmd_set_scale", float(scale))

    PROPERTY_NAMES = ("uKinetic", "uPotential", "uTotal", "temperature", "virial", "feaVirial", "pressure",
                      "clusterUKinetic", "clusterVirial", "molPressure")

    def properties(self):
        """Properties::evaluate at the current state (dict by the reference's names)."""
        out = (C.c_double * 10)()
        self._call("femmd_get_properties", out)
        return dict(zip(self.PROPERTY_NAMES, list(out)))

    def clusters(self):
        """FeaElements::calcClusterProps: per elastomer the centre of mass and
        its velocity (unfolded) and the periodic centroid, each (n, 2)."""
        n = int(self.info()["nelastomers"])
        cm, cv, ce = (np.zeros((max(n, 1), 2)) for _ in range(3))
        if n:
            self._call("femmd_get_clusters", _d(cm), _d(cv), _d(ce))
        return dict(cm=cm[:n], cm_vel=cv[:n], centroid=ce[:n])

    def set_property_averaging(self, on=True, step_avg=1000, step_equi=10000):
        """Properties::compute after every step: sums of the properties, closed
        into an average and standard deviation at steps past step_equi that
        are multiples of step_avg."""
        self._call("femmd_set_property_averaging", int(bool(on)), int(step_avg), int(step_equi))

    def average_properties(self):
        """The last closed window (avg, stdv), the last step's values (val),
        the steps in the open window (count), the windows closed so far and
        the step that closed the last one."""
        a, sd, v = (C.c_double * 10)(), (C.c_double * 10)(), (C.c_double * 10)()
        n, w, ls = C.c_int(), C.c_int(), C.c_int()
        self._call("femmd_get_average_properties", a, sd, v, C.byref(n), C.byref(w), C.byref(ls))
        names = self.PROPERTY_NAMES
        return dict(avg=dict(zip(names, list(a))), stdv=dict(zip(names, list(sd))), val=dict(zip(names, list(v))),
                    count=n.value, windows=w.value, last_step=ls.value)

    def adjoint_forward(self, steps, every=20):
        self._call("femmd_adjoint_forward", int(steps), int(every))

    def adjoint_observable(self):
        ws, fe = C.c_double(), C.c_double()
        self._call("femmd_adjoint_observable", C.byref(ws), C.byref(fe))
        return ws.value, fe.value

    def adjoint_backward(self, c_wall=1.0, c_fea=1.0, xbar_final=None, vbar_final=None):
        """Gradients of c_wall * wall stress + c_fea * FEA energy (+ <xbar_final,
        x_N> + <vbar_final, v_N>) after adjoint_forward: dict with x0, v0
        (N x 2 float32), E, nu (per elastomer), log_eps, log_sigma."""
        n = self.N
        ne = self._L.femmd_get_num_elastomers(self._h)
        fp = C.POINTER(C.c_float)
        dp = C.POINTER(C.c_double)

        def seed(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, np.float32).reshape(n, 2)
            return a

        xs, vs = seed(xbar_final), seed(vbar_final)
        gx = np.zeros((n, 2), np.float32)
        gv = np.zeros((n, 2), np.float32)
        gE = np.zeros(max(ne, 1), np.float64)
        gnu = np.zeros(max(ne, 1), np.float64)
        ge, gs = C.c_double(), C.c_double()
        self._call("femmd_adjoint_backward", float(c_wall), float(c_fea),
                   xs.ctypes.data_as(fp) if xs is not None else None,
                   vs.ctypes.data_as(fp) if vs is not None else None,
                   gx.ctypes.data_as(fp), gv.ctypes.data_as(fp), gE.ctypes.data_as(dp), gnu.ctypes.data_as(dp),
                   C.byref(ge), C.byref(gs))
        return dict(x0=gx, v0=gv, E=gE[:ne], nu=gnu[:ne], log_eps=ge.value, log_sigma=gs.value)

    def set_cell_factor(self, f):
        self._call("femmd_set_cell_factor", float(f))

    def set_skin(self, s):
        self._call("femmd_set_skin", float(s))

    def set_fea_law(self, law):
        self._call("femmd_set_fea_law", int(law))

    def set_bond_k_mode(self, m):
        self._call("femmd_set_bond_k_mode", int(m))

    def set_image_mode(self, m):
        self._call("femmd_set_image_mode", int(m))

    def set_force_mode(self, m):
        """0: reference-exact arithmetic and list order; 1: fast (same sets,
        forces within 1e-5 of FP64, free particles stored in cell order)."""
        self._call("femmd_set_force_mode", int(m))

    def force_mode(self):
        m = C.c_int()
        self._call("femmd_get_force_mode", C.byref(m))
        return m.value

    def set_elastomer_bonds(self, m):
        self._call("femmd_set_elastomer_bonds", int(m))

    def set_capacity(self, ppc, nbr):
        """The reference sizes its fixed cell/list arrays here; here cells are
        CSR and lists grow on overflow, so nothing is needed."""

    def add_particles(self, x, y, vx, vy, m, sig, typ):
        cols = [np.ascontiguousarray(c, np.float64) for c in (x, y, vx, vy, m, sig)]
        t = np.ascontiguousarray(typ, np.int32)
        self._call("femmd_add_particles", int(t.size), *[_d(c) for c in cols], _i(t))

    def create_bond(self, i, j):
        self._call("femmd_create_bond", int(i), int(j))

    def do_step(self):
        self._call("femmd_do_step")

    def zero_stuff(self):
        self._call("femmd_zero_stuff")

    def calc_forces(self):
        """c_zeroStuff + c_calcForces on the current positions and lists."""
        self._call("femmd_zero_stuff")
        self._call("femmd_calc_forces")

    def set_neighbor_capacity(self, cap):
        self._call("femmd_set_neighbor_capacity", int(cap))

    def neighbor_capacity(self):
        c = C.c_int()
        self._call("femmd_get_neighbor_capacity", C.byref(c))
        return c.value

    def build_nn(self):
        self._call("femmd_build_neighbor_list")

    def sync(self):
        self._call("femmd_sync")

    def set_velocities_array(self, v):
        v = np.ascontiguousarray(v, np.float32).ravel()
        self._call("femmd_set_state", None, _f(v))

    def set_positions_array(self, p):
        p = np.ascontiguousarray(p, np.float32).ravel()
        self._call("femmd_set_state", _f(p), None)

    def set_profiling(self, on):
        self._call("femmd_set_profiling", int(bool(on)))

    def test_expire_next_exchange(self):
        """Tests of the failure path: the next small-system run's first
        grid-wide exchange is left to time out (run() raises FEMMD_TIMEOUT)."""
        self._call("femmd_test_expire_next_exchange")

    def counts(self):
        return dict(bonds=self._L.femmd_get_num_bonds(self._h), triangles=self._L.femmd_get_num_triangles(self._h),
                    elastomers=self._L.femmd_get_num_elastomers(self._h))

    def profile(self):
        fms, rms = C.c_double(), C.c_double()
        fl, rb, kl = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self._call("femmd_get_profile", C.byref(fms), C.byref(fl), C.byref(rms), C.byref(rb), C.byref(kl))
        return dict(force_ms=fms.value, force_launches=fl.value, kernel_launches=kl.value)

    # --------------------------------------------------------------- getters
    @property
    def N(self):
        return self._L.femmd_get_num_particles(self._h)

    def _get2(self, name):
        o = np.empty((self.N, 2), np.float32)
        self._call(name, _f(o))
        return o

    def positions(self):
        return self._get2("femmd_get_positions")

    def velocities(self):
        return self._get2("femmd_get_velocities")

    def accelerations(self):
        return self._get2("femmd_get_accelerations")

    def forces(self):
        return self._get2("femmd_get_forces")

    def particle_energies(self):
        o = np.empty(self.N, np.float32)
        self._call("femmd_get_particle_energies", _f(o))
        return o

    def masses(self):
        o = np.empty(self.N, np.float32)
        self._call("femmd_get_masses", _f(o))
        return o

    def steps(self):
        return self._L.femmd_get_steps(self._h)

    def energies(self):
        """FP64 (U, W, sum m v^2, max v^2, dispHi, totalUpdates) of the last evaluation."""
        o = np.zeros(6)
        self._call("femmd_get_energies", _d(o))
        return o

    def step_observables(self):
        rows = C.c_int()
        self._call("femmd_get_step_observables", None, 0, C.byref(rows))
        o = np.zeros((rows.value, 6))
        if rows.value:
            self._call("femmd_get_step_observables", _d(o), rows.value, C.byref(rows))
        return o

    def grid(self):
        a, b = C.c_int(), C.c_int()
        self._call("femmd_get_grid", C.byref(a), C.byref(b))
        return a.value, b.value

    def cells(self):
        nx, ny = self.grid()
        st = np.empty(nx * ny + 1, np.int32)
        ids = np.empty(max(self.N, 1), np.int32)
        self._call("femmd_get_cells", _i(st), _i(ids))
        return st, ids[:self.N]

    def neighbors(self):
        tot = C.c_longlong()
        self._call("femmd_get_neighbor_total", C.byref(tot))
        st = np.empty(self.N + 1, np.int32)
        lst = np.empty(max(tot.value, 1), np.int32)
        self._call("femmd_get_neighbors", _i(st), _i(lst))
        return st, lst[:st[-1]]

    def nn_stats(self):
        m, mx, b = C.c_double(), C.c_int(), C.c_longlong()
        self._call("femmd_get_nn_stats", C.byref(m), C.byref(mx), C.byref(b))
        return dict(mean_neighbors=m.value, max_neighbors=mx.value, builds=b.value)

    def total_updates(self):
        return int(self.energies()[5])

    def setup_arrays(self):
        nb = self._L.femmd_get_num_bonds(self._h)
        nt = self._L.femmd_get_num_triangles(self._h)
        ij = np.empty((max(nb, 1), 2), np.int32)
        r0 = np.empty(max(nb, 1), np.float32)
        self._call("femmd_get_bonds", _i(ij), _f(r0))
        t = np.empty((max(nt, 1), 3), np.int32)
        xm = np.empty((max(nt, 1), 9), np.float32)
        vol = np.empty(max(nt, 1), np.float32)
        self._call("femmd_get_triangles", _i(t), _f(xm), _f(vol))
        excl = np.empty(self.N, np.int32)
        self._call("femmd_get_exclusion_groups", _i(excl))
        ref = np.empty((self.N, 2), np.float32)
        self._call("femmd_get_reference_positions", _f(ref))
        return dict(mass=self.masses(), excl=excl, bonds=ij[:nb], r0=r0[:nb], tris=t[:nt], xm=xm[:nt],
                    refVol=vol[:nt], refPos=ref[:self._vertex_count()])

    def _vertex_count(self):
        # elastomer vertices come first (reference constraint): 1 + highest triangle vertex
        ncl = self._L.femmd_get_num_elastomers(self._h)
        if ncl == 0:
            return 0
        nt = self._L.femmd_get_num_triangles(self._h)
        t = np.empty((max(nt, 1), 3), np.int32)
        self._call("femmd_get_triangles", _i(t), None, None)
        return int(t[:nt].max()) + 1 if nt else 0

    def get_state(self):
        n = self.N
        p, v, a = (np.empty((n, 2), np.float32) for _ in range(3))
        self._call("femmd_get_state", _f(p), _f(v), _f(a))
        return p, v, a

    def set_state(self, pos=None, vel=None):
        p = None if pos is None else np.ascontiguousarray(pos, np.float32).ravel()
        v = None if vel is None else np.ascontiguousarray(vel, np.float32).ravel()
        self._call("femmd_set_state", None if p is None else _f(p), None if v is None else _f(v))

    def set_trace(self, on):
        self._call("femmd_set_trace", int(bool(on)))

    def trace(self):
        """Per-step device timestamps (ns): tri start/end, step start/end, rebuild start/end."""
        rows = C.c_int()
        self._call("femmd_get_trace", None, 0, C.byref(rows))
        o = np.zeros((rows.value, 6), np.uint64)
        if rows.value:
            self._call("femmd_get_trace", o.ctypes.data_as(C.POINTER(C.c_ulonglong)), rows.value, C.byref(rows))
        return o

    def event_record(self, slot):
        self._call("femmd_event_record", int(slot))

    def event_elapsed_ms(self, a, b):
        ms = C.c_float()
        self._call("femmd_event_elapsed", int(a), int(b), C.byref(ms))
        return ms.value

    def set_state_ptr(self, pos_ptr, vel_ptr):
        """set_state from raw host pointers (e.g. pinned buffers)."""
        self._call("femmd_set_state", C.cast(pos_ptr, C.POINTER(C.c_float)), C.cast(vel_ptr, C.POINTER(C.c_float)))

    def get_state_ptr(self, pos_ptr, vel_ptr, acc_ptr=None):
        cast = lambda p: None if p is None else C.cast(p, C.POINTER(C.c_float))  # noqa: E731
        self._call("femmd_get_state", cast(pos_ptr), cast(vel_ptr), cast(acc_ptr))

    def stream_handle(self):
        return self._L.femmd_get_stream(self._h)

    # ------------------------------------------------- dump records (tests)
    def dump_state(self):
        e = self.energies()
        self.__dict__.setdefault("dumps", []).append(("state", dict(
            pos=self.positions(), vel=self.velocities(), acc=self.accelerations(), force=self.forces(),
            energies=e, steps=self.steps(), total_updates=int(e[5]))))

    def dump_nn(self):
        st, ids = self.cells()
        nst, lst = self.neighbors()
        self.__dict__.setdefault("dumps", []).append(("nn", dict(
            grid=self.grid(), cell_start=st, cell_ids=ids, nbr_start=nst, nbr_list=lst)))

    def dump_setup(self):
        self.__dict__.setdefault("dumps", []).append(("setup", self.setup_arrays()))


class Batch:
    """Many Systems advanced together in one persistent launch
    (femmd_batch_*): run(n) does System.run(n) on every replica, with the same
    results as running them one by one."""

    def __init__(self, device: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        st = self._L.femmd_batch_create(int(device), C.byref(h))
        if st:
            raise FemmdError(st, "batch create")
        self._h = h
        self.systems = []

    def close(self):
        if getattr(self, "_h", None):
            self._L.femmd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        st = getattr(self._L, name)(self._h, *args)
        if st != 0:
            msg = self._L.femmd_batch_last_error(self._h)
            raise FemmdError(st, msg.decode() if msg else "")

    def add(self, system: "System") -> int:
        idx = C.c_int()
        self._call("femmd_batch_add", system._h, C.byref(idx))
        self.systems.append(system)
        return idx.value

    def __len__(self):
        return self._L.femmd_batch_size(self._h)

    def run(self, n):
        self._call("femmd_batch_run", int(n))

    def set_launch(self, threads, ctas_per_sm):
        self._call("femmd_batch_set_launch", int(threads), int(ctas_per_sm))

    def set_split(self, on=True):
        """Run replicas heavier than a CTA's average share on CTA pairs."""
        self._call("femmd_batch_set_split", int(bool(on)))

    def launch(self):
        t, c, k = C.c_int(), C.c_int(), C.c_int()
        self._call("femmd_batch_get_launch", C.byref(t), C.byref(c), C.byref(k))
        return dict(threads=t.value, ctas_per_sm=c.value, ctas=k.value)

    def autotune(self, trial_steps=10):
        t, c, ms = C.c_int(), C.c_int(), C.c_double()
        self._call("femmd_batch_autotune", int(trial_steps), C.byref(t), C.byref(c), C.byref(ms))
        return dict(threads=t.value, ctas_per_sm=c.value, trial_ms=ms.value)

    def autotune_lists(self, trial_steps=20, skins=(0.3, 0.45, 0.6), factors=(1.0,)):
        """Opt-in: pick the skin (rebuild cadence) and cell factor by timing."""
        sk = (C.c_double * len(skins))(*skins)
        fa = (C.c_double * len(factors))(*factors)
        bs, bf, ms = C.c_double(), C.c_double(), C.c_double()
        self._call("femmd_batch_autotune_lists", int(trial_steps), sk, len(skins), fa, len(factors),
                   C.byref(bs), C.byref(bf), C.byref(ms))
        return dict(skin=bs.value, cell_factor=bf.value, trial_ms=ms.value)

    def event_record(self, slot):
        self._call("femmd_batch_event_record", int(slot))

    def event_elapsed_ms(self, a, b):
        ms = C.c_float()
        self._call("femmd_batch_event_elapsed", int(a), int(b), C.byref(ms))
        return ms.value
