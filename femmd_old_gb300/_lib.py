"""ctypes binding of libfemmd.so (the C ABI declared in include/femmd.h).

The library is the only compute path.  Importing this module without the
built library raises ImportError; there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
# FEMMD_LIBRARY names another build of the same library (same C ABI) to load
LIB_PATH = os.environ.get("FEMMD_LIBRARY") or os.path.join(PKG, "libfemmd.so")

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "CAPACITY_OVERFLOW", 3: "NONFINITE", 4: "CUDA_ERROR", 5: "TIMEOUT",
          6: "NOT_READY", 7: "UNSUPPORTED"}

P = C.c_void_p
fp, ip, dp = C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_double)
llp = C.POINTER(C.c_longlong)
i_ = C.c_int
d_ = C.c_double

# name -> (restype, argtypes); every symbol of include/femmd.h
SIGNATURES = {
    "femmd_create": (i_, [i_, C.POINTER(P)]),
    "femmd_destroy": (None, [P]),
    "femmd_last_error": (C.c_char_p, [P]),
    "femmd_version": (C.c_char_p, []),
    "femmd_init": (i_, [P, d_, d_]),
    "femmd_reset": (i_, [P]),
    "femmd_set_box": (i_, [P, d_, d_]),
    "femmd_get_box": (i_, [P, dp, dp]),
    "femmd_set_pbc": (i_, [P, i_]),
    "femmd_set_dev": (i_, [P, i_]),
    "femmd_set_dt": (i_, [P, d_]),
    "femmd_get_dt": (i_, [P, dp]),
    "femmd_set_num_types": (i_, [P, i_]),
    "femmd_set_pair_potential": (i_, [P, dp, dp, dp, i_]),
    "femmd_set_kbond": (i_, [P, d_]),
    "femmd_set_youngs_modulus": (i_, [P, d_]),
    "femmd_set_poisson_ratio": (i_, [P, d_]),
    "femmd_set_gravity": (i_, [P, d_]),
    "femmd_set_karea": (i_, [P, d_]),
    "femmd_set_skin": (i_, [P, d_]),
    "femmd_set_elastomer_material": (i_, [P, i_, d_, d_]),
    "femmd_set_moving_wall": (i_, [P, d_, d_, d_]),
    "femmd_get_wall_forces": (i_, [P, dp, dp]),
    "femmd_get_properties": (i_, [P, dp]),
    "femmd_set_property_averaging": (i_, [P, i_, i_, i_]),
    "femmd_batch_set_split": (i_, [P, i_]),
    "femmd_get_clusters": (i_, [P, dp, dp, dp]),
    "femmd_get_average_properties": (i_, [P, dp, dp, dp, C.POINTER(i_), C.POINTER(i_), C.POINTER(i_)]),
    "femmd_set_trajectory": (i_, [P, C.c_char_p, i_, i_]),
    "femmd_flush_trajectory": (i_, [P, llp]),
    "femmd_save_frame": (i_, [P, C.c_char_p, i_, i_]),
    "femmd_set_scale": (i_, [P, d_]),
    "femmd_adjoint_forward": (i_, [P, i_, i_]),
    "femmd_adjoint_backward": (i_, [P, d_, d_, fp, fp, fp, fp, dp, dp, dp, dp]),
    "femmd_adjoint_observable": (i_, [P, dp, dp]),
    "femmd_set_neighbor_capacity": (i_, [P, i_]),
    "femmd_get_neighbor_capacity": (i_, [P, ip]),
    "femmd_set_fea_law": (i_, [P, i_]),
    "femmd_set_bond_k_mode": (i_, [P, i_]),
    "femmd_set_image_mode": (i_, [P, i_]),
    "femmd_set_force_mode": (i_, [P, i_]),
    "femmd_get_force_mode": (i_, [P, ip]),
    "femmd_set_elastomer_bonds": (i_, [P, i_]),
    "femmd_add_particle": (i_, [P, d_, d_, d_, d_, d_, d_, i_]),
    "femmd_add_particles": (i_, [P, i_, dp, dp, dp, dp, dp, dp, ip]),
    "femmd_add_elastomer": (i_, [P, fp, i_, ip, i_, d_, d_, i_, i_, d_, d_, i_]),
    "femmd_create_bond": (i_, [P, i_, i_]),
    "femmd_set_velocities": (i_, [P, d_, C.c_uint64]),
    "femmd_allocate_cuda": (i_, [P]),
    "femmd_init_neighbor_list": (i_, [P]),
    "femmd_run": (i_, [P, i_]),
    "femmd_do_step": (i_, [P]),
    "femmd_calc_forces": (i_, [P]),
    "femmd_zero_stuff": (i_, [P]),
    "femmd_build_neighbor_list": (i_, [P]),
    "femmd_sync": (i_, [P]),
    "femmd_get_num_particles": (i_, [P]),
    "femmd_get_num_bonds": (i_, [P]),
    "femmd_get_num_triangles": (i_, [P]),
    "femmd_get_num_elastomers": (i_, [P]),
    "femmd_get_steps": (i_, [P]),
    "femmd_get_positions": (i_, [P, fp]),
    "femmd_get_velocities": (i_, [P, fp]),
    "femmd_get_accelerations": (i_, [P, fp]),
    "femmd_get_forces": (i_, [P, fp]),
    "femmd_get_particle_energies": (i_, [P, fp]),
    "femmd_get_masses": (i_, [P, fp]),
    "femmd_get_bonds": (i_, [P, ip, fp]),
    "femmd_get_triangles": (i_, [P, ip, fp, fp]),
    "femmd_get_exclusion_groups": (i_, [P, ip]),
    "femmd_get_reference_positions": (i_, [P, fp]),
    "femmd_get_energies": (i_, [P, dp]),
    "femmd_get_step_observables": (i_, [P, dp, i_, ip]),
    "femmd_get_grid": (i_, [P, ip, ip]),
    "femmd_get_cells": (i_, [P, ip, ip]),
    "femmd_get_neighbor_total": (i_, [P, llp]),
    "femmd_get_neighbors": (i_, [P, ip, ip]),
    "femmd_get_nn_stats": (i_, [P, dp, ip, llp]),
    "femmd_info": (i_, [P, dp]),
    "femmd_set_state": (i_, [P, fp, fp]),
    "femmd_get_state": (i_, [P, fp, fp, fp]),
    "femmd_get_stream": (P, [P]),
    "femmd_set_trace": (i_, [P, i_]),
    "femmd_get_trace": (i_, [P, C.POINTER(C.c_ulonglong), i_, ip]),
    "femmd_event_record": (i_, [P, i_]),
    "femmd_event_elapsed": (i_, [P, i_, i_, fp]),
    "femmd_set_profiling": (i_, [P, i_]),
    "femmd_test_expire_next_exchange": (i_, [P]),
    "femmd_get_profile": (i_, [P, dp, llp, dp, llp, llp]),
    "femmd_bin_cells_noalloc": (i_, [P, i_, d_, d_, i_, i_, P, P, P]),
    "femmd_batch_create": (i_, [i_, C.POINTER(P)]),
    "femmd_batch_destroy": (None, [P]),
    "femmd_batch_last_error": (C.c_char_p, [P]),
    "femmd_batch_add": (i_, [P, P, ip]),
    "femmd_batch_size": (i_, [P]),
    "femmd_batch_run": (i_, [P, i_]),
    "femmd_batch_set_launch": (i_, [P, i_, i_]),
    "femmd_batch_get_launch": (i_, [P, ip, ip, ip]),
    "femmd_batch_autotune": (i_, [P, i_, ip, ip, dp]),
    "femmd_batch_autotune_lists": (i_, [P, i_, dp, i_, dp, i_, dp, dp, dp]),
    "femmd_set_cell_factor": (i_, [P, d_]),
    "femmd_batch_event_record": (i_, [P, i_]),
    "femmd_batch_event_elapsed": (i_, [P, i_, i_, fp]),
}

_lib = None


def load(path: str | None = None):
    """Load libfemmd.so and bind every entry point (ImportError if absent)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class FemmdError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status
