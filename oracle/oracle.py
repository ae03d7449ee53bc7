"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

The oracle (oracle/oracle.cc) restates the reference's single-partition CPU
FLIP step.  It is the checker in tests/, in __graft_entry__.smoke() and the
timed CPU baseline of bench.py; nothing else may load it.  It runs one host
thread unless set_threads() says otherwise; its results do not depend on the
thread count.  Parity status:
unpinned against the reference binary (it cannot be built here); pinned by
the known-answer tests in tests/test_oracle_kat.py.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "build" / "liboracle_fsim.so"


class orc_shape(C.Structure):
    _fields_ = [("kind", C.c_int32), ("a", C.c_float * 3), ("b", C.c_float * 3),
                ("r", C.c_float)]


class orc_seed_pass(C.Structure):
    _fields_ = [("nshapes", C.c_int32), ("shapes", orc_shape * 8), ("velocity", C.c_float * 3)]


class orc_pcg_stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("n_rows", C.c_int32), ("status", C.c_int32),
                ("pad", C.c_int32), ("rr", C.c_double), ("bb", C.c_double)]


class orc_source(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("lo2", C.c_float * 3),
                ("hi2", C.c_float * 3), ("box_period", C.c_float), ("velocity", C.c_float * 3),
                ("velocity2", C.c_float * 3), ("velocity_period", C.c_float),
                ("box_oscillating", C.c_int32), ("velocity_oscillating", C.c_int32),
                ("timed", C.c_int32), ("start_time", C.c_float), ("end_time", C.c_float)]


_P = C.c_void_p
_SIGS = {
    "orc_create": (_P, [C.POINTER(C.c_int32), C.c_int32, C.c_float, C.POINTER(C.c_float),
                        C.c_float, C.c_int32]),
    "orc_destroy": (None, [_P]),
    "orc_set_threads": (None, [C.c_int32]),
    "orc_get_threads": (C.c_int32, []),
    "orc_add_solid_cuboid": (None, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "orc_is_solid": (C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "orc_seed": (C.c_int64, [_P, C.POINTER(orc_seed_pass), C.c_int32, C.c_uint64]),
    "orc_perturb_velocities": (None, [_P, C.c_float, C.c_uint64]),
    "orc_set_particles": (None, [_P, _P, _P, _P, C.c_int64]),
    "orc_particle_count": (C.c_int64, [_P]),
    "orc_get_particles": (None, [_P, _P, _P, _P]),
    "orc_get_particle_keys": (None, [_P, _P]),
    "orc_get_leaves": (C.c_int64, [_P, _P, C.c_int64]),
    "orc_cfl": (C.c_float, [_P]),
    "orc_move_particles": (None, [_P, C.c_float]),
    "orc_delete_particles_in_solids": (None, [_P]),
    "orc_clear_grid": (None, [_P]),
    "orc_transfer_particles_to_grid": (None, [_P]),
    "orc_apply_boundary_conditions": (None, [_P]),
    "orc_save_grid_velocities": (None, [_P]),
    "orc_delete_outside_particles": (None, [_P]),
    "orc_reinitialize_phi": (None, [_P]),
    "orc_add_gravity": (None, [_P, C.c_float]),
    "orc_compute_divergence": (None, [_P]),
    "orc_pcg_solve": (C.c_int32, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                  C.POINTER(orc_pcg_stats)]),
    "orc_update_velocity_from_pressure": (None, [_P]),
    "orc_get_velocity_update": (C.c_int32, [_P]),
    "orc_extrapolate_to_boundary": (None, [_P, C.c_int32]),
    "orc_update_particles_from_grid": (None, [_P]),
    "orc_step": (C.c_int32, [_P, C.c_float, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                             C.c_double, C.POINTER(orc_pcg_stats)]),
    "orc_compute_dt": (C.c_float, [C.c_float, C.c_int32, C.c_float, C.POINTER(C.c_float)]),
    "orc_get_field": (None, [_P, C.c_int32, _P, _P]),
    "orc_get_marker": (None, [_P, _P, _P]),
    "orc_get_pressure_f64": (None, [_P, _P]),
    "orc_set_divergence": (None, [_P, _P]),
    "orc_set_marker": (None, [_P, _P]),
    "orc_seed_uniform": (C.c_float, [C.c_uint64, C.c_int32, C.c_int64, C.c_int32, C.c_int32]),
    "orc_add_source": (None, [_P, C.POINTER(orc_source)]),
    "orc_set_time": (None, [_P, C.c_double]),
    "orc_get_time": (C.c_double, [_P]),
    "orc_add_contribution_from_sources": (None, [_P, C.c_float]),
    "orc_delete_fluid_in_sources": (None, [_P, C.c_float]),
}

_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} missing: run __graft_entry__.build()")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleSim:
    """CPU restatement of one single-partition reference simulation."""

    def __init__(self, dims, boundary=0, gravity=9.8, force=(0.0, 9.8, 0.0), flip=0.95, nppc=8):
        self.lib = load()
        d = (C.c_int32 * 3)(*[int(x) for x in dims])
        f = (C.c_float * 3)(*force)
        self.dims = tuple(int(x) for x in dims)
        self.h = self.lib.orc_create(d, boundary, C.c_float(gravity), f, C.c_float(flip), nppc)

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_solid_cuboid(self, lo, hi):
        self.lib.orc_add_solid_cuboid(self.h, (C.c_int32 * 3)(*lo), (C.c_int32 * 3)(*hi))

    def is_solid(self, i, j, k) -> bool:
        return bool(self.lib.orc_is_solid(self.h, i, j, k))

    def seed(self, passes, seed=0) -> int:
        arr = (orc_seed_pass * max(1, len(passes)))()
        for i, p in enumerate(passes):
            arr[i].nshapes = len(p.shapes)
            for s, sh in enumerate(p.shapes):
                arr[i].shapes[s].kind = sh.kind
                for d in range(3):
                    arr[i].shapes[s].a[d] = sh.a[d]
                    arr[i].shapes[s].b[d] = sh.b[d]
                arr[i].shapes[s].r = sh.r
            for d in range(3):
                arr[i].velocity[d] = p.velocity[d]
        return self.lib.orc_seed(self.h, arr, len(passes), C.c_uint64(seed))

    def perturb_velocities(self, sigma, seed):
        self.lib.orc_perturb_velocities(self.h, C.c_float(sigma), C.c_uint64(seed))

    def set_particles(self, pos, vel, gvel):
        pos = np.ascontiguousarray(pos, np.float32)
        vel = np.ascontiguousarray(vel, np.float32)
        gvel = np.ascontiguousarray(gvel, np.float32)
        self.lib.orc_set_particles(self.h, _ptr(pos), _ptr(vel), _ptr(gvel), pos.shape[0])

    def particle_count(self) -> int:
        return self.lib.orc_particle_count(self.h)

    def particles(self):
        n = self.particle_count()
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        gvel = np.empty((n, 3), np.float32)
        self.lib.orc_get_particles(self.h, _ptr(pos), _ptr(vel), _ptr(gvel))
        return pos, vel, gvel

    def keys(self):
        k = np.empty(self.particle_count(), np.uint32)
        self.lib.orc_get_particle_keys(self.h, _ptr(k))
        return k

    def leaves(self):
        n = self.lib.orc_get_leaves(self.h, None, 0)
        out = np.empty((max(1, n), 3), np.int32)
        self.lib.orc_get_leaves(self.h, _ptr(out), n)
        return out[:n].copy()

    # stages
    def cfl(self):
        return self.lib.orc_cfl(self.h)

    def move_particles(self, dt):
        self.lib.orc_move_particles(self.h, C.c_float(dt))

    def clear_grid(self):
        self.lib.orc_clear_grid(self.h)

    def transfer_particles_to_grid(self):
        self.lib.orc_transfer_particles_to_grid(self.h)

    def apply_boundary_conditions(self):
        self.lib.orc_apply_boundary_conditions(self.h)

    def save_grid_velocities(self):
        self.lib.orc_save_grid_velocities(self.h)

    def delete_outside_particles(self):
        self.lib.orc_delete_outside_particles(self.h)

    def reinitialize_phi(self):
        self.lib.orc_reinitialize_phi(self.h)

    def add_gravity(self, dt):
        self.lib.orc_add_gravity(self.h, C.c_float(dt))

    def compute_divergence(self):
        self.lib.orc_compute_divergence(self.h)

    def pcg_solve(self, mode=0, precision=0, max_iterations=1500, threshold=0.0, tol=1e-5):
        st = orc_pcg_stats()
        self.lib.orc_pcg_solve(self.h, mode, precision, max_iterations, threshold, tol,
                               C.byref(st))
        return st

    def update_velocity_from_pressure(self):
        self.lib.orc_update_velocity_from_pressure(self.h)

    def get_velocity_update(self) -> int:
        return self.lib.orc_get_velocity_update(self.h)

    def extrapolate_to_boundary(self, field):
        self.lib.orc_extrapolate_to_boundary(self.h, field)

    def update_particles_from_grid(self):
        self.lib.orc_update_particles_from_grid(self.h)

    def add_source(self, src):
        """src: any structure with the fsim_source / orc_source fields."""
        o = orc_source()
        C.memmove(C.byref(o), C.byref(src), C.sizeof(orc_source))
        self.lib.orc_add_source(self.h, C.byref(o))

    @property
    def time(self):
        return self.lib.orc_get_time(self.h)

    @time.setter
    def time(self, t):
        self.lib.orc_set_time(self.h, C.c_double(t))

    def add_contribution_from_sources(self, t):
        self.lib.orc_add_contribution_from_sources(self.h, C.c_float(t))

    def delete_fluid_in_sources(self, t):
        self.lib.orc_delete_fluid_in_sources(self.h, C.c_float(t))

    def seed_scene(self, scene, seed=0):
        """Seeds the passes of a parsed fsim_scene."""
        n = max(1, scene.npasses)
        arr = (orc_seed_pass * n)()
        C.memmove(arr, scene.passes, C.sizeof(orc_seed_pass) * scene.npasses)
        return self.lib.orc_seed(self.h, arr, scene.npasses, C.c_uint64(seed))

    def step(self, dt, mode=0, precision=0, max_iterations=1500, threshold=0.0, tol=1e-5):
        st = orc_pcg_stats()
        self.lib.orc_step(self.h, C.c_float(dt), mode, precision, max_iterations, threshold, tol,
                          C.byref(st))
        return st

    # downloads (dense over voxels [-1, N]^3)
    def _shape(self):
        return tuple(d + 2 for d in self.dims)

    def field(self, which):
        vec = which <= 2
        out = np.empty(self._shape() + ((3,) if vec else ()), np.float32)
        act = np.empty(self._shape(), np.uint8)
        self.lib.orc_get_field(self.h, which, _ptr(out), _ptr(act))
        return out, act

    def marker(self):
        out = np.empty(self._shape(), np.int32)
        act = np.empty(self._shape(), np.uint8)
        self.lib.orc_get_marker(self.h, _ptr(out), _ptr(act))
        return out, act

    def pressure_f64(self):
        out = np.empty(self._shape(), np.float64)
        self.lib.orc_get_pressure_f64(self.h, _ptr(out))
        return out

    def set_divergence(self, div):
        div = np.ascontiguousarray(div, np.float32)
        self.lib.orc_set_divergence(self.h, _ptr(div))

    def set_marker(self, marker):
        marker = np.ascontiguousarray(marker, np.int32)
        self.lib.orc_set_marker(self.h, _ptr(marker))


def set_threads(n: int) -> None:
    """Host threads of the oracle's thread-count-independent loops (results
    are bit-identical for any n); process-wide."""
    load().orc_set_threads(int(n))


def get_threads() -> int:
    return int(load().orc_get_threads())


def compute_dt(inv_speed, cfl, frame_step, time_in_frame):
    t = C.c_float(time_in_frame)
    dt = load().orc_compute_dt(C.c_float(inv_speed), cfl, C.c_float(frame_step), C.byref(t))
    return dt, t.value


def seed_uniform(seed, pass_, cell, draw, d):
    return load().orc_seed_uniform(C.c_uint64(seed), pass_, cell, draw, d)
