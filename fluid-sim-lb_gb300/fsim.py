"""Python binding of the C ABI in include/fsim.h (ctypes; numpy buffers).

``Simulation`` wraps one fsim_t handle and mirrors the stage methods of the
reference's ``FlipSimulation`` (schinmayee/fluid-sim-lb,
common/flip_simulation.h) plus ``PCGDriver::Solve`` (common/solver_driver.h).
Every call goes through libfsim.so; there is no Python or CPU fallback --
loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import weakref
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libfsim.so"

OK, ERR_INVALID, ERR_CUDA, ERR_CAPACITY, ERR_NOT_CONVERGED, ERR_BREAKDOWN, ERR_STATE, \
    ERR_NO_DEVICE, ERR_TIMEOUT = range(9)
AIR, FLUID, SOLID = 0, 1, 2
BOUNDARY_BOX, BOUNDARY_TANK = 0, 1
SHAPE_CUBOID, SHAPE_SPHERE, SHAPE_POOL = 0, 1, 2
PCG_ABSOLUTE, PCG_RELATIVE, PCG_FIXED = 0, 1, 2
PREC_FP32, PREC_MIXED, PREC_FP64 = 0, 1, 2
FIELD_VELOCITY, FIELD_VELOCITY_UPDATE, FIELD_WEIGHT, FIELD_DIVERGENCE, FIELD_PRESSURE, \
    FIELD_PHI = range(6)


class fsim_config(C.Structure):
    _fields_ = [("global_dims", C.c_int32 * 3), ("boundary", C.c_int32),
                ("gravity", C.c_float), ("force", C.c_float * 3), ("flip_factor", C.c_float),
                ("nparticles_per_cell", C.c_int32), ("max_particles", C.c_int64),
                ("device", C.c_int32)]


class fsim_shape(C.Structure):
    _fields_ = [("kind", C.c_int32), ("a", C.c_float * 3), ("b", C.c_float * 3),
                ("r", C.c_float)]


class fsim_seed_pass(C.Structure):
    _fields_ = [("nshapes", C.c_int32), ("shapes", fsim_shape * 8), ("velocity", C.c_float * 3)]


class fsim_pcg_params(C.Structure):
    _fields_ = [("mode", C.c_int32), ("precision", C.c_int32), ("max_iterations", C.c_int32),
                ("max_refinements", C.c_int32), ("threshold", C.c_double),
                ("tolerance", C.c_double), ("inner_tolerance", C.c_double)]


class fsim_pcg_stats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("n_rows", C.c_int32),
                ("status", C.c_int32), ("rr", C.c_double), ("bb", C.c_double),
                ("loop_ms", C.c_double)]


class fsim_step_stats(C.Structure):
    _fields_ = [("particles", C.c_int64), ("particle_leaves", C.c_int32),
                ("grid_leaves", C.c_int32), ("pcg", fsim_pcg_stats),
                ("next_inv_speed", C.c_float)]


MAX_SOURCES = 16
SCENE_MAX_SOLIDS = 32


class fsim_run_stats(C.Structure):
    _fields_ = [("frames", C.c_int32), ("steps", C.c_int32), ("pcg_iterations", C.c_int64),
                ("time", C.c_double), ("last_dt", C.c_float)]


FRAME_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int32, C.c_void_p)


class fsim_source(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("lo2", C.c_float * 3),
                ("hi2", C.c_float * 3), ("box_period", C.c_float), ("velocity", C.c_float * 3),
                ("velocity2", C.c_float * 3), ("velocity_period", C.c_float),
                ("box_oscillating", C.c_int32), ("velocity_oscillating", C.c_int32),
                ("timed", C.c_int32), ("start_time", C.c_float), ("end_time", C.c_float)]


class fsim_scene(C.Structure):
    _fields_ = [("fluid", C.c_int32), ("boundary", C.c_int32), ("gravity", C.c_float),
                ("force", C.c_float * 3), ("nsolids", C.c_int32),
                ("solid_lo", (C.c_int32 * 3) * SCENE_MAX_SOLIDS),
                ("solid_hi", (C.c_int32 * 3) * SCENE_MAX_SOLIDS),
                ("npasses", C.c_int32), ("passes", fsim_seed_pass * 8),
                ("nsources", C.c_int32), ("sources", fsim_source * MAX_SOURCES)]


# every symbol include/fsim.h declares, with its ctypes signature
_P = C.c_void_p
_SIGS = {
    "fsim_create": (C.c_int, [C.POINTER(fsim_config), C.POINTER(_P)]),
    "fsim_destroy": (C.c_int, [_P]),
    "fsim_last_error": (C.c_char_p, [_P]),
    "fsim_version": (C.c_char_p, []),
    "fsim_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "fsim_synchronize": (C.c_int, [_P]),
    "fsim_add_solid_cuboid": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "fsim_seed_fluid": (C.c_int, [_P, C.POINTER(fsim_seed_pass), C.c_int32, C.c_uint64]),
    "fsim_perturb_velocities": (C.c_int, [_P, C.c_float, C.c_uint64]),
    "fsim_upload_particles": (C.c_int, [_P, _P, _P, _P, C.c_int64]),
    "fsim_particle_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "fsim_download_particles": (C.c_int, [_P, _P, _P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "fsim_cfl": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "fsim_move_particles": (C.c_int, [_P, C.c_float]),
    "fsim_clear_grid": (C.c_int, [_P]),
    "fsim_transfer_particles_to_grid": (C.c_int, [_P]),
    "fsim_apply_boundary_conditions": (C.c_int, [_P]),
    "fsim_save_grid_velocities": (C.c_int, [_P]),
    "fsim_delete_outside_particles": (C.c_int, [_P]),
    "fsim_reinitialize_phi": (C.c_int, [_P]),
    "fsim_add_gravity": (C.c_int, [_P, C.c_float]),
    "fsim_compute_divergence": (C.c_int, [_P]),
    "fsim_update_velocity_from_pressure": (C.c_int, [_P]),
    "fsim_get_velocity_update": (C.c_int, [_P]),
    "fsim_update_particles_from_grid": (C.c_int, [_P]),
    "fsim_pcg_default_params": (C.c_int, [_P, C.POINTER(fsim_pcg_params)]),
    "fsim_pcg_solve": (C.c_int, [_P, C.POINTER(fsim_pcg_params), C.POINTER(fsim_pcg_stats)]),
    "fsim_step": (C.c_int, [_P, C.c_float, C.POINTER(fsim_pcg_params),
                            C.POINTER(fsim_step_stats)]),
    "fsim_step_host": (C.c_int, [_P, C.c_float, C.POINTER(fsim_pcg_params), _P, _P, _P,
                                 C.c_int64, _P, _P, _P, C.c_int64, C.POINTER(C.c_int64),
                                 C.POINTER(fsim_step_stats)]),
    "fsim_compute_dt": (C.c_int, [C.c_float, C.c_int32, C.c_float, C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]),
    "fsim_download_field": (C.c_int, [_P, C.c_int32, _P, _P]),
    "fsim_download_marker": (C.c_int, [_P, _P, _P]),
    "fsim_download_leaves": (C.c_int, [_P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "fsim_set_profiling": (C.c_int, [_P, C.c_int32]),
    "fsim_get_kernel_times": (C.c_int, [_P, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                        C.POINTER(C.c_int64), C.c_int32,
                                        C.POINTER(C.c_int32)]),
    "fsim_reset_kernel_times": (C.c_int, [_P]),
    "fsim_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "fsim_cfl_noalloc": (C.c_int, [_P, _P, C.POINTER(C.c_int32), C.c_float, _P, _P]),
    "fsim_add_source": (C.c_int, [_P, C.POINTER(fsim_source)]),
    "fsim_set_time": (C.c_int, [_P, C.c_double]),
    "fsim_get_time": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "fsim_add_contribution_from_sources": (C.c_int, [_P, C.c_float]),
    "fsim_delete_fluid_in_sources": (C.c_int, [_P, C.c_float]),
    "fsim_scene_parse": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(fsim_scene)]),
    "fsim_particles_to_level_set": (C.c_int, [_P, C.c_float, C.c_float, C.c_int32, _P, _P]),
    "fsim_run_frames": (C.c_int, [_P, C.c_int32, C.c_float, C.c_int32, C.POINTER(fsim_pcg_params),
                                  FRAME_FN, _P, C.POINTER(fsim_run_stats)]),
    "fsim_rollout_create": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "fsim_rollout_destroy": (C.c_int, [_P]),
    "fsim_rollout_particle_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "fsim_rollout_get_initial_velocity": (C.c_int, [_P, _P, _P]),
    "fsim_rollout_set_initial_velocity": (C.c_int, [_P, _P, _P]),
    "fsim_rollout_forward": (C.c_int, [_P, C.c_float, C.POINTER(fsim_pcg_params), _P,
                                       C.POINTER(C.c_double)]),
    "fsim_rollout_backward": (C.c_int, [_P, C.c_int32, C.POINTER(fsim_pcg_params), _P, _P]),
    "fsim_rollout_replay_loss": (C.c_int, [_P, _P, _P, C.POINTER(C.c_double)]),
}

_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libfsim.so and bind every declared entry point (raises if absent)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with __graft_entry__.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class FsimError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fsim error {code}: {msg}")
        self.code = code


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


@dataclass
class SceneShape:
    kind: int
    a: tuple = (0.0, 0.0, 0.0)
    b: tuple = (0.0, 0.0, 0.0)
    r: float = 0.0


@dataclass
class SeedPass:
    shapes: list
    velocity: tuple = (0.0, 0.0, 0.0)

    def to_c(self) -> fsim_seed_pass:
        p = fsim_seed_pass()
        p.nshapes = len(self.shapes)
        for i, sh in enumerate(self.shapes):
            p.shapes[i].kind = sh.kind
            for d in range(3):
                p.shapes[i].a[d] = sh.a[d]
                p.shapes[i].b[d] = sh.b[d]
            p.shapes[i].r = sh.r
        for d in range(3):
            p.velocity[d] = self.velocity[d]
        return p


def pcg_params(mode=PCG_ABSOLUTE, precision=PREC_FP32, max_iterations=1500, threshold=0.0,
               tolerance=1e-5, inner_tolerance=1e-2, max_refinements=8) -> fsim_pcg_params:
    p = fsim_pcg_params()
    p.mode, p.precision, p.max_iterations = mode, precision, max_iterations
    p.max_refinements = max_refinements
    p.threshold, p.tolerance, p.inner_tolerance = threshold, tolerance, inner_tolerance
    return p


def parse_scene(text: str, dims) -> fsim_scene:
    """fsim_scene_parse: an init file's text for a grid of dims cells."""
    lib = load_library()
    sc = fsim_scene()
    rc = lib.fsim_scene_parse(text.encode(), (C.c_int32 * 3)(*[int(d) for d in dims]),
                              C.byref(sc))
    if rc:
        raise FsimError(rc, lib.fsim_last_error(None).decode())
    return sc


def compute_dt(inv_speed: float, cfl: int, frame_step: float, time_in_frame: float):
    """FlipDriver::WhileAndComputeDt rule; returns (dt, new time_in_frame)."""
    lib = load_library()
    t = C.c_float(time_in_frame)
    dt = C.c_float(0.0)
    rc = lib.fsim_compute_dt(C.c_float(inv_speed), cfl, C.c_float(frame_step), C.byref(t),
                             C.byref(dt))
    if rc:
        raise FsimError(rc, "compute_dt")
    return dt.value, t.value


class Simulation:
    """One simulation domain on one GPU (a fsim_t handle)."""

    def __init__(self, dims, boundary=BOUNDARY_BOX, gravity=9.8, force=(0.0, 9.8, 0.0),
                 flip=0.95, nppc=8, max_particles=0, device=0):
        self.lib = load_library()
        cfg = fsim_config()
        for d in range(3):
            cfg.global_dims[d] = int(dims[d])
            cfg.force[d] = float(force[d])
        cfg.boundary = boundary
        cfg.gravity = gravity
        cfg.flip_factor = flip
        cfg.nparticles_per_cell = nppc
        cfg.max_particles = max_particles
        cfg.device = device
        self.dims = tuple(int(x) for x in dims)
        self._rollouts = weakref.WeakSet()  # closed before the handle
        h = C.c_void_p()
        rc = self.lib.fsim_create(C.byref(cfg), C.byref(h))
        if rc:
            raise FsimError(rc, "fsim_create failed")
        self.h = h

    # -- plumbing ---------------------------------------------------------
    def _ck(self, rc: int, what: str = ""):
        if rc:
            raise FsimError(rc, f"{what}: {self.lib.fsim_last_error(self.h).decode()}")

    def close(self):
        for ro in list(getattr(self, "_rollouts", ())):
            ro.close()
        if getattr(self, "h", None):
            self.lib.fsim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def synchronize(self):
        self._ck(self.lib.fsim_synchronize(self.h), "synchronize")

    def stream(self) -> int:
        s = C.c_void_p()
        self._ck(self.lib.fsim_get_stream(self.h, C.byref(s)), "get_stream")
        return s.value or 0

    # -- scene ------------------------------------------------------------
    def add_solid_cuboid(self, lo, hi):
        a = (C.c_int32 * 3)(*lo)
        b = (C.c_int32 * 3)(*hi)
        self._ck(self.lib.fsim_add_solid_cuboid(self.h, a, b), "add_solid_cuboid")

    def seed(self, passes: list[SeedPass], seed: int = 0):
        arr = (fsim_seed_pass * max(1, len(passes)))()
        for i, p in enumerate(passes):
            arr[i] = p.to_c()
        self._ck(self.lib.fsim_seed_fluid(self.h, arr, len(passes), C.c_uint64(seed)), "seed")

    def seed_scene(self, scene: "fsim_scene", seed: int = 0):
        """Seeds the passes of a parsed scene (one fsim_seed_fluid call)."""
        self._ck(self.lib.fsim_seed_fluid(self.h, scene.passes, scene.npasses, C.c_uint64(seed)),
                 "seed_fluid")

    def add_source(self, src: fsim_source):
        self._ck(self.lib.fsim_add_source(self.h, C.byref(src)), "add_source")

    @property
    def time(self) -> float:
        t = C.c_double()
        self._ck(self.lib.fsim_get_time(self.h, C.byref(t)), "get_time")
        return t.value

    @time.setter
    def time(self, t: float):
        self._ck(self.lib.fsim_set_time(self.h, C.c_double(t)), "set_time")

    def add_contribution_from_sources(self, t: float):
        self._ck(self.lib.fsim_add_contribution_from_sources(self.h, C.c_float(t)),
                 "add_contribution_from_sources")

    def delete_fluid_in_sources(self, t: float):
        self._ck(self.lib.fsim_delete_fluid_in_sources(self.h, C.c_float(t)),
                 "delete_fluid_in_sources")

    @classmethod
    def from_scene(cls, text: str, dims, flip=0.95, nppc=8, seed=0, max_particles=0, device=0):
        """A Simulation set up as FlipDriver::Initialize sets up an init-file
        scene: config, sources, boundary, solids, then the seeding passes."""
        sc = parse_scene(text, dims)
        sim = cls(dims, sc.boundary, sc.gravity, tuple(sc.force), flip, nppc, max_particles, device)
        for q in range(sc.nsources):
            sim.add_source(sc.sources[q])
        for q in range(sc.nsolids):
            sim.add_solid_cuboid(tuple(sc.solid_lo[q]), tuple(sc.solid_hi[q]))
        sim.seed_scene(sc, seed)
        return sim, sc

    def perturb_velocities(self, sigma: float, seed: int):
        self._ck(self.lib.fsim_perturb_velocities(self.h, C.c_float(sigma), C.c_uint64(seed)),
                 "perturb")

    def upload_particles(self, pos, vel, gvel):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        gvel = np.ascontiguousarray(gvel, dtype=np.float32)
        n = pos.shape[0]
        self._ck(self.lib.fsim_upload_particles(self.h, _ptr(pos), _ptr(vel), _ptr(gvel), n),
                 "upload")

    def particle_count(self) -> int:
        n = C.c_int64()
        self._ck(self.lib.fsim_particle_count(self.h, C.byref(n)), "particle_count")
        return n.value

    def download_particles(self):
        n = self.particle_count()
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        gvel = np.empty((n, 3), np.float32)
        got = C.c_int64()
        self._ck(self.lib.fsim_download_particles(self.h, _ptr(pos), _ptr(vel), _ptr(gvel), n,
                                                  C.byref(got)), "download_particles")
        return pos, vel, gvel

    # -- stages (FlipSimulation methods) ------------------------------------
    def cfl(self) -> float:
        v = C.c_float()
        self._ck(self.lib.fsim_cfl(self.h, C.byref(v)), "cfl")
        return v.value

    def move_particles(self, dt):
        self._ck(self.lib.fsim_move_particles(self.h, C.c_float(dt)), "move_particles")

    def clear_grid(self):
        self._ck(self.lib.fsim_clear_grid(self.h), "clear_grid")

    def transfer_particles_to_grid(self):
        self._ck(self.lib.fsim_transfer_particles_to_grid(self.h), "p2g")

    def apply_boundary_conditions(self):
        self._ck(self.lib.fsim_apply_boundary_conditions(self.h), "bc")

    def save_grid_velocities(self):
        self._ck(self.lib.fsim_save_grid_velocities(self.h), "save")

    def delete_outside_particles(self):
        self._ck(self.lib.fsim_delete_outside_particles(self.h), "delete_outside")

    def reinitialize_phi(self):
        self._ck(self.lib.fsim_reinitialize_phi(self.h), "reinit_phi")

    def add_gravity(self, dt):
        self._ck(self.lib.fsim_add_gravity(self.h, C.c_float(dt)), "gravity")

    def compute_divergence(self):
        self._ck(self.lib.fsim_compute_divergence(self.h), "divergence")

    def update_velocity_from_pressure(self):
        self._ck(self.lib.fsim_update_velocity_from_pressure(self.h), "pressure_update")

    def get_velocity_update(self):
        self._ck(self.lib.fsim_get_velocity_update(self.h), "velocity_update")

    def update_particles_from_grid(self):
        self._ck(self.lib.fsim_update_particles_from_grid(self.h), "g2p")

    def default_pcg_params(self) -> fsim_pcg_params:
        p = fsim_pcg_params()
        self._ck(self.lib.fsim_pcg_default_params(self.h, C.byref(p)), "pcg_default")
        return p

    def pcg_solve(self, params: fsim_pcg_params) -> fsim_pcg_stats:
        st = fsim_pcg_stats()
        self._ck(self.lib.fsim_pcg_solve(self.h, C.byref(params), C.byref(st)), "pcg_solve")
        return st

    def step(self, dt: float, params: fsim_pcg_params) -> fsim_step_stats:
        st = fsim_step_stats()
        self._ck(self.lib.fsim_step(self.h, C.c_float(dt), C.byref(params), C.byref(st)), "step")
        return st

    def step_host(self, dt: float, params: fsim_pcg_params, pos, vel, gvel, out=None):
        """fsim_step_host: upload (pos, vel, gvel), one step, download.  pos,
        vel, gvel are (n, 3) float32 arrays (numpy, or any object exposing
        data_ptr() and shape, e.g. pinned torch tensors); out = (pos, vel,
        gvel) receives the result (default: new numpy arrays of n rows).
        Returns (stats, particle count after the step)."""
        def addr(a):
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        n = int(pos.shape[0])
        if out is None:
            out = tuple(np.empty((n, 3), np.float32) for _ in range(3))
        cap = int(out[0].shape[0])
        st = fsim_step_stats()
        got = C.c_int64()
        self._ck(self.lib.fsim_step_host(self.h, C.c_float(dt), C.byref(params), addr(pos),
                                         addr(vel), addr(gvel), n, addr(out[0]), addr(out[1]),
                                         addr(out[2]), cap, C.byref(got), C.byref(st)),
                 "step_host")
        return st, got.value

    # -- downloads ----------------------------------------------------------
    def _dense_shape(self):
        return tuple(d + 2 for d in self.dims)

    def field(self, which: int):
        shp = self._dense_shape()
        vec = which in (FIELD_VELOCITY, FIELD_VELOCITY_UPDATE, FIELD_WEIGHT)
        out = np.empty(shp + ((3,) if vec else ()), np.float32)
        act = np.empty(shp, np.uint8)
        self._ck(self.lib.fsim_download_field(self.h, which, _ptr(out), _ptr(act)), "field")
        return out, act

    def run_frames(self, nframes: int, params: fsim_pcg_params, frame_rate=30.0, cfl=1,
                   on_frame=None) -> fsim_run_stats:
        """The driver's frame loop (fsim_run_frames); on_frame(frame) after each frame."""
        cb = FRAME_FN(lambda h, f, u: on_frame(int(f))) if on_frame else FRAME_FN()
        st = fsim_run_stats()
        self._ck(self.lib.fsim_run_frames(self.h, nframes, C.c_float(frame_rate), cfl,
                                          C.byref(params), cb, None, C.byref(st)), "run_frames")
        return st

    def level_set(self, radius=3.0, half_width=3.0, mean_iterations=1):
        """Particles to a narrow-band level set (fsim_particles_to_level_set):
        dense phi over voxels [-1, N] and its band mask."""
        shp = self._dense_shape()
        phi = np.empty(shp, np.float32)
        act = np.empty(shp, np.uint8)
        self._ck(self.lib.fsim_particles_to_level_set(self.h, C.c_float(radius),
                                                      C.c_float(half_width), mean_iterations,
                                                      _ptr(phi), _ptr(act)), "level_set")
        return phi, act

    def marker(self):
        shp = self._dense_shape()
        out = np.empty(shp, np.int32)
        act = np.empty(shp, np.uint8)
        self._ck(self.lib.fsim_download_marker(self.h, _ptr(out), _ptr(act)), "marker")
        return out, act

    def leaves(self):
        n = C.c_int64()
        cap = max(1, self.particle_count())
        out = np.empty((cap, 3), np.int32)
        self._ck(self.lib.fsim_download_leaves(self.h, _ptr(out), cap, C.byref(n)), "leaves")
        return out[: n.value].copy()

    # -- timing -------------------------------------------------------------
    def set_profiling(self, on: bool):
        self._ck(self.lib.fsim_set_profiling(self.h, 1 if on else 0), "profiling")

    def kernel_times(self) -> dict:
        cnt = C.c_int32()
        self._ck(self.lib.fsim_get_kernel_times(self.h, None, None, None, 0, C.byref(cnt)), "kt")
        n = cnt.value
        names = (C.c_char_p * max(1, n))()
        ms = (C.c_double * max(1, n))()
        la = (C.c_int64 * max(1, n))()
        self._ck(self.lib.fsim_get_kernel_times(self.h, names, ms, la, n, C.byref(cnt)), "kt")
        return {names[i].decode(): (ms[i], la[i]) for i in range(n)}

    def reset_kernel_times(self):
        self._ck(self.lib.fsim_reset_kernel_times(self.h), "reset_kt")

    def launch_count(self) -> int:
        n = C.c_int64()
        self._ck(self.lib.fsim_launch_count(self.h, C.byref(n)), "launch_count")
        return n.value


# ---- synthetic scenes of the benchmark configurations ----------------------
def scene_passes(name: str, n: int) -> list[SeedPass]:
    """Seeding passes (index space) for the named synthetic scene at N^3.

    sphere_drop: sphere r=0.15 at (0.5,0.7,0.5) over a pool y<0.2
    dam_break:   block x<0.4, y<0.6, all z
    multidam:    four 0.2x0.5x0.2 blocks at the x/z quadrant corners + pool y<0.05
    sphere_pool: sphere r=0.1 at (0.5,0.6,0.5) + pool y<0.1
    """
    N = float(n)
    if name == "sphere_drop":
        return [SeedPass([SceneShape(SHAPE_POOL, a=(0.0, 0.2 * N, 0.0)),
                          SceneShape(SHAPE_SPHERE, a=(0.5 * N, 0.7 * N, 0.5 * N), r=0.15 * N)])]
    if name == "dam_break":
        return [SeedPass([SceneShape(SHAPE_CUBOID, a=(0.0, 0.0, 0.0), b=(0.4 * N, 0.6 * N, N))])]
    if name == "multidam":
        shapes = [SceneShape(SHAPE_POOL, a=(0.0, 0.05 * N, 0.0))]
        for x0 in (0.0, 0.8):
            for z0 in (0.0, 0.8):
                shapes.append(SceneShape(SHAPE_CUBOID, a=(x0 * N, 0.0, z0 * N),
                                         b=((x0 + 0.2) * N, 0.5 * N, (z0 + 0.2) * N)))
        return [SeedPass(shapes)]
    if name == "sphere_pool":
        return [SeedPass([SceneShape(SHAPE_POOL, a=(0.0, 0.1 * N, 0.0)),
                          SceneShape(SHAPE_SPHERE, a=(0.5 * N, 0.6 * N, 0.5 * N), r=0.1 * N)])]
    raise ValueError(name)


def physical_gravity(n: int) -> tuple[float, tuple]:
    """Gravity -9.8 with dx = 1/N in index space: 9.8*N cells/s^2."""
    g = float(np.float32(9.8 * n))
    return g, (0.0, g, 0.0)


class Rollout:
    """Differentiable rollout of a Simulation (fsim_rollout_*).

    Captures the simulation's particle state as the initial state.  forward()
    runs `steps` production steps at a fixed dt and returns the loss
    0.5 * sum (u - target)^2 over the active in-box faces after the last step
    (target: a dense face field as Simulation.field(FIELD_VELOCITY) returns);
    backward() returns the gradients w.r.t. the initial particle velocity
    and grid velocity ((n, 3) float64 each, initial particle order).
    """

    def __init__(self, sim: "Simulation", steps: int, checkpoint_every: int = 4):
        self.sim = sim
        self.lib = sim.lib
        h = C.c_void_p()
        sim._ck(self.lib.fsim_rollout_create(sim.h, steps, checkpoint_every, C.byref(h)),
                "fsim_rollout_create")
        self.h = h
        sim._rollouts.add(self)
        n = C.c_int64()
        self.lib.fsim_rollout_particle_count(self.h, C.byref(n))
        self.n = int(n.value)

    def close(self):
        # a rollout must be destroyed before its simulation's handle
        if getattr(self, "h", None) and getattr(self.sim, "h", None):
            self.lib.fsim_rollout_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _soa(a):
        """(n, 3) -> contiguous SoA float64 (x | y | z)."""
        return np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)

    def initial_velocity(self):
        v = np.empty((3, self.n), np.float64)
        g = np.empty((3, self.n), np.float64)
        self.sim._ck(self.lib.fsim_rollout_get_initial_velocity(self.h, _ptr(v), _ptr(g)),
                     "fsim_rollout_get_initial_velocity")
        return v.T.copy(), g.T.copy()

    def set_initial_velocity(self, vel, gvel=None):
        v = self._soa(vel)
        g = self._soa(vel if gvel is None else gvel)
        self.sim._ck(self.lib.fsim_rollout_set_initial_velocity(self.h, _ptr(v), _ptr(g)),
                     "fsim_rollout_set_initial_velocity")

    def forward(self, dt: float, pcg: "fsim_pcg_params", target: np.ndarray) -> float:
        t = np.ascontiguousarray(target, dtype=np.float32)
        loss = C.c_double()
        self.sim._ck(self.lib.fsim_rollout_forward(self.h, C.c_float(dt), C.byref(pcg), _ptr(t),
                                                   C.byref(loss)), "fsim_rollout_forward")
        return float(loss.value)

    def backward(self, adj: "fsim_pcg_params", tape: int = 0):
        gv = np.empty((3, self.n), np.float64)
        gg = np.empty((3, self.n), np.float64)
        self.sim._ck(self.lib.fsim_rollout_backward(self.h, tape, C.byref(adj), _ptr(gv),
                                                    _ptr(gg)), "fsim_rollout_backward")
        return gv.T.copy(), gg.T.copy()

    def replay_loss(self, vel=None, gvel=None) -> float:
        v = None if vel is None else self._soa(vel)
        g = None if gvel is None else self._soa(gvel)
        loss = C.c_double()
        self.sim._ck(self.lib.fsim_rollout_replay_loss(self.h, _ptr(v), _ptr(g), C.byref(loss)),
                     "fsim_rollout_replay_loss")
        return float(loss.value)


def rollout_case(n: int, steps: int = 16, every: int = 4, dt: float = 1.0 / 300.0,
                 sigma: float | None = None, noise_seed: int = 1, target_seed: int = 2,
                 pcg: "fsim_pcg_params | None" = None, device: int = 0):
    """The differentiable-rollout workload: the N^3 sphere drop (walls), 8
    particles per cell from seed 0, initial velocities perturbed by Gaussian
    noise sigma (index units; default 0.1 m/s with dx = 1/N, i.e. 0.1*N
    cells/s) from noise_seed.  The target is the velocity field after the
    same rollout with target_seed's noise.  Steps use a fixed dt and, unless
    given, MIXED PCG to relative residual 1e-9.

    Returns (sim, rollout, target, pcg)."""
    g, f = physical_gravity(n)
    sig = 0.1 * n if sigma is None else float(sigma)
    if pcg is None:
        pcg = pcg_params(PCG_RELATIVE, PREC_MIXED, 4000, tolerance=1e-9, inner_tolerance=1e-3,
                         max_refinements=30)
    t = Simulation((n, n, n), BOUNDARY_BOX, g, f, device=device)
    t.seed(scene_passes("sphere_drop", n), seed=0)
    t.perturb_velocities(sig, target_seed)
    for _ in range(steps):
        t.step(dt, pcg)
    target, _ = t.field(FIELD_VELOCITY)
    t.close()
    sim = Simulation((n, n, n), BOUNDARY_BOX, g, f, device=device)
    sim.seed(scene_passes("sphere_drop", n), seed=0)
    sim.perturb_velocities(sig, noise_seed)
    ro = Rollout(sim, steps, every)
    return sim, ro, np.ascontiguousarray(target, dtype=np.float32), pcg
