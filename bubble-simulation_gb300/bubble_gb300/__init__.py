"""Python face of the GB300 lattice time step (C ABI via ctypes).

Names follow the reference's Rust host: `Model` (src/physics.rs:44-218),
`make_schedule` (src/physics.rs:248-296), `SimulationSpec`
(src/gpu/sim.rs:246-255) and `Simulation` (src/gpu/sim.rs:180-1026).  Every
call goes through lib/libbubble_gb300.so; nothing here computes physics.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import BubbleError, check, load

__all__ = ["Model", "SimulationSpec", "Simulation", "Diagnostics", "make_schedule", "derived",
           "validate_model", "stage_slots", "rk3_coefficients", "lattice_bytes", "max_cubic_size",
           "vram_query", "vram_available", "lattice_budget", "BubbleError", "load", "render_settings", "camera",
           "render_view", "write_png", "checkpoint_spec"]


@dataclass
class Model:
    lambda_: float = 0.5
    eps_ratio: float = 0.3
    alpha: float = 0.1
    eta: float = 0.3
    phi_b: float = 1.0
    dx: float = 1.0
    cfl: float = 0.2
    seed_kind: str = "critical"  # "critical" (factor of R_c) or "cells"
    seed_value: float = 1.15

    def c(self) -> _lib.Model:
        return _lib.Model(self.lambda_, self.eps_ratio, self.alpha, self.eta, self.phi_b, self.dx,
                          self.cfl, _lib.SEED_CRITICAL if self.seed_kind == "critical" else _lib.SEED_CELLS,
                          self.seed_value)

    @classmethod
    def from_c(cls, m: _lib.Model) -> "Model":
        return cls(m.lambda_, m.eps_ratio, m.alpha, m.eta, m.phi_b, m.dx, m.cfl,
                   "critical" if m.seed_kind == _lib.SEED_CRITICAL else "cells", m.seed_value)


def derived(model: Model) -> dict:
    d = _lib.Derived()
    check(load().bubble_model_derived(ctypes.byref(model.c()), ctypes.byref(d)))
    return {n: getattr(d, n) for n, _ in _lib.Derived._fields_}


def validate_eos(spec: "SimulationSpec") -> str | None:
    """The spec's equation-of-state selection: None if valid, else the message."""
    L = load()
    if L.bubble_eos_validate(ctypes.byref(spec.c())) == _lib.OK:
        return None
    return L.bubble_last_error().decode()


def validate_model(model: Model) -> str | None:
    rc = load().bubble_model_validate(ctypes.byref(model.c()))
    return None if rc == _lib.OK else load().bubble_last_error().decode()


def make_schedule(mode: str, count: int, radius: float, grid: Sequence[int], duration: float,
                  seed: int) -> list[tuple]:
    L = load()
    g = (ctypes.c_uint32 * 3)(*grid)
    out = (_lib.Event * max(count, 1))()
    n = ctypes.c_uint64()
    check(L.bubble_make_schedule(_lib.NUCLEATION[mode], count, radius, g, duration, seed, out,
                                 count, ctypes.byref(n)))
    return [(out[k].time, tuple(out[k].pos), out[k].radius) for k in range(n.value)]


def stage_slots(cur: int) -> list[tuple[int, int]]:
    o = (ctypes.c_uint32 * 6)()
    check(load().bubble_stage_slots(cur, o))
    return [(o[0], o[1]), (o[2], o[3]), (o[4], o[5])]


def rk3_coefficients() -> list[tuple[float, float]]:
    o = (ctypes.c_float * 6)()
    load().bubble_rk3_coefficients(o)
    return [(o[0], o[1]), (o[2], o[3]), (o[4], o[5])]


def lattice_bytes(grid: Sequence[int]) -> int:
    return load().bubble_lattice_bytes((ctypes.c_uint32 * 3)(*grid))


def max_cubic_size(max_buffer_bytes: int, budget_bytes: int | None) -> tuple[int, bool]:
    side = ctypes.c_uint32()
    lim = ctypes.c_int32()
    check(load().bubble_max_cubic_size(max_buffer_bytes, budget_bytes or 0, budget_bytes is not None,
                                       ctypes.byref(side), ctypes.byref(lim)))
    return side.value, bool(lim.value)


def vram_query() -> _lib.VramInfo:
    v = _lib.VramInfo()
    check(load().bubble_vram_query(ctypes.byref(v)))
    return v


def vram_available(capacity: int, budget: int | None = None, used: int | None = None) -> int:
    v = _lib.VramInfo(capacity, budget or 0, used or 0, int(budget is not None and used is not None))
    return load().bubble_vram_available(ctypes.byref(v))


def lattice_budget(available: int, current_lattice: int) -> int:
    return load().bubble_lattice_budget(available, current_lattice)


@dataclass
class SimulationSpec:
    model: Model = field(default_factory=Model)
    grid: tuple = (192, 192, 192)
    nucleation: str = "exponential"
    bubbles: int = 12
    nucleation_duration: float = 60.0
    seed: int = 1
    precision: str = "single"  # single | mixed | double | perturbation
    math: str = "fast"  # fast | strict
    eos: str = "bag"  # bag | bag_dof (eos_param = (dof ratio, -)) | gamma_law (eos_param = (Gamma, e0))
    #                   | thermal (eos_param = (gamma, A) of the temperature-dependent potential)
    eos_param: tuple = (1.0, 0.0)

    def c(self) -> _lib.Spec:
        return _lib.Spec(self.model.c(), (ctypes.c_uint32 * 3)(*self.grid), _lib.NUCLEATION[self.nucleation],
                         self.bubbles, self.nucleation_duration, self.seed, _lib.PRECISION[self.precision],
                         _lib.MATH[self.math], _lib.EOS[self.eos], (ctypes.c_float * 2)(*self.eos_param))

    @classmethod
    def from_c(cls, c: _lib.Spec) -> "SimulationSpec":
        inv = lambda d, v: next(k for k, x in d.items() if x == v)  # noqa: E731
        return cls(Model.from_c(c.model), tuple(c.grid), inv(_lib.NUCLEATION, c.nucleation), c.bubbles,
                   c.nucleation_duration, c.seed, inv(_lib.PRECISION, c.precision), inv(_lib.MATH, c.math),
                   inv(_lib.EOS, c.eos), tuple(c.eos_param))


@dataclass
class Diagnostics:
    mean_energy: float
    broken_fraction: float
    mean_kinetic: float
    mean_fluid_energy: float
    max_velocity: float
    kinetic_fraction: float
    sum_energy: float
    sum_broken: float
    sum_kinetic: float
    sum_fluid_energy: float
    mean_energy_f64: float
    mean_kinetic_f64: float
    cells: int


class Simulation:
    """The device-resident lattice (src/gpu/sim.rs:180-1026) behind the C ABI."""

    def __init__(self, spec: SimulationSpec):
        self._L = load()
        self.spec = spec
        h = ctypes.c_void_p()
        check(self._L.bubble_create(ctypes.byref(spec.c()), ctypes.byref(h)))
        self._h = h
        self._dtype = np.float64 if spec.precision == "double" else np.float32

    def close(self):
        if getattr(self, "_h", None):
            self._L.bubble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    # -- lifecycle ------------------------------------------------------------
    def reset(self, schedule: list | None = None):
        if schedule is None:
            check(self._L.bubble_reset(self._h, None, 0))
        else:
            ev = (_lib.Event * max(len(schedule), 1))()
            for k, (t, pos, r) in enumerate(schedule):
                ev[k] = _lib.Event(t, (ctypes.c_float * 3)(*pos), r)
            check(self._L.bubble_reset(self._h, ev, len(schedule)))

    def set_model(self, model: Model):
        check(self._L.bubble_set_model(self._h, ctypes.byref(model.c())))

    def resize(self, grid: Sequence[int]):
        check(self._L.bubble_resize(self._h, (ctypes.c_uint32 * 3)(*grid)))

    def set_stream(self, stream_ptr: int | None):
        check(self._L.bubble_set_stream(self._h, stream_ptr))

    def set_path(self, path: str):
        """"fused" (default) or "reference" (primitives + stage passes)."""
        check(self._L.bubble_ext_set_path(self._h, _lib.PATHS[path]))

    def set_tile(self, ty: int, lz: int):
        check(self._L.bubble_ext_set_tile(self._h, ty, lz))

    def set_stage_form(self, form: str):
        """Form of the fused kernel for FP32 16 x 16 tiles: "auto" (default),
        "registers" or "shared" (identical bits; include/bubble_ext.h)."""
        check(self._L.bubble_ext_set_stage_form(self._h, _lib.STAGE_FORMS[form]))

    def tile(self) -> tuple[int, int]:
        ty, lz = ctypes.c_int32(), ctypes.c_int32()
        check(self._L.bubble_ext_get_tile(self._h, ctypes.byref(ty), ctypes.byref(lz)))
        return ty.value, lz.value

    # -- stepping -------------------------------------------------------------
    def record_steps(self, n: int = 1):
        check(self._L.bubble_record_steps(self._h, n))

    def advance(self, n: int):
        check(self._L.bubble_advance(self._h, n))

    def synchronize(self):
        check(self._L.bubble_synchronize(self._h))

    def nucleate_now(self, rng_seed: int):
        check(self._L.bubble_nucleate_now(self._h, rng_seed))

    def diagnostics(self, allow_nonfinite: bool = False) -> Diagnostics:
        d = _lib.Diag()
        rc = self._L.bubble_diagnostics(self._h, ctypes.byref(d))
        if not (allow_nonfinite and rc == _lib.ERR_NONFINITE):
            check(rc)
        return Diagnostics(**{n: getattr(d, n) for n, _ in _lib.Diag._fields_})

    # -- accessors ------------------------------------------------------------
    @property
    def time(self) -> float:
        return self._L.bubble_time(self._h)

    @property
    def steps(self) -> int:
        return self._L.bubble_steps(self._h)

    def cell_count(self) -> int:
        return self._L.bubble_cell_count(self._h)

    def remaining_bubbles(self) -> int:
        return self._L.bubble_remaining_bubbles(self._h)

    def device_memory_bytes(self) -> int:
        return self._L.bubble_device_memory_bytes(self._h)

    @property
    def grid(self) -> tuple:
        g = (ctypes.c_uint32 * 3)()
        check(self._L.bubble_get_grid(self._h, g))
        return tuple(g)

    @property
    def model(self) -> Model:
        m = _lib.Model()
        check(self._L.bubble_get_model(self._h, ctypes.byref(m)))
        return Model.from_c(m)

    def schedule(self) -> list[tuple]:
        n = ctypes.c_uint64()
        check(self._L.bubble_get_schedule(self._h, None, 0, ctypes.byref(n)))
        ev = (_lib.Event * max(n.value, 1))()
        check(self._L.bubble_get_schedule(self._h, ev, n.value, ctypes.byref(n)))
        return [(ev[k].time, tuple(ev[k].pos), ev[k].radius) for k in range(n.value)]

    def launches(self) -> int:
        return self._L.bubble_ext_launches(self._h)

    def stream_ptr(self) -> int:
        return self._L.bubble_ext_stream(self._h) or 0

    # -- state ----------------------------------------------------------------
    def copy_state(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.cell_count()
        field = np.empty((n, 2), dtype=self._dtype)
        fluid = np.empty((n, 4), dtype=self._dtype)
        fn = self._L.bubble_copy_state_f64 if self._dtype == np.float64 else self._L.bubble_copy_state
        check(fn(self._h, field.ctypes.data, fluid.ctypes.data))
        return field, fluid

    def load_state(self, field: np.ndarray, fluid: np.ndarray):
        n = self.cell_count()
        field = np.ascontiguousarray(field, dtype=self._dtype).reshape(n, 2)
        fluid = np.ascontiguousarray(fluid, dtype=self._dtype).reshape(n, 4)
        fn = self._L.bubble_load_state_f64 if self._dtype == np.float64 else self._L.bubble_load_state
        check(fn(self._h, field.ctypes.data, fluid.ctypes.data))

    # -- checkpoint and resume (include/bubble_checkpoint.h) ------------------
    def save_checkpoint(self, path: str):
        check(self._L.bubble_checkpoint_save(self._h, str(path).encode()))

    def restore_checkpoint(self, path: str):
        check(self._L.bubble_checkpoint_restore(self._h, str(path).encode()))

    @classmethod
    def from_checkpoint(cls, path: str, precision: str | None = None, math: str | None = None) -> "Simulation":
        """A simulation created with the checkpoint's spec (optionally another
        arithmetic of the same FP32/FP64 layout) and restored from it."""
        spec = checkpoint_spec(path)
        if precision is not None:
            spec.precision = precision
        if math is not None:
            spec.math = math
        sim = cls(spec)
        sim.restore_checkpoint(path)
        return sim

    # -- visualisation (include/bubble_render.h) ------------------------------
    def visualise(self):
        """record_visualisation (src/gpu/sim.rs:918-942) into the vis texture."""
        check(self._L.bubble_visualise(self._h))

    def vis_texture(self) -> np.ndarray:
        """The vis texture as (nz, ny, nx, 4) uint16 binary16 bits."""
        nx, ny, nz = self.grid
        out = np.empty((nz, ny, nx, 4), dtype=np.uint16)
        check(self._L.bubble_vis_copy(self._h, out.ctypes.data))
        return out

    def render(self, settings: "_lib.RenderSettings | None" = None, camera: "_lib.Camera | None" = None,
               size: tuple = (1280, 960), frame: int = 1) -> np.ndarray:
        """One frame of the volume renderer: (height, width, 4) uint8."""
        settings = settings or render_settings()
        w, h = size
        out = np.empty((h, w, 4), dtype=np.uint8)
        check(self._L.bubble_render(self._h, ctypes.byref(settings), ctypes.byref(camera) if camera else None,
                                    w, h, frame, out.ctypes.data))
        return out

    def render_png(self, path: str, settings: "_lib.RenderSettings | None" = None, size: tuple = (1280, 960)):
        """capture::render_to_png (src/capture.rs:19-117)."""
        settings = settings or render_settings()
        check(self._L.bubble_render_png(self._h, ctypes.byref(settings), size[0], size[1], str(path).encode()))


def checkpoint_spec(path: str) -> SimulationSpec:
    """The SimulationSpec stored in a checkpoint file (no device work)."""
    c = _lib.Spec()
    check(load().bubble_checkpoint_spec(str(path).encode(), ctypes.byref(c)))
    return SimulationSpec.from_c(c)


def render_settings(field: str | None = None) -> _lib.RenderSettings:
    """RenderSettings::default, or RenderSettings::with_field(field)."""
    L = load()
    s = _lib.RenderSettings()
    if field is None:
        check(L.bubble_render_settings_default(ctypes.byref(s)))
    else:
        check(L.bubble_render_settings_with_field(_lib.FIELDS[field], ctypes.byref(s)))
    return s


def camera(half_extent: Sequence[float] | None = None) -> _lib.Camera:
    """OrbitCamera::default, framed on a box of `half_extent` if given."""
    L = load()
    c = _lib.Camera()
    check(L.bubble_camera_default(ctypes.byref(c)))
    if half_extent is not None:
        check(L.bubble_camera_frame_box(ctypes.byref(c), (ctypes.c_float * 3)(*half_extent)))
    return c


def render_view(grid: Sequence[int], settings: _lib.RenderSettings, size: tuple, frame: int = 1,
                cam: _lib.Camera | None = None) -> np.ndarray:
    """The 176-byte view uniform of one frame as 44 float32."""
    v = _lib.View()
    check(load().bubble_render_view((ctypes.c_uint32 * 3)(*grid), ctypes.byref(settings),
                                    ctypes.byref(cam) if cam else None, size[0], size[1], frame, ctypes.byref(v)))
    return np.frombuffer(bytes(v), dtype=np.float32).copy()


def write_png(path: str, rgba: np.ndarray):
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w, c = rgba.shape
    assert c == 4
    check(load().bubble_write_png(str(path).encode(), rgba.ctypes.data, w, h))


class Batch:
    """Many independent lattices advanced by one persistent, graph-captured
    launch per chunk of steps (include/bubble_batch.h)."""

    def __init__(self, specs: list[SimulationSpec], tile_y: int = 16, autotune: bool = True,
                 use_graph: bool = True, max_grid: int = 0):
        self._L = load()
        self.specs = list(specs)
        arr = (_lib.Spec * len(specs))(*[s.c() for s in specs])
        opt = _lib.BatchOptions(tile_y, int(autotune), int(use_graph), max_grid)
        h = ctypes.c_void_p()
        check(self._L.bubble_batch_create(arr, len(specs), ctypes.byref(opt), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.bubble_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.specs)

    def advance(self, n: int):
        check(self._L.bubble_batch_advance(self._h, n))

    def diagnostics(self, k: int) -> Diagnostics:
        d = _lib.Diag()
        check(self._L.bubble_batch_diagnostics(self._h, k, ctypes.byref(d)))
        return Diagnostics(**{n: getattr(d, n) for n, _ in _lib.Diag._fields_})

    def copy_state(self, k: int) -> tuple[np.ndarray, np.ndarray]:
        g = self.specs[k].grid
        n = g[0] * g[1] * g[2]
        field = np.empty((n, 2), dtype=np.float32)
        fluid = np.empty((n, 4), dtype=np.float32)
        check(self._L.bubble_batch_copy_state(self._h, k, field.ctypes.data, fluid.ctypes.data))
        return field, fluid

    def load_state(self, k: int, field: np.ndarray, fluid: np.ndarray):
        field = np.ascontiguousarray(field, dtype=np.float32)
        fluid = np.ascontiguousarray(fluid, dtype=np.float32)
        check(self._L.bubble_batch_load_state(self._h, k, field.ctypes.data, fluid.ctypes.data))

    def time(self, k: int) -> float:
        return self._L.bubble_batch_time(self._h, k)

    def info(self) -> dict:
        i = _lib.BatchInfo()
        check(self._L.bubble_batch_info_get(self._h, ctypes.byref(i)))
        return {n: getattr(i, n) for n, _ in _lib.BatchInfo._fields_}


def autotune_chunk(grid, tile_y: int = 16, math: str = "fast") -> int:
    lz = ctypes.c_int32()
    check(load().bubble_autotune_chunk((ctypes.c_uint32 * 3)(*grid), tile_y, _lib.MATH[math], ctypes.byref(lz)))
    return lz.value


class Server:
    """Request loop with continuous batching (include/bubble_server.h)."""

    def __init__(self, math: str = "fast", chunk_steps: int = 50, max_active: int = 64,
                 memory_fraction: float = 0.85, use_graph: bool = True, tile_y: int = 16,
                 resident_cells: int = 0, policy: str = "fifo", chunk_planes: int = 0):
        self._L = load()
        opt = _lib.ServerOptions(_lib.MATH[math], tile_y, chunk_steps, max_active, memory_fraction, int(use_graph),
                                 resident_cells, _lib.SERVE_POLICY[policy], chunk_planes)
        h = ctypes.c_void_p()
        check(self._L.bubble_server_create(ctypes.byref(opt), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.bubble_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, spec: SimulationSpec, steps: int) -> int:
        i = ctypes.c_uint64()
        check(self._L.bubble_server_submit(self._h, ctypes.byref(spec.c()), steps, ctypes.byref(i)))
        return i.value

    def tick(self) -> bool:
        busy = ctypes.c_int32()
        check(self._L.bubble_server_tick(self._h, ctypes.byref(busy)))
        return bool(busy.value)

    def run_until_idle(self):
        check(self._L.bubble_server_run_until_idle(self._h))

    def poll(self) -> list[dict]:
        out = (_lib.ServerResult * 256)()
        n = ctypes.c_uint64()
        res = []
        while True:
            check(self._L.bubble_server_poll(self._h, out, 256, ctypes.byref(n)))
            for k in range(n.value):
                r = out[k]
                res.append(dict(id=r.id, status=r.status, grid=tuple(r.grid), steps=r.steps, submit_s=r.submit_s,
                                admit_s=r.admit_s, done_s=r.done_s,
                                diag=Diagnostics(**{f: getattr(r.diag, f) for f, _ in _lib.Diag._fields_})))
            if n.value < 256:
                return res

    def stats(self) -> dict:
        s = _lib.ServerStats()
        check(self._L.bubble_server_stats_get(self._h, ctypes.byref(s)))
        return {n: getattr(s, n) for n, _ in _lib.ServerStats._fields_}

    def now(self) -> float:
        return self._L.bubble_server_now(self._h)
