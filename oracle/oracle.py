"""ORACLE -- test infrastructure only.

CPU restatement of the reference's lattice time step, used by the tests,
`__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` as the
checker.  The product (the CUDA library under bubble-simulation_gb300/)
never imports, links or calls anything here.

Contents
  * Model derivations (src/physics.rs:85-189) in numpy float32, reference
    evaluation order; SimParams values (src/gpu/sim.rs:613-644).
  * Pcg64Mcg / make_schedule (src/physics.rs:243-308) in pure Python: the
    128-bit MCG with XSL-RR output (O'Neill 2014, rand_pcg 0.9
    Mcg128Xsl64), rand_core 0.9 seed_from_u64 (PCG32 fill of the 16 seed
    bytes), rand 0.9 f32 sampling (top 24 bits of next_u32 times 2^-24).
    f32 exp/ln call the C library's expf/logf, as Rust's f32::exp/ln do on
    Linux.  The rand crates are not in the reference tree, so bit parity of
    seeding with the Rust binary itself is unpinned.
  * OracleSim: the host driver of src/gpu/sim.rs (record_steps 827-841,
    record_nucleation 843-879, record_step 881-916, stage_slots 1046-1051,
    diagnostics 948-1010) over the C kernels in oracle.cpp.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_DIR = HERE / "lib"
LIB_PATH = LIB_DIR / "liboracle_bubble.so"

f32 = np.float32

# ---------------------------------------------------------------------------
#  Build / load
# ---------------------------------------------------------------------------


NATIVE_LIB_PATH = LIB_DIR / "liboracle_bubble_native.so"


def _native_flags() -> list[str]:
    """Tuning flags for the host CPU (the timed CPU baseline's build)."""
    import platform

    return ["-mcpu=native"] if platform.machine() in ("aarch64", "arm64") else ["-march=native"]


def build(force: bool = False, native: bool = False) -> Path:
    """Compile oracle.cpp into lib/.  The parity build (the checker) is
    g++ -O3 -fopenmp -ffp-contract=off, one IEEE rounding per operation; the
    native build (only ever timed, as the CPU baseline) adds the host CPU's
    tuning flags and lets the compiler contract multiply-adds."""
    LIB_DIR.mkdir(exist_ok=True)
    src = HERE / "oracle.cpp"
    out = NATIVE_LIB_PATH if native else LIB_PATH
    if not force and out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    cxx = os.environ.get("CXX", "g++")
    fp = ["-ffp-contract=fast"] + _native_flags() if native else ["-ffp-contract=off"]
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math"] + fp + \
          [str(src), "-o", str(out)]
    subprocess.run(cmd, check=True)
    return out


_libs: dict = {}


def lib(native: bool = False) -> ctypes.CDLL:
    """The parity build (default) or the native timing build of the oracle."""
    if native not in _libs:
        path = NATIVE_LIB_PATH if native else LIB_PATH
        if not path.exists():
            build(native=native)
        L = ctypes.CDLL(str(path))
        P = ctypes.c_void_p
        for sfx in ("f32", "f64", "pert_f32"):
            getattr(L, f"oracle_init_{sfx}").argtypes = [P, P, P]
            getattr(L, f"oracle_primitives_{sfx}").argtypes = [P, P, P, P]
            getattr(L, f"oracle_step_{sfx}").argtypes = [P] * 9
            getattr(L, f"oracle_reduce_{sfx}").argtypes = [P, P, P, P, P, P]
            getattr(L, f"oracle_vis_{sfx}").argtypes = [P] * 5
        for sfx in ("f32", "f64"):
            getattr(L, f"oracle_nucleate_{sfx}").argtypes = [P, P, ctypes.c_uint32, P]
        L.oracle_tanh_f64.argtypes = [ctypes.c_double]
        L.oracle_tanh_f64.restype = ctypes.c_double
        L.oracle_tanh_f32.argtypes = [ctypes.c_float]
        L.oracle_tanh_f32.restype = ctypes.c_float
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_eos.argtypes = [ctypes.c_float] * 3
        L.oracle_primitives_gamma_f32.argtypes = [P, P, P, P]
        L.oracle_primitives_mixed_f32.argtypes = [P, P, P, P]
        L.oracle_step_gamma_f32.argtypes = [P] * 9
        L.oracle_set_thermal.argtypes = [ctypes.c_float] * 6
        L.oracle_init_thermal_f32.argtypes = [P, P, P]
        L.oracle_primitives_thermal_f32.argtypes = [P, P, P, P]
        L.oracle_step_thermal_f32.argtypes = [P] * 9
        L.oracle_reduce_thermal_f32.argtypes = [P, P, P, P, P, P]
        L.oracle_vis_thermal_f32.argtypes = [P] * 5
        L.oracle_render.argtypes = [P, P] + [ctypes.c_int] * 6 + [P]
        L.oracle_f32_to_f16.argtypes = [ctypes.c_float]
        L.oracle_f32_to_f16.restype = ctypes.c_uint16
        _libs[native] = L
    return _libs[native]


_libm = ctypes.CDLL("libm.so.6")
_libm.expf.argtypes = [ctypes.c_float]
_libm.expf.restype = ctypes.c_float
_libm.logf.argtypes = [ctypes.c_float]
_libm.logf.restype = ctypes.c_float


def expf(x) -> np.float32:
    return f32(_libm.expf(float(f32(x))))


def logf(x) -> np.float32:
    return f32(_libm.logf(float(f32(x))))


def render(view: np.ndarray, tex: np.ndarray, width: int, height: int, quant: int = 1) -> np.ndarray:
    """fs_main of shaders/volume.wgsl over the half4 texels `tex` ((nz, ny,
    nx, 4) uint16) with the 176-byte view uniform `view` (44 float32):
    (height, width, 4) uint8.  `quant` sets the trilinear weights' fraction:
    0 exact, 1 rounded to 1/256, 2 truncated to 1/256."""
    view = np.ascontiguousarray(view, dtype=np.float32)
    tex = np.ascontiguousarray(tex, dtype=np.uint16)
    assert view.size == 44 and tex.ndim == 4 and tex.shape[3] == 4
    nz, ny, nx, _ = tex.shape
    out = np.zeros((height, width, 4), dtype=np.uint8)
    lib().oracle_render(_ptr(view), _ptr(tex), nx, ny, nz, width, height, quant, _ptr(out))
    return out


def f32_to_f16(x) -> int:
    return int(lib().oracle_f32_to_f16(float(f32(x))))


# ---------------------------------------------------------------------------
#  Model (src/physics.rs:44-218)
# ---------------------------------------------------------------------------
DEFAULT_MODEL = dict(lambda_=0.5, eps_ratio=0.3, alpha=0.1, eta=0.3, phi_b=1.0, dx=1.0,
                     cfl=0.2, seed_kind="critical", seed_value=1.15)


def powi(x, n: int) -> np.float32:
    x = f32(x)
    r = f32(1.0)
    a = x
    while True:
        if n & 1:
            r = f32(r * a)
        n >>= 1
        if n == 0:
            break
        a = f32(a * a)
    return r


def derived(m: dict) -> dict:
    """impl Model (src/physics.rs:85-189) in float32."""
    lam, er, al, eta = f32(m["lambda_"]), f32(m["eps_ratio"]), f32(m["alpha"]), f32(m["eta"])
    phi_b, dx, cfl = f32(m["phi_b"]), f32(m["dx"]), f32(m["cfl"])
    d = {}
    d["eps"] = f32(f32(f32(er * lam) * powi(phi_b, 4)) / f32(12.0))
    d["m2"] = f32(f32(f32(0.5) * lam) * powi(phi_b, 2)) - f32(f32(f32(6.0) * d["eps"]) / powi(phi_b, 2))
    d["delta"] = f32(f32(f32(1.5) * lam) * phi_b) - f32(f32(f32(6.0) * d["eps"]) / powi(phi_b, 3))
    sqrt2 = f32(math.sqrt(2.0))
    d["wall_width"] = f32(f32(f32(2.0) * sqrt2) / f32(phi_b * np.sqrt(lam)))
    d["surface_tension"] = f32(f32(np.sqrt(f32(lam / f32(2.0))) * powi(phi_b, 3)) / f32(6.0))
    d["critical_radius"] = f32(f32(f32(2.0) * d["surface_tension"]) / d["eps"])
    d["e_ref"] = f32(d["eps"] / al)
    d["t_ref"] = f32(1.0)
    d["a_rad"] = f32(d["e_ref"] / powi(d["t_ref"], 4))
    d["dt"] = f32(cfl * dx)
    if m["seed_kind"] == "critical":
        seed = f32(f32(m["seed_value"]) * d["critical_radius"])
    else:
        seed = f32(m["seed_value"])
    d["seed_radius"] = max(seed, f32(f32(0.25) * dx))
    d["critical_to_wall_ratio"] = f32(f32(1.0) / er)
    x = f32(d["eps"] / f32(max(eta, f32(1e-6)) * d["surface_tension"]))
    d["estimated_wall_velocity"] = f32(x / np.sqrt(f32(f32(1.0) + f32(x * x))))
    d["sound_speed"] = np.sqrt(f32(f32(1.0) / f32(3.0)))
    d["p_floor"] = f32(f32(1e-7) * d["e_ref"])
    d["e_floor"] = f32(f32(1e-7) * d["e_ref"])
    d["z_max"] = f32(0.9999)
    return d


def validate(m: dict) -> str | None:
    """Model::validate (src/physics.rs:191-217); None when valid."""
    er = f32(m["eps_ratio"])
    if not (f32(0.0) <= er < f32(1.0)) or er <= 0.0:
        return "eps_ratio must lie in (0, 1)"
    if f32(m["lambda_"]) <= 0.0:
        return "lambda must be positive"
    if f32(m["alpha"]) <= 0.0:
        return "alpha must be positive"
    if f32(m["eta"]) < 0.0:
        return "eta must be non-negative"
    if f32(m["cfl"]) <= 0.0 or f32(m["cfl"]) > f32(0.5):
        return "cfl must lie in (0, 0.5]; see docs/NUMERICS.md"
    if m["seed_kind"] == "critical" and f32(m["seed_value"]) <= 0.0:
        return "seed factor must be positive"
    if m["seed_kind"] == "cells" and f32(m["seed_value"]) <= 0.0:
        return "seed radius must be positive"
    return None


# ---------------------------------------------------------------------------
#  PRNG and schedule (src/physics.rs:243-308)
# ---------------------------------------------------------------------------
M64 = (1 << 64) - 1
M128 = (1 << 128) - 1
MCG_MULT = 47026247687942121848144207491837523525  # PCG default 128-bit multiplier


def _rotr32(x: int, r: int) -> int:
    r &= 31
    return ((x >> r) | (x << (32 - r))) & 0xFFFFFFFF if r else x


def _rotr64(x: int, r: int) -> int:
    r &= 63
    return ((x >> r) | (x << (64 - r))) & M64 if r else x


class Pcg64Mcg:
    def __init__(self, state: int):
        self.state = state | 1

    @classmethod
    def seed_from_u64(cls, s: int) -> "Pcg64Mcg":
        seed = bytearray()
        s &= M64
        for _ in range(4):
            s = (s * 6364136223846793005 + 11634580027462260723) & M64
            xorshifted = (((s >> 18) ^ s) >> 27) & 0xFFFFFFFF
            rot = s >> 59
            seed += _rotr32(xorshifted, rot).to_bytes(4, "little")
        return cls(int.from_bytes(bytes(seed), "little"))

    def next_u64(self) -> int:
        self.state = (self.state * MCG_MULT) & M128
        rot = self.state >> 122
        xsl = ((self.state >> 64) ^ self.state) & M64
        return _rotr64(xsl, rot)

    def next_u32(self) -> int:
        return self.next_u64() & 0xFFFFFFFF

    def next_f32(self) -> np.float32:
        return f32(f32(1.0 / 16777216.0) * f32(self.next_u32() >> 8))


MODES = {"simultaneous": 0, "exponential": 1, "centre": 2, "uniform": 3}


def periodic_distance(a, b, n) -> np.float32:
    s = f32(0.0)
    for i in range(3):
        d = f32(abs(f32(a[i] - b[i])))
        if d > f32(f32(0.5) * n[i]):
            d = f32(n[i] - d)
        s = f32(s + f32(d * d))
    return np.sqrt(s)


def make_schedule(mode: str, count: int, radius, grid, duration, seed: int) -> list[tuple]:
    """Events (time, (x, y, z), radius) as float32, sorted stably by time."""
    rng = Pcg64Mcg.seed_from_u64(seed)
    n = [f32(g) for g in grid]
    radius = f32(radius)
    duration = f32(duration)
    min_sep = f32(f32(2.5) * radius)
    events = []
    for k in range(count):
        t = f32(0.0)
        if mode == "exponential":
            growth = f32(4.0)
            frac = f32(f32(f32(k) + f32(0.5)) / f32(count))
            t = f32(f32(duration / growth) * logf(f32(f32(1.0) + f32(frac * f32(expf(growth) - f32(1.0))))))
        elif mode == "uniform":
            t = f32(rng.next_f32() * duration)
        if mode == "centre":
            pos = (f32(f32(0.5) * n[0]), f32(f32(0.5) * n[1]), f32(f32(0.5) * n[2]))
        else:
            pos = (f32(0.0),) * 3
            for _ in range(64):
                cand = (f32(rng.next_f32() * n[0]), f32(rng.next_f32() * n[1]),
                        f32(rng.next_f32() * n[2]))
                ok = all(periodic_distance(cand, e[1], n) > min_sep for e in events)
                pos = cand
                if ok:
                    break
        events.append((t, pos, radius))
    events.sort(key=lambda e: e[0])  # list.sort is stable
    return events


def stage_slots(cur: int) -> list[tuple[int, int]]:
    a, b, c = cur % 3, (cur + 1) % 3, (cur + 2) % 3
    return [(a, b), (b, c), (c, b)]


RK3_F32 = [(f32(0.0), f32(1.0)), (f32(0.75), f32(0.25)), (f32(f32(1.0) / f32(3.0)), f32(f32(2.0) / f32(3.0)))]
RK3_F64 = [(0.0, 1.0), (0.75, 0.25), (1.0 / 3.0, 2.0 / 3.0)]


# ---------------------------------------------------------------------------
#  Simulation driver over the C kernels
# ---------------------------------------------------------------------------
def thermal_constants(a_rad, gamma, a_cubic):
    """The thermal potential's constants as the library's host rounds them
    (binary32): a/3, gamma, A/3, A, sqrt(3 gamma / (4a)), 1/(2a)."""
    a, g, A = f32(a_rad), f32(gamma), f32(a_cubic)
    return (f32(a / f32(3.0)), g, f32(A / f32(3.0)), A,
            f32(np.sqrt(f32(f32(f32(3.0) * g) / f32(f32(4.0) * a)))), f32(f32(1.0) / f32(f32(2.0) * a)))


def _sim_params(dtype, m: dict, grid, time=0.0) -> np.ndarray:
    d = derived(m)
    fields = [f32(m["dx"]), f32(f32(1.0) / f32(m["dx"])), d["dt"], f32(m["eta"]),
              f32(m["lambda_"]), d["eps"], f32(m["phi_b"]), d["m2"],
              d["delta"], d["a_rad"], d["wall_width"], d["p_floor"],
              d["e_floor"], d["z_max"], d["e_ref"], d["t_ref"],
              f32(time), f32(1.0), f32(0.0), f32(0.0)]
    if dtype == np.float32:
        buf = np.zeros(24, dtype=np.uint32)
        buf[:3] = grid
        buf[4:] = np.array(fields, dtype=np.float32).view(np.uint32)
        return buf
    # FP64 instance: four u32 (16 bytes) then twenty doubles = 22 doubles
    buf = np.zeros(22, dtype=np.float64)
    head = np.zeros(2, dtype=np.uint64)
    h32 = head.view(np.uint32)
    h32[:3] = grid
    buf[:2] = head.view(np.float64)
    buf[2:] = np.array([float(x) for x in fields], dtype=np.float64)
    return buf


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


class OracleSim:
    """CPU restatement of `Simulation` (src/gpu/sim.rs:180-1026)."""

    def __init__(self, grid, model: dict | None = None, schedule=None, precision: str = "f32",
                 eos: tuple = ("bag", 1.0, 0.0), native: bool = False):
        """precision: "f32", "f64", "mixed" (FP32 with the primitive recovery
        redone in FP64 where v^2 > 8/9, include/bubble.h
        BUBBLE_PRECISION_MIXED) or "pert" (the MIXED form with the fluid
        energy stored as E - e_ref, BUBBLE_PRECISION_PERTURBATION).
        eos: ("bag", -, -), ("bag_dof", ratio, -), ("gamma_law", Gamma, e0) or
        ("thermal", gamma, A) (include/bubble.h BUBBLE_EOS_*; the gamma law and
        the thermal potential in FP32 only).  native: run on the native timing
        build of the oracle (the CPU baseline) instead of the parity build."""
        self.L = lib(native)
        self.eos = (eos[0], f32(eos[1]), f32(eos[2]))
        self.gamma = eos[0] == "gamma_law"
        self.thermal = eos[0] == "thermal"
        self.model = dict(DEFAULT_MODEL, **(model or {}))
        err = validate(self.model)
        if err:
            raise ValueError(err)
        self.grid = tuple(int(g) for g in grid)
        self.n = self.grid[0] * self.grid[1] * self.grid[2]
        if precision not in ("f32", "f64", "mixed", "pert"):
            raise ValueError(f"unknown precision {precision!r}")
        self.pert = precision == "pert"
        self.mixed = precision == "mixed"
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.sfx = "f64" if precision == "f64" else "f32"
        self.ksfx = "pert_f32" if self.pert else self.sfx  # kernels that differ in the perturbation form
        self.gsfx = "gamma_f32" if self.gamma else self.ksfx  # kernels that differ for the gamma law
        if self.thermal:  # every kernel but init and nucleation differs for the thermal potential
            self.gsfx = self.ksfx = "thermal_f32"
        # the primitives pass is the one kernel of the MIXED form that differs
        self.psfx = "mixed_f32" if self.mixed else self.gsfx
        if self.mixed and (self.gamma or self.thermal):
            raise ValueError("the MIXED form is the bag model's")
        self.d = derived(self.model)
        self.P = _sim_params(self.dtype, self.model, self.grid)
        self.field = np.zeros((3, self.n, 2), dtype=self.dtype)
        self.fluid = np.zeros((3, self.n, 4), dtype=self.dtype)
        self.prim = np.zeros((self.n, 4), dtype=self.dtype)
        self.schedule = list(schedule or [])
        self.reset()

    # Simulation::reset (src/gpu/sim.rs:790-821)
    def reset(self, schedule=None):
        self.time = f32(0.0)
        self.steps = 0
        self.cur = 0
        self.next_event = 0
        if schedule is not None:
            self.schedule = list(schedule)
        getattr(self.L, f"oracle_init_{self.ksfx}")(_ptr(self.P), _ptr(self.field[0]), _ptr(self.fluid[0]))

    def set_state(self, field: np.ndarray, fluid: np.ndarray):
        self.field[self.cur] = field.reshape(self.n, 2)
        self.fluid[self.cur] = fluid.reshape(self.n, 4)

    def state(self):
        return self.field[self.cur].copy(), self.fluid[self.cur].copy()

    def nucleate(self, bubbles: np.ndarray):
        b = np.ascontiguousarray(bubbles, dtype=np.float32).reshape(-1, 4)
        getattr(self.L, f"oracle_nucleate_{self.sfx}")(_ptr(self.P), _ptr(b), len(b), _ptr(self.field[self.cur]))

    # record_nucleation (src/gpu/sim.rs:843-879)
    def record_nucleation(self):
        batch = []
        while (self.next_event < len(self.schedule) and self.schedule[self.next_event][0] <= self.time
               and len(batch) < 1024):
            t, pos, r = self.schedule[self.next_event]
            batch.append([pos[0], pos[1], pos[2], r])
            self.next_event += 1
        if batch:
            self.nucleate(np.array(batch, dtype=np.float32))

    def stage(self, stage: int, in_slot: int, out_slot: int):
        L = self.L
        self._set_eos()
        a0, a1 = (RK3_F32 if self.dtype == np.float32 else RK3_F64)[stage]
        S = np.array([a0, a1, self.d["dt"], 0.0], dtype=self.dtype)
        getattr(L, f"oracle_primitives_{self.psfx}")(_ptr(self.P), _ptr(self.field[in_slot]),
                                                    _ptr(self.fluid[in_slot]), _ptr(self.prim))
        getattr(L, f"oracle_step_{self.gsfx}")(
            _ptr(self.P), _ptr(S), _ptr(self.field[self.cur]), _ptr(self.fluid[self.cur]),
            _ptr(self.field[in_slot]), _ptr(self.fluid[in_slot]), _ptr(self.prim),
            _ptr(self.field[out_slot]), _ptr(self.fluid[out_slot]))

    def _set_eos(self):
        kind, a, b = self.eos
        c2 = f32(a - f32(1.0)) if kind == "gamma_law" else f32(0.0)
        e0 = b if kind == "gamma_law" else f32(0.0)
        dof = a if kind == "bag_dof" else f32(1.0)
        self.L.oracle_set_eos(float(c2), float(e0), float(dof))
        if kind == "thermal":
            self.L.oracle_set_thermal(*[float(x) for x in thermal_constants(self.d["a_rad"], a, b)])

    # record_step (src/gpu/sim.rs:881-916)
    def record_step(self):
        for stage, (i, o) in enumerate(stage_slots(self.cur)):
            self.stage(stage, i, o)
        self.cur = (self.cur + 1) % 3
        self.time = f32(self.time + self.d["dt"])
        self.steps += 1

    # record_steps (src/gpu/sim.rs:827-841)
    def record_steps(self, n: int):
        self.record_nucleation()
        for _ in range(n):
            self.record_step()

    # headless::advance loop (src/headless.rs:126-131)
    def advance(self, n: int):
        for _ in range(n):
            self.record_steps(1)

    def remaining_bubbles(self) -> int:
        return max(len(self.schedule) - self.next_event, 0)

    # record_visualisation (src/gpu/sim.rs:918-942): primitives pass + vis pass
    def visualise(self) -> np.ndarray:
        """The vis texture of the current slot as (nz, ny, nx, 4) uint16
        (binary16 bits of phi/phi_b, |v|, T/T_ref - 1, (E+p)v^2/e_ref)."""
        L = self.L
        self._set_eos()
        getattr(L, f"oracle_primitives_{self.psfx}")(_ptr(self.P), _ptr(self.field[self.cur]),
                                                    _ptr(self.fluid[self.cur]), _ptr(self.prim))
        nx, ny, nz = self.grid
        out = np.zeros((nz, ny, nx, 4), dtype=np.uint16)
        getattr(L, f"oracle_vis_{self.ksfx}")(_ptr(self.P), _ptr(self.field[self.cur]),
                                             _ptr(self.fluid[self.cur]), _ptr(self.prim), _ptr(out))
        return out

    # record_visualisation's primitives pass + reduce (src/gpu/sim.rs:918-1010)
    def diagnostics(self) -> dict:
        L = self.L
        self._set_eos()
        getattr(L, f"oracle_primitives_{self.psfx}")(_ptr(self.P), _ptr(self.field[self.cur]),
                                                    _ptr(self.fluid[self.cur]), _ptr(self.prim))
        sums = np.zeros(4, dtype=np.float64)
        vmax = np.zeros(1, dtype=self.dtype)
        getattr(L, f"oracle_reduce_{self.ksfx}")(_ptr(self.P), _ptr(self.field[self.cur]),
                                                _ptr(self.fluid[self.cur]), _ptr(self.prim),
                                                _ptr(sums), _ptr(vmax))
        n = self.n
        if self.pert:  # the kernel summed E - e_ref: add the background in FP64
            sums[0] += float(self.d["e_ref"]) * n
            sums[3] += float(self.d["e_ref"]) * n
        inv_n = f32(f32(1.0) / f32(n))
        out = dict(sum_energy=sums[0], sum_broken=sums[1], sum_kinetic=sums[2],
                   sum_fluid_energy=sums[3], max_velocity=float(vmax[0]),
                   mean_energy_f64=sums[0] / n, mean_kinetic_f64=sums[2] / n)
        out["mean_energy"] = float(f32(f32(sums[0]) * inv_n))
        out["broken_fraction"] = float(f32(f32(sums[1]) * inv_n))
        out["mean_kinetic"] = float(f32(f32(sums[2]) * inv_n))
        me = f32(out["mean_energy"])
        out["kinetic_fraction"] = 0.0 if abs(me) < 1e-20 else float(f32(f32(out["mean_kinetic"]) / me))
        return out
