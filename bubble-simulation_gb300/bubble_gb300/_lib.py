"""ctypes declarations of include/bubble*.h.

Loads lib/libbubble_gb300.so from this package's source tree.  There is no
fallback: if the library has not been built, loading raises with the build
command to run.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "lib" / "libbubble_gb300.so"
CLI_PATH = PKG_ROOT / "lib" / "bubble-sim"

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_MEMORY = -3
ERR_NONFINITE = -4
ERR_STATE = -5
ERR_TIMEOUT = -6

SEED_CRITICAL = 0
SEED_CELLS = 1
NUCLEATION = {"simultaneous": 0, "exponential": 1, "centre": 2, "uniform": 3}
PRECISION = {"single": 0, "mixed": 1, "double": 2, "perturbation": 3}
MATH = {"fast": 0, "strict": 1}
EOS = {"bag": 0, "bag_dof": 1, "gamma_law": 2, "thermal": 3}
PATH_FUSED = 0
PATH_REFERENCE = 1
PATHS = {"fused": PATH_FUSED, "reference": PATH_REFERENCE}
STAGE_FORMS = {"auto": 0, "registers": 1, "shared": 2}
MIN_GRID = 8
MAX_GRID = 2048
MAX_BATCH = 1024


class Model(ctypes.Structure):
    _fields_ = [("lambda_", ctypes.c_float), ("eps_ratio", ctypes.c_float),
                ("alpha", ctypes.c_float), ("eta", ctypes.c_float), ("phi_b", ctypes.c_float),
                ("dx", ctypes.c_float), ("cfl", ctypes.c_float), ("seed_kind", ctypes.c_int32),
                ("seed_value", ctypes.c_float)]


class Derived(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in (
        "eps", "m2", "delta", "wall_width", "surface_tension", "critical_radius", "e_ref",
        "t_ref", "a_rad", "dt", "seed_radius", "critical_to_wall_ratio",
        "estimated_wall_velocity", "sound_speed", "p_floor", "e_floor", "z_max")]


class Event(ctypes.Structure):
    _fields_ = [("time", ctypes.c_float), ("pos", ctypes.c_float * 3), ("radius", ctypes.c_float)]


class Spec(ctypes.Structure):
    _fields_ = [("model", Model), ("grid", ctypes.c_uint32 * 3), ("nucleation", ctypes.c_int32),
                ("bubbles", ctypes.c_uint64), ("nucleation_duration", ctypes.c_float),
                ("seed", ctypes.c_uint64), ("precision", ctypes.c_int32), ("math", ctypes.c_int32),
                ("eos", ctypes.c_int32), ("eos_param", ctypes.c_float * 2)]


class Diag(ctypes.Structure):
    _fields_ = [("mean_energy", ctypes.c_float), ("broken_fraction", ctypes.c_float),
                ("mean_kinetic", ctypes.c_float), ("mean_fluid_energy", ctypes.c_float),
                ("max_velocity", ctypes.c_float), ("kinetic_fraction", ctypes.c_float),
                ("sum_energy", ctypes.c_double), ("sum_broken", ctypes.c_double),
                ("sum_kinetic", ctypes.c_double), ("sum_fluid_energy", ctypes.c_double),
                ("mean_energy_f64", ctypes.c_double), ("mean_kinetic_f64", ctypes.c_double),
                ("cells", ctypes.c_uint64)]


class BatchOptions(ctypes.Structure):
    _fields_ = [("tile_y", ctypes.c_int32), ("autotune", ctypes.c_int32), ("use_graph", ctypes.c_int32),
                ("max_grid", ctypes.c_int32)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("lattices", ctypes.c_uint32), ("grid", ctypes.c_uint32), ("items", ctypes.c_uint32),
                ("tile_y", ctypes.c_int32), ("graph", ctypes.c_int32), ("autotuned", ctypes.c_int32),
                ("cells", ctypes.c_uint64), ("launches", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("math", ctypes.c_int32), ("tile_y", ctypes.c_int32), ("chunk_steps", ctypes.c_uint32),
                ("max_active", ctypes.c_uint32), ("memory_fraction", ctypes.c_float), ("use_graph", ctypes.c_int32),
                ("resident_cells", ctypes.c_uint64), ("policy", ctypes.c_int32), ("chunk_planes", ctypes.c_uint32)]


SERVE_POLICY = {"fifo": 0, "shortest": 1}


class ServerResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int32), ("grid", ctypes.c_uint32 * 3),
                ("steps", ctypes.c_uint64), ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("done_s", ctypes.c_double), ("diag", Diag)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "admitted", "completed", "queued", "active", "rounds")] + \
               [(n, ctypes.c_double) for n in ("p50_latency_s", "p99_latency_s", "mean_latency_s", "solves_per_s",
                                               "cell_updates")]


class VramInfo(ctypes.Structure):
    _fields_ = [("capacity", ctypes.c_uint64), ("budget", ctypes.c_uint64),
                ("used", ctypes.c_uint64), ("has_budget", ctypes.c_int32)]


FIELDS = {"phi": 0, "speed": 1, "temperature": 2, "kinetic": 3}
COLORMAPS = {"viridis": 0, "inferno": 1, "signed": 2}


class RenderSettings(ctypes.Structure):
    _fields_ = [("field_mode", ctypes.c_int32), ("colormap", ctypes.c_int32), ("iso_level", ctypes.c_float),
                ("wall_opacity", ctypes.c_float), ("samples_per_cell", ctypes.c_float), ("exposure", ctypes.c_float),
                ("field_gain", ctypes.c_float), ("absorption", ctypes.c_float), ("show_iso", ctypes.c_int32),
                ("show_volume", ctypes.c_int32), ("show_box", ctypes.c_int32), ("background", ctypes.c_float),
                ("clip_axis", ctypes.c_int32), ("clip_pos", ctypes.c_float)]


class Camera(ctypes.Structure):
    _fields_ = [("target", ctypes.c_float * 3), ("distance", ctypes.c_float), ("yaw", ctypes.c_float),
                ("pitch", ctypes.c_float), ("fov_y", ctypes.c_float), ("znear", ctypes.c_float),
                ("zfar", ctypes.c_float)]


class View(ctypes.Structure):
    _fields_ = [("inv_view_proj", ctypes.c_float * 16)] + \
               [(n, ctypes.c_float * 4) for n in ("cam_pos", "box_half", "grid", "render0", "render1", "render2",
                                                  "render3")]


# (name, restype, argtypes) of every exported symbol declared in include/*.h
_P = ctypes.c_void_p
_U32P = ctypes.POINTER(ctypes.c_uint32)
_U64P = ctypes.POINTER(ctypes.c_uint64)
_I32P = ctypes.POINTER(ctypes.c_int32)
_F32P = ctypes.POINTER(ctypes.c_float)
SIGNATURES = [
    ("bubble_model_default", None, [ctypes.POINTER(Model)]),
    ("bubble_model_validate", ctypes.c_int, [ctypes.POINTER(Model)]),
    ("bubble_model_derived", ctypes.c_int, [ctypes.POINTER(Model), ctypes.POINTER(Derived)]),
    ("bubble_eos_validate", ctypes.c_int, [ctypes.POINTER(Spec)]),
    ("bubble_make_schedule", ctypes.c_int, [ctypes.c_int32, ctypes.c_uint64, ctypes.c_float, _U32P,
                                            ctypes.c_float, ctypes.c_uint64, ctypes.POINTER(Event),
                                            ctypes.c_uint64, _U64P]),
    ("bubble_spec_default", None, [ctypes.POINTER(Spec)]),
    ("bubble_stage_slots", ctypes.c_int, [ctypes.c_uint32, _U32P]),
    ("bubble_rk3_coefficients", None, [ctypes.POINTER(ctypes.c_float)]),
    ("bubble_lattice_bytes", ctypes.c_uint64, [_U32P]),
    ("bubble_bytes_per_cell", ctypes.c_uint64, [ctypes.c_int32]),
    ("bubble_max_cubic_size", ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, _U32P, _I32P]),
    ("bubble_vram_query", ctypes.c_int, [ctypes.POINTER(VramInfo)]),
    ("bubble_vram_available", ctypes.c_uint64, [ctypes.POINTER(VramInfo)]),
    ("bubble_lattice_budget", ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_uint64]),
    ("bubble_create", ctypes.c_int, [ctypes.POINTER(Spec), ctypes.POINTER(_P)]),
    ("bubble_destroy", None, [_P]),
    ("bubble_set_stream", ctypes.c_int, [_P, _P]),
    ("bubble_reset", ctypes.c_int, [_P, ctypes.POINTER(Event), ctypes.c_uint64]),
    ("bubble_set_model", ctypes.c_int, [_P, ctypes.POINTER(Model)]),
    ("bubble_resize", ctypes.c_int, [_P, _U32P]),
    ("bubble_record_steps", ctypes.c_int, [_P, ctypes.c_uint32]),
    ("bubble_advance", ctypes.c_int, [_P, ctypes.c_uint64]),
    ("bubble_diagnostics", ctypes.c_int, [_P, ctypes.POINTER(Diag)]),
    ("bubble_nucleate_now", ctypes.c_int, [_P, ctypes.c_uint64]),
    ("bubble_synchronize", ctypes.c_int, [_P]),
    ("bubble_time", ctypes.c_float, [_P]),
    ("bubble_steps", ctypes.c_uint64, [_P]),
    ("bubble_cell_count", ctypes.c_uint64, [_P]),
    ("bubble_remaining_bubbles", ctypes.c_uint64, [_P]),
    ("bubble_device_memory_bytes", ctypes.c_uint64, [_P]),
    ("bubble_get_grid", ctypes.c_int, [_P, _U32P]),
    ("bubble_get_model", ctypes.c_int, [_P, ctypes.POINTER(Model)]),
    ("bubble_get_schedule", ctypes.c_int, [_P, ctypes.POINTER(Event), ctypes.c_uint64, _U64P]),
    ("bubble_copy_state", ctypes.c_int, [_P, _P, _P]),
    ("bubble_load_state", ctypes.c_int, [_P, _P, _P]),
    ("bubble_copy_state_f64", ctypes.c_int, [_P, _P, _P]),
    ("bubble_load_state_f64", ctypes.c_int, [_P, _P, _P]),
    ("bubble_version", ctypes.c_char_p, []),
    ("bubble_last_error", ctypes.c_char_p, []),
    # bubble_ext.h
    ("bubble_ext_set_path", ctypes.c_int, [_P, ctypes.c_int32]),
    ("bubble_ext_set_tile", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    ("bubble_ext_get_tile", ctypes.c_int, [_P, _I32P, _I32P]),
    ("bubble_ext_set_stage_form", ctypes.c_int, [_P, ctypes.c_int32]),
    ("bubble_ext_device_state", ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    ("bubble_ext_stream", _P, [_P]),
    ("bubble_ext_launches", ctypes.c_uint64, [_P]),
    ("bubble_ext_inject_allocation_failure", None, []),
    ("bubble_ext_test_expire_stage_wait", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_int32]),
    ("bubble_ext_test_expire_batch_barrier", ctypes.c_int, [_P, ctypes.c_int32]),
    ("bubble_diagnostics_noalloc", ctypes.c_int, [_P, _P, ctypes.POINTER(Spec), _P, _P]),
    # bubble_batch.h
    ("bubble_batch_options_default", None, [ctypes.POINTER(BatchOptions)]),
    ("bubble_batch_create", ctypes.c_int, [ctypes.POINTER(Spec), ctypes.c_uint32, ctypes.POINTER(BatchOptions),
                                           ctypes.POINTER(_P)]),
    ("bubble_batch_destroy", None, [_P]),
    ("bubble_batch_advance", ctypes.c_int, [_P, ctypes.c_uint64]),
    ("bubble_batch_diagnostics", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.POINTER(Diag)]),
    ("bubble_batch_copy_state", ctypes.c_int, [_P, ctypes.c_uint32, _P, _P]),
    ("bubble_batch_load_state", ctypes.c_int, [_P, ctypes.c_uint32, _P, _P]),
    ("bubble_batch_info_get", ctypes.c_int, [_P, ctypes.POINTER(BatchInfo)]),
    ("bubble_batch_time", ctypes.c_float, [_P, ctypes.c_uint32]),
    ("bubble_autotune_chunk", ctypes.c_int, [_U32P, ctypes.c_int32, ctypes.c_int32, _I32P]),
    # bubble_server.h
    ("bubble_server_options_default", None, [ctypes.POINTER(ServerOptions)]),
    ("bubble_server_create", ctypes.c_int, [ctypes.POINTER(ServerOptions), ctypes.POINTER(_P)]),
    ("bubble_server_destroy", None, [_P]),
    ("bubble_server_submit", ctypes.c_int, [_P, ctypes.POINTER(Spec), ctypes.c_uint64, _U64P]),
    ("bubble_server_tick", ctypes.c_int, [_P, _I32P]),
    ("bubble_server_run_until_idle", ctypes.c_int, [_P]),
    ("bubble_server_poll", ctypes.c_int, [_P, ctypes.POINTER(ServerResult), ctypes.c_uint64, _U64P]),
    ("bubble_server_stats_get", ctypes.c_int, [_P, ctypes.POINTER(ServerStats)]),
    ("bubble_server_now", ctypes.c_double, [_P]),
    # bubble_render.h
    ("bubble_render_settings_default", ctypes.c_int, [ctypes.POINTER(RenderSettings)]),
    ("bubble_render_settings_with_field", ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(RenderSettings)]),
    ("bubble_camera_default", ctypes.c_int, [ctypes.POINTER(Camera)]),
    ("bubble_camera_frame_box", ctypes.c_int, [ctypes.POINTER(Camera), _F32P]),
    ("bubble_camera_orbit", ctypes.c_int, [ctypes.POINTER(Camera), ctypes.c_float, ctypes.c_float]),
    ("bubble_camera_pan", ctypes.c_int, [ctypes.POINTER(Camera), ctypes.c_float, ctypes.c_float]),
    ("bubble_camera_zoom", ctypes.c_int, [ctypes.POINTER(Camera), ctypes.c_float]),
    ("bubble_camera_dolly", ctypes.c_int, [ctypes.POINTER(Camera), ctypes.c_float]),
    ("bubble_camera_eye", ctypes.c_int, [ctypes.POINTER(Camera), _F32P]),
    ("bubble_camera_basis", ctypes.c_int, [ctypes.POINTER(Camera), _F32P, _F32P, _F32P]),
    ("bubble_camera_view_proj", ctypes.c_int, [ctypes.POINTER(Camera), ctypes.c_float, _F32P]),
    ("bubble_render_box", ctypes.c_int, [_U32P, _F32P, _F32P]),
    ("bubble_render_view", ctypes.c_int, [_U32P, ctypes.POINTER(RenderSettings), ctypes.POINTER(Camera),
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(View)]),
    ("bubble_visualise", ctypes.c_int, [_P]),
    ("bubble_vis_copy", ctypes.c_int, [_P, _P]),
    ("bubble_render", ctypes.c_int, [_P, ctypes.POINTER(RenderSettings), ctypes.POINTER(Camera), ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_uint32, _P]),
    ("bubble_render_png", ctypes.c_int, [_P, ctypes.POINTER(RenderSettings), ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_char_p]),
    ("bubble_write_png", ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_uint32, ctypes.c_uint32]),
    # bubble_checkpoint.h
    ("bubble_checkpoint_save", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("bubble_checkpoint_restore", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("bubble_checkpoint_spec", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Spec)]),
    ("bubble_checkpoint_open", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P)]),
]

_lib = None


class BubbleError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code
        self.message = message


def load() -> ctypes.CDLL:
    """Load the in-tree library (build it with `python bubble-simulation_gb300/build.py`)."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("BUBBLE_GB300_LIB", LIB_PATH))
    if not path.exists():
        raise ImportError(f"{path} is missing: build it with "
                          f"`python {PKG_ROOT / 'build.py'}` (there is no CPU fallback)")
    L = ctypes.CDLL(str(path))
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != OK:
        raise BubbleError(rc, load().bubble_last_error().decode())
