"""Host side of the headless visualisation, on the CPU.

The reference's own renderer and camera unit tests (src/camera.rs:107-137,
src/gpu/render.rs:404-420, src/config.rs:209-215), restated against the
library's C ABI; the PNG writer decoded independently with zlib; the
oracle's binary16 rounding against numpy's; and the oracle's ray-march on a
constructed texture against closed-form pixels.
"""
from __future__ import annotations

import ctypes
import struct
import subprocess
import zlib

import numpy as np
import pytest

from conftest import PKG


def cam_call(bubble, name, c, *args):
    bubble._lib.check(getattr(bubble.load(), name)(ctypes.byref(c), *args))


def eye_of(bubble, c):
    out = (ctypes.c_float * 3)()
    cam_call(bubble, "bubble_camera_eye", c, out)
    return np.array(out[:], dtype=np.float64)


def basis_of(bubble, c):
    r, u, f = (ctypes.c_float * 3)(), (ctypes.c_float * 3)(), (ctypes.c_float * 3)()
    cam_call(bubble, "bubble_camera_basis", c, r, u, f)
    return [np.array(x[:], dtype=np.float64) for x in (r, u, f)]


def view_proj(bubble, c, aspect):
    out = (ctypes.c_float * 16)()
    cam_call(bubble, "bubble_camera_view_proj", c, ctypes.c_float(aspect), out)
    return np.array(out[:], dtype=np.float64).reshape(4, 4).T  # column-major -> row-major


# src/camera.rs:113-116
def test_eye_sits_at_the_requested_distance(bubble):
    c = bubble.camera()
    e = eye_of(bubble, c)
    assert abs(np.linalg.norm(e - np.array(c.target[:])) - c.distance) < 1e-5


# src/camera.rs:118-128
def test_pitch_is_clamped_short_of_the_pole(bubble):
    c = bubble.camera()
    cam_call(bubble, "bubble_camera_orbit", c, ctypes.c_float(0.0), ctypes.c_float(100.0))
    assert np.float32(c.pitch) <= np.float32(1.5533)
    cam_call(bubble, "bubble_camera_orbit", c, ctypes.c_float(0.0), ctypes.c_float(-200.0))
    assert np.float32(c.pitch) >= np.float32(-1.5533)
    r, u, _ = basis_of(bubble, c)
    assert np.linalg.norm(r) > 0.5 and np.linalg.norm(u) > 0.5


# src/camera.rs:130-137
def test_zoom_stays_positive(bubble):
    c = bubble.camera()
    for _ in range(200):
        cam_call(bubble, "bubble_camera_zoom", c, ctypes.c_float(5.0))
    assert c.distance > 0.0


# src/camera.rs:139-145
def test_projection_maps_the_target_to_the_screen_centre(bubble):
    c = bubble.camera()
    clip = view_proj(bubble, c, 1.6) @ np.array(list(c.target[:]) + [1.0])
    ndc = clip[:3] / clip[3]
    assert abs(ndc[0]) < 1e-4 and abs(ndc[1]) < 1e-4


def test_pan_and_dolly_move_the_target_in_the_camera_frame(bubble):
    c = bubble.camera()
    r, u, f = basis_of(bubble, c)
    cam_call(bubble, "bubble_camera_pan", c, ctypes.c_float(0.1), ctypes.c_float(0.0))
    np.testing.assert_allclose(np.array(c.target[:]), -0.1 * c.distance * 0.9 * r, atol=1e-6)
    c2 = bubble.camera()
    cam_call(bubble, "bubble_camera_dolly", c2, ctypes.c_float(0.5))
    np.testing.assert_allclose(np.array(c2.target[:]), 0.5 * c2.distance * f, atol=1e-6)


# src/gpu/render.rs:406-410
def test_view_uniform_matches_the_wgsl_struct(bubble):
    assert ctypes.sizeof(bubble._lib.View) == 176
    assert ctypes.sizeof(bubble._lib.RenderSettings) == 14 * 4


# src/gpu/render.rs:412-419
def test_every_field_mode_has_a_valid_default_colormap(bubble):
    for name, mode in bubble._lib.FIELDS.items():
        s = bubble.render_settings(name)
        assert s.field_mode == mode
        assert 0 <= s.colormap < len(bubble._lib.COLORMAPS)
        assert s.field_gain > 0.0
    d = bubble.render_settings()
    assert (d.field_mode, d.colormap, d.field_gain) == (3, 1, 20.0)
    assert (d.iso_level, d.absorption, d.clip_axis) == (pytest.approx(0.5), 12.0, -1)


def test_view_uniform_contents(bubble):
    s = bubble.render_settings("temperature")
    v = bubble.render_view((64, 32, 16), s, (320, 240), frame=1)
    # box normalised so the longest axis spans 1, w = one cell
    np.testing.assert_allclose(v[20:24], [0.5, 0.25, 0.125, 1.0 / 64], rtol=1e-7)
    np.testing.assert_allclose(v[24:27], [64, 32, 16])
    assert v[40] == np.float32(0.618034)  # frame 1 dither offset
    assert bubble.render_view((8, 8, 8), s, (4, 4), frame=65)[40] == np.float32(0.618034)
    # inv_view_proj inverts the framed camera's view_proj
    c = bubble.camera((0.5, 0.25, 0.125))
    vp = view_proj(bubble, c, 320 / 240)
    inv = v[:16].astype(np.float64).reshape(4, 4).T
    # entries of the inverse reach ~800 (near plane 0.002): f32 rounding of those
    np.testing.assert_allclose(inv @ vp, np.eye(4), atol=5e-4)
    # the eye of the framed camera
    np.testing.assert_allclose(v[16:19], eye_of(bubble, c), rtol=1e-6)


def test_view_rejects_bad_settings(bubble):
    s = bubble.render_settings()
    s.clip_axis = 3
    with pytest.raises(bubble.BubbleError):
        bubble.render_view((8, 8, 8), s, (4, 4))
    s = bubble.render_settings()
    with pytest.raises(bubble.BubbleError):
        bubble.render_view((8, 8, 8), s, (0, 4))


def decode_png(data: bytes):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF, typ
        chunks.append((typ, body))
        pos += 12 + n
    assert chunks[0][0] == b"IHDR" and chunks[-1][0] == b"IEND"
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 6, 0, 0, 0)
    raw = zlib.decompress(b"".join(b for t, b in chunks if t == b"IDAT"))
    rows = np.frombuffer(raw, dtype=np.uint8).reshape(h, 1 + 4 * w)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 4)


@pytest.mark.parametrize("size", [(1, 1), (37, 5), (300, 250)])
def test_png_writer_round_trip(bubble, tmp_path, size):
    w, h = size
    img = np.random.default_rng(w * h).integers(0, 256, size=(h, w, 4), dtype=np.uint8)
    path = tmp_path / "x.png"
    bubble.write_png(str(path), img)
    np.testing.assert_array_equal(decode_png(path.read_bytes()), img)


# parse_size (src/config.rs:209-215), through the CLI's argument parser
@pytest.mark.parametrize("arg,ok", [("1920x1080", True), ("800X600", True), ("1920", False), ("0x600", False),
                                    ("12xq", False)])
def test_screenshot_size_parsing(bubble, arg, ok):
    cli = PKG / "lib" / "bubble-sim"
    r = subprocess.run([str(cli), "--screenshot-size", arg, "--help"], capture_output=True, text=True)
    assert (r.returncode == 0) == ok, r.stderr
    if not ok:
        assert "--screenshot-size" in r.stderr


def test_cli_rejects_unknown_field(bubble):
    cli = PKG / "lib" / "bubble-sim"
    r = subprocess.run([str(cli), "--field", "colour", "--help"], capture_output=True, text=True)
    assert r.returncode == 2 and "--field" in r.stderr


def test_oracle_half_rounding_matches_numpy(oracle_mod):
    rng = np.random.default_rng(7)
    xs = np.concatenate([
        rng.standard_normal(4000).astype(np.float32) * np.float32(10.0) ** rng.integers(-9, 6, 4000).astype(np.float32),
        np.array([0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e9, -1e9, 6.1e-5, 5.96e-8, 2.98e-8, 2.99e-8, 1e-12,
                  np.inf, -np.inf], dtype=np.float32),
        # exact ties between two halves
        (np.arange(1, 400, dtype=np.float32) + np.float32(0.5)) * np.float32(2.0 ** -10),
    ]).astype(np.float32)
    got = np.array([oracle_mod.f32_to_f16(x) for x in xs], dtype=np.uint16)
    with np.errstate(over="ignore"):
        want = xs.astype(np.float16).view(np.uint16)
    np.testing.assert_array_equal(got, want)


def test_oracle_render_background_and_empty_box(bubble, oracle_mod):
    """A zero texture with the wall and volume switched off leaves the
    background gradient (shaders/volume.wgsl:240-243), tonemapped."""
    n = 8
    tex = np.zeros((n, n, n, 4), dtype=np.uint16)
    s = bubble.render_settings()
    s.show_iso = 0
    s.show_volume = 0
    s.show_box = 0
    w, h = 24, 18
    v = bubble.render_view((n, n, n), s, (w, h))
    img = oracle_mod.render(v, tex, w, h)
    assert (img[..., 3] == 255).all()
    # reconstruct the background per pixel in float64
    M = v[:16].astype(np.float64).reshape(4, 4).T
    ro = v[16:19].astype(np.float64)
    for py in (0, h // 2, h - 1):
        for px in (0, w // 2, w - 1):
            ndc = np.array([(px + 0.5) / w * 2 - 1, 1 - (py + 0.5) / h * 2, 1.0, 1.0])
            far = M @ ndc
            rd = far[:3] / far[3] - ro
            rd /= np.linalg.norm(rd)
            t = np.clip(rd[1] * 0.5 + 0.5, 0, 1)
            c = np.array([0.015, 0.017, 0.028]) * (1 - t) + np.array([0.045, 0.055, 0.085]) * t
            c = (c / (1 + c)) ** (1 / 2.2)
            assert np.abs(img[py, px, :3].astype(float) - np.round(c * 255)).max() <= 1, (px, py)
