"""Checkpoint files on the CPU: the library's reader checks magic, header
consistency, size and CRC-32 before touching any device state.  The file is
built here from the layout documented in include/bubble_checkpoint.h and
csrc/checkpoint.cpp."""
from __future__ import annotations

import ctypes
import struct
import zlib

import numpy as np
import pytest


def header_type(bubble):
    class Header(ctypes.Structure):
        _fields_ = [("spec", bubble._lib.Spec), ("time", ctypes.c_float), ("field_bytes", ctypes.c_uint32),
                    ("steps", ctypes.c_uint64), ("next_event", ctypes.c_uint64), ("n_events", ctypes.c_uint64),
                    ("cells", ctypes.c_uint64), ("fluid_bytes", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]
    return Header


def make_file(bubble, grid=(8, 9, 10), precision="single", events=((1.5, (1.0, 2.0, 3.0), 4.0),), next_event=0):
    spec = bubble.SimulationSpec(grid=grid, precision=precision, nucleation="uniform", bubbles=len(events))
    H = header_type(bubble)
    f64 = precision == "double"
    cells = grid[0] * grid[1] * grid[2]
    h = H(spec.c(), 12.25, 16 if f64 else 8, 61, next_event, len(events), cells, 32 if f64 else 16, 0)
    body = b"BUBCKPT1" + struct.pack("<I", ctypes.sizeof(H)) + bytes(h)
    for t, pos, r in events:
        body += struct.pack("<fffff", t, *pos, r)
    dt = np.float64 if f64 else np.float32
    rng = np.random.default_rng(3)
    body += rng.standard_normal(cells * 2).astype(dt).tobytes() + rng.standard_normal(cells * 4).astype(dt).tobytes()
    return body + struct.pack("<I", zlib.crc32(body) & 0xFFFFFFFF)


def read_spec(bubble, path):
    return bubble.checkpoint_spec(str(path))


@pytest.mark.parametrize("precision", ["single", "mixed", "double"])
def test_valid_file_spec(bubble, tmp_path, precision):
    p = tmp_path / "a.ckpt"
    p.write_bytes(make_file(bubble, precision=precision))
    s = read_spec(bubble, p)
    assert s.grid == (8, 9, 10) and s.precision == precision and s.nucleation == "uniform"


@pytest.mark.parametrize("damage", ["magic", "crc", "truncate", "extend", "header_size", "next_event", "cells"])
def test_damaged_files_are_rejected(bubble, tmp_path, damage):
    data = bytearray(make_file(bubble))
    H = header_type(bubble)
    if damage == "magic":
        data[0:8] = b"NOTACKPT"
    elif damage == "crc":
        data[200] ^= 0x01
    elif damage == "truncate":
        data = data[:-100]
    elif damage == "extend":
        data += b"\0" * 16
    elif damage == "header_size":
        data[8:12] = struct.pack("<I", ctypes.sizeof(H) + 8)
    else:
        h = H.from_buffer_copy(bytes(data[12:12 + ctypes.sizeof(H)]))
        if damage == "next_event":
            h.next_event = h.n_events + 1
        else:
            h.cells += 1
        data[12:12 + ctypes.sizeof(H)] = bytes(h)
        body = bytes(data[:-4])
        data[-4:] = struct.pack("<I", zlib.crc32(body) & 0xFFFFFFFF)
    p = tmp_path / "bad.ckpt"
    p.write_bytes(bytes(data))
    with pytest.raises(bubble.BubbleError) as e:
        read_spec(bubble, p)
    assert e.value.code == bubble._lib.ERR_INVALID


def test_missing_file(bubble, tmp_path):
    with pytest.raises(bubble.BubbleError):
        read_spec(bubble, tmp_path / "none.ckpt")
