"""NCBI BLAST protein database volumes (.pin index + .psq sequences).

``write_volume`` writes residues/offsets as a version 4 (or 5) protein volume
in the layout libblaze103's reader takes (see csrc/volume.cpp): big-endian
index integers, the total length as 8 little-endian bytes, sequences in
NCBIstdaa each followed by a 0 byte after a leading 0 byte. Header (.phr)
records are written empty: the preliminary search stage reads no deflines.
``read_volume`` reads one back on the host through the library
(blaze_volume_info / blaze_volume_read); ``SeqSrc.open`` loads one straight
into the device database.
"""
from __future__ import annotations

import ctypes
import os
import struct
import time

import numpy as np

from ._lib import check, load, u8ptr, u64ptr


def _string(b: bytes) -> bytes:
    return struct.pack(">I", len(b)) + b


def write_volume(path: str, residues, offsets, title: str = "blaze synthetic", version: int = 4) -> None:
    """Writes <path>.pin, <path>.psq and an empty-header <path>.phr."""
    res = np.ascontiguousarray(residues, dtype=np.uint8)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    n = off.size - 1
    lens = (off[1:] - off[:-1]).astype(np.int64)
    seq_off = np.zeros(n + 1, dtype=np.int64)
    seq_off[0] = 1  # leading 0 byte
    np.cumsum(lens + 1, out=seq_off[1:])
    seq_off[1:] += 1
    if seq_off[-1] >= 1 << 32:
        raise ValueError("a volume holds at most 4 GiB of sequence data")
    psq = np.zeros(int(seq_off[-1]), dtype=np.uint8)
    for i in range(n):
        a, b = int(off[i]), int(off[i + 1])
        psq[int(seq_off[i]):int(seq_off[i]) + (b - a)] = res[a:b]
    hdr = bytearray()
    hdr += struct.pack(">II", version, 1)
    if version == 5:
        hdr += struct.pack(">I", 0)  # volume number
    hdr += _string(title.encode())
    if version == 5:
        hdr += _string(b"")  # LMDB file name
    hdr += _string(time.strftime("%b %d, %Y  %I:%M %p").encode())
    hdr += struct.pack(">I", n) + struct.pack("<Q", int(lens.sum())) + struct.pack(">I", int(lens.max(initial=0)))
    hdr += np.zeros(n + 1, dtype=">u4").tobytes()  # header offsets: all empty
    hdr += seq_off.astype(">u4").tobytes()
    with open(path + ".pin", "wb") as f:
        f.write(bytes(hdr))
    with open(path + ".psq", "wb") as f:
        f.write(psq.tobytes())
    with open(path + ".phr", "wb") as f:
        f.write(b"")


def volume_info(path: str) -> dict:
    n, tot, mx = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint32()
    check(load().blaze_volume_info(os.fsencode(path), ctypes.byref(n), ctypes.byref(tot), ctypes.byref(mx)),
          "blaze_volume_info")
    return {"n_subjects": n.value, "total_residues": tot.value, "max_length": mx.value}


def read_volume(path: str):
    """(residues, offsets) of a volume, read by the library on the host."""
    info = volume_info(path)
    res = np.zeros(max(info["total_residues"], 1), dtype=np.uint8)
    off = np.zeros(info["n_subjects"] + 1, dtype=np.uint64)
    check(load().blaze_volume_read(os.fsencode(path), u8ptr(res), info["total_residues"], u64ptr(off)),
          "blaze_volume_read")
    return res[: info["total_residues"]], off
