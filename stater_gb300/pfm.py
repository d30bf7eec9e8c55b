"""PFM files of statistics buffers with the reference's naming.

The reference writes every registered buffer as ``<stem>[-<suffix>]-<name>.pfm``
(OutputBufferSelection::Write, src/statistics/buffer.cpp:48-63) and a
denoise-only run reads ``<stem>-<spp>-film.pfm`` and
``<stem>-<spp>-t<T>-b<j>-<suffix>.pfm`` back (statpath.cpp:506-547), where the
suffix is ``film-<name>`` for the untransformed set and ``<name>`` for the
transformed one. Arrays here are planar ``[channels, height, width]`` with row 0
at the top; files store interleaved channels, rows bottom to top, as PFM does.
The C++ side of the same format is stater_gb300/host/pfm.hpp.
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np


def write_pfm(path, img) -> None:
    """Writes a [3, H, W] or [H, W] / [1, H, W] array as float32 PFM."""
    a = np.asarray(img, dtype=np.float32)
    if a.ndim == 2:
        a = a[None]
    if a.ndim != 3 or a.shape[0] not in (1, 3):
        raise ValueError("PFM images have 1 or 3 channels")
    C, H, W = a.shape
    le = sys.byteorder == "little"
    with open(path, "wb") as f:
        f.write(f"{'PF' if C == 3 else 'Pf'}\n{W} {H}\n{'-1.0' if le else '1.0'}\n".encode())
        f.write(np.ascontiguousarray(a[:, ::-1].transpose(1, 2, 0)).tobytes())


def read_pfm(path) -> np.ndarray:
    """Reads a PFM file into a planar float32 array [C, H, W]."""
    with open(path, "rb") as f:
        data = f.read()
    toks, pos = [], 0
    while len(toks) < 4:
        m = re.compile(rb"\s*(\S+)\s").match(data, pos)
        if m is None:
            raise ValueError(f"{path}: bad PFM header")
        toks.append(m.group(1))
        pos = m.end()
    magic, w, h, scale = toks[0], int(toks[1]), int(toks[2]), float(toks[3])
    C = {b"PF": 3, b"Pf": 1}.get(magic)
    if C is None or w <= 0 or h <= 0 or scale == 0.0:
        raise ValueError(f"{path}: bad PFM header")
    dt = np.dtype("<f4" if scale < 0 else ">f4")
    n = w * h * C
    if len(data) - pos < 4 * n:
        raise ValueError(f"{path}: truncated PFM data")
    a = np.frombuffer(data, dt, count=n, offset=pos).astype(np.float32).reshape(h, w, C)
    return np.ascontiguousarray(a[::-1].transpose(2, 0, 1))


def buffer_name(name: str, j: int = 0, untransformed: bool = False, stat_type: int = 0) -> str:
    """Reference buffer name: t<type>-b<j>-[film-]<name> (ALLOC_BUF, estimator.cpp:21-24)."""
    return f"t{stat_type}-b{j}-{'film-' if untransformed else ''}{name}"


def output_path(stem, suffix: str, name: str, ext: str = "pfm") -> Path:
    """<stem>[-<suffix>]-<name>.<ext> (buffer.cpp:50-52)."""
    stem = str(stem)
    return Path(f"{stem if not suffix else stem + '-' + suffix}-{name}.{ext}")


def parse_file_id(file_id: str):
    """(t, b, suffix) of a replay id "t<T>-b<j>-<suffix>"; -1/-1/"" where absent (statpath.cpp:522-531)."""
    t = b = -1
    suffix = ""
    m = re.search(r"^t([0-9]+)-", file_id)
    if m:
        t = int(m.group(1))
    m = re.search(r"^t[0-9]+-b([0-9]+)-", file_id)
    if m:
        b = int(m.group(1))
    m = re.search(r"^t[0-9]+-b[0-9]+-(.*)", file_id)
    if m:
        suffix = m.group(1)
    return t, b, suffix
