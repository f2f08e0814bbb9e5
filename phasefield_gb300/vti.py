"""Microstructure files: korn/conc fields as the reference's writers define
them, and a reader for the appended-binary pieces and .pvti index written by
pf_write_vti_binary (zhubq/PhaseField C++-MPI/source/write_data.cpp:30-110 for
the piece/index layout, C++-openmp-cuda/src/write_data.cpp:42-82 for the
fields)."""
from __future__ import annotations

import os
import re

import numpy as np

from . import _ptr, check, lib


def fields(ids: np.ndarray, C: np.ndarray, N: int) -> tuple[np.ndarray, np.ndarray]:
    """korn (0 where the second slot is occupied, else the phase of the first
    grain: id // 100000, 1 for ids below 100000, 0 for an empty slot) and conc
    (total carbon as float32) of a reference-layout state."""
    ids = ids.reshape(-1, 6)[:N]
    g = ids[:, 0]
    ph = np.where(g == 0, 0, np.maximum(g // 100000, 1))
    korn = np.where(ids[:, 1] > 0, 0, ph).astype(np.int32)
    return korn, C[:N].astype(np.float32)


def write_host(directory: str, index: int, pieces: int, grid, dx: float, korn: np.ndarray, conc: np.ndarray) -> None:
    """pf_write_vti_binary_host: the same files from host arrays."""
    korn = np.ascontiguousarray(korn, np.int32)
    conc = np.ascontiguousarray(conc, np.float32)
    check(lib().pf_write_vti_binary_host(directory.encode(), index, pieces, grid[0], grid[1], grid[2], dx,
                                         _ptr(korn), _ptr(conc)), "pf_write_vti_binary_host")


def _extent(text: str, tag: str) -> list[int]:
    m = re.search(tag + r'="([-0-9 ]+)"', text)
    return [int(v) for v in m.group(1).split()]


def read_piece(path: str) -> dict:
    """One appended-raw ImageData piece: its extent and arrays (in file order)."""
    raw = open(path, "rb").read()
    head_end = raw.index(b"<AppendedData")
    head = raw[:head_end].decode()
    start = raw.index(b"_", head_end) + 1
    ext = _extent(head, "Piece Extent")
    out = {"extent": ext, "spacing": [float(v) for v in re.search(r'Spacing="([^"]+)"', head).group(1).split()]}
    for typ, name, off in re.findall(r'<DataArray type="(\w+)" Name="(\w+)" format="appended" offset="(\d+)"', head):
        o = start + int(off)
        nbytes = int(np.frombuffer(raw, np.uint64, 1, o)[0])
        dt = {"Int32": np.int32, "Float32": np.float32}[typ]
        out[name] = np.frombuffer(raw, dt, nbytes // np.dtype(dt).itemsize, o + 8).copy()
    return out


def read_pvti(path: str) -> dict:
    """The whole image from a .pvti index and its pieces: korn and conc in
    cell order (x fastest), plus the whole extent."""
    text = open(path).read()
    whole = _extent(text, "WholeExtent")
    ix, iy, iz = whole[1] - whole[0] + 1, whole[3] - whole[2] + 1, whole[5] - whole[4] + 1
    korn = np.zeros(ix * iy * iz, np.int32)
    conc = np.zeros(ix * iy * iz, np.float32)
    seen = np.zeros(iz, bool)
    for ext, src in re.findall(r'<Piece Extent="([-0-9 ]+)" Source="([^"]+)"', text):
        e = [int(v) for v in ext.split()]
        p = read_piece(os.path.join(os.path.dirname(path), src))
        assert p["extent"] == e
        k0, k1 = e[4] - whole[4], e[5] - whole[4]
        a, b = k0 * ix * iy, (k1 + 1) * ix * iy
        korn[a:b] = p["korn"]
        conc[a:b] = p["conc"]
        seen[k0:k1 + 1] = True
    assert seen.all(), "pieces do not cover the image"
    return {"whole_extent": whole, "korn": korn, "conc": conc, "grid": (ix, iy, iz)}
