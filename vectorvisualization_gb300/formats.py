"""The reference's on-disk formats and the headless image dump, over the library's C ABI.

    info = parse_dat("helix.dat")            # DatFile::parseDatFile (reader.cpp:80-262)
    field = read_dat(info, timestep)         # DatFile::readRawData, shaped (nz, ny, nx, comps)
    noise = read_noise("noise_256")          # NoiseDataSet::loadRawData (dataset.cpp:1347-1389)
    write_image("frame.png", img)            # Renderer::saveTexture + pngWrite
    present("frame.png", img)                # composited over white (background_fragment.glsl)

Parsing, reading and writing run in the library (formats.cpp); errors raise capi.VVLICError
with the library's message.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import capi

_NP = {capi.DAT_UCHAR: np.uint8, capi.DAT_USHORT: np.uint16, capi.DAT_FLOAT: np.float32}


def _err(st: int, what: str):
    raise capi.VVLICError(st, f"{what}: {capi.load().vvlic_io_error().decode()}")


@dataclass
class DatInfo:
    raw_file: str
    resolution: tuple
    slice_thickness: tuple
    format: int
    components: int
    timestep_begin: int
    timestep_end: int
    _c: capi.DatInfo = None

    @property
    def dtype(self):
        return _NP.get(self.format)


def parse_dat(path: str) -> DatInfo:
    c = capi.DatInfo()
    st = capi.load().vvlic_dat_parse(os.fsencode(path), C.byref(c))
    if st:
        _err(st, f"parse_dat({path})")
    return DatInfo(c.raw_file.decode(), tuple(c.resolution), tuple(c.slice_thickness), c.format, c.components,
                   c.timestep_begin, c.timestep_end, c)


def read_dat(info: DatInfo, timestep: int | None = None) -> np.ndarray:
    """One timestep as (nz, ny, nx, components) (components axis dropped when 1)."""
    t = info.timestep_begin if timestep is None else timestep
    nx, ny, nz = info.resolution
    dt = info.dtype
    if dt is None:
        raise capi.VVLICError(capi.ERR_FORMAT, "read_dat: no data type")
    out = np.empty((nz, ny, nx, info.components), dt)
    st = capi.load().vvlic_dat_read(C.byref(info._c), t, out.ctypes.data, out.nbytes)
    if st:
        _err(st, f"read_dat({info.raw_file}, {t})")
    return out[..., 0] if info.components == 1 else out


def load_vector_dataset(path: str, timestep: int | None = None):
    """VectorDataSet::loadData: a 3-component UCHAR or FLOAT field and its slice distances."""
    info = parse_dat(path)
    if info.components != 3 or info.format not in (capi.DAT_UCHAR, capi.DAT_FLOAT):
        raise capi.VVLICError(capi.ERR_FORMAT, f"{path} is not a 3-component UCHAR/FLOAT vector data set")
    return read_dat(info, timestep), info.slice_thickness


def write_dat(path: str, data: np.ndarray, slice_thickness=(1.0, 1.0, 1.0), raw_name: str | None = None,
              timesteps: list | None = None):
    """Write a .dat description and its raw file(s): data (nz, ny, nx[, comps]) or, with
    `timesteps`, one array per timestep (raw_name then holds a %d-style pattern)."""
    arrays = timesteps if timesteps is not None else [data]
    a0 = np.asarray(arrays[0])
    fmt = {np.dtype(np.uint8): "UCHAR", np.dtype(np.uint16): "USHORT", np.dtype(np.float32): "FLOAT"}[a0.dtype]
    comps = a0.shape[3] if a0.ndim == 4 else 1
    base = os.path.splitext(os.path.basename(path))[0]
    raw = raw_name or (base + ("_%d.raw" if timesteps is not None else ".raw"))
    d = os.path.dirname(path)
    for t, a in enumerate(arrays):
        name = raw % t if timesteps is not None else raw
        np.ascontiguousarray(a).tofile(os.path.join(d, name))
    with open(path, "w") as fh:
        fh.write(f"ObjectFileName: {raw}\n")
        fh.write(f"Resolution: {a0.shape[2]} {a0.shape[1]} {a0.shape[0]}\n")
        fh.write("SliceThickness: %r %r %r\n" % tuple(float(v) for v in slice_thickness))
        fh.write(f"Format: {fmt}{comps if comps > 1 else ''}\n")
        if timesteps is not None:
            fh.write(f"TimeDependent: 0 {len(arrays) - 1}\n")


def read_noise(path: str) -> np.ndarray:
    dims = np.zeros(3, np.int32)
    lib = capi.load()
    st = lib.vvlic_noise_read(os.fsencode(path), None, 0, dims.ctypes.data)
    if st:
        _err(st, f"read_noise({path})")
    out = np.empty((dims[2], dims[1], dims[0]), np.uint8)
    st = lib.vvlic_noise_read(os.fsencode(path), out.ctypes.data, out.nbytes, dims.ctypes.data)
    if st:
        _err(st, f"read_noise({path})")
    return out


def write_noise(path: str, noise: np.ndarray):
    a = np.ascontiguousarray(noise, dtype=np.uint8)
    dims = np.array(a.shape[::-1], np.int32)
    st = capi.load().vvlic_noise_write(os.fsencode(path), a.ctypes.data, dims.ctypes.data)
    if st:
        _err(st, f"write_noise({path})")


def write_image(path: str, rgba: np.ndarray, kind: str | None = None, composite: bool = False):
    """Dump an (h, w, 4) float image (row 0 = bottom) as 8-bit PNG or PPM (by extension)."""
    a = np.ascontiguousarray(rgba, dtype=np.float32)
    h, w = a.shape[:2]
    k = kind or ("ppm" if path.lower().endswith(".ppm") else "png")
    st = capi.load().vvlic_image_write(os.fsencode(path), a.ctypes.data, w, h,
                                        capi.IMAGE_PPM if k == "ppm" else capi.IMAGE_PNG, int(composite))
    if st:
        _err(st, f"write_image({path})")


def read_png(path: str) -> np.ndarray:
    """pngRead: (h, w, channels) uint8, rows top first (8-bit gray / gray+alpha / RGB / RGBA)."""
    w, h, ch = capi._I(0), capi._I(0), capi._I(0)
    lib = capi.load()
    st = lib.vvlic_png_read(os.fsencode(path), None, 0, C.byref(w), C.byref(h), C.byref(ch))
    if st:
        _err(st, f"read_png({path})")
    out = np.empty((h.value, w.value, ch.value), np.uint8)
    st = lib.vvlic_png_read(os.fsencode(path), out.ctypes.data, out.nbytes, C.byref(w), C.byref(h), C.byref(ch))
    if st:
        _err(st, f"read_png({path})")
    return out


def present(path: str, rgba: np.ndarray):
    """The window image: the render composited over white, written as an image file."""
    write_image(path, rgba, composite=True)
