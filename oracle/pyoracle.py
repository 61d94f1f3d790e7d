"""ORACLE — test infrastructure, not product code.

ctypes front end of the CPU restatement (oracle/vvlic_oracle.hpp via _build/libvvoracle.so) and
of the reference's own gradient code compiled by build_ref.sh (_ref/libvvref_*.so).  Only tests/,
the smoke check and bench.py's CPU baseline may import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from vectorvisualization_gb300 import capi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libvvoracle.so")
REF_DIR = os.path.join(HERE, "_ref")


class Inputs(C.Structure):
    _fields_ = [
        ("field", C.c_void_p),
        ("n", C.c_int32 * 3),
        ("slice_dist", C.c_float * 3),
        ("noise", C.c_void_p),
        ("m", C.c_int32 * 3),
        ("noise_channels", C.c_int32),
        ("scalar", C.c_void_p),
        ("sn", C.c_int32 * 3),
        ("tf_rgba", C.c_void_p),
        ("tf_opac", C.c_void_p),
        ("filter_table", C.c_void_p),
        ("filter_width", C.c_int32),
        ("filter_clamp", C.c_int32),
        ("filter_is_box", C.c_int32),
        ("taps", C.c_void_p),
        ("inv_filter_area", C.c_double),
        ("licvol", C.c_void_p),
        ("ln", C.c_int32 * 3),
        ("luts", C.c_void_p),
        ("lut_w", C.c_int32),
        ("lut_h", C.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle (make -C oracle)."""
    if force or not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(LIB)
        P, I = C.c_void_p, C.c_int32
        l.vvo_encode_field.argtypes = [P, I, P, P]
        l.vvo_encode_field_interp.argtypes = [P, P, I, P, I, I, P]
        l.vvo_round_storage.argtypes = [P, C.c_uint64, I]
        l.vvo_illum_luts.argtypes = [P, I, I, P]
        l.vvo_noise_gradients.argtypes = [P, P, I, P, P]
        l.vvo_noise_filter_weights.argtypes = [P]
        l.vvo_filter_inv_area.argtypes = [P, I, I]
        l.vvo_filter_inv_area.restype = C.c_float
        l.vvo_filter_taps.argtypes = [P, I, I, I, I, P]
        l.vvo_view_rays.argtypes = [P, P, P, I, I, P]
        l.vvo_geometry.argtypes = [P, P, P]
        l.vvo_render.argtypes = [C.POINTER(Inputs), P, P, I, I, P, I, P, P, I, I, P]
        l.vvo_lic_volume.argtypes = [C.POINTER(Inputs), P, P, P]
        l.vvo_lic_volume.restype = I
        l.vvo_render.restype = I
        l.vvo_max_threads.restype = I
        l.vvo_adjoint.argtypes = [C.POINTER(Inputs), P, P, I, I, P, P, P, P, I]
        l.vvo_adjoint.restype = I
        l.vvo_params_default.argtypes = [C.POINTER(capi.Params)]
        l.vvo_view_default.argtypes = [C.POINTER(capi.View)]
        l.vvo_line_material_default.argtypes = [C.POINTER(capi.LineMaterial)]
        l.vvo_filter_table.argtypes = [I, I, P]
        l.vvo_filter_table.restype = I
        _lib = l
    return _lib


# ---- defaults and filter tables restated by the oracle (no libvvlic involved) -------------
def params_default() -> capi.Params:
    """LICParams() and the reference's fixed shader state (oracle restatement)."""
    p = capi.Params()
    lib().vvo_params_default(C.byref(p))
    return p


def view_default() -> capi.View:
    v = capi.View()
    lib().vvo_view_default(C.byref(v))
    return v


def line_material_default() -> capi.LineMaterial:
    m = capi.LineMaterial()
    lib().vvo_line_material_default(C.byref(m))
    return m


def filter_table(kind, width: int = 256) -> np.ndarray:
    """Filter-kernel table (uint8) of `kind` ("box", "triangle", "cos2", "gaussian")."""
    k = capi.FILTER[kind] if isinstance(kind, str) else int(kind)
    out = np.zeros(1024, np.uint8)
    w = lib().vvo_filter_table(k, width, out.ctypes.data)
    if w == 0:
        raise ValueError(f"oracle filter_table: bad kind {kind!r} or width {width}")
    return out[:w].copy()


class Defaults:
    """The provider workloads.* take as `defaults=`: inputs of a configuration built by the
    oracle alone, so a CPU run of the oracle needs no libvvlic."""

    params = staticmethod(params_default)
    view = staticmethod(view_default)
    filter_table = staticmethod(filter_table)


DEFAULTS = Defaults()


def _dims(a: np.ndarray) -> np.ndarray:
    """(z, y, x, ...) array -> int32 [x, y, z]"""
    return np.array([a.shape[2], a.shape[1], a.shape[0]], np.int32)


def encode_field(xyz: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(xyz)
    dtype = capi.DTYPE_UINT8 if a.dtype == np.uint8 else capi.DTYPE_FLOAT32
    if dtype == capi.DTYPE_FLOAT32:
        a = a.astype(np.float32, copy=False)
    out = np.empty(a.shape[:3] + (4,), np.float32)
    lib().vvo_encode_field(a.ctypes.data, dtype, _dims(a).ctypes.data, out.ctypes.data)
    return out


def encode_field_interp(xyz0: np.ndarray, xyz1: np.ndarray, index: int, size: int) -> np.ndarray:
    """Encoding of the time interpolation of two timesteps at t = index / size."""
    a0, a1 = np.ascontiguousarray(xyz0), np.ascontiguousarray(xyz1)
    dtype = capi.DTYPE_UINT8 if a0.dtype == np.uint8 else capi.DTYPE_FLOAT32
    if dtype == capi.DTYPE_FLOAT32:
        a0, a1 = a0.astype(np.float32, copy=False), a1.astype(np.float32, copy=False)
    out = np.empty(a0.shape[:3] + (4,), np.float32)
    lib().vvo_encode_field_interp(a0.ctypes.data, a1.ctypes.data, dtype, _dims(a0).ctypes.data, index, size,
                                  out.ctypes.data)
    return out


def illum_luts(material: "capi.LineMaterial | None" = None) -> np.ndarray:
    """Zoeckler, Mallo diffuse and Mallo specular tables, (3, h, w, 4) uint8."""
    m = material if material is not None else line_material_default()
    w, h = capi.lut_size(m.width), capi.lut_size(m.height)
    out = np.empty((3, h, w, 4), np.uint8)
    lib().vvo_illum_luts(C.byref(m), w, h, out.ctypes.data)
    return out


def round_storage(rgba: np.ndarray, storage: str) -> np.ndarray:
    out = np.ascontiguousarray(rgba, dtype=np.float32).copy()
    lib().vvo_round_storage(out.ctypes.data, out.size, capi.STORAGE[storage])
    return out


def noise_gradients(noise: np.ndarray, mode: int, slice_dist=None) -> np.ndarray:
    a = np.ascontiguousarray(noise, dtype=np.uint8)
    out = np.empty(a.shape + (4,), np.uint8)
    sd = None if slice_dist is None else np.asarray(slice_dist, np.float32)
    lib().vvo_noise_gradients(a.ctypes.data, _dims(a).ctypes.data, mode, None if sd is None else sd.ctypes.data, out.ctypes.data)
    return out


def noise_filter_weights() -> np.ndarray:
    w = np.empty(27, np.float32)
    lib().vvo_noise_filter_weights(w.ctypes.data)
    return w


def filter_taps(table: np.ndarray, lb: int, lf: int, clamp: int = capi.KERNEL_CLAMP_BORDER) -> np.ndarray:
    t = np.ascontiguousarray(table, dtype=np.uint8)
    out = np.empty(lb + lf + 1, np.float64)
    lib().vvo_filter_taps(t.ctypes.data, t.size, clamp, lb, lf, out.ctypes.data)
    return out


def filter_inv_area(table: np.ndarray, is_box: bool) -> float:
    t = np.ascontiguousarray(table, dtype=np.uint8)
    return float(lib().vvo_filter_inv_area(t.ctypes.data, t.size, int(is_box)))


def view_rays(view: capi.View, dims_xyz, w: int, h: int, slice_dist=None) -> np.ndarray:
    n = np.asarray(dims_xyz, np.int32)
    sd = None if slice_dist is None else np.asarray(slice_dist, np.float32)
    out = np.zeros(21, np.float64)
    lib().vvo_view_rays(C.byref(view), n.ctypes.data, None if sd is None else sd.ctypes.data, w, h, out.ctypes.data)
    return out


def geometry(dims_xyz, slice_dist=None) -> dict:
    n = np.asarray(dims_xyz, np.int32)
    sd = None if slice_dist is None else np.asarray(slice_dist, np.float32)
    out = np.zeros(15, np.float64)
    lib().vvo_geometry(n.ctypes.data, None if sd is None else sd.ctypes.data, out.ctypes.data)
    return {k: out[3 * i : 3 * i + 3] for i, k in enumerate(["scale", "scale_inv", "extent", "center", "tex_max"])}


class Scene:
    """Oracle-side copy of everything a render needs (field already encoded)."""

    def __init__(self, field_rgba: np.ndarray, noise: np.ndarray, tf_rgba: np.ndarray, tf_opac: np.ndarray,
                 filter_table: np.ndarray | None = None, filter_clamp: int = capi.KERNEL_CLAMP_BORDER,
                 taps: np.ndarray | None = None, inv_filter_area: float = 0.5, scalar: np.ndarray | None = None,
                 slice_dist=(1.0, 1.0, 1.0)):
        self.field = np.ascontiguousarray(field_rgba, dtype=np.float32)
        self.noise = np.ascontiguousarray(noise, dtype=np.uint8)
        self.tf_rgba = np.ascontiguousarray(tf_rgba, dtype=np.float32).reshape(-1)
        self.tf_opac = np.ascontiguousarray(tf_opac, dtype=np.float32).reshape(-1)
        self.table = None if filter_table is None else np.ascontiguousarray(filter_table, dtype=np.uint8)
        self.taps = None if taps is None else np.ascontiguousarray(taps, dtype=np.float64)
        self.scalar = None if scalar is None else np.ascontiguousarray(scalar, dtype=np.float32)
        self.inputs = Inputs()
        i = self.inputs
        i.field = self.field.ctypes.data
        for k, v in enumerate(_dims(self.field)):
            i.n[k] = int(v)
        for k in range(3):
            i.slice_dist[k] = float(slice_dist[k])
        i.noise = self.noise.ctypes.data
        if self.noise.ndim == 4:
            i.noise_channels = 4
        else:
            i.noise_channels = 1
        for k, v in enumerate(_dims(self.noise)):
            i.m[k] = int(v)
        if self.scalar is not None:
            i.scalar = self.scalar.ctypes.data
            for k, v in enumerate(_dims(self.scalar)):
                i.sn[k] = int(v)
        i.tf_rgba = self.tf_rgba.ctypes.data
        i.tf_opac = self.tf_opac.ctypes.data
        if self.table is not None:
            i.filter_table = self.table.ctypes.data
            i.filter_width = self.table.size
            i.filter_clamp = filter_clamp
            i.filter_is_box = int(bool(np.all(self.table == 255)))
        if self.taps is not None:
            i.taps = self.taps.ctypes.data
            i.inv_filter_area = inv_filter_area

    @property
    def dims(self):
        return [int(v) for v in self.inputs.n]

    def render(self, params: capi.Params, view: capi.View, w: int, h: int, rows=None, precision: int = 64,
               threads: int = 0):
        """Returns (image (nrows, w, 4) float32, samples (nrows, w) uint32)."""
        if params.illum in (capi.ILLUM_ZOECKLER, capi.ILLUM_MALLO) and not self.inputs.luts:
            self.attach_line_material()
        rc = view_rays(view, self.dims, w, h, list(self.inputs.slice_dist))
        r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
        nr = h if r is None else r.size
        img = np.zeros((nr, w, 4), np.float32)
        smp = np.zeros((nr, w), np.uint32)
        st = lib().vvo_render(C.byref(self.inputs), C.byref(params), rc.ctypes.data, w, h,
                              None if r is None else r.ctypes.data, nr, img.ctypes.data, smp.ctypes.data, precision,
                              threads, C.byref(view))
        if st != 0:
            raise RuntimeError(f"oracle render failed ({st})")
        return img, smp

    def lic_volume(self, params: capi.Params, dims) -> np.ndarray:
        """LIC volume of dims (nx, ny, nz), returned (nz, ny, nx)."""
        ln = np.asarray(dims, np.int32)
        out = np.empty((dims[2], dims[1], dims[0]), np.float32)
        st = lib().vvo_lic_volume(C.byref(self.inputs), C.byref(params), ln.ctypes.data, out.ctypes.data)
        if st != 0:
            raise RuntimeError(f"oracle LIC volume failed ({st})")
        return out

    def attach_line_material(self, material: "capi.LineMaterial | None" = None):
        """Line-illumination tables for ZOECKLER / MALLO renders (default material if None)."""
        self._luts = illum_luts(material)
        self.inputs.luts = self._luts.ctypes.data
        self.inputs.lut_w = self._luts.shape[2]
        self.inputs.lut_h = self._luts.shape[1]

    def attach_lic_volume(self, licvol: np.ndarray):
        self._licvol = np.ascontiguousarray(licvol, dtype=np.float32)
        self.inputs.licvol = self._licvol.ctypes.data
        for k, v in enumerate(self._licvol.shape[::-1]):
            self.inputs.ln[k] = int(v)


def adjoint(scene: "Scene", params: capi.Params, view: capi.View, w: int, h: int, g_img: np.ndarray,
            threads: int = 0):
    """FP64 adjoint of the render: (dL/dTF (256,4), dL/dopacity (256,), dL/dtaps)."""
    if params.illum in (capi.ILLUM_ZOECKLER, capi.ILLUM_MALLO) and not scene.inputs.luts:
        scene.attach_line_material()
    rc = view_rays(view, scene.dims, w, h, list(scene.inputs.slice_dist))
    g = np.ascontiguousarray(g_img, dtype=np.float32).reshape(h, w, 4)
    lb, lf = (15, 15) if params.low_res else (params.steps_backward, params.steps_forward)
    d_tf = np.zeros(1024, np.float64)
    d_op = np.zeros(256, np.float64)
    d_taps = np.zeros(lb + lf + 1, np.float64)
    st = lib().vvo_adjoint(C.byref(scene.inputs), C.byref(params), rc.ctypes.data, w, h, g.ctypes.data,
                           d_tf.ctypes.data, d_op.ctypes.data, d_taps.ctypes.data, threads)
    if st != 0:
        raise RuntimeError(f"oracle adjoint failed ({st})")
    return d_tf.reshape(256, 4), d_op, d_taps


def max_threads() -> int:
    return int(lib().vvo_max_threads())


# ---- the reference's own gradient code (oracle/_ref) ----------------------------------------
def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libvvref_sobel.so"))


def ref_noise_gradients(noise: np.ndarray, mode: int, slice_dist=None) -> np.ndarray:
    name = "libvvref_sobel.so" if mode == capi.NOISE_GRAD_SOBEL else "libvvref_central.so"
    l = C.CDLL(os.path.join(REF_DIR, name))
    l.vvref_noise_gradients.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    a = np.ascontiguousarray(noise, dtype=np.uint8)
    out = np.empty(a.shape + (4,), np.uint8)
    sd = np.asarray(slice_dist if slice_dist is not None else (1, 1, 1), np.float32)
    st = l.vvref_noise_gradients(a.ctypes.data, _dims(a).ctypes.data, sd.ctypes.data, out.ctypes.data)
    if st != 0:
        raise RuntimeError(f"reference gradient code failed ({st})")
    return out
