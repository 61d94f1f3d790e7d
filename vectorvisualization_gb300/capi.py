"""ctypes binding of the C ABI in include/vvlic.h (libvvlic.so).

This module only marshals arguments; all work happens in the CUDA library.  Loading fails
loudly when the library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libvvlic.so")

MAX_STEPS = 256
TF_ENTRIES = 256

# status codes
OK, ERR_INVALID_ARGUMENT, ERR_OUT_OF_MEMORY, ERR_CUDA, ERR_NO_DEVICE, ERR_NOT_READY = 0, 1, 2, 3, 4, 5
ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_BAD_HANDLE, ERR_IO, ERR_FORMAT = 6, 7, 8, 9, 10
DTYPE_FLOAT32, DTYPE_UINT8 = 0, 1
STORAGE = {"f32": 0, "f16": 1, "bf16": 2, "u8": 3}
SAMPLER = {"gather": 0, "cell": 1, "texture": 2, "hybrid": 3, "brick": 4}
SCHEDULE = {"queue": 0, "static": 1}
TECHNIQUE = {"volume": 0, "raycast": 1, "slicing": 2, "licvolume": 3}
NOISE_SCALAR, NOISE_GRAD_SOBEL, NOISE_GRAD_CENTRAL = 0, 1, 2
EULER, HEUN, RK4 = 0, 1, 2
ILLUM_NONE, ILLUM_GRADIENT, ILLUM_ZOECKLER, ILLUM_MALLO = 0, 1, 2, 3
TF_INDEX_DIR_Z, TF_INDEX_MAGNITUDE = 0, 1
KERNEL_CLAMP_BORDER, KERNEL_CLAMP_EDGE = 0, 1
FILTER = {"box": 0, "triangle": 1, "cos2": 2, "gaussian": 3}
PERSPECTIVE, ORTHOGRAPHIC = 0, 1
QUIRK_LUMINANCE_NOISE, QUIRK_UNIFORM_SCALE_BUG, QUIRK_GRAD_NOISE_NO_FREQ, QUIRK_ZOECKLER_LUMINANCE = 1, 2, 4, 8
QUIRKS_REFERENCE = QUIRK_UNIFORM_SCALE_BUG | QUIRK_GRAD_NOISE_NO_FREQ | QUIRK_ZOECKLER_LUMINANCE
CHECK_FIELD, CHECK_NOISE, CHECK_SCALAR, CHECK_TAPE, CHECK_IMAGE, CHECK_TAPE_OVERFLOW, CHECK_BRICK = 1, 2, 4, 8, 16, 32, 64

_f3 = C.c_float * 3


class Params(C.Structure):
    """vvlic_params (include/vvlic.h)."""

    _fields_ = [
        ("step_size_vol", C.c_float),
        ("gradient_scale", C.c_float),
        ("illum_scale", C.c_float),
        ("freq_scale", C.c_float),
        ("num_iterations", C.c_int32),
        ("steps_forward", C.c_int32),
        ("steps_backward", C.c_int32),
        ("step_size_lic", C.c_float),
        ("integrator", C.c_int32),
        ("illum", C.c_int32),
        ("tf_index", C.c_int32),
        ("speed_of_flow", C.c_int32),
        ("low_res", C.c_int32),
        ("scalar_gate", C.c_int32),
        ("gate_lo", C.c_float),
        ("gate_hi", C.c_float),
        ("eye_dist_factor", C.c_float),
        ("alpha_threshold", C.c_float),
        ("quirks", C.c_uint32),
        ("light_pos", _f3),
        ("spec_exp", C.c_float),
        ("light_diffuse", _f3),
        ("light_specular", _f3),
        ("light_ambient", _f3),
        ("sampler", C.c_int32),
        ("schedule", C.c_int32),
        ("record_tape", C.c_int32),
        ("technique", C.c_int32),
        ("tape_max_samples", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class View(C.Structure):
    """vvlic_view (include/vvlic.h)."""

    _fields_ = [
        ("projection", C.c_int32),
        ("quat", C.c_float * 4),
        ("distance", C.c_float),
        ("pan", _f3),
        ("fovy_deg", C.c_float),
        ("aspect", C.c_float),
        ("ortho_center", _f3),
        ("ortho_right", _f3),
        ("ortho_up", _f3),
        ("ortho_dir", _f3),
    ]


class Job(C.Structure):
    """vvlic_job (include/vvlic.h)."""

    _fields_ = [
        ("vol_id", C.c_int32),
        ("w", C.c_int32),
        ("h", C.c_int32),
        ("d_out", C.c_void_p),
        ("view", View),
        ("params", Params),
        ("filter_table", C.c_void_p),
        ("filter_width", C.c_int32),
        ("filter_clamp", C.c_int32),
    ]


class LineMaterial(C.Structure):
    _fields_ = [
        ("light_color", C.c_float * 4),
        ("ambient", C.c_float * 4),
        ("diffuse", C.c_float * 4),
        ("specular", C.c_float * 4),
        ("spec_exp", C.c_float),
        ("diff_exp", C.c_float),
        ("width", C.c_int32),
        ("height", C.c_int32),
    ]


class DatInfo(C.Structure):
    _fields_ = [
        ("raw_file", C.c_char * 1024),
        ("resolution", C.c_int32 * 3),
        ("slice_thickness", C.c_float * 3),
        ("format", C.c_int32),
        ("components", C.c_int32),
        ("timestep_begin", C.c_int32),
        ("timestep_end", C.c_int32),
    ]


DAT_NONE, DAT_UCHAR, DAT_USHORT, DAT_FLOAT = 0, 1, 2, 3
IMAGE_PPM, IMAGE_PNG = 0, 1


class Stats(C.Structure):
    _fields_ = [
        ("samples", C.c_uint64),
        ("sample_steps", C.c_uint64),
        ("rays", C.c_uint64),
        ("kernel_ms", C.c_float),
        ("check_flags", C.c_uint32),
    ]


class FetchCeiling(C.Structure):
    _fields_ = [
        ("tex_per_s", C.c_double),
        ("ld256_per_s", C.c_double),
        ("group_per_s", C.c_double * 3),
        ("ms", C.c_float * 5),
        ("num_sms", C.c_int32),
        ("spread4", C.c_int32),
    ]


_P = C.c_void_p
_I = C.c_int32
_SIGS = {
    "vvlic_params_default": (None, [C.POINTER(Params)]),
    "vvlic_view_default": (None, [C.POINTER(View)]),
    "vvlic_status_string": (C.c_char_p, [_I]),
    "vvlic_abi_version": (_I, []),
    "vvlic_make_filter_table": (_I, [_I, _I, _P, C.POINTER(_I)]),
    "vvlic_line_material_default": (None, [C.POINTER(LineMaterial)]),
    "vvlic_set_line_material": (_I, [_P, C.POINTER(LineMaterial)]),
    "vvlic_get_illum_luts": (_I, [_P, _P, _P, _P, C.POINTER(_I), C.POINTER(_I)]),
    "vvlic_dat_parse": (_I, [C.c_char_p, C.POINTER(DatInfo)]),
    "vvlic_dat_bytes": (C.c_uint64, [C.POINTER(DatInfo)]),
    "vvlic_dat_read": (_I, [C.POINTER(DatInfo), _I, _P, C.c_uint64]),
    "vvlic_upload_dat": (_I, [_P, C.c_char_p, _I, _I, C.POINTER(_I)]),
    "vvlic_noise_read": (_I, [C.c_char_p, _P, C.c_uint64, _P]),
    "vvlic_noise_write": (_I, [C.c_char_p, _P, _P]),
    "vvlic_image_write": (_I, [C.c_char_p, _P, _I, _I, _I, _I]),
    "vvlic_io_error": (C.c_char_p, []),
    "vvlic_synchronize": (_I, [_P, _P, _I]),
    "vvlic_get_tf": (_I, [_P, _P, _P]),
    "vvlic_upload_noise_rgba": (_I, [_P, _P, _I, _I, _I, _I]),
    "vvlic_upload_noise_file": (_I, [_P, C.c_char_p, _I]),
    "vvlic_png_read": (_I, [C.c_char_p, _P, C.c_uint64, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "vvlic_load_filter_png": (_I, [_P, C.c_char_p]),
    "vvlic_load_tf_png": (_I, [_P, C.c_char_p]),
    "vvlic_save_tf_png": (_I, [_P, C.c_char_p]),
    "vvlic_create": (_I, [C.POINTER(_P), _I]),
    "vvlic_destroy": (_I, [_P]),
    "vvlic_last_error": (C.c_char_p, [_P]),
    "vvlic_upload_field": (_I, [_P, _P, _I, _I, _I, _I, _P, _I, C.POINTER(_I)]),
    "vvlic_upload_field_device": (_I, [_P, _P, _I, _I, _I, _P, _I, _P, C.POINTER(_I)]),
    "vvlic_upload_field_interp": (_I, [_P, _P, _P, _I, _I, _I, _I, _P, _I, _I, _I, C.POINTER(_I)]),
    "vvlic_update_field": (_I, [_P, _I, _P, _I, _I, _I, _I]),
    "vvlic_update_field_interp": (_I, [_P, _I, _P, _P, _I, _I, _I, _I, _I, _I]),
    "vvlic_update_field_async": (_I, [_P, _I, _P, _I, _I, _I, _I, _P]),
    "vvlic_update_field_device": (_I, [_P, _I, _P, _I, _I, _I, _P]),
    "vvlic_upload_noise_async": (_I, [_P, _P, _I, _I, _I, _I, _P]),
    "vvlic_render_to_host_async": (_I, [_P, _I, _P, _I, _I, _P]),
    "vvlic_free_volume": (_I, [_P, _I]),
    "vvlic_volume_bytes": (_I, [_P, _I, C.POINTER(C.c_uint64)]),
    "vvlic_upload_noise": (_I, [_P, _P, _I, _I, _I, _I]),
    "vvlic_upload_scalar": (_I, [_P, _P, _I, _I, _I]),
    "vvlic_set_tf": (_I, [_P, _P, _P]),
    "vvlic_set_filter_table": (_I, [_P, _P, _I, _I]),
    "vvlic_set_filter_taps": (_I, [_P, _P, _I, _I, C.c_float]),
    "vvlic_get_filter_taps": (_I, [_P, _P, _I, C.POINTER(C.c_float)]),
    "vvlic_set_params": (_I, [_P, C.POINTER(Params)]),
    "vvlic_get_params": (_I, [_P, C.POINTER(Params)]),
    "vvlic_set_view": (_I, [_P, C.POINTER(View)]),
    "vvlic_view_rays": (_I, [_P, _I, _I, _I, _P]),
    "vvlic_render": (_I, [_P, _I, _P, _I, _I]),
    "vvlic_render_device": (_I, [_P, _I, _P, _I, _I, _P, _P]),
    "vvlic_get_stats": (_I, [_P, C.POINTER(Stats)]),
    "vvlic_render_adjoint": (_I, [_P, _I, _P, _I, _I, _P, _P, _P, _P]),
    "vvlic_compute_lic_volume": (_I, [_P, _I, _I, _I, _I]),
    "vvlic_download_lic_volume": (_I, [_P, _I, _P, C.c_uint64]),
    "vvlic_batch_render": (_I, [_P, C.POINTER(Job), _I, _P]),
    "vvlic_batch_autotune": (_I, [_P, C.POINTER(Job), _I, _P, C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_float)]),
    "vvlic_composite_background": (_I, [_P, _I, _I, _P]),
    "vvlic_noise_gradients_device": (_I, [_P, _I, _I, _I, _I, _P, _P, _P]),
    "vvlic_noise_gradients_device_noalloc": (_I, [_P, _I, _I, _I, _I, _P, _P, _P]),
    "vvlic_download_field": (_I, [_P, _I, _P, C.c_uint64]),
    "vvlic_download_noise": (_I, [_P, _P, C.c_uint64]),
    "vvlic_measure_fetch_ceiling": (_I, [_I, _I, C.POINTER(FetchCeiling)]),
}

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load libvvlic.so (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"libvvlic.so not found at {p}: build it with `python -m vectorvisualization_gb300.build` "
            "(the CUDA library is required; there is no CPU fallback)"
        )
    lib = C.CDLL(p)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class VVLICError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"vvlic status {status}: {message}")
        self.status = status


def params_default() -> Params:
    p = Params()
    load().vvlic_params_default(C.byref(p))
    return p


def view_default() -> View:
    v = View()
    load().vvlic_view_default(C.byref(v))
    return v


def line_material_default() -> LineMaterial:
    m = LineMaterial()
    load().vvlic_line_material_default(C.byref(m))
    return m


def lut_size(v: int) -> int:
    """Table size the library uses for a requested width/height (next power of two)."""
    p = 1
    while p < v:
        p <<= 1
    return p


def make_filter_table(kind: str | int, width: int = 256) -> np.ndarray:
    """Filter-kernel table (uint8) as the library builds it (vvlic_make_filter_table)."""
    k = FILTER[kind] if isinstance(kind, str) else int(kind)
    out = np.zeros(1024, np.uint8)
    w = _I(0)
    st = load().vvlic_make_filter_table(k, width, out.ctypes.data, C.byref(w))
    if st:
        raise VVLICError(st, "make_filter_table")
    return out[: w.value].copy()


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def make_job(vol_id: int, d_out: int, w: int, h: int, view: View, params: Params,
             filter_table: np.ndarray | None = None, clamp: int = KERNEL_CLAMP_BORDER) -> Job:
    """A vvlic_job; keeps a reference to the filter table for the call's lifetime."""
    j = Job()
    j.vol_id, j.w, j.h, j.d_out = vol_id, w, h, d_out
    j.view = view
    j.params = params
    if filter_table is not None:
        t = np.ascontiguousarray(filter_table, dtype=np.uint8)
        j._table = t
        j.filter_table = t.ctypes.data
        j.filter_width = t.size
        j.filter_clamp = clamp
    return j


class Context:
    """One vvlic_ctx on one CUDA device."""

    def __init__(self, device: int = 0, lib: C.CDLL | None = None):
        self._lib = lib or load()
        h = _P()
        st = self._lib.vvlic_create(C.byref(h), device)
        if st:
            raise VVLICError(st, self._lib.vvlic_status_string(st).decode())
        self.h = h

    # -- lifetime -------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self._lib.vvlic_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int, what: str):
        if st:
            msg = self._lib.vvlic_last_error(self.h).decode() if self.h else ""
            raise VVLICError(st, f"{what}: {msg or self._lib.vvlic_status_string(st).decode()}")

    # -- inputs ---------------------------------------------------------------------
    def upload_field(self, xyz: np.ndarray, slice_dist=None, storage: str = "f32") -> int:
        """xyz: (nz, ny, nx, 3) float32 or uint8 (x fastest)."""
        a = np.ascontiguousarray(xyz)
        if a.ndim != 4 or a.shape[3] != 3:
            raise ValueError("field must have shape (nz, ny, nx, 3)")
        dtype = DTYPE_UINT8 if a.dtype == np.uint8 else DTYPE_FLOAT32
        if dtype == DTYPE_FLOAT32:
            a = a.astype(np.float32, copy=False)
        nz, ny, nx = a.shape[:3]
        sd = None if slice_dist is None else np.asarray(slice_dist, np.float32)
        vid = _I(0)
        self._check(
            self._lib.vvlic_upload_field(self.h, a.ctypes.data, dtype, nx, ny, nz, _ptr(sd), STORAGE[storage], C.byref(vid)),
            "upload_field",
        )
        return vid.value

    def upload_field_interp(self, xyz0: np.ndarray, xyz1: np.ndarray, index: int, size: int, slice_dist=None,
                            storage: str = "f32") -> int:
        """Encode the time interpolation of two timesteps at index/size."""
        a0, a1 = np.ascontiguousarray(xyz0), np.ascontiguousarray(xyz1)
        if a0.shape != a1.shape or a0.dtype != a1.dtype or a0.ndim != 4:
            raise ValueError("timesteps must have the same (nz, ny, nx, 3) shape and dtype")
        dtype = DTYPE_UINT8 if a0.dtype == np.uint8 else DTYPE_FLOAT32
        if dtype == DTYPE_FLOAT32:
            a0, a1 = a0.astype(np.float32, copy=False), a1.astype(np.float32, copy=False)
        nz, ny, nx = a0.shape[:3]
        sd = None if slice_dist is None else np.asarray(slice_dist, np.float32)
        vid = _I(0)
        self._check(self._lib.vvlic_upload_field_interp(self.h, a0.ctypes.data, a1.ctypes.data, dtype, nx, ny, nz,
                                                         _ptr(sd), STORAGE[storage], index, size, C.byref(vid)),
                    "upload_field_interp")
        return vid.value

    def update_field(self, vid: int, xyz: np.ndarray):
        """Replace volume `vid`'s field in place with new (nz, ny, nx, 3) vectors of its dimensions."""
        a = np.ascontiguousarray(xyz)
        if a.ndim != 4 or a.shape[3] != 3:
            raise ValueError("field must have shape (nz, ny, nx, 3)")
        dtype = DTYPE_UINT8 if a.dtype == np.uint8 else DTYPE_FLOAT32
        if dtype == DTYPE_FLOAT32:
            a = a.astype(np.float32, copy=False)
        nz, ny, nx = a.shape[:3]
        self._check(self._lib.vvlic_update_field(self.h, vid, a.ctypes.data, dtype, nx, ny, nz), "update_field")

    def update_field_interp(self, vid: int, xyz0: np.ndarray, xyz1: np.ndarray, index: int, size: int):
        """Replace volume `vid`'s field in place with the time interpolation at index/size."""
        a0, a1 = np.ascontiguousarray(xyz0), np.ascontiguousarray(xyz1)
        if a0.shape != a1.shape or a0.dtype != a1.dtype or a0.ndim != 4:
            raise ValueError("timesteps must have the same (nz, ny, nx, 3) shape and dtype")
        dtype = DTYPE_UINT8 if a0.dtype == np.uint8 else DTYPE_FLOAT32
        if dtype == DTYPE_FLOAT32:
            a0, a1 = a0.astype(np.float32, copy=False), a1.astype(np.float32, copy=False)
        nz, ny, nx = a0.shape[:3]
        self._check(self._lib.vvlic_update_field_interp(self.h, vid, a0.ctypes.data, a1.ctypes.data, dtype, nx, ny,
                                                         nz, index, size), "update_field_interp")

    def upload_field_device(self, d_xyz: int, dims, slice_dist=None, storage: str = "f32", stream: int = 0) -> int:
        nx, ny, nz = dims
        sd = None if slice_dist is None else np.asarray(slice_dist, np.float32)
        vid = _I(0)
        self._check(
            self._lib.vvlic_upload_field_device(self.h, d_xyz, nx, ny, nz, _ptr(sd), STORAGE[storage], stream or None, C.byref(vid)),
            "upload_field_device",
        )
        return vid.value

    def free_volume(self, vid: int):
        self._check(self._lib.vvlic_free_volume(self.h, vid), "free_volume")

    def volume_bytes(self, vid: int) -> int:
        b = C.c_uint64(0)
        self._check(self._lib.vvlic_volume_bytes(self.h, vid, C.byref(b)), "volume_bytes")
        return b.value

    def download_field(self, vid: int, dims, storage: str) -> np.ndarray:
        """Encoded texels as float32 (nz, ny, nx, 4), decoded from the storage precision."""
        nx, ny, nz = dims
        if storage == "f32":
            out = np.empty((nz, ny, nx, 4), np.float32)
        elif storage == "u8":
            out = np.empty((nz, ny, nx, 4), np.uint8)
        else:
            out = np.empty((nz, ny, nx, 4), np.uint16)
        self._check(self._lib.vvlic_download_field(self.h, vid, out.ctypes.data, out.nbytes), "download_field")
        if storage == "u8":
            return out.astype(np.float32) / np.float32(255.0)
        if storage == "f16":
            return out.view(np.float16).astype(np.float32)
        if storage == "bf16":
            return (out.astype(np.uint32) << 16).view(np.float32)
        return out

    def download_noise(self, dims, channels: int) -> np.ndarray:
        mx, my, mz = dims
        out = np.empty((mz, my, mx, channels) if channels == 4 else (mz, my, mx), np.uint8)
        self._check(self._lib.vvlic_download_noise(self.h, out.ctypes.data, out.nbytes), "download_noise")
        return out

    def upload_noise(self, noise: np.ndarray, mode: int = NOISE_SCALAR):
        """noise: (mz, my, mx) uint8."""
        a = np.ascontiguousarray(noise, dtype=np.uint8)
        mz, my, mx = a.shape
        self._check(self._lib.vvlic_upload_noise(self.h, a.ctypes.data, mx, my, mz, mode), "upload_noise")

    def upload_scalar(self, scalar: np.ndarray):
        a = np.ascontiguousarray(scalar, dtype=np.float32)
        nz, ny, nx = a.shape
        self._check(self._lib.vvlic_upload_scalar(self.h, a.ctypes.data, nx, ny, nz), "upload_scalar")

    def set_tf(self, rgba: np.ndarray | None = None, opacity: np.ndarray | None = None):
        r = None if rgba is None else np.ascontiguousarray(rgba, dtype=np.float32).reshape(TF_ENTRIES * 4)
        o = None if opacity is None else np.ascontiguousarray(opacity, dtype=np.float32).reshape(TF_ENTRIES)
        self._check(self._lib.vvlic_set_tf(self.h, _ptr(r), _ptr(o)), "set_tf")

    def upload_dat(self, dat_path: str, timestep: int = -1, storage: str = "f32") -> int:
        """Load a .dat/.raw vector data set (VectorDataSet::loadData) into a volume."""
        vid = _I(0)
        st = self._lib.vvlic_upload_dat(self.h, os.fsencode(dat_path), timestep, STORAGE[storage], C.byref(vid))
        if st:
            msg = self._lib.vvlic_io_error().decode() or self._lib.vvlic_last_error(self.h).decode()
            raise VVLICError(st, f"upload_dat: {msg}")
        return vid.value

    def synchronize(self, stream: int = 0, timeout_ms: int = 60000) -> bool:
        """Wait for the work on `stream` and the context's stream; False on VVLIC_ERR_TIMEOUT."""
        st = self._lib.vvlic_synchronize(self.h, stream or None, timeout_ms)
        if st == ERR_TIMEOUT:
            return False
        self._check(st, "synchronize")
        return True

    def set_line_material(self, material: LineMaterial):
        self._check(self._lib.vvlic_set_line_material(self.h, C.byref(material)), "set_line_material")

    def illum_luts(self) -> np.ndarray:
        """Zoeckler, Mallo diffuse and Mallo specular tables as sampled, (3, h, w, 4) uint8."""
        w, h = _I(0), _I(0)
        self._check(self._lib.vvlic_get_illum_luts(self.h, None, None, None, C.byref(w), C.byref(h)), "illum_luts")
        out = np.empty((3, h.value, w.value, 4), np.uint8)
        self._check(self._lib.vvlic_get_illum_luts(self.h, out[0].ctypes.data, out[1].ctypes.data,
                                                    out[2].ctypes.data, None, None), "illum_luts")
        return out

    def get_tf(self):
        rgba = np.empty((TF_ENTRIES, 4), np.float32)
        op = np.empty(TF_ENTRIES, np.float32)
        self._check(self._lib.vvlic_get_tf(self.h, rgba.ctypes.data, op.ctypes.data), "get_tf")
        return rgba, op

    def _io(self, st: int, what: str):
        if st:
            msg = self._lib.vvlic_io_error().decode() or self._lib.vvlic_last_error(self.h).decode()
            raise VVLICError(st, f"{what}: {msg}")

    def upload_noise_file(self, path: str, mode: int = NOISE_GRAD_SOBEL):
        """A noise file, with gradients from (or cached to) <path>.grd."""
        self._io(self._lib.vvlic_upload_noise_file(self.h, os.fsencode(path), mode), "upload_noise_file")

    def upload_noise_rgba(self, rgba: np.ndarray, mode: int = NOISE_GRAD_SOBEL):
        a = np.ascontiguousarray(rgba, dtype=np.uint8)
        mz, my, mx = a.shape[:3]
        self._check(self._lib.vvlic_upload_noise_rgba(self.h, a.ctypes.data, mx, my, mz, mode), "upload_noise_rgba")

    def load_tf_png(self, name: str):
        """TransferEdit::loadTF: <name>_rgba.png (else <name>_alpha.png)."""
        self._io(self._lib.vvlic_load_tf_png(self.h, os.fsencode(name)), "load_tf_png")

    def save_tf_png(self, name: str):
        self._io(self._lib.vvlic_save_tf_png(self.h, os.fsencode(name)), "save_tf_png")

    def load_filter_png(self, path: str):
        """LICFilter::loadData: the first row's first channel as the filter table."""
        self._io(self._lib.vvlic_load_filter_png(self.h, os.fsencode(path)), "load_filter_png")

    def set_filter_table(self, table: np.ndarray, clamp: int = KERNEL_CLAMP_BORDER):
        t = np.ascontiguousarray(table, dtype=np.uint8)
        self._check(self._lib.vvlic_set_filter_table(self.h, t.ctypes.data, t.size, clamp), "set_filter_table")

    def set_filter_taps(self, taps: np.ndarray | None, lb: int = 0, lf: int = 0, inv_area: float = 0.5):
        t = None if taps is None else np.ascontiguousarray(taps, dtype=np.float32)
        self._check(self._lib.vvlic_set_filter_taps(self.h, _ptr(t), lb, lf, inv_area), "set_filter_taps")

    def filter_taps(self):
        out = np.zeros(2 * MAX_STEPS + 1, np.float32)
        ia = C.c_float(0)
        self._check(self._lib.vvlic_get_filter_taps(self.h, out.ctypes.data, out.size, C.byref(ia)), "get_filter_taps")
        p = self.params
        lb, lf = (15, 15) if p.low_res else (p.steps_backward, p.steps_forward)
        return out[: lb + lf + 1].copy(), ia.value

    @property
    def params(self) -> Params:
        p = Params()
        self._check(self._lib.vvlic_get_params(self.h, C.byref(p)), "get_params")
        return p

    def set_params(self, p: Params):
        self._check(self._lib.vvlic_set_params(self.h, C.byref(p)), "set_params")

    def set_view(self, v: View):
        self._check(self._lib.vvlic_set_view(self.h, C.byref(v)), "set_view")

    def view_rays(self, vid: int, w: int, h: int) -> np.ndarray:
        out = np.zeros(21, np.float64)
        self._check(self._lib.vvlic_view_rays(self.h, vid, w, h, out.ctypes.data), "view_rays")
        return out

    # -- rendering ------------------------------------------------------------------
    def render(self, vid: int, w: int, h: int, out: np.ndarray | None = None) -> np.ndarray:
        """Render into host memory; returns (h, w, 4) float32 (row 0 = bottom)."""
        if out is None:
            out = np.empty((h, w, 4), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == w * h * 4
        self._check(self._lib.vvlic_render(self.h, vid, out.ctypes.data, w, h), "render")
        return out

    def render_device(self, vid: int, d_out: int, w: int, h: int, d_samples: int | None = None, stream: int = 0):
        self._check(self._lib.vvlic_render_device(self.h, vid, d_out, w, h, d_samples, stream or None), "render_device")

    def render_adjoint(self, vid: int, d_grad_img: int, w: int, h: int, d_tf: int | None, d_opac: int | None,
                       d_taps: int | None, stream: int = 0):
        """Gradients of the last recording render (params.record_tape = 1) into device buffers."""
        self._check(self._lib.vvlic_render_adjoint(self.h, vid, d_grad_img, w, h, d_tf, d_opac, d_taps, stream or None),
                    "render_adjoint")

    # -- stream-ordered animation step (pointers must stay valid until the stream has run) --
    def update_field_async(self, vid: int, h_xyz: int, dims, stream: int, dtype: int = DTYPE_FLOAT32):
        nx, ny, nz = dims
        self._check(self._lib.vvlic_update_field_async(self.h, vid, h_xyz, dtype, nx, ny, nz, stream or None),
                    "update_field_async")

    def update_field_device(self, vid: int, d_xyz: int, dims, stream: int):
        nx, ny, nz = dims
        self._check(self._lib.vvlic_update_field_device(self.h, vid, d_xyz, nx, ny, nz, stream or None),
                    "update_field_device")

    def upload_noise_async(self, h_noise: int, dims, mode: int, stream: int):
        mx, my, mz = dims
        self._check(self._lib.vvlic_upload_noise_async(self.h, h_noise, mx, my, mz, mode, stream or None),
                    "upload_noise_async")

    def render_to_host_async(self, vid: int, h_out: int, w: int, h: int, stream: int):
        self._check(self._lib.vvlic_render_to_host_async(self.h, vid, h_out, w, h, stream or None),
                    "render_to_host_async")

    def compute_lic_volume(self, vid: int, dims) -> None:
        nx, ny, nz = dims
        self._check(self._lib.vvlic_compute_lic_volume(self.h, vid, nx, ny, nz), "compute_lic_volume")

    def download_lic_volume(self, vid: int, dims) -> np.ndarray:
        nx, ny, nz = dims
        out = np.empty((nz, ny, nx), np.float32)
        self._check(self._lib.vvlic_download_lic_volume(self.h, vid, out.ctypes.data, out.nbytes), "download_lic_volume")
        return out

    def batch_render(self, jobs: "list[Job]", stream: int = 0):
        arr = (Job * len(jobs))(*jobs)
        self._keep = (arr, [getattr(j, "_table", None) for j in jobs])
        self._check(self._lib.vvlic_batch_render(self.h, arr, len(jobs), stream or None), "batch_render")

    def batch_autotune(self, jobs: "list[Job]", stream: int = 0):
        arr = (Job * len(jobs))(*jobs)
        tw, smp, ms = _I(0), _I(0), C.c_float(0)
        self._check(self._lib.vvlic_batch_autotune(self.h, arr, len(jobs), stream or None, C.byref(tw), C.byref(smp),
                                                   C.byref(ms)), "batch_autotune")
        return tw.value, smp.value, ms.value

    def stats(self) -> Stats:
        s = Stats()
        self._check(self._lib.vvlic_get_stats(self.h, C.byref(s)), "get_stats")
        return s


def measure_fetch_ceiling(device: int = 0, spread4: int = 1) -> dict:
    """vvlic_measure_fetch_ceiling as a dict of rates (per second)."""
    f = FetchCeiling()
    st = load().vvlic_measure_fetch_ceiling(device, spread4, C.byref(f))
    if st:
        raise VVLICError(st, "measure_fetch_ceiling")
    return {"tex_per_s": f.tex_per_s, "ld256_per_s": f.ld256_per_s,
            "group_per_s": {"euler": f.group_per_s[0], "heun": f.group_per_s[1], "rk4": f.group_per_s[2]},
            "ms": list(f.ms), "num_sms": f.num_sms, "spread_texels": f.spread4 / 4.0}


def noise_gradients_device(d_noise: int, dims, mode: int, d_rgba: int, slice_dist=None, stream: int = 0):
    mx, my, mz = dims
    sd = None if slice_dist is None else np.asarray(slice_dist, np.float32)
    st = load().vvlic_noise_gradients_device(d_noise, mx, my, mz, mode, _ptr(sd), d_rgba, stream or None)
    if st:
        raise VVLICError(st, "noise_gradients_device")
