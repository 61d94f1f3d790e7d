"""CPU tests of the C ABI: the library loads, exports every declared entry point, and its
host-only functions (defaults, filter tables, background composite, argument checks) behave.
No kernel is launched here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(vvlic_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(vvlic_lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(vvlic_lib, n)]
    assert not missing, missing


def test_bindings_cover_declarations(vvlic_lib):
    names = declared_functions()
    unbound = [n for n in names if n not in capi._SIGS]
    assert not unbound, unbound


def test_abi_version(vvlic_lib):
    assert vvlic_lib.vvlic_abi_version() == 1


def test_params_default_is_reference_licparams(vvlic_lib):
    p = capi.params_default()
    # LICParams() in types.h:91-99
    assert p.step_size_vol == np.float32(1.0 / 128.0)
    assert p.gradient_scale == 30.0 and p.illum_scale == 1.0 and p.freq_scale == 1.0
    assert p.num_iterations == 255 and p.steps_forward == 32 and p.steps_backward == 32
    assert p.step_size_lic == np.float32(0.01)
    assert p.integrator == capi.HEUN and p.illum == capi.ILLUM_NONE and p.tf_index == capi.TF_INDEX_DIR_Z
    assert p.eye_dist_factor == np.float32(0.3) and p.alpha_threshold == np.float32(0.95)
    assert p.quirks == capi.QUIRKS_REFERENCE and p.spec_exp == 40.0
    assert list(p.light_pos) == [0.5, 0.5, 1.5]
    assert list(p.light_ambient) == [0.0, 0.0, 0.0] and list(p.light_specular) == [1.0, 1.0, 1.0]
    assert p.sampler == capi.SAMPLER["hybrid"] and p.schedule == capi.SCHEDULE["queue"]


def test_view_default_is_reference_camera(vvlic_lib):
    v = capi.view_default()
    assert v.projection == capi.PERSPECTIVE
    assert list(v.quat) == [0, 0, 0, 1] and v.distance == 4.0 and v.fovy_deg == 35.0


def test_status_strings(vvlic_lib):
    assert vvlic_lib.vvlic_status_string(0) == b"ok"
    assert vvlic_lib.vvlic_status_string(capi.ERR_NO_DEVICE) == b"no CUDA device"
    assert vvlic_lib.vvlic_status_string(99) == b"unknown status"


def test_make_filter_table_rejects_bad_args(vvlic_lib):
    out = np.zeros(1024, np.uint8)
    w = C.c_int32(0)
    assert vvlic_lib.vvlic_make_filter_table(9, 256, out.ctypes.data, C.byref(w)) == capi.ERR_INVALID_ARGUMENT
    assert vvlic_lib.vvlic_make_filter_table(0, 1, out.ctypes.data, C.byref(w)) == capi.ERR_INVALID_ARGUMENT
    assert vvlic_lib.vvlic_make_filter_table(0, 4096, out.ctypes.data, C.byref(w)) == capi.ERR_INVALID_ARGUMENT


def test_composite_background(vvlic_lib):
    img = np.array([[[0.2, 0.1, 0.0, 0.5], [0.0, 0.0, 0.0, 0.0]]], np.float32)
    assert vvlic_lib.vvlic_composite_background(img.ctypes.data, 2, 1, None) == 0
    np.testing.assert_allclose(img[0, 0], [0.7, 0.6, 0.5, 1.0], rtol=1e-6)
    np.testing.assert_allclose(img[0, 1], [1.0, 1.0, 1.0, 1.0])


def test_null_handles_are_rejected(vvlic_lib):
    assert vvlic_lib.vvlic_destroy(None) == capi.ERR_BAD_HANDLE
    assert vvlic_lib.vvlic_render(None, 1, None, 1, 1) == capi.ERR_BAD_HANDLE
    assert vvlic_lib.vvlic_set_params(None, None) == capi.ERR_BAD_HANDLE
    assert vvlic_lib.vvlic_create(None, 0) == capi.ERR_INVALID_ARGUMENT
    assert vvlic_lib.vvlic_noise_gradients_device(None, 4, 4, 4, 1, None, None, None) == capi.ERR_INVALID_ARGUMENT


def test_create_without_gpu_reports_no_device(vvlic_lib):
    from conftest import HAS_GPU

    if HAS_GPU:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert vvlic_lib.vvlic_create(C.byref(h), 0) == capi.ERR_NO_DEVICE
    with pytest.raises(capi.VVLICError):
        capi.Context(0)


def test_splitmix64_reference_values():
    # SplitMix64 with state 0: first outputs of the published generator
    r = wl.SplitMix64(0).u64(3)
    assert [int(x) for x in r] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
