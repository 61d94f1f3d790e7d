"""The no-allocation noise-gradient entry point, called through the C ABI.

vvlic_noise_gradients_device_noalloc serves callers that may not allocate GPU memory while it
runs (hosts that fix their memory budget at start-up, frame loops that cannot take allocator
latency or cudaFree's synchronisation).  It keeps its temporary gradients in a fixed array
inside the library instead.  Its output must equal the allocating entry point's bit for bit —
the tolerance of every preprocessing test here — on consecutive calls that reuse the shared
array, and it must refuse sizes above its fixed maximum.

This file is named to be collected last, so a run that stops at the first failure has run
every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

pytestmark = pytest.mark.gpu


def _run(lib, fn, d_in, dims, mode, d_out, sd):
    sd_arr = np.asarray(sd, np.float32)
    mx, my, mz = dims
    return fn(d_in, mx, my, mz, mode, sd_arr.ctypes.data, d_out, None)


def test_noalloc_matches_allocating_entry_on_consecutive_calls(vvlic_lib):
    import torch

    lib = vvlic_lib
    # two different volumes back to back: the second call reuses the array holding the first
    # call's gradients, so a stale value would show up as a mismatch
    cases = [(wl.dense_noise((48, 40, 36), seed=31), (1.0, 1.0, 1.0)),
             (wl.sparse_noise((29, 23, 17), seed=32), (1.0, 0.5, 2.0))]
    for mode in (capi.NOISE_GRAD_SOBEL, capi.NOISE_GRAD_CENTRAL):
        for noise, sd in cases:
            dims = noise.shape[::-1]
            d_in = torch.from_numpy(noise).cuda()
            want = torch.zeros(noise.shape + (4,), dtype=torch.uint8, device="cuda")
            got = torch.full(noise.shape + (4,), 7, dtype=torch.uint8, device="cuda")
            assert _run(lib, lib.vvlic_noise_gradients_device, d_in.data_ptr(), dims, mode, want.data_ptr(), sd) == 0
            assert _run(lib, lib.vvlic_noise_gradients_device_noalloc, d_in.data_ptr(), dims, mode,
                        got.data_ptr(), sd) == 0
            torch.cuda.synchronize()
            np.testing.assert_array_equal(got.cpu().numpy(), want.cpu().numpy())


def test_noalloc_elongated_shapes_match_the_oracle(vvlic_lib, oracle):
    """The entry point takes any shape up to 2^20 voxels, including axes longer than the grid's
    y / z limit (65535), which the kernels step over; the bytes equal the oracle's (the FP32
    restatement that is pinned to the reference's own gradient code)."""
    import torch

    lib = vvlic_lib
    for dims, mode in (((4, 2, 131072), capi.NOISE_GRAD_SOBEL), ((2, 98304, 4), capi.NOISE_GRAD_CENTRAL),
                       ((131072, 2, 4), capi.NOISE_GRAD_CENTRAL)):
        mx, my, mz = dims
        noise = wl.dense_noise((mx, my, mz), seed=35)
        assert noise.shape == (mz, my, mx)
        d_in = torch.from_numpy(noise).cuda()
        out = torch.full(noise.shape + (4,), 3, dtype=torch.uint8, device="cuda")
        assert lib.vvlic_noise_gradients_device_noalloc(d_in.data_ptr(), mx, my, mz, mode, None, out.data_ptr(),
                                                        None) == 0, dims
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), oracle.noise_gradients(noise, mode), err_msg=str(dims))


def test_noalloc_rejects_sizes_above_its_maximum(vvlic_lib):
    import torch

    lib = vvlic_lib
    # every axis >= 2, so the voxel-count limit (VVLIC_NOALLOC_MAX_VOXELS = 2^20) is what refuses
    # them; nothing is launched, so the small buffers are never touched
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    for dims in ((1 << 19, 2, 2), (1024, 513, 2), (129, 128, 64)):
        assert dims[0] * dims[1] * dims[2] > (1 << 20) and min(dims) >= 2
        st = lib.vvlic_noise_gradients_device_noalloc(d.data_ptr(), *dims, capi.NOISE_GRAD_SOBEL, None,
                                                      d.data_ptr(), None)
        assert st == capi.ERR_INVALID_ARGUMENT, dims
    # the largest accepted size still runs (exactly the maximum number of voxels)
    big = torch.from_numpy(wl.dense_noise((128, 128, 64), seed=33)).cuda()
    out_a = torch.zeros((64, 128, 128, 4), dtype=torch.uint8, device="cuda")
    out_b = torch.ones((64, 128, 128, 4), dtype=torch.uint8, device="cuda")
    assert lib.vvlic_noise_gradients_device_noalloc(big.data_ptr(), 128, 128, 64, capi.NOISE_GRAD_CENTRAL, None,
                                                    out_a.data_ptr(), None) == 0
    assert lib.vvlic_noise_gradients_device(big.data_ptr(), 128, 128, 64, capi.NOISE_GRAD_CENTRAL, None,
                                            out_b.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(out_a, out_b)


def test_noalloc_takes_no_device_memory(vvlic_lib):
    """The call's defining property: device free memory is the same before and after a call at
    the maximum size (after a first call, which loads the library's module on this device)."""
    import torch

    lib = vvlic_lib
    big = torch.from_numpy(wl.dense_noise((128, 128, 64), seed=34)).cuda()
    out = torch.empty((64, 128, 128, 4), dtype=torch.uint8, device="cuda")

    def call():
        assert lib.vvlic_noise_gradients_device_noalloc(big.data_ptr(), 128, 128, 64, capi.NOISE_GRAD_SOBEL, None,
                                                        out.data_ptr(), None) == 0
        torch.cuda.synchronize()

    call()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        call()
    assert torch.cuda.mem_get_info()[0] == free0
