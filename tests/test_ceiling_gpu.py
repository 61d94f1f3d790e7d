"""The L1TEX fetch-ceiling measurement (vvlic_measure_fetch_ceiling) runs and its rates are
consistent: a group with more field fetches per noise load runs at a lower group rate, and no
group rate exceeds what its fetches alone would allow."""
import pytest

from vectorvisualization_gb300 import capi

pytestmark = pytest.mark.gpu


def test_fetch_ceiling_is_consistent(vvlic_lib):
    c = capi.measure_fetch_ceiling(0, 1)
    print(c)
    assert c["num_sms"] > 0 and c["tex_per_s"] > 1e9 and c["ld256_per_s"] > 1e9
    g = c["group_per_s"]
    assert g["euler"] > g["heun"] > g["rk4"] > 0
    for k, name in ((1, "euler"), (2, "heun"), (4, "rk4")):
        assert g[name] * k <= 1.15 * c["tex_per_s"], name   # k texture fetches per group
        assert g[name] <= 1.15 * c["ld256_per_s"], name      # one 256-bit load per group


def test_fetch_ceiling_rejects_bad_arguments(vvlic_lib):
    f = capi.FetchCeiling()
    assert vvlic_lib.vvlic_measure_fetch_ceiling(0, -1, capi.C.byref(f)) == capi.ERR_INVALID_ARGUMENT
    assert vvlic_lib.vvlic_measure_fetch_ceiling(0, 1, None) == capi.ERR_INVALID_ARGUMENT
    assert vvlic_lib.vvlic_measure_fetch_ceiling(99, 1, capi.C.byref(f)) == capi.ERR_NO_DEVICE
