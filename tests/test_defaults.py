"""Defaults and filter tables: the library's against the oracle's own restatement and against the
analytic definitions, and a CPU render of a named configuration that never loads libvvlic.

The oracle builds parameters, views and filter tables itself (oracle/vvlic_oracle.hpp
`params_default`, `view_default`, `filter_table`), so the CPU reference path needs nothing from
the product library; these tests pin the two against each other bit for bit.  No kernel runs.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def analytic_table(kind: str, width: int) -> np.ndarray:
    """LICFilter::createBoxFilter (dataset.cpp:1405-1413) and the triangle / cos^2 / Gaussian
    (sigma = L/3) profiles over texel centres x in [-1, 1], rounded to 8 bits."""
    W = 1
    while W < width:
        W <<= 1
    x = (2.0 * np.arange(W) + 1.0) / W - 1.0
    v = {"box": np.ones_like(x), "triangle": 1.0 - np.abs(x), "cos2": np.cos(0.5 * np.pi * x) ** 2,
         "gaussian": np.exp(-(x * 3.0) ** 2 / 2.0)}[kind]
    return np.floor(255.0 * np.clip(v, 0.0, 1.0) + 0.5).astype(np.uint8)


@pytest.mark.parametrize("kind", ["box", "triangle", "cos2", "gaussian"])
@pytest.mark.parametrize("width", [2, 3, 100, 256, 1000, 1024])
def test_library_filter_table_matches_oracle_and_definition(vvlic_lib, oracle, kind, width):
    lib_t = capi.make_filter_table(kind, width)
    ora_t = oracle.filter_table(kind, width)
    np.testing.assert_array_equal(lib_t, ora_t)
    ref = analytic_table(kind, width)
    assert lib_t.size == ref.size
    # the numpy profile rounds through other float operations: at most one 8-bit step apart
    assert int(np.abs(lib_t.astype(int) - ref.astype(int)).max()) <= 1


def test_box_table_is_the_reference_box(oracle):
    t = oracle.filter_table("box", 256)
    assert t.size == 256 and np.all(t == 255)
    assert oracle.filter_table("box", 100).size == 128  # nextPowerTwo
    with pytest.raises(ValueError):
        oracle.filter_table("box", 1)


def _fields(struct):
    return {name: (list(getattr(struct, name)) if hasattr(getattr(struct, name), "__len__") else getattr(struct, name))
            for name, _ in struct._fields_}


def test_oracle_defaults_match_library(vvlic_lib, oracle):
    lib_p, ora_p = _fields(capi.params_default()), _fields(oracle.params_default())
    # kernel selection has no reference counterpart: the oracle leaves it at 0
    for k in ("sampler", "schedule"):
        lib_p.pop(k)
        assert ora_p.pop(k) == 0
    assert lib_p == ora_p
    assert _fields(capi.view_default()) == _fields(oracle.view_default())
    assert _fields(capi.line_material_default()) == _fields(oracle.line_material_default())


def test_workloads_built_from_oracle_defaults_equal_library_ones(vvlic_lib, oracle):
    a = wl.c1(size=8, image=16)
    b = wl.c1(size=8, image=16, defaults=oracle.DEFAULTS)
    pa, pb = _fields(a.params), _fields(b.params)
    pa.pop("sampler"), pa.pop("schedule"), pb.pop("sampler"), pb.pop("schedule")
    assert pa == pb
    np.testing.assert_array_equal(a.filter_table, b.filter_table)
    assert _fields(a.views[0]) == _fields(b.views[0])
    c, d = wl.c2(size=8, image=16), wl.c2(size=8, image=16, defaults=oracle.DEFAULTS)
    np.testing.assert_array_equal(c.filter_table, d.filter_table)
    assert _fields(c.views[0]) == _fields(d.views[0])


def test_cpu_reference_path_does_not_load_the_library(oracle):
    """A CPU render of a small C5-shaped frame with oracle-built inputs, in a fresh process:
    libvvlic.so must not be mapped into it."""
    code = r"""
import sys
sys.path.insert(0, %r)
from oracle import pyoracle
from vectorvisualization_gb300 import workloads as wl
w = wl.c5(size=16, image=24, frames=4, defaults=pyoracle.DEFAULTS)
w.params.steps_forward = w.params.steps_backward = 4
rgba = pyoracle.round_storage(pyoracle.encode_field(w.field), w.storage)
sc = pyoracle.Scene(rgba, pyoracle.noise_gradients(w.noise, w.noise_mode), w.tf_rgba, w.tf_opac,
                    filter_table=w.filter_table)
img, smp = sc.render(w.params, w.views[1], w.width, w.height, rows=[12], precision=32, threads=1)
assert smp.sum() > 0
maps = open("/proc/self/maps").read()
print("LOADED" if "libvvlic" in maps else "CLEAN")
""" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().endswith("CLEAN"), r.stdout
