"""The C++ host side: tests/cpp/renderer_demo.cpp drives the library through vvlic::Renderer
(include/vvlic_renderer.hpp) the way the reference's 3DLIC.cpp drives its Renderer.  It must
compile and link against libvvlic.so on any machine, and on a GPU its images must equal the
same renders made through the Python binding, and match the FP64 oracle; its stream-ordered
animation step (updateDataTexAsync + renderToHostAsync) must give the first ray-cast again."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from vectorvisualization_gb300 import capi, formats, workloads as wl

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def demo(tmp_path_factory, vvlic_lib):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("cpp") / "renderer_demo"
    libdir = os.path.dirname(capi.LIB_PATH)
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "cpp", "renderer_demo.cpp"), "-o", str(out), "-L", libdir, "-lvvlic",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


def test_demo_compiles_and_links(demo):
    assert os.access(demo, os.X_OK)


def _inputs(tmp_path):
    field = wl.vortex_field((20, 18, 16), seed=9)
    noise = wl.dense_noise(16, seed=90)
    dat = str(tmp_path / "vortex.dat")
    formats.write_dat(dat, field, slice_thickness=(1.0, 1.0, 1.0))
    nz = str(tmp_path / "noise_16")
    formats.write_noise(nz, noise)
    return field, noise, dat, nz


@pytest.mark.gpu
def test_demo_images_equal_python_binding_and_match_oracle(demo, tmp_path, ctx, oracle):
    field, noise, dat, nzf = _inputs(tmp_path)
    W = H = 48
    prefix = str(tmp_path / "img")
    r = subprocess.run([demo, dat, nzf, prefix, str(W), str(H)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert os.path.getsize(prefix + "_raycast.png") > 100

    def load(tag):
        return np.fromfile(f"{prefix}_{tag}.f32", np.float32).reshape(H, W, 4)

    # the same renders through the Python binding
    vid = ctx.upload_field(field, storage="f32")
    ctx.upload_noise(noise)
    ctx.set_filter_table(capi.make_filter_table("box", 256))
    p = capi.params_default()
    p.step_size_vol = 1.0 / 64.0
    p.steps_forward = p.steps_backward = 8
    p.gradient_scale = 12.0
    p.sampler = capi.SAMPLER["cell"]
    p.tf_index = capi.TF_INDEX_MAGNITUDE
    v = capi.view_default()
    v.distance = 2.4
    ctx.set_view(v)
    imgs = {}
    for tag, tech, illum in (("raycast", "raycast", capi.ILLUM_NONE), ("slicing", "slicing", capi.ILLUM_NONE),
                             ("zoeckler", "raycast", capi.ILLUM_ZOECKLER)):
        p.technique = capi.TECHNIQUE[tech]
        p.illum = illum
        ctx.set_params(p)
        imgs[tag] = ctx.render(vid, W, H)
        np.testing.assert_array_equal(load(tag), imgs[tag], err_msg=tag)
    # the demo's stream-ordered step (updateDataTexAsync of the same field + renderToHostAsync)
    np.testing.assert_array_equal(load("async"), imgs["raycast"], err_msg="async")
    rgba, op = wl.default_tf()
    sc = oracle.Scene(oracle.encode_field(field), noise, rgba, op, filter_table=capi.make_filter_table("box", 256))
    p.technique = capi.TECHNIQUE["raycast"]
    p.illum = capi.ILLUM_NONE
    ref, _ = sc.render(p, v, W, H)
    assert float(np.sqrt(np.mean((imgs["raycast"] - ref) ** 2))) <= 1e-3
    assert float(imgs["raycast"][..., 3].max()) > 0.1
