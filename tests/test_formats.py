"""On-disk formats (vectorvisualization_gb300.formats over formats.cpp): the .dat/.raw reader
against the reference's own DatFile (golden results generated by tests/golden/make_dat_golden.py
from reader.cpp compiled unmodified, and live when oracle/_ref is built), the noise file, and the
PNG / PPM image dump."""
import ctypes as C
import json
import os
import struct
import sys
import zlib

import numpy as np
import pytest

from vectorvisualization_gb300 import capi, formats

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from dat_cases import CASES, make_case  # noqa: E402

REF = os.path.join(HERE, "..", "oracle", "_ref", "libvvref_sobel.so")


def ours(path):
    try:
        i = formats.parse_dat(path)
    except capi.VVLICError:
        return {"ok": False}
    return {"ok": True, "raw_file": i.raw_file, "resolution": list(i.resolution),
            "slice_thickness": [float(v) for v in i.slice_thickness], "format": i.format,
            "components": i.components, "timestep_begin": i.timestep_begin, "timestep_end": i.timestep_end}


@pytest.fixture
def empty_cwd(tmp_path, monkeypatch):
    d = tmp_path / "_cwd"
    d.mkdir()
    monkeypatch.chdir(d)
    return tmp_path


def test_dat_parse_matches_reference_golden(empty_cwd):
    with open(os.path.join(HERE, "golden", "dat_golden.json")) as fh:
        golden = json.load(fh)
    assert set(golden) == {c[0] for c in CASES}
    for name, text, raws in CASES:
        p = make_case(str(empty_cwd), name, text, raws)
        got = ours(p)
        want = dict(golden[name])
        if got["ok"]:
            got["raw_file"] = got["raw_file"].replace(os.path.join(str(empty_cwd), name), "<DIR>")
        assert got == want, name


def _ref_lib():
    if not os.path.exists(REF):
        pytest.skip("oracle/_ref not built (the reference sources are not present)")
    return C.CDLL(os.path.abspath(REF))


def _ref_parse(lib, path):
    raw = C.create_string_buffer(1024)
    sizes, dists = (C.c_int * 3)(), (C.c_float * 3)()
    t, dim, b, e = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    if lib.vvref_dat_parse(path.encode(), raw, 1024, sizes, dists, C.byref(t), C.byref(dim), C.byref(b), C.byref(e)):
        return {"ok": False}
    return {"ok": True, "raw_file": raw.value.decode(), "resolution": list(sizes),
            "slice_thickness": [float(v) for v in dists], "format": t.value, "components": dim.value,
            "timestep_begin": b.value, "timestep_end": e.value}


def test_dat_parse_fuzz_against_reference(empty_cwd):
    """Random key orders, spacing, comments, number spellings and bad lines, parsed by both."""
    lib = _ref_lib()
    rng = np.random.default_rng(7)
    ints = lambda v: rng.choice([str(v), f"0x{v:x}", f"0{v:o}", f"+{v}", f" {v} "])  # noqa: E731
    fmts = ["UCHAR3", "FLOAT3", "USHORT", "FLOAT", "UCHAR 3", "FLOAT x3 data", "uchar3", "INT3"]
    for k in range(150):
        nx, ny, nz = (int(v) for v in rng.integers(1, 9, 3))
        lines = [
            f"ObjectFileName{rng.choice([':', ' :', ':  '])}r{k}.raw{rng.choice(['', '  # c', ' extra'])}",
            f"Resolution:{ints(nx)} {ints(ny)} {ints(nz)}",
            f"SliceThickness: {rng.choice(['1 1 1', '0.5 2 1e0', '2.5e-1 1 3', '1 2'])}",
            f"Format: {rng.choice(fmts)}",
        ]
        if rng.random() < 0.3:
            lines.append(f"TimeDependent: {rng.choice(['0 0', '1 0', '-1 2', '0'])}")
        if rng.random() < 0.3:
            lines.insert(int(rng.integers(0, len(lines))), rng.choice(["# comment", "Unknown: 3", "", "   "]))
        rng.shuffle(lines)
        text = rng.choice(["\n", "\r\n"]).join(lines) + "\n"
        p = make_case(str(empty_cwd), f"f{k}", text, {f"r{k}.raw": 8 * 3 * 512})
        want = _ref_parse(lib, p)
        got = ours(p)
        if want["ok"] and want["format"] == 0:  # no Format line parsed: the reference leaves
            want.pop("components"), got.pop("components", None)  # the component count unset
        assert got == want, text


def test_dat_read_matches_reference_and_numpy(empty_cwd):
    rng = np.random.default_rng(3)
    field = rng.standard_normal((3, 4, 5, 3)).astype(np.float32)
    p = str(empty_cwd / "v.dat")
    formats.write_dat(p, field, slice_thickness=(1.0, 0.5, 2.0))
    info = formats.parse_dat(p)
    assert info.resolution == (5, 4, 3) and info.components == 3 and info.format == capi.DAT_FLOAT
    np.testing.assert_array_equal(formats.read_dat(info), field)
    got, sd = formats.load_vector_dataset(p)
    np.testing.assert_array_equal(got, field)
    assert sd == (1.0, 0.5, 2.0)
    if os.path.exists(REF):
        lib = _ref_lib()
        buf = np.empty_like(field)
        assert lib.vvref_dat_read(p.encode(), 0, buf.ctypes.data, C.c_long(buf.nbytes)) == 0
        np.testing.assert_array_equal(buf, field)


def test_dat_timesteps_and_errors(empty_cwd):
    steps = [np.full((2, 3, 4, 3), t, np.uint8) for t in range(3)]
    p = str(empty_cwd / "t.dat")
    formats.write_dat(p, None, timesteps=steps)
    info = formats.parse_dat(p)
    assert (info.timestep_begin, info.timestep_end) == (0, 2)
    for t in range(3):
        np.testing.assert_array_equal(formats.read_dat(info, t), steps[t])
    with pytest.raises(capi.VVLICError):
        formats.read_dat(info, 3)
    # a truncated raw file is an error (the reference returns a partly filled buffer)
    with open(str(empty_cwd / "t_1.raw"), "r+b") as fh:
        fh.truncate(10)
    with pytest.raises(capi.VVLICError, match="holds 10 of 72 bytes"):
        formats.read_dat(info, 1)
    with pytest.raises(capi.VVLICError, match="cannot open"):
        formats.parse_dat(str(empty_cwd / "nope.dat"))
    # a raw-file pattern with a non-integer conversion is rejected, not formatted
    bad = str(empty_cwd / "bad.dat")
    with open(bad, "w") as fh:
        fh.write("ObjectFileName: x%s.raw\nResolution: 1 1 1\nFormat: UCHAR3\n")
    with pytest.raises(capi.VVLICError):
        formats.parse_dat(bad)
    # a scalar set is not a vector data set
    s = str(empty_cwd / "s.dat")
    formats.write_dat(s, np.zeros((2, 2, 2), np.uint8))
    with pytest.raises(capi.VVLICError):
        formats.load_vector_dataset(s)


def test_noise_file_layout_and_roundtrip(tmp_path):
    rng = np.random.default_rng(1)
    noise = rng.integers(0, 256, (3, 5, 7), dtype=np.uint8)
    p = str(tmp_path / "noise_7_5_3")
    formats.write_noise(p, noise)
    raw = open(p, "rb").read()
    assert struct.unpack("<3i", raw[:12]) == (7, 5, 3)  # x, y, z sizes, x fastest
    assert raw[12:] == noise.tobytes()
    np.testing.assert_array_equal(formats.read_noise(p), noise)
    with open(p, "r+b") as fh:
        fh.truncate(12 + 50)
    with pytest.raises(capi.VVLICError):
        formats.read_noise(p)
    with open(p, "wb") as fh:
        fh.write(struct.pack("<3i", -1, 5, 3))
    with pytest.raises(capi.VVLICError):
        formats.read_noise(p)


def _decode_png(data: bytes):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert zlib.crc32(typ + body) & 0xFFFFFFFF == crc
        chunks.setdefault(typ, b"")
        chunks[typ] += body
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert (depth, ctype) == (8, 6)
    raw = zlib.decompress(chunks[b"IDAT"])
    rows = np.frombuffer(raw, np.uint8).reshape(h, 4 * w + 1)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 4)


def test_png_dump_is_the_saved_texture(tmp_path):
    rng = np.random.default_rng(2)
    img = rng.uniform(-0.2, 1.2, (37, 300, 4)).astype(np.float32)  # > 64 KiB of rows: several blocks
    p = str(tmp_path / "a.png")
    formats.write_image(p, img)
    got = _decode_png(open(p, "rb").read())
    want = np.clip((np.float32(255.0) * img).astype(np.int64), 0, 255).astype(np.uint8)[::-1]  # (int)(255 v)
    np.testing.assert_array_equal(got, want)
    # over white: clamp((1 - a) * 1 + c, 0, 1)
    formats.present(p, img)
    comp = np.clip((1.0 - img[..., 3:4]) + img, 0, 1).astype(np.float32)
    want = np.clip((np.float32(255.0) * comp).astype(np.int64), 0, 255).astype(np.uint8)[::-1]
    np.testing.assert_array_equal(_decode_png(open(p, "rb").read()), want)


def test_ppm_dump(tmp_path):
    img = np.zeros((2, 3, 4), np.float32)
    img[0, 0] = (1.0, 0.5, 0.25, 1.0)  # bottom-left pixel
    p = str(tmp_path / "a.ppm")
    formats.write_image(p, img)
    data = open(p, "rb").read()
    head = b"P6\n3 2\n255\n"
    assert data.startswith(head)
    px = np.frombuffer(data[len(head):], np.uint8).reshape(2, 3, 3)
    assert tuple(px[1, 0]) == (255, 127, 63) and px[0].max() == 0


@pytest.mark.gpu
def test_upload_dat_matches_upload_field(ctx, oracle, tmp_path):
    from vectorvisualization_gb300 import workloads as wl

    field = wl.vortex_field((12, 10, 8), seed=4)
    p = str(tmp_path / "v.dat")
    formats.write_dat(p, field, slice_thickness=(1.0, 1.0, 2.0))
    vid = ctx.upload_dat(p, storage="f32")
    np.testing.assert_array_equal(ctx.download_field(vid, (12, 10, 8), "f32"), oracle.encode_field(field))
    steps = [wl.abc_field((6, 6, 6)), wl.vortex_field((6, 6, 6), seed=2)]
    p2 = str(tmp_path / "t.dat")
    formats.write_dat(p2, None, timesteps=steps)
    vid = ctx.upload_dat(p2, timestep=1)
    np.testing.assert_array_equal(ctx.download_field(vid, (6, 6, 6), "f32"), oracle.encode_field(steps[1]))


# ---- PNG reading (pngRead) and the TF / filter PNG loaders -----------------------------------
def _png(path, img, filters, level=9, ctype=None, depth=8, interlace=0, corrupt=False):
    """A PNG written here with Python's zlib and per-row filter types (the forward filters)."""
    h, w = img.shape[:2]
    ch = img.shape[2] if img.ndim == 3 else 1
    ctype = ctype if ctype is not None else {1: 0, 2: 4, 3: 2, 4: 6}[ch]
    a = img.reshape(h, w * ch).astype(np.int64)
    raw = bytearray()
    for y in range(h):
        ft = filters[y % len(filters)]
        row = a[y]
        up = a[y - 1] if y else np.zeros_like(row)
        left = np.concatenate([np.zeros(ch, np.int64), row[:-ch]])
        ul = np.concatenate([np.zeros(ch, np.int64), up[:-ch]])
        if ft == 0:
            pred = np.zeros_like(row)
        elif ft == 1:
            pred = left
        elif ft == 2:
            pred = up
        elif ft == 3:
            pred = (left + up) // 2
        else:
            pa, pb, pc = np.abs(up - ul), np.abs(left - ul), np.abs(left + up - 2 * ul)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, up, ul))
        raw.append(ft)
        raw += bytes(((row - pred) & 0xFF).astype(np.uint8))

    def chunk(t, d):
        c = struct.pack(">I", len(d)) + t + d
        crc = zlib.crc32(t + d) & 0xFFFFFFFF
        return c + struct.pack(">I", crc ^ (1 if corrupt and t == b"IDAT" else 0))

    z = zlib.compress(bytes(raw), level)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    data += chunk(b"IDAT", z[: len(z) // 2]) + chunk(b"IDAT", z[len(z) // 2:]) + chunk(b"IEND", b"")
    with open(path, "wb") as fh:
        fh.write(data)


@pytest.mark.parametrize("channels", [1, 2, 3, 4])
@pytest.mark.parametrize("level", [0, 1, 9])
def test_png_read_all_filters_and_colour_types(tmp_path, channels, level):
    rng = np.random.default_rng(channels * 10 + level)
    # smooth content compresses with back-references and dynamic codes; noise with literals
    y, x = np.mgrid[0:23, 0:37]
    smooth = ((x * 7 + y * 3) % 256).astype(np.uint8)
    img = np.stack([smooth] * channels, -1) if channels > 1 else smooth[..., None]
    img[::3] = rng.integers(0, 256, img[::3].shape, dtype=np.uint8)
    p = str(tmp_path / "t.png")
    _png(p, img, filters=[0, 1, 2, 3, 4, 4, 3], level=level)
    np.testing.assert_array_equal(formats.read_png(p), img)


def test_png_read_of_the_image_dump(tmp_path):
    img = np.random.default_rng(4).uniform(0, 1, (9, 11, 4)).astype(np.float32)
    p = str(tmp_path / "d.png")
    formats.write_image(p, img)
    want = np.clip((np.float32(255.0) * img).astype(np.int64), 0, 255).astype(np.uint8)[::-1]
    np.testing.assert_array_equal(formats.read_png(p), want)


def test_png_read_rejects_what_pngread_rejects(tmp_path):
    img = np.zeros((4, 4, 3), np.uint8)
    cases = {"depth16": dict(depth=16), "palette": dict(ctype=3), "interlaced": dict(interlace=1),
             "crc": dict(corrupt=True)}
    for name, kw in cases.items():
        p = str(tmp_path / f"{name}.png")
        _png(p, img, [0], **kw)
        with pytest.raises(capi.VVLICError):
            formats.read_png(p)
    p = str(tmp_path / "text.png")
    open(p, "wb").write(b"not a png at all")
    with pytest.raises(capi.VVLICError, match="not a PNG"):
        formats.read_png(p)
    with pytest.raises(capi.VVLICError, match="cannot open"):
        formats.read_png(str(tmp_path / "missing.png"))


@pytest.mark.gpu
def test_tf_and_filter_png_loaders(ctx, tmp_path):
    rng = np.random.default_rng(8)
    n = capi.TF_ENTRIES
    # RGBA file present: r, g, b, a set; opacity untouched, the alpha file is not read
    rgba = rng.integers(0, 256, (2, n, 4), dtype=np.uint8)
    alpha = rng.integers(0, 256, (1, n, 2), dtype=np.uint8)
    _png(str(tmp_path / "tf_rgba.png"), rgba, [1])
    _png(str(tmp_path / "tf_alpha.png"), alpha, [2])
    _, op0 = ctx.get_tf()
    ctx.load_tf_png(str(tmp_path / "tf.png"))
    got, op = ctx.get_tf()
    np.testing.assert_array_equal(got, rgba[0].astype(np.float32) / 255.0)
    np.testing.assert_array_equal(op, op0)
    # no RGBA file: the alpha file sets alpha and opacity; a name without extension
    _png(str(tmp_path / "only_alpha.png"), alpha, [4])
    ctx.load_tf_png(str(tmp_path / "only"))
    got2, op2 = ctx.get_tf()
    np.testing.assert_array_equal(got2[:, :3], got[:, :3])
    np.testing.assert_array_equal(got2[:, 3], alpha[0, :, 0].astype(np.float32) / 255.0)
    np.testing.assert_array_equal(op2, alpha[0, :, 1].astype(np.float32) / 255.0)
    with pytest.raises(capi.VVLICError):
        ctx.load_tf_png(str(tmp_path / "nothing.png"))
    # a gray RGBA file too short for 256 entries
    _png(str(tmp_path / "short_rgba.png"), rng.integers(0, 256, (10, 20, 1), dtype=np.uint8), [0])
    with pytest.raises(capi.VVLICError):
        ctx.load_tf_png(str(tmp_path / "short.png"))
    # save and load back
    ctx.save_tf_png(str(tmp_path / "saved.png"))
    a = formats.read_png(str(tmp_path / "saved_rgba.png"))
    b = formats.read_png(str(tmp_path / "saved_alpha.png"))
    assert a.shape == (10, n, 4) and b.shape == (10, n, 2)
    np.testing.assert_array_equal(a[3], np.round(got2 * 255).astype(np.uint8))
    np.testing.assert_array_equal(b[7, :, 1], np.round(op2 * 255).astype(np.uint8))
    # filter kernel: the first channel of the first row, centred like vvlic_set_filter_table
    k = np.zeros((3, 100, 2), np.uint8)
    k[0, :, 0] = (255 * np.hanning(100)).astype(np.uint8)
    _png(str(tmp_path / "kernel.png"), k, [3])
    ctx.load_filter_png(str(tmp_path / "kernel.png"))
    t1, ia1 = ctx.filter_taps()
    ctx.set_filter_table(k[0, :, 0])
    t2, ia2 = ctx.filter_taps()
    np.testing.assert_array_equal(t1, t2)
    assert ia1 == ia2 and ia1 != 0.5  # not the box filter


# ---- the noise gradient cache (.grd) ------------------------------------------------------------
def test_reference_grd_layout_is_the_quantised_gradient_xyz(tmp_path):
    """The reference's own saveGradients writes 3 bytes per voxel, x fastest: the RGB of the
    gradient texels (pins the cache format vvlic_upload_noise_file reads and writes)."""
    lib = _ref_lib()
    from oracle import pyoracle

    noise = np.random.default_rng(11).integers(0, 256, (5, 6, 7), dtype=np.uint8)
    dims = np.array([7, 6, 5], np.int32)
    base = str(tmp_path / "n")
    lib.vvref_save_gradients.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p]
    assert lib.vvref_save_gradients(noise.ctypes.data, dims.ctypes.data, base.encode()) == 0
    grd = np.fromfile(base + ".grd", np.uint8)
    want = pyoracle.noise_gradients(noise, capi.NOISE_GRAD_SOBEL)[..., :3]
    np.testing.assert_array_equal(grd, want.reshape(-1))


@pytest.mark.gpu
def test_noise_file_gradient_cache(ctx, oracle, tmp_path):
    noise = np.random.default_rng(12).integers(0, 256, (9, 10, 11), dtype=np.uint8)
    path = str(tmp_path / "noise_11")
    formats.write_noise(path, noise)
    ctx.upload_noise_file(path, capi.NOISE_GRAD_SOBEL)
    ref = oracle.noise_gradients(noise, capi.NOISE_GRAD_SOBEL)
    np.testing.assert_array_equal(ctx.download_noise((11, 10, 9), 4), ref)
    # the cache written for the next time: the quantised gradient xyz
    grd = np.fromfile(path + ".grd", np.uint8)
    np.testing.assert_array_equal(grd, ref[..., :3].reshape(-1))
    # a cache present is used as is (the reference does not record the gradient mode either)
    fake = np.full(grd.shape, 7, np.uint8)
    fake.tofile(path + ".grd")
    ctx.upload_noise_file(path, capi.NOISE_GRAD_CENTRAL)
    got = ctx.download_noise((11, 10, 9), 4)
    assert (got[..., :3] == 7).all()
    np.testing.assert_array_equal(got[..., 3], noise)
    # a short cache is ignored and rewritten
    fake[:10].tofile(path + ".grd")
    ctx.upload_noise_file(path, capi.NOISE_GRAD_SOBEL)
    np.testing.assert_array_equal(ctx.download_noise((11, 10, 9), 4), ref)
    assert os.path.getsize(path + ".grd") == 3 * noise.size
    # scalar noise needs no cache
    p2 = str(tmp_path / "noise_scalar")
    formats.write_noise(p2, noise)
    ctx.upload_noise_file(p2, capi.NOISE_SCALAR)
    assert not os.path.exists(p2 + ".grd")
    np.testing.assert_array_equal(ctx.download_noise((11, 10, 9), 1), noise)
