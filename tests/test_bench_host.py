"""Host logic of bench.py that needs no GPU: the frames each replica renders, the roofline and
cacheless byte arithmetic, the digest gate on committed DRAM traffic, the schedule choice and
the command-line defaults the driver relies on."""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_orbit_frames_spread_evenly_and_partition_over_replicas():
    assert bench.orbit_frames(8, 1, 0) == [0, 8, 16, 24, 32, 40, 48, 56]
    assert bench.orbit_frames(64, 1, 0) == list(range(64))
    for world in (2, 4, 8):
        per_rank = [bench.orbit_frames(8, world, r) for r in range(world)]
        assert all(len(f) == 8 for f in per_rank)
        union = sorted(f for fr in per_rank for f in fr)
        total = 8 * world
        if total <= bench.ORBIT_FRAMES:  # distinct frames while the orbit has enough of them
            assert len(set(union)) == total
        assert union == sorted((k * bench.ORBIT_FRAMES // total) % bench.ORBIT_FRAMES for k in range(total))


def test_roofline_arithmetic():
    ceiling = {"group_per_s": {"euler": 400e9, "heun": 230e9, "rk4": 130e9}}
    steps, samples, ms = 1.2e11, 1.0e9, 1000.0
    r = bench.roofline(steps, samples, ms, 2, "f16", True, 2048 * 2048, ceiling, "no such key")
    assert r["bound"] == "l1tex" and r["traffic"] is None
    assert r["per_launch"]["noise_cell_loads"] == steps + samples
    assert r["per_launch"]["field_fetches"] == 4 * steps + samples
    assert r["achieved"] == pytest.approx((steps + samples) / 1.0 / 1e9)
    assert r["peak"] == pytest.approx(130.0) and r["frac"] == pytest.approx(r["achieved"] / 130.0)
    assert bench.roofline(steps, samples, ms, 1, "f16", True, 1, None, "")["frac"] is None


def test_cacheless_bytes_model():
    # 8 * (k * s_F + s_N) per sample-step, 8 * s_F per sample, 16 B per pixel
    assert bench.cacheless_bytes(10, 2, 1, "f16", False, 3) == 10 * 8 * (2 * 8 + 1) + 2 * 8 * 8 + 3 * 16
    assert bench.cacheless_bytes(1, 0, 2, "f32", True, 0) == 8 * (4 * 16 + 4)
    assert [bench.bytes_per_texel(s) for s in ("f32", "f16", "bf16", "u8")] == [16, 8, 8, 4]


def test_traffic_is_reported_only_for_the_sources_it_was_captured_from(tmp_path, monkeypatch):
    from vectorvisualization_gb300 import build

    (tmp_path / "profiles").mkdir()
    rec = {"k": {"bytes_per_launch": 123, "source_digest": build.source_digest()},
           "stale": {"bytes_per_launch": 456, "source_digest": "0000000000000000"}}
    (tmp_path / "profiles" / "ncu_traffic.json").write_text(json.dumps(rec))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.load_traffic("k") == 123
    assert bench.load_traffic("stale") is None
    assert bench.load_traffic("missing") is None


def test_schedule_and_defaults(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert (a.gpus, a.steps, a.warmup, a.impl) == (1, 8, 3, "ours")
    assert a.warmup >= 3
    assert bench.schedule(a, "orbit") == "static" and bench.schedule(a, "c2") == "queue"
    monkeypatch.setattr(sys, "argv", ["bench.py", "--schedule", "queue", "--no-rows"])
    a = bench.parse()
    assert bench.schedule(a, "orbit") == "queue" and a.no_rows
