"""Replica (multi-GPU) host logic on CPU: the work partition and the process-group plumbing of
vectorvisualization_gb300.replicas, as two gloo ranks.  Each rank renders its share of an orbit's
frames with the CPU oracle (standing in for its GPU) and the frames are checked against a
single-process render: sharding changes which rank renders a frame, never the frame."""
import os
import socket

import numpy as np
import pytest

from vectorvisualization_gb300.replicas import shard, shard_by_cost


def test_shard_partitions_round_robin():
    for n in (0, 1, 7, 64):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_shard_by_cost_balances_and_agrees():
    rng = np.random.default_rng(0)
    costs = rng.uniform(1, 100, 97)
    world = 4
    parts = [shard_by_cost(costs, r, world) for r in range(world)]
    assert sorted(i for p in parts for i in p) == list(range(97))
    loads = [costs[p].sum() for p in parts]
    assert max(loads) - min(loads) <= costs.max()  # greedy longest-first bound
    assert parts == [shard_by_cost(costs, r, world) for r in range(world)]  # deterministic


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scene():
    from oracle import pyoracle
    from vectorvisualization_gb300 import capi, workloads as wl

    w = wl.c1(size=16, image=12)
    w.params.steps_forward = w.params.steps_backward = 4
    w.params.integrator = capi.HEUN
    sc = pyoracle.Scene(pyoracle.encode_field(w.field), w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    views = [wl.orbit_view(f, 6, distance=2.4) for f in range(6)]
    return w, sc, views


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from vectorvisualization_gb300.replicas import Replicas

    rep = Replicas(backend="gloo")
    w, sc, views = _scene()
    mine = rep.shard(len(views))
    rep.barrier()
    steps = 0
    for f in mine:
        img, smp = sc.render(w.params, views[f], w.width, w.height, threads=1)
        np.save(os.path.join(out_dir, f"frame{f}.npy"), img)
        steps += int(smp.sum())
    total = rep.sum(float(steps))
    slowest = rep.max(float(rank + 1))
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as fh:
        fh.write(f"{len(mine)} {total} {slowest}\n")
    rep.close()


def test_two_gloo_ranks_render_the_orbit_like_one_process(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    w, sc, views = _scene()
    steps = 0
    for f, v in enumerate(views):
        ref, smp = sc.render(w.params, v, w.width, w.height, threads=1)
        np.testing.assert_array_equal(np.load(tmp_path / f"frame{f}.npy"), ref)
        steps += int(smp.sum())
    for r in range(world):
        n, total, slowest = open(tmp_path / f"rank{r}.txt").read().split()
        assert int(n) == 3 and float(total) == steps and float(slowest) == world


def _batch():
    from oracle import pyoracle
    from vectorvisualization_gb300 import workloads as wl

    vols, noise, base = wl.c3(volumes=5, max_views=3, dims=(8, 12, 16), defaults=pyoracle.DEFAULTS)
    specs, costs = wl.c3_jobs(vols, image=8)
    return vols, noise, base, specs, costs


def _render_job(spec, noise, base):
    from oracle import pyoracle
    from vectorvisualization_gb300 import capi, workloads as wl

    bv, v = spec
    p = capi.Params.from_buffer_copy(base)
    p.steps_forward = p.steps_backward = max(2, bv.L // 10)
    rgba, op = wl.default_tf()
    sc = pyoracle.Scene(pyoracle.round_storage(pyoracle.encode_field(bv.field), "f16"), noise, rgba, op,
                        filter_table=pyoracle.filter_table(bv.filter_kind, 8))
    return sc.render(p, v, 8, 8, threads=1)[0]


def _batch_rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from vectorvisualization_gb300.replicas import Replicas

    rep = Replicas(backend="gloo")
    vols, noise, base, specs, costs = _batch()
    mine = shard_by_cost(costs, rep.rank, rep.world)
    for i in mine:
        np.save(os.path.join(out_dir, f"job{i}_rank{rank}.npy"), _render_job(specs[i], noise, base))
    total = rep.sum(float(len(mine)))
    with open(os.path.join(out_dir, f"batch_rank{rank}.txt"), "w") as fh:
        fh.write(f"{len(mine)} {total}\n")
    rep.close()


def test_two_gloo_ranks_split_the_batch_like_one_process(tmp_path):
    """The batch dealt by cost over two ranks: every job rendered by exactly one rank, the union
    equal to the single-process batch."""
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_batch_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    vols, noise, base, specs, costs = _batch()
    assert len(specs) >= 4
    for i, spec in enumerate(specs):
        owners = [r for r in range(world) if (tmp_path / f"job{i}_rank{r}.npy").exists()]
        assert len(owners) == 1, (i, owners)
        np.testing.assert_array_equal(np.load(tmp_path / f"job{i}_rank{owners[0]}.npy"),
                                      _render_job(spec, noise, base))
    counts = [open(tmp_path / f"batch_rank{r}.txt").read().split() for r in range(world)]
    assert sum(int(c[0]) for c in counts) == len(specs) and all(float(c[1]) == len(specs) for c in counts)
