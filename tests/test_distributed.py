"""Replica sharding across ranks, checked with world_size-2 gloo process groups
on the CPU.

The step loop shards by independent replicas (no data-path collective); these
tests check that every rank derives the same partition on its own, that the
shares cover each replica exactly once with balanced particle counts, that
each rank's share packs into valid per-replica parameter blocks, and that the
benchmark's job time is the max over ranks."""
import os
import socket
import sys
import pathlib

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def id_of(system):
    """A replica's identity: its size and first position (the generator draws
    every replica's size and positions from one seeded stream)."""
    return (int(system.num_slots), float(system.state.pos[0, 0]), float(system.state.pos[0, 1]))


def _worker(rank, world, port, result_dir):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import __graft_entry__ as graft
    mg = graft.load_package()
    from mavi_gb300 import abi, replicas, workloads
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        systems, step = workloads.lj_batch(num_replicas=12, n_min=200, n_max=3000, precision="mixed")
        sizes = [s.num_slots for s in systems]
        mine = replicas.my_replicas(sizes, rank, world)
        # every rank packs its own share; the parameter blocks stay per replica
        params = (abi.MaviReplicaParams * len(mine))()
        for k, i in enumerate(mine):
            systems[i].fill_params(params[k], step.kind)
            assert params[k].num_particles == sizes[i]
        gathered = [None] * world
        dist.all_gather_object(gathered, {"rank": rank, "mine": mine,
                                          "load": int(sum(sizes[i] for i in mine)),
                                          "partition": replicas.shard_replicas(sizes, world)})
        t = replicas.max_over_ranks(1.5 + rank, dist)
        # the benchmark's own sharding path: lj_batch_512 at two ranks is 1,024
        # replicas, each rank building only its share
        import importlib.util
        spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
        bench = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(bench)
        share, _ = bench.workload_share("lj_batch_512", "mixed", rank, world)
        bench_ids = [id_of(s) for s in share]
        bench_gathered = [None] * world
        dist.all_gather_object(bench_gathered, {"ids": bench_ids, "n": int(sum(s.num_slots for s in share))})
        np.save(os.path.join(result_dir, f"r{rank}.npy"),
                np.array([{"gathered": gathered, "sizes": sizes, "tmax": t, "bench": bench_gathered}],
                         dtype=object))
    finally:
        dist.destroy_process_group()


def test_shard_replicas_partition_properties(mg):
    from mavi_gb300 import replicas
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 8):
        sizes = rng.integers(1, 10000, size=37).tolist()
        shares = replicas.shard_replicas(sizes, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(37))
        loads = [sum(sizes[i] for i in s) for s in shares]
        assert max(loads) - min(loads) <= max(sizes)
        assert all(s == sorted(s) for s in shares)
    assert replicas.shard_replicas([], 2) == [[], []]
    assert replicas.shard_replicas([5], 3) == [[0], [], []]
    with pytest.raises(ValueError):
        replicas.my_replicas([1, 2], 2, 2)


def test_two_rank_gloo_replica_sharding(tmp_path, mg):
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    mp.start_processes(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    out = [np.load(tmp_path / f"r{r}.npy", allow_pickle=True)[0] for r in range(world)]
    g0 = out[0]["gathered"]
    assert [g["rank"] for g in g0] == [0, 1]
    # both ranks computed the same partition without communicating
    assert g0[0]["partition"] == g0[1]["partition"] == out[1]["gathered"][0]["partition"]
    covered = sorted(g0[0]["mine"] + g0[1]["mine"])
    assert covered == list(range(len(out[0]["sizes"])))
    assert not set(g0[0]["mine"]) & set(g0[1]["mine"])
    assert abs(g0[0]["load"] - g0[1]["load"]) <= max(out[0]["sizes"])
    # job time = the slowest rank
    assert out[0]["tmax"] == out[1]["tmax"] == 2.5
    # the benchmark's split of the 1,024-replica batch: disjoint shares that
    # together are exactly the replicas the generator makes, balanced by particles
    b = out[0]["bench"]
    from mavi_gb300 import workloads
    every, _ = workloads.lj_batch(num_replicas=1024, precision="mixed")
    assert sorted(b[0]["ids"] + b[1]["ids"]) == sorted(id_of(s) for s in every)
    assert not set(b[0]["ids"]) & set(b[1]["ids"])
    assert b[0]["n"] + b[1]["n"] == sum(s.num_slots for s in every)
    assert abs(b[0]["n"] - b[1]["n"]) <= max(s.num_slots for s in every)
