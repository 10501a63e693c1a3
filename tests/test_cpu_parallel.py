"""Multi-process (gloo, world size 2, CPU) tests of prc_d2z.parallel: the
max-over-ranks timing reduction used by bench.py's replicas, and the merge of
radius shards (packed-key elementwise max) against the serial oracle loop."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, outdir):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    for p in (repo, os.path.join(repo, "pr-calc_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    from oracle import d2z_ref as orc
    from prc_d2z import parallel
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # replica timing: every rank reports its own time; all see the max
        m = parallel.max_over_ranks(1.0 + rank)
        # radius shards of one box, merged
        g = dict(np.load(os.path.join(here, "golden", "d2z_n16.npz")))
        R, B = g["radii_mpc"], g["barrier_b"]
        shard = parallel.shard_radii(len(R), world, rank)
        z, am, _ = orc.d2z(g["delta"].astype(np.float64), float(g["box_mpc"]), R, float(g["barrier_a"]), B,
                           float(g["dinit"]), mode="fp64", radii_idx=list(shard))
        zt = torch.from_numpy(z.astype(np.float32))
        at = torch.from_numpy(am)
        parallel.merge_radius_shards(zt, at)
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), z=zt.numpy(), am=at.numpy(), m=m,
                 shard=np.array([shard.start, shard.stop]))
    finally:
        dist.destroy_process_group()


def test_two_rank_merge_and_timing(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    here = os.path.dirname(os.path.abspath(__file__))
    import sys
    sys.path.insert(0, os.path.dirname(here))
    from oracle import d2z_ref as orc
    g = dict(np.load(os.path.join(here, "golden", "d2z_n16.npz")))
    zf, af, _ = orc.d2z(g["delta"].astype(np.float64), float(g["box_mpc"]), g["radii_mpc"], float(g["barrier_a"]),
                        g["barrier_b"], float(g["dinit"]), mode="fp64")
    shards = []
    for r in range(2):
        o = np.load(os.path.join(tmp_path, f"rank{r}.npz"))
        assert float(o["m"]) == 2.0
        assert np.array_equal(o["z"], zf.astype(np.float32))
        assert np.array_equal(o["am"], af)
        shards.append(tuple(o["shard"]))
    assert shards[0][0] == 0 and shards[0][1] == shards[1][0] and shards[1][1] == len(g["radii_mpc"])


def test_pack_keys_order_and_ties():
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "pr-calc_gb300"))
    from prc_d2z.parallel import pack_keys, shard_radii, unpack_keys
    z = torch.tensor([-3.0, -1.0, 0.0, 0.0, 2.5, 2.5, 7.0], dtype=torch.float32)
    am = torch.tensor([4, 2, 255, 255, 9, 3, 0], dtype=torch.uint8)
    k = pack_keys(z, am)
    zz, aa = unpack_keys(k)
    assert torch.equal(zz, z) and torch.equal(aa, am)
    assert bool((k[:-1] <= k[1:])[[0, 1, 2, 5]].all())
    assert int(k[5]) > int(k[4])       # equal z: the smaller radius wins
    assert [len(shard_radii(10, 3, q)) for q in range(3)] == [4, 3, 3]
