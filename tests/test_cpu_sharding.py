"""Sharding a run's photon index range across ranks (world size 2, gloo, CPU).

Photon k of a run draws the MWC stream (key, photon_offset + k), so ranks
that transport disjoint index ranges of one seed produce integer tallies
whose sum is the tally of the whole range, bit for bit.  Each rank runs the
oracle's photon-indexed restatement (the CUDA engine's exact kernel equals
it bit for bit, tests/test_gpu_parity.py) on its range with
photon_offset = rank x share; an all-reduce sums R, T and the photon hitting
density; rank 0's sum must equal the single-process run.  This is the
multi-GPU decomposition of the path (one exchange: the integer sum);
benchmark runs use one GPU per replica.  With the reference's first-photon
random-number reuse on, the reuse follows the photon's index in the whole
run (photon_offset + k < 32768), so the shards still sum to the whole run.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, total, reuse, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import pyoracle
        from tests import cases
        o = pyoracle.Oracle()
        table = o.multipliers(32769)[1:].copy()
        share = total // world
        case = cases.mismatch(photons=share, per_voxel=0)
        case.do_fl = 2  # photon hitting density, no emission phase
        sim = case.oracle_sim()
        sim.photon_offset = rank * share
        sim.launch_rng_reuse = reuse
        r = o.run_photon(sim, table, 5, 6, libm=False, nthreads=2)
        parts = [r.Rd, r.Tt, r.fhd, np.array(r.balance, dtype=np.uint64), np.array([r.steps_exc], dtype=np.uint64)]
        t = torch.from_numpy(np.concatenate(parts).view(np.int64).copy())
        dist.all_reduce(t)  # integer sum, wraps modulo 2^64 like the tallies
        if rank == 0:
            np.save(out_path, t.numpy().view(np.uint64))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("reuse", [0, 1])
def test_two_rank_shards_sum_to_the_whole_run(reuse, oracle, table32768, tmp_path):
    import torch.multiprocessing as mp
    total = 40000  # with reuse, the first 32768 photons span both shards
    out = str(tmp_path / "sum.npy")
    mp.start_processes(_worker, args=(2, _free_port(), total, reuse, out), nprocs=2, join=True,
                       start_method="spawn")
    from tests import cases
    case = cases.mismatch(photons=total, per_voxel=0)
    case.do_fl = 2
    sim = case.oracle_sim()
    sim.launch_rng_reuse = reuse
    whole = oracle.run_photon(sim, table32768, 5, 6, libm=False)
    expect = np.concatenate([whole.Rd, whole.Tt, whole.fhd, np.array(whole.balance, dtype=np.uint64),
                             np.array([whole.steps_exc], dtype=np.uint64)])
    got = np.load(out)
    assert whole.Rd.sum() > 0
    assert np.array_equal(got, expect)
