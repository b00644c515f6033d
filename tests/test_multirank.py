"""Sharding histories across ranks (the multi-GPU replica path) on the CPU with
torch.distributed/gloo, world size 2: each rank runs its contiguous share of the
history range with the same seed and stream; the summed tallies equal one run
over the whole range (event counts exactly)."""
import os

import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P
import parity

H_PER_EXP = 3000
N_EXP = 4


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    from oracle import oracle as O

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ph = parity.small_cylinder(scale=4)
    w = O.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials)
    beam = P.dx_beam_params(particles=H_PER_EXP, exposures=N_EXP)
    total = H_PER_EXP * N_EXP
    lo, hi = rank * total // world, (rank + 1) * total // world
    st = w.run(beam, seed=9, stream=4, threads=2, hist_begin=lo, hist_end=hi)
    e, e2, c = w.tally()
    te = torch.from_numpy(e)
    tc = torch.from_numpy(c.astype(np.int64))
    tn = torch.tensor([st["n_histories"]], dtype=torch.int64)
    for t in (te, tc, tn):
        dist.all_reduce(t)
    if rank == 0:
        np.save(os.path.join(out_dir, "e.npy"), te.numpy())
        np.save(os.path.join(out_dir, "c.npy"), tc.numpy())
        np.save(os.path.join(out_dir, "n.npy"), tn.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_sum_to_the_full_run(oracle, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = 29500 + (os.getpid() % 2000)
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    ph = parity.small_cylinder(scale=4)
    w = oracle.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials)
    st = w.run(P.dx_beam_params(particles=H_PER_EXP, exposures=N_EXP), seed=9, stream=4, threads=4)
    e, _, c = w.tally()
    assert int(np.load(tmp_path / "n.npy")[0]) == st["n_histories"] == H_PER_EXP * N_EXP
    np.testing.assert_array_equal(np.load(tmp_path / "c.npy"), c.astype(np.int64))
    np.testing.assert_allclose(np.load(tmp_path / "e.npy"), e, rtol=1e-12, atol=1e-9)
