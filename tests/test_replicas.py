"""The multi-rank path on CPU: world size 2 over gloo (127.0.0.1).  Frame
shards cover the list exactly once; the timing reduction takes the slowest
rank, the count reduction sums the ranks; each rank's decode of its shard
(oracle, CPU) equals the single-process decode of the same frames."""
import os
import socket

import numpy as np
import pytest

from cusat_gb300 import replicas


def test_shards_partition():
    for n in (0, 1, 5, 64, 1023):
        for world in (1, 2, 3, 8):
            spans = [replicas.shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.dirname(here))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle_lib as O
    from channel import frames
    from cusat_gb300 import enums as E
    from cusat_gb300 import replicas as R
    fs, rate, mod = E.FECFRAME_SHORT, E.RATE_1_2, E.MOD_QPSK
    _, _, noisy, n0, gain = frames(mod, rate, fs, 6, 1.6, seed=11)
    import cusat_gb300 as cs
    llr = O.demap_modcod(noisy, O.modcod(mod, rate, fs), n0, gain)
    a, b = R.shard(len(llr), rank, world)
    hard, trials = O.ldpc_decode(fs, rate, llr[a:b], 30, nthreads=1)
    t_max = R.reduce_timing([1.0 + rank, 5.0 - rank])
    n_sum = R.reduce_sum([b - a, 1])
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), a=a, b=b, hard=hard, trials=trials, t_max=t_max, n_sum=n_sum)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_over_gloo(tmp_path):
    import torch.multiprocessing as mp
    import oracle_lib as O
    from channel import frames
    import cusat_gb300 as cs
    from cusat_gb300 import enums as E
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r = [np.load(tmp_path / f"rank{k}.npz") for k in range(2)]
    assert int(r[0]["a"]) == 0 and int(r[0]["b"]) == int(r[1]["a"]) and int(r[1]["b"]) == 6
    for k in range(2):
        assert list(r[k]["t_max"]) == [2.0, 5.0]
        assert list(r[k]["n_sum"]) == [6.0, 2.0]
    fs, rate, mod = E.FECFRAME_SHORT, E.RATE_1_2, E.MOD_QPSK
    _, _, noisy, n0, gain = frames(mod, rate, fs, 6, 1.6, seed=11)
    llr = O.demap_modcod(noisy, O.modcod(mod, rate, fs), n0, gain)
    hard, trials = O.ldpc_decode(fs, rate, llr, 30, nthreads=2)
    assert (np.concatenate([r[0]["hard"], r[1]["hard"]]) == hard).all()
    assert (np.concatenate([r[0]["trials"], r[1]["trials"]]) == trials).all()
