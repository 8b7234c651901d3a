"""Multi-rank lane sharding on CPU (gloo, world size 2): each rank searches the cells it owns
under the reference's interleaved ownership and the ranks agree on the global first hit,
which equals a single-rank scan of all cells. The per-cell search is the oracle (CPU); the
product part under test is the ownership and the cross-rank reduction (shard.py)."""
import itertools
import os
import socket

import numpy as np
import pytest


def _cells(n, c, d, m=6):
    def one(L, total):
        cnt = [len(range(k, L, m)) for k in range(m)]
        out = []
        for v in itertools.product(*[range(-k, k + 1, 2) for k in cnt[:-1]]):
            last = total - sum(v)
            if abs(last) <= cnt[-1] and (last + cnt[-1]) % 2 == 0:
                out.append(list(v) + [last])
        return out
    return [(x, y) for x in one(n, c) for y in one(n, d)]


def _first_hit_in(oracle, n, sig, cells, owned):
    """(raw cell index, candidate index in the cell) of the first hit in `owned`, or None."""
    for pi in owned:
        tx, ty = cells[pi]
        rows, _, _ = oracle.cd_stream(n, tx, ty, m=6)
        for k, cand in enumerate(rows):
            v, _, _, _ = oracle.complete_ab(n, sig[0], sig[1], cand[0], cand[1], 0, m=6)
            if v == 0:
                return (pi, k)
    return None


def _worker(rank, world, port, n, sig, result_path):
    import torch.distributed as dist
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import pyoracle
    from bs45_quantum_explorer_gb300.shard import global_first_hit, owned_cells
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    cells = _cells(n, sig[2], sig[3])
    local = _first_hit_in(pyoracle, n, sig, cells, owned_cells(len(cells), rank, world))
    best = global_first_hit(local)
    with open(f"{result_path}.{rank}", "w") as f:
        f.write(repr(best))
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.mark.parametrize("n,sig", [(8, (1, 1, 4, 4)), (10, (1, 1, 2, 6))])
def test_two_rank_first_hit_equals_single_rank(oracle, tmp_path, n, sig):
    import torch.multiprocessing as mp
    from bs45_quantum_explorer_gb300.shard import owned_cells
    cells = _cells(n, sig[2], sig[3])
    single = _first_hit_in(oracle, n, sig, cells, owned_cells(len(cells), 0, 1))
    path = str(tmp_path / "res")
    mp.start_processes(_worker, args=(2, _free_port(), n, sig, path), nprocs=2, join=True,
                       start_method="spawn")
    got = [eval(open(f"{path}.{r}").read()) for r in range(2)]
    assert got[0] == got[1] == single, (got, single)


def test_owned_cells_partition():
    from bs45_quantum_explorer_gb300.shard import owned_cells
    for ncells in (0, 1, 7, 100):
        for world in (1, 2, 3, 5):
            parts = [owned_cells(ncells, r, world) for r in range(world)]
            flat = sorted(itertools.chain(*parts))
            assert flat == list(range(ncells))
            # windows [skip, end) are disjoint across lanes and stay inside the list
            a = owned_cells(ncells, 0, world, skip=1, end=3)
            assert all(world <= pi < 3 * world for pi in a)
    with pytest.raises(ValueError):
        owned_cells(10, 2, 2)
