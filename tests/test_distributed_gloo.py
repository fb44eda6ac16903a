"""The multi-process path on CPU: two gloo ranks shard a batch (or a pattern file), each runs
a stand-in band detector on its slice (no GPU here), rank 0 gathers the records in order,
and the timing reduction takes the maximum over ranks."""
import os
import socket

import numpy as np
import pytest

from pyebsdindex_gb300.band_detect import record_dtype
from pyebsdindex_gb300.distributed import shard_bounds


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                s, e = shard_bounds(n, r, world)
                seen.extend(range(s, e))
                assert e - s in (n // world, n // world + 1)
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


class _StubDetect:
    """Records whose 'max' is the pattern's sum: checks which patterns a rank processed."""
    nBands = 3
    dataType = record_dtype(10)

    def find_bands(self, pats, **kw):
        out = np.zeros((len(pats), self.nBands), dtype=self.dataType)
        out["max"] = pats.reshape(len(pats), -1).sum(1, dtype=np.float64)[:, None]
        return out

    def find_bands_file(self, path, patStart=0, nPat=-1, **kw):
        from pyebsdindex_gb300.ebsd_pattern import get_pattern_file_obj
        pats, _ = get_pattern_file_obj(path).read_data(patStartCount=[patStart, nPat], returnArrayOnly=True)
        return self.find_bands(pats.astype(np.float32))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from pyebsdindex_gb300.distributed import find_bands_sharded, gather_records, max_time
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pats = np.arange(11 * 4 * 4, dtype=np.float32).reshape(11, 4, 4)
    start, rec = find_bands_sharded(_StubDetect(), pats, rank, world)
    allrec = gather_records(start, rec)
    t = max_time(0.5 + rank)
    if rank == 0:
        q.put((allrec["max"][:, 0].tolist(), t))
    dist.barrier()
    dist.destroy_process_group()


def _file_worker(rank, world, port, path, q):
    import torch.distributed as dist
    from pyebsdindex_gb300.distributed import find_bands_file_sharded, gather_records
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    start, rec = find_bands_file_sharded(_StubDetect(), path, rank, world)
    allrec = gather_records(start, rec)
    if rank == 0:
        q.put(allrec["max"][:, 0].tolist())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_a_pattern_file(tmp_path, built_lib):
    """Each rank reads only its share of an .ebsp file; rank 0 gathers the records in order."""
    import multiprocessing as mp
    from pyebsdindex_gb300.ebsd_pattern import write_ebsp
    pats = (np.arange(13 * 6 * 6) % 251).astype(np.uint8).reshape(13, 6, 6)
    path = os.path.join(tmp_path, "s.ebsp")
    write_ebsp(path, pats, nCols=13, nRows=1)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_file_worker, args=(r, 2, port, path, q)) for r in range(2)]
    for p in procs:
        p.start()
    maxes = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert maxes == pats.reshape(13, -1).sum(1, dtype=np.float64).tolist()


def test_two_gloo_ranks_shard_and_gather():
    import multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    maxes, t = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    pats = np.arange(11 * 4 * 4, dtype=np.float32).reshape(11, 4, 4)
    assert maxes == pats.reshape(11, -1).sum(1, dtype=np.float64).tolist()
    assert t == 1.5
