"""Host-side checks that need no GPU: the C-ABI library loads and exports
every symbol include/jpxlg.h declares; generators and covers are valid;
the multi-process replica bookkeeping of bench.py works over gloo."""
import os
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol():
    from jpxl_gb300 import _lib, build

    build.build()
    header = (ROOT / "include" / "jpxlg.h").read_text()
    declared = set(re.findall(r"\b(jpxlg_[a-z0-9_]+)\s*\(", header))
    assert declared, "no declarations parsed"
    assert declared == set(_lib.SIGNATURES), declared ^ set(_lib.SIGNATURES)
    lib = _lib.load()
    for name in declared:
        assert getattr(lib, name) is not None


def test_missing_library_fails_loudly(tmp_path):
    from jpxl_gb300 import _lib

    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(tmp_path / "libjpxlg.so")


def test_synthetic_generator_is_deterministic_and_in_range():
    from jpxl_gb300 import synth

    a = synth.synthetic_rgb(130, 70, seed=11)
    b = synth.synthetic_rgb(130, 70, seed=11)
    assert a.dtype == np.uint8 and a.shape == (70, 130, 3) and np.array_equal(a, b)
    c = synth.synthetic_rgb(130, 70, seed=11, bits=16)
    assert c.dtype == np.uint16 and np.array_equal(c, a.astype(np.uint16) * 257)
    assert a.std() > 10


def _check_cover(m):
    from jpxl_gb300 import SHAPES

    bh, bw = m.shape
    covered = np.zeros_like(m, dtype=int)
    for by in range(bh):
        for bx in range(bw):
            if m[by, bx] & 0x80:
                r, c = SHAPES[int(m[by, bx] & 0x1F)]
                assert bx % c == 0 and by % r == 0
                assert (m[by:by + r, bx:bx + c] & 0x1F == m[by, bx] & 0x1F).all()
                covered[by:by + r, bx:bx + c] += 1
    assert (covered == 1).all()


@pytest.mark.parametrize("w,h", [(64, 64), (100, 37), (257, 263)])
def test_covers_tile_the_block_grid(w, h):
    from jpxl_gb300 import synth

    _check_cover(synth.fixed_dct8_map(w, h))
    _check_cover(synth.mixed_cover(w, h, seed=5))
    _check_cover(synth.activity_cover(synth.synthetic_rgb(w, h, seed=2)))


def _replica_worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    units = bench.shard_units(list(range(10)), rank, world)
    t = bench.max_over_ranks(float(rank + 1))
    q.put((rank, units, t))
    dist.destroy_process_group()


def test_replica_sharding_over_gloo():
    """bench.py at N > 1: disjoint image lists per rank, no data-path
    collective, the timed region's maximum taken over ranks."""
    import multiprocessing as mp
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    (r0, u0, t0), (r1, u1, t1) = res
    assert sorted(u0 + u1) == list(range(10)) and not set(u0) & set(u1)
    assert t0 == t1 == 2.0
