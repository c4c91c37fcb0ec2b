"""Multi-process paths on CPU with the gloo backend (world size 2): the
bench's barrier / max-over-ranks timing and the seed-sharded walk with an
integer sum of the hit maps."""
import multiprocessing as mp
import socket

import numpy as np
import pytest

import _dist_worker as W


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run(fn, tmp_path, world=2):
    ctx = mp.get_context("spawn")
    port = _port()
    procs = [ctx.Process(target=fn, args=(r, world, port, tmp_path)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    for p in procs:
        if p.is_alive():
            p.kill()
            pytest.fail("a rank did not finish")
        assert p.exitcode == 0


def test_bench_max_over_ranks_gloo(tmp_path):
    _run(W.bench_timing, tmp_path)
    vals = [float(np.load(tmp_path / f"timing_{r}.npy")[0]) for r in range(2)]
    assert vals == [11.0, 11.0]


def test_seed_sharded_walk_equals_whole_walk_gloo(tmp_path):
    _run(W.sharded_walk, tmp_path)
    assert np.array_equal(np.load(tmp_path / "sharded.npy"), np.load(tmp_path / "whole.npy"))
