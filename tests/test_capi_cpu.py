"""C ABI checks that need no GPU: the library loads, exports every function include/bubblephysics.h declares, the
record layouts match, the host helpers agree with their restatements, and the multi-rank bench combination works
over gloo with two processes."""
import ctypes as C
import os
import re
import socket
from pathlib import Path

import numpy as np
import pytest

from bubblephysics_gb300 import _native as N
from bubblephysics_gb300 import scenes
from bubblephysics_gb300.solver import static_polygon_edges

HEADER = Path(__file__).resolve().parent.parent / "include" / "bubblephysics.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bp_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = N.library()
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(N.EXPORTED_SYMBOLS) | {"bp_batch_adjacency_entries"}


def test_abi_version_and_status_strings():
    lib = N.library()
    assert lib.bp_abi_version() == 1
    assert lib.bp_status_string(N.E_CONTACT_VIOLATION) == b"contact violation"


def test_record_sizes_match_the_header():
    for record, size in N.RECORD_SIZES.items():
        assert C.sizeof(record) == size
    assert N.BUBBLE_DTYPE.itemsize == 80 and N.SEGMENT_DTYPE.itemsize == 64 and N.BODY_DTYPE.itemsize == 80
    assert N.REPORT_DTYPE.itemsize == 96 and N.CONTACT_DTYPE.itemsize == 64 and N.KEY_DTYPE.itemsize == 24


def test_no_device_is_reported_without_failing():
    status = N.library().bp_device_available(0)
    assert status in (N.OK, N.E_UNAVAILABLE)


@pytest.mark.parametrize("seed", range(12))
def test_static_polygon_edges_match_the_restatement(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 9))
    angles = np.sort(rng.uniform(0, 2 * np.pi, n))
    if seed % 2:
        angles = angles[::-1]  # clockwise ring
    radius = rng.uniform(5, 50, n)
    pts = np.stack([np.cos(angles) * radius, np.sin(angles) * radius], 1).astype(np.float32)
    if seed % 3 == 0:  # add a collinear midpoint that the merge must remove
        mid = ((pts[0].astype(np.float64) + pts[1]) / 2).astype(np.float32)
        pts = np.insert(pts, 1, mid, axis=0)
    native = static_polygon_edges(pts, 100, 7)
    restated = scenes.polygon_edges(pts, 100, 7)
    assert len(native) == len(restated)
    for f in ("id", "owner_id", "a", "b", "previous_start", "outward_sign", "flags"):
        assert np.array_equal(native[f], restated[f]), f


def test_degenerate_polygon_gives_plain_segments():
    pts = np.array([[0, 0], [1, 1], [2, 2]], np.float32)
    out = static_polygon_edges(pts, 5)
    assert len(out) == 3
    assert (out["flags"] & N.SEGMENT_POLYGON_EDGE == 0).all()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    device_s = 1.0 + rank          # rank 1 is slower
    substeps = 1000.0 * (rank + 1)
    t, total = bench.combine_ranks(device_s, substeps, dist)
    out.put((rank, t, total))
    dist.destroy_process_group()


def test_multi_rank_combination_over_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, total in results:
        assert t == 2.0 and total == 3000.0
