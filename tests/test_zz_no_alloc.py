"""The allocation-free LBVH entry point against the allocating one.

rg_lbvh_build_device_noalloc exists for callers that may not allocate device memory once they are
running (an engine that owns a fixed arena, a frame loop that cannot take the stall of a
cudaMalloc).  It must give the same LBVH as rg_lbvh_build_host -- bit for bit, the bar of every
LBVH test here -- on consecutive calls that share its fixed scratch array, and must reject sizes
beyond its stated maximum.  This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from test_oracle import random_boxes

pytestmark = pytest.mark.gpu

MAX_PRIMS = 65536


def _noalloc(rg, boxes):
    import torch
    n = len(boxes)
    dev = torch.device("cuda", 0)
    d_boxes = torch.from_numpy(np.ascontiguousarray(boxes, np.float32)).to(dev)
    m = max(n - 1, 1)
    outs = {"morton": torch.empty(n, dtype=torch.int32, device=dev), "order": torch.empty(n, dtype=torch.int32, device=dev),
            "left": torch.empty(m, dtype=torch.int32, device=dev), "right": torch.empty(m, dtype=torch.int32, device=dev),
            "nodeboxes": torch.empty((m, 6), dtype=torch.float32, device=dev)}
    torch.cuda.synchronize(dev)
    lib = rg.load()
    P = ctypes.c_void_p
    rc = lib.rg_lbvh_build_device_noalloc(P(d_boxes.data_ptr()), n, P(outs["morton"].data_ptr()),
                                          P(outs["order"].data_ptr()), P(outs["left"].data_ptr()),
                                          P(outs["right"].data_ptr()), P(outs["nodeboxes"].data_ptr()), None)
    torch.cuda.synchronize(dev)
    res = {k: v.cpu().numpy() for k, v in outs.items()}
    for k in ("morton", "order", "left", "right"):
        res[k] = res[k].view(np.uint32)
    if n <= 1:
        res["left"], res["right"] = res["left"][:0], res["right"][:0]
        res["nodeboxes"] = res["nodeboxes"][:0]
    return rc, res


def test_noalloc_lbvh_matches_allocating_entry_point(rg):
    ctx = rg.Context()
    # two calls in a row share the scratch array: a full-size build, then a smaller one
    for n, dup, seed in ((MAX_PRIMS, True, 11), (3001, False, 12)):
        boxes = random_boxes(n, seed, dup)
        rc, got = _noalloc(rg, boxes)
        assert rc == 0
        ref = ctx.lbvh_build_host(boxes)
        for k in ("morton", "order", "left", "right", "nodeboxes"):
            assert np.array_equal(got[k], ref[k]), (n, k)


def test_noalloc_rejects_too_large(rg):
    lib = rg.load()
    P = ctypes.c_void_p
    rc = lib.rg_lbvh_build_device_noalloc(P(16), MAX_PRIMS + 1, P(16), P(16), P(16), P(16), P(16), None)
    assert rc == -8  # RG_ERR_TOO_LARGE, returned before any pointer is touched
