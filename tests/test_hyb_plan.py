"""The HYB form's warp work lists (hbicg__hyb_plan, host code in libhbicg.so,
no GPU): every item in exactly one list, each list in order of dealing
(non-increasing cost), loads within the greedy bound (a list's load exceeds
the least one by at most the cost of the item last dealt to it), and the same
lists on every call."""
import ctypes as C

import numpy as np
import pytest


def _plan(lib, cost, hnw):
    f = lib.hbicg__hyb_plan
    f.restype = C.c_int
    f.argtypes = [C.c_size_t, C.c_void_p, C.c_uint, C.c_void_p, C.c_void_p]
    cost = np.ascontiguousarray(cost, dtype=np.uint32)
    hwbeg = np.zeros(hnw + 1, dtype=np.uint32)
    hitem = np.zeros(max(len(cost), 1), dtype=np.uint32)
    assert f(len(cost), cost.ctypes.data, hnw, hwbeg.ctypes.data, hitem.ctypes.data) == 0
    return hwbeg, hitem[:len(cost)]


def _greedy(cost, hnw):
    """The rule restated: costliest first (ties: lower item), each to the list
    with the least load so far (ties: lower list)."""
    order = sorted(range(len(cost)), key=lambda i: (-int(cost[i]), i))
    load = [0] * hnw
    lists = [[] for _ in range(hnw)]
    for i in order:
        w = min(range(hnw), key=lambda w: (load[w], w))
        lists[w].append(i)
        load[w] += int(cost[i])
    return lists


@pytest.mark.parametrize("ni,hnw,seed", [(0, 4, 0), (5, 1, 1), (3, 16, 2), (200, 7, 3), (1000, 96, 4),
                                         (3000, 96, 5)])
def test_lists_follow_the_greedy_rule(lib, ni, hnw, seed):
    rng = np.random.default_rng(seed)
    # the mix of a power-law matrix: many cheap slices, a tail of long rows
    cost = np.where(rng.random(ni) < 0.8, rng.integers(3, 12, ni), rng.integers(3, 140, ni)).astype(np.uint32)
    hwbeg, hitem = _plan(lib, cost, hnw)
    assert hwbeg[0] == 0 and hwbeg[-1] == ni and np.all(np.diff(hwbeg.astype(np.int64)) >= 0)
    assert sorted(hitem.tolist()) == list(range(ni))
    want = _greedy(cost, hnw)
    for w in range(hnw):
        got = hitem[hwbeg[w]:hwbeg[w + 1]].tolist()
        assert got == want[w], w
        c = cost[got].astype(np.int64)
        assert np.all(np.diff(c) <= 0)
    loads = np.array([cost[hitem[hwbeg[w]:hwbeg[w + 1]]].sum() for w in range(hnw)], dtype=np.int64)
    if ni:
        last = np.array([cost[hitem[hwbeg[w + 1] - 1]] if hwbeg[w + 1] > hwbeg[w] else 0 for w in range(hnw)])
        assert np.all(loads - last <= loads.min())
    hwbeg2, hitem2 = _plan(lib, cost, hnw)
    assert np.array_equal(hwbeg, hwbeg2) and np.array_equal(hitem, hitem2)


def test_equal_costs_deal_round_robin(lib):
    """With equal costs the rule deals items to lists 0, 1, ... in turn."""
    hwbeg, hitem = _plan(lib, np.full(10, 5), 4)
    lists = [hitem[hwbeg[w]:hwbeg[w + 1]].tolist() for w in range(4)]
    assert lists == [[0, 4, 8], [1, 5, 9], [2, 6], [3, 7]]
