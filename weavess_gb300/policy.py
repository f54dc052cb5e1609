"""The search policies of IndexBuilder::search (src/builder.cpp:187-487): the
beam width L chosen by L_SEARCH_SET_RECALL (an adaptive walk toward the
smallest L with 10-NN accuracy >= 0.99), L_SEARCH_ASCEND (ten widths of a
Fibonacci sequence) or L_SEARCH_ASSIGN (one given width), with the
reference's accuracy figure.  The searches themselves run on the GPU
(`Context.search`, `Context.search_hnsw`); this is the host loop around them,
step for step the reference's, so that the widths it visits -- and with the
same rand stream the results, DistCount and HopCount -- match.

`search(L)` is any callable returning (ids nq x >=K, dist_count, hop_count).
"""
from __future__ import annotations

import time

import numpy as np

K_SEARCH = 10  # IndexBuilder::search fixes K = 10 (builder.cpp:190)


def reference_accuracy(res, gt, n_ground: int | None = None, K: int = K_SEARCH) -> np.float32:
    """`1 - misses / (GroundLen * K)` in FP32 (builder.cpp:306-320): a miss is
    a result id among a query's first K that is not among its first K
    ground-truth ids; ground-truth rows past the queries add no misses but
    count in the denominator."""
    res = np.asarray(res)
    gt = np.asarray(gt)
    n_ground = gt.shape[0] if n_ground is None else n_ground
    cnt = 0
    for i in range(min(res.shape[0], n_ground)):
        cnt += int(K - np.isin(res[i, :K], gt[i, :K]).sum())
    return np.float32(1) - np.float32(np.float32(cnt) / np.float32(n_ground * K))


def _step(search, L, gt, n_ground, K):
    t = time.perf_counter()
    res, dc, hc = search(L)
    dt = time.perf_counter() - t
    acc = reference_accuracy(res, gt, n_ground, K)
    return {"L": int(L), "accuracy": float(acc), "dist_count": int(dc), "hop_count": int(hc), "seconds": dt,
            "_acc32": acc}


def set_recall(search, gt, n_ground: int | None = None, K: int = K_SEARCH):
    """L_SEARCH_SET_RECALL (builder.cpp:262-351).  Returns (steps, L_min):
    every width searched, in order, and the smallest one that reached
    accuracy 0.99 (0x7fffffff if none did)."""
    sg = np.float32(1000)
    acc_set = np.float32(0.99)
    flag = False
    L_sl = 1
    L = K
    visited = {L}
    L_min = 0x7FFFFFFF
    steps = []
    while True:
        if L < K:
            raise ValueError("search_L cannot be smaller than search_K")
        st = _step(search, L, gt, n_ground, K)
        steps.append(st)
        acc = st.pop("_acc32")
        if acc_set - acc <= 0:
            L_min = min(L_min, L)
            if L == K or L_sl == 1:
                break
            if not flag:
                L_sl = L_sl - 1 if L_sl < 0 else L_sl + 1
                flag = True
            L_sl = int(L_sl / 2)  # C++ integer division truncates toward zero
            if L_sl == 0:
                break
            if L_sl > 0:
                L_sl = -L_sl
        else:
            if L_min < L:
                break
            L_sl = int(np.float32(sg * np.float32(acc_set - acc)))
            if L_sl == 0:
                L_sl += 1
            flag = False
        L = (L + L_sl) & 0xFFFFFFFF  # unsigned arithmetic, as in the reference
        if L in visited:
            break
        visited.add(L)
    return steps, L_min


def ascend(search, gt, n_ground: int | None = None, K: int = K_SEARCH):
    """L_SEARCH_ASCEND (builder.cpp:352-428): L = 13, 21, 34, ..., 987."""
    L_st, L_st2 = 5, 8
    steps = []
    for _ in range(10):
        L = L_st + L_st2
        L_st, L_st2 = L_st2, L
        st = _step(search, L, gt, n_ground, K)
        st.pop("_acc32")
        steps.append(st)
    return steps


def assign(search, L: int, gt, n_ground: int | None = None, K: int = K_SEARCH):
    """L_SEARCH_ASSIGN (builder.cpp:429-487): the one given width."""
    if L < K:
        raise ValueError("search_L cannot be smaller than search_K")
    st = _step(search, L, gt, n_ground, K)
    st.pop("_acc32")
    return [st]
