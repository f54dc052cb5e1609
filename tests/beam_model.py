"""A plain-Python statement of the throughput form of the route search
(weavess_gb300/csrc/wv_beam.cu), the checker of its GPU kernel.

The throughput form has no counterpart in the reference: it is a best-first
beam search over the same graph that expands the E best unexpanded pool
entries per step.  Its rules:

* seeds: distances in drawn order, stably sorted by distance, a repeated id
  keeps its first entry, the pool padded to L with empty (+inf) slots; the
  seeds are marked visited;
* a step takes the first E unexpanded pool positions (from the restart
  position on) and marks them expanded; the pool's last distance at that
  moment is the acceptance threshold;
* the parents' rows are walked in pool order, each in adjacency order; an id
  not visited before is fresh (and becomes visited); every fresh id costs a
  distance;
* fresh ids closer than the threshold are merged into the pool stably (pool
  entries before equal candidates, candidates in visit order among equals),
  truncated to L;
* the next step restarts at min(the smallest final position of a merged
  candidate, the last parent's position + 1);
* low-precision candidates: the finite head of the final pool (up to
  `rerank` entries) is re-scored by `exact` and stably re-sorted -- except
  bf16 candidates of integer data at d <= 128, which are exact and are not
  re-scored (pass rerank=0).

On integer data in [0, 255] (d <= 128) every distance path of the kernel is
exact, so this statement and the kernel agree id for id, distance for
distance, counter for counter.
"""
from __future__ import annotations

import numpy as np

NONE = 0x7FFFFFFF
INF = np.float32(np.inf)


def int_dist(base, q, ids):
    """Exact squared L2 of integer rows (as float32)."""
    x = base[np.asarray(ids, np.int64)].astype(np.int64)
    return ((x - q.astype(np.int64)[None, :]) ** 2).sum(1).astype(np.float32)


def beam_search(base, query, ids, deg, seeds, L, K, E, dist=int_dist, rerank=0, exact=None):
    nq = query.shape[0]
    out_ids = np.zeros((nq, K), np.uint32)
    out_d = np.zeros((nq, K), np.float32)
    dcount = hcount = 0
    for qi in range(nq):
        q = query[qi]
        s = seeds[qi, :L].astype(np.int64)
        d = dist(base, q, s)
        dcount += L
        order = sorted(range(L), key=lambda i: (d[i], i))
        seen = set()
        pool = []  # [dist, id, unexpanded]
        for i in order:
            if int(s[i]) in seen:
                continue
            seen.add(int(s[i]))
            pool.append([float(d[i]), int(s[i]), True])
        while len(pool) < L:
            pool.append([float(INF), NONE, False])

        def first_flag(frm):
            for p in range(frm, L):
                if pool[p][2]:
                    return p
            return L

        k = first_flag(0)
        while k < L:
            parents = []
            p = k
            while p < L and len(parents) < E:
                if pool[p][2]:
                    parents.append(p)
                p += 1
            for p in parents:
                pool[p][2] = False
            hcount += len(parents)
            thr = pool[L - 1][0]
            fresh = []
            for p in parents:
                node = pool[p][1]
                for m in range(int(deg[node])):
                    nid = int(ids[node, m])
                    if nid not in seen:
                        seen.add(nid)
                        fresh.append(nid)
            cands = []
            if fresh:
                fd = dist(base, q, np.array(fresh, np.int64))
                dcount += len(fresh)
                cands = [[float(fd[i]), fresh[i], True] for i in range(len(fresh)) if fd[i] < thr]
            nk = L
            if cands:
                cands.sort(key=lambda c: c[0])  # stable: visit order among equals
                tagged = [(e[0], 0, e) for e in pool] + [(c[0], 1, c) for c in cands]
                tagged.sort(key=lambda t: t[0])  # stable: pool entries first among equals
                pool = [t[2] for t in tagged[:L]]
                pos = [i for i, t in enumerate(tagged[:L]) if t[1] == 1]
                nk = min(pos) if pos else L
            k = first_flag(min(nk, parents[-1] + 1))
        if exact is not None and rerank > 0:
            finite = sum(1 for e in pool if e[0] != float(INF))
            R = min(rerank, finite)
            head = pool[:R]
            ed = exact(base, q, np.array([e[1] for e in head], np.int64))
            dcount += R
            o = sorted(range(R), key=lambda i: (ed[i], i))
            pool = [[float(ed[i]), head[i][1], False] for i in o] + pool[R:]
        out_ids[qi] = [e[1] for e in pool[:K]]
        out_d[qi] = [e[0] for e in pool[:K]]
    return out_ids, out_d, dcount, hcount
