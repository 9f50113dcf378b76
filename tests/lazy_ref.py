"""CPU restatement of the lazy check loop for the tests: the search loop of
src/dbastar/dbastar.cpp:809-919 walks a node's neighbours in order,
exact-checks each and stops after limit_branching_factor motions were taken
(:916-918).  Given every candidate's exact verdict (from the oracle) and a
ranking, the motions a node takes are the first `limit` valid ones in rank
order, and the checks it needs are the candidates up to the last of those
(all of them when the node has fewer valid ones)."""
import numpy as np


def ord_score(score):
    """order-preserving float32 -> uint32 map of the library (NaN last)"""
    s = np.asarray(score, np.float32)
    u = s.view(np.uint32).astype(np.uint64)
    out = np.where(u & 0x80000000, (~u) & 0xFFFFFFFF, u | 0x80000000)
    return np.where(np.isnan(s), 0xFFFFFFFF, out).astype(np.uint64)


def lazy_accept(node, prim, valid, score, limit):
    """node, prim: candidate lists; valid: bool per candidate; score: float32
    per candidate or None (motion order).  Returns (accepted mask, needed
    mask): the accepted candidates and the ranked prefix of every node up to
    its last accepted candidate (the whole list if it has fewer than
    `limit` valid candidates)."""
    node = np.asarray(node, np.int64)
    prim = np.asarray(prim, np.int64)
    hi = ord_score(score) if score is not None else np.zeros(len(node), np.uint64)
    key = (hi << np.uint64(32)) | prim.astype(np.uint64)
    order = np.lexsort((key, node))
    accepted = np.zeros(len(node), bool)
    needed = np.zeros(len(node), bool)
    n_s = node[order]
    starts = np.flatnonzero(np.r_[True, n_s[1:] != n_s[:-1]]) if len(n_s) else np.zeros(0, np.int64)
    ends = np.r_[starts[1:], len(n_s)]
    for s, e in zip(starts, ends):
        idx = order[s:e]
        v = valid[idx]
        c = np.cumsum(v)
        take = v & (c <= limit)
        accepted[idx[take]] = True
        if c[-1] >= limit:
            last = int(np.searchsorted(c, limit))   # position of the limit-th valid
            needed[idx[:last + 1]] = True
        else:
            needed[idx] = True
    return accepted, needed
