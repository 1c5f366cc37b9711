"""Compare two group catalogues that label the same particles.

Group ids are order-dependent (the reference numbers groups in tree
discovery order, kd.c:840-847), so catalogues are compared after matching
groups one-to-one by membership overlap: pairs (a, b) are taken greedily by
decreasing shared-member count.  Per-particle agreement counts a particle as
agreeing when both catalogues leave it ungrouped (id 0) or put it in matched
groups.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Match:
    agreement: float          # fraction of particles that agree
    n_a: int                  # groups in A (id 0 excluded)
    n_b: int
    pairs: dict               # a -> b for matched groups
    unmatched_a: list         # groups of A with no partner
    unmatched_b: list

    def same_groups(self) -> bool:
        return not self.unmatched_a and not self.unmatched_b


def match_groups(a: np.ndarray, b: np.ndarray) -> Match:
    a = np.asarray(a, np.int64)
    b = np.asarray(b, np.int64)
    if a.shape != b.shape:
        raise ValueError("catalogues label different particle counts")
    n = len(a)
    na = int(a.max(initial=0))
    nb = int(b.max(initial=0))
    both = (a > 0) & (b > 0)
    key = a[both] * (nb + 1) + b[both]
    uk, cnt = np.unique(key, return_counts=True)
    ga, gb = uk // (nb + 1), uk % (nb + 1)
    order = np.lexsort((gb, ga, -cnt))
    used_a = np.zeros(na + 1, bool)
    used_b = np.zeros(nb + 1, bool)
    pairs = {}
    agree = int(np.count_nonzero((a == 0) & (b == 0)))
    for k in order:
        x, y = int(ga[k]), int(gb[k])
        if used_a[x] or used_b[y]:
            continue
        used_a[x] = used_b[y] = True
        pairs[x] = y
        agree += int(cnt[k])
    present_a = np.zeros(na + 1, bool)
    present_a[a] = True
    present_b = np.zeros(nb + 1, bool)
    present_b[b] = True
    un_a = [int(g) for g in np.nonzero(present_a & ~used_a)[0] if g > 0]
    un_b = [int(g) for g in np.nonzero(present_b & ~used_b)[0] if g > 0]
    return Match(agree / max(n, 1), len([g for g in np.unique(a) if g > 0]),
                 len([g for g in np.unique(b) if g > 0]), pairs, un_a, un_b)


def relabel_like(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Return a copy of ``b`` whose matched groups carry the ids of ``a``."""
    m = match_groups(a, b)
    inv = {v: k for k, v in m.pairs.items()}
    out = np.zeros_like(np.asarray(b))
    nxt = int(np.max(a, initial=0)) + 1
    for g in np.unique(b):
        if g == 0:
            continue
        if g in inv:
            out[b == g] = inv[g]
        else:
            out[b == g] = nxt
            nxt += 1
    return out
