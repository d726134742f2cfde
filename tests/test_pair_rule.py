"""The pair rule decided chunk by chunk (as the drift kernel does) against
the rule over all atoms at once (as the oracle does), on the CPU.

Each chunk takes its two largest reported squared displacements b1 >= b2
(reported: at or above the bound), swaps b1 into the step's running largest
and gets the previous running largest back (old), and decides on the
candidate pair (max(b1, old), max(min(b1, old), b2)). Whatever order the
chunks arrive in, some chunk reaches a threshold exactly when the step's two
largest displacements do. The check runs in binary32 like the kernel."""
from __future__ import annotations

import numpy as np


def _pair_sum(p1, p2, low2):
    return np.float32(np.sqrt(np.float32(p1))) + np.float32(np.sqrt(np.float32(max(p2, low2))))


def _global(d2, low2, skin):
    rep = np.sort(d2[d2 >= low2])[::-1]
    if rep.size == 0:
        return 0
    t1 = rep[0]
    t2 = rep[1] if rep.size > 1 else np.float32(0)
    s = _pair_sum(t1, t2, low2)
    return 2 if s >= skin else (1 if s >= np.float32(0.5) * skin else 0)


def _chunked(d2, low2, skin, chunk, order):
    running = np.float32(0)
    best = 0
    for c in order:
        v = d2[c * chunk:(c + 1) * chunk]
        v = np.sort(v[v >= low2])[::-1]
        if v.size == 0:
            continue  # the chunk reports nothing
        b1 = v[0]
        b2 = v[1] if v.size > 1 else np.float32(0)
        old = running
        running = max(running, b1)
        s = _pair_sum(max(b1, old), max(min(b1, old), b2), low2)
        best = max(best, 2 if s >= skin else (1 if s >= np.float32(0.5) * skin else 0))
    return best


def test_chunked_decision_equals_global_rule():
    rng = np.random.default_rng(7)
    skin = np.float32(0.594)            # 0.99 x 0.6 A
    low2 = np.float32((skin / 4) ** 2)
    chunk = 8
    hits = {0: 0, 1: 0, 2: 0}
    for case in range(3000):
        n = int(rng.integers(1, 12)) * chunk
        d = rng.uniform(0.0, rng.uniform(0.05, 0.35), n).astype(np.float32)
        # a few fast atoms, sometimes two in one chunk, sometimes ties
        for _ in range(int(rng.integers(0, 3))):
            d[rng.integers(n)] = np.float32(rng.uniform(0.2, 0.6))
        if case % 7 == 0 and n > 1:
            d[1] = d[0]
        d2 = (d * d).astype(np.float32)
        want = _global(d2, low2, skin)
        hits[want] += 1
        for _ in range(3):
            order = rng.permutation(n // chunk)
            assert _chunked(d2, low2, skin, chunk, order) == want, (case, order)
    assert min(hits.values()) > 100, hits  # every outcome exercised
