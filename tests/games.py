"""Seeded workloads of the parity tests, by family, at sizes the oracle
finishes in seconds.  Families follow the measured configurations:
  c1       random game, n=10,000, out-degree U[2,10], priority U[0,n)
  c2       random game, out-degree U[2,5], priority U[0,n)      (scaled n)
  c3       long-path game, priority U[0,1024), owner alternating (scaled n)
  c4       random game, out-degree U[2,8], priority U[0,n)      (one batch member)
  ring10   the 10-vertex game v -> v+1, v+2 (mod 10), priority = owner = v mod 2
  evencyc  no cycle with an odd top priority (the precondition of the reference's
           Bellman-Ford solver, cpu_bv.cpp:73-85): see evencyc_csr
  cycles   Odd cycles of lengths 2^k - 1, 2^k, 2^k + 1 with trees hanging off them:
           see cycle_forest
"""
import numpy as np

import psi


def ring10():
    n = 10
    owner = np.array([v % 2 for v in range(n)], np.int32)
    pri = owner.copy()
    off = np.arange(0, 2 * n + 1, 2, dtype=np.int32)
    tg = np.array([x for v in range(n) for x in ((v + 1) % n, (v + 2) % n)], np.int32)
    return psi.Game.from_csr(owner, pri, off, tg)


def _splitmix64(state):
    """One step of splitmix64 over a one-element list holding the state."""
    state[0] = (state[0] + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = state[0]
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def evencyc_csr(n: int, seed: int):
    """A random game in which every cycle has an even top priority.  Hubs
    (vertices [0, h), h = max(2, n/32)) carry the highest priorities, all
    even; every other vertex has successors among higher ids and hubs only.
    A cycle needs an edge to a lower id, so it passes through a hub, and its
    top priority is a hub's.  Owner uniform, out-degree uniform in [2, 5]
    (fewer where fewer successors are allowed), distinct non-self
    successors, other priorities uniform in [0, 256).  Drawn from splitmix64
    in plain Python, so the game is the same on every machine."""
    st = [seed * 0xD1B54A32D192ED03 & 0xFFFFFFFFFFFFFFFF]
    below = lambda k: (_splitmix64(st) >> 11) % k   # noqa: E731 (bias < 2^-40: irrelevant here)
    h = max(2, n // 32)
    base = 256
    owner = np.array([below(2) for _ in range(n)], np.int32)
    pri = np.array([below(base) for _ in range(n)], np.int32)
    pri[:h] = base + 2 * np.arange(h)
    off = [0]
    tg = []
    for v in range(n):
        avail = n - 1 if v < h else (n - 1 - v) + h   # distinct choices there are
        deg = min(2 + below(4), avail)
        succ = []
        while len(succ) < deg:
            if v < h:
                u = below(n)
            elif v + 1 < n and below(4) != 0:
                u = v + 1 + below(n - v - 1)
            else:
                u = below(h)
            if u != v and u not in succ:
                succ.append(u)
        tg += succ
        off.append(len(tg))
    return owner, pri, np.array(off, np.int32), np.array(tg, np.int32)


CYCLE_LENGTHS = (1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257, 1000)


def cycle_forest(scale, seed):
    """Odd vertices whose first successors form cycles of the lengths above
    (powers of two and their neighbours, where the cycle pass's doubling
    windows just fit or just miss a cycle) with trees hanging off them, some
    of them long chains; a quarter of the Odd vertices may also leave for an
    Even vertex, and the Even vertices (an eighth of all) choose among random
    vertices.  Vertex ids are shuffled and priorities lie in [0, 48), so
    equal priorities are common.  In the first evaluation every Odd vertex is
    unreached (its strategy stays in the forest); later ones also meet solved
    vertices."""
    rng = np.random.default_rng(seed)
    succ = []
    for c in CYCLE_LENGTHS[:scale]:
        b = len(succ)
        succ += [b + (i + 1) % c for i in range(c)]
    n_cyc = len(succ)
    for k in range(4):                      # long chains into random cycle vertices
        prev = int(rng.integers(n_cyc))
        for _ in range(50 + 150 * k):
            succ.append(prev)
            prev = len(succ) - 1
    for _ in range(5 * n_cyc):              # random trees
        succ.append(int(rng.integers(len(succ))))
    n_odd = len(succ)
    n_even = max(2, n_odd // 7)
    n = n_odd + n_even
    perm = rng.permutation(n)               # perm[i]: the id of construction vertex i
    lists = [None] * n
    for i, s in enumerate(succ):
        out = [int(perm[s])]
        if rng.random() < 0.25:
            out.append(int(perm[n_odd + rng.integers(n_even)]))
        lists[perm[i]] = out
    for j in range(n_even):
        lists[perm[n_odd + j]] = [int(x) for x in rng.integers(n, size=int(rng.integers(2, 4)))]
    owner = np.zeros(n, np.int32)
    owner[perm[:n_odd]] = 1
    pri = rng.integers(0, 48, n).astype(np.int32)
    off = np.zeros(n + 1, np.int32)
    off[1:] = np.cumsum([len(x) for x in lists])
    tgt = np.array([u for x in lists for u in x], np.int32)
    return psi.Game.from_csr(owner, pri, off, tgt)


def make(family: str, n: int, seed: int):
    if family == "c1":
        return psi.Game.random(n, 2, 10, n, seed)
    if family == "c2":
        return psi.Game.random(n, 2, 5, n, seed)
    if family == "c3":
        return psi.Game.longpath(n, 1024, seed)
    if family == "c4":
        return psi.Game.random(n, 2, 8, n, seed)
    if family == "smallpri":
        return psi.Game.random(n, 2, 5, 8, seed)
    if family == "ring10":
        return ring10()
    if family == "evencyc":
        return psi.Game.from_csr(*evencyc_csr(n, seed))
    if family == "cycles":   # n: how many of CYCLE_LENGTHS
        return cycle_forest(n, seed)
    raise ValueError(family)
