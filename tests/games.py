"""Seeded workloads of the parity tests, by family, at sizes the oracle
finishes in seconds.  Families follow the measured configurations:
  c1       random game, n=10,000, out-degree U[2,10], priority U[0,n)
  c2       random game, out-degree U[2,5], priority U[0,n)      (scaled n)
  c3       long-path game, priority U[0,1024), owner alternating (scaled n)
  c4       random game, out-degree U[2,8], priority U[0,n)      (one batch member)
  ring10   the 10-vertex game v -> v+1, v+2 (mod 10), priority = owner = v mod 2
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
    raise ValueError(family)
