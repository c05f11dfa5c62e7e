"""Run two StrategyImprovement-shaped solvers step by step through the
reference driver loop (main.cpp:20-55) and compare their state after every
call."""
import hashlib

import numpy as np


def state_digest(si, finite_rows=True):
    """(strategy, infinite, dense rows of finite vertices) of a solver."""
    inf = si.get_infinite()
    rows = si.get_valuation() if finite_rows else None
    if rows is not None:
        rows = rows.copy()
        rows[inf != 0] = 0
    return si.get_strategy(), inf, rows


def compare_states(a, b, where):
    sa, ia, ra = a
    sb, ib, rb = b
    assert np.array_equal(sa, sb), f"{where}: strategies differ at {np.nonzero(sa != sb)[0][:10]}"
    assert np.array_equal(ia, ib), f"{where}: infinite flags differ at {np.nonzero(ia != ib)[0][:10]}"
    if ra is not None and rb is not None:
        bad = np.nonzero((ra != rb).any(axis=1))[0]
        assert bad.size == 0, f"{where}: valuations differ at vertices {bad[:10]}"


def compare_summaries(x, y, where):
    """Path-form valuations (path length, top priority, its count per vertex)
    of two solvers that both have get_summary()."""
    for name, a, b in zip(("path lengths", "top priorities", "top counts"), x.get_summary(), y.get_summary()):
        assert np.array_equal(a, b), f"{where}: {name} differ at {np.nonzero(a != b)[0][:10]}"


def lockstep(x, y, reset=False, rows=True, max_evals=100000, summary=False):
    """Drive x and y together; returns (iters, brs).  rows: compare the dense
    valuation rows after every evaluation; summary: compare the path-form
    summaries instead (for games whose dense rows would not fit)."""
    x.init_strat()
    y.init_strat()
    assert np.array_equal(x.get_strategy(), y.get_strategy()), "init_strat differs"
    iters = brs = 0
    first = True
    while True:
        if not first and reset:
            x.reset_opponent_strategy()
            y.reset_opponent_strategy()
        while True:
            if first:
                x.compute_first_val()
                y.compute_first_val()
            else:
                x.compute_valuation()
                y.compute_valuation()
            brs += 1
            compare_states(state_digest(x, rows), state_digest(y, rows), f"evaluation {brs}")
            if summary:
                compare_summaries(x, y, f"evaluation {brs}")
            x.mark_solved(1)
            y.mark_solved(1)
            a = x.switch_strategy(1)
            b = y.switch_strategy(1)
            assert a == b, f"switch(1) after evaluation {brs}: {a} != {b}"
            assert np.array_equal(x.get_strategy(), y.get_strategy()), f"strategy after switch(1) #{brs}"
            if a == 0:
                break
            assert brs < max_evals
        first = False
        x.mark_solved(0)
        y.mark_solved(0)
        iters += 1
        a = x.switch_strategy(0)
        b = y.switch_strategy(0)
        assert a == b, f"switch(0) in iteration {iters}: {a} != {b}"
        assert np.array_equal(x.get_strategy(), y.get_strategy()), f"strategy after switch(0) #{iters}"
        if a == 0:
            break
    for p in (0, 1):
        assert np.array_equal(x.get_winning(p), y.get_winning(p)), f"winning set of player {p}"
    return iters, brs


class TraceRecorder:
    """Digest of every step of a solve: sha256 of the state after each
    evaluation and after each switch, plus the switch counts."""

    def __init__(self):
        self.h = []

    def add(self, kind, *arrays, extra=None):
        d = hashlib.sha256()
        d.update(kind.encode())
        for a in arrays:
            d.update(np.ascontiguousarray(a).tobytes())
        if extra is not None:
            d.update(str(extra).encode())
        self.h.append(d.hexdigest()[:16])


def traced_solve(si, reset=False, rows=True):
    """solve_si with a digest of each step; returns (iters, brs, trace)."""
    tr = TraceRecorder()
    si.init_strat()
    tr.add("init", si.get_strategy())
    iters = brs = 0
    first = True
    while True:
        if not first and reset:
            si.reset_opponent_strategy()
        while True:
            if first:
                si.compute_first_val()
            else:
                si.compute_valuation()
            brs += 1
            _, inf, r = state_digest(si, rows)
            tr.add("eval", inf, r if r is not None else np.zeros(0, np.int32))
            si.mark_solved(1)
            k = si.switch_strategy(1)
            tr.add("sw1", si.get_strategy(), extra=k)
            if k == 0:
                break
        first = False
        si.mark_solved(0)
        iters += 1
        k = si.switch_strategy(0)
        tr.add("sw0", si.get_strategy(), extra=k)
        if k == 0:
            break
    return iters, brs, tr.h


def br_state(si):
    """State after one of Odd's best responses: (strategy, infinite, solved,
    dense rows with the rows of infinite or solved vertices zeroed)."""
    inf = si.get_infinite()
    sol = si.get_solved()
    rows = si.get_valuation().copy()
    rows[(inf != 0) | (sol != 0)] = 0
    return si.get_strategy(), inf, sol, rows


def si_best_responses(si):
    """solve_si (main.cpp:20-55, plain variant) over a StrategyImprovement-
    shaped solver, yielding br_state after each of Odd's best responses (the
    inner loop has converged), before mark_solved(0) and Even's switch."""
    si.init_strat()
    first = True
    while True:
        while True:
            if first:
                si.compute_first_val()
            else:
                si.compute_valuation()
            si.mark_solved(1)
            if si.switch_strategy(1) == 0:
                break
        first = False
        yield br_state(si)
        si.mark_solved(0)
        if si.switch_strategy(0) == 0:
            return


def bf_best_responses(bf):
    """solve_bf (main.cpp:58-76) over a Bellman-Ford solver (oracle.BellmanFord
    or oracle.RefBellmanFord), yielding (Bellman-Ford rounds so far, br_state)
    after each best response."""
    bf.init_strat()
    rounds = 0
    while True:
        rounds += bf.best_response()
        yield rounds, br_state(bf)
        bf.mark_solved(0)
        if bf.switch_strategy(0) == 0:
            return


def br_digest(owner, state, even_only=True):
    """Digest of a best response's state: Even's strategy (every vertex's with
    even_only False), infinite flags, solved flags and the finite rows."""
    strat, inf, sol, rows = state
    d = hashlib.sha256()
    d.update(np.ascontiguousarray(strat[owner == 0] if even_only else strat).tobytes())
    for a in (inf, sol, rows):
        d.update(np.ascontiguousarray(a).tobytes())
    return d.hexdigest()[:16]


def compare_br(a, b, owner, where, odd_too=False):
    """Two best-response states agree: Even's strategy (with odd_too also
    Odd's), infinite and solved flags, and the rows of finite vertices."""
    sa, ia, la, ra = a
    sb, ib, lb, rb = b
    ev = owner == 0
    sel = np.ones_like(ev) if odd_too else ev
    assert np.array_equal(sa[sel], sb[sel]), f"{where}: strategies differ at {np.nonzero(sel & (sa != sb))[0][:10]}"
    assert np.array_equal(ia, ib), f"{where}: infinite flags differ at {np.nonzero(ia != ib)[0][:10]}"
    assert np.array_equal(la, lb), f"{where}: solved flags differ at {np.nonzero(la != lb)[0][:10]}"
    bad = np.nonzero((ra != rb).any(axis=1))[0]
    assert bad.size == 0, f"{where}: valuations differ at vertices {bad[:10]}"
