"""Certificate check of solutions (psi_check_solution).

CPU: the oracle's solutions pass; planted mistakes of every kind are caught;
on small games the verdict agrees with a brute-force statement of the same
conditions for randomly perturbed solutions.  GPU: the solver's own results
pass, up to the full 2^24-vertex headline game, where the oracle cannot run
(a size-independent property of the result)."""
import numpy as np
import pytest

import oracle
import psi
from games import make, ring10


def oracle_solution(g, reset=False):
    o = oracle.Oracle(*g.csr())
    o.solve(reset=reset)
    out = o.get_strategy(), o.get_infinite()
    o.close()
    return out


def brute_force_ok(g, strategy, infinite):
    """The same certificate conditions, stated directly: legal entries,
    closure and trap, and for every priority p of the wrong parity no vertex
    of priority p on a cycle through vertices of priority <= p (per region,
    with the winner's strategy fixed)."""
    owner, pri, off, tgt = g.csr()
    n = g.n
    succ = [list(tgt[off[v]:off[v + 1]]) for v in range(n)]
    w0 = infinite == 1
    for v in range(n):
        s = strategy[v]
        if not ((s == -1 and owner[v] == 0) or s in succ[v]):
            return False
        if (owner[v] == 0) == w0[v]:
            if s < 0 or w0[s] != w0[v]:
                return False
        elif any(w0[u] != w0[v] for u in succ[v]):
            return False
    for region, bad, fixed_owner in ((True, 1, 0), (False, 0, 1)):
        verts = [v for v in range(n) if w0[v] == region]
        edges = {v: ([strategy[v]] if owner[v] == fixed_owner else succ[v]) for v in verts}
        for u in verts:
            if pri[u] % 2 != bad:
                continue
            # can u reach itself through vertices of priority <= pri[u] in the region?
            seen, frontier = set(), [x for x in edges[u] if x in edges and pri[x] <= pri[u]]
            while frontier:
                x = frontier.pop()
                if x == u:
                    return False
                if x in seen:
                    continue
                seen.add(x)
                frontier.extend(y for y in edges[x] if y in edges and pri[y] <= pri[u])
    return True


@pytest.mark.parametrize("fam,n,seed", [
    ("ring10", 10, 0), ("c1", 10000, 1), ("c2", 20000, 2), ("c3", 5000, 3), ("c4", 8000, 4), ("smallpri", 6000, 5)])
def test_oracle_solutions_pass(fam, n, seed):
    g = ring10() if fam == "ring10" else make(fam, n, seed)
    st, inf = oracle_solution(g)
    r = psi.check_solution(g, st, inf)
    assert r["status"] == "ok", r
    assert 0 < r["edge_visits"] <= 4 * (g.n + g.m)


def test_reset_variant_regions_are_right_but_odd_strategy_is_no_certificate():
    """The reset variant (main.cpp:27-28) also resets Odd's solved vertices
    (cpu_parity.cpp:300-307): they take their first successor again, and as
    their value is frozen no later evaluation notices when those choices
    close a cycle with an even top priority.  The regions stay right."""
    g = make("c2", 8000, 6)
    st0, inf0 = oracle_solution(g)
    st1, inf1 = oracle_solution(g, reset=True)
    assert np.array_equal(inf0 == 1, inf1 == 1)
    r = psi.check_solution(g, st1, inf1)
    assert r["status"] == "bad cycle" and inf1[r["vertex"]] != 1   # inside Odd's region
    assert psi.check_solution(g, st0, inf1)["status"] == "ok"


def test_planted_mistakes_are_caught():
    g = make("c2", 3000, 9)
    st, inf = oracle_solution(g)
    owner, pri, off, tgt = g.csr()
    # an entry that is not a successor
    bad = st.copy()
    v = int(np.flatnonzero(owner == 1)[0])
    bad[v] = next(u for u in range(g.n) if u not in set(tgt[off[v]:off[v + 1]]))
    r = psi.check_solution(g, bad, inf)
    assert (r["status"], r["vertex"]) == ("bad strategy", v)
    # Odd at the sink
    bad = st.copy()
    bad[v] = -1
    assert psi.check_solution(g, bad, inf)["status"] == "bad strategy"
    # swapping the regions breaks closure or traps
    swapped = np.where(inf == 1, -1, 1).astype(np.int32)
    assert psi.check_solution(g, st, swapped)["status"] in ("not closed", "not a trap")
    # one vertex moved to the other region
    caught = 0
    for v in range(0, g.n, 97):
        moved = inf.copy()
        moved[v] = -1 if inf[v] == 1 else 1
        caught += psi.check_solution(g, st, moved)["status"] != "ok"
    assert caught > 0


def test_bad_cycle_is_caught():
    # one Even vertex of priority 1 with a self-loop: Odd wins it; claiming it
    # for Even passes closure and trap but not the cycle parity
    g = psi.Game.from_csr([0], [1], [0, 1], [0])
    r = psi.check_solution(g, [0], [1])
    assert (r["status"], r["vertex"]) == ("bad cycle", 0)
    assert psi.check_solution(g, [0], [-1])["status"] == "ok"
    # a 3-cycle 0 -> 1 -> 2 -> 0 with top priority 5 (odd) inside a claimed W0
    g = psi.Game.from_csr([0, 1, 0], [2, 5, 4], [0, 1, 2, 3], [1, 2, 0])
    r = psi.check_solution(g, [1, 2, 0], [1, 1, 1])
    assert (r["status"], r["vertex"]) == ("bad cycle", 1)
    assert psi.check_solution(g, [1, 2, 0], [-1, -1, -1])["status"] == "ok"


def test_cycle_check_budget():
    g = make("c1", 5000, 11)
    st, inf = oracle_solution(g)
    assert psi.check_solution(g, st, inf, work_budget=10)["status"] == "incomplete"
    assert psi.check_solution(g, st, inf, work_budget=10 * (g.n + g.m))["status"] == "ok"


@pytest.mark.parametrize("seed", range(6))
def test_agrees_with_brute_force_on_perturbed_solutions(seed):
    rng = np.random.default_rng(seed)
    for trial in range(30):
        fam = ("c1", "smallpri", "c3")[trial % 3]
        g = make(fam, 12 + trial % 9, seed * 1000 + trial)
        st, inf = oracle_solution(g)
        owner, pri, off, tgt = g.csr()
        st, inf = st.copy(), inf.copy()
        for _ in range(int(rng.integers(0, 3))):
            v = int(rng.integers(g.n))
            if rng.random() < 0.5:
                inf[v] = 1 if inf[v] != 1 else -1
            else:
                st[v] = int(rng.choice(tgt[off[v]:off[v + 1]]))
        expect = brute_force_ok(g, st, inf)
        got = psi.check_solution(g, st, inf)["status"] == "ok"
        assert got == expect, (fam, g.n, trial)


@pytest.mark.gpu
@pytest.mark.parametrize("fam,n,seed", [("c1", 10000, 21), ("c2", 1 << 20, 22), ("c3", 1 << 18, 23), ("c4", 1 << 19, 24)])
def test_gpu_solutions_pass(fam, n, seed):
    g = make(fam, n, seed)
    s = psi.GPUList(g)
    s.solve()
    r = psi.check_solution(g, s.get_strategy(), s.get_infinite())
    s.close()
    assert r["status"] == "ok", r


@pytest.mark.gpu
def test_gpu_headline_game_solution_passes():
    """The 2^24-vertex random game (out-degree U[2,5], priority U[0,n)): no
    oracle can solve it, but its solution can be certified."""
    g = psi.Game.random(1 << 24, 2, 5, 1 << 24, 1)
    s = psi.GPUList(g)
    s.solve()
    st, inf = s.get_strategy(), s.get_infinite()
    s.close()
    r = psi.check_solution(g, st, inf, work_budget=40 * (g.n + g.m))
    assert r["status"] == "ok", r
