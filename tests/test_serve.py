"""Continuous-batching server: games submitted at different times share one
resident arena, join at step boundaries and leave when done; each must end
exactly as its solo solve -- strategy, infinity flags (hence winning sets),
iteration and evaluation counts -- whatever else is resident."""
import numpy as np
import pytest

import oracle
import psi
from games import make, ring10
from test_batch import c4_games


def oracle_result(g, reset=False):
    o = oracle.Oracle(*g.csr())
    it_br = o.solve(reset=reset)
    out = it_br, o.get_strategy(), o.get_infinite()
    o.close()
    return out


def check_against(srv, ticket, expected, label):
    state, it, br = srv.status(ticket)
    assert state == psi.Server.FINISHED, label
    strat, inf = srv.take(ticket)
    (eit, ebr), estrat, einf = expected
    assert (it, br) == (eit, ebr), label
    assert np.array_equal(strat, estrat), label
    assert np.array_equal(inf, einf), label


def test_server_rejects_oversize_arena_before_touching_a_device():
    with pytest.raises(psi.PsiError) as e:
        psi.Server(1 << 31, 1 << 20, 4)
    assert e.value.code == 4   # PSI_ERR_TOO_LARGE


@pytest.mark.gpu
def test_serve_staggered_arrivals_match_solo_oracle():
    games = c4_games(30, 20, 3000, 13) + [psi.Game.longpath(400, 64, 5), ring10(), make("smallpri", 700, 2),
                                          make("cycles", 12, 7)]
    expected = [oracle_result(g) for g in games]
    srv = psi.Server(max_vertices=20000, max_edges=120000, max_games=12)
    tickets = {}
    pending = list(range(len(games)))
    steps = 0
    while pending or srv.info()[:2] != (0, 0):
        # a few arrivals before every step
        for _ in range(3):
            if pending:
                k = pending.pop(0)
                tickets[srv.submit(games[k])] = k
        srv.step()
        steps += 1
        for t, k in list(tickets.items()):
            if srv.status(t)[0] == psi.Server.FINISHED:
                check_against(srv, t, expected[k], f"game {k}")
                del tickets[t]
        assert steps < 10000
    assert not tickets
    assert srv.info() == (0, 0, 0, 0)


@pytest.mark.gpu
def test_serve_reset_variant_matches_solo_oracle():
    games = c4_games(16, 20, 2000, 21) + [ring10()]
    expected = [oracle_result(g, reset=True) for g in games]
    srv = psi.Server(max_vertices=40000, max_edges=300000, max_games=32, reset=True)
    tickets = [srv.submit(g) for g in games]
    srv.drain()
    for k, t in enumerate(tickets):
        check_against(srv, t, expected[k], f"game {k}")


@pytest.mark.gpu
def test_serve_first_fit_admission_and_reuse():
    # Four small games hold 4,304 of 8,000 vertex slots; a 6,000-vertex game
    # submitted next cannot fit and waits, while a 2,500-vertex game submitted
    # after it is admitted past it.  As games leave, their ranges are freed and
    # coalesced; every result matches the solo GPU solve.
    first = [make("c4", n, 40 + i) for i, n in enumerate([900, 1500, 700, 1200])]
    big = make("c4", 6000, 31)
    late = make("c4", 2500, 50)
    arena_v, arena_e = 8000, 8 * 8000
    srv = psi.Server(max_vertices=arena_v, max_edges=arena_e, max_games=6)
    t_first = [srv.submit(g) for g in first]
    srv.step()
    t_big = srv.submit(big)
    t_late = srv.submit(late)
    srv.step()
    states = [srv.status(t)[0] for t in t_first]
    assert srv.status(t_late)[0] != psi.Server.QUEUED
    if all(x == psi.Server.RESIDENT for x in states):
        assert srv.status(t_big)[0] == psi.Server.QUEUED
    resident, queued, used_v, used_e = srv.info()
    assert used_v <= arena_v and used_e <= arena_e
    srv.drain()
    for t, g in zip(t_first + [t_big, t_late], first + [big, late]):
        s = psi.GPUList(g)
        it_br = s.solve()
        expected = (it_br, s.get_strategy(), s.get_infinite())
        s.close()
        check_against(srv, t, expected, f"n={g.n}")
    assert srv.info() == (0, 0, 0, 0)
    # the whole arena is one free range again: a game filling it is admitted
    full = make("c4", arena_v - 1, 77)
    assert full.m <= arena_e
    t = srv.submit(full)
    srv.step()
    assert srv.status(t)[0] != psi.Server.QUEUED


@pytest.mark.gpu
def test_serve_rejects_games_that_never_fit():
    srv = psi.Server(max_vertices=1000, max_edges=10000, max_games=2)
    with pytest.raises(psi.PsiError) as e:
        srv.submit(make("c4", 1000, 3))   # needs 1001 vertex slots
    assert e.value.code == 4
    g = make("c4", 999, 3)
    t = srv.submit(g)
    srv.drain()
    assert srv.status(t)[0] == psi.Server.FINISHED
    check_against(srv, t, oracle_result(g), "n=999")


@pytest.mark.gpu
def test_serve_stress_random_arrivals_and_sizes():
    """Many admissions and retirements in a small arena (the vertex count of
    the arena grows and shrinks, ranges are reused at once, tiny games sit
    next to large ones); every result equals the game's solo GPU solve."""
    rng = np.random.default_rng(2024)
    games = []
    for i in range(90):
        r = rng.random()
        if r < 0.15:
            games.append(psi.Game.from_csr([int(rng.integers(2))], [int(rng.integers(4))], [0, 1], [0]))
        elif r < 0.25:
            games.append(ring10())
        else:
            n = int(rng.integers(20, 6000))
            games.append(make(("c1", "c2", "c3", "c4", "smallpri")[i % 5], n, 500 + i))
    expected = []
    for g in games:
        s = psi.GPUList(g)
        it_br = s.solve()
        expected.append((it_br, s.get_strategy(), s.get_infinite()))
        s.close()
    srv = psi.Server(max_vertices=24000, max_edges=24000 * 8, max_games=10)
    pending = list(range(len(games)))
    open_tickets = {}
    steps = 0
    while pending or open_tickets:
        for _ in range(int(rng.integers(0, 4))):
            if pending:
                k = pending.pop(0)
                open_tickets[srv.submit(games[k])] = k
        srv.step()
        steps += 1
        for t in srv.finished():
            k = open_tickets.pop(int(t))
            check_against(srv, int(t), expected[k], f"game {k}")
        assert steps < 20000
    assert srv.info() == (0, 0, 0, 0)
