"""Generates the golden fixtures of the Bellman-Ford comparison from the
REFERENCE itself.

Each case is a seeded game of the evencyc family (tests/games.py: every cycle
has an even top priority, the precondition of the reference's Bellman-Ford
solver), handed to the reference's own CPU_BellmanFord<ArrayVal> -- compiled
from the reference sources by oracle/build_ref.sh and fed the game as .gm
text through the reference parser -- and solved with the reference's
solve_bf loop (main.cpp:58-76).  The fixture records the game's digest, the
iteration count, the Bellman-Ford rounds so far after every best response,
and two digests of the state after every best response (tests/lockstep.py,
br_digest): one over Even's strategy, the infinite and solved flags and the
finite valuation rows, which any exact best response must reproduce, and one
over the whole strategy, Odd's choices included.

Run in a container that has the reference tree:
    python tests/golden/make_golden_bf.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "parallel-si_gb300"), os.path.dirname(HERE)]

import oracle  # noqa: E402
from games import evencyc_csr  # noqa: E402
from lockstep import bf_best_responses, br_digest  # noqa: E402
from make_golden import game_digest  # noqa: E402

CASES = [(10, 1), (300, 2), (1000, 3), (2000, 5), (3000, 6), (6000, 4)]   # (n, seed)


def main():
    oracle.build()
    if not oracle.refbf_available():
        raise SystemExit("reference Bellman-Ford library not built (needs the reference tree)")
    cases = []
    for n, seed in CASES:
        csr = evencyc_csr(n, seed)
        ref = oracle.RefBellmanFord(oracle.to_gm(*csr))
        rounds, even, full = [], [], []
        for r, state in bf_best_responses(ref):
            rounds.append(r)
            even.append(br_digest(csr[0], state))
            full.append(br_digest(csr[0], state, even_only=False))
        cases.append({"family": "evencyc", "n": n, "seed": seed, "game_digest": game_digest(csr),
                      "max_pri": int(csr[1].max()), "iters": len(rounds), "rounds": rounds,
                      "br_digest": even, "br_digest_full": full})
        print(f"evencyc n={n} seed={seed}: iters={len(rounds)} rounds={rounds}")
        ref.close()
    with open(os.path.join(HERE, "reference_bf_solves.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden_bf.py",
                   "source": "reference CPU_BellmanFord<ArrayVal> (cpu_bf.cpp, cpu_bv.cpp)", "cases": cases},
                  f, indent=1)


if __name__ == "__main__":
    main()
