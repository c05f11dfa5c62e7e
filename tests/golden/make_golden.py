"""Generates the golden fixtures of the parity tests from the REFERENCE itself.

Each case is a seeded game from the product generator (or the 10-vertex ring
game), handed to the reference's own CPUParity solver -- compiled from the
reference sources by oracle/build_ref.sh and fed the game as .gm text through
the reference parser -- and solved with the reference's solve_si loop.  The
fixture records the game's digest, iter/br counts, the final strategy, the
winning set and a digest of every step (state after each evaluation and each
switch, switch counts included; tests/lockstep.py defines the digests).

Run in a container that has the reference tree:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "parallel-si_gb300"), os.path.dirname(HERE)]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from games import make  # noqa: E402
from lockstep import traced_solve  # noqa: E402

CASES = [
    # (family, n, seed, reset)
    ("ring10", 10, 0, False),
    ("ring10", 10, 0, True),
    ("c1", 10000, 1, False),
    ("c1", 10000, 2, False),
    ("c2", 2000, 1, False),
    ("c2", 2000, 2, False),
    ("c2", 5000, 3, False),
    ("c2", 3000, 4, True),
    ("c3", 2000, 1, False),
    ("c3", 6000, 2, False),
    ("c4", 100, 5, False),
    ("c4", 400, 6, False),
    ("c4", 1500, 7, False),
    ("smallpri", 3000, 1, False),
    ("smallpri", 3000, 2, True),
]


def game_digest(csr):
    d = hashlib.sha256()
    for a in csr:
        d.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return d.hexdigest()[:16]


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference library not built (needs the reference tree)")
    cases = []
    for fam, n, seed, reset in CASES:
        g = make(fam, n, seed)
        csr = g.csr()
        ref = oracle.RefSolver(oracle.to_gm(*csr))
        assert all(np.array_equal(a, b) for a, b in zip(ref.game_arrays(), csr)), "reference parser disagrees"
        iters, brs, trace = traced_solve(ref, reset=reset)
        strat = ref.get_strategy()
        w0 = ref.get_winning(0)
        case = {
            "family": fam, "n": n, "seed": seed, "reset": reset,
            "game_digest": game_digest(csr), "max_pri": int(g.max_pri), "m": int(g.m),
            "iters": iters, "brs": brs, "trace": trace,
            "strategy_digest": hashlib.sha256(strat.tobytes()).hexdigest()[:16],
            "w0_size": int(w0.size),
            "w0_digest": hashlib.sha256(w0.tobytes()).hexdigest()[:16],
        }
        if n <= 100:
            case["csr"] = [a.tolist() for a in csr]
            case["strategy"] = strat.tolist()
            case["w0"] = w0.tolist()
        cases.append(case)
        print(f"{fam} n={n} seed={seed} reset={reset}: iters={iters} brs={brs} |W0|={w0.size}")
        ref.close()
    with open(os.path.join(HERE, "reference_solves.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "source": "reference CPUParity (cpu_parity.cpp)",
                   "cases": cases}, f, indent=1)


if __name__ == "__main__":
    main()
