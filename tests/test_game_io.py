"""The .gm reader/writer and the game generators.

The reader follows the reference parser (Game::parse_pgsolver, game.cpp:51-107):
where the reference was compiled here, both parse the same texts and must give
the same arrays and the same error messages.
"""
import gzip
import hashlib
import os

import numpy as np
import pytest

import oracle
import psi
from psi._lib import PSI_ERR_INVALID, PSI_ERR_IO, PSI_ERR_PARSE, PsiError
from games import make


def digest(arrays):
    d = hashlib.sha256()
    for a in arrays:
        d.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return d.hexdigest()[:16]


def test_write_then_read_round_trip(tmp_path):
    for g in (make("c2", 700, 1), make("c3", 500, 2), make("ring10", 10, 0)):
        p = str(tmp_path / "g.gm")
        g.write_pgsolver(p)
        h = psi.Game.parse_pgsolver(p)
        for a, b in zip(g.csr(), h.csr()):
            assert np.array_equal(a, b)
        assert (h.n, h.m, h.max_pri) == (g.n, g.m, g.max_pri)


def test_gzip_input(tmp_path):
    g = make("c2", 300, 4)
    p = str(tmp_path / "g.gm")
    g.write_pgsolver(p)
    gz = p + ".gz"
    with open(p, "rb") as f, gzip.open(gz, "wb") as out:
        out.write(f.read())
    try:
        h = psi.Game.parse_pgsolver(gz)
    except PsiError as e:
        assert e.code == PSI_ERR_IO and "zlib" in e.message
        pytest.skip("library built without zlib")
    for a, b in zip(g.csr(), h.csr()):
        assert np.array_equal(a, b)


def test_bz2_is_reported_unsupported(tmp_path):
    with pytest.raises(PsiError) as e:
        psi.Game.parse_pgsolver(str(tmp_path / "g.gm.bz2"))
    assert e.value.code == PSI_ERR_IO


def test_labels_blank_lines_and_header():
    text = 'parity 2;\n0 4 0 1,2 "zero";\n\n1 3 1 2 "one";\n   \n2 0 0 0;\n'
    g = psi.Game.parse_text(text)
    assert g.n == 3 and g.max_pri == 4
    assert g.get_edges(0) == [1, 2] and g.get_edges(1) == [2] and g.get_edges(2) == [0]
    assert [g.get_player(v) for v in range(3)] == [0, 1, 0]


def test_empty_input_is_an_empty_game():
    assert psi.Game.parse_text("").n == 0
    assert psi.Game.parse_text("parity 0;\n").n == 0


BAD = [
    ("parity 1;\n0\n", "missing priority"),
    ("parity 1;\n0 1\n", "missing player"),
    ("parity 1;\n0 1 2 0;\n", "invalid player"),
    ("parity 1;\n1 1 0 0;\n", "vertices must be listed in order starting at 0!"),
    ("parity 1;\n0 1 0\n", "missing successor"),
    ("parity 1;\n0 1 0 0\n", "missing ; to end line"),
    ("parity 1;\n-1 1 0 0;\n", "invalid id"),
]


@pytest.mark.parametrize("text,msg", BAD)
def test_parse_errors_carry_the_reference_message(text, msg):
    with pytest.raises(PsiError) as e:
        psi.Game.parse_text(text)
    assert e.value.code == PSI_ERR_PARSE and msg in e.value.message
    if oracle.ref_available():
        with pytest.raises(ValueError) as r:
            oracle.RefSolver(text)
        assert msg in str(r.value)


@pytest.mark.parametrize("text", ["parity 1;\n0 -2 0 0;\n", "parity 1;\n0 1 0 5;\n"])
def test_inputs_the_reference_would_index_out_of_bounds_are_rejected(text):
    with pytest.raises(PsiError) as e:
        psi.Game.parse_text(text)
    assert e.value.code == PSI_ERR_PARSE


@pytest.mark.parametrize("fam,n,seed", [("c1", 800, 3), ("c2", 1000, 5), ("c3", 900, 6), ("smallpri", 600, 7)])
def test_reader_matches_the_reference_parser(fam, n, seed):
    if not oracle.ref_available():
        pytest.skip("reference not compiled here")
    g = make(fam, n, seed)
    text = oracle.to_gm(*g.csr())
    ref = oracle.RefSolver(text)
    for a, b in zip(ref.game_arrays(), psi.Game.parse_text(text).csr()):
        assert np.array_equal(a, b)


def test_from_csr_validation():
    ow = np.array([0, 1], np.int32)
    pr = np.array([1, 2], np.int32)
    with pytest.raises(PsiError) as e:
        psi.Game.from_csr(ow, pr, np.array([0, 1, 1], np.int32), np.array([1], np.int32))
    assert e.value.code == PSI_ERR_INVALID          # vertex 1 has no successor
    with pytest.raises(PsiError):
        psi.Game.from_csr(ow, pr, np.array([0, 1, 2], np.int32), np.array([1, 2], np.int32))


GEN_CASES = [
    ("random", 1000, 2, 5, 1000, 1),
    ("random", 2000, 2, 10, 2000, 7),
    ("longpath", 1500, 1024, 3),
]


def _gen(key):
    if key[0] == "random":
        return psi.Game.random(*key[1:5], seed=key[5])
    return psi.Game.longpath(key[1], key[2], seed=key[3])


def test_generators_are_deterministic_and_well_formed():
    for key in GEN_CASES:
        a, b = _gen(key), _gen(key)
        assert digest(a.csr()) == digest(b.csr())
        ow, pr, off, tg = a.csr()
        assert set(np.unique(ow)) <= {0, 1}
        assert (np.diff(off) >= 1).all() and tg.min() >= 0 and tg.max() < a.n
        if key[0] == "random":
            _, n, lo, hi, phi, _ = key
            deg = np.diff(off)
            assert deg.min() >= lo and deg.max() <= hi and pr.max() < phi
            for v in range(0, n, 97):                 # distinct, non-self successors
                s = tg[off[v]:off[v + 1]]
                assert len(set(s.tolist())) == len(s) and v not in s
        else:
            assert (ow == np.arange(a.n) % 2).all()
            assert tg[off[0]] == 1 and tg[off[a.n - 1]] < a.n - 1


def test_generator_output_is_pinned():
    """Golden digests of the generator (the parity fixtures depend on them)."""
    assert digest(_gen(("random", 1000, 2, 5, 1000, 1)).csr()) == digest(make("c2", 1000, 1).csr())
    golden = {c["family"] + str(c["n"]) + "-" + str(c["seed"]): c["game_digest"]
              for c in __import__("json").load(open(os.path.join(os.path.dirname(__file__), "golden",
                                                                 "reference_solves.json")))["cases"]}
    assert digest(make("c2", 2000, 1).csr()) == golden["c22000-1"]
    assert digest(make("c3", 2000, 1).csr()) == golden["c32000-1"]
