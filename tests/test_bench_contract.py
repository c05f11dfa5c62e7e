"""bench.py's output contract on CPU: the reference arm's JSON line (rank 0,
one process) and the per-launch byte and random-access formulas the roofline
figures are computed from."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


# runs the reference arm in-process, then reports whether the product package
# or its CUDA library was loaded on the way
_PROBE = """
import json, runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
try:
    runpy.run_path(sys.argv[0], run_name="__main__")
except SystemExit:
    pass
maps = open("/proc/self/maps").read()
print(json.dumps({"psi_imported": "psi" in sys.modules, "libpsi_mapped": "libpsi_gb300" in maps}))
"""


def _reference_arm(*extra):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "-c", _PROBE, "--impl", "reference", *extra], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [x for x in r.stdout.splitlines() if x.strip()]
    assert len(lines) == 2, r.stdout
    return json.loads(lines[0]), json.loads(lines[1])


def test_reference_arm_prints_one_complete_line():
    d, probe = _reference_arm("--n", "65536", "--steps", "2", "--warmup", "3")
    assert probe == {"psi_imported": False, "libpsi_mapped": False}, "the reference arm must not load the product"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]
    # the same workload description as this arm's own line
    assert d["config"] == bench.workload_config(65536, d["config"]["m"], 1, "single")


def test_reference_arm_c1_is_the_dense_restatement_on_one_thread():
    d, probe = _reference_arm("--workload", "c1", "--steps", "1", "--warmup", "3")
    assert not probe["psi_imported"] and not probe["libpsi_mapped"]
    assert d["config"]["n"] == 10000 and d["cpu_baseline"]["cores"] == 1 and d["value"] > 0


def test_phase_byte_formulas():
    n, nsub = 1 << 24, ((2 * (1 << 24) + 1) + 63) // 64 + 1
    L = 2 * n + 2
    assert bench.phase_bytes("sublist", n, 0, nsub, None, 1, 0, 0, 0, 0) == 4 * L + 8 * n + 8 * nsub
    assert bench.phase_bytes("tour", n, 0, nsub, None, 1, 0, 0, 0, 0) == 14 * n
    t = {"tour_parents": 100, "tour_entries": 350, "tour_children": 120}
    # two full evaluations: per-vertex scans plus half of the relink work each
    assert bench.phase_bytes("tour", n, 0, nsub, t, 2, 0, 0, 0, 0) == 14 * n + (1700 + 2800 + 480) / 2
    assert bench.phase_bytes("broadcast", n, 0, nsub, None, 1, 0, 0, 0, 0) == 69 * n
    # the ruling set at this size: 48 B per item, Wyllie over the rulers
    nr = (nsub - 1) // 8 + 2
    assert bench.phase_bytes("reduced", n, 0, nsub, None, 1, 0, 0, 0, 0) == 48 * nsub + 24 * nr * (
        (nr - 1).bit_length() + 2)
    # short reduced lists: Wyllie over all items
    small = 1000
    assert bench.phase_bytes("reduced", n, 0, small, None, 1, 0, 0, 0, 0) == 24 * small * (
        (small - 1).bit_length() + 1)
    c = {"switches": 2, "sw_edges": 1000, "sw_loads": 10, "sw_changed": 7}
    # one Odd step of 300 vertices and one Even step of 200: (16*500 + 8*1000 + 8*10 + 6*7) / 2
    assert bench.phase_bytes("switch", n, 0, nsub, c, 2, 200, 300, 1, 1) == (16 * 500 + 8000 + 80 + 42) / 2


def test_random_access_formulas():
    n = 1000
    assert bench.random_accesses("sublist", n, None, 0, 0, 0, 0) == (2 * n + 2) + n
    c = {"switches": 2, "sw_edges": 1000, "sw_loads": 10, "sw_changed": 7}
    assert bench.random_accesses("switch", n, c, 200, 300, 1, 1) == (1000 + 500 + 10 + 14) / 2
    assert bench.random_accesses("tour", n, c, 200, 300, 1, 1) is None
