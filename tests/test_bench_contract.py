"""The benchmark's JSON-line contract, on the CPU: the reference arm (the
CPU restatement of the check rule, timed on the host cores) prints one line
with the keys and units the gb300 arm prints, and its e2e block moves no
bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line(oracle_lib):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--workload", "small"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "checks/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_roofline_traffic_comes_from_the_committed_ncu_summary():
    """roofline.traffic (DRAM bytes per launch of the check kernel) is read
    from the committed ncu summary of that kernel on the benchmark's workload."""
    sys.path.insert(0, ROOT)
    import bench
    t = bench.load_traffic()
    assert isinstance(t, int) and 1e9 < t < 1e10


def test_cell_records_unpack_to_clause_word_mask():
    """The 8-byte {clause * n_words + word, mask} records of the e2e leg
    unpack to the report fields."""
    import numpy as np
    import gpusharesat_gb300 as g
    cells = np.zeros(3, dtype=g.CELL_REPORT_DTYPE)
    cells["cell"] = [0 * 32 + 5, 7 * 32 + 31, 123456 * 32 + 0]
    cells["mask"] = [1, 0xFFFFFFFF, 0x80000000]
    rep = g.cells_to_reports(cells, 32)
    assert rep["clause"].tolist() == [0, 7, 123456]
    assert rep["word"].tolist() == [5, 31, 0]
    assert rep["mask"].tolist() == [1, 0xFFFFFFFF, 0x80000000]
