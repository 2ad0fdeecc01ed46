"""Host-side pieces of bench.py (no GPU): the algorithmic byte counts behind
the HBM rooflines, the rasteriser's issue roofline from the committed ncu
instruction count, and the reference arm's JSON line, which must come from
the oracle without loading the product library."""
import importlib.util
import io
import json
import types
from contextlib import redirect_stdout
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_depth_sort_bytes_follow_the_pass_count(bench):
    N = 760_000
    # one histogram read, then per pass a read, and a write of the keys (the
    # last pass writes 4-byte order words)
    assert bench.pass_bytes("depth_sort", N, 0, 0, 0, 6, depth_passes=2) == N * (8 + 2 * 8 + 8 + 4)
    assert bench.pass_bytes("depth_sort", N, 0, 0, 0, 6, depth_passes=4) == N * (8 + 4 * 8 + 3 * 8 + 4)
    assert bench.pass_bytes("raster", N, 0, 0, 0, 6) is None  # not an HBM-bound pass
    Q = 2_297_583
    assert bench.pass_bytes("chunk_masks", N, 0, Q, 0, 6) == Q * 8 + (Q + 31) // 32 * 8


def test_raster_issue_roofline_uses_the_committed_count(bench):
    d = json.loads((ROOT / "profiles" / "raster_issue.json").read_text())
    inst = d["inst_executed_per_launch"]
    r = bench.raster_issue_roofline(0.25, 2000.0, 152)
    assert r["bound"] == "issue" and r["inst_per_launch"] == inst
    assert r["peak"] == pytest.approx(152 * 4 * 2.0, rel=1e-6)  # G warp-instructions/s at 2 GHz
    assert r["achieved"] == pytest.approx(inst / 0.25e-3 / 1e9, rel=1e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-3)
    assert bench.raster_issue_roofline(None, 2000.0, 152) is None


def _libhdsr_loaded() -> bool:
    maps = Path("/proc/self/maps")
    return maps.exists() and "libhdsr.so" in maps.read_text()


def test_reference_arm_line_comes_from_the_oracle(bench):
    args = types.SimpleNamespace(workload="plain50k", steps=2, warmup=3)
    loaded_before = _libhdsr_loaded()
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args, 0, 1)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "frames/s" and line["value"] > 0
    assert line["steps_run"] >= 1 and line["config"]["workload"].startswith("plain50k")
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "frames/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the arm never loads the product library (checked when no earlier test
    # of this process has)
    if not loaded_before:
        assert not _libhdsr_loaded()
