"""The benchmark line recorded from a GB300 run (profiles/bench_config3.json,
the line bench.py printed) carries every key of the bench contract, with sane
values, and the keys the bench writes today are the ones recorded.  CPU only:
it reads the recorded file."""

import json
from pathlib import Path

from conftest import REPO

TOP = {"metric": str, "value": float, "unit": str, "n_gpus": int, "steps": int, "warmup": int,
       "ms_per_step": float, "higher_is_better": bool, "scaling": str, "dtype": str, "data": str,
       "config": dict, "gpu_launches": int, "e2e": dict, "roofline": dict, "cpu_baseline": dict, "clocks": dict}


def recorded_line() -> dict:
    return json.loads(Path(REPO, "profiles", "bench_config3.json").read_text())


def test_the_recorded_line_keeps_the_contract():
    line = recorded_line()
    for key, typ in TOP.items():
        assert key in line, key
        assert isinstance(line[key], typ) or (typ is float and isinstance(line[key], int)), key
    assert "vs_baseline" in line  # null: no published number for this metric
    assert line["unit"] == "body-steps/s" and line["higher_is_better"] is True and line["scaling"] == "weak"
    assert line["n_gpus"] == 1 and line["warmup"] >= 3 and line["steps"] >= 1
    assert "workload" in line["config"] and "l2" in line["config"]
    assert abs(line["value"] - line["config"]["bodies"] * 1e3 / line["ms_per_step"]) < 1e-6 * line["value"]
    e2e = line["e2e"]
    assert {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"} <= set(e2e)
    assert e2e["unit"] == line["unit"] and 0 < e2e["value"] <= line["value"]
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    roof = line["roofline"]
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= set(roof)
    assert roof["bound"] in ("hbm", "tensor") and roof["unit"] in ("GB/s", "TFLOP/s")
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-9
    cpu = line["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= set(cpu)
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1
    clocks = line["clocks"]
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(clocks)
    bad = {"hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"}
    assert not bad & set(clocks["reasons"])
    assert line["gpu_launches"] > 0


def test_the_bench_still_writes_every_recorded_key():
    src = Path(REPO, "bench.py").read_text()
    line = recorded_line()
    keys = set(line) | set(line["e2e"]) | set(line["roofline"]) | set(line["cpu_baseline"]) | set(line["clocks"])
    missing = sorted(k for k in keys if f'"{k}"' not in src)
    assert not missing, f"recorded but no longer written: {missing}"
