"""The CPU parts of bench.py's JSON lines (runs without a GPU).

`bench.py --impl reference` times the CPU restatement of the reference step on
the headline workload, and the GPU arm's cpu_baseline object comes from the
same code. Here both run on a shrunken case (a 9x9-marker plate in a
32x24x24 block) and their output is checked against the benchmark contract:
the keys, their types and the agreement of value, cpu_baseline and e2e.
"""
import json
import types


def test_reference_arm_line(monkeypatch, capsys):
    import bench
    monkeypatch.setattr(bench, "FSI_GRID", (32, 24, 24))
    monkeypatch.setattr(bench, "FSI_NODES", 9)
    a = types.SimpleNamespace(steps=1, warmup=1)
    bench.main_reference(a, 0, 1, None)
    out = [l for l in capsys.readouterr().out.splitlines() if l.strip()]
    assert len(out) == 1, out
    line = json.loads(out[0])
    for key, typ in (("impl", str), ("metric", str), ("value", float), ("unit", str), ("n_gpus", int),
                     ("steps", int), ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool),
                     ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)):
        assert isinstance(line[key], typ), (key, line.get(key))
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "MLUPS"
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"] == bench.WORKLOAD and line["config"]["grid"] == [32, 24, 24]
    assert line["config"]["markers"] == 81
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["unit"] == "MLUPS" and cb["kind"] in ("port", "reference")
    assert isinstance(cb["cores"], int) and cb["cores"] >= 1 and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == "MLUPS"
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_silent_on_other_ranks(capsys):
    import bench
    a = types.SimpleNamespace(steps=1, warmup=1)
    bench.main_reference(a, 1, 2, None)
    assert capsys.readouterr().out.strip() == ""


def test_cpu_baseline_leg(monkeypatch):
    import bench
    monkeypatch.setattr(bench, "FSI_GRID", (32, 24, 24))
    monkeypatch.setattr(bench, "FSI_NODES", 9)
    cb = bench.cpu_baseline_leg(2, seconds=0.05)
    assert set(cb) == {"value", "unit", "cores", "kind", "sample"}
    assert cb["value"] > 0 and cb["unit"] == "MLUPS" and cb["cores"] == 2 and cb["kind"] == "port"
    assert "build" in cb["sample"] and "steps" in cb["sample"]
