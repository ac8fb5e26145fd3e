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


def test_algorithmic_bytes_per_update():
    # one read and one write of the 19 populations, plus each model's fields
    import bench
    for s in (8, 4, 2):
        assert bench.model_bytes(1, s, "f16") == bench.model_bytes(3, s, "f16") == 38 * s
    assert bench.model_bytes(11, 2, "f16") == 80       # + tau_all written (FP32)
    assert bench.model_bytes(15, 2, "f16") == 146      # + velocity pass, gradient pass, tau_all read
    assert bench.model_bytes(14, 2, "f16") == 170      # + rotation entries, tau_all read and written
    assert bench.model_bytes(11, 8, "f64") == 312
    assert bench.model_bytes(15, 8, "f64") == 304 + 152 + 32 + 24 + 8


def test_headline_launches_per_step():
    # IB stage, bulk step, IB-window fix-up, and one launch per axis whose two
    # faces need a face kernel (x: 101/104, y: 101/101; the z faces of code
    # 101 are written by the bulk kernel)
    import bench
    assert bench.BND == (101, 104, 101, 101, 101, 101)
    assert bench.n_face_kernels() == 2
