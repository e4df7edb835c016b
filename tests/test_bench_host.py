"""Host-side parts of bench.py on CPU: the strided pair sample keeps the
workload's mix of pair types, and the reference arm (the CPU restatement timed
on the host cores) prints one JSON line with the contract's keys and an e2e
entry equal to its value."""
import io
import json
import types
from contextlib import redirect_stdout

import numpy as np


def test_pair_sample_keeps_type_mix():
    import bench
    import workloads
    w = workloads.contact_pairs(50_000, seed=1)
    t, idx = bench._pair_sample(w, 5_000)
    assert t.shape == (5_000,) and idx.shape == (5_000, 4)
    full = np.bincount(w["type"], minlength=4) / w["type"].size
    part = np.bincount(t, minlength=4) / t.size
    assert np.abs(full - part).max() <= 0.01
    t2, _ = bench._pair_sample(w, 10 ** 6)  # larger than the list: the whole list
    assert np.array_equal(t2, w["type"])


def test_reference_arm_line(monkeypatch):
    import bench
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    args = types.SimpleNamespace(pairs=20_000, steps=2, warmup=1, gpus=1)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
