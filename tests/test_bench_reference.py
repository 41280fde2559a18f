"""bench.py's reference arm on the host cores: the JSON line's contract keys
for a one-view workload, the batch rate's weighting over volumes, and the
`unavailable` line of the adjoint workload, which the reference lacks."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_bench(*args):
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    return json.loads(lines[0])


def test_reference_arm_line_c1():
    line = run_bench("--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "1")
    assert line["impl"] == "reference"
    assert line["metric"] == "Msamples/s" and line["unit"] == "Msamples/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 1
    assert line["config"]["workload"].startswith("c1-")
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert "crop" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_adjoint_unavailable():
    line = run_bench("--impl", "reference", "--workload", "c4")
    assert line["impl"] == "reference" and "unavailable" in line


class Cam:
    def __init__(self, w, h):
        self.film_size = (w, h)


def test_batched_reference_rate_weighting(monkeypatch):
    """each volume's rate is the harmonic mean of views spread over its orbit
    (here both of its views), and the batch's rate is its samples over the
    time each volume's samples take at that rate"""
    bench = load_bench()
    rates = {8: 100.0, 4: 300.0, 16: 400.0, 32: 200.0}
    seen = []

    def fake_rate(scene, seconds_target=12.0, nthreads=None, steps=1):
        k = scene.tracer.camera.film_size[0]          # the view's film width names the volume here
        seen.append((k, seconds_target, steps))
        return rates[k], "port", 3, "16x16 centre crop x 1 spp per step"

    class Tracer:
        camera = None
        settings = type("St", (), {})()

    class Sc:
        def __init__(self):
            self.tracer = Tracer()

    monkeypatch.setattr(bench, "cpu_reference_rate", fake_rate)
    monkeypatch.setattr(bench, "reference_path", lambda sc: Sc())
    views = [(0, Cam(8, 8), 10), (1, Cam(16, 16), 2), (0, Cam(4, 4), 5), (1, Cam(32, 32), 1)]
    rate, kind, cores, sample = bench.batched_reference_rate([None, None], views, seconds_target=6.0, steps=2)
    n0, n1 = 8 * 8 * 10 + 4 * 4 * 5, 16 * 16 * 2 + 32 * 32 * 1
    t0 = n0 * (1 / 100.0 + 1 / 300.0) / 2
    t1 = n1 * (1 / 400.0 + 1 / 200.0) / 2
    assert rate == pytest.approx((n0 + n1) / (t0 + t1))
    assert (kind, cores) == ("port", 3)
    assert [s[0] for s in seen] == [8, 4, 16, 32]         # every view of each volume (two each), in volume order
    assert all(s[1] == pytest.approx(1.5) and s[2] == 2 for s in seen)
    assert "100 .. 400" not in sample and "0.0001 .. 0.0004" in sample
    assert "volume 0: 2 views, 16x16" in sample and "volume 1: 2 views, 16x16" in sample
