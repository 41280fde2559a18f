"""The arithmetic behind bench.py's equal-RMSE figures, on synthetic curves:
the crossing of a curve with the target and the speed-up at equal RMSE from
samples-to-target and measured rates (one view and batched)."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_summaries_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def curve(var, spps, bias=0.0):
    """rmse of an estimator with per-sample variance `var` and a bias"""
    return [float(np.sqrt(var / n + bias * bias)) for n in spps]


def film_conv(fast_var, plain_var, plain_bias=0.0):
    sched = [8, 16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048]
    import convergence as CV
    out = {"reference": {"spp": 8192, "noise": 1e-3, "film": [256, 256]}}
    for label, var, bias in (("fast", fast_var, 0.0), ("plain", plain_var, plain_bias)):
        spps, errs = [], []
        for n, e in zip(sched, curve(var, sched, bias)):
            spps.append(n)
            errs.append(e)
            if e <= 1e-2:
                break
        out[label] = {"spp": spps, "rmse": errs, "spp_to_target": CV.spp_to_rmse(spps, errs, 1e-2)}
    return out


def test_film_summary_equal_rmse_speedup():
    """an unbiased curve var/n crosses 1e-2 at var/1e-4 samples; the speed-up
    is the ratio of the two paths' times to their crossings"""
    bench = load_bench()
    fc = film_conv(fast_var=0.04, plain_var=0.07)
    assert fc["fast"]["spp_to_target"] == pytest.approx(400.0, rel=1e-6)
    assert fc["plain"]["spp_to_target"] == pytest.approx(700.0, rel=1e-6)
    s = bench.film_rmse_summary(fc, fast_value=1500.0, plain_value=50.0, npix=1024 * 1024)
    assert s["fast"]["seconds"] == pytest.approx(400.0 * 1024 * 1024 / 1.5e9)
    assert s["speedup_equal_rmse"] == pytest.approx((700.0 / 50.0) / (400.0 / 1500.0))


def test_biased_curve_crosses_later():
    """a bias in the plain path (the fixed-step march) delays its crossing
    beyond var/1e-4: the summary uses the measured crossing"""
    fc = film_conv(fast_var=0.04, plain_var=0.07, plain_bias=0.006)
    assert fc["plain"]["spp_to_target"] > 1.3 * 700.0


def test_batched_summary_is_throughput_times_geomean_of_sample_ratios():
    bench = load_bench()
    conv = {"a": film_conv(0.01, 0.03), "b": film_conv(0.02, 0.02 * 1.5)}
    s = bench.batched_rmse_summary(conv, value=2000.0, plain_value=100.0)
    g = float(np.exp(np.mean(np.log([3.0, 1.5]))))
    assert s["throughput_ratio"] == pytest.approx(20.0)
    assert s["spp_ratio_geomean"] == pytest.approx(g, rel=1e-6)
    assert s["speedup_equal_rmse"] == pytest.approx(20.0 * g, rel=1e-6)


def test_batched_summary_needs_every_view():
    """a view whose plain path never reached the target leaves the speed-up
    out rather than averaging over the others"""
    bench = load_bench()
    conv = {"a": film_conv(0.01, 0.03), "b": film_conv(0.02, 50.0)}
    assert conv["b"]["plain"]["spp_to_target"] is None
    s = bench.batched_rmse_summary(conv, value=2000.0, plain_value=100.0)
    assert "speedup_equal_rmse" not in s and s["throughput_ratio"] == pytest.approx(20.0)
