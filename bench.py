"""Throughput benchmark of the GB300 transport path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload c2|c1|c3|c4|c5]

A step is one full render of the workload: every pixel of the film at the
configured samples per pixel (c2: 1024x1024 x 256 spp over the 512^3 CT-like
shell volume; c1: 256x256 x 64 spp over the 128^3 blob volume; c3: 64 views
over three blob volumes in one batch; c4: the differentiable medium's
forward and adjoint; c5: 16 views of 2048^2 x 64 spp over a 1024x1024x512
volume in one batch, plus the adjoint on a 256^3 block of it).  Inputs are
seeded synthetic volumes (the reference ships no dataset).

value : samples/s of the transport kernel with the scene resident in HBM,
        CUDA events on the launching stream, max over ranks.
e2e   : the same metric through the C ABI a user calls, with host buffers:
        per step the volume and tracer descriptor are copied host->device
        (BindVolume / BindTracer), the render runs (RenderSpp) and the RGBA8
        estimate is read back (GetEstimate).
--impl reference : the reference's transport code on the host cores (the
        reference build in oracle/_ref when it exists for this machine, else
        the C restatement of oracle/), all threads, each step a bounded
        sample (a film crop at 1 spp) of the same workload.
Multi-GPU (torchrun): c1/c2/c3/c5 render one set of images over all ranks,
each rank its own sample ranges of every view, with the per-pixel sums
all-reduced each step (the path's one exchange); c4 runs independent
replicas.  value = all ranks' samples / max time (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
R = importlib.import_module("exposure-render_gb300.replicas")

WORKLOADS = {
    "c2": dict(name="c2-ct-shells-512^3-1024^2-256spp", res=512, film=(1024, 1024), spp=256),
    "c1": dict(name="c1-blobs-128^3-256^2-64spp", res=128, film=(256, 256), spp=64),
}
# algorithmic bytes: 16 per volume lookup (8 corners x uint16)
BYTES_PER_LOOKUP = 16.0


def make_scene(wl):
    S = importlib.import_module("exposure-render_gb300.scenes")
    if wl == "c2":
        return S.scene_c2(res=512, film=WORKLOADS[wl]["film"], spp=WORKLOADS[wl]["spp"])
    # c1 is specified with the isotropic phase function at every volume event
    return S.scene_c1(res=128, film=WORKLOADS[wl]["film"], spp=WORKLOADS[wl]["spp"], phase=True)


def describe_shading(scene):
    s = scene.tracer.settings
    shading = {0: "brdf", 1: "phase", 2: "hybrid", 3: "modulation", 4: "threshold"}.get(s.shading_type, "?")
    if not s.apply_shading_type:
        shading = "brdf (reference live path)"
    return {"shading": shading, "mis": "full" if s.mis else "light-sampling",
            "free_flight": "delta+ratio tracking, %d^3 majorant bricks" % (s.majorant_brick or 8) if s.free_flight else "fixed-step march",
            "bilateral": bool(s.bilateral)}


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    QUERY = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.after = False

    def __enter__(self):
        q = self.QUERY
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if not self.lines:
                # the timed region ended before nvidia-smi's first sample (a
                # region of a few ms): one query right after it
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=20)
                    self.lines = [x.strip() for x in out.stdout.splitlines() if x.strip()]
                    self.after = bool(self.lines)
                except (OSError, subprocess.TimeoutExpired):
                    pass

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[3:7]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}
        if self.after:
            out["when"] = "right after the timed region, which ended before nvidia-smi's first sample"
        return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p)), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


def profile_traffic(wl):
    """DRAM bytes per sample of the transport kernel from a committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"traffic_{wl}.json")
    if os.path.exists(p):
        return json.load(open(p))
    return None


def cpu_reference_rate(scene, seconds_target=12.0, nthreads=None, steps=1):
    """Samples/s of the reference transport on the host cores (all threads)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as OL
    nthreads = nthreads or os.cpu_count() or 1
    kind = "port"
    lib = OL.load_oracle()
    ref = OL.load_ref()
    if ref is not None:
        lib, kind = ref, "reference"
    h = OL.SceneHandle(lib, scene)
    W, H = scene.width, scene.height
    # calibrate a crop that takes about seconds_target / steps
    side = 16
    t0 = time.perf_counter()
    h.render_sum(1, rect=(W // 2 - side // 2, H // 2 - side // 2, side, side), nthreads=nthreads)
    dt = max(time.perf_counter() - t0, 1e-3)
    rate = side * side / dt
    want = rate * seconds_target / max(steps, 1)
    side = int(max(16, min(min(W, H), np.sqrt(want))))
    x0, y0 = W // 2 - side // 2, H // 2 - side // 2
    rates = []
    for s in range(steps):
        t0 = time.perf_counter()
        h.render_sum(1, first=s, rect=(x0, y0, side, side), nthreads=nthreads)
        rates.append(side * side / (time.perf_counter() - t0))
    h.close()
    return float(np.median(rates)), kind, nthreads, f"{side}x{side} centre crop x 1 spp per step"


def read_profile(lib, C):
    """(ms, launches) per wavefront stage since the previous read"""
    ms = np.zeros(4, dtype=np.float64)
    n = np.zeros(4, dtype=np.int64)
    C.check(lib.er_profile_read(ms.ctypes.data, n.ctypes.data))
    return ms, n


def oracle_work(scene, settings, nthreads, spp=2):
    """Per-sample work counters of the estimator (oracle, same settings) over
    the whole field of view at a 128^2 film."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as OL
    C = importlib.import_module("exposure-render_gb300.capi")
    t = C.er_tracer_desc.from_buffer_copy(scene.tracer)
    ctypes.memmove(ctypes.byref(t.settings), ctypes.byref(settings), ctypes.sizeof(settings))
    t.camera.film_size[0] = t.camera.film_size[1] = 128
    saved = scene.tracer
    scene.tracer = t
    orc = OL.load_oracle()
    h = OL.SceneHandle(orc, scene)
    h.render_sum(spp, nthreads=nthreads)
    h.close()
    scene.tracer = saved
    return OL.render_stats(orc)


# bytes of the queue records (er_wavefront.cu): event 5 float4, shadow job 6 float4, result 1 float4
EVENT_BYTES, JOB_BYTES, RESULT_BYTES = 80.0, 96.0, 16.0


def stage_bytes(w):
    """Algorithmic bytes per sample of each wavefront stage: 16 per volume
    lookup (8 uint16 corners), 4 per majorant-grid read, the queue records
    written and read.  The event normal is computed by the shade stage."""
    ev = w["events"]
    ff = w["free_flight_lookups"] - w["normal_lookups"]
    shade_lk = w["lookups"] - ff - w["shadow_lookups"]
    return {
        "primary": BYTES_PER_LOOKUP * ff + 4.0 * (w["majorant_reads"] - w["shadow_majorant_reads"])
        + RESULT_BYTES * (1.0 - ev) + EVENT_BYTES * ev,
        "shade": EVENT_BYTES * ev + BYTES_PER_LOOKUP * shade_lk + JOB_BYTES * ev,
        "shadow": JOB_BYTES * ev + BYTES_PER_LOOKUP * w["shadow_lookups"] + 4.0 * w["shadow_majorant_reads"] + RESULT_BYTES * ev,
        "reduce": RESULT_BYTES,
    }


def stage_roofline(work, ref_work, stage_ms, stage_launches, samples, peaks, peak_kind, wl):
    """roofline of the dominant wavefront stage: its own algorithmic bytes
    per sample (this estimator's volume lookups at 16 B, majorant reads at
    4 B, the queue records it reads and writes) times the samples of one
    launch, over that stage's average launch time from CUDA events on the
    launching stream, against the measured HBM copy bandwidth.  `traffic`
    is the stage's measured DRAM bytes per launch (ncu, profiles/), so
    traffic / algorithmic bytes says how much of the gather the caches
    absorb.  The reference estimator's bytes over the whole window (its
    fixed-step march makes far more lookups) are kept apart as
    `reference_equivalent`: a throughput figure, not a roofline."""
    names = ("primary", "shade", "shadow", "reduce")
    bps = stage_bytes(work)
    total = float(sum(stage_ms)) or 1.0
    stages = {}
    for i, n in enumerate(names):
        t = float(stage_ms[i])
        stages[n] = {"ms": t, "share": t / total, "launches": int(stage_launches[i]),
                     "bytes_per_sample": bps[n], "achieved_gbs": (bps[n] * samples / (t / 1e3) / 1e9) if t > 0 else None}
    top = max(names, key=lambda n: stages[n]["ms"])
    launches = max(int(stages[top]["launches"]), 1)
    top_ms = stages[top]["ms"] / launches
    alg = bps[top] * samples / launches
    achieved = alg / (top_ms / 1e3) / 1e9
    traffic = profile_traffic(wl)
    b_ref = BYTES_PER_LOOKUP * ref_work["lookups"] + 32.0
    ref_gbs = b_ref * samples / (total / 1e3) / 1e9
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
        "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured" else peak_kind,
        "kernel": "k_wf_" + top, "avg_launch_ms": top_ms, "algorithmic_bytes_per_launch": alg,
        "basis": "%.1f B/sample of this stage (lookups x 16 B + majorant reads x 4 B + queue records, oracle work counts)"
                 " x %d samples per launch" % (bps[top], samples // launches),
        "traffic": (traffic.get(top) if traffic else None),
        "traffic_source": (traffic.get("note") if traffic else None),
        "reference_equivalent": {"gbs": ref_gbs, "what": "the reference estimator's algorithmic bytes (%.1f lookups/sample of the "
                                 "fixed-step march x 16 B + 32 B) per wavefront-window time: throughput in the reference's "
                                 "currency, not a bandwidth" % ref_work["lookups"]},
    }
    return roofline, stages


def convergence(lib, runtime, torch, names, patches, max_spp=4096, target=1e-2):
    """RMSE against the FP64 references (tests/golden/fp64_<name>.npz) of the
    views `names` of scenes.rmse_views(), for each estimator configuration in
    `patches` (settings overrides), at 1, 2, 4, ... samples per pixel, and the
    samples per pixel at which each reaches `target`."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import convergence as CV
    S = importlib.import_module("exposure-render_gb300.scenes")
    out = {}
    for name, sc in S.rmse_views(names=names):
        ref = CV.load_reference(name)
        r = runtime.Renderer(sc, lib)
        W, H = sc.width, sc.height
        res = {}
        for label, patch in patches.items():
            for k, v in patch.items():
                setattr(r.tracer_desc.settings, k, v)
            r.rebind_tracer()
            acc = torch.zeros((H, W, 4), dtype=torch.float64, device="cuda")
            d = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
            n, spps, errs = 0, [], []
            while n < max_spp:
                chunk = max(n, 1)
                r.trace_sum_device(d.data_ptr(), chunk, 0, n, 0, None)
                acc += d.double()
                n += chunk
                err = CV.rmse((acc / n).cpu().numpy(), ref)
                spps.append(n)
                errs.append(err)
                if err < 0.5 * target:
                    break
            res[label] = {"spp": spps, "rmse": errs, "spp_to_target": CV.spp_to_rmse(spps, errs, target)}
        res["reference_noise"] = float(np.sqrt(ref["noise2"]))
        res["reference_spp"] = int(ref["spp"])
        out[name] = res
        r.close()
    return out


FILM_SCHEDULE = (8, 16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048)


def film_convergence(lib, torch, r, patches, ref_patch, ref_spp, target=1e-2, budget_s=45.0, stream=None, film=None,
                     unbiased=("fast",)):
    """Samples per pixel to image RMSE `target` at the workload's own film.

    The converged image is the unbiased estimator (`ref_patch`: delta
    tracking, ratio-tracked shadows, full MIS) rendered on the GPU at
    `ref_spp` from its own random stream (view 97), as two independent
    halves whose difference gives its own noise (subtracted in quadrature,
    as for the FP64 references).  That estimator's convergence to the FP64
    oracle is checked on 128^2 views of the same workloads
    (tests/test_gpu_convergence.py, and `fp64_128` below).  Each
    configuration of `patches` then renders from view 0 along FILM_SCHEDULE
    until its RMSE reaches `target` (or `budget_s` of rendering is spent).
    `film`: (W, H) of the bound tracer's camera when it differs from the
    scene's.  Samples-to-target is where the measured curve crosses the
    target (log-log interpolation between the bracketing points);
    `unbiased` names the configurations with the reference's expectation,
    for which a fit of the whole curve is reported beside it."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import convergence as CV
    W, H = film if film else (r.width, r.height)
    d = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")

    def apply(patch):
        for k, v in patch.items():
            setattr(r.tracer_desc.settings, k, v)
        r.rebind_tracer()

    def accumulate(acc, spp, view, first, chunk=64):
        n = 0
        while n < spp:
            c = min(chunk, spp - n)
            r.trace_sum_device(d.data_ptr(), c, view, first + n, 0, stream)
            acc += d.double()
            n += c

    saved = {k: getattr(r.tracer_desc.settings, k) for p in [ref_patch, *patches.values()] for k in p}
    apply(ref_patch)
    half = ref_spp // 2
    a = torch.zeros((H, W, 4), dtype=torch.float64, device="cuda")
    b = torch.zeros((H, W, 4), dtype=torch.float64, device="cuda")
    t0 = time.perf_counter()
    accumulate(a, half, 97, 0)
    accumulate(b, half, 97, half)
    torch.cuda.synchronize()
    ref_s = time.perf_counter() - t0
    e = float(r.tracer_desc.camera.exposure)
    an, bn = (a / half).cpu().numpy(), (b / half).cpu().numpy()
    diff = CV.tonemap_rgb(an, e) - CV.tonemap_rgb(bn, e)
    ref = {"mean_xyz": 0.5 * (an + bn)[..., :3], "exposure": e, "noise2": float(np.mean(diff * diff)) / 4.0}
    del a, b, an, bn
    out = {"reference": {"spp": 2 * half, "noise": float(np.sqrt(ref["noise2"])), "seconds": ref_s, "film": [W, H],
                         "what": "the unbiased estimator (delta tracking, ratio-tracked shadows, full MIS) at the "
                                 "workload's film, GPU, own random stream"}}
    for label, patch in patches.items():
        apply(patch)
        acc = torch.zeros((H, W, 4), dtype=torch.float64, device="cuda")
        n, spps, errs, spent = 0, [], [], 0.0
        for m in FILM_SCHEDULE:
            t1 = time.perf_counter()
            accumulate(acc, m - n, 0, n)
            torch.cuda.synchronize()
            spent += time.perf_counter() - t1
            n = m
            err = CV.rmse((acc / n).cpu().numpy(), ref)
            spps.append(n)
            errs.append(err)
            if err <= target or spent > budget_s:
                break
        crossing = CV.spp_to_rmse(spps, errs, target)
        out[label] = {"spp": spps, "rmse": errs, "spp_to_target": crossing}
        if label in unbiased:
            # a cross-check for an estimator with the reference's expectation,
            # which converges as rmse^2 = var / n: every schedule point from
            # 32 spp on implies n (rmse / target)^2; their geometric mean
            implied = [n_ * (e_ / target) ** 2 for n_, e_ in zip(spps, errs) if n_ >= 32 and e_ > 0]
            if implied:
                out[label]["spp_to_target_fit"] = float(np.exp(np.mean(np.log(implied))))
        del acc
    apply(saved)
    return out


def film_rmse_summary(fc, fast_value, plain_value, npix, target=1e-2):
    """time to image RMSE `target` at the workload's own film from the
    measured samples-to-target and the measured rates of each path"""
    if not fc:
        return None
    f, p = fc["fast"]["spp_to_target"], fc["plain"]["spp_to_target"]
    out = {"target": target, "reference": fc["reference"],
           "fast": {"spp": f, "seconds": f * npix / (fast_value * 1e6) if f else None, "curve": [fc["fast"]["spp"], fc["fast"]["rmse"]],
                    "spp_fit": fc["fast"].get("spp_to_target_fit")},
           "plain": {"spp": p, "seconds": p * npix / (plain_value * 1e6) if p else None,
                     "curve": [fc["plain"]["spp"], fc["plain"]["rmse"]]}}
    if f and p:
        out["speedup_equal_rmse"] = out["plain"]["seconds"] / out["fast"]["seconds"]
    return out


def rmse_summary(conv, name, fast_value, plain_value, npix, target=1e-2):
    """time to reach image RMSE `target` on the workload's film, from the
    samples per pixel the 128^2 reference view needed and the measured rates"""
    if not conv or name not in conv:
        return None
    c = conv[name]
    f, p = c["fast"]["spp_to_target"], c["plain"]["spp_to_target"]
    out = {"target": target, "reference": f"FP64 oracle, {c['reference_spp']} spp, noise {c['reference_noise']:.1e}",
           "fast": {"spp": f, "seconds": f * npix / (fast_value * 1e6) if f else None},
           "plain": {"spp": p, "seconds": p * npix / (plain_value * 1e6) if p else None,
                     "rmse_at_max_spp": c["plain"]["rmse"][-1]},
           "curves": c}
    if f and p:
        out["speedup_equal_rmse"] = out["plain"]["seconds"] / out["fast"]["seconds"]
    return out


def batched_rmse_summary(conv, value, plain_value, target=1e-2):
    """speed-up of the batched path over the plain path at equal RMSE: the
    throughput ratio times the geometric mean over the three volumes' views of
    the ratio of samples per pixel each estimator needs to reach `target`"""
    if not conv:
        return None
    ratios, per = [], {}
    for name, c in conv.items():
        f, p = c["fast"]["spp_to_target"], c["plain"]["spp_to_target"]
        per[name] = {"fast_spp": f, "plain_spp": p, "plain_rmse_at_max_spp": c["plain"]["rmse"][-1],
                     "reference_noise": c["reference_noise"] if "reference_noise" in c else c["reference"]["noise"]}
        if "reference" in c and isinstance(c["reference"], dict):
            per[name]["film"] = c["reference"]["film"]
            per[name]["curves"] = {k: [c[k]["spp"], c[k]["rmse"]] for k in ("fast", "plain")}
            if "spp_to_target_fit" in c["fast"]:
                per[name]["fast_spp_fit"] = c["fast"]["spp_to_target_fit"]
        if f and p:
            ratios.append(p / f)
    out = {"target": target, "views": per, "throughput_ratio": value / plain_value}
    if ratios and len(ratios) == len(conv):
        g = float(np.exp(np.mean(np.log(ratios))))
        out["spp_ratio_geomean"] = g
        out["speedup_equal_rmse"] = value / plain_value * g
    return out


def reference_path(scene):
    """the scene with the reference's live estimator: fixed-step march, BRDF
    at every volume event, light sampling only (bit-exact with the reference)"""
    C = importlib.import_module("exposure-render_gb300.capi")
    t = C.er_tracer_desc.from_buffer_copy(scene.tracer)
    t.settings.free_flight = 0
    t.settings.mis = 0
    t.settings.apply_shading_type = 0
    t.settings.stratify = 0
    import copy
    out = copy.copy(scene)
    out.tracer = t
    return out


def batched_workload(wl, n_views=0):
    """(scenes, views, workload name) of the batched workloads: c3, 64 orbit
    views over three blob volumes; c5, 16 views of 2048^2 at 64 spp over the
    1024x1024x512 volume"""
    S = importlib.import_module("exposure-render_gb300.scenes")
    if wl == "c5":
        views = S.c5_views(n_views=n_views or 16)
        return [S.scene_c5(S.c5_volume())], views, "c5-batched-%d-views-2048^2-1024x1024x512-volume" % len(views)
    views = S.c3_views(n_views=n_views or 64)
    return S.c3_scenes(), views, "c3-batched-%d-views-3-blob-volumes" % len(views)


def batched_reference_rate(scenes, views, seconds_target=12.0, steps=1, per_volume=4):
    """Samples/s of the reference transport on the host cores over a batch of
    views: up to `per_volume` views of each volume, spread over its orbit,
    each timed on a centre crop at 1 spp (equal shares of `seconds_target`);
    a volume's rate is the harmonic mean of its timed views' rates (each
    stands for an equal share of the volume's samples), and the batch's rate
    weights the volumes by their views' samples, sum(n_k) / sum(n_k / rate_k).
    Returns the per-view spread with the rate."""
    cams, n = {}, {}
    for k, cam, spp in views:
        cams.setdefault(k, []).append(cam)
        n[k] = n.get(k, 0) + cam.film_size[0] * cam.film_size[1] * spp
    picks = {}
    for k, cs in cams.items():
        m = min(per_volume, len(cs))
        picks[k] = [cs[(i * len(cs)) // m] for i in range(m)]
    n_timed = sum(len(v) for v in picks.values())
    seconds, kind, cores, crops, rates = 0.0, None, None, [], []
    for k in sorted(picks):
        inv = 0.0
        for cam in picks[k]:
            sc = reference_path(scenes[k])
            sc.tracer.camera = cam
            rate, kind, cores, sample = cpu_reference_rate(sc, seconds_target=seconds_target / n_timed, steps=steps)
            inv += 1.0 / rate
            rates.append(rate)
        seconds += n[k] * inv / len(picks[k])
        crops.append("volume %d: %d views, %s" % (k, len(picks[k]), sample.split(" centre")[0]))
    rate = sum(n.values()) / seconds
    sample = ("views spread over each volume's orbit, centre crop x 1 spp per step (%s); harmonic mean per volume, "
              "weighted by the volume's samples; per-view rates %.3g .. %.3g Msamples/s"
              % ("; ".join(crops), min(rates) / 1e6, max(rates) / 1e6))
    return rate, kind, cores, sample


def batched_work(scenes, views, settings_of, nthreads, spp=2, reference=False):
    """Per-sample work counters of a batch: the oracle's counts on the first
    view of each volume (whole field of view at 128^2, that volume's tracer
    settings, or the reference estimator's), weighted by the samples of the
    volume's views."""
    import copy
    first, n = {}, {}
    for k, cam, s in views:
        first.setdefault(k, cam)
        n[k] = n.get(k, 0) + cam.film_size[0] * cam.film_size[1] * s
    total = float(sum(n.values()))
    out = {}
    for k in sorted(first):
        sc = copy.copy(reference_path(scenes[k]) if reference else scenes[k])
        C = importlib.import_module("exposure-render_gb300.capi")
        sc.tracer = C.er_tracer_desc.from_buffer_copy(sc.tracer)
        sc.tracer.camera = first[k]
        w = oracle_work(sc, sc.tracer.settings if reference else settings_of(k), nthreads, spp=spp)
        for key, v in w.items():
            out[key] = out.get(key, 0.0) + v * n[k] / total
    return out


def run_reference(args, wl, rank, world):
    if rank != 0:
        return
    if wl == "c4":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no differentiable medium and no "
                          "adjoint (its transport is forward only)"}), flush=True)
        return
    if wl in ("c3", "c5"):
        scenes, views, name = batched_workload(wl, args.views)
        shading = describe_shading(reference_path(scenes[0]))
        for _ in range(args.warmup):
            batched_reference_rate(scenes, views, seconds_target=2.0, steps=1)
        rate, kind, cores, sample = batched_reference_rate(scenes, views, seconds_target=10.0 * max(1, args.steps) / 3.0,
                                                           steps=args.steps)
        config = {"workload": name, "views": len(views),
                  "samples_per_step": sum(c.film_size[0] * c.film_size[1] * s for _, c, s in views), **shading}
    else:
        scene = reference_path(make_scene(wl))
        shading = describe_shading(scene)
        W = WORKLOADS[wl]
        for _ in range(args.warmup):
            cpu_reference_rate(scene, seconds_target=2.0, steps=1)
        rate, kind, cores, sample = cpu_reference_rate(scene, seconds_target=10.0 * max(1, args.steps) / 3.0, steps=args.steps)
        config = {"workload": W["name"], "film": list(W["film"]), "spp": W["spp"], **shading}
    line = {
        "impl": "reference", "metric": "Msamples/s", "value": rate / 1e6, "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config,
        "cpu_baseline": {"value": rate / 1e6, "unit": "Msamples/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": rate / 1e6, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, wl, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    pkg = importlib.import_module("exposure-render_gb300")
    runtime = importlib.import_module("exposure-render_gb300.runtime")
    C = pkg.capi
    lib = C.load_library()
    C.check(lib.er_set_device(local_rank))
    W = WORKLOADS[wl]
    scene = make_scene(wl)
    scene.tracer.settings.free_flight = 1                # the fast path: delta tracking, full MIS,
    scene.tracer.settings.mis = 1                        # stratified light samples
    scene.tracer.settings.stratify = 1
    shading = describe_shading(scene)
    # one image over all ranks: the same seed and view, and in step k rank r
    # renders the sample range [(k world + r) spp, (k world + r + 1) spp) of
    # the view's stream; the per-pixel sums are all-reduced every step
    scene.tracer.settings.seed = R.view_seed(1, 0)
    r = runtime.Renderer(scene, lib)
    spp = W["spp"]
    width, height = scene.width, scene.height
    stream = torch.cuda.current_stream()
    C.check(lib.er_set_stream(ctypes.c_void_p(stream.cuda_stream)))
    tuned = r.autotune(2) if not args.no_tune else None     # majorant brick and stage occupancy
    d_sum = torch.zeros((height, width, 4), dtype=torch.float32, device="cuda")
    dist = None
    if world > 1:
        import torch.distributed as dist

    def step(k):
        r.trace_sum_device(d_sum.data_ptr(), spp, 0, (k * world + rank) * spp, 0, ctypes.c_void_p(stream.cuda_stream))
        R.sum_over_ranks(d_sum, dist)
    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stage_ms, stage_launches = read_profile(lib, C)          # clears earlier marks
    C.check(lib.er_profile_enable(1))
    with ClockSampler(local_rank) as clk:
        ev0.record(stream)
        for k in range(args.steps):
            step(args.warmup + k)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    C.check(lib.er_profile_enable(0))
    stage_ms, stage_launches = read_profile(lib, C)
    ms = R.max_over_ranks(ms, dist)
    R.barrier(dist)
    samples_per_step = width * height * spp
    value = R.whole_job_rate(samples_per_step * args.steps, ms / 1e3, world) / 1e6

    # the plain single-view path on the same workload and shading: the
    # reference's fixed-step march (one warm-up, one timed step)
    def timed_plain(settings_patch):
        saved = {k: getattr(r.tracer_desc.settings, k) for k in settings_patch}
        for k, v in settings_patch.items():
            setattr(r.tracer_desc.settings, k, v)
        r.rebind_tracer()
        step(0)
        torch.cuda.synchronize()
        # one timed step, or the median of five when a step is shorter than 0.2 s
        times = []
        for k in range(5):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step(1 + k)
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
            if times[0] >= 200.0:
                break
        for k, v in saved.items():
            setattr(r.tracer_desc.settings, k, v)
        r.rebind_tracer()
        return samples_per_step / (statistics.median(times) / 1e3) / 1e6

    plain = timed_plain({"free_flight": 0, "stratify": 0})
    ref_order = timed_plain({"free_flight": 0, "mis": 0, "apply_shading_type": 0, "bilateral": 0, "stratify": 0})

    # end to end through the C ABI with host buffers: the volume and the RGBA8
    # estimate live in pinned host memory (BindVoxels' source, GetEstimate's target)
    pinned_vol = torch.from_numpy(np.ascontiguousarray(scene.volume).view(np.int16)).pin_memory()
    vd = scene.volume_desc()
    vd.voxels = ctypes.cast(ctypes.c_void_p(pinned_vol.data_ptr()), ctypes.POINTER(ctypes.c_uint16))
    vol_bytes = scene.volume.nbytes
    tr_bytes = ctypes.sizeof(r.tracer_desc)
    out = torch.empty((height, width, 4), dtype=torch.uint8, pin_memory=True)
    e2e_steps = max(1, min(args.steps, 3))

    def e2e_step():
        vid = ctypes.c_int32(r.volume_id)
        C.check(lib.er_bind_volume(ctypes.byref(vd), ctypes.byref(vid)))
        tid = ctypes.c_int32(r.tracer_id)
        C.check(lib.er_bind_tracer(ctypes.byref(r.tracer_desc), ctypes.byref(tid)))
        C.check(lib.er_reset_accumulation(r.tracer_id))
        C.check(lib.er_render_spp(r.tracer_id, spp))
        C.check(lib.er_get_estimate(r.tracer_id, out.data_ptr()))

    e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = R.max_over_ranks(time.perf_counter() - t0, dist)
    e2e_value = R.whole_job_rate(samples_per_step * e2e_steps, e2e_s, world) / 1e6

    if rank != 0:
        return
    conv = None
    rmse_name = {"c1": "c1p"}.get(wl, wl)      # the FP64 view with the workload's shading
    if world == 1 and not args.no_rmse and wl in ("c1", "c2"):
        conv = convergence(lib, runtime, torch, [rmse_name], {
            "fast": {"free_flight": 1, "mis": 1, "stratify": 1, "majorant_brick": r.tracer_desc.settings.majorant_brick},
            "plain": {"free_flight": 0, "mis": 1, "stratify": 0}})
    film_conv = None
    if world == 1 and not args.no_rmse and wl in ("c1", "c2"):
        film_conv = film_convergence(
            lib, torch, r,
            {"fast": {"free_flight": 1, "mis": 1, "stratify": 1}, "plain": {"free_flight": 0, "mis": 1, "stratify": 0}},
            {"free_flight": 1, "mis": 1, "stratify": 0}, 8192 if wl == "c2" else 16384,
            stream=ctypes.c_void_p(stream.cuda_stream))
    peaks, peak_kind = measured_peaks()
    nthreads = os.cpu_count() or 1
    # work per sample of the measured configuration (oracle, whole field of view at 128^2)
    work = oracle_work(scene, r.tracer_desc.settings, nthreads)
    ref_work = oracle_work(reference_path(scene), reference_path(scene).tracer.settings, nthreads, spp=1)
    roofline, stages = stage_roofline(work, ref_work, stage_ms, stage_launches, samples_per_step * args.steps, peaks, peak_kind, wl)
    cpu_rate, kind, cores, sample = (None, None, None, None)
    if world == 1:
        cpu_rate, kind, cores, sample = cpu_reference_rate(reference_path(scene), seconds_target=12.0, steps=1)
    line = {
        "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": W["name"], "film": list(W["film"]), "spp": W["spp"], **shading,
                   "kernels": "k_wf_primary / k_wf_shade / k_wf_shadow / k_wf_reduce (wavefront stages)",
                   "autotune": tuned,
                   "l2": "inputs larger than L2 (volume %d MiB)" % (vol_bytes >> 20) if vol_bytes > (129 << 20) else
                   "volume fits in L2 (%d MiB); transport re-reads it from L2" % (vol_bytes >> 20),
                   "parallelism": "sample ranges of one image per rank, per-pixel sums all-reduced each step" if world > 1
                   else "single"},
        "roofline": roofline,
        "cpu_baseline": ({"value": cpu_rate / 1e6, "unit": "Msamples/s", "cores": cores, "kind": kind, "sample": sample}
                         if cpu_rate else None),
        "e2e": {"value": e2e_value, "unit": "Msamples/s", "h2d_bytes_per_step": int(vol_bytes + tr_bytes),
                "d2h_bytes_per_step": int(out.nbytes)},
        "clocks": clk.summary(),
        "gpu_launches": int(sum(stage_launches)),
        "stages": stages,
        "work_per_sample": work,
        "reference_work_per_sample": ref_work,
        "plain": {"value": plain, "unit": "Msamples/s", "speedup": value / plain,
                  "what": "same workload and estimator, the reference's fixed-step march for free flight and shadows"},
        "time_to_rmse": film_rmse_summary(film_conv, value, plain, width * height),
        "time_to_rmse_fp64_128": (dict(rmse_summary(conv, rmse_name, value, plain, width * height) or {},
                                       note="samples per pixel to RMSE 1e-2 measured on a 128^2 view against the FP64 "
                                            "oracle, times the workload's pixels") if conv else None),
        "reference_order": {"value": ref_order, "unit": "Msamples/s",
                            "what": "reference live path (march, BRDF, light sampling), bit-exact with the reference"},
    }
    print(json.dumps(line), flush=True)
    r.close()


def run_batched(args, rank, world, local_rank, wl="c3"):
    """c3: 64 orbit views over three blob volumes; c5: 16 orbit views of 2048^2
    at 64 spp over the 1024x1024x512 volume, plus the path-replay adjoint on
    a 256^3 density sub-block of it.  One CUDA-graph launch per step
    (er_batch_launch), against the same views rendered one batch per view and
    against the reference estimator one view and one frame at a time."""
    import torch
    torch.cuda.set_device(local_rank)
    runtime = importlib.import_module("exposure-render_gb300.runtime")
    C = importlib.import_module("exposure-render_gb300.capi")
    lib = C.load_library()
    C.check(lib.er_set_device(local_rank))
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    C.check(lib.er_set_stream(sp))
    t_gen = time.perf_counter()
    scenes, views, wl_name = batched_workload(wl, args.views)
    gen_s = time.perf_counter() - t_gen
    c5_vol = scenes[0].volume if wl == "c5" else None
    # every rank renders every view, from its own sample range of each view's
    # stream (step k, rank r: the range k world + r), and the views' sums are
    # all-reduced each step: one set of images over all ranks
    for sc in scenes:
        sc.tracer.settings.seed = R.view_seed(1, 0)
    if args.bricks:
        # fixed tuning (profiling runs with --no-tune): one majorant brick per volume
        for sc, b in zip(scenes, (int(x) for x in args.bricks.split(","))):
            sc.tracer.settings.majorant_brick = b
    if args.stages is not None:
        for sc in scenes:
            sc.tracer.settings.tune_stages = args.stages
    dist = None
    if world > 1:
        import torch.distributed as dist
    rs = [runtime.Renderer(sc, lib) for sc in scenes]
    # autotune each volume's tracer on one of its views (probe: 2 spp)
    tuned = []
    for k, r in enumerate(rs):
        cams = [cam for (kk, cam, _) in views if kk == k]
        if cams and not args.no_tune:
            r.tracer_desc.camera = cams[0]
            r.rebind_tracer()
            tuned.append(r.autotune(2))
    # the views' sums in one buffer (one all-reduce per step)
    sizes = [cam.film_size[1] * cam.film_size[0] * 4 for _, cam, _ in views]
    flat = torch.zeros(sum(sizes), dtype=torch.float32, device="cuda")
    sums, o = [], 0
    for (_, cam, _), n in zip(views, sizes):
        sums.append(flat[o:o + n].view(cam.film_size[1], cam.film_size[0], 4))
        o += n
    table = [(rs[k].tracer_id, spp, d.data_ptr(), cam) for (k, cam, spp), d in zip(views, sums)]
    samples_per_step = sum(cam.film_size[0] * cam.film_size[1] * spp for _, cam, spp in views)
    max_spp = max(spp for _, _, spp in views)
    batch = runtime.Batch(table, flags=C.ER_BATCH_GRAPH)
    # the tracking stages' persistent-lane mode, timed on whole launches of
    # this batch
    batch_tune = batch.autotune(sp) if not args.no_tune else None
    if batch_tune:
        # the batch tuner writes the tracers' bricks: keep the Python-side
        # descriptors in step, so that later rebinds keep them
        for r in rs:
            st = C.er_render_settings()
            C.check(lib.er_get_render_settings(r.tracer_id, st))
            r.tracer_desc.settings = st
        batch_tune["bricks"] = [r.tracer_desc.settings.majorant_brick for r in rs]
    info = batch.info()

    def timed(fn, steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    def step():
        batch.advance(world * max_spp, sp)      # fresh samples every step
        batch.launch(sp)
        R.sum_over_ranks(flat, dist)

    if rank:
        batch.advance(rank * max_spp, sp)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    R.barrier(dist)
    with ClockSampler(local_rank) as clk:
        ms = timed(step, args.steps)
    ms = R.max_over_ranks(ms, dist)
    value = R.whole_job_rate(samples_per_step * args.steps, ms / 1e3, world) / 1e6

    # stage shares: the same batch launched without the graph, profiled
    prof = runtime.Batch(table, flags=0)
    if batch_tune:
        prof.set_stages(batch_tune["tune_stages"])
    prof.launch(sp)
    torch.cuda.synchronize()
    read_profile(lib, C)
    C.check(lib.er_profile_enable(1))
    prof_ms = timed(lambda: prof.launch(sp), 1)
    C.check(lib.er_profile_enable(0))
    stage_ms, stage_launches = read_profile(lib, C)
    prof.close()

    # the same views, one single-view batch (graph) per view, back to back
    singles = [runtime.Batch([t], flags=C.ER_BATCH_GRAPH) for t in table]
    for b in singles:
        b.launch(sp)
    ms_seq = timed(lambda: [b.launch(sp) for b in singles], 1)
    for b in singles:
        b.close()
    seq_value = samples_per_step / (ms_seq / 1e3) / 1e6

    # plain: the single-view GPU path at its best - each view's full spp in
    # one er_trace_sum_device call (the wavefront stages, as c2's plain path),
    # one view at a time - with the same estimator except the reference's
    # fixed-step march for free flight and shadows and no stratification
    plain_samples, plain_ms = 0, 0.0
    n_plain = args.plain_views if args.plain_views is not None else (2 if wl == "c5" else len(views))
    plain_sum = torch.zeros((max(c.film_size[1] for _, c, _ in views), max(c.film_size[0] for _, c, _ in views), 4),
                            dtype=torch.float32, device="cuda")
    for i, (k, cam, spp) in enumerate(views[:n_plain]):
        r = rs[k]
        saved = C.er_tracer_desc.from_buffer_copy(r.tracer_desc)
        r.tracer_desc.camera = cam
        r.tracer_desc.settings.free_flight = 0
        r.tracer_desc.settings.stratify = 0
        r.rebind_tracer()
        if i == 0:
            r.trace_sum_device(plain_sum.data_ptr(), 1, i, 0, 0, sp)      # warm-up
            torch.cuda.synchronize()
        plain_ms += timed(lambda: r.trace_sum_device(plain_sum.data_ptr(), spp, i, 0, 0, sp), 1)
        plain_samples += spp * cam.film_size[0] * cam.film_size[1]
        ctypes.memmove(ctypes.byref(r.tracer_desc), ctypes.byref(saved), ctypes.sizeof(saved))
        r.rebind_tracer()
    del plain_sum
    plain_value = plain_samples / (plain_ms / 1e3) / 1e6

    # equal-RMSE comparison on the first view of each volume: at 128^2 against
    # the FP64 references, and at each view's own film against a converged
    # GPU render of the unbiased estimator
    conv, film_conv = None, None
    if world == 1 and not args.no_rmse and wl == "c5":
        # c5: its first view on a 128^2 film against the FP64 oracle's
        # converged image (tests/golden/fp64_c5v0.npz), and at 2048^2
        # against the converged GPU render of the unbiased estimator
        conv = convergence(lib, runtime, torch, ["c5v0"],
                           {"fast": {"free_flight": 1, "stratify": 1}, "plain": {"free_flight": 0, "stratify": 0}})
        r = rs[0]
        cam = views[0][1]
        saved = C.er_tracer_desc.from_buffer_copy(r.tracer_desc)
        r.tracer_desc.camera = cam
        r.rebind_tracer()
        film_conv = {"c5v0": film_convergence(
            lib, torch, r, {"fast": {"free_flight": 1, "stratify": 1}, "plain": {"free_flight": 0, "stratify": 0}},
            {"free_flight": 1, "stratify": 0}, 4096, budget_s=75.0, stream=sp, film=(cam.film_size[0], cam.film_size[1]))}
        ctypes.memmove(ctypes.byref(r.tracer_desc), ctypes.byref(saved), ctypes.sizeof(saved))
        r.rebind_tracer()
    if world == 1 and not args.no_rmse and wl == "c3":
        conv = convergence(lib, runtime, torch, ["c3v0", "c3v1", "c3v2"],
                           {"fast": {"free_flight": 1, "stratify": 1}, "plain": {"free_flight": 0, "stratify": 0}})
        film_conv = {}
        for k, r in enumerate(rs):
            cam = [c for (kk, c, _) in views if kk == k][0]
            saved = C.er_tracer_desc.from_buffer_copy(r.tracer_desc)
            r.tracer_desc.camera = cam
            r.rebind_tracer()
            film_conv["c3v%d" % k] = film_convergence(
                lib, torch, r, {"fast": {"free_flight": 1, "stratify": 1}, "plain": {"free_flight": 0, "stratify": 0}},
                {"free_flight": 1, "stratify": 0}, 8192, budget_s=30.0, stream=sp, film=(cam.film_size[0], cam.film_size[1]))
            ctypes.memmove(ctypes.byref(r.tracer_desc), ctypes.byref(saved), ctypes.sizeof(saved))
            r.rebind_tracer()

    # end to end with host buffers: volumes bound from host memory, one batch
    # launch, every view's sums read back into pinned host memory
    host_sums = [torch.empty(d.shape, dtype=torch.float32, pin_memory=True) for d in sums]
    pinned_vols = [torch.from_numpy(np.ascontiguousarray(sc.volume).view(np.int16)).pin_memory() for sc in scenes]
    vds = [sc.volume_desc() for sc in scenes]
    for vd, pv in zip(vds, pinned_vols):
        vd.voxels = ctypes.cast(ctypes.c_void_p(pv.data_ptr()), ctypes.POINTER(ctypes.c_uint16))

    def e2e_step():
        for r, vd in zip(rs, vds):
            vid = ctypes.c_int32(r.volume_id)
            C.check(lib.er_bind_volume(ctypes.byref(vd), ctypes.byref(vid)))
        step()
        for h, d in zip(host_sums, sums):
            h.copy_(d, non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = R.max_over_ranks(time.perf_counter() - t0, dist)
    e2e_value = R.whole_job_rate(samples_per_step * e2e_steps, e2e_s, world) / 1e6
    d2h_bytes = int(sum(h.numel() * 4 for h in host_sums))
    adjoint = None
    if wl == "c5":
        # the batch's queues and films are released before the adjoint's buffers are made
        batch.close()
        del sums, host_sums, table
        torch.cuda.empty_cache()
        adjoint = c5_adjoint(args, lib, runtime, torch, stream, c5_vol)
    if rank != 0:
        return
    # the reference transport on the host cores (rank 0 at N = 1 only)
    cpu = batched_reference_rate(scenes, views) if world == 1 else None
    vol_bytes = sum(sc.volume.nbytes for sc in scenes)
    # roofline of the dominant stage of the profiled launch (one pass of the batch)
    peaks, peak_kind = measured_peaks()
    nthreads = os.cpu_count() or 1
    work = batched_work(scenes, views, lambda k: rs[k].tracer_desc.settings, nthreads)
    ref_work = batched_work(scenes, views, None, nthreads, spp=1, reference=True)
    roofline, stages = stage_roofline(work, ref_work, stage_ms, stage_launches, samples_per_step, peaks, peak_kind, wl)
    line = {
        "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl_name, "views": len(views),
                   "samples_per_step": samples_per_step, "films": sorted({c.film_size[0] for _, c, _ in views}),
                   "spp_range": [min(s for _, _, s in views), max_spp], **describe_shading(scenes[0]),
                   "free_flight": "delta+ratio tracking, majorant bricks per volume below",
                   "windows": info["windows"], "segments": info["segments"], "queue_bytes": info["queue_bytes"],
                   "autotune": tuned, "batch_autotune": batch_tune,
                   "majorant_bricks": [r.tracer_desc.settings.majorant_brick for r in rs],
                   "l2": "volumes %d MiB in total; every step renders fresh samples" % (vol_bytes >> 20),
                   "parallelism": "sample ranges of every view per rank, sums all-reduced each step" if world > 1 else "single"},
        "cpu_baseline": ({"value": cpu[0] / 1e6, "unit": "Msamples/s", "cores": cpu[2], "kind": cpu[1], "sample": cpu[3]}
                         if cpu else None),
        "e2e": {"value": e2e_value, "unit": "Msamples/s", "h2d_bytes_per_step": int(vol_bytes),
                "d2h_bytes_per_step": d2h_bytes},
        "clocks": clk.summary(),
        "gpu_launches": args.steps * (4 * info["windows"]),
        "roofline": roofline,
        "stages": stages,
        "work_per_sample": work,
        "profiled_pass_ms": prof_ms,
        "one_batch_per_view": {"value": seq_value, "unit": "Msamples/s", "speedup": value / seq_value},
        "plain": {"value": plain_value, "unit": "Msamples/s", "speedup": value / plain_value, "views": n_plain,
                  "what": "same estimator with the fixed-step march and no stratification, each view's full spp in one "
                          "er_trace_sum_device call, one view at a time"},
        "equal_rmse": batched_rmse_summary(film_conv, value, plain_value) if film_conv else
        {"throughput_ratio": value / plain_value, "note": "no samples-to-RMSE measurement in this run (--no-rmse or N > 1)"},
        "equal_rmse_fp64_128": (dict(batched_rmse_summary(conv, value, plain_value) or {},
                                     note="samples to RMSE 1e-2 on 128^2 views against the FP64 oracle") if conv else None),
    }
    if wl == "c5":
        line["volume_generation_s"] = gen_s
        line["adjoint"] = adjoint
    print(json.dumps(line), flush=True)
    if wl != "c5":
        batch.close()
    for r in rs:
        r.close()


def c5_adjoint(args, lib, runtime, torch, stream, vol, film=(2048, 2048), spp=8, size=256):
    """c5's adjoint: the differentiable tracer model (64-node opacity PLF
    with its node values as parameters, colour TFs, hybrid shading; --medium
    spline: the B-spline medium) on the centred 256^3 block of the c5 volume
    (a float intensity window), one 2048^2 view at 8 spp; forward, adjoint
    with the forward's samples kept, and adjoint with seed-replay
    recomputation (nothing kept)"""
    medium = importlib.import_module("exposure-render_gb300.medium")
    S = importlib.import_module("exposure-render_gb300.scenes")
    rho_np = S.density_subblock(vol, size)
    rho = torch.from_numpy(rho_np).cuda()
    if args.medium == "tracer":
        sc = S.tf_medium_scene(res=(size, size, size), film=film, n_nodes=64)
        r = runtime.Renderer(sc, lib)
        tf = torch.from_numpy(S.plf_node_values(sc.tracer.opacity)).cuda()
        m = medium.Medium(r, rho, tf, 40.0, nee_probability=0.5, brick=8, model="tracer",
                          gradient_magnitude_inv=S.gradient_magnitude_range(rho_np))
    else:
        tf = torch.from_numpy(S.ramp_opacity(64)).cuda()
        sc = S.medium_scene(res=(size, size, size), film=film)
        r = runtime.Renderer(sc, lib)
        m = medium.Medium(r, rho, tf, 40.0, albedo=(0.8, 0.7, 0.6), nee_probability=0.5, brick=8)
    target = torch.zeros((film[1], film[0], 3), device="cuda")

    def timed(fn, steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps

    state = {}

    def fwd():
        state["smp"], state["s"] = m.render_samples(rho, tf, spp)

    def bwd():
        d = 2.0 * (state["s"] / spp - target) / spp / target.numel()
        state["g"] = m.adjoint(rho, tf, spp, d, state["smp"])

    def bwd_recompute():
        d = 2.0 * (state["s"] / spp - target) / spp / target.numel()
        state["g2"] = m.adjoint(rho, tf, spp, d, None)

    steps = max(1, min(args.steps, 2))
    for _ in range(max(1, min(args.warmup, 2))):
        fwd()
        bwd()
    torch.cuda.synchronize()
    f_ms = timed(fwd, steps)
    b_ms = timed(bwd, steps)
    br_ms = timed(bwd_recompute, 1)
    # the adjoints gather with atomics, so the two agree to float summation order
    rel = max(float((state["g"][i] - state["g2"][i]).norm() / max(float(state["g"][i].norm()), 1e-30)) for i in range(2))
    out = {"what": "%s on the centred %d^3 block of the c5 volume, %dx%d x %d spp"
                   % ("the differentiable tracer model (64-node opacity PLF, colour TFs, hybrid shading)" if args.medium == "tracer"
                      else "the B-spline medium (64 opacity values)", size, film[0], film[1], spp),
           "samples": film[0] * film[1] * spp, "forward_ms": f_ms, "adjoint_ms": b_ms, "adjoint_over_forward": b_ms / f_ms,
           "adjoint_recompute_ms": br_ms, "adjoint_recompute_over_forward": br_ms / f_ms,
           "forward_msamples_per_s": film[0] * film[1] * spp / (f_ms / 1e3) / 1e6,
           "recompute_vs_kept_rel_diff": rel,
           "grad_norm": {"density": float(state["g"][0].norm()), "opacity": float(state["g"][1].norm())}}
    del state
    r.close()
    return out


def medium_cpu_rate(sc, rho, tf, m, seconds_target=10.0):
    """forward samples/s of the same differentiable estimator in the CPU
    oracle (the reference has no differentiable path; kind "port"), all host
    threads, on a film crop of the workload's camera (the oracle renders
    whole films: the camera's film is shrunk, which keeps the field of view),
    with the forward+adjoint time ratio of the same run"""
    import copy
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as OL
    C = importlib.import_module("exposure-render_gb300.capi")
    orc = OL.load_oracle()
    nthreads = os.cpu_count() or 1
    maj = m.majorant.cpu().numpy()

    def run(side, spp):
        s2 = copy.copy(sc)
        s2.tracer = C.er_tracer_desc.from_buffer_copy(sc.tracer)
        s2.tracer.camera.film_size[0] = s2.tracer.camera.film_size[1] = side
        h = OL.MediumHandle(orc, s2, rho, tf, m.scale, np.array(m.albedo), m.q, maj, m.brick, model=m.model, gm_inv=m.gm_inv)
        t0 = time.perf_counter()
        img, smp = h.render(spp, keep_samples=True, nthreads=nthreads)
        t1 = time.perf_counter()
        h.adjoint(spp, np.ones_like(img) * 1e-3, smp, nthreads=nthreads)
        t2 = time.perf_counter()
        h.close()
        return side * side * spp / max(t1 - t0, 1e-6), (t2 - t1) / max(t1 - t0, 1e-6)

    side = 32
    rate, _ = run(side, 2)
    side = int(max(32, min(256, np.sqrt(rate * seconds_target / 4.0))))
    rate, ratio = run(side, 4)
    return {"value": rate / 1e6, "unit": "Msamples/s", "cores": nthreads, "kind": "port",
            "sample": "%dx%d film of the workload's camera x 4 spp, forward (the oracle's float restatement of the same "
                      "estimator; the reference has no differentiable path)" % (side, side),
            "adjoint_over_forward": ratio}


def run_medium(args, rank, world, local_rank):
    """c4: the differentiable tracer model (ER_MEDIUM_TRACER: the tracer's
    64-node opacity PLF with its node values as parameters, its colour
    transfer functions and hybrid BRDF/phase shading) over a 128^3 float
    intensity grid, 256^2 x 32 spp; forward (every sample kept) and
    path-replay adjoint of an L2 image loss against a target rendered at
    1024 spp from parameters perturbed by N(0, 0.05).  --medium spline
    runs the B-spline/isotropic medium instead."""
    import torch
    torch.cuda.set_device(local_rank)
    runtime = importlib.import_module("exposure-render_gb300.runtime")
    medium = importlib.import_module("exposure-render_gb300.medium")
    S = importlib.import_module("exposure-render_gb300.scenes")
    C = importlib.import_module("exposure-render_gb300.capi")
    lib = C.load_library()
    C.check(lib.er_set_device(local_rank))
    stream = torch.cuda.current_stream()
    C.check(lib.er_set_stream(ctypes.c_void_p(stream.cuda_stream)))
    res, film, spp = (128, 128, 128), (256, 256), 32
    tracer_model = args.medium == "tracer"
    sc = S.tf_medium_scene(res=res, film=film, n_nodes=64) if tracer_model else S.medium_scene(res=res, film=film)
    sc.tracer.settings.seed = R.view_seed(1, rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
    r = runtime.Renderer(sc, lib)
    rho_np = S.blob_density(res, n_blobs=10, seed=40)
    rho = torch.from_numpy(rho_np).cuda()
    if tracer_model:
        tf = torch.from_numpy(S.plf_node_values(sc.tracer.opacity)).cuda()
        m = medium.Medium(r, rho, tf, 40.0, nee_probability=0.5, brick=8, model="tracer",
                          gradient_magnitude_inv=S.gradient_magnitude_range(rho_np))
    else:
        tf = torch.from_numpy(S.ramp_opacity(64)).cuda()
        m = medium.Medium(r, rho, tf, 40.0, albedo=(0.8, 0.7, 0.6), nee_probability=0.5, brick=8)
    gen = torch.Generator(device="cuda").manual_seed(7)
    rho_t = (rho + 0.05 * torch.randn(rho.shape, device="cuda", generator=gen)).contiguous()
    tf_t = (tf + 0.05 * torch.randn(tf.shape, device="cuda", generator=gen)).contiguous()
    maj0 = m.majorant.clone()
    m.rebuild_majorant(rho_t, tf_t)
    m.majorant = torch.maximum(maj0, m.majorant).contiguous()
    _, ts = m.render_samples(rho_t, tf_t, 1024, view=1)
    target = ts / 1024

    def timed(fn, steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps

    state = {}

    def fwd():
        state["smp"], state["s"] = m.render_samples(rho, tf, spp)

    def bwd():
        d = 2.0 * (state["s"] / spp - target) / spp / target.numel()
        state["g"] = m.adjoint(rho, tf, spp, d, state["smp"])

    def bwd_recompute():
        d = 2.0 * (state["s"] / spp - target) / spp / target.numel()
        m.adjoint(rho, tf, spp, d, None)

    for _ in range(args.warmup):
        fwd()
        bwd()
    torch.cuda.synchronize()
    R.barrier(dist)
    with ClockSampler(local_rank) as clk:
        f_ms = timed(fwd, args.steps)
        b_ms = timed(bwd, args.steps)
    f_ms, b_ms = R.max_over_ranks(f_ms, dist), R.max_over_ranks(b_ms, dist)
    br_ms = timed(bwd_recompute, 1)
    C.check(lib.er_synchronize())
    samples = film[0] * film[1] * spp

    # end to end, each step: the parameters (density grid, node values) from
    # pinned host memory, forward, loss gradient, adjoint, both gradients back
    # into pinned host memory (the optimiser on the host side of the API)
    h_rho, h_tf = rho.cpu().pin_memory(), tf.cpu().pin_memory()
    g_rho_h = torch.empty(rho.shape, dtype=torch.float32, pin_memory=True)
    g_tf_h = torch.empty(tf.shape, dtype=torch.float32, pin_memory=True)
    d_rho, d_tf = torch.empty_like(rho), torch.empty_like(tf)

    def e2e_step():
        d_rho.copy_(h_rho, non_blocking=True)
        d_tf.copy_(h_tf, non_blocking=True)
        smp, s = m.render_samples(d_rho, d_tf, spp)
        d = 2.0 * (s / spp - target) / spp / target.numel()
        g = m.adjoint(d_rho, d_tf, spp, d, smp)
        g_rho_h.copy_(g[0], non_blocking=True)
        g_tf_h.copy_(g[1], non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = R.max_over_ranks(time.perf_counter() - t0, dist)
    e2e = {"value": R.whole_job_rate(samples * e2e_steps, e2e_s, world) / 1e6, "unit": "Msamples/s (forward + adjoint)",
           "h2d_bytes_per_step": int(h_rho.numel() * 4 + h_tf.numel() * 4),
           "d2h_bytes_per_step": int(g_rho_h.numel() * 4 + g_tf_h.numel() * 4),
           "ms_per_step": e2e_s / e2e_steps * 1e3}
    loss = float(((state["s"] / spp - target) ** 2).mean())
    if rank != 0:
        return
    cpu = medium_cpu_rate(sc, rho_np, tf.cpu().numpy(), m) if world == 1 else None
    line = {
        "metric": "Msamples/s", "value": R.whole_job_rate(samples, f_ms / 1e3, world) / 1e6, "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": f_ms + b_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "c4-differentiable-128^3-grid-64-node-opacity-256^2-32spp", "scale": 40.0, "nee_probability": 0.5,
                   "majorant_brick": 8, "loss": "mean squared error vs 1024-spp target of perturbed parameters",
                   "model": ("the tracer's transfer functions: 64-node opacity PLF (node values are parameters), colour TFs, "
                             "hybrid BRDF/phase shading (expected value over the shader choice), float intensity grid"
                             if tracer_model else "B-spline opacity (64 values), isotropic phase, float density grid"),
                   "parallelism": "independent replicas (own seeds)" if world > 1 else "single"},
        "forward_ms": f_ms, "adjoint_ms": b_ms, "adjoint_over_forward": b_ms / f_ms,
        "adjoint_recompute_ms": br_ms, "adjoint_recompute_over_forward": br_ms / f_ms,
        "e2e": e2e,
        "loss": loss, "grad_norm": {"density": float(state["g"][0].norm()), "opacity": float(state["g"][1].norm())},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        # per window of 2^21 items: forward count, jobs, shadow, gather (+ one reduce per step);
        # adjoint primary replay and shadow replay (one window: against the forward's kept jobs;
        # several: count, jobs and shadow again per window)
        "gpu_launches": args.steps * ((6 if spp * film[0] * film[1] <= (1 << 21) else 9)
                                      * (-(-spp // max(1, (1 << 21) // (film[0] * film[1])))) + 1),
    }
    print(json.dumps(line), flush=True)
    r.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS) + ["c3", "c4", "c5"])
    ap.add_argument("--views", type=int, default=0, help="c3/c5: number of views (0: 64 for c3, 16 for c5)")
    ap.add_argument("--plain-views", type=int, default=None, help="c3/c5: views timed on the plain one-view path (all / 2)")
    ap.add_argument("--film", type=int, default=0, help="square film edge (smaller profiling cases; 0 = the workload's)")
    ap.add_argument("--spp", type=int, default=0, help="samples per pixel (0 = the workload's)")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (default settings)")
    ap.add_argument("--bricks", default="", help="c3/c5: majorant brick per volume, comma-separated (with --no-tune)")
    ap.add_argument("--stages", type=int, default=None, help="c3/c5: tune_stages of every volume's tracer (with --no-tune)")
    ap.add_argument("--no-rmse", action="store_true", help="skip the time-to-RMSE measurement")
    ap.add_argument("--medium", default="tracer", choices=["tracer", "spline"],
                    help="c4/c5 adjoint: the tracer's transfer functions and shading, or the B-spline medium")
    args = ap.parse_args()
    if (args.film or args.spp) and args.workload in WORKLOADS:
        W = dict(WORKLOADS[args.workload])
        if args.film:
            W["film"] = (args.film, args.film)
        if args.spp:
            W["spp"] = args.spp
        W["name"] = W["name"].split("-")[0] + "-%s-%dx%d-%dspp" % (W["name"].split("-")[1], W["film"][0], W["film"][1], W["spp"])
        WORKLOADS[args.workload] = W
    rank, world, local_rank = R.rank_info()
    if args.impl == "reference":
        run_reference(args, args.workload, rank, world)
        return
    # replicas: one process per GPU; the process group carries only the
    # barrier and the max-over-ranks timing of every workload
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    if args.workload in ("c3", "c5"):
        run_batched(args, rank, world, local_rank, args.workload)
    elif args.workload == "c4":
        run_medium(args, rank, world, local_rank)
    else:
        run_ours(args, args.workload, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
