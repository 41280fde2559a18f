"""Generates tests/golden/fp64_<view>.npz: converged images of the views of
scenes.rmse_views() from the FP64 oracle (oracle/_build/liberfp64.so, the C
restatement evaluated in binary64).

Each image is the mean of N samples per pixel of the unbiased estimator
(delta-tracked free flight, ratio-tracked shadows, full MIS, independent
random draws) from its own
random stream (seed 0x5EED64, view 7), rendered as two independent halves;
the squared tone-mapped difference of the halves / 4 is the reference's own
noise, stored as noise2.

    python tests/golden/make_fp64.py [spp [view ...]]     (c5v0 only when named)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import convergence as CV  # noqa: E402
import oracle_lib as OL  # noqa: E402

C = OL.C
S = OL.PKG.scenes


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 8192
    names = sys.argv[2:] if len(sys.argv) > 2 else None
    f64 = OL.load_fp64()
    nthreads = os.cpu_count() or 1
    for name, sc in S.rmse_views(names=names or None):
        st = sc.tracer.settings
        st.free_flight = C.FREE_FLIGHT_DELTA
        st.mis = C.MIS_FULL
        st.stratify = 0          # independent random draws: every pixel converges on its own
        st.majorant_brick = 2
        st.seed = 0x5EED64
        h = OL.SceneHandle(f64, sc)
        t0 = time.time()
        half = spp // 2
        a = h.render_sum(half, view=7, first=0, nthreads=nthreads)
        b = h.render_sum(half, view=7, first=half, nthreads=nthreads)
        h.close()
        e = float(sc.tracer.camera.exposure)
        d = CV.tonemap_rgb(a / half, e) - CV.tonemap_rgb(b / half, e)
        noise2 = float(np.mean(d * d)) / 4.0
        mean = (a + b) / (2 * half)
        np.savez_compressed(os.path.join(HERE, f"fp64_{name}.npz"), mean_xyz=mean[..., :3].astype(np.float64),
                            alpha=mean[..., 3].astype(np.float64), exposure=np.float64(e), noise2=np.float64(noise2),
                            spp=np.int64(2 * half), seconds=np.float64(time.time() - t0))
        print(f"{name}: {2 * half} spp, reference noise {np.sqrt(noise2):.2e}, {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main()
