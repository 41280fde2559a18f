"""Image RMSE against the converged FP64 references of tests/golden/fp64_*.npz
(measurement infrastructure of the tests and of bench.py).

RMSE is taken over the tone-mapped linear RGB of every pixel and channel
(XYZ -> RGB and 1 - exp(-c / exposure), clamped to [0, 1], the arithmetic of
the tone map, Source/tonemap.cuh:30-59), before 8-bit quantisation.  The
reference's own noise (estimated at generation from two independent halves)
is subtracted in quadrature."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
XYZ_TO_RGB = np.array([[3.240479, -1.537150, -0.498535],
                       [-0.969256, 1.875991, 0.041556],
                       [0.055648, -0.204043, 1.057311]])


def tonemap_rgb(xyz: np.ndarray, exposure: float = 1.0) -> np.ndarray:
    rgb = np.asarray(xyz, dtype=np.float64)[..., :3] @ XYZ_TO_RGB.T
    return np.clip(1.0 - np.exp(-rgb / exposure), 0.0, 1.0)


def load_reference(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, f"fp64_{name}.npz"))
    return {k: z[k] for k in z.files}


def rmse(mean_xyz: np.ndarray, ref: dict) -> float:
    """noise-corrected RMSE of an image estimate (mean XYZ per pixel)"""
    e = float(ref["exposure"])
    d = tonemap_rgb(mean_xyz, e) - tonemap_rgb(ref["mean_xyz"], e)
    mse = float(np.mean(d * d)) - float(ref["noise2"])
    return float(np.sqrt(max(mse, 0.0)))


def spp_to_rmse(spp_list, rmse_list, target=1e-2):
    """samples per pixel at which the RMSE curve reaches `target`:
    log-log interpolation between the bracketing measurements (RMSE ~
    spp^-1/2 between them); None if the last measurement is above it."""
    for i, (n, r) in enumerate(zip(spp_list, rmse_list)):
        if r <= target:
            if i == 0:
                return float(n) * (r / target) ** 2
            n0, r0 = spp_list[i - 1], rmse_list[i - 1]
            if r0 <= r:
                return float(n)
            a = np.log(r / r0) / np.log(n / n0)
            return float(n0 * np.exp(np.log(target / r0) / a))
    return None
