"""Error metrics of a radiance image against a float64 evaluation.

Per pixel, the relative error over RGB is |k - o| / max(|o|, floor) with
floor = 1e-6 * max|o| over the image; pixels whose reference value is NaN (sky,
untouched) are skipped.

The float64 reference is normally evaluated with the kernel's own branch decisions at
the cuts of pbr_direct_light (range, NdL == 0, radiance < 0.002; oracle.shade_forced
with the pairs hl_set_pair_log recorded), so every pixel is compared; ``flips`` then
counts the pixels where a decision differs from the float64 one, as information.
Given per-pixel full-evaluation counts instead, pixels whose counts differ are
reported as flips and left out of the statistics."""
from __future__ import annotations

import numpy as np


def radiance_error(kernel: np.ndarray, ref: np.ndarray, kernel_full=None, ref_full=None, floor_rel: float = 1e-6,
                   flip_pixels=None):
    """flip_pixels: per-pixel counts of differing branch decisions of a forced-branch
    reference (counted; every pixel is compared)."""
    k = np.asarray(kernel, np.float64)[..., :3]
    o = np.asarray(ref, np.float64)[..., :3]
    valid = ~np.isnan(o[..., 0])
    flips = np.zeros(valid.shape, bool)
    use = valid
    if flip_pixels is not None:
        flips = (np.asarray(flip_pixels) != 0) & valid
    elif kernel_full is not None and ref_full is not None:
        flips = (np.asarray(kernel_full) != np.asarray(ref_full)) & valid
        use = valid & ~flips
    if not use.any():
        return dict(max=0.0, p9999=0.0, mean=0.0, n=0, flips=int(flips.sum()), n_over_1e5=0, n_over_2e3=0)
    mx = float(np.abs(o[use]).max())
    floor = max(floor_rel * mx, 1e-30)
    den = np.maximum(np.abs(o[use]), floor)
    r = (np.abs(k[use] - o[use]) / den).max(-1)
    return dict(
        max=float(r.max()),
        p9999=float(np.quantile(r, 0.9999)),
        mean=float(r.mean()),
        n=int(use.sum()),
        flips=int(flips.sum()),
        n_over_1e5=int((r > 1e-5).sum()),
        n_over_2e3=int((r > 2e-3).sum()),
    )
