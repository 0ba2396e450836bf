"""Error metrics of a radiance image against a float64 evaluation.

Per pixel, the relative error over RGB is |k - o| / max(|o|, floor) with
floor = 1e-6 * max|o| over the image; pixels whose reference value is NaN (sky,
untouched) are skipped. ``flip`` pixels are those where the two evaluations took a
different branch at a cut (counted from per-pixel full-evaluation counts when
given) and are reported separately."""
from __future__ import annotations

import numpy as np


def radiance_error(kernel: np.ndarray, ref: np.ndarray, kernel_full=None, ref_full=None, floor_rel: float = 1e-6):
    k = np.asarray(kernel, np.float64)[..., :3]
    o = np.asarray(ref, np.float64)[..., :3]
    valid = ~np.isnan(o[..., 0])
    flips = np.zeros(valid.shape, bool)
    if kernel_full is not None and ref_full is not None:
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
