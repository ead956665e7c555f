"""Dose-comparison metrics: max |difference| / Dmax and the global gamma
index pass rate (Low et al. 1998) with sub-voxel search of the evaluated
distribution."""
from __future__ import annotations

import numpy as np


def max_rel_diff(dose: np.ndarray, ref: np.ndarray) -> float:
    return float(np.abs(dose.astype(np.float64) - ref).max() / np.abs(ref).max())


def gamma_pass_rate(evaluated: np.ndarray, reference: np.ndarray, voxel_mm, dose_tol: float = 0.01,
                    dist_mm: float = 1.0, threshold: float = 0.10, step_mm: float = 0.25) -> float:
    """Fraction of reference voxels with dose >= threshold*Dmax whose global
    gamma (dose_tol * Dmax, dist_mm) is <= 1.  The evaluated distribution is
    sampled by trilinear interpolation on a step_mm grid within dist_mm."""
    from scipy.ndimage import map_coordinates

    ref = np.asarray(reference, np.float64)
    ev = np.asarray(evaluated, np.float64)
    vox = np.broadcast_to(np.asarray(voxel_mm, np.float64), (3,))  # (x, y, z) mm
    dmax = ref.max()
    mask = ref >= threshold * dmax
    idx = np.nonzero(mask)  # (z, y, x)
    if idx[0].size == 0:
        return 1.0
    base = np.stack([idx[0], idx[1], idx[2]]).astype(np.float64)
    dref = ref[idx]
    best = ((ev[idx] - dref) / (dose_tol * dmax)) ** 2
    n = int(np.floor(dist_mm / step_mm))
    offs = np.arange(-n, n + 1) * step_mm
    for oz in offs:
        for oy in offs:
            for ox in offs:
                r2 = (ox * ox + oy * oy + oz * oz) / (dist_mm * dist_mm)
                if r2 == 0 or r2 > 1.0:
                    continue
                coords = base + np.array([[oz / vox[2]], [oy / vox[1]], [ox / vox[0]]])
                e = map_coordinates(ev, coords, order=1, mode="nearest")
                g2 = ((e - dref) / (dose_tol * dmax)) ** 2 + r2
                np.minimum(best, g2, out=best)
    return float(np.mean(best <= 1.0))
