"""Beamlet coefficients at the stated size: 200 beamlets (8 beams x 25) of
40x40 maps of 2.5 mm on the 200x200x160 head-and-neck phantom at 2 mm, kernel
extent 2 cm, threshold 1e-4 of each column's maximum, against the
reference's dosecalc-beamlet kernels (CCCS/dosecalc-beamlet/
nvbbRayConvolve_device.cu, sparsified as CCCS/DoseCalcIO/sparse_io.cpp:22-59)
through the fixture tests/golden/beamlet_cfg4 (per-column summaries).

Every column: maximum and sums over 8^3-voxel blocks within 0.5 % of the
column maximum (of the largest block sum) plus the reference's own change
under twelve rounding-level moves (1e-5 and 1e-6) of the isocentre and the
REV lattice; entry counts within 5 %.  The reference's 128 largest entries,
voxel by voxel: within the same tolerance in at least 98 % of the columns,
within 1.5 % of the column maximum plus the reference's change in all, and
a median error below 0.1 %.  The allowance covers compact clusters of a few
voxels where a discrete decision at an exact tie goes the other way: which
beamlet a REV sample on a beamlet boundary belongs to is decided in FP64
here and in FP32 by the reference, and an FP32 build of that one test
brings one such column (0.89 % against 0.88 % allowed) inside the
per-column tolerance.
"""
import numpy as np
import pytest

import golden_cases
from endtoend_gb300 import engine

pytestmark = pytest.mark.gpu

COLUMN_TOL = 0.005
ENTRY_ALL = 0.015      # every column's top entries: of the column maximum, plus the reference's change
ENTRY_SHARE = 0.98     # share of columns whose top entries meet the per-column tolerance


def test_beamlet_columns_200_vs_reference():
    vol, phys, beams, ke, max_rev, thresh, z = golden_cases.load_cfg4()
    worst = {"max": 0.0, "top": 0.0, "blocks": 0.0, "nnz": 0.0}
    ncol = 0
    tops, outliers = [], []
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="table")
        e.set_beamlet_options(ke, max_rev)
        for k, b in enumerate(beams):
            bidx, cp, rows, vals = e.beamlet_columns(b, thresh)
            np.testing.assert_array_equal(bidx, z[f"beam{k}_beamlet_index"])
            noise = z[f"beam{k}_ref_noise"]
            for c in range(len(bidx)):
                a, bb = int(cp[c]), int(cp[c + 1])
                rk, rv = rows[a:bb].astype(np.int64), vals[a:bb].astype(np.float64)
                mx, sm, nnz, _, _, bkeys, bsums = golden_cases.column_summary(rk, rv, vol.size)
                rmax = float(z[f"beam{k}_max"][c])
                tol = COLUMN_TOL + float(noise[c])
                e_max = abs(mx - rmax) / rmax
                # the reference's largest entries, looked up in the engine's column
                t0, t1 = z[f"beam{k}_top_key_ptr"][c:c + 2]
                tk, tv = z[f"beam{k}_top_key"][t0:t1], z[f"beam{k}_top_val"][t0:t1]
                pos = np.searchsorted(rk, tk)
                hit = (pos < len(rk)) & (rk[np.minimum(pos, len(rk) - 1)] == tk)
                ev = np.where(hit, rv[np.minimum(pos, len(rk) - 1)], 0.0)
                e_top = float(np.abs(ev - tv).max() / rmax)
                # block sums over the union of blocks
                b0, b1 = z[f"beam{k}_blk_key_ptr"][c:c + 2]
                rkeys, rsums = z[f"beam{k}_blk_key"][b0:b1], z[f"beam{k}_blk_sum"][b0:b1]
                allk = np.union1d(rkeys, bkeys)
                re = np.zeros(len(allk))
                ee = np.zeros(len(allk))
                re[np.searchsorted(allk, rkeys)] = rsums
                ee[np.searchsorted(allk, bkeys)] = bsums
                e_blk = float(np.abs(ee - re).max() / re.max())
                e_nnz = abs(nnz - int(z[f"beam{k}_nnz"][c])) / int(z[f"beam{k}_nnz"][c])
                for key, v in (("max", e_max), ("top", e_top), ("blocks", e_blk), ("nnz", e_nnz)):
                    worst[key] = max(worst[key], v)
                assert e_max <= tol and e_blk <= tol, (k, c, e_max, e_blk, noise[c])
                assert e_top <= ENTRY_ALL + float(noise[c]), (k, c, e_top, noise[c])
                tops.append(e_top)
                if e_top > tol:
                    outliers.append((k, c, round(e_top, 5), round(float(noise[c]), 5)))
                assert e_nnz <= 0.05, (k, c, nnz, int(z[f"beam{k}_nnz"][c]))
                ncol += 1
    print(f"beamlet columns: {ncol} vs the reference kernels, worst {worst}, median top-entry error "
          f"{np.median(tops):.2e}, columns past the per-column entry tolerance: {outliers}")
    assert ncol == 200
    assert len(outliers) <= (1.0 - ENTRY_SHARE) * ncol, outliers
    assert np.median(tops) < 1e-3
