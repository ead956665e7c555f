"""CPU restatement of the reference's ROI reduction of a sparse dose column
(test infrastructure only: tests/ may import it; the engine never does).

reduce_by_roi follows _reduce_by_roi, CCCS/DoseCalcIO/sparse_io.cpp:62-158,
loop for loop: the column is expanded into a dense vector over the full
volume (:80-84), then for every ROI in list order its crop box is walked with
x outermost and z innermost (:107-112), every masked voxel advances the ROI's
element counter, and a masked voxel with non-zero dose emits the key
mark + element counter (:126-134); mark advances by the ROI's masked voxel
count (:147).  Pure Python loops: for the small cases of the tests.
"""
from __future__ import annotations

import numpy as np


def reduce_by_roi(keys, vals, size_xyz, rois):
    """keys/vals: one sparse column (full-volume linear keys, x fastest).
    rois: list of (crop_start xyz, mask [nz][ny][nx] of the crop box).
    Returns (keys uint64, vals float32, row_block_sizes)."""
    nx, ny, nz = (int(v) for v in size_xyz)
    sparsevect = np.zeros(nx * ny * nz, np.float32)
    for k, v in zip(keys, vals):
        sparsevect[int(k)] = v
    out_k, out_v, blocks = [], [], []
    mark = 0
    for c0, mask in rois:
        mz, my, mx = mask.shape
        flat = np.ascontiguousarray(mask).ravel()
        nkept = 0
        elem = 0
        for ii in range(mx):
            for jj in range(my):
                for kk in range(mz):
                    crop_key = (kk * my + jj) * mx + ii
                    orig_key = ((kk + c0[2]) * ny + (jj + c0[1])) * nx + (ii + c0[0])
                    if flat[crop_key]:
                        d = sparsevect[orig_key]
                        if d:
                            out_k.append(mark + elem)
                            out_v.append(d)
                            nkept += 1
                        elem += 1
        mark += elem
        blocks.append(nkept)
    return np.array(out_k, np.uint64), np.array(out_v, np.float32), np.array(blocks, np.int64)
