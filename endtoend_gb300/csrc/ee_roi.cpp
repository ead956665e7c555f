// ee_roi.cpp -- reduction of sparse beamlet columns to ROI row blocks
// (dosecalc-beamlet with the header's `reduce` flag), host code as in the
// reference, whose sparsify workers run it on the CPU after each column
// comes back from the GPU.
//
// Restates _reduce_by_roi (CCCS/DoseCalcIO/sparse_io.cpp:62-158): a column's
// rows are kept only where the voxel lies in an ROI; the ROIs form row blocks
// in list order, and a kept row's key is the block's first row plus the
// voxel's position among the ROI's masked voxels, counted over the ROI's crop
// box with x slowest and z fastest (the reference's loop order, :107-112).  A
// voxel in several ROIs gives one row in each block.  The reference looks
// every masked voxel up in a dense copy of the column; here each ROI's
// positions are tabulated once (ee_roi_list_create) and the column's entries
// are looked up instead, then sorted by key, which gives the same rows in the
// same order.
#include <algorithm>
#include <cstring>
#include <utility>
#include <vector>

#include "../../include/ee_cccs.h"

int ee_internal_fail(int code, const char* msg);

struct ee_roi_list {
    int size[3] = {0, 0, 0};
    struct Roi {
        int c0[3], cn[3];
        std::vector<int> pos;  // crop-box voxel (x fastest) -> position among masked voxels, or -1
        long long count = 0;
    };
    std::vector<Roi> rois;
};

extern "C" {

int ee_roi_list_create(const int size[3], const ee_roi_mask* rois, int nrois, ee_roi_list** out) {
    if (!size || !out || nrois < 0 || (nrois > 0 && !rois)) return ee_internal_fail(EE_ERR_INVALID_ARG, "null argument");
    for (int a = 0; a < 3; a++)
        if (size[a] <= 0) return ee_internal_fail(EE_ERR_INVALID_ARG, "volume size must be positive");
    ee_roi_list* L = new ee_roi_list();
    std::memcpy(L->size, size, sizeof(L->size));
    L->rois.resize(nrois);
    for (int r = 0; r < nrois; r++) {
        const ee_roi_mask& m = rois[r];
        auto& R = L->rois[r];
        for (int a = 0; a < 3; a++) {
            R.c0[a] = m.crop_start[a];
            R.cn[a] = m.crop_size[a];
            if (m.crop_start[a] < 0 || m.crop_size[a] <= 0 || m.crop_start[a] + m.crop_size[a] > size[a] || !m.mask) {
                delete L;
                return ee_internal_fail(EE_ERR_INVALID_ARG, "ROI crop box outside the volume, or no mask");
            }
        }
        const int cx = R.cn[0], cy = R.cn[1], cz = R.cn[2];
        R.pos.assign((size_t)cx * cy * cz, -1);
        long long e = 0;
        for (int i = 0; i < cx; i++)
            for (int j = 0; j < cy; j++)
                for (int k = 0; k < cz; k++) {
                    const size_t ck = ((size_t)k * cy + j) * cx + i;
                    if (m.mask[ck]) R.pos[ck] = (int)e++;
                }
        R.count = e;
    }
    *out = L;
    return EE_OK;
}

int ee_roi_list_capacities(const ee_roi_list* L, long long* capacities) {
    if (!L || !capacities) return ee_internal_fail(EE_ERR_INVALID_ARG, "null argument");
    for (size_t r = 0; r < L->rois.size(); r++) capacities[r] = L->rois[r].count;
    return EE_OK;
}

int ee_roi_reduce(const ee_roi_list* L, const int* row_index, const float* values, long long n,
                  unsigned long long* out_keys, float* out_values, long long capacity, long long* out_n,
                  long long* row_block_sizes) {
    if (!L || !out_n || (n > 0 && (!row_index || !values)) || n < 0)
        return ee_internal_fail(EE_ERR_INVALID_ARG, "null argument");
    const long long nvox = (long long)L->size[0] * L->size[1] * L->size[2];
    const int nx = L->size[0], ny = L->size[1];
    std::vector<std::pair<unsigned long long, float>> block;
    long long mark = 0, m = 0;
    for (size_t r = 0; r < L->rois.size(); r++) {
        const auto& R = L->rois[r];
        block.clear();
        for (long long e = 0; e < n; e++) {
            const long long key = row_index[e];
            if (key < 0 || key >= nvox) return ee_internal_fail(EE_ERR_INVALID_ARG, "row index outside the volume");
            if (values[e] == 0.f) continue;  // the reference keeps non-zero dose only (:128)
            const int x = (int)(key % nx), y = (int)((key / nx) % ny), z = (int)(key / ((long long)nx * ny));
            const int i = x - R.c0[0], j = y - R.c0[1], k = z - R.c0[2];
            if (i < 0 || j < 0 || k < 0 || i >= R.cn[0] || j >= R.cn[1] || k >= R.cn[2]) continue;
            const int p = R.pos[((size_t)k * R.cn[1] + j) * R.cn[0] + i];
            if (p >= 0) block.emplace_back((unsigned long long)(mark + p), values[e]);
        }
        std::sort(block.begin(), block.end(),
                  [](const std::pair<unsigned long long, float>& a, const std::pair<unsigned long long, float>& b) {
                      return a.first < b.first;
                  });
        if (row_block_sizes) row_block_sizes[r] = (long long)block.size();
        for (const auto& kv : block) {
            if (m < capacity && out_keys && out_values) {
                out_keys[m] = kv.first;
                out_values[m] = kv.second;
            }
            m++;
        }
        mark += R.count;
    }
    *out_n = m;
    if (m > capacity) return ee_internal_fail(EE_ERR_CAPACITY, "output capacity too small for the reduced column");
    return EE_OK;
}

int ee_roi_list_destroy(ee_roi_list* L) {
    delete L;
    return EE_OK;
}

}  // extern "C"
