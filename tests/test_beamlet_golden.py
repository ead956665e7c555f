"""The beamlet-column fixtures (CPU): their CSR structure follows the
reference's sparsification (CCCS/DoseCalcIO/sparse_io.cpp:22-59), and -- where
the reference checkout is present -- the reference's own dosecalc-beamlet
kernels, run on the CPU by oracle/ref_harness, reproduce them."""
import numpy as np
import pytest

import golden_cases


@pytest.mark.parametrize("name", golden_cases.beamlet_names())
def test_fixture_structure(name):
    vol, phys, beam, ke, max_rev, thresh, ref = golden_cases.load_beamlet(name)
    cp, rows, vals = ref["col_ptr"], ref["row_index"], ref["value"]
    assert len(ref["beamlet_index"]) == int((beam.fluence.ravel() > 0).sum())
    assert cp[0] == 0 and cp[-1] == len(rows) == len(vals)
    for c in range(len(cp) - 1):
        r, v = rows[cp[c]:cp[c + 1]], vals[cp[c]:cp[c + 1]]
        assert len(r) > 0 and np.all(np.diff(r) > 0)
        assert np.all(v > np.float32(thresh) * v.max())


def test_harness_reproduces_fixture():
    from oracle import ref_harness
    if not ref_harness.available():
        pytest.skip("reference checkout not present")
    name = "bl_headneck40"
    vol, phys, beam, ke, max_rev, thresh, ref = golden_cases.load_beamlet(name)
    h = ref_harness.BeamletHarness(vol, phys, tex_emulate=True)
    idx, cols, info = h.columns(beam, kernel_extent=ke, max_rev_size=max_rev)
    np.testing.assert_array_equal(idx, ref["beamlet_index"])
    for c in range(len(idx)):
        k, v = ref_harness.sparsify(cols[c], thresh, vol.bbox_start, vol.size)
        a, b = int(ref["col_ptr"][c]), int(ref["col_ptr"][c + 1])
        np.testing.assert_array_equal(k, ref["row_index"][a:b])
        np.testing.assert_allclose(v, ref["value"][a:b], rtol=1e-5, atol=0)
