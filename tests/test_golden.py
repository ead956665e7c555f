"""The oracle against golden outputs of the reference's own dosecalc-beam
kernel source (cudaSiddon, cudaRaytrace, RowConvolve, REV2XYZdose compiled
unmodified and run on the CPU; see tests/golden/make_golden.py), with and
without TERMA supersampling (fixtures *_ss<k>: ss_factor k).  With
supersampling a few sub-voxel samples per fixture sit within FP32 rounding of
a beamlet edge and the reference's arithmetic decides them; the fixtures store
the reference's own change under 1e-6 .. 1e-5 cm isocentre shifts (dose,
TERMA), which is added to the bounds below.

Tolerances: crop boxes identical; TERMA within 1e-4 of its maximum in
99.9 % of voxels and within 2e-3 everywhere (FP32 vs FP64 can resolve a
near-tie between Siddon plane crossings differently at density interfaces);
dose within 6e-4 of Dmax (the reference is FP32, the oracle FP64; both
filter with 8-bit texture weights, so last-bit differences in a texel
coordinate can move a weight by 1/256)."""
import numpy as np
import pytest

import golden_cases
from oracle.oracle import Oracle


@pytest.mark.parametrize("name", golden_cases.names())
def test_oracle_matches_reference_kernels(name):
    vol, phys, beams, doses, termas, bevs = golden_cases.load(name)
    o = Oracle(vol, phys, kernel_mode=0, tex_emulate=True, ss_factor=golden_cases.ss_factor(name))
    for b, dref, tref, bev, (dn, tn) in zip(beams, doses, termas, bevs, golden_cases.ref_noise(name)):
        d, info, t = o.beam_dose(b, return_terma=True)
        assert list(info.bev_size) == bev
        rel = np.abs(t - tref) / tref.max()
        assert np.mean(rel > 1e-4) <= 1e-3 and rel.max() <= 2e-3 + tn
        assert np.abs(d - dref).max() <= (6e-4 + dn) * dref.max(), np.abs(d - dref).max() / dref.max()


def test_golden_fixtures_reproduce_from_reference_source():
    """When the reference checkout is present, the harness regenerates the
    committed fixtures."""
    from oracle import ref_harness
    if not ref_harness.available():
        pytest.skip("reference checkout not present")
    vol, phys, beams, doses, _, _ = golden_cases.load("slab32")
    d, _, _ = ref_harness.ReferenceHarness(vol, phys, tex_emulate=True).beam_dose(beams[1])
    assert np.abs(d - doses[1]).max() <= 1e-6 * doses[1].max()


def test_beamlet_cfg4_fixture_matches_its_problem():
    """The config-4 beamlet fixture describes the problem that
    golden_cases.cfg4_problem builds: same phantom (density digest), the 8
    beams' active beamlets, 200 columns, and per-column summaries that are
    consistent (top entries and block sums within the column maximum, the
    reference's change non-negative)."""
    vol, phys, beams, ke, max_rev, thresh, z = golden_cases.load_cfg4()
    assert int(z["nbeams"]) == len(beams) == 8
    ncol = 0
    for k, b in enumerate(beams):
        idx = z[f"beam{k}_beamlet_index"]
        np.testing.assert_array_equal(idx, np.flatnonzero(b.fluence.ravel() > 0))
        mx, noise = z[f"beam{k}_max"], z[f"beam{k}_ref_noise"]
        assert len(mx) == len(idx) == len(noise) and (mx > 0).all() and (noise >= 0).all()
        tv, tp = z[f"beam{k}_top_val"], z[f"beam{k}_top_key_ptr"]
        bs, bp = z[f"beam{k}_blk_sum"], z[f"beam{k}_blk_key_ptr"]
        assert len(tp) == len(bp) == len(idx) + 1
        for c in range(len(idx)):
            top = tv[tp[c]:tp[c + 1]]
            assert 0 < len(top) <= golden_cases.CFG4_TOP
            assert abs(top.max() - mx[c]) <= 1e-6 * mx[c]
            assert bs[bp[c]:bp[c + 1]].sum() <= z[f"beam{k}_sum"][c] * (1 + 1e-6)
        ncol += len(idx)
    assert ncol == 200 and ke == 2.0 and thresh == 1e-4
