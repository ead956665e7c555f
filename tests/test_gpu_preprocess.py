"""GPU preprocessing (ee_ct_to_density, ee_fluence_projection) against the
oracle's restatement of dosecalc-preprocess (texture weights emulated)."""
import numpy as np
import pytest

from endtoend_gb300 import engine, inputs
from oracle import oracle

pytestmark = pytest.mark.gpu


def _ct(seed=3):
    rng = np.random.default_rng(seed)
    vol = inputs.head_neck_phantom(shape=(37, 33, 29), voxel_cm=0.3, seed=seed)
    # density -> a HU-like image with noise, anisotropic voxels
    hu = (vol.density * 1000.0 - 1000.0 + rng.normal(0, 30, vol.density.shape)).astype(np.float32)
    return hu, (0.3, 0.27, 0.33)


@pytest.mark.parametrize("lut", [engine.SIEMENS_LUT, None])
def test_ct_to_density_matches_oracle(lut):
    hu, vox = _ct()
    got = engine.ct_to_density(hu, vox, 0.2, lut=lut)
    ref = oracle.ct_to_density(hu, vox, 0.2, lut=lut, tex_emulate=1)
    assert got.shape == ref.shape
    # The texture unit filters with 8-bit weights, which the oracle emulates
    # by rounding; on GB300 the result still moves by about one weight step
    # where neighbouring CT values differ by ~2000 HU (air / bone next to
    # tissue): up to ~8 HU, 0.01 g/cc on the steep low-density part of the
    # table.  Elsewhere the two agree to 1e-5.
    d = np.abs(got - ref)
    print("max", d.max(), "p99.9", np.quantile(d, 0.999), "median", np.median(d))
    assert d.max() <= 1.5e-2, d.max()
    assert np.quantile(d, 0.999) <= 6e-3, np.quantile(d, 0.999)
    assert np.median(d) <= 1e-4, np.median(d)


def test_fluence_projection_matches_oracle():
    vol = inputs.head_neck_phantom(shape=(48, 44, 40), voxel_cm=0.25, seed=1, with_oars=True)
    mask = inputs.Volume(density=(vol.masks["PTV"] | vol.masks["OAR0"]).astype(np.float32), voxel=vol.voxel,
                         start=vol.start, bbox_start=vol.bbox_start, bbox_size=vol.bbox_size)
    beams = [inputs.single_beam(fmap=(24, 20), beamlet_cm=0.5, gantry_deg=g, couch_deg=c)
             for g, c in [(0.0, 0.0), (47.0, 15.0), (200.0, -30.0), (300.0, 70.0)]]
    got = engine.fluence_projection(mask, beams, supersample=True)
    for b, g in zip(beams, got):
        ref = oracle.fluence_projection(mask, b, supersample=True)
        # binary maps: pixels whose sub-rays only graze the mask may flip with rounding
        assert (g != ref).sum() <= max(2, int(0.01 * ref.size)), (g != ref).sum()
        assert ref.sum() > 0
    ap = engine.fluence_projection(mask, beams, supersample=False, aperture_ready=True)
    for b, a in zip(beams, ap):
        ref = oracle.aperture_ready(oracle.fluence_projection(mask, b, supersample=False))
        assert (a != ref).sum() <= max(2, int(0.01 * ref.size))
