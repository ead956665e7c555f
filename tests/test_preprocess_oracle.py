"""Preprocessing restatements in the oracle (CPU): the reference's own
known-answer vectors for the aperture-ready fill
(CCCS/unit_tests/fmap_post_apertureready.cpp:9-34), the HU -> density table
arithmetic, and a projection sanity check."""
import numpy as np

from endtoend_gb300 import inputs
from oracle import oracle


def test_aperture_ready_reference_vectors():
    f = np.array([[1, 0, 1], [0, 1, 0], [1, 1, 0]], np.float32)
    np.testing.assert_array_equal(oracle.aperture_ready(f), [[1, 1, 1], [0, 1, 0], [1, 1, 0]])
    f = np.array([[1, 0, 1, 0, 1], [1, 0, 0, 1, 0], [0, 0, 1, 0, 1]], np.float32)
    np.testing.assert_array_equal(oracle.aperture_ready(f), [[1, 1, 1, 1, 1], [1, 1, 1, 1, 0], [0, 0, 1, 1, 1]])


def test_lut_and_linear_rule_on_a_uniform_ct():
    lut = ([-969.8, -5.6, 1173.7], [0.0, 1.0, 1.823])
    for hu_val, want in [(-2000.0, 0.0), (-5.6, 1.0), (500.0, 1.0 + (505.6) * 0.823 / 1179.3),
                         (2000.0, 1.0 + 2005.6 * 0.823 / 1179.3)]:
        hu = np.full((8, 8, 8), hu_val, np.float32)
        d = oracle.ct_to_density(hu, (0.25, 0.25, 0.25), 0.25, lut=lut)
        np.testing.assert_allclose(d[2:6, 2:6, 2:6], want, rtol=1e-5, atol=1e-6)
    hu = np.full((8, 8, 8), -1024.0 + 512.0, np.float32)
    d = oracle.ct_to_density(hu, (0.25, 0.25, 0.25), 0.25, lut=None)
    np.testing.assert_allclose(d[2:6, 2:6, 2:6], 0.5, rtol=1e-6)
    hu[:] = -3000.0
    np.testing.assert_allclose(oracle.ct_to_density(hu, (0.25,) * 3, 0.25, lut=None)[3, 3, 3], 0.05, rtol=1e-6)


def test_projection_of_a_sphere_is_a_disc():
    vol = inputs.head_neck_phantom(shape=(40, 40, 40), voxel_cm=0.25, seed=1)
    mask = inputs.Volume(density=vol.masks["PTV"].astype(np.float32), voxel=vol.voxel, start=vol.start,
                         bbox_start=vol.bbox_start, bbox_size=vol.bbox_size)
    b = inputs.single_beam(fmap=(20, 20), beamlet_cm=0.5, gantry_deg=35.0, couch_deg=10.0)
    f = oracle.fluence_projection(mask, b)
    # PTV radius 2.5 cm at the isocentre: about a 5 cm disc of 0.5 cm pixels
    n = f.sum()
    assert 60 <= n <= 130, n
    yy, xx = np.nonzero(f)
    assert abs(xx.mean() - 9.5) < 1.0 and abs(yy.mean() - 9.5) < 1.0
