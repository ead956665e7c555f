"""CPU tests of the oracle (the parity checker) and of the host geometry.

* the O(L) recurrence equals the reference walk with an exact
  double-exponential kernel (same discrete operator);
* the oracle's adjoint is the transpose of its forward (dot-product test);
* the angle -> direction -> angle round trip of the reference's own unit
  test CCCS/unit_tests/beam.cpp:16-67, for the oracle geometry and for the
  engine's host geometry (ee_beam_source, no GPU needed).
"""
import math

import numpy as np
import pytest

from endtoend_gb300 import inputs
from oracle.oracle import Oracle, rotate


@pytest.fixture(scope="module")
def small():
    vol = inputs.slab_phantom(24, 0.25)
    phys = inputs.make_physics(seed=0, spacing_cm=0.25)
    return vol, phys


def test_recurrence_equals_walk_rows(small):
    vol, phys = small
    rng = np.random.default_rng(0)
    o1 = Oracle(vol, phys, kernel_mode=1)
    o2 = Oracle(vol, phys, kernel_mode=2)
    for trial in range(20):
        L = int(rng.integers(1, 200))
        dens = rng.uniform(0.001, 2.0, L)
        # sentinel runs at both ends (outside BEV box / calc bbox)
        a, b = sorted(rng.integers(0, L + 1, 2))
        dens[:a] = -3.0
        dens[b:] = -2.0
        terma = rng.uniform(0, 1, L) * (dens >= 0)
        P = int(rng.integers(0, phys.ntheta // 2))
        d1 = o1.row_convolve(dens, terma, P)
        d2 = o2.row_convolve(dens, terma, P)
        assert np.allclose(d1, d2, rtol=1e-10, atol=1e-14), (trial, np.abs(d1 - d2).max())


@pytest.mark.parametrize("mode", [0, 2])
def test_row_adjoint_dot_product(small, mode):
    vol, phys = small
    o = Oracle(vol, phys, kernel_mode=mode)
    rng = np.random.default_rng(1)
    for _ in range(10):
        L = int(rng.integers(2, 150))
        dens = rng.uniform(0.01, 2.0, L)
        dens[: int(rng.integers(0, 5))] = -3.0
        t = rng.standard_normal(L) * (dens >= 0)
        g = rng.standard_normal(L)
        P = int(rng.integers(0, phys.ntheta // 2))
        lhs = np.dot(o.row_convolve(dens, t, P), g)
        rhs = np.dot(t, o.row_convolve_T(dens, g, P))
        assert abs(lhs - rhs) <= 1e-10 * (abs(lhs) + 1e-30), (lhs, rhs)


@pytest.mark.parametrize("mode", [0, 2])
def test_beam_adjoint_dot_product(mode):
    vol = inputs.slab_phantom(20, 0.25)
    phys = inputs.make_physics(seed=0, spacing_cm=0.25)
    beam = inputs.single_beam(fmap=(6, 6), beamlet_cm=0.5, gantry_deg=30.0, couch_deg=20.0)
    rng = np.random.default_rng(2)
    beam.fluence = rng.uniform(0.2, 1.0, beam.fluence.shape).astype(np.float32)
    o = Oracle(vol, phys, kernel_mode=mode)
    dose, _ = o.beam_dose(beam)
    g = rng.standard_normal(dose.shape)
    fg, _ = o.beam_dose_adjoint(beam, g)
    lhs = float(np.sum(dose * g))
    rhs = float(np.sum(fg * beam.fluence.astype(np.float64)))
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs), (lhs, rhs)


def _angles_from_dir(d):
    """BEAM::calc_angles_from_dir (CCCS/DoseCalcIO/beam.cpp:98-113)."""
    eps = 1e-6
    close = lambda a, b: abs(b - a) <= 1e-6
    nd = -np.asarray(d) / np.linalg.norm(d)
    theta = math.acos(-nd[1])
    phi = math.atan(nd[2] / nd[0]) if nd[0] != 0 else math.copysign(math.pi / 2, nd[2])
    if close(nd[2], 0.0):
        phi = 0.0
    elif close(nd[0], 0.0):
        phi = math.pi / 2
    if close(nd[0], 0.0) and close(nd[2], 0.0):
        theta = 0.0 if nd[1] <= -eps else math.pi
    elif nd[0] < -eps or (close(nd[0], 0.0) and nd[2] < -eps):
        theta *= -1
    return theta, phi


def _dir_oracle(g, c):
    a = math.fmod(g, 2 * math.pi)
    z = math.fmod(c, 2 * math.pi)
    if abs(z) > 1e-6 and (abs(a) <= 1e-6 or abs(a - math.pi) <= 1e-6):
        z = 0.0
    src = rotate(1, [0.0, -100.0, 0.0], a, z, 0.0)
    d = -src
    return d / np.linalg.norm(d)


def _kat_angles():
    # the reference's test set: 12 coplanar + 12x12 non-coplanar (degrees)
    out = [(45.0 * i, 0.0) for i in range(12)]
    out += [(45.0 * i, 45.0 * j) for j in range(12) for i in range(12)]
    return out


def test_geometry_roundtrip_kat_oracle():
    for g, c in _kat_angles():
        d1 = _dir_oracle(math.radians(g), math.radians(c))
        th, ph = _angles_from_dir(d1)
        d3 = _dir_oracle(th, ph)
        assert np.all(np.abs(d1 - d3) <= 1e-6 * 10), (g, c, d1, d3)


def test_geometry_roundtrip_kat_engine_host():
    from endtoend_gb300 import engine
    engine.load_library(build_if_missing=True)
    for g, c in _kat_angles():
        b = inputs.single_beam(gantry_deg=g, couch_deg=c)
        _, d1 = engine.beam_source(b)
        th, ph = _angles_from_dir(d1)
        b3 = inputs.single_beam()
        b3.azimuth, b3.zenith = th, ph
        _, d3 = engine.beam_source(b3)
        # float32 host geometry: the reference's closeto tolerance is 1e-6
        assert np.all(np.abs(d1 - d3) <= 2e-6), (g, c, d1, d3)
        # engine host geometry agrees with the oracle's restatement
        assert np.allclose(d1, _dir_oracle(b.azimuth, b.zenith), atol=1e-6)


def test_table_matches_exponential_within_half_percent():
    """The reference's 24-radius cumulative table vs the exact double
    exponential on config-0 sizes: the kernel-discretisation part of the
    engine-vs-reference difference."""
    vol, phys, beams = inputs.config0()
    d0, _ = Oracle(vol, phys, kernel_mode=0).beam_dose(beams[0])
    d2, _ = Oracle(vol, phys, kernel_mode=2).beam_dose(beams[0])
    rel = np.abs(d2 - d0).max() / d0.max()
    assert rel < 5e-3, rel
