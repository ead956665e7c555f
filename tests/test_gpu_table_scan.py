"""The exact O(L * nradii) evaluation of the cumulative-kernel table
(EE_KERNEL_TABLE) against the reference's step-by-step walk
(EE_KERNEL_TABLE_WALK, RowConvolve of CCCS/dosecalc-beam/
nvbbRayConvolve_device.cu:87-218) on the GPU, and against the FP64 oracle of
the same table, forward dose and adjoint (fluence gradient).

Both GPU modes share the TERMA, the REV resample, the gather and the scatter;
they differ only in how each line's sums are evaluated, so they agree to FP32
summation order: <= 1e-4 of the dose maximum (forward) and of the gradient
maximum (adjoint).  Against the FP64 oracle: <= 1e-3 (the table-mode parity
bar).  Cases: config 0, the measured 6 MV table on an oblique beam, an
oblique beam on the head-and-neck phantom, and a 20 x 960 x 20 column whose
lines run to ~950 samples (close to the 1024-sample line limit), where the
FP32 error of the exp recurrence is also pinned against FP64.
"""
import numpy as np
import pytest

import golden_cases
from endtoend_gb300 import engine, inputs
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _column():
    """20 x 960 x 20 voxels of 0.25 cm, water with a lung and a bone band
    across the long (y) axis; the gantry-0 beam runs along +y, so the axial
    cones' lines cross the whole column (the crop box, column plus penumbra,
    stays under the reference's 1000-voxel limit)."""
    ny = 960
    dens = np.ones((20, ny, 20), np.float32)
    dens[:, 300:400, :] = 0.25
    dens[:, 600:620, :] = 1.85
    voxel = 0.25
    start = -0.5 * (np.array([20, ny, 20]) - 1) * voxel + np.array([0.013, 0.0, -0.011])
    vol = inputs.Volume(density=dens, voxel=np.full(3, voxel), start=start, bbox_start=np.zeros(3, np.int64),
                        bbox_size=np.array([20, ny, 20], np.int64))
    beam = inputs.single_beam(fmap=(8, 8), beamlet_cm=0.5)
    beam.sad = 200.0
    return vol, beam


def _case(name):
    if name == "config0":
        vol, phys, beams = inputs.config0()
        return vol, phys, beams[0]
    if name == "measured6x_oblique":
        phys, _ = golden_cases.measured_physics(0.25)
        vol = inputs.slab_phantom(48, 0.25)
        return vol, phys, inputs.single_beam(fmap=(12, 10), beamlet_cm=0.5, gantry_deg=40.0, couch_deg=20.0)
    if name == "headneck_oblique":
        vol = inputs.head_neck_phantom(shape=(96, 96, 80), voxel_cm=0.2)
        phys = inputs.make_physics(seed=0, spacing_cm=0.2)
        b = inputs.single_beam(fmap=(20, 16), beamlet_cm=0.25, gantry_deg=123.0, couch_deg=-37.0, coll_deg=15.0)
        b.fluence = np.random.default_rng(5).uniform(0.0, 1.0, b.fluence.shape).astype(np.float32)
        return vol, phys, b
    if name == "column960":
        vol, beam = _column()
        return vol, inputs.make_physics(seed=0, spacing_cm=0.25), beam
    raise KeyError(name)


CASES = ["config0", "measured6x_oblique", "headneck_oblique", "column960"]


def _rel(a, ref):
    return float(np.abs(a - ref).max() / np.abs(ref).max())


@pytest.fixture(scope="module", params=CASES)
def case(request):
    vol, phys, beam = _case(request.param)
    g = np.random.default_rng(17).standard_normal(vol.density.shape).astype(np.float32)
    out = {"name": request.param, "vol": vol, "phys": phys, "beam": beam, "g": g}
    with engine.Engine(0) as e:
        e.set_volume(vol)
        for mode in ("table", "walk"):
            e.set_physics(phys, mode=mode)
            out[mode] = e.beam_dose([beam])
            out[mode + "_adj"] = e.beam_dose_adjoint([beam], g)[0]
        out["max_line"] = e.beam_info(0)["max_line"]
        e.set_mode("exp")
        out["exp"] = e.beam_dose([beam])
    return out


def test_scan_equals_walk_forward(case):
    err = _rel(case["table"], case["walk"])
    print(f"{case['name']}: table scan vs walk {err:.2e} (longest line {case['max_line']})")
    assert case["walk"].max() > 0
    assert err <= 1e-4


def test_scan_equals_walk_adjoint(case):
    err = _rel(case["table_adj"], case["walk_adj"])
    print(f"{case['name']}: adjoint table scan vs walk {err:.2e}")
    assert np.abs(case["walk_adj"]).max() > 0
    assert err <= 1e-4


def test_scan_vs_fp64_oracle(case):
    ref, _ = Oracle(case["vol"], case["phys"], kernel_mode=0).beam_dose(case["beam"])
    err = _rel(case["table"], ref)
    print(f"{case['name']}: table scan vs FP64 oracle {err:.2e}")
    assert err <= 1e-3


def test_scan_adjoint_dot_product(case):
    """<A x, g> = <x, A^T g> for the table-mode operator (FP32: rel 1e-4)."""
    x = case["beam"].fluence.astype(np.float64)
    lhs = float(np.dot(case["table"].astype(np.float64).ravel(), case["g"].astype(np.float64).ravel()))
    rhs = float(np.dot(x.ravel(), case["table_adj"].astype(np.float64).ravel()))
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), abs(rhs))


def test_long_lines_exp_recurrence_vs_fp64():
    """The exp fast path's plain FP32 recurrence on lines of ~950 samples
    against the FP64 oracle of the same operator: <= 1e-3 of Dmax."""
    vol, beam = _column()
    phys = inputs.make_physics(seed=0, spacing_cm=0.25)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        d = e.beam_dose([beam])
        L = e.beam_info(0)["max_line"]
    ref, _ = Oracle(vol, phys, kernel_mode=2).beam_dose(beam)
    err = _rel(d, ref)
    print(f"exp recurrence, longest line {L}: FP32 vs FP64 {err:.2e}")
    assert L >= 900
    assert err <= 1e-3
