"""GPU parity of the sm_103a engine against the CPU oracle, through the C ABI.

Tolerances (max |difference| / Dmax of the oracle dose):
  * engine vs FP64 oracle of the SAME discretisation:          <= 1e-3
    (FP32 arithmetic and FP32 affine geometry vs FP64)
  * engine (exp kernel) vs the reference discretisation
    (24-radius cumulative table, texture-unit 8-bit weights):  <= 5e-3
    plus a 1%/1 mm gamma pass rate >= 99.5 %.
"""
import numpy as np
import pytest

from endtoend_gb300 import engine, inputs, metrics
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg0():
    return inputs.config0()


@pytest.fixture(scope="module")
def eng(cfg0):
    vol, phys, _ = cfg0
    e = engine.Engine(0)
    e.set_volume(vol)
    e.set_physics(phys, mode="exp")
    yield e
    e.close()


def _rel(a, ref):
    return float(np.abs(a - ref).max() / np.abs(ref).max())


def test_config0_exp_vs_fp64_oracle(cfg0, eng):
    vol, phys, beams = cfg0
    eng.set_mode("exp")
    d = eng.beam_dose(beams)
    ref, info = Oracle(vol, phys, kernel_mode=2).beam_dose(beams[0])
    gi = eng.beam_info(0)
    assert gi["bev_size"] == list(info.bev_size)
    assert _rel(d, ref) <= 1e-3


def test_config0_table_vs_fp64_oracle(cfg0, eng):
    vol, phys, beams = cfg0
    eng.set_mode("table")
    try:
        d = eng.beam_dose(beams)
    finally:
        eng.set_mode("exp")
    ref, _ = Oracle(vol, phys, kernel_mode=0).beam_dose(beams[0])
    assert _rel(d, ref) <= 1e-3


def test_config0_exp_vs_reference_discretisation(cfg0, eng):
    vol, phys, beams = cfg0
    eng.set_mode("exp")
    d = eng.beam_dose(beams)
    ref, _ = Oracle(vol, phys, kernel_mode=0, tex_emulate=True).beam_dose(beams[0])
    assert _rel(d, ref) <= 5e-3
    pr = metrics.gamma_pass_rate(d, ref, voxel_mm=2.5, dose_tol=0.01, dist_mm=1.0)
    assert pr >= 0.995, pr


@pytest.mark.parametrize("gantry,couch,coll", [(30.0, 20.0, 0.0), (200.0, -35.0, 10.0), (90.0, 0.0, 0.0)])
def test_oblique_beams(gantry, couch, coll):
    vol = inputs.slab_phantom(40, 0.25)
    phys = inputs.make_physics(seed=1, spacing_cm=0.25)
    beam = inputs.single_beam(fmap=(10, 8), beamlet_cm=0.5, gantry_deg=gantry, couch_deg=couch, coll_deg=coll)
    beam.fluence = np.random.default_rng(3).uniform(0.1, 1.0, beam.fluence.shape).astype(np.float32)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        d = e.beam_dose([beam])
        e.set_mode("table")
        dt = e.beam_dose([beam])
    ref2, _ = Oracle(vol, phys, kernel_mode=2).beam_dose(beam)
    ref0, _ = Oracle(vol, phys, kernel_mode=0).beam_dose(beam)
    assert _rel(d, ref2) <= 1e-3
    assert _rel(dt, ref0) <= 1e-3


def test_source_inside_the_volume():
    """A 3 cm source-axis distance puts the source inside the phantom, so some
    samples lie behind it (where the field's projection mirrors): dose and
    adjoint still follow the oracle (the cone kernels' field span is not used
    on such lines)."""
    vol = inputs.slab_phantom(32, 0.25)
    phys = inputs.make_physics(seed=5, spacing_cm=0.25)
    beam = inputs.single_beam(fmap=(6, 6), beamlet_cm=0.2, gantry_deg=30.0, couch_deg=10.0, sad_cm=3.0)
    rng = np.random.default_rng(8)
    beam.fluence = rng.uniform(0.2, 1.0, beam.fluence.shape).astype(np.float32)
    g = rng.standard_normal(vol.density.shape).astype(np.float32)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        d = e.beam_dose([beam])
        fg = e.beam_dose_adjoint([beam], g)[0]
    o = Oracle(vol, phys, kernel_mode=2)
    ref, _ = o.beam_dose(beam)
    assert ref.max() > 0
    assert _rel(d, ref) <= 1e-3
    fref, _ = o.beam_dose_adjoint(beam, g)
    assert _rel(fg, fref) <= 2e-3


def test_multi_beam_sum_and_per_beam(eng, cfg0):
    vol, phys, _ = cfg0
    beams = [inputs.single_beam(fmap=(8, 8), beamlet_cm=0.5, gantry_deg=g, couch_deg=c) for g, c in
             [(0, 0), (72, 0), (144, 15), (216, -20)]]
    for i, b in enumerate(beams):
        b.fluence = np.random.default_rng(10 + i).uniform(0.0, 1.0, b.fluence.shape).astype(np.float32)
    per = eng.beam_dose(beams, per_beam=True)
    tot = eng.beam_dose(beams)
    assert np.allclose(per.sum(0), tot, rtol=1e-5, atol=1e-6 * tot.max())
    acc = np.zeros_like(tot)
    eng.beam_dose(beams[:2], accumulate_into=acc)
    eng.beam_dose(beams[2:], accumulate_into=acc)
    assert np.allclose(acc, tot, rtol=1e-5, atol=1e-6 * tot.max())
    # each beam alone equals its slot in the batch
    one = eng.beam_dose([beams[2]])
    assert np.allclose(one, per[2], rtol=1e-6, atol=1e-7 * one.max())


@pytest.mark.parametrize("mode", ["exp", "table"])
def test_adjoint_vs_oracle_and_dot_product(mode):
    vol = inputs.slab_phantom(32, 0.25)
    phys = inputs.make_physics(seed=2, spacing_cm=0.25)
    beams = [inputs.single_beam(fmap=(8, 8), beamlet_cm=0.5, gantry_deg=g, couch_deg=c) for g, c in [(20, 0), (250, 30)]]
    rng = np.random.default_rng(4)
    for b in beams:
        b.fluence = rng.uniform(0.2, 1.0, b.fluence.shape).astype(np.float32)
    g = rng.standard_normal(vol.density.shape).astype(np.float32)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode=mode)
        dose = e.beam_dose(beams)
        fg = e.beam_dose_adjoint(beams, g)
    # <A x, g> == <x, A^T g>
    lhs = float(np.sum(dose.astype(np.float64) * g))
    rhs = float(sum(np.sum(b.fluence.astype(np.float64) * f) for b, f in zip(beams, fg)))
    assert abs(lhs - rhs) <= 2e-4 * abs(lhs) + 1e-6, (lhs, rhs)
    o = Oracle(vol, phys, kernel_mode=2 if mode == "exp" else 0)
    for b, f in zip(beams, fg):
        ref, _ = o.beam_dose_adjoint(b, g)
        assert _rel(f, ref) <= 2e-3


def test_error_paths(eng, cfg0):
    vol, phys, beams = cfg0
    b = inputs.single_beam(fmap=(4, 4), beamlet_cm=0.5, iso=(100.0, 100.0, 100.0))
    with pytest.raises(engine.CropBoxError):
        eng.beam_dose([b])
    # the context stays usable after an error
    d = eng.beam_dose(beams)
    assert d.max() > 0


def test_fused_dose_and_adjoint_matches_separate_calls():
    import ctypes as C
    vol = inputs.slab_phantom(32, 0.25)
    phys = inputs.make_physics(seed=3, spacing_cm=0.25)
    beams = [inputs.single_beam(fmap=(8, 8), beamlet_cm=0.5, gantry_deg=g, couch_deg=c) for g, c in [(40, 10), (300, -15)]]
    rng = np.random.default_rng(6)
    for b in beams:
        b.fluence = rng.uniform(0.1, 1.0, b.fluence.shape).astype(np.float32)
    g = rng.standard_normal(vol.density.shape).astype(np.float32)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        d_sep = e.beam_dose(beams)
        f_sep = np.concatenate([f.ravel() for f in e.beam_dose_adjoint(beams, g)])
        fl = engine.concat_fluence(beams)
        d = np.zeros_like(d_sep)
        f = np.zeros_like(fl)
        st = e.lib.ee_dose_and_adjoint(e.h, engine.to_ee_beams(beams), len(beams), C.c_void_p(fl.ctypes.data),
                                       C.c_void_p(d.ctypes.data), engine.DOSE_SUM, C.c_void_p(g.ctypes.data),
                                       C.c_void_p(f.ctypes.data))
        e._check(st)
    assert np.allclose(d, d_sep, rtol=1e-5, atol=1e-6 * d_sep.max())
    assert np.allclose(f, f_sep, rtol=1e-4, atol=1e-5 * np.abs(f_sep).max())


def test_rev_array_over_the_limit_is_an_array_size_error(cfg0):
    """A cone's REV array larger than max_rev_size fails the beam with
    EE_ERR_REV_SIZE, the reference's ArraySizeError (host.cu:71-74,148-154);
    the context stays usable once the limit is lifted."""
    vol, phys, beams = cfg0
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp", max_rev_size=(16, 16, 16))
        with pytest.raises(engine.ArraySizeError) as ei:
            e.beam_dose(beams)
        assert ei.value.code == engine.EE_ERR_REV_SIZE
        e.set_physics(phys, mode="exp")
        ref, _ = Oracle(vol, phys, kernel_mode=2).beam_dose(beams[0])
        assert _rel(e.beam_dose(beams), ref) <= 1e-3


def test_all_zero_fluence_is_a_crop_box_error(cfg0, eng):
    """No voxel with TERMA leaves the crop-box scan (host.cu:442-459) empty:
    the beam fails (the oracle refuses it too), and the next call works."""
    vol, phys, beams = cfg0
    z = inputs.Beam(**{**beams[0].__dict__, "fluence": np.zeros_like(beams[0].fluence)})
    with pytest.raises(RuntimeError):
        Oracle(vol, phys, kernel_mode=2).beam_dose(z)
    with pytest.raises(engine.CropBoxError):
        eng.beam_dose([z])
    assert eng.beam_dose(beams).max() > 0


def test_single_beamlet_map(cfg0, eng):
    """A 1 x 1 fluence map: forward against the FP64 oracle, adjoint by the
    dot-product identity <A x, g> = <x, A^T g>."""
    vol, phys, _ = cfg0
    b = inputs.single_beam(fmap=(1, 1), beamlet_cm=1.0)
    d = eng.beam_dose([b])
    ref, _ = Oracle(vol, phys, kernel_mode=2).beam_dose(b)
    assert _rel(d, ref) <= 1e-3
    g = np.random.default_rng(5).standard_normal(d.shape).astype(np.float32)
    fg = eng.beam_dose_adjoint([b], g)
    lhs = float(np.dot(d.ravel().astype(np.float64), g.ravel()))
    rhs = float(np.dot(b.fluence.ravel().astype(np.float64), np.asarray(fg, np.float64).ravel()))
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs)


@pytest.mark.parametrize("ss", [2, 3])
def test_supersampled_terma_adjoint(ss):
    """Adjoint with TERMA supersampling (ss^3 sub-voxel centres per voxel,
    each with its own beamlet; cudaSiddon.cu:248-258, 297-306): the
    dot-product identity <A x, g> = <x, A^T g> (rel 2e-4), single beamlets'
    gradients against <A (x + d e_p) - A x, g> / d (the dose is linear in the
    fluence and every beamlet stays on, so the crop boxes do not move;
    2e-3 of the largest gradient), and the planned batch's adjoint against
    the direct call's (rel 1e-5)."""
    import torch

    vol = inputs.slab_phantom(32, 0.25)
    phys = inputs.make_physics(seed=2, spacing_cm=0.25)
    beams = [inputs.single_beam(fmap=(8, 8), beamlet_cm=0.5, gantry_deg=g, couch_deg=c) for g, c in [(20, 0), (250, 30)]]
    rng = np.random.default_rng(14)
    for b in beams:
        b.fluence = rng.uniform(0.2, 1.0, b.fluence.shape).astype(np.float32)
    g = rng.standard_normal(vol.density.shape).astype(np.float32)
    g64 = g.astype(np.float64)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        e.set_terma_supersampling(ss)
        dose = e.beam_dose(beams)
        fg = e.beam_dose_adjoint(beams, g)
        lhs = float(np.sum(dose.astype(np.float64) * g64))
        rhs = float(sum(np.sum(b.fluence.astype(np.float64) * f) for b, f in zip(beams, fg)))
        assert abs(lhs - rhs) <= 2e-4 * abs(lhs), (lhs, rhs)
        scale = max(float(np.abs(f).max()) for f in fg)
        for k, b in enumerate(beams):
            base = float(np.sum(e.beam_dose([b]).astype(np.float64) * g64))
            for p in rng.choice(b.fluence.size, 4, replace=False):
                bp = inputs.Beam(**{**b.__dict__, "fluence": b.fluence.copy()})
                bp.fluence.ravel()[p] += 0.5
                d = (float(np.sum(e.beam_dose([bp]).astype(np.float64) * g64)) - base) / 0.5
                assert abs(d - float(fg[k].ravel()[p])) <= 2e-3 * scale, (k, p, d, fg[k].ravel()[p])
        fl = torch.from_numpy(engine.concat_fluence(beams)).cuda()
        dd = torch.zeros(vol.nvoxels, device="cuda")
        dg = torch.from_numpy(g.ravel()).cuda()
        xg = torch.zeros_like(fl)
        plan = e.plan(beams, fl.data_ptr(), dd.data_ptr(), dg.data_ptr(), xg.data_ptr())
        plan.launch()
        e.synchronize()
        plan.status()
        plan.close()
        want = np.concatenate([f.ravel() for f in fg])
        np.testing.assert_allclose(xg.cpu().numpy(), want, rtol=1e-5, atol=1e-6 * np.abs(want).max())
