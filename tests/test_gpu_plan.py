"""Planned batches: the chain captured into a CUDA graph (ee_plan_*) gives
the same dose and fluence gradient as the direct pipeline call, also after
the fluence buffer is rewritten between graph replays."""
import numpy as np
import pytest

from endtoend_gb300 import engine, inputs

pytestmark = pytest.mark.gpu


def _setup():
    vol = inputs.slab_phantom(40, 0.25)
    phys = inputs.make_physics(seed=7, spacing_cm=0.25)
    rng = np.random.default_rng(8)
    beams = []
    for g, c in [(10, 0), (75, 20), (160, -40), (230, 15), (300, 60), (90, 0)]:
        n = int(rng.integers(6, 14))
        b = inputs.single_beam(fmap=(n, n), beamlet_cm=0.4, gantry_deg=g, couch_deg=c)
        b.fluence = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
        beams.append(b)
    return vol, phys, beams, rng


def test_plan_matches_pipeline_and_replays():
    import torch
    vol, phys, beams, rng = _setup()
    nvox = vol.nvoxels
    fl = torch.from_numpy(engine.concat_fluence(beams)).cuda()
    g = torch.from_numpy(rng.standard_normal(nvox).astype(np.float32)).cuda()
    dose_p = torch.zeros(nvox, device="cuda")
    fg_p = torch.zeros_like(fl)
    dose_r = torch.zeros(nvox, device="cuda")
    fg_r = torch.zeros_like(fl)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        plan = e.plan(beams, fl.data_ptr(), dose_p.data_ptr(), g.data_ptr(), fg_p.data_ptr())
        assert plan.info()["lane_block"] in (64, 128, 256)
        for rep in range(2):
            if rep == 1:  # new fluence values, same buffers
                fl.mul_(torch.rand_like(fl) * 0.8 + 0.2)
            plan.launch()
            assert plan.status() == 0
            e.dose_and_adjoint_device(beams, fl.data_ptr(), dose_r.data_ptr(), g.data_ptr(), fg_r.data_ptr())
            e.synchronize()
            torch.cuda.synchronize()
            d1, d2 = dose_p.cpu().numpy(), dose_r.cpu().numpy()
            f1, f2 = fg_p.cpu().numpy(), fg_r.cpu().numpy()
            assert np.allclose(d1, d2, rtol=1e-5, atol=1e-6 * d2.max()), (rep, np.abs(d1 - d2).max() / d2.max())
            assert np.allclose(f1, f2, rtol=1e-4, atol=1e-5 * np.abs(f2).max()), rep
        plan.close()


def test_forward_only_plan():
    import torch
    vol, phys, beams, _ = _setup()
    fl = torch.from_numpy(engine.concat_fluence(beams)).cuda()
    dose_p = torch.zeros(vol.nvoxels, device="cuda")
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        plan = e.plan(beams, fl.data_ptr(), dose_p.data_ptr())
        plan.launch()
        assert plan.status() == 0
        ref = e.beam_dose(beams)
        plan.close()
    torch.cuda.synchronize()
    d = dose_p.cpu().numpy().reshape(ref.shape)
    assert np.allclose(d, ref, rtol=1e-5, atol=1e-6 * ref.max())
