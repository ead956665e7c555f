"""The allocation-free entry point ee_beam_dose_noalloc, through the C ABI.

Some callers cannot allocate device memory once they are running -- their
GPU memory belongs to a pool carved up in advance (another framework's
caching allocator, a hard per-process budget), or they run in a loop where a
cudaMalloc/cudaFree would stall the device.  For them the library keeps one
static 64 MiB device array as scratch.  This test calls that entry point
twice in a row (two different beams, so the second call reuses scratch the
first one left behind) and checks each result against the allocating entry
point ee_beam_dose_device, in both kernel modes (the double-exponential
recurrence and the cumulative-kernel table), with the tolerance of the other multi-call tests
(rtol 1e-5, atol 1e-6 of the dose maximum); the second call must not change
the device's free memory.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from endtoend_gb300 import engine, inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["exp", "table"])
def test_noalloc_matches_allocating_entry_point_two_calls(mode):
    import torch

    vol, phys, beams = inputs.config0()
    second = inputs.single_beam(fmap=(12, 10), beamlet_cm=0.5, gantry_deg=35.0, couch_deg=15.0)
    second.fluence = np.random.default_rng(21).uniform(0.1, 1.0, second.fluence.shape).astype(np.float32)
    nvox = vol.nvoxels
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode=mode)
        stream = C.c_void_p(e.stream)
        for call, beam in enumerate([beams[0], second]):
            fl = torch.from_numpy(np.ascontiguousarray(beam.fluence.ravel())).cuda()
            ref = torch.zeros(nvox, dtype=torch.float32, device="cuda")
            out = torch.full((nvox,), float("nan"), dtype=torch.float32, device="cuda")
            e.beam_dose_device([beam], fl.data_ptr(), ref.data_ptr(), engine.DOSE_SUM)
            e.synchronize()
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            st = e.lib.ee_beam_dose_noalloc(e.h, engine.to_ee_beams([beam]), C.c_void_p(fl.data_ptr()),
                                            C.c_void_p(out.data_ptr()), stream)
            assert st == 0, e.lib.ee_last_error()
            e.synchronize()
            free_after = torch.cuda.mem_get_info()[0]
            r = ref.cpu().numpy()
            o = out.cpu().numpy()
            assert np.isfinite(o).all()
            assert r.max() > 0
            assert np.allclose(o, r, rtol=1e-5, atol=1e-6 * r.max()), (call, np.abs(o - r).max() / r.max())
            if call == 1:
                assert free_after == free_before, (free_before, free_after)


def test_noalloc_rejects_oversized_beam():
    import torch

    vol = inputs.head_neck_phantom(shape=(120, 120, 100), voxel_cm=0.2)
    phys = inputs.make_physics(seed=0, spacing_cm=0.2)
    beam = inputs.single_beam(fmap=(40, 40), beamlet_cm=0.25, gantry_deg=40.0, couch_deg=20.0)
    fl = torch.ones(beam.fluence.size, dtype=torch.float32, device="cuda")
    out = torch.zeros(vol.nvoxels, dtype=torch.float32, device="cuda")
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="exp")
        st = e.lib.ee_beam_dose_noalloc(e.h, engine.to_ee_beams([beam]), C.c_void_p(fl.data_ptr()),
                                        C.c_void_p(out.data_ptr()), C.c_void_p(e.stream))
        assert st == engine.EE_ERR_CAPACITY
        assert b"scratch" in e.lib.ee_last_error()
