"""The engine against golden outputs of the reference's own kernel source
(tests/golden).  Table kernel (the reference's discretisation): <= 1.5e-3 of
Dmax.  Double-exponential kernel (fast path): <= 5e-3 of Dmax and a
1 %/1 mm gamma pass rate >= 99.5 %.  Fixtures *_ss<k> were made with TERMA
supersampling ss_factor k."""
import numpy as np
import pytest

import golden_cases
from endtoend_gb300 import engine, metrics

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_cases.names())
def test_engine_matches_reference_kernels(name):
    vol, phys, beams, doses, _, bevs = golden_cases.load(name)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="table")
        e.set_terma_supersampling(golden_cases.ss_factor(name))
        dt = e.beam_dose(beams, per_beam=True)
        e.set_mode("exp")
        de = e.beam_dose(beams, per_beam=True)
        infos = [e.beam_info(i) for i in range(len(beams))]
    vmm = float(vol.voxel[0]) * 10.0
    noise = golden_cases.ref_noise(name)
    for k, dref in enumerate(doses):
        dn = noise[k][0]  # the reference's own rounding sensitivity (supersampled fixtures)
        assert infos[k]["bev_size"] == bevs[k]
        assert metrics.max_rel_diff(dt[k], dref) <= 1.5e-3 + dn
        assert metrics.max_rel_diff(de[k], dref) <= 5e-3 + dn
        assert metrics.gamma_pass_rate(de[k], dref, voxel_mm=vmm, dose_tol=0.01, dist_mm=1.0) >= 0.995


def test_supersampling_with_the_adjoint():
    """The fused dose + adjoint call with TERMA supersampling 3 (table mode):
    its gradient satisfies <A x, g> = <x, A^T g> (rel 2e-4); an ss_factor
    below 1 is refused."""
    import torch
    vol, phys, beams, _, _, _ = golden_cases.load("slab32_ss3")
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="table")
        e.set_terma_supersampling(3)
        fl = torch.from_numpy(engine.concat_fluence(beams)).cuda()
        dose = torch.zeros(vol.nvoxels, device="cuda")
        g = torch.from_numpy(np.random.default_rng(3).standard_normal(vol.nvoxels).astype(np.float32)).cuda()
        fg = torch.zeros_like(fl)
        e.dose_and_adjoint_device(beams, fl.data_ptr(), dose.data_ptr(), g.data_ptr(), fg.data_ptr())
        e.synchronize()
        lhs = float((dose.double() * g.double()).sum())
        rhs = float((fl.double() * fg.double()).sum())
        assert abs(lhs - rhs) <= 2e-4 * abs(lhs), (lhs, rhs)
        with pytest.raises(engine.EEError):
            e.set_terma_supersampling(0)
