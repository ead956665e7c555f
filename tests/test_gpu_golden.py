"""The engine against golden outputs of the reference's own kernel source
(tests/golden).  Table kernel (the reference's discretisation): <= 1.5e-3 of
Dmax.  Double-exponential kernel (fast path): <= 5e-3 of Dmax and a
1 %/1 mm gamma pass rate >= 99.5 %."""
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
        dt = e.beam_dose(beams, per_beam=True)
        e.set_mode("exp")
        de = e.beam_dose(beams, per_beam=True)
        infos = [e.beam_info(i) for i in range(len(beams))]
    vmm = float(vol.voxel[0]) * 10.0
    for k, dref in enumerate(doses):
        assert infos[k]["bev_size"] == bevs[k]
        assert metrics.max_rel_diff(dt[k], dref) <= 1.5e-3
        assert metrics.max_rel_diff(de[k], dref) <= 5e-3
        assert metrics.gamma_pass_rate(de[k], dref, voxel_mm=vmm, dose_tol=0.01, dist_mm=1.0) >= 0.995
