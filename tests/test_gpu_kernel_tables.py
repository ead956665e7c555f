"""Kernel tables on the GPU (ee_cumulative_kernel) and the dose they give.

- The GPU build from the library's file readers equals the reference's own
  spectra.cpp / kernel.cpp build (fixtures in tests/golden/kernel) bit for bit,
  for every (ntheta, nphi) fixture configuration.
- With the measured 6 MV cumulative table (fixture spec_6X_measured):
    * the engine's table walk against the FP64 oracle of the same table:
      max |difference| <= 1e-3 Dmax (the table-mode parity bar);
    * the exp fast path on the fitted double exponentials against that table
      walk: max |difference| <= 3.5 % Dmax, plus a 2 %/2 mm gamma pass rate
      >= 99 %.  The fit, not the engine, sets this gap: the FP64 oracle's
      own exp-vs-table difference on these two beams is 2.8 % Dmax (a double
      exponential per cone follows the measured cumulative kernel to 2-5 %
      of its maximum).
"""
import os

import numpy as np
import pytest

import golden_cases
from endtoend_gb300 import engine, inputs, metrics
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["synth11", "synth12"])
def test_gpu_tables_match_reference(name, tmp_path):
    z = golden_cases.load_kernel(name)
    spec_path, dsa = golden_cases.write_dsa_files(str(tmp_path), z["spec"], z["mono"])
    energy, fluence, mu, mu_en, names = engine.read_spectrum_file(spec_path)
    mono = np.stack([engine.read_mono_kernel(os.path.join(dsa, n)) for n in names])
    for nt, nph in golden_cases.KERNEL_CONFIGS:
        t = engine.cumulative_kernel(energy, fluence, mu, mono, nt, nph)
        np.testing.assert_array_equal(t["poly_total"], z["poly_total"])
        np.testing.assert_array_equal(t["poly_weights"], z["poly_weights"])
        for k in ("cum_total", "cum_weights", "conv_theta", "conv_phi"):
            np.testing.assert_array_equal(t[k], z[f"nt{nt}_np{nph}_{k}"], err_msg=f"{k} ntheta={nt}")
    phys = engine.physics_from_kernel_files(spec_path, dsa, 8, 6)
    np.testing.assert_array_equal(phys.cumkern.astype(np.float32), z["nt8_np6_cum_total"])
    np.testing.assert_array_equal(phys.fluence, z["fluence"])


def test_gpu_tables_errors():
    z = golden_cases.load_kernel("synth11")
    with pytest.raises(engine.EEError):
        engine.cumulative_kernel(z["energy"], z["fluence"], z["mu"], z["mono"], 5, 6)  # 5 does not divide 48


def _measured_physics(spacing=0.25):
    return golden_cases.measured_physics(spacing)


@pytest.mark.parametrize("gantry,couch", [(0.0, 0.0), (40.0, 20.0)])
def test_measured_6mv_table_and_exp_fit(gantry, couch):
    phys, fit_err = _measured_physics()
    vol = inputs.slab_phantom(48, 0.25)
    beam = inputs.single_beam(fmap=(16, 16), beamlet_cm=0.5, gantry_deg=gantry, couch_deg=couch)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="table")
        d_table = e.beam_dose([beam])
        e.set_mode("exp")
        d_exp = e.beam_dose([beam])
    ref, _ = Oracle(vol, phys, kernel_mode=0).beam_dose(beam)
    dmax = float(np.abs(ref).max())
    table_err = float(np.abs(d_table - ref).max() / dmax)
    exp_err = float(np.abs(d_exp - d_table).max() / dmax)
    gamma = metrics.gamma_pass_rate(d_exp, d_table, 10.0 * np.asarray(vol.voxel), dose_tol=0.02, dist_mm=2.0,
                                    threshold=0.1)
    print(f"measured 6MV g={gantry} c={couch}: table vs oracle {table_err:.2e}, exp fit vs table {exp_err:.4f}, "
          f"gamma(2%/2mm) {gamma:.4f}, cumulative fit error per cone {np.round(fit_err, 4)}")
    assert table_err <= 1e-3
    assert exp_err <= 0.035
    assert gamma >= 0.99
