"""Regenerate the golden fixtures in tests/golden/ from the reference's own
dosecalc-beam kernel source, executed on the CPU by oracle/ref_harness
(cudaSiddon, cudaRaytrace, RowConvolve, REV2XYZdose compiled unmodified from
the reference checkout; texture filtering emulated with 8-bit weights).

Needs the reference checkout (default /root/reference, or $CCCS_REFERENCE).
Each fixture stores its complete inputs, so tests never depend on the
generators in endtoend_gb300/inputs.py staying unchanged.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from endtoend_gb300 import inputs  # noqa: E402
from oracle.ref_harness import ReferenceHarness  # noqa: E402


def cases():
    vol = inputs.slab_phantom(32, 0.25)
    phys = inputs.make_physics(seed=0, spacing_cm=0.25)
    rng = np.random.default_rng(2024)
    beams = []
    for g, c, cl in [(0.0, 0.0, 0.0), (30.0, 20.0, 0.0), (200.0, -35.0, 10.0)]:
        b = inputs.single_beam(fmap=(8, 8), beamlet_cm=0.5, gantry_deg=g, couch_deg=c, coll_deg=cl)
        b.fluence = rng.uniform(0.2, 1.0, b.fluence.shape).astype(np.float32)
        beams.append(b)
    yield "slab32", vol, phys, beams
    vol = inputs.head_neck_phantom(shape=(48, 48, 40), voxel_cm=0.4, seed=1)
    phys = inputs.make_physics(seed=4, spacing_cm=0.4)
    b = inputs.single_beam(fmap=(12, 12), beamlet_cm=0.4, gantry_deg=130.0, couch_deg=25.0)
    b.fluence = rng.uniform(0.0, 1.0, b.fluence.shape).astype(np.float32)
    yield "headneck48", vol, phys, [b]


def main():
    for name, vol, phys, beams in cases():
        h = ReferenceHarness(vol, phys, tex_emulate=True)
        out = {
            "density": vol.density, "voxel": vol.voxel, "start": vol.start, "bbox_start": vol.bbox_start,
            "bbox_size": vol.bbox_size, "energy": phys.energy, "sp_fluence": phys.fluence, "mu": phys.mu,
            "mu_en": phys.mu_en, "ntheta": phys.ntheta, "nphi": phys.nphi, "radii": phys.radii,
            "exp_params": phys.exp_params, "cumkern": phys.cumkern, "theta_deg": phys.theta_deg,
            "phi_deg": phys.phi_deg, "spacing": [phys.rev_latspacing, phys.rev_longspacing], "penumbra": phys.penumbra,
        }
        for k, b in enumerate(beams):
            dose, terma, bev = h.beam_dose(b)
            out[f"beam{k}_angles"] = [b.azimuth, b.zenith, b.coll]
            out[f"beam{k}_iso"] = b.isocenter
            out[f"beam{k}_sad"] = b.sad
            out[f"beam{k}_fmap"] = list(b.fmap_size)
            out[f"beam{k}_beamlet"] = list(b.beamlet_size)
            out[f"beam{k}_fluence"] = b.fluence
            out[f"beam{k}_dose"] = dose.astype(np.float32)
            out[f"beam{k}_terma"] = terma.astype(np.float32)
            out[f"beam{k}_bev"] = bev
            print(name, k, "Dmax", float(dose.max()), "bev", bev)
        out["nbeams"] = len(beams)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


if __name__ == "__main__":
    main()
