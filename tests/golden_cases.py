"""Loader of the golden fixtures in tests/golden (written by
tests/golden/make_golden.py from the reference's own kernel source run on the
CPU)."""
import glob
import os

import numpy as np

from endtoend_gb300 import inputs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    vol = inputs.Volume(density=z["density"].astype(np.float32), voxel=z["voxel"], start=z["start"],
                        bbox_start=z["bbox_start"], bbox_size=z["bbox_size"])
    sp = z["spacing"]
    phys = inputs.Physics(energy=z["energy"], fluence=z["sp_fluence"], mu=z["mu"], mu_en=z["mu_en"],
                          ntheta=int(z["ntheta"]), nphi=int(z["nphi"]), radii=z["radii"], exp_params=z["exp_params"],
                          cumkern=z["cumkern"], theta_deg=z["theta_deg"], phi_deg=z["phi_deg"],
                          rev_latspacing=float(sp[0]), rev_longspacing=float(sp[1]), penumbra=float(z["penumbra"]))
    beams, doses, termas, bevs = [], [], [], []
    for k in range(int(z["nbeams"])):
        az, zen, coll = (float(v) for v in z[f"beam{k}_angles"])
        fm = tuple(int(v) for v in z[f"beam{k}_fmap"])
        bl = tuple(float(v) for v in z[f"beam{k}_beamlet"])
        beams.append(inputs.Beam(azimuth=az, zenith=zen, coll=coll, isocenter=z[f"beam{k}_iso"],
                                 sad=float(z[f"beam{k}_sad"]), fmap_size=fm, beamlet_size=bl,
                                 fluence=z[f"beam{k}_fluence"].astype(np.float32)))
        doses.append(z[f"beam{k}_dose"])
        termas.append(z[f"beam{k}_terma"])
        bevs.append([int(v) for v in z[f"beam{k}_bev"]])
    return vol, phys, beams, doses, termas, bevs


BEAMLET = os.path.join(GOLDEN, "beamlet")


def beamlet_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(BEAMLET, "*.npz")))


def load_beamlet(name):
    """(vol, phys, beam, kernel_extent, max_rev, thresh, reference CSR dict)."""
    z = np.load(os.path.join(BEAMLET, name + ".npz"))
    vol = inputs.Volume(density=z["density"].astype(np.float32), voxel=z["voxel"], start=z["start"],
                        bbox_start=z["bbox_start"], bbox_size=z["bbox_size"])
    sp = z["spacing"]
    phys = inputs.Physics(energy=z["energy"], fluence=z["sp_fluence"], mu=z["mu"], mu_en=z["mu_en"],
                          ntheta=int(z["ntheta"]), nphi=int(z["nphi"]), radii=z["radii"], exp_params=z["exp_params"],
                          cumkern=z["cumkern"], theta_deg=z["theta_deg"], phi_deg=z["phi_deg"],
                          rev_latspacing=float(sp[0]), rev_longspacing=float(sp[1]), penumbra=float(z["penumbra"]))
    az, zen, coll = (float(v) for v in z["beam_angles"])
    beam = inputs.Beam(azimuth=az, zenith=zen, coll=coll, isocenter=z["beam_iso"], sad=float(z["beam_sad"]),
                       fmap_size=tuple(int(v) for v in z["beam_fmap"]),
                       beamlet_size=tuple(float(v) for v in z["beam_beamlet"]),
                       fluence=z["beam_fluence"].astype(np.float32))
    ref = {k: z[k] for k in ("beamlet_index", "col_ptr", "row_index", "value", "info", "ref_noise")}
    return (vol, phys, beam, float(z["kernel_extent"]), tuple(int(v) for v in z["max_rev"]), float(z["thresh"]), ref)
