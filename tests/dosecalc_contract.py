"""Writers of the temp-directory contract that the reference's
dosecalc-preprocess leaves for dosecalc-beam (test infrastructure):

  omni-header.txt       write_omni_header    CCCS/DoseCalcIO/calc_header.cpp:13-80
  density.raw           write_debug_data     CCCS/DoseCalcIO/binary_io.h:56-84
  omni_beam_list.txt    write_omni_beam_list CCCS/DoseCalcIO/beam.cpp:582-607
  fluence_maps/<name>   write_fluence_map    CCCS/DoseCalcIO/fluence.cpp:45-78
  convolution_{theta,phi}_angles.raw         CCCS/DoseCalcIO/kernel.cpp:413-419

and of the data directory (spectra/<name>.spec, dsa/*) through
golden_cases.write_dsa_files.  Values are printed with the reference's "%f"
and "%u" formats.
"""
import os

import numpy as np

import golden_cases
from endtoend_gb300 import engine, inputs

PI_F = np.float32(np.pi)


def rad_of_deg(deg):
    """load_omni_beam_list's conversion: (deg * PI) / 180 in FP32."""
    return float(np.float32(np.float32(np.float32(deg) * PI_F) / np.float32(180.0)))


def write_header(temp, vol, ntheta, nphi, spacing, penumbra, beam_count, spec_name, ss_factor=1,
                 kernel_extent=2.0, max_rev=(400, 400, 400)):
    f = lambda v: "%f" % float(np.float32(v))
    lines = ["# " + "=" * 68, "# ==   OMNI-HEADER (written by the tests' contract writer)   ==", "# " + "=" * 68, ""]
    lines += ["%u %u %u" % tuple(int(v) for v in vol.size),
              " ".join(f(v) for v in vol.voxel),
              " ".join(f(v) for v in vol.start),
              "%u %u %u" % tuple(int(v) for v in vol.bbox_start),
              "%u %u %u" % tuple(int(v) for v in vol.bbox_size),
              "%u %u %u" % tuple(max_rev),
              f(spacing), f(spacing), f(kernel_extent), "%u" % ss_factor,
              "%d %d %d" % (nphi, ntheta, 24), f(penumbra), "%d" % beam_count, spec_name, "PTV", "0"]
    open(os.path.join(temp, "omni-header.txt"), "w").write("\n".join(lines) + "\n")


def write_beams(temp, beams_deg):
    """beams_deg: list of dicts with gantry, couch, coll [deg], iso [cm], sad,
    fmap (fx, fy), beamlet (bx, by), fluence [fy][fx] float32."""
    os.makedirs(os.path.join(temp, "fluence_maps"), exist_ok=True)
    out = ["%d" % len(beams_deg)]
    for b, d in enumerate(beams_deg):
        name = "fmap-%06d.raw" % b
        np.ascontiguousarray(d["fluence"], np.float32).tofile(os.path.join(temp, "fluence_maps", name))
        eb = as_engine_beam(d)
        src, direction = engine.beam_source(eb)
        f = lambda v: "%f" % float(np.float32(v))
        out.append(" ".join(["%d" % b, f(d["gantry"]), f(d["couch"]), f(d["coll"]), f(d["sad"]), "man", "in"] +
                            [f(v) for v in d["iso"]] + [f(v) for v in src] + ["auto"] + [f(v) for v in direction] +
                            [f(v) for v in d["beamlet"]] + ["%d" % d["fmap"][0], "%d" % d["fmap"][1], name]))
    out.append("")
    out.append("#beam_id  azimuth zenith coll sad | iso_type iso_loc isocenter.x isocenter.y isocenter.z | ...")
    open(os.path.join(temp, "omni_beam_list.txt"), "w").write("\n".join(out) + "\n")


def as_engine_beam(d):
    """The inputs.Beam that dosecalc-beam builds from a beam-list record."""
    f32 = lambda v: float(np.float32(float("%f" % float(np.float32(v)))))
    return inputs.Beam(azimuth=rad_of_deg(f32(d["gantry"])), zenith=rad_of_deg(f32(d["couch"])),
                       coll=rad_of_deg(f32(d["coll"])), isocenter=np.array([f32(v) for v in d["iso"]]),
                       sad=f32(d["sad"]), fmap_size=tuple(d["fmap"]), beamlet_size=tuple(f32(v) for v in d["beamlet"]),
                       fluence=np.ascontiguousarray(d["fluence"], np.float32))


def write_contract(root, vol, beams_deg, seed=11, ntheta=8, nphi=6, spacing=0.25, penumbra=1.0, ss_factor=1,
                   angle_files=True):
    """temp/ and data/ under root; returns (temp, data)."""
    temp, data = os.path.join(root, "temp"), os.path.join(root, "data")
    os.makedirs(temp, exist_ok=True)
    spec, mono = golden_cases.synthetic_dsa(seed)
    golden_cases.write_dsa_files(data, spec, mono)
    write_header(temp, vol, ntheta, nphi, spacing, penumbra, len(beams_deg), golden_cases.SYNTH_SPECTRUM, ss_factor)
    np.ascontiguousarray(vol.density, np.float32).tofile(os.path.join(temp, "density.raw"))
    write_beams(temp, beams_deg)
    if angle_files:
        th, ph = inputs.cone_angles(ntheta, nphi)
        th.astype(np.float32).tofile(os.path.join(temp, "convolution_theta_angles.raw"))
        ph.astype(np.float32).tofile(os.path.join(temp, "convolution_phi_angles.raw"))
    return temp, data


def slab_case(seed=5):
    vol = inputs.slab_phantom(32, 0.25)
    rng = np.random.default_rng(seed)
    beams = []
    for g, c, cl in [(0.0, 0.0, 0.0), (30.0, 20.0, 0.0), (200.0, -35.0, 10.0)]:
        beams.append(dict(gantry=g, couch=c, coll=cl, iso=list(inputs.ISO_OFFSET_CM), sad=100.0, fmap=(8, 8),
                          beamlet=(0.5, 0.5), fluence=rng.uniform(0.2, 1.0, (8, 8)).astype(np.float32)))
    return vol, beams
