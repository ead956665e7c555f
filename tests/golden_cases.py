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


def ss_factor(name):
    """TERMA supersampling the fixture was made with (1 when not stored)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return int(z["ss_factor"]) if "ss_factor" in z else 1


def ref_noise(name):
    """Per beam (dose, TERMA) change of the reference itself under
    rounding-level isocentre shifts, relative to the maxima (supersampled
    fixtures); zeros where not stored."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return [tuple(float(v) for v in z[f"beam{k}_ref_noise"]) if f"beam{k}_ref_noise" in z else (0.0, 0.0)
            for k in range(int(z["nbeams"]))]


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


# ---------------------------------------------------- kernel-table fixtures --
KERNEL = os.path.join(GOLDEN, "kernel")
KERNEL_CONFIGS = [(8, 6), (12, 8), (4, 4), (48, 2)]   # (ntheta, nphi)
SYNTH_SPECTRUM = "spec_synth"


def synthetic_dsa(seed, nE=4):
    """Seeded FP32 inputs of a kernel-table build with the magnitudes of the
    measured kernels (forward-peaked, falling with radius, five categories):
    spectrum rows (energy, raw fluence, mu, mu_en) and mono [nE][5][48][24]."""
    rng = np.random.default_rng(seed)
    E = np.sort(rng.uniform(0.2, 6.0, nE))
    spec = np.stack([E, rng.uniform(0.01, 0.1, nE), 0.07 * E ** -0.48, 0.03 * E ** -0.08], 1).astype(np.float32)
    r = inputs.KERNEL_RADII_CM
    th = (np.arange(48) + 0.5) * np.pi / 48
    dr = np.diff(np.concatenate([[0.0], r]))
    fwd = np.exp(-3.0 * th)[None, :, None] * rng.uniform(0.8, 1.2, (nE, 48, 1))
    mono = np.zeros((nE, 5, 48, 24))
    for e in range(nE):
        mono[e, 0] = np.exp(-(4.0 + e) * r)[None, :] * dr * rng.uniform(0.5, 1.5, (48, 24))
        for c in (1, 2, 3):
            mono[e, c] = 0.1 * np.exp(-0.4 * r)[None, :] * dr * rng.uniform(0.5, 1.5, (48, 24))
        mono[e, 4] = 1e-4 * rng.uniform(0.0, 1.0, (48, 24))
        mono[e] *= fwd[e][None]
    return spec, mono.astype(np.float32)


def write_dsa_files(data_dir, spec, mono):
    """The inputs as the reference's text files: spectra/spec_synth.spec,
    dsa/synth<e>, dsa/radii.dat, dsa/polar.dat.  Every FP32 value is printed
    with nine significant digits, so any reader gets it back exactly."""
    os.makedirs(os.path.join(data_dir, "spectra"), exist_ok=True)
    os.makedirs(os.path.join(data_dir, "dsa"), exist_ok=True)
    f9 = lambda v: "%.8E" % float(v)
    lines = ["%s %s %s %s synth%d" % (f9(a), f9(b), f9(c), f9(d), e) for e, (a, b, c, d) in enumerate(spec)]
    open(os.path.join(data_dir, "spectra", SYNTH_SPECTRUM + ".spec"), "w").write("\n".join(lines) + "\n")
    radii = inputs.KERNEL_RADII_CM.astype(np.float32)
    open(os.path.join(data_dir, "dsa", "radii.dat"), "w").write("".join(" %s\n" % f9(v) for v in radii))
    open(os.path.join(data_dir, "dsa", "polar.dat"), "w").write(
        "".join("  %s\n" % f9(np.float32((j + 0.5) * np.pi / 48)) for j in range(48)))
    for e in range(mono.shape[0]):
        rows = []
        for j in range(48):
            for i in range(24):
                vals = list(mono[e, :, j, i]) + [radii[i], np.float32((j + 0.5) * 3.75)]
                rows += ["  %s    %s" % (f9(v), f9(0.0)) for v in vals]
        open(os.path.join(data_dir, "dsa", "synth%d" % e), "w").write("\n".join(rows) + "\n")
    return os.path.join(data_dir, "spectra", SYNTH_SPECTRUM + ".spec"), os.path.join(data_dir, "dsa")


def kernel_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(KERNEL, "*.npz")))


def load_kernel(name):
    return dict(np.load(os.path.join(KERNEL, name + ".npz")))


def measured_physics(spacing=0.25):
    """Physics with the measured 6 MV cumulative table of the fixture
    spec_6X_measured (the reference's kernel build from its own data files)
    and the double-exponential fit of it; also returns the fit's error per
    cone."""
    from endtoend_gb300 import engine
    z = load_kernel("spec_6X_measured")
    g = lambda k: z["nt8_np6_" + k]
    params, err = engine.fit_exp_kernel(g("radii"), g("cum_total"))
    return inputs.Physics(energy=g("energy"), fluence=g("fluence"), mu=g("mu"), mu_en=g("mu_en"), ntheta=8, nphi=6,
                          radii=g("radii").astype(np.float64), exp_params=params.astype(np.float64),
                          cumkern=g("cum_total").astype(np.float64), theta_deg=g("conv_theta").astype(np.float64),
                          phi_deg=g("conv_phi").astype(np.float64), rev_latspacing=spacing, rev_longspacing=spacing,
                          penumbra=1.0), err


# ------------------------------------------- config-4 beamlet-column fixture --
# 200 beamlets of the beamlet-coefficient configuration, checked column by
# column against the reference's dosecalc-beamlet kernels.  The dense columns
# (~35 k voxels each above the 1e-4 threshold) do not fit a fixture, so each
# column is stored as a summary: its maximum, sum and entry count, its
# CFG4_TOP largest entries exactly, and its sums over CFG4_BLOCK^3 voxel
# blocks.  The phantom is regenerated from its generator and checked
# against a stored SHA-256 of its density.
CFG4 = os.path.join(GOLDEN, "beamlet_cfg4", "cfg4_200.npz")
CFG4_BLOCK = 8
CFG4_TOP = 128


def cfg4_problem():
    """The 200x200x160 head-and-neck phantom at 2 mm, 8x6 cones, and 8 beams
    of the 1162-beam 4-pi grid (seed 5) with 40x40 beamlets of 2.5 mm, 25
    seeded beamlets active per beam at unit weight: 200 beamlets."""
    vol = inputs.head_neck_phantom(shape=(200, 200, 160), voxel_cm=0.2)
    phys = inputs.make_physics(seed=0, spacing_cm=0.2)
    angs = inputs.four_pi_angles(1162, seed=5)
    rng = np.random.default_rng(404)
    pick = np.sort(rng.choice(len(angs), 8, replace=False))
    beams = []
    for g, c in angs[pick]:
        b = inputs.single_beam(fmap=(40, 40), beamlet_cm=0.25, gantry_deg=float(g), couch_deg=float(c))
        f = np.zeros((40, 40), np.float32)
        f.ravel()[rng.choice(1600, 25, replace=False)] = 1.0
        b.fluence = f
        beams.append(b)
    return vol, phys, beams


def density_digest(vol):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(vol.density, np.float32).tobytes()).hexdigest()


def column_summary(keys, vals, size):
    """Summary of one sparse column (full-grid linear keys, values):
    (max, sum, nnz, top keys, top values, block keys, block sums)."""
    keys = np.asarray(keys, np.int64)
    vals = np.asarray(vals, np.float64)
    nx, ny = int(size[0]), int(size[1])
    B = CFG4_BLOCK
    x, y, z = keys % nx, (keys // nx) % ny, keys // (nx * ny)
    bx, by = (nx + B - 1) // B, (ny + B - 1) // B
    bk = ((z // B) * by + y // B) * bx + x // B
    ub, inv = np.unique(bk, return_inverse=True)
    bs = np.bincount(inv, weights=vals)
    top = np.argsort(-vals, kind="stable")[:CFG4_TOP]
    return (float(vals.max()), float(vals.sum()), int(len(vals)), keys[top], vals[top], ub, bs)


def load_cfg4():
    """(vol, phys, beams, kernel_extent, max_rev, thresh, fixture dict)."""
    z = dict(np.load(CFG4))
    vol, _, beams = cfg4_problem()
    if density_digest(vol) != str(z["density_sha256"]):
        raise RuntimeError("the head-and-neck phantom generator no longer gives the fixture's density")
    sp = z["spacing"]
    phys = inputs.Physics(energy=z["energy"], fluence=z["sp_fluence"], mu=z["mu"], mu_en=z["mu_en"],
                          ntheta=int(z["ntheta"]), nphi=int(z["nphi"]), radii=z["radii"], exp_params=z["exp_params"],
                          cumkern=z["cumkern"], theta_deg=z["theta_deg"], phi_deg=z["phi_deg"],
                          rev_latspacing=float(sp[0]), rev_longspacing=float(sp[1]), penumbra=float(z["penumbra"]))
    for k, b in enumerate(beams):
        b.azimuth, b.zenith, b.coll = (float(v) for v in z[f"beam{k}_angles"])
        b.isocenter = z[f"beam{k}_iso"]
        b.fluence = z[f"beam{k}_fluence"].astype(np.float32)
    return (vol, phys, beams, float(z["kernel_extent"]), tuple(int(v) for v in z["max_rev"]), float(z["thresh"]), z)
