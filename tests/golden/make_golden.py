"""Regenerate the golden fixtures in tests/golden/ from the reference's own
dosecalc-beam kernel source, executed on the CPU by oracle/ref_harness
(cudaSiddon, cudaRaytrace, RowConvolve, REV2XYZdose compiled unmodified from
the reference checkout; texture filtering emulated with 8-bit weights), and
the beamlet-column fixtures in tests/golden/beamlet/ from the reference's
dosecalc-beamlet kernel source (cudaBeamletRaytrace, PackRowConvolve,
PackedREVtoBEVdose, UnpackBEVDosePillar) sparsified as sparse_io.cpp does.

Needs the reference checkout: $CCCS_REFERENCE, or a `reference` directory
beside this repository (oracle/ref_harness/build.py, reference_root).
Each fixture stores its complete inputs, so tests never depend on the
generators in endtoend_gb300/inputs.py staying unchanged.

    python tests/golden/make_golden.py          # every fixture
    python tests/golden/make_golden.py kernel   # the kernel-table fixtures only
    python tests/golden/make_golden.py beam [name ...]   # dosecalc-beam fixtures (all, or the named)
    python tests/golden/make_golden.py beamlet [name ...]   # dosecalc-beamlet fixtures (all, or the named)
    python tests/golden/make_golden.py cfg4     # 200 beamlets of the beamlet-coefficient configuration
    python tests/golden/make_golden.py cfg4_noise   # ... its reference sensitivity over the full shift set

The kernel-table fixtures in tests/golden/kernel come from the reference's
spectrum and kernel-table build (spectra.cpp, kernel.cpp) run on the CPU by
oracle/ref_harness/ref_kernel_harness.cpp.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from endtoend_gb300 import inputs  # noqa: E402
from oracle.ref_harness import BeamletHarness, ReferenceHarness, kernel_build, sparsify  # noqa: E402
import golden_cases  # noqa: E402


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
    # TERMA supersampling (omni-header ss_factor 3 = the preprocessing
    # default, and 2): the same slab, two of the beams
    yield "slab32_ss3", vol, phys, beams[:2]
    yield "slab32_ss2", vol, phys, beams[1:2]
    vol = inputs.head_neck_phantom(shape=(48, 48, 40), voxel_cm=0.4, seed=1)
    phys = inputs.make_physics(seed=4, spacing_cm=0.4)
    b = inputs.single_beam(fmap=(12, 12), beamlet_cm=0.4, gantry_deg=130.0, couch_deg=25.0)
    b.fluence = rng.uniform(0.0, 1.0, b.fluence.shape).astype(np.float32)
    yield "headneck48", vol, phys, [b]
    # a calc bbox inside the volume (dosecalc-preprocess crops it to the
    # body): TERMA, the crop box and the dose stop at its faces; a
    # non-square fluence map of non-square beamlets, larger than the bbox
    vol = inputs.slab_phantom(32, 0.25)
    vol.bbox_start = np.array([5, 3, 7], np.int64)
    vol.bbox_size = np.array([22, 26, 18], np.int64)
    phys = inputs.make_physics(seed=0, spacing_cm=0.25)
    b = inputs.single_beam(fmap=(10, 6), beamlet_cm=0.4, gantry_deg=60.0, couch_deg=15.0, coll_deg=20.0)
    b.beamlet_size = (0.4, 0.6)
    b.fluence = rng.uniform(0.2, 1.0, b.fluence.shape).astype(np.float32)
    yield "slab32_bbox", vol, phys, [b]


def beamlet_cases():
    vol = inputs.slab_phantom(32, 0.25)
    phys = inputs.make_physics(seed=7, spacing_cm=0.25)
    b = inputs.single_beam(fmap=(3, 3), beamlet_cm=0.5, gantry_deg=30.0, couch_deg=0.0)
    b.fluence = np.array([[1, 0.5, 0], [1, 1, 1], [0.2, 1, 1]], np.float32)
    yield "bl_slab32", vol, phys, b, 2.0, (500, 500, 500), 1e-4
    yield "bl_slab32_batched", vol, phys, b, 2.0, (110, 110, 110), 1e-4
    vol = inputs.head_neck_phantom(shape=(40, 40, 32), voxel_cm=0.4, seed=3)
    phys = inputs.make_physics(seed=5, spacing_cm=0.4)
    rng = np.random.default_rng(77)
    b = inputs.single_beam(fmap=(4, 4), beamlet_cm=0.4, gantry_deg=130.0, couch_deg=25.0, coll_deg=10.0)
    f = rng.uniform(0.3, 1.0, (4, 4)).astype(np.float32)
    f[0, 3] = 0.0
    f[2, 1] = 0.0
    b.fluence = f
    yield "bl_headneck40", vol, phys, b, 1.5, (500, 500, 500), 1e-4
    # a calc bbox inside the volume: pillars, columns and CSR rows clipped
    # to it (rows keyed in the full volume)
    vol = inputs.slab_phantom(32, 0.25)
    vol.bbox_start = np.array([4, 2, 5], np.int64)
    vol.bbox_size = np.array([24, 28, 22], np.int64)
    phys = inputs.make_physics(seed=7, spacing_cm=0.25)
    b = inputs.single_beam(fmap=(3, 3), beamlet_cm=0.5, gantry_deg=30.0, couch_deg=10.0)
    b.fluence = np.array([[1, 0.5, 0], [1, 1, 1], [0.2, 1, 1]], np.float32)
    yield "bl_slab32_bbox", vol, phys, b, 2.0, (500, 500, 500), 1e-4


def physics_fields(vol, phys):
    return {
        "density": vol.density, "voxel": vol.voxel, "start": vol.start, "bbox_start": vol.bbox_start,
        "bbox_size": vol.bbox_size, "energy": phys.energy, "sp_fluence": phys.fluence, "mu": phys.mu,
        "mu_en": phys.mu_en, "ntheta": phys.ntheta, "nphi": phys.nphi, "radii": phys.radii,
        "exp_params": phys.exp_params, "cumkern": phys.cumkern, "theta_deg": phys.theta_deg,
        "phi_deg": phys.phi_deg, "spacing": [phys.rev_latspacing, phys.rev_longspacing], "penumbra": phys.penumbra,
    }


def main_beamlet(only=None):
    os.makedirs(os.path.join(HERE, "beamlet"), exist_ok=True)
    for name, vol, phys, b, ke, max_rev, thresh in beamlet_cases():
        if only and name not in only:
            continue
        h = BeamletHarness(vol, phys, tex_emulate=True)
        idx, cols, info = h.columns(b, kernel_extent=ke, max_rev_size=max_rev)
        out = physics_fields(vol, phys)
        out.update({"beam_angles": [b.azimuth, b.zenith, b.coll], "beam_iso": b.isocenter, "beam_sad": b.sad,
                    "beam_fmap": list(b.fmap_size), "beam_beamlet": list(b.beamlet_size), "beam_fluence": b.fluence,
                    "kernel_extent": ke, "max_rev": list(max_rev), "thresh": thresh, "beamlet_index": idx,
                    "info": info})
        col_ptr, rows, vals = [0], [], []
        for c in cols:
            k, v = sparsify(c, thresh, vol.bbox_start, vol.size)
            rows.append(k.astype(np.int32))
            vals.append(v.astype(np.float32))
            col_ptr.append(col_ptr[-1] + len(k))
        # the reference's own sensitivity: the same columns with the
        # isocentre (or the REV lattice) moved by rounding-level amounts (1e-6 .. 1e-5 cm along
        # several directions), per column max |change| / column max -- thin
        # beamlets sampled on a rotated REV lattice put samples exactly on
        # the footprint edge, where FP32 rounding decides (the reference's
        # own GPU run, with its hardware sin/cos, lands on either side)
        noise = np.zeros(len(idx))
        shifts = [(1, -1, 1), (-1, 1, -1), (1, 0, 0), (0, 1, 0), (0, 0, 1), (-1, -1, 0), (0, -1, 1), (1, 1, 1)]
        for k, sh in enumerate(shifts):
            bp = inputs.Beam(**{**b.__dict__})
            bp.isocenter = np.asarray(b.isocenter, np.float64) + (1e-5 if k % 2 == 0 else 1e-6) * np.array(sh, float)
            _, cp_, _ = h.columns(bp, kernel_extent=ke, max_rev_size=max_rev)
            for c in range(len(idx)):
                noise[c] = max(noise[c], float(np.abs(cp_[c] - cols[c]).max() / cols[c].max()))
        # ... and with the REV lattice origin moved by the same amounts
        for jit in (1e-5, -1e-5, 1e-6, -1e-6):
            _, cp_, _ = h.columns(b, kernel_extent=ke, max_rev_size=max_rev, rev_jitter=jit)
            for c in range(len(idx)):
                noise[c] = max(noise[c], float(np.abs(cp_[c] - cols[c]).max() / cols[c].max()))
        out["ref_noise"] = noise
        out["col_ptr"] = np.array(col_ptr, np.int64)
        out["row_index"] = np.concatenate(rows) if rows else np.zeros(0, np.int32)
        out["value"] = np.concatenate(vals) if vals else np.zeros(0, np.float32)
        print(name, "beamlets", len(idx), "nnz", int(col_ptr[-1]), "info", info, "ref noise", np.round(noise, 4))
        np.savez_compressed(os.path.join(HERE, "beamlet", f"{name}.npz"), **out)


KT_KEYS = ("energy", "fluence", "mu", "mu_en", "poly_total", "poly_weights", "cum_total", "cum_weights", "radii",
           "ang_bounds", "conv_theta", "conv_phi")


def main_kernel():
    """Kernel-table fixtures from the reference's read_spectrum_file /
    read_kernel / make_poly_kernel / make_cumulative_kernel: seeded synthetic
    point kernels (inputs stored) in every (ntheta, nphi) of KERNEL_CONFIGS,
    and the outputs only of the 6 MV spectrum with the measured dsa kernels."""
    os.makedirs(golden_cases.KERNEL, exist_ok=True)
    from oracle.ref_harness import build as ref_build
    ref = ref_build.reference_root()
    if ref is None:
        raise RuntimeError("reference checkout not found: " + ref_build.HOW)
    scratch = os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref", "tmp")
    for seed in (11, 12):
        spec, mono = golden_cases.synthetic_dsa(seed)
        d = os.path.join(scratch, f"synth{seed}")
        golden_cases.write_dsa_files(d, spec, mono)
        out = {"spec": spec, "mono": mono}
        for nt, nph in golden_cases.KERNEL_CONFIGS:
            r = kernel_build(d, golden_cases.SYNTH_SPECTRUM, nt, nph)
            for k in KT_KEYS:   # the spectrum and poly kernel do not depend on the cones
                once = k in ("energy", "fluence", "mu", "mu_en", "poly_total", "poly_weights", "radii")
                out[k if once else f"nt{nt}_np{nph}_{k}"] = r[k]
        np.savez_compressed(os.path.join(golden_cases.KERNEL, f"synth{seed}.npz"), **out)
        print("kernel fixture synth", seed, "cum_total[0,-1]", float(out["nt8_np6_cum_total"][0, -1]))
    r = kernel_build(os.path.join(ref, "CCCS", "data"), "spec_6X", 8, 6)
    np.savez_compressed(os.path.join(golden_cases.KERNEL, "spec_6X_measured.npz"),
                        **{f"nt8_np6_{k}": r[k] for k in KT_KEYS if k not in ("poly_weights",)})
    print("kernel fixture spec_6X", r["cum_total"][:, -1])


def main():
    if sys.argv[1:] == ["kernel"]:
        main_kernel()
        return
    if sys.argv[1:2] == ["beam"]:
        main_beam(sys.argv[2:] or None)
        return
    if sys.argv[1:2] == ["beamlet"]:
        main_beamlet(sys.argv[2:] or None)
        return
    if sys.argv[1:] == ["cfg4"]:
        main_cfg4()
        return
    if sys.argv[1:] == ["cfg4_noise"]:
        main_cfg4_noise()
        return
    main_kernel()
    main_beamlet()
    main_beam()
    main_cfg4()


# the rounding-level shifts of the other beamlet fixtures: isocentre moves
# of 1e-5 / 1e-6 cm along eight directions and REV lattice moves
ISO_SHIFTS = [(1, -1, 1), (-1, 1, -1), (1, 0, 0), (0, 1, 0), (0, 0, 1), (-1, -1, 0), (0, -1, 1), (1, 1, 1)]
REV_JITTERS = (1e-5, -1e-5, 1e-6, -1e-6)


def main_cfg4_noise():
    """Extend the config-4 fixture's per-column reference sensitivity to the
    full shift set of the other beamlet fixtures (the first pass used four
    of these moves); the stored value becomes the maximum over all."""
    z = dict(np.load(golden_cases.CFG4))
    vol, phys, beams, ke, max_rev, thresh, _ = golden_cases.load_cfg4()
    h = BeamletHarness(vol, phys, tex_emulate=True)
    for k, b in enumerate(beams):
        idx, cols, _ = h.columns(b, kernel_extent=ke, max_rev_size=max_rev)
        noise = np.array(z[f"beam{k}_ref_noise"], np.float64)
        moves = [("iso", (1e-5 if j % 2 == 0 else 1e-6) * np.array(sh, float)) for j, sh in enumerate(ISO_SHIFTS)]
        moves += [("rev", jit) for jit in REV_JITTERS]
        for kind, amount in moves:
            if kind == "iso":
                bp = inputs.Beam(**{**b.__dict__})
                bp.isocenter = np.asarray(b.isocenter, np.float64) + amount
                _, cp_, _ = h.columns(bp, kernel_extent=ke, max_rev_size=max_rev)
            else:
                _, cp_, _ = h.columns(b, kernel_extent=ke, max_rev_size=max_rev, rev_jitter=amount)
            for c in range(len(idx)):
                noise[c] = max(noise[c], float(np.abs(cp_[c] - cols[c]).max() / cols[c].max()))
            del cp_
        z[f"beam{k}_ref_noise"] = noise
        print("cfg4 noise beam", k, np.round(noise, 4), flush=True)
        del cols
    np.savez_compressed(golden_cases.CFG4, **z)


def main_cfg4():
    """200 beamlet columns of the beamlet-coefficient configuration
    (golden_cases.cfg4_problem: the 200x200x160 phantom at 2 mm, 8 beams of
    the 1162-beam grid, 25 beamlets each, kernel extent 2 cm, threshold 1e-4
    of each column's maximum) from the reference's dosecalc-beamlet kernels,
    stored as per-column summaries (golden_cases.column_summary), with the
    reference's own change per column under rounding-level isocentre and REV
    lattice shifts."""
    vol, phys, beams = golden_cases.cfg4_problem()
    ke, max_rev, thresh = 2.0, (500, 500, 500), 1e-4
    h = BeamletHarness(vol, phys, tex_emulate=True)
    out = physics_fields(vol, phys)
    del out["density"]
    out.update({"density_sha256": golden_cases.density_digest(vol), "kernel_extent": ke, "max_rev": list(max_rev),
                "thresh": thresh, "nbeams": len(beams)})
    fields = ("max", "sum", "nnz")
    for k, b in enumerate(beams):
        idx, cols, info = h.columns(b, kernel_extent=ke, max_rev_size=max_rev)
        summ = []
        for c in cols:
            keys, vals = sparsify(c, thresh, vol.bbox_start, vol.size)
            summ.append(golden_cases.column_summary(keys, vals, vol.size))
        noise = np.zeros(len(idx))
        for kind, amount in (("iso", (1e-5, 1e-5, -1e-5)), ("iso", (-1e-6, 1e-6, 1e-6)), ("rev", 1e-5),
                             ("rev", -1e-5)):
            if kind == "iso":
                bp = inputs.Beam(**{**b.__dict__})
                bp.isocenter = np.asarray(b.isocenter, np.float64) + np.array(amount)
                _, cp_, _ = h.columns(bp, kernel_extent=ke, max_rev_size=max_rev)
            else:
                _, cp_, _ = h.columns(b, kernel_extent=ke, max_rev_size=max_rev, rev_jitter=amount)
            for c in range(len(idx)):
                noise[c] = max(noise[c], float(np.abs(cp_[c] - cols[c]).max() / cols[c].max()))
            del cp_
        out[f"beam{k}_angles"] = [b.azimuth, b.zenith, b.coll]
        out[f"beam{k}_iso"] = b.isocenter
        out[f"beam{k}_fluence"] = b.fluence
        out[f"beam{k}_beamlet_index"] = idx
        out[f"beam{k}_ref_noise"] = noise
        for j, f in enumerate(fields):
            out[f"beam{k}_{f}"] = np.array([s_[j] for s_ in summ])
        for j, f in ((3, "top_key"), (4, "top_val"), (5, "blk_key"), (6, "blk_sum")):
            out[f"beam{k}_{f}_ptr"] = np.cumsum([0] + [len(s_[j]) for s_ in summ]).astype(np.int64)
            out[f"beam{k}_{f}"] = np.concatenate([s_[j] for s_ in summ])
        print("cfg4 beam", k, "beamlets", len(idx), "info", info, "nnz", out[f"beam{k}_nnz"].tolist()[:5],
              "ref noise", np.round(noise, 4), flush=True)
        del cols
    np.savez_compressed(golden_cases.CFG4, **out)


def main_beam(only=None):
    for name, vol, phys, beams in cases():
        if only and name not in only:
            continue
        ss = int(name.rsplit("_ss", 1)[1]) if "_ss" in name else 1
        h = ReferenceHarness(vol, phys, tex_emulate=True, ss_factor=ss)
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
            if ss > 1:
                # the reference's own sensitivity with supersampling: sub-voxel
                # samples within FP32 rounding of a beamlet edge (a few per
                # fixture) resolve by the arithmetic's rounding, moving one
                # voxel's TERMA by up to a sub-voxel's share.  Max |change|
                # of dose and TERMA (relative to their maxima) when the
                # isocentre moves by 1e-6 .. 1e-5 cm along several directions.
                dn = tn = 0.0
                shifts = [(1, -1, 1), (-1, 1, -1), (1, 0, 0), (0, 1, 0), (0, 0, 1), (-1, -1, 0), (0, -1, 1), (1, 1, 1)]
                for j, sh in enumerate(shifts):
                    bp = inputs.Beam(**{**b.__dict__})
                    bp.isocenter = np.asarray(b.isocenter, np.float64) + (1e-5 if j % 2 == 0 else 1e-6) * np.array(sh)
                    d2, t2, _ = h.beam_dose(bp)
                    dn = max(dn, float(np.abs(d2 - dose).max() / dose.max()))
                    tn = max(tn, float(np.abs(t2 - terma).max() / terma.max()))
                out[f"beam{k}_ref_noise"] = [dn, tn]
            print(name, k, "Dmax", float(dose.max()), "bev", bev, "ref noise", out.get(f"beam{k}_ref_noise"))
        out["nbeams"] = len(beams)
        out["ss_factor"] = ss
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


if __name__ == "__main__":
    main()
