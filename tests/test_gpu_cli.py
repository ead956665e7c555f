"""dosecalc-beam end to end on the GPU: the program reads the reference's
temp-directory contract (tests/dosecalc_contract.py), rebuilds the cumulative
kernel from the spectrum and point-kernel files, and writes Dose.raw.

- Its dose equals the same computation made through the library's Python API
  (same kernel tables, beams, supersampling, kernel mode) to 1e-6 of Dmax:
  beams are summed into the dose with float atomics, so the order of the
  additions, and with it the last bit of a voxel, can differ between runs.
- Against the FP64 oracle of the same tables: <= 1e-3 of Dmax without TERMA
  supersampling; <= 5e-3 with ss_factor 3, where a few sub-voxel samples sit
  within FP32 rounding of a beamlet edge and FP32 and FP64 decide them
  differently (each moves one voxel's TERMA by up to 1/27 of its share).
"""
import os
import subprocess

import numpy as np
import pytest

import dosecalc_contract as dc
import golden_cases
from endtoend_gb300 import _build, engine
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _library_dose(vol, beams, data, ss, mode):
    phys = engine.physics_from_kernel_files(os.path.join(data, "spectra", golden_cases.SYNTH_SPECTRUM + ".spec"),
                                            os.path.join(data, "dsa"), 8, 6, spacing_cm=0.25, penumbra_cm=1.0)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode=mode)
        e.set_terma_supersampling(ss)
        return e.beam_dose([dc.as_engine_beam(d) for d in beams]), phys


@pytest.mark.parametrize("ss,mode", [(1, "table"), (3, "table"), (1, "exp")])
def test_cli_dose(ss, mode, tmp_path):
    cli = _build.build_cli()
    vol, beams = dc.slab_case()
    temp, data = dc.write_contract(str(tmp_path), vol, beams, ss_factor=ss)
    out = tmp_path / "results" / "Dose.h5"
    r = subprocess.run([cli, f"--temp={temp}", f"--data={data}", f"--out={out}", f"--kernel={mode}", "--timing"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    print(r.stdout)
    dose = np.fromfile(tmp_path / "results" / "Dose.raw", np.float32).reshape(vol.density.shape)
    ref, phys = _library_dose(vol, beams, data, ss, mode)
    assert np.abs(dose - ref).max() <= 1e-6 * ref.max()
    if mode == "table":
        o = Oracle(vol, phys, kernel_mode=0, ss_factor=ss)
        od = sum(o.beam_dose(dc.as_engine_beam(d))[0] for d in beams)
        err = float(np.abs(dose - od).max() / od.max())
        print(f"ss_factor {ss}: dosecalc-beam vs FP64 oracle {err:.2e} of Dmax")
        assert err <= (1e-3 if ss == 1 else 5e-3)


def test_beamlet_program_columns(tmp_path):
    """dosecalc-beamlet's raw CSR files equal the library's beamlet columns
    for the same inputs (kernel extent and REV limits from the header)."""
    cli = _build.build_cli()
    bl = os.path.join(os.path.dirname(cli), "dosecalc-beamlet")
    vol, beams = dc.slab_case()
    for d in beams:
        d["fmap"], d["fluence"] = (4, 4), d["fluence"][:4, :4].copy()
        d["beamlet"] = (1.0, 1.0)
    beams[1]["fluence"][0, :] = 0.0
    temp, data = dc.write_contract(str(tmp_path), vol, beams)
    out = tmp_path / "res" / "Dose_Coefficients.h5"
    r = subprocess.run([bl, f"--temp={temp}", f"--data={data}", f"--out={out}", "--thresh=1e-4", "--timing"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    print(r.stdout)
    odir = tmp_path / "res" / "Dose_Coefficients"
    specs = dict(l.split(" ", 1) for l in (odir / "calc_specs.txt").read_text().splitlines())
    assert specs["N_beams"] == "3" and float(specs["sparsity_thresh"]) == np.float32(1e-4)
    phys = engine.physics_from_kernel_files(os.path.join(data, "spectra", golden_cases.SYNTH_SPECTRUM + ".spec"),
                                            os.path.join(data, "dsa"), 8, 6, spacing_cm=0.25, penumbra_cm=1.0)
    n = vol.nvoxels
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="table")
        e.set_beamlet_options(2.0, (400, 400, 400))
        for b, d in enumerate(beams):
            bidx, cp, rows, vals = e.beamlet_columns(dc.as_engine_beam(d), 1e-4)
            got_idx = np.fromfile(odir / f"beam_{b:05d}_beamlet_index.raw", np.int32)
            got_cp = np.fromfile(odir / f"beam_{b:05d}_col_ptr.raw", np.int64)
            got_rows = np.fromfile(odir / f"beam_{b:05d}_lindex.raw", np.uint32)
            got_vals = np.fromfile(odir / f"beam_{b:05d}_coeffs.raw", np.float32)
            np.testing.assert_array_equal(got_idx, bidx)
            assert len(got_idx) == int((d["fluence"] > 0).sum())
            assert got_cp[0] == 0 and got_cp[-1] == len(got_rows) == len(got_vals)
            for c in range(len(bidx)):
                g = np.zeros(n, np.float32)
                g[got_rows[got_cp[c]:got_cp[c + 1]]] = got_vals[got_cp[c]:got_cp[c + 1]]
                ref = np.zeros(n, np.float32)
                ref[rows[cp[c]:cp[c + 1]]] = vals[cp[c]:cp[c + 1]]
                assert np.abs(g - ref).max() <= 1e-6 * ref.max(), (b, c)


def test_beamlet_program_roi_reduction(tmp_path):
    """dosecalc-beamlet with ROI masks (--roi-list): every column reduced to
    the ROI row blocks equals the loop-for-loop restatement of the
    reference's _reduce_by_roi (oracle/sparse_io.py) applied to the
    library's columns for the same inputs (values to 1e-6 of the column
    maximum); calc_specs lists the ROI order and capacities."""
    from oracle.sparse_io import reduce_by_roi

    cli = _build.build_cli()
    bl = os.path.join(os.path.dirname(cli), "dosecalc-beamlet")
    vol, beams = dc.slab_case()
    for d in beams:
        d["fmap"], d["fluence"] = (4, 4), d["fluence"][:4, :4].copy()
        d["beamlet"] = (1.0, 1.0)
    temp, data = dc.write_contract(str(tmp_path), vol, beams)
    nx, ny, nz = (int(v) for v in vol.size)
    rng = np.random.default_rng(3)
    rois, lines = [], []
    for k, (c0, cn) in enumerate([((4, 6, 5), (20, 18, 22)), ((0, 0, 0), (nx, ny, nz)), ((10, 12, 8), (9, 7, 11))]):
        m = rng.random((cn[2], cn[1], cn[0])) < (0.5 if k != 1 else 0.2)
        m.astype(np.uint8).tofile(os.path.join(temp, f"roi{k}.raw"))
        rois.append((c0, m))
        lines.append(f"roi{k} {c0[0]} {c0[1]} {c0[2]} {cn[0]} {cn[1]} {cn[2]} roi{k}.raw")
    lst = os.path.join(temp, "rois_for_test.txt")
    open(lst, "w").write("# name x0 y0 z0 nx ny nz mask\n" + "\n".join(lines) + "\n")
    out = tmp_path / "res" / "Dose_Coefficients.h5"
    r = subprocess.run([bl, f"--temp={temp}", f"--data={data}", f"--out={out}", "--thresh=1e-4",
                        f"--roi-list={lst}"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    odir = tmp_path / "res" / "Dose_Coefficients"
    specs = dict(l.split(" ", 1) for l in (odir / "calc_specs.txt").read_text().splitlines())
    assert specs["roi_order"].split() == ["roi0", "roi1", "roi2"]
    caps = [int(v) for v in specs["row_block_capacities"].split()]
    assert caps == [int(m.sum()) for _, m in rois]
    phys = engine.physics_from_kernel_files(os.path.join(data, "spectra", golden_cases.SYNTH_SPECTRUM + ".spec"),
                                            os.path.join(data, "dsa"), 8, 6, spacing_cm=0.25, penumbra_cm=1.0)
    nrows = sum(caps)
    with engine.Engine(0) as e:
        e.set_volume(vol)
        e.set_physics(phys, mode="table")
        e.set_beamlet_options(2.0, (400, 400, 400))
        for b, d in enumerate(beams):
            bidx, cp, rows, vals = e.beamlet_columns(dc.as_engine_beam(d), 1e-4)
            got_cp = np.fromfile(odir / f"beam_{b:05d}_col_ptr.raw", np.int64)
            got_keys = np.fromfile(odir / f"beam_{b:05d}_lindex.raw", np.uint64)
            got_vals = np.fromfile(odir / f"beam_{b:05d}_coeffs.raw", np.float32)
            got_blk = np.fromfile(odir / f"beam_{b:05d}_row_blocks.raw", np.int64).reshape(len(bidx), 3)
            assert got_cp[-1] == len(got_keys) == len(got_vals)
            for c in range(len(bidx)):
                rk, rv, rb = reduce_by_roi(rows[cp[c]:cp[c + 1]], vals[cp[c]:cp[c + 1]], (nx, ny, nz), rois)
                g = np.zeros(nrows, np.float32)
                g[got_keys[got_cp[c]:got_cp[c + 1]].astype(np.int64)] = got_vals[got_cp[c]:got_cp[c + 1]]
                ref = np.zeros(nrows, np.float32)
                ref[rk.astype(np.int64)] = rv
                assert np.abs(g - ref).max() <= 1e-6 * max(float(vals[cp[c]:cp[c + 1]].max()), 1e-30), (b, c)
                np.testing.assert_array_equal(got_blk[c], rb)
                assert np.all(np.diff(got_keys[got_cp[c]:got_cp[c + 1]].astype(np.int64)) > 0)
