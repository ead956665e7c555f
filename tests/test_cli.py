"""dosecalc-beam (endtoend_gb300/_lib/dosecalc-beam, csrc/ee_dosecalc_beam.cpp)
on the CPU: it builds, answers --help, reads the reference's temp-directory
contract (tests/dosecalc_contract.py) with --dry-run exactly as
load_omni_header / load_omni_beam_list do, and fails with a message and a
non-zero status on missing or malformed inputs.  The dose itself is checked
on the GPU (tests/test_gpu_cli.py)."""
import os
import re
import subprocess

import numpy as np
import pytest

import dosecalc_contract as dc
from endtoend_gb300 import _build


@pytest.fixture(scope="module")
def cli():
    return _build.build_cli()


def run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=120)


def test_help(cli):
    r = run(cli, "--help")
    assert r.returncode == 0 and "--kernel=table|exp" in r.stdout


def test_dry_run_reads_the_contract(cli, tmp_path):
    vol, beams = dc.slab_case()
    temp, data = dc.write_contract(str(tmp_path), vol, beams, ss_factor=3)
    r = run(cli, f"--temp={temp}", f"--data={data}", "--dry-run")
    assert r.returncode == 0, r.stderr
    assert "size 32 32 32" in r.stdout and "ss_factor 3" in r.stdout and "nphi 6 ntheta 8" in r.stdout
    assert "(4 energies)" in r.stdout
    got = re.findall(r"beam (\d+): gantry (\S+) couch (\S+) coll (\S+) rad", r.stdout)
    assert len(got) == len(beams)
    for (k, g, c, cl), d in zip(got, beams):
        eb = dc.as_engine_beam(d)
        assert np.isclose(float(g), eb.azimuth, atol=1e-6) and np.isclose(float(c), eb.zenith, atol=1e-6)
        assert np.isclose(float(cl), eb.coll, atol=1e-6)
    assert "cone angles from the temp directory" in r.stdout


def test_beam_count_limits_the_list(cli, tmp_path):
    """load_omni_beam_list reads min(header beam_count, list count) beams."""
    vol, beams = dc.slab_case()
    temp, data = dc.write_contract(str(tmp_path), vol, beams, angle_files=False)
    dc.write_header(temp, vol, 8, 6, 0.25, 1.0, 2, "spec_synth")
    r = run(cli, f"--temp={temp}", f"--data={data}", "--dry-run")
    assert r.returncode == 0, r.stderr
    assert len(re.findall(r"^beam \d+:", r.stdout, flags=re.M)) == 2
    assert "cone angles from the kernel build" in r.stdout


def test_errors(cli, tmp_path):
    vol, beams = dc.slab_case()
    temp, data = dc.write_contract(str(tmp_path), vol, beams)
    r = run(cli, f"--temp={tmp_path}/nowhere", f"--data={data}", "--dry-run")
    assert r.returncode != 0 and "omni-header" in r.stderr
    r = run(cli, f"--temp={temp}", f"--data={data}", "--kernel=fast")
    assert r.returncode != 0 and "--kernel" in r.stderr
    os.remove(os.path.join(temp, "fluence_maps", "fmap-000001.raw"))
    r = run(cli, f"--temp={temp}", f"--data={data}", "--dry-run")
    assert r.returncode != 0 and "fmap-000001.raw" in r.stderr
    dc.write_beams(temp, beams)
    with open(os.path.join(temp, "density.raw"), "r+b") as f:
        f.truncate(1000)
    r = run(cli, f"--temp={temp}", f"--data={data}", "--dry-run")
    assert r.returncode != 0 and "density.raw" in r.stderr
    np.ascontiguousarray(vol.density, np.float32).tofile(os.path.join(temp, "density.raw"))
    lst = open(os.path.join(temp, "omni_beam_list.txt")).read().split("\n")
    lst[2] = " ".join(lst[2].split()[:10])
    open(os.path.join(temp, "omni_beam_list.txt"), "w").write("\n".join(lst))
    r = run(cli, f"--temp={temp}", f"--data={data}", "--dry-run")
    assert r.returncode != 0 and "beam record" in r.stderr
    dc.write_beams(temp, beams)
    os.remove(os.path.join(data, "dsa", "synth2"))
    r = run(cli, f"--temp={temp}", f"--data={data}", "--dry-run")
    assert r.returncode != 0 and "point kernel" in r.stderr


def test_beamlet_program_dry_run_and_errors(cli, tmp_path):
    bl = os.path.join(os.path.dirname(cli), "dosecalc-beamlet")
    r = run(bl, "--help")
    assert r.returncode == 0 and "--sparsify-threshold" in r.stdout
    vol, beams = dc.slab_case()
    beams[0]["fluence"][:2] = 0.0  # 16 beamlets without fluence: no column
    temp, data = dc.write_contract(str(tmp_path), vol, beams)
    r = run(bl, f"--temp={temp}", f"--data={data}", "--dry-run", "--thresh=1e-4")
    assert r.returncode == 0, r.stderr
    assert "3 beams, 176 beamlets with fluence, threshold 0.0001" in r.stdout
    assert "kernel_extent 2 cm" in r.stdout
    r = run(bl, f"--temp={temp}", f"--data={data}", "--dry-run", "--sparsify-threshold=abc")
    assert r.returncode != 0 and "threshold" in r.stderr


def test_beamlet_program_roi_list(cli, tmp_path):
    """dosecalc-beamlet reads an ROI list for the row reduction (dry run:
    parsing and mask files checked, no GPU work), and rejects a malformed
    list or a mask file that is too short."""
    bl = os.path.join(os.path.dirname(cli), "dosecalc-beamlet")
    vol, beams = dc.slab_case()
    temp, data = dc.write_contract(str(tmp_path), vol, beams)
    np.ones(4 * 5 * 6, np.uint8).tofile(os.path.join(temp, "ptv.raw"))
    lst = os.path.join(temp, "rois.txt")
    open(lst, "w").write("# name x0 y0 z0 nx ny nz mask\nptv 3 4 5 4 5 6 ptv.raw\n")
    r = subprocess.run([bl, f"--temp={temp}", f"--data={data}", "--dry-run", f"--roi-list={lst}"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ROI reduction: 1 ROIs" in r.stdout
    open(lst, "w").write("ptv 3 4 5 4 5 7 ptv.raw\n")  # 140 flags needed, 120 present
    r = subprocess.run([bl, f"--temp={temp}", f"--data={data}", "--dry-run", f"--roi-list={lst}"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "short" in (r.stdout + r.stderr)
    open(lst, "w").write("ptv 3 4 5\n")
    r = subprocess.run([bl, f"--temp={temp}", f"--data={data}", "--dry-run", f"--roi-list={lst}"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "malformed" in (r.stdout + r.stderr)
