"""CPU restatement of the reference's kernel-table build (test infrastructure
only: tests/, __graft_entry__.smoke() and bench.py's CPU leg may import it;
the engine never does).

Follows, in the reference's FP32 arithmetic and summation order:
  read_spectrum_file      CCCS/DoseCalcIO/spectra.cpp:7-62
  read_kernel             CCCS/DoseCalcIO/kernel.cpp:27-122
  make_poly_kernel        CCCS/DoseCalcIO/kernel.cpp:123-258
  make_cumulative_kernel  CCCS/DoseCalcIO/kernel.cpp:260-431
Parity is pinned against the reference's own sources, run on the CPU by
oracle/ref_harness (ref_kernel_harness.cpp), through the fixtures under
tests/golden/kernel written by tests/golden/make_golden.py.

Every value is a numpy float32 and every array operation is elementwise, so
each element sees the same sequence of IEEE single-precision roundings as
the reference's scalar loops (no fused multiply-add: x86-64 host code).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

NRADII = 24       # N_KERNEL_RADII, kernel.h:10
NANGLES = 48      # N_KERNEL_ANGLES, kernel.h:11
NCAT = 5          # N_KERNEL_CATEGORIES, kernel.h:12

_libc = C.CDLL(None)
_libc.strtof.restype = C.c_float
_libc.strtof.argtypes = [C.c_char_p, C.POINTER(C.c_char_p)]


def _f32(tok: str) -> np.float32:
    """fscanf("%f") of one token: the correctly rounded strtof value (a
    parse through double could round twice)."""
    return np.float32(_libc.strtof(tok.encode(), None))


def read_spectrum_file(path: str):
    """spectra.cpp:7-62: lines of `energy fluence mu mu_en kernel_file`, read
    until the first line that does not parse as five fields; fluence divided
    by its FP32 running sum."""
    toks = open(path).read().split()
    energy, fluence, mu, mu_en, names = [], [], [], [], []
    k = 0
    while k + 5 <= len(toks):
        try:
            vals = [_f32(t) for t in toks[k:k + 4]]
            float(toks[k]), float(toks[k + 1]), float(toks[k + 2]), float(toks[k + 3])
        except ValueError:
            break
        energy.append(vals[0]); fluence.append(vals[1]); mu.append(vals[2]); mu_en.append(vals[3])
        names.append(toks[k + 4])
        k += 5
    s = np.float32(0)
    for f in fluence:
        s = np.float32(s + f)
    fluence = [np.float32(f / s) for f in fluence]
    a = lambda v: np.array(v, np.float32)
    return a(energy), a(fluence), a(mu), a(mu_en), names


def read_mono_kernel(path: str) -> np.ndarray:
    """kernel.cpp:27-122: for theta (48) then radius (24), seven (value,
    uncertainty) pairs: the five categories, mean radius, mean angle.
    Returns the category values [5][48][24]."""
    toks = open(path).read().split()
    need = NANGLES * NRADII * 14
    if len(toks) < need:
        raise ValueError(f"{path}: {len(toks)} values, expected {need}")
    v = np.array([_f32(t) for t in toks[:need]], np.float32).reshape(NANGLES, NRADII, 7, 2)
    return np.ascontiguousarray(v[:, :, :NCAT, 0].transpose(2, 0, 1))


def read_radii(path: str) -> np.ndarray:
    """radii.dat: the 24 radial boundaries [cm] (kernel.cpp:61-66)."""
    return np.array([_f32(t) for t in open(path).read().split()[:NRADII]], np.float32)


def poly_kernel(energy, fluence, mu, mono):
    """kernel.cpp:145-207: per category, sum_e (phi_e E_e mu_e) k_e / sum_e
    (phi_e E_e mu_e), accumulated over e in order; the total is the sum of
    the five category values in category order.  mono: [nE][5][48][24]."""
    n = len(energy)
    w = [np.float32(np.float32(fluence[e] * energy[e]) * mu[e]) for e in range(n)]
    s = np.float32(0)
    for e in range(n):
        s = np.float32(s + w[e])
    cat = np.zeros((NCAT, NANGLES, NRADII), np.float32)
    for e in range(n):
        cat = cat + w[e] * mono[e]
    cat = cat / s
    total = np.zeros((NANGLES, NRADII), np.float32)
    for c in range(NCAT):
        total = total + cat[c]
    return total, cat


def cumulative_kernel(poly_total, poly_cat, ntheta: int):
    """kernel.cpp:364-396: sum each group of 48/ntheta polar bins in order,
    then a running sum over radius (categories and total separately)."""
    if NANGLES % ntheta:
        raise ValueError("ntheta must divide 48")
    g = NANGLES // ntheta
    tot = np.zeros((ntheta, NRADII), np.float32)
    cat = np.zeros((NCAT, ntheta, NRADII), np.float32)
    for t in range(ntheta):
        for k in range(g):
            tot[t] = tot[t] + poly_total[t * g + k]
            cat[:, t] = cat[:, t] + poly_cat[:, t * g + k]
    for r in range(1, NRADII):
        tot[:, r] = tot[:, r] + tot[:, r - 1]
        cat[:, :, r] = cat[:, :, r] + cat[:, :, r - 1]
    return tot, cat


def conv_angles(ntheta: int, nphi: int):
    """kernel.cpp:274-276, 398-408: angular boundaries (180/ntheta)(t+1) in
    FP32, cone theta = bin centre (FP32), phi = (p+0.5)*360/nphi (double,
    stored as FP32)."""
    step = np.float32(np.float32(180.0) / np.float32(ntheta))
    bound = [np.float32(step * np.float32(t + 1)) for t in range(ntheta + 1)]
    na = nphi * (ntheta // 2)
    th = np.zeros(na, np.float32)
    ph = np.zeros(na, np.float32)
    for p in range(nphi):
        for t in range(ntheta // 2):
            a = p * (ntheta // 2) + t
            lo = bound[t - 1] if t > 0 else np.float32(0)
            th[a] = np.float32(np.float32(0.5) * np.float32(bound[t] + lo))
            ph[a] = np.float32((p + 0.5) * 360.0 / nphi)
    return np.array(bound[:ntheta], np.float32), th, ph


def build_from_files(spectrum_path: str, kernel_dir: str, ntheta: int, nphi: int):
    """The whole chain from files, as the reference's preprocessing runs it."""
    energy, fluence, mu, mu_en, names = read_spectrum_file(spectrum_path)
    mono = np.stack([read_mono_kernel(os.path.join(kernel_dir, n)) for n in names])
    radii = read_radii(os.path.join(kernel_dir, "radii.dat"))
    ptot, pcat = poly_kernel(energy, fluence, mu, mono)
    tot, cat = cumulative_kernel(ptot, pcat, ntheta)
    bound, th, ph = conv_angles(ntheta, nphi)
    return dict(energy=energy, fluence=fluence, mu=mu, mu_en=mu_en, mono=mono, radii=radii,
                poly_total=ptot, poly_weights=pcat, cum_total=tot, cum_weights=cat,
                ang_bounds=bound, conv_theta=th, conv_phi=ph)
