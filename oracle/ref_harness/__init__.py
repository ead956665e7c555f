"""ctypes front end of the reference harness (test infrastructure only): the
reference's own dosecalc-beam kernel source executed on the CPU.  Needs the
reference checkout (see build.py); tests skip it when that is absent."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build


class RefSetup(C.Structure):
    _fields_ = [("size", C.c_int * 3), ("voxel", C.c_float * 3), ("start", C.c_float * 3),
                ("bbox_start", C.c_int * 3), ("bbox_size", C.c_int * 3), ("density", C.POINTER(C.c_float)),
                ("nE", C.c_int), ("energy", C.POINTER(C.c_float)), ("fluence", C.POINTER(C.c_float)),
                ("mu", C.POINTER(C.c_float)), ("mu_en", C.POINTER(C.c_float)),
                ("ntheta", C.c_int), ("nphi", C.c_int), ("nradii", C.c_int),
                ("radii", C.POINTER(C.c_float)), ("cumkern", C.POINTER(C.c_float)),
                ("theta_deg", C.POINTER(C.c_float)), ("phi_deg", C.POINTER(C.c_float)),
                ("rev_latspacing", C.c_float), ("rev_longspacing", C.c_float), ("penumbra", C.c_float),
                ("tex_emulate", C.c_int), ("nthreads", C.c_int), ("ss_factor", C.c_int)]


class RefBeam(C.Structure):
    _fields_ = [("azimuth", C.c_float), ("zenith", C.c_float), ("coll", C.c_float), ("iso", C.c_float * 3),
                ("sad", C.c_float), ("fmap", C.c_int * 2), ("beamlet", C.c_float * 2)]


available = _build.available
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        lib = C.CDLL(_build.build())
        lib.ccref_beam_dose.argtypes = [C.POINTER(RefSetup), C.POINTER(RefBeam), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int)]
        lib.ccref_beam_dose.restype = C.c_int
        _LIB = lib
    return _LIB


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class ReferenceHarness:
    """The reference's cudaSiddon / cudaRaytrace / RowConvolve / REV2XYZdose
    kernels (cumulative-kernel table) run on the CPU for one beam."""

    def __init__(self, vol, phys, tex_emulate=True, nthreads=None, ss_factor=1):
        self.lib = _lib()
        self.vol, self.phys = vol, phys
        keep = self._keep = []

        def farr(x):
            a = np.ascontiguousarray(np.asarray(x, dtype=np.float32).ravel())
            keep.append(a)
            return _fp(a)

        s = RefSetup()
        s.size[:] = [int(v) for v in vol.size]
        s.voxel[:] = [float(v) for v in vol.voxel]
        s.start[:] = [float(v) for v in vol.start]
        s.bbox_start[:] = [int(v) for v in vol.bbox_start]
        s.bbox_size[:] = [int(v) for v in vol.bbox_size]
        s.density = farr(vol.density)
        fl = np.asarray(phys.fluence, np.float64)
        s.nE = len(phys.energy)
        s.energy, s.fluence, s.mu, s.mu_en = farr(phys.energy), farr(fl / fl.sum()), farr(phys.mu), farr(phys.mu_en)
        s.ntheta, s.nphi, s.nradii = phys.ntheta, phys.nphi, phys.nradii
        s.radii, s.cumkern = farr(phys.radii), farr(phys.cumkern)
        s.theta_deg, s.phi_deg = farr(phys.theta_deg), farr(phys.phi_deg)
        s.rev_latspacing, s.rev_longspacing, s.penumbra = phys.rev_latspacing, phys.rev_longspacing, phys.penumbra
        s.tex_emulate = int(bool(tex_emulate))
        s.nthreads = int(nthreads or os.cpu_count() or 1)
        s.ss_factor = int(ss_factor)
        self.setup = s

    def beam_dose(self, beam):
        b = RefBeam()
        b.azimuth, b.zenith, b.coll = beam.azimuth, beam.zenith, beam.coll
        b.iso[:] = [float(v) for v in beam.isocenter]
        b.sad = beam.sad
        b.fmap[:] = [int(v) for v in beam.fmap_size]
        b.beamlet[:] = [float(v) for v in beam.beamlet_size]
        fl = np.ascontiguousarray(beam.fluence, np.float32).ravel()
        dose = np.zeros(self.vol.density.shape, np.float32)
        bs = self.vol.bbox_size
        terma = np.zeros((bs[2], bs[1], bs[0]), np.float32)
        info = (C.c_int * 4)()
        st = self.lib.ccref_beam_dose(C.byref(self.setup), C.byref(b), _fp(fl), _fp(dose), _fp(terma), info)
        if st != 0:
            raise RuntimeError(f"reference harness status {st}")
        return dose, terma, list(info)[:3]


_LIB_BL = None


def _lib_beamlet():
    global _LIB_BL
    if _LIB_BL is None:
        lib = C.CDLL(_build.build(which="beamlet"))
        lib.ccref_beamlet_columns.argtypes = [C.POINTER(RefSetup), C.POINTER(RefBeam), C.POINTER(C.c_float), C.c_float,
                                              C.POINTER(C.c_int), C.c_float, C.c_int, C.POINTER(C.c_float),
                                              C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.ccref_beamlet_columns.restype = C.c_int
        _LIB_BL = lib
    return _LIB_BL


def sparsify(column, thresh, bbox_start, size):
    """dcio::_sparsify (CCCS/DoseCalcIO/sparse_io.cpp:22-59): keep the voxels
    of a dense calc-bbox column whose value exceeds thresh * column max, keyed
    by their linear index on the full grid.  Returned sorted by key."""
    col = np.asarray(column, np.float32)
    vmax = float(col.max()) if col.size else 0.0
    keep = col > np.float32(thresh) * np.float32(vmax)
    kz, ky, kx = np.nonzero(keep)
    nx, ny = int(size[0]), int(size[1])
    keys = ((kz + int(bbox_start[2])) * ny + (ky + int(bbox_start[1]))) * nx + (kx + int(bbox_start[0]))
    order = np.argsort(keys, kind="stable")
    return keys[order].astype(np.int64), col[keep][order]


class BeamletHarness(ReferenceHarness):
    """The reference's dosecalc-beamlet kernels (cudaBeamletRaytrace,
    PackRowConvolve, PackedREVtoBEVdose, UnpackBEVDosePillar) run on the CPU."""

    def __init__(self, vol, phys, tex_emulate=True, nthreads=None):
        super().__init__(vol, phys, tex_emulate=tex_emulate, nthreads=nthreads)
        self.lib = _lib_beamlet()

    def columns(self, beam, kernel_extent=2.0, max_rev_size=(500, 500, 500), rev_jitter=0.0):
        """(fluence-map indices of the active beamlets, dense calc-bbox
        columns [n, bz, by, bx], info: [active, pillar dims x3, batches, ...])."""
        b = RefBeam()
        b.azimuth, b.zenith, b.coll = beam.azimuth, beam.zenith, beam.coll
        b.iso[:] = [float(v) for v in beam.isocenter]
        b.sad = beam.sad
        b.fmap[:] = [int(v) for v in beam.fmap_size]
        b.beamlet[:] = [float(v) for v in beam.beamlet_size]
        fl = np.ascontiguousarray(beam.fluence, np.float32).ravel()
        n = int((fl > 0).sum())
        bs = self.vol.bbox_size
        cols = np.zeros((max(n, 1), bs[2], bs[1], bs[0]), np.float32)
        idx = np.zeros(max(n, 1), np.int32)
        info = (C.c_int * 8)()
        mr = (C.c_int * 3)(*[int(v) for v in max_rev_size])
        st = self.lib.ccref_beamlet_columns(C.byref(self.setup), C.byref(b), _fp(fl), float(kernel_extent), mr,
                                            float(rev_jitter), max(n, 1),
                                            _fp(cols), idx.ctypes.data_as(C.POINTER(C.c_int)), info)
        if st != 0:
            raise RuntimeError(f"reference beamlet harness status {st}")
        return idx[:n], cols[:n], list(info)


_LIB_KT = None


def _lib_kernel():
    global _LIB_KT
    if _LIB_KT is None:
        lib = C.CDLL(_build.build(which="kernel"))
        lib.ccref_kernel_build.restype = C.c_int
        _LIB_KT = lib
    return _LIB_KT


def kernel_build(data_dir: str, spectrum: str, ntheta: int = 8, nphi: int = 6) -> dict:
    """The reference's own spectrum + kernel-table build (read_spectrum_file,
    read_kernel, make_poly_kernel, make_cumulative_kernel) run on the CPU on
    data_dir/spectra/<spectrum>.spec and data_dir/dsa/*."""
    lib = _lib_kernel()
    tmp = os.path.join(_build.OUT, "tmp")
    os.makedirs(tmp, exist_ok=True)
    z = lambda *s: np.zeros(s, np.float32)
    nang = nphi * (ntheta // 2)
    sp = [z(64) for _ in range(4)]
    out = dict(poly_total=z(48, 24), poly_weights=z(5, 48, 24), cum_total=z(ntheta, 24),
               cum_weights=z(5, ntheta, 24), radii=z(24), ang_bounds=z(ntheta), conv_theta=z(nang), conv_phi=z(nang))
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    n = lib.ccref_kernel_build(os.fsencode(data_dir), os.fsencode(tmp), spectrum.encode(), int(nphi), int(ntheta),
                               *[p(a) for a in sp], *[p(out[k]) for k in ("poly_total", "poly_weights", "cum_total",
                                                                          "cum_weights", "radii", "ang_bounds",
                                                                          "conv_theta", "conv_phi")])
    if n <= 0:
        raise RuntimeError(f"reference kernel build failed for {spectrum} ({n})")
    out.update(energy=sp[0][:n].copy(), fluence=sp[1][:n].copy(), mu=sp[2][:n].copy(), mu_en=sp[3][:n].copy())
    return out
