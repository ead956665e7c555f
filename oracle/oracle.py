"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module; the engine never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_MAX_RAYS = 256


class OrcSetup(C.Structure):
    _fields_ = [
        ("size", C.c_int * 3), ("voxel", C.c_double * 3), ("start", C.c_double * 3),
        ("bbox_start", C.c_int * 3), ("bbox_size", C.c_int * 3),
        ("density", C.POINTER(C.c_float)),
        ("nE", C.c_int),
        ("energy", C.POINTER(C.c_double)), ("fluence", C.POINTER(C.c_double)),
        ("mu", C.POINTER(C.c_double)), ("mu_en", C.POINTER(C.c_double)),
        ("ntheta", C.c_int), ("nphi", C.c_int), ("nradii", C.c_int),
        ("radii", C.POINTER(C.c_double)), ("cumkern", C.POINTER(C.c_double)),
        ("exp_params", C.POINTER(C.c_double)),
        ("theta_deg", C.POINTER(C.c_double)), ("phi_deg", C.POINTER(C.c_double)),
        ("kernel_mode", C.c_int),
        ("rev_latspacing", C.c_double), ("rev_longspacing", C.c_double), ("penumbra", C.c_double),
        ("max_rev_size", C.c_int * 3),
        ("tex_emulate", C.c_int), ("nthreads", C.c_int), ("ss_factor", C.c_int),
    ]


class OrcBeam(C.Structure):
    _fields_ = [
        ("azimuth", C.c_double), ("zenith", C.c_double), ("coll", C.c_double),
        ("iso", C.c_double * 3), ("sad", C.c_double),
        ("fmap", C.c_int * 2), ("beamlet", C.c_double * 2),
    ]


class OrcBeamInfo(C.Structure):
    _fields_ = [
        ("source", C.c_double * 3), ("direction", C.c_double * 3),
        ("azimuth", C.c_double), ("zenith", C.c_double),
        ("b_min", C.c_double * 3), ("b_max", C.c_double * 3),
        ("bev_size", C.c_int * 3), ("lim_min", C.c_double * 3),
        ("nrays", C.c_int),
        ("rev_size", (C.c_int * 3) * _MAX_RAYS), ("rev_min", (C.c_double * 3) * _MAX_RAYS),
        ("v_beam", C.c_long), ("n_terma_nonzero", C.c_long), ("status", C.c_int),
    ]


_LIBS = {}


def _lib(precision: int = 64):
    if precision not in _LIBS:
        paths = _build.build()
        path = paths[0] if precision == 64 else paths[1]
        lib = C.CDLL(path)
        real = C.c_double if precision == 64 else C.c_float
        rp = C.POINTER(real)
        for name, args in (
            ("orc_beam_dose", [C.POINTER(OrcSetup), C.POINTER(OrcBeam), C.POINTER(C.c_float), rp, rp, C.POINTER(OrcBeamInfo)]),
            ("orc_beam_terma", [C.POINTER(OrcSetup), C.POINTER(OrcBeam), C.POINTER(C.c_float), rp, C.POINTER(OrcBeamInfo)]),
            ("orc_beam_dose_adjoint", [C.POINTER(OrcSetup), C.POINTER(OrcBeam), C.POINTER(C.c_float), rp, rp, C.POINTER(OrcBeamInfo)]),
        ):
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int
        lib.orc_row_convolve.argtypes = [C.POINTER(OrcSetup), rp, rp, C.c_int, C.c_int, rp]
        lib.orc_row_convolve.restype = None
        lib.orc_row_convolve_T.argtypes = [C.POINTER(OrcSetup), rp, rp, C.c_int, C.c_int, rp]
        lib.orc_row_convolve_T.restype = None
        lib.orc_rotate.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]
        lib.orc_rotate.restype = None
        lib.orc_iso_size.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_int)]
        lib.orc_iso_size.restype = None
        lib.orc_ct_to_density.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_double,
                                          C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int, C.c_int, rp]
        lib.orc_ct_to_density.restype = C.c_int
        lib.orc_fluence_projection.argtypes = [C.POINTER(OrcSetup), C.POINTER(OrcBeam), C.c_int, C.POINTER(C.c_float)]
        lib.orc_fluence_projection.restype = C.c_int
        lib.orc_aperture_ready.argtypes = [C.POINTER(C.c_float), C.c_int, C.c_int, C.c_float]
        lib.orc_aperture_ready.restype = None
        assert lib.orc_sizeof_info() == C.sizeof(OrcBeamInfo), "OrcBeamInfo layout mismatch"
        assert lib.orc_sizeof_setup() == C.sizeof(OrcSetup), "OrcSetup layout mismatch"
        lib._real = real
        lib._np = np.float64 if precision == 64 else np.float32
        _LIBS[precision] = lib
    return _LIBS[precision]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _rp(lib, a):
    return a.ctypes.data_as(C.POINTER(lib._real))


class Oracle:
    """CPU restatement of the reference dosecalc-beam chain.

    kernel_mode: 0 = cumulative table (reference), 1 = exact double
    exponential on the reference walk, 2 = O(L) recurrence (same operator as
    1 without radial truncation).  tex_emulate=True rounds texture filter
    weights to 8 fractional bits like the GPU texture unit.  ss_factor > 1
    supersamples TERMA with ss^3 sub-voxels per voxel (forward only).
    """

    def __init__(self, vol, phys, kernel_mode=0, tex_emulate=False, precision=64, nthreads=None,
                 max_rev_size=(0, 0, 0), ss_factor=1):
        self.lib = _lib(precision)
        self.vol, self.phys = vol, phys
        self._keep = []
        keep = self._keep
        dens = np.ascontiguousarray(vol.density, dtype=np.float32)
        keep.append(dens)

        def darr(x):
            # values rounded to float32 first: the engine receives float32
            # through its C ABI, so the oracle evaluates the same numbers
            a = np.ascontiguousarray(np.asarray(x, dtype=np.float32).astype(np.float64).ravel())
            keep.append(a)
            return _dp(a)

        s = OrcSetup()
        s.size[:] = [int(v) for v in vol.size]
        f32 = lambda v: float(np.float32(v))
        s.voxel[:] = [f32(v) for v in vol.voxel]
        s.start[:] = [f32(v) for v in vol.start]
        s.bbox_start[:] = [int(v) for v in vol.bbox_start]
        s.bbox_size[:] = [int(v) for v in vol.bbox_size]
        s.density = dens.ctypes.data_as(C.POINTER(C.c_float))
        s.nE = len(phys.energy)
        s.energy, s.fluence, s.mu, s.mu_en = (darr(phys.energy), darr(phys.fluence), darr(phys.mu), darr(phys.mu_en))
        s.ntheta, s.nphi, s.nradii = phys.ntheta, phys.nphi, phys.nradii
        s.radii = darr(phys.radii)
        s.cumkern = darr(phys.cumkern)
        s.exp_params = darr(phys.exp_params)
        s.theta_deg, s.phi_deg = darr(phys.theta_deg), darr(phys.phi_deg)
        s.kernel_mode = int(kernel_mode)
        s.rev_latspacing, s.rev_longspacing, s.penumbra = (f32(phys.rev_latspacing), f32(phys.rev_longspacing),
                                                            f32(phys.penumbra))
        s.max_rev_size[:] = list(max_rev_size)
        s.tex_emulate = int(bool(tex_emulate))
        s.nthreads = int(nthreads or os.cpu_count() or 1)
        s.ss_factor = int(ss_factor)
        self.setup = s

    def _beam(self, b):
        f32 = lambda v: float(np.float32(v))
        ob = OrcBeam()
        ob.azimuth, ob.zenith, ob.coll = f32(b.azimuth), f32(b.zenith), f32(b.coll)
        ob.iso[:] = [f32(v) for v in b.isocenter]
        ob.sad = f32(b.sad)
        ob.fmap[:] = [int(v) for v in b.fmap_size]
        ob.beamlet[:] = [f32(v) for v in b.beamlet_size]
        fl = np.ascontiguousarray(b.fluence, dtype=np.float32).ravel()
        return ob, fl

    @staticmethod
    def _check(st, what):
        if st != 0:
            raise RuntimeError(f"oracle {what} failed with status {st}")

    def beam_dose(self, beam, return_terma=False):
        """Dose of one beam on the full grid [nz, ny, nx], plus beam info."""
        lib = self.lib
        ob, fl = self._beam(beam)
        nz, ny, nx = self.vol.density.shape
        dose = np.zeros((nz, ny, nx), dtype=lib._np)
        bs = self.vol.bbox_size
        terma = np.zeros((bs[2], bs[1], bs[0]), dtype=lib._np)
        info = OrcBeamInfo()
        st = lib.orc_beam_dose(C.byref(self.setup), C.byref(ob), fl.ctypes.data_as(C.POINTER(C.c_float)),
                               _rp(lib, dose), _rp(lib, terma), C.byref(info))
        self._check(st, "beam_dose")
        return (dose, info, terma) if return_terma else (dose, info)

    def beam_terma(self, beam):
        lib = self.lib
        ob, fl = self._beam(beam)
        bs = self.vol.bbox_size
        terma = np.zeros((bs[2], bs[1], bs[0]), dtype=lib._np)
        info = OrcBeamInfo()
        st = lib.orc_beam_terma(C.byref(self.setup), C.byref(ob), fl.ctypes.data_as(C.POINTER(C.c_float)),
                                _rp(lib, terma), C.byref(info))
        self._check(st, "beam_terma")
        return terma, info

    def beam_dose_adjoint(self, beam, dose_grad):
        lib = self.lib
        ob, fl = self._beam(beam)
        g = np.ascontiguousarray(dose_grad, dtype=lib._np)
        out = np.zeros(beam.fluence.shape, dtype=lib._np)
        info = OrcBeamInfo()
        st = lib.orc_beam_dose_adjoint(C.byref(self.setup), C.byref(ob), fl.ctypes.data_as(C.POINTER(C.c_float)),
                                       _rp(lib, g), _rp(lib, out), C.byref(info))
        self._check(st, "beam_dose_adjoint")
        return out, info

    def row_convolve(self, dens, terma, P):
        lib = self.lib
        d = np.ascontiguousarray(dens, dtype=lib._np)
        t = np.ascontiguousarray(terma, dtype=lib._np)
        out = np.zeros_like(d)
        lib.orc_row_convolve(C.byref(self.setup), _rp(lib, d), _rp(lib, t), len(d), int(P), _rp(lib, out))
        return out

    def row_convolve_T(self, dens, g, P):
        lib = self.lib
        d = np.ascontiguousarray(dens, dtype=lib._np)
        gg = np.ascontiguousarray(g, dtype=lib._np)
        out = np.zeros_like(d)
        lib.orc_row_convolve_T(C.byref(self.setup), _rp(lib, d), _rp(lib, gg), len(d), int(P), _rp(lib, out))
        return out


def rotate(which, vec, a, b, c=0.0, precision=64):
    """which: 0 RCS->BEV, 1 BEV->RCS, 2 BEV->REV, 3 REV->BEV."""
    lib = _lib(precision)
    v = np.ascontiguousarray(vec, dtype=np.float64)
    out = np.zeros(3)
    lib.orc_rotate(int(which), _dp(v), float(a), float(b), float(c), _dp(out))
    return out


# ---- preprocessing (CCCS/dosecalc-preprocess) ----
def ct_to_density(hu, voxel, iso_voxel, lut=None, tex_emulate=1, precision=64):
    """Isotropic density from a CT volume [nz, ny, nx] in HU (cudaMakeIsotropicWithLUT,
    or the linear HU rule without a LUT).  lut: (hu values, densities), sorted.
    tex_emulate: 0 exact, 1 rounded, 2 truncated 8-bit filter weights."""
    lib = _lib(precision)
    hu = np.ascontiguousarray(hu, np.float32)
    size = (C.c_int * 3)(hu.shape[2], hu.shape[1], hu.shape[0])
    vox = (C.c_double * 3)(*[float(np.float32(v)) for v in voxel])
    out_size = (C.c_int * 3)()
    lib.orc_iso_size(size, vox, float(np.float32(iso_voxel)), out_size)
    nx, ny, nz = list(out_size)
    out = np.zeros((nz, ny, nx), dtype=lib._np)
    if lut is not None:
        lh = np.ascontiguousarray(np.asarray(lut[0], np.float32).astype(np.float64))
        ld = np.ascontiguousarray(np.asarray(lut[1], np.float32).astype(np.float64))
        n = len(lh)
    else:
        lh = ld = np.zeros(1)
        n = 0
    st = lib.orc_ct_to_density(hu.ctypes.data_as(C.POINTER(C.c_float)), size, vox, float(np.float32(iso_voxel)),
                               _dp(lh), _dp(ld), n, int(tex_emulate), _rp(lib, out))
    if st != 0:
        raise RuntimeError(f"oracle ct_to_density failed with status {st}")
    return out


def fluence_projection(mask_vol, beam, supersample=True, tex_emulate=True, precision=64):
    """Binary conformal fluence map of `beam` through the mask volume
    (cudaRaycast); mask_vol is an inputs.Volume whose density is the mask."""
    o = Oracle(mask_vol, _dummy_physics(), tex_emulate=tex_emulate, precision=precision)
    ob, _ = o._beam(beam)
    fm = np.zeros((int(beam.fmap_size[1]), int(beam.fmap_size[0])), np.float32)
    st = o.lib.orc_fluence_projection(C.byref(o.setup), C.byref(ob), int(bool(supersample)),
                                      fm.ctypes.data_as(C.POINTER(C.c_float)))
    if st != 0:
        raise RuntimeError(f"oracle fluence_projection failed with status {st}")
    return fm


def aperture_ready(fmap, fill=1.0):
    """fmap_post_apertureready on a [fy, fx] map (returns a copy)."""
    lib = _lib(64)
    f = np.ascontiguousarray(fmap, np.float32).copy()
    lib.orc_aperture_ready(f.ctypes.data_as(C.POINTER(C.c_float)), f.shape[1], f.shape[0], float(fill))
    return f


def _dummy_physics():
    import types
    z = np.zeros(1)
    return types.SimpleNamespace(energy=z + 1, fluence=z + 1, mu=z, mu_en=z, ntheta=2, nphi=1, nradii=1, radii=z + 1,
                                 cumkern=np.zeros((2, 1)), exp_params=np.zeros((2, 4)) + 1, theta_deg=z, phi_deg=z,
                                 rev_latspacing=1.0, rev_longspacing=1.0, penumbra=1.0)
