"""Seeded synthetic inputs for the CCCS dose engine.

There is no public dataset for this path, so every workload is generated
here from a seed: phantoms, a 6 MV-like polyenergetic spectrum, a
double-exponential collapsed-cone kernel per zenith bin, beam lists and
fluence maps.  Units follow the reference engine: centimetres, radians for
beam angles, degrees for the convolution-cone angles.

The cumulative-kernel table and cone-angle layout follow the reference's
preprocessing (CCCS/DoseCalcIO/kernel.cpp:374-408): ntheta zenith bins of
180/ntheta degrees, cone theta = bin centre, phi = (p + 0.5) * 360 / nphi,
ray index = p * ntheta/2 + t.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

# Radial boundaries of the reference's kernel tables [cm]
# (CCCS/data/dsa/radii.dat, 24 values).
KERNEL_RADII_CM = np.array(
    [0.05, 0.1, 0.15, 0.2, 0.3, 0.4, 0.5, 0.6, 0.8, 1.0, 1.5, 2.0, 3.0, 4.0, 5.0, 6.0,
     8.0, 10.0, 15.0, 20.0, 30.0, 40.0, 50.0, 60.0], dtype=np.float64)


# Default isocentre: a generic sub-voxel offset (<= 0.13 mm) from the phantom
# centre.  The reference's Siddon trace starts all three plane-crossing
# parameters at a common a_min (cudaSiddon.cu:69-72), so on a grid where
# source-to-voxel vectors have rational component ratios, exact ties between
# crossings are common and resolve by floating-point rounding; likewise voxel
# centres can sit exactly on a field-edge ray.  The offset makes the
# geometry generic, so FP32 and FP64 evaluations of the same algorithm agree.
ISO_OFFSET_CM = (0.0131, 0.0077, -0.0093)


@dataclasses.dataclass
class Volume:
    density: np.ndarray          # float32 [nz, ny, nx], x fastest
    voxel: np.ndarray            # (3,) cm
    start: np.ndarray            # (3,) cm, centre of voxel (0, 0, 0)
    bbox_start: np.ndarray       # (3,) int
    bbox_size: np.ndarray        # (3,) int
    masks: dict = dataclasses.field(default_factory=dict)  # name -> bool [nz, ny, nx]

    @property
    def size(self):
        nz, ny, nx = self.density.shape
        return np.array([nx, ny, nz], dtype=np.int64)

    @property
    def nvoxels(self):
        return int(self.density.size)


@dataclasses.dataclass
class Physics:
    energy: np.ndarray
    fluence: np.ndarray      # normalised to unit sum (spectra.cpp:56-58)
    mu: np.ndarray
    mu_en: np.ndarray
    ntheta: int
    nphi: int
    radii: np.ndarray        # (nradii,) cm
    exp_params: np.ndarray   # (ntheta, 4): A, a, B, b
    cumkern: np.ndarray      # (ntheta, nradii)
    theta_deg: np.ndarray    # (nrays,)
    phi_deg: np.ndarray      # (nrays,)
    rev_latspacing: float
    rev_longspacing: float
    penumbra: float

    @property
    def nrays(self):
        return self.nphi * (self.ntheta // 2)

    @property
    def nradii(self):
        return int(self.radii.size)


@dataclasses.dataclass
class Beam:
    azimuth: float            # gantry [rad]
    zenith: float             # couch [rad]
    coll: float               # collimator [rad]
    isocenter: np.ndarray     # (3,) cm
    sad: float                # cm
    fmap_size: tuple          # (fx, fy)
    beamlet_size: tuple       # (bx, by) cm
    fluence: np.ndarray       # float32 [fy, fx]


def cone_angles(ntheta: int, nphi: int):
    """Convolution cone angles in degrees (kernel.cpp:398-408)."""
    bound = [(180.0 / ntheta) * (t + 1) for t in range(ntheta + 1)]
    th = np.zeros(nphi * (ntheta // 2))
    ph = np.zeros_like(th)
    for p in range(nphi):
        for t in range(ntheta // 2):
            a = p * (ntheta // 2) + t
            th[a] = np.float32(0.5 * (bound[t] + (bound[t - 1] if t > 0 else 0.0)))
            ph[a] = np.float32((p + 0.5) * 360.0 / nphi)
    return th, ph


def cumulative_table(exp_params: np.ndarray, radii: np.ndarray) -> np.ndarray:
    """K_theta(r_k) = A/a (1 - e^{-a r_k}) + B/b (1 - e^{-b r_k})."""
    A, a, B, b = (exp_params[:, i:i + 1] for i in range(4))
    r = radii[None, :]
    return A / a * (1 - np.exp(-a * r)) + B / b * (1 - np.exp(-b * r))


def make_physics(seed: int = 0, ntheta: int = 8, nphi: int = 6, nE: int = 10,
                 spacing_cm: float = 0.25, penumbra_cm: float = 1.0) -> Physics:
    """6 MV-like spectrum + seeded double-exponential kernels.

    Spectrum: nE bins log-spaced 0.2-6 MeV, weights w(E) ~ E^-q (seeded q)
    with a small seeded smooth ripple, normalised to unit sum; power-law mass
    attenuation mu = c E^-p and mu_en = c' E^-p'.
    Kernel: per zenith bin theta, (A, a, B, b) with a in [3, 6] /cm
    (primary), b in [0.3, 0.7] /cm (scatter), forward-peaked energy split,
    normalised so sum_theta (A/a + B/b) = 1.
    """
    rng = np.random.default_rng(seed)
    E = np.geomspace(0.2, 6.0, nE)
    q = rng.uniform(0.5, 1.0)
    ripple = 1.0 + 0.05 * np.sin(np.linspace(0, math.pi, nE) * rng.uniform(0.5, 1.5))
    w = E ** (-q) * ripple
    w = w / w.sum()
    mu = 0.0707 * E ** (-0.48)
    mu_en = 0.0290 * E ** (-0.08)
    tc = (np.arange(ntheta) + 0.5) * 180.0 / ntheta
    energy_frac = np.exp(-tc / 45.0) * rng.uniform(0.8, 1.2, ntheta)
    energy_frac /= energy_frac.sum()
    a = rng.uniform(3.0, 6.0, ntheta)
    b = rng.uniform(0.3, 0.7, ntheta)
    prim = rng.uniform(0.5, 0.8, ntheta)
    A = a * energy_frac * prim
    B = b * energy_frac * (1.0 - prim)
    params = np.stack([A, a, B, b], axis=1)
    radii = KERNEL_RADII_CM.copy()
    th, ph = cone_angles(ntheta, nphi)
    return Physics(energy=E, fluence=w, mu=mu, mu_en=mu_en, ntheta=ntheta, nphi=nphi,
                   radii=radii, exp_params=params, cumkern=cumulative_table(params, radii),
                   theta_deg=th, phi_deg=ph, rev_latspacing=spacing_cm,
                   rev_longspacing=spacing_cm, penumbra=penumbra_cm)


def slab_phantom(n: int = 64, voxel_cm: float = 0.25) -> Volume:
    """Water cube with a lung slab (0.25 g/cc, depth 4-6 cm) and a bone slab
    (1.85 g/cc, depth 10-11 cm); depth runs along +y, the gantry-0 beam
    direction; the isocentre is the cube centre (a voxel corner)."""
    dens = np.ones((n, n, n), dtype=np.float32)
    depth = (np.arange(n) + 0.5) * voxel_cm
    lung = (depth >= 4.0) & (depth < 6.0)
    bone = (depth >= 10.0) & (depth < 11.0)
    dens[:, lung, :] = 0.25
    dens[:, bone, :] = 1.85
    start = -0.5 * (n - 1) * voxel_cm * np.ones(3)
    return Volume(density=dens, voxel=np.full(3, voxel_cm), start=start,
                  bbox_start=np.zeros(3, np.int64), bbox_size=np.array([n, n, n], np.int64))


def _ellipsoid(shape_xyz, voxel, start, center, semi):
    nx, ny, nz = shape_xyz
    x = start[0] + np.arange(nx) * voxel[0] - center[0]
    y = start[1] + np.arange(ny) * voxel[1] - center[1]
    z = start[2] + np.arange(nz) * voxel[2] - center[2]
    return ((z[:, None, None] / semi[2]) ** 2 + (y[None, :, None] / semi[1]) ** 2
            + (x[None, None, :] / semi[0]) ** 2) <= 1.0


def head_neck_phantom(shape=(200, 200, 160), voxel_cm: float = 0.2, seed: int = 1,
                      with_oars: bool = False) -> Volume:
    """Head-and-neck-like phantom: ellipsoidal water body, 5 mm bone shell
    (1.8 g/cc), two air cavities (0.001 g/cc), PTV sphere r = 2.5 cm at the
    isocentre (origin, a voxel corner).  Optional OAR ellipsoids."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    voxel = np.full(3, voxel_cm)
    start = -0.5 * (np.array(shape) - 1) * voxel_cm
    ext = np.array(shape) * voxel_cm
    semi = np.array([0.42 * ext[0], 0.45 * ext[1], 0.46 * ext[2]])
    dens = np.zeros((nz, ny, nx), dtype=np.float32)
    body = _ellipsoid(shape, voxel, start, np.zeros(3), semi)
    dens[body] = 1.0
    outer = _ellipsoid(shape, voxel, start, np.zeros(3), semi - 0.3)
    inner = _ellipsoid(shape, voxel, start, np.zeros(3), semi - 0.8)
    dens[outer & ~inner] = 1.8
    for _ in range(2):
        c = np.array([rng.uniform(-0.35, 0.35) * semi[0], rng.uniform(-0.5, -0.25) * semi[1],
                      rng.uniform(0.1, 0.4) * semi[2]])
        s = rng.uniform(1.0, 2.0, 3)
        dens[_ellipsoid(shape, voxel, start, c, s) & inner] = 0.001
    masks = {"PTV": _ellipsoid(shape, voxel, start, np.zeros(3), np.full(3, 2.5))}
    dens[masks["PTV"]] = 1.0
    if with_oars:
        for k in range(3):
            c = rng.uniform(-1, 1, 3) * np.array([4.0, 4.0, 4.0])
            c = c + np.sign(c) * 3.0
            s = rng.uniform(1.0, 2.5, 3)
            masks[f"OAR{k}"] = _ellipsoid(shape, voxel, start, c, s) & ~masks["PTV"]
    return Volume(density=dens, voxel=voxel, start=start, bbox_start=np.zeros(3, np.int64),
                  bbox_size=np.array(shape, np.int64), masks=masks)


def single_beam(fmap=(16, 16), beamlet_cm=0.5, gantry_deg=0.0, couch_deg=0.0, coll_deg=0.0,
                sad_cm=100.0, iso=ISO_OFFSET_CM, value=1.0) -> Beam:
    return Beam(azimuth=math.radians(gantry_deg), zenith=math.radians(couch_deg),
                coll=math.radians(coll_deg), isocenter=np.asarray(iso, dtype=np.float64),
                sad=sad_cm, fmap_size=tuple(fmap), beamlet_size=(beamlet_cm, beamlet_cm),
                fluence=np.full((fmap[1], fmap[0]), value, dtype=np.float32))


def four_pi_angles(n_beams: int, step_deg: float = 6.0, seed: int = 2):
    """(gantry, couch) pairs in degrees on a ~step_deg 4-pi grid with a
    seeded collision-zone exclusion (gantry in a band around 180 deg is
    excluded for large couch kicks, with a seeded band half-width)."""
    rng = np.random.default_rng(seed)
    gs = np.arange(0.0, 360.0, step_deg)
    cs = np.arange(-90.0, 90.0 + 1e-9, step_deg)
    half = rng.uniform(40.0, 60.0)
    cands = []
    for c in cs:
        for g in gs:
            if abs(c) > 30.0 and abs(g - 180.0) < half:
                continue
            if abs(c) > 1e-9 and (abs(g) < 1e-9 or abs(g - 180.0) < 1e-9):
                continue  # couch kick is ignored at gantry 0/180 (beam.cpp:308-312)
            cands.append((g, c))
    cands = np.array(cands)
    idx = rng.choice(len(cands), size=min(n_beams, len(cands)), replace=False)
    idx.sort()
    return cands[idx]


def candidate_beams(n_beams: int = 1024, seed: int = 3, sad_cm: float = 100.0,
                    beamlet_cm: float = 0.25, nmin: int = 8, nmax: int = 40) -> List[Beam]:
    """Batched-candidate workload: non-coplanar beams, each with a fluence
    map cropped to a target projection of seeded size (n x n beamlets,
    nmin <= n <= nmax), U(0,1) inside the projected disc, 0 outside."""
    rng = np.random.default_rng(seed)
    angs = four_pi_angles(n_beams, seed=seed + 1)
    beams = []
    for g, c in angs:
        n = int(rng.integers(nmin, nmax + 1))
        yy, xx = np.mgrid[0:n, 0:n]
        rr = np.hypot(xx + 0.5 - n / 2, yy + 0.5 - n / 2)
        fl = rng.uniform(0.0, 1.0, (n, n)).astype(np.float32)
        fl[rr > n / 2] = 0.0
        fl[n // 2, n // 2] = max(fl[n // 2, n // 2], 0.5)
        b = single_beam(fmap=(n, n), beamlet_cm=beamlet_cm, gantry_deg=float(g), couch_deg=float(c),
                        sad_cm=sad_cm)
        b.fluence = fl
        beams.append(b)
    return beams


def config0():
    """64^3 slab phantom at 2.5 mm, 8x6 cones, 16x16 beamlets of 5 mm, SAD 100 cm."""
    return slab_phantom(64, 0.25), make_physics(seed=0, spacing_cm=0.25), [single_beam()]


def config1(n_beams: int = 1024, shape=(200, 200, 160)):
    """200x200x160 head-and-neck-like phantom at 2 mm with n_beams candidates."""
    vol = head_neck_phantom(shape=shape, voxel_cm=0.2)
    return vol, make_physics(seed=0, spacing_cm=0.2), candidate_beams(n_beams)


SERVING_SHAPES = [(96, 96, 96), (128, 128, 128), (160, 160, 160), (256, 256, 192)]


def serving_workload(n_requests: int = 100, rate_hz: float = 50.0, seed: int = 9, beamlet_cm: float = 0.25):
    """Serving-loop workload: head-and-neck-like phantoms at 2 mm of the four
    SERVING_SHAPES, and n_requests requests with Poisson arrival times
    (rate_hz), each on a phantom drawn uniformly, with 1-40 beams of fluence
    grids n x n, 16 <= n <= 64 (U(0,1) in the projected disc), half of them
    dose-only and half dose + fluence gradient (kind drawn per request).
    Returns (volumes, requests) with requests as dicts
    {t: arrival s, volume: index, beams: [Beam], grad: bool}."""
    rng = np.random.default_rng(seed)
    vols = [head_neck_phantom(shape=s, voxel_cm=0.2, seed=seed + k) for k, s in enumerate(SERVING_SHAPES)]
    t = np.cumsum(rng.exponential(1.0 / rate_hz, n_requests))
    reqs = []
    for k in range(n_requests):
        nb = int(rng.integers(1, 41))
        angs = four_pi_angles(nb, seed=int(rng.integers(1 << 30)))
        beams = []
        for g, c in angs:
            n = int(rng.integers(16, 65))
            yy, xx = np.mgrid[0:n, 0:n]
            rr = np.hypot(xx + 0.5 - n / 2, yy + 0.5 - n / 2)
            fl = rng.uniform(0.0, 1.0, (n, n)).astype(np.float32)
            fl[rr > n / 2] = 0.0
            fl[n // 2, n // 2] = max(fl[n // 2, n // 2], 0.5)
            b = single_beam(fmap=(n, n), beamlet_cm=beamlet_cm, gantry_deg=float(g), couch_deg=float(c))
            b.fluence = fl
            beams.append(b)
        reqs.append({"t": float(t[k]), "volume": int(rng.integers(0, len(vols))), "beams": beams,
                     "grad": bool(rng.integers(0, 2))})
    return vols, reqs
