"""Python host binding of the CCCS engine's C ABI (include/ee_cccs.h).

This is a thin ctypes layer: every computation runs in
``endtoend_gb300/_lib/libee_cccs.so`` (hand-written sm_103a kernels).  There
is no CPU fallback; constructing an :class:`Engine` without the built
library raises.

Exceptions mirror the reference's error behaviour
(CCCS/dosecalc-beam/nvbbRayConvolve_host.cu): :class:`ArraySizeError` for REV
arrays over their limit (``ArraySizeError``, host.cu:71-74,148-154 and the
rev.x > 1024 runtime_error, host.cu:567) and :class:`CropBoxError` for an
empty or oversized crop box (runtime_error, host.cu:494-498).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Sequence

import numpy as np

from . import _build

EE_OK = 0
EE_ERR_INVALID_ARG = 1
EE_ERR_CUDA = 2
EE_ERR_CROPBOX = 3
EE_ERR_REV_SIZE = 4
EE_ERR_NOMEM = 5
EE_ERR_NOT_READY = 6
EE_ERR_SIDDON_ITER = 7
EE_ERR_CAPACITY = 8
EE_ERR_IO = 9

KERNEL_TABLE = 0
KERNEL_EXP = 1
KERNEL_TABLE_WALK = 2

DOSE_SUM = 0
DOSE_ACCUMULATE = 1
DOSE_PER_BEAM = 2

REQ_DOSE = 0
REQ_DOSE_AND_GRAD = 1


class EEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[ee status {code}] {msg}")
        self.code = code


class ArraySizeError(EEError):
    pass


class CropBoxError(EEError):
    pass


class NotReadyError(EEError):
    pass


class Frame(C.Structure):
    _fields_ = [("size", C.c_int * 3), ("voxel", C.c_float * 3), ("start", C.c_float * 3),
                ("bbox_start", C.c_int * 3), ("bbox_size", C.c_int * 3)]


class ConvParams(C.Structure):
    _fields_ = [("ntheta", C.c_int), ("nphi", C.c_int), ("nradii", C.c_int),
                ("rev_latspacing", C.c_float), ("rev_longspacing", C.c_float), ("penumbra", C.c_float),
                ("max_rev_size", C.c_int * 3)]


class EEBeam(C.Structure):
    _fields_ = [("azimuth", C.c_float), ("zenith", C.c_float), ("coll", C.c_float),
                ("isocenter", C.c_float * 3), ("sad", C.c_float),
                ("fmap_size", C.c_int * 2), ("beamlet_size", C.c_float * 2)]


class Loss(C.Structure):
    _fields_ = [("ptv_weight", C.c_void_p), ("ptv_target", C.c_void_p), ("oar_weight", C.c_void_p),
                ("oar_target", C.c_void_p), ("eta", C.c_float), ("spread_sigma", C.c_float)]


class BeamInfo(C.Structure):
    _fields_ = [("source", C.c_float * 3), ("direction", C.c_float * 3), ("b_min", C.c_float * 3),
                ("bev_size", C.c_int * 3), ("lim_min", C.c_float * 3), ("v_beam", C.c_longlong),
                ("rev_samples", C.c_longlong), ("terma_nonzero", C.c_longlong), ("max_line", C.c_int),
                ("status", C.c_int)]


class AnnealParams(C.Structure):
    _fields_ = [("iterations", C.c_int), ("step_size", C.c_float), ("sigma_deg", C.c_float),
                ("temperature", C.c_float), ("cooling", C.c_float), ("fluence_steps", C.c_int),
                ("seed", C.c_ulonglong)]


class AnnealRecord(C.Structure):
    _fields_ = [("zenith", C.c_void_p), ("azimuth", C.c_void_p), ("perturbation_loss", C.c_void_p),
                ("possibility", C.c_void_p), ("taken", C.c_void_p), ("dose_loss", C.c_void_p),
                ("smoothness_loss", C.c_void_p)]


class Csr(C.Structure):
    _fields_ = [("nbeamlets", C.c_int), ("nnz", C.c_longlong), ("beamlet_index", C.c_void_p), ("col_ptr", C.c_void_p),
                ("row_index", C.c_void_p), ("value", C.c_void_p)]


class Request(C.Structure):
    _fields_ = [("volume_id", C.c_int), ("kind", C.c_int), ("beams", C.POINTER(EEBeam)), ("nbeams", C.c_int),
                ("fluence", C.c_void_p), ("dose_grad", C.c_void_p), ("dose_out", C.c_void_p),
                ("fluence_grad_out", C.c_void_p)]


# every symbol include/ee_cccs.h declares, with its ctypes signature
_SIGS = {
    "ee_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "ee_destroy": (C.c_int, [C.c_void_p]),
    "ee_last_error": (C.c_char_p, []),
    "ee_abi_version": (C.c_int, []),
    "ee_set_volume": (C.c_int, [C.c_void_p, C.POINTER(Frame), C.c_void_p]),
    "ee_set_spectrum": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ee_set_kernel_table": (C.c_int, [C.c_void_p, C.POINTER(ConvParams), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ee_set_kernel_exp": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ee_set_kernel_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "ee_set_terma_supersampling": (C.c_int, [C.c_void_p, C.c_int]),
    "ee_beam_dose": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "ee_beam_dose_device": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "ee_beam_dose_adjoint": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ee_beam_dose_adjoint_device": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ee_get_beam_info": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(BeamInfo)]),
    "ee_synchronize": (C.c_int, [C.c_void_p]),
    "ee_get_stream": (C.c_void_p, [C.c_void_p]),
    "ee_beam_source": (C.c_int, [C.POINTER(EEBeam), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "ee_loss_and_grad": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.POINTER(Loss), C.c_void_p,
                                   C.c_void_p, C.POINTER(C.c_double)]),
    "ee_dose_and_adjoint_device": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                             C.c_void_p, C.c_void_p]),
    "ee_dose_and_adjoint": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_void_p]),
    "ee_beam_dose_noalloc": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_void_p, C.c_void_p, C.c_void_p]),
    "ee_plan_create": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.POINTER(C.c_void_p)]),
    "ee_plan_launch": (C.c_int, [C.c_void_p]),
    "ee_plan_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "ee_plan_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_int)]),
    "ee_plan_destroy": (C.c_int, [C.c_void_p]),
    "ee_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "ee_set_scratch_limit": (C.c_int, [C.c_void_p, C.c_longlong]),
    "ee_read_profile": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.c_int]),
    "ee_set_beamlet_options": (C.c_int, [C.c_void_p, C.c_float, C.POINTER(C.c_int)]),
    "ee_beamlet_columns_device": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_void_p, C.c_float, C.POINTER(Csr)]),
    "ee_roi_list_create": (C.c_int, [C.POINTER(C.c_int), C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "ee_roi_list_capacities": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ee_roi_reduce": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p,
                                C.c_longlong, C.POINTER(C.c_longlong), C.c_void_p]),
    "ee_roi_list_destroy": (C.c_int, [C.c_void_p]),
    "ee_beamlet_columns": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_void_p, C.c_float, C.c_longlong, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_int)]),
    "ee_copy_to_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong]),
    "ee_optimize_fluence": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.POINTER(Loss), C.c_int,
                                      C.c_float, C.c_void_p, C.c_void_p]),
    "ee_optimize_annealing": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_void_p, C.POINTER(Loss),
                                        C.POINTER(AnnealParams), C.POINTER(AnnealRecord)]),
    "ee_evaluate_proposals": (C.c_int, [C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_int, C.c_void_p, C.POINTER(Loss),
                                        C.POINTER(C.c_double)]),
    "ee_ct_to_density": (C.c_int, [C.c_int, C.POINTER(Frame), C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_int,
                                   C.c_void_p, C.POINTER(C.c_int)]),
    "ee_fluence_projection": (C.c_int, [C.c_int, C.POINTER(Frame), C.c_void_p, C.POINTER(EEBeam), C.c_int, C.c_int,
                                        C.c_int, C.c_void_p]),
    "ee_read_spectrum_file": (C.c_int, [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_char_p, C.c_int, C.POINTER(C.c_int)]),
    "ee_read_mono_kernel": (C.c_int, [C.c_char_p, C.c_void_p]),
    "ee_read_kernel_radii": (C.c_int, [C.c_char_p, C.c_void_p]),
    "ee_cumulative_kernel": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "ee_fit_exp_kernel": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ee_server_create": (C.c_int, [C.c_int, C.c_int, C.c_longlong, C.c_int, C.POINTER(C.c_void_p)]),
    "ee_server_set_physics": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.POINTER(ConvParams), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    "ee_server_add_volume": (C.c_int, [C.c_void_p, C.POINTER(Frame), C.c_void_p, C.POINTER(C.c_int)]),
    "ee_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_longlong)]),
    "ee_server_wait": (C.c_int, [C.c_void_p, C.c_longlong, C.c_double, C.POINTER(C.c_int)]),
    "ee_server_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_double)]),
    "ee_server_reset_stats": (C.c_int, [C.c_void_p]),
    "ee_server_destroy": (C.c_int, [C.c_void_p]),
}

STAGES = ["terma", "geometry", "cone", "gather", "gather_T", "cone_T", "terma_T"]

_LIB = None


def library_path() -> str:
    return _build.LIB


def load_library(build_if_missing: bool = False):
    """Load libee_cccs.so (raises if it is not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"CCCS engine library not built ({path}); run endtoend_gb300._build.build()")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def to_ee_beams(beams) -> "C.Array":
    arr = (EEBeam * len(beams))()
    for i, b in enumerate(beams):
        e = arr[i]
        e.azimuth, e.zenith, e.coll = float(b.azimuth), float(b.zenith), float(b.coll)
        e.isocenter[:] = [float(v) for v in b.isocenter]
        e.sad = float(b.sad)
        e.fmap_size[:] = [int(v) for v in b.fmap_size]
        e.beamlet_size[:] = [float(v) for v in b.beamlet_size]
    return arr


def _frame_of(vol) -> Frame:
    f = Frame()
    f.size[:] = [int(v) for v in vol.size]
    f.voxel[:] = [float(v) for v in vol.voxel]
    f.start[:] = [float(v) for v in vol.start]
    f.bbox_start[:] = [int(v) for v in vol.bbox_start]
    f.bbox_size[:] = [int(v) for v in vol.bbox_size]
    return f


def _raise_status(lib, st):
    if st == EE_OK:
        return
    msg = lib.ee_last_error().decode(errors="replace")
    cls = {EE_ERR_REV_SIZE: ArraySizeError, EE_ERR_CROPBOX: CropBoxError,
           EE_ERR_NOT_READY: NotReadyError}.get(st, EEError)
    raise cls(st, msg)


def concat_fluence(beams) -> np.ndarray:
    return np.ascontiguousarray(np.concatenate([np.asarray(b.fluence, np.float32).ravel() for b in beams]))


class Engine:
    """One engine context on one GPU (device-resident density, spectrum and
    kernel; reusable scratch).  Mirrors the reference call sequence
    initCudaConstandTex -> radconvolveTexture -> cuda_sum_device_float_dose
    -> freeCudaTexture as set_* -> beam_dose -> close."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        self._check(self.lib.ee_create(int(device), C.byref(h)))
        self.h = h
        self.vol = None
        self.phys = None

    # -- errors
    def _check(self, st):
        _raise_status(self.lib, st)

    # -- set-up
    def set_volume(self, vol):
        d = np.ascontiguousarray(vol.density, dtype=np.float32)
        self._check(self.lib.ee_set_volume(self.h, C.byref(_frame_of(vol)), _ptr(d)))
        self.vol = vol

    def set_physics(self, phys, mode: str = "exp", max_rev_size=(0, 0, 0)):
        f32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32))
        E, fl, mu, muen = f32(phys.energy), f32(phys.fluence), f32(phys.mu), f32(phys.mu_en)
        self._check(self.lib.ee_set_spectrum(self.h, len(E), _ptr(E), _ptr(fl), _ptr(mu), _ptr(muen)))
        cp = ConvParams()
        cp.ntheta, cp.nphi, cp.nradii = phys.ntheta, phys.nphi, phys.nradii
        cp.rev_latspacing, cp.rev_longspacing, cp.penumbra = phys.rev_latspacing, phys.rev_longspacing, phys.penumbra
        cp.max_rev_size[:] = list(max_rev_size)
        radii, ck, th, ph = f32(phys.radii), f32(phys.cumkern), f32(phys.theta_deg), f32(phys.phi_deg)
        self._check(self.lib.ee_set_kernel_table(self.h, C.byref(cp), _ptr(radii), _ptr(ck), _ptr(th), _ptr(ph)))
        ep = f32(phys.exp_params)
        self._check(self.lib.ee_set_kernel_exp(self.h, _ptr(ep)))
        self.set_mode(mode)
        self.phys = phys

    def set_mode(self, mode: str):
        modes = {"exp": KERNEL_EXP, "table": KERNEL_TABLE, "walk": KERNEL_TABLE_WALK}
        if mode not in modes:
            raise ValueError(f"kernel mode {mode!r}: one of {sorted(modes)}")
        self._check(self.lib.ee_set_kernel_mode(self.h, modes[mode]))

    def set_terma_supersampling(self, ss_factor: int):
        """TERMA supersampling (omni-header ss_factor); the adjoint recomputes the sub-voxel beamlets."""
        self._check(self.lib.ee_set_terma_supersampling(self.h, int(ss_factor)))

    # -- forward dose
    def beam_dose(self, beams: Sequence, per_beam: bool = False, accumulate_into: np.ndarray = None) -> np.ndarray:
        """Host buffers in and out (the end-to-end path)."""
        nz, ny, nx = self.vol.density.shape
        eb = to_ee_beams(beams)
        fl = concat_fluence(beams)
        if per_beam:
            out = np.zeros((len(beams), nz, ny, nx), np.float32)
            mode = DOSE_PER_BEAM
        elif accumulate_into is not None:
            out = accumulate_into
            assert out.dtype == np.float32 and out.flags.c_contiguous and out.shape == (nz, ny, nx)
            mode = DOSE_ACCUMULATE
        else:
            out = np.zeros((nz, ny, nx), np.float32)
            mode = DOSE_SUM
        self._check(self.lib.ee_beam_dose(self.h, eb, len(beams), _ptr(fl), _ptr(out), mode))
        return out

    def beam_dose_device(self, beams: Sequence, d_fluence: int, d_dose: int, mode: int = DOSE_SUM):
        """Device pointers (e.g. torch tensor .data_ptr()); enqueued on the
        engine stream (the call returns after the per-batch geometry read-back)."""
        eb = to_ee_beams(beams)
        self._check(self.lib.ee_beam_dose_device(self.h, eb, len(beams), C.c_void_p(d_fluence), C.c_void_p(d_dose), mode))

    # -- adjoint
    def beam_dose_adjoint(self, beams: Sequence, dose_grad: np.ndarray) -> List[np.ndarray]:
        eb = to_ee_beams(beams)
        fl = concat_fluence(beams)
        g = np.ascontiguousarray(dose_grad, dtype=np.float32)
        assert g.shape == self.vol.density.shape
        out = np.zeros(fl.size, np.float32)
        self._check(self.lib.ee_beam_dose_adjoint(self.h, eb, len(beams), _ptr(fl), _ptr(g), _ptr(out)))
        res, o = [], 0
        for b in beams:
            n = int(b.fmap_size[0] * b.fmap_size[1])
            res.append(out[o:o + n].reshape(b.fmap_size[1], b.fmap_size[0]))
            o += n
        return res

    def beam_dose_adjoint_device(self, beams: Sequence, d_fluence: int, d_dose_grad: int, d_fluence_grad: int):
        eb = to_ee_beams(beams)
        self._check(self.lib.ee_beam_dose_adjoint_device(self.h, eb, len(beams), C.c_void_p(d_fluence),
                                                         C.c_void_p(d_dose_grad), C.c_void_p(d_fluence_grad)))

    def dose_and_adjoint_device(self, beams, d_fluence: int, d_dose: int, d_dose_grad: int, d_fluence_grad: int,
                                mode: int = DOSE_SUM):
        """Forward dose and adjoint in one call (shared TERMA / geometry)."""
        eb = to_ee_beams(beams)
        self._check(self.lib.ee_dose_and_adjoint_device(self.h, eb, len(beams), C.c_void_p(d_fluence),
                                                        C.c_void_p(d_dose or 0), mode, C.c_void_p(d_dose_grad or 0),
                                                        C.c_void_p(d_fluence_grad or 0)))

    @staticmethod
    def make_loss(ptv=(0, 0), oar=(0, 0), eta: float = 0.0, spread_sigma: float = 0.0) -> Loss:
        L = Loss()
        L.ptv_weight, L.ptv_target = ptv
        L.oar_weight, L.oar_target = oar
        L.eta, L.spread_sigma = float(eta), float(spread_sigma)
        return L

    def optimize_fluence(self, beams, d_x: int, loss: Loss, iterations: int, step_size: float):
        """Projected gradient descent of the fluence (EndtoEnd
        optimize_stationary_smoothness).  Returns (dose_loss[it],
        smoothness_loss[it, nbeams])."""
        eb = to_ee_beams(beams)
        dl = np.zeros(iterations, np.float32)
        sl = np.zeros((iterations, len(beams)), np.float32)
        self._check(self.lib.ee_optimize_fluence(self.h, eb, len(beams), C.c_void_p(d_x), C.byref(loss), int(iterations),
                                                 float(step_size), _ptr(dl), _ptr(sl)))
        return dl, sl

    def optimize_annealing(self, beams, d_x: int, loss: Loss, iterations: int, step_size: float = 0.0,
                           sigma_deg: float = 5.0, temperature: float = 0.0, cooling: float = 1.0,
                           fluence_steps: int = 1, seed: int = 0):
        """Simulated annealing of the angles + fluence gradient descent
        (EndtoEnd optimize_annealing_constrain).  Returns (final
        (azimuth, zenith) per beam, record dict of the README's arrays)."""
        n = len(beams)
        eb = to_ee_beams(beams)
        p = AnnealParams()
        p.iterations, p.step_size, p.sigma_deg = int(iterations), float(step_size), float(sigma_deg)
        p.temperature, p.cooling, p.fluence_steps, p.seed = float(temperature), float(cooling), int(fluence_steps), int(seed)
        rec = {"zenith": np.zeros((iterations, n, 2), np.float32), "azimuth": np.zeros((iterations, n, 2), np.float32),
               "perturbation_loss": np.zeros((iterations, n, 2), np.float32),
               "possibility": np.zeros((iterations, n), np.float32), "taken": np.zeros((iterations, n), np.uint8),
               "dose_loss": np.zeros(iterations, np.float32), "smoothness_loss": np.zeros((iterations, n), np.float32)}
        r = AnnealRecord()
        for k, v in rec.items():
            setattr(r, k, v.ctypes.data)
        self._check(self.lib.ee_optimize_annealing(self.h, eb, n, C.c_void_p(d_x), C.byref(loss), C.byref(p),
                                                   C.byref(r)))
        return [(eb[b].azimuth, eb[b].zenith) for b in range(n)], rec

    def evaluate_proposals(self, proposals, d_x: int, loss: Loss) -> np.ndarray:
        """Dose terms of the loss for each proposal (a list of beam lists of
        equal fluence-map sizes, all sharing the fluence d_x)."""
        nprop, n = len(proposals), len(proposals[0])
        eb = to_ee_beams([b for prop in proposals for b in prop])
        out = (C.c_double * nprop)()
        self._check(self.lib.ee_evaluate_proposals(self.h, eb, nprop, n, C.c_void_p(d_x), C.byref(loss), out))
        return np.array(list(out))

    def loss_and_grad_device(self, beams, d_x: int, d_dose: int, d_xgrad: int, ptv=(0, 0), oar=(0, 0),
                             eta: float = 0.0, spread_sigma: float = 0.0):
        """EndtoEnd loss (README.md:20) and its gradient w.r.t. the fluence maps.
        ptv/oar: (weight_ptr, target_ptr) device pointers or (0, 0)."""
        eb = to_ee_beams(beams)
        L = Loss()
        L.ptv_weight, L.ptv_target = ptv
        L.oar_weight, L.oar_target = oar
        L.eta, L.spread_sigma = float(eta), float(spread_sigma)
        out = (C.c_double * 3)()
        self._check(self.lib.ee_loss_and_grad(self.h, eb, len(beams), C.c_void_p(d_x), C.byref(L), C.c_void_p(d_dose),
                                              C.c_void_p(d_xgrad), out))
        return list(out)

    def beam_dose_noalloc(self, beam, d_fluence: int, d_dose: int, stream: int = 0):
        """One beam's dose without any device allocation (static 64 MiB
        scratch); for callers that cannot allocate per call."""
        eb = to_ee_beams([beam])
        self._check(self.lib.ee_beam_dose_noalloc(self.h, eb, C.c_void_p(d_fluence), C.c_void_p(d_dose),
                                                  C.c_void_p(stream or None)))

    def plan(self, beams, d_fluence: int, d_dose: int, d_dose_grad: int = 0, d_fluence_grad: int = 0) -> "Plan":
        """Capture a batch into a replayable CUDA graph (see ee_plan_create)."""
        return Plan(self, beams, d_fluence, d_dose, d_dose_grad, d_fluence_grad)

    # -- diagnostics
    def beam_info(self, i: int) -> dict:
        bi = BeamInfo()
        self._check(self.lib.ee_get_beam_info(self.h, int(i), C.byref(bi)))
        return {"source": list(bi.source), "direction": list(bi.direction), "b_min": list(bi.b_min),
                "bev_size": list(bi.bev_size), "lim_min": list(bi.lim_min), "v_beam": bi.v_beam,
                "rev_samples": bi.rev_samples, "terma_nonzero": bi.terma_nonzero, "max_line": bi.max_line,
                "status": bi.status}

    # -- beamlet dose columns (dosecalc-beamlet)
    def set_beamlet_options(self, kernel_extent_cm: float = 2.0, max_rev_size=None):
        mr = None
        if max_rev_size is not None:
            mr = (C.c_int * 3)(*[int(v) for v in max_rev_size])
        self._check(self.lib.ee_set_beamlet_options(self.h, float(kernel_extent_cm), mr))

    def beamlet_columns_device(self, beam, thresh: float = 1e-4) -> Csr:
        """Device CSR of one beam's beamlet columns (pointers owned by the
        context until its next beamlet call)."""
        eb = to_ee_beams([beam])
        fl = np.ascontiguousarray(beam.fluence, np.float32).ravel()
        out = Csr()
        self._check(self.lib.ee_beamlet_columns_device(self.h, eb, _ptr(fl), float(thresh), C.byref(out)))
        return out

    def beamlet_columns(self, beam, thresh: float = 1e-4):
        """(beamlet_index, col_ptr, row_index, value) numpy arrays of one
        beam's sparse beamlet dose columns (dosecalc-beamlet semantics)."""
        d = self.beamlet_columns_device(beam, thresh)
        n, nnz = d.nbeamlets, d.nnz
        bidx = np.zeros(n, np.int32)
        cp = np.zeros(n + 1, np.int64)
        rows = np.zeros(nnz, np.int32)
        vals = np.zeros(nnz, np.float32)
        for arr, src in ((bidx, d.beamlet_index), (cp, d.col_ptr), (rows, d.row_index), (vals, d.value)):
            if arr.nbytes:
                self._check(self.lib.ee_copy_to_host(self.h, _ptr(arr), C.c_void_p(src), arr.nbytes))
        return bidx, cp, rows, vals

    def set_scratch_limit(self, nbytes: int):
        self._check(self.lib.ee_set_scratch_limit(self.h, int(nbytes)))

    def set_profiling(self, on: bool = True):
        self._check(self.lib.ee_set_profiling(self.h, 1 if on else 0))

    def read_profile(self) -> dict:
        """{stage: (ms, launches)} accumulated since the last read."""
        n = len(STAGES)
        ms = (C.c_double * n)()
        nl = (C.c_longlong * n)()
        self._check(self.lib.ee_read_profile(self.h, ms, nl, n))
        return {s: (ms[i], nl[i]) for i, s in enumerate(STAGES)}

    def synchronize(self):
        self._check(self.lib.ee_synchronize(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.ee_get_stream(self.h) or 0)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ee_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Plan:
    """A batch of beams captured into a CUDA graph (ee_plan_*)."""

    def __init__(self, eng: Engine, beams, d_fluence, d_dose, d_dose_grad=0, d_fluence_grad=0):
        self.eng = eng
        self._eb = to_ee_beams(beams)
        h = C.c_void_p()
        eng._check(eng.lib.ee_plan_create(eng.h, self._eb, len(beams), C.c_void_p(d_fluence), C.c_void_p(d_dose),
                                          C.c_void_p(d_dose_grad or None), C.c_void_p(d_fluence_grad or None),
                                          C.byref(h)))
        self.h = h

    def launch(self):
        self.eng._check(self.eng.lib.ee_plan_launch(self.h))

    def status(self):
        n = C.c_int()
        self.eng._check(self.eng.lib.ee_plan_status(self.h, C.byref(n)))
        return n.value

    def info(self):
        lb, by, nc = C.c_int(), C.c_longlong(), C.c_int()
        self.eng._check(self.eng.lib.ee_plan_info(self.h, C.byref(lb), C.byref(by), C.byref(nc)))
        return {"lane_block": lb.value, "device_bytes": by.value, "chunks": nc.value}

    def close(self):
        if getattr(self, "h", None):
            self.eng.lib.ee_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request server on one GPU (ee_server_*).

    ``submit`` copies a request's inputs and returns a ticket at once;
    ``wait`` returns its summed dose (and, for gradient requests, the
    per-beam fluence gradients)."""

    def __init__(self, device: int = 0, slots: int = 2, hbm_budget: int = 0, max_batch_beams: int = 256):
        self.lib = load_library()
        h = C.c_void_p()
        _raise_status(self.lib, self.lib.ee_server_create(int(device), int(slots), int(hbm_budget),
                                                          int(max_batch_beams), C.byref(h)))
        self.h = h
        self.volumes = []
        self._pending = {}

    def set_physics(self, phys, mode: str = "exp"):
        f32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32))
        E, fl, mu, muen = f32(phys.energy), f32(phys.fluence), f32(phys.mu), f32(phys.mu_en)
        cp = ConvParams()
        cp.ntheta, cp.nphi, cp.nradii = phys.ntheta, phys.nphi, phys.nradii
        cp.rev_latspacing, cp.rev_longspacing, cp.penumbra = phys.rev_latspacing, phys.rev_longspacing, phys.penumbra
        cp.max_rev_size[:] = [0, 0, 0]
        radii, ck, th, ph = f32(phys.radii), f32(phys.cumkern), f32(phys.theta_deg), f32(phys.phi_deg)
        ep = f32(phys.exp_params) if mode == "exp" else None
        _raise_status(self.lib, self.lib.ee_server_set_physics(
            self.h, len(E), _ptr(E), _ptr(fl), _ptr(mu), _ptr(muen), C.byref(cp), _ptr(radii), _ptr(ck), _ptr(th),
            _ptr(ph), _ptr(ep) if ep is not None else None))

    def add_volume(self, vol) -> int:
        d = np.ascontiguousarray(vol.density, dtype=np.float32)
        vid = C.c_int()
        _raise_status(self.lib, self.lib.ee_server_add_volume(self.h, C.byref(_frame_of(vol)), _ptr(d),
                                                              C.byref(vid)))
        self.volumes.append(vol)
        return vid.value

    def submit(self, volume_id: int, beams: Sequence, dose_grad: np.ndarray = None) -> int:
        if not 0 <= int(volume_id) < len(self.volumes):
            raise EEError(EE_ERR_INVALID_ARG, f"unknown volume id {volume_id}")
        vol = self.volumes[volume_id]
        eb = to_ee_beams(beams)
        fl = concat_fluence(beams)
        dose = np.zeros(vol.density.shape, np.float32)
        q = Request()
        q.volume_id, q.nbeams, q.beams = int(volume_id), len(beams), eb
        q.fluence, q.dose_out = fl.ctypes.data, dose.ctypes.data
        fg = g = None
        if dose_grad is not None:
            g = np.ascontiguousarray(dose_grad, dtype=np.float32)
            assert g.shape == vol.density.shape
            fg = np.zeros_like(fl)
            q.kind, q.dose_grad, q.fluence_grad_out = REQ_DOSE_AND_GRAD, g.ctypes.data, fg.ctypes.data
        else:
            q.kind = REQ_DOSE
        t = C.c_longlong()
        _raise_status(self.lib, self.lib.ee_server_submit(self.h, C.byref(q), C.byref(t)))
        self._pending[t.value] = (beams, dose, fg)
        return t.value

    def wait(self, ticket: int, timeout: float = None):
        """(dose, fluence_grads or None); None while still pending after `timeout` s."""
        st = C.c_int()
        r = self.lib.ee_server_wait(self.h, C.c_longlong(ticket), -1.0 if timeout is None else float(timeout),
                                    C.byref(st))
        if r == EE_OK and st.value < 0:
            return None
        beams, dose, fg = self._pending.pop(ticket)
        _raise_status(self.lib, r)
        if fg is None:
            return dose, None
        out, o = [], 0
        for b in beams:
            n = int(b.fmap_size[0]) * int(b.fmap_size[1])
            out.append(fg[o:o + n].reshape(int(b.fmap_size[1]), int(b.fmap_size[0])))
            o += n
        return dose, out

    def stats(self) -> dict:
        p50, p99, bps = C.c_double(), C.c_double(), C.c_double()
        n = C.c_longlong()
        _raise_status(self.lib, self.lib.ee_server_stats(self.h, C.byref(p50), C.byref(p99), C.byref(n),
                                                         C.byref(bps)))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "completed": n.value, "beams_per_s": bps.value}

    def reset_stats(self):
        _raise_status(self.lib, self.lib.ee_server_reset_stats(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.ee_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---- preprocessing (dosecalc-preprocess) ----
SIEMENS_LUT = (  # HU -> g/cc, the reference's default table (dosecalc-preprocess/main.cu:187-200)
    [-969.8, -712.9, -536.5, -95.6, -45.6, -5.6, -1.9, 25.7, 65.6, 207.5, 220.7, 429.9, 775.3, 1173.7],
    [0.0, 0.290, 0.450, 0.943, 0.985, 1.000, 1.016, 1.052, 1.089, 1.145, 1.159, 1.335, 1.560, 1.823])


class RoiMask(C.Structure):
    _fields_ = [("crop_start", C.c_int * 3), ("crop_size", C.c_int * 3), ("mask", C.c_void_p)]


class RoiList:
    """ROI row blocks for sparse beamlet columns (ee_roi_*; the reference's
    _reduce_by_roi, CCCS/DoseCalcIO/sparse_io.cpp:62-158).  rois: list of
    (crop_start xyz, mask [nz][ny][nx] bool array of the crop box)."""

    def __init__(self, size_xyz, rois):
        self.lib = load_library()
        self._masks = [np.ascontiguousarray(m, np.uint8) for _, m in rois]
        arr = (RoiMask * max(1, len(rois)))()
        for k, ((c0, _), m) in enumerate(zip(rois, self._masks)):
            arr[k].crop_start[:] = [int(v) for v in c0]
            arr[k].crop_size[:] = [m.shape[2], m.shape[1], m.shape[0]]
            arr[k].mask = m.ctypes.data
        h = C.c_void_p()
        size = (C.c_int * 3)(*[int(v) for v in size_xyz])
        _raise_status(self.lib, self.lib.ee_roi_list_create(size, arr, len(rois), C.byref(h)))
        self.h = h
        self.nrois = len(rois)

    def capacities(self) -> np.ndarray:
        out = np.zeros(max(1, self.nrois), np.int64)
        _raise_status(self.lib, self.lib.ee_roi_list_capacities(self.h, out.ctypes.data))
        return out[:self.nrois]

    def reduce(self, row_index, values):
        """(keys uint64, values float32, row_block_sizes int64) of one column."""
        ri = np.ascontiguousarray(row_index, np.int32)
        va = np.ascontiguousarray(values, np.float32)
        cap = len(ri) * max(1, self.nrois)
        keys = np.zeros(max(1, cap), np.uint64)
        vals = np.zeros(max(1, cap), np.float32)
        blocks = np.zeros(max(1, self.nrois), np.int64)
        n = C.c_longlong()
        _raise_status(self.lib, self.lib.ee_roi_reduce(self.h, ri.ctypes.data, va.ctypes.data, len(ri), keys.ctypes.data,
                                                       vals.ctypes.data, cap, C.byref(n), blocks.ctypes.data))
        return keys[:n.value], vals[:n.value], blocks[:self.nrois]

    def close(self):
        if getattr(self, "h", None):
            self.lib.ee_roi_list_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ct_to_density(hu: np.ndarray, voxel_cm, iso_voxel_cm: float, lut=SIEMENS_LUT, start_cm=(0.0, 0.0, 0.0),
                  device: int = 0):
    """Isotropic density volume [nz, ny, nx] from a CT in HU (ee_ct_to_density);
    lut=None selects the linear HU rule."""
    lib = load_library()
    h = np.ascontiguousarray(hu, np.float32)
    f = Frame()
    f.size[:] = [h.shape[2], h.shape[1], h.shape[0]]
    f.voxel[:] = [float(v) for v in voxel_cm]
    f.start[:] = [float(v) for v in start_cm]
    f.bbox_size[:] = list(f.size)
    if lut is not None:
        lh, ld = np.ascontiguousarray(lut[0], np.float32), np.ascontiguousarray(lut[1], np.float32)
        n = len(lh)
    else:
        lh = ld = np.zeros(1, np.float32)
        n = 0
    os_ = (C.c_int * 3)()
    _raise_status(lib, lib.ee_ct_to_density(int(device), C.byref(f), None, float(iso_voxel_cm), _ptr(lh), _ptr(ld), n,
                                            None, os_))
    out = np.zeros((os_[2], os_[1], os_[0]), np.float32)
    _raise_status(lib, lib.ee_ct_to_density(int(device), C.byref(f), _ptr(h), float(iso_voxel_cm), _ptr(lh), _ptr(ld),
                                            n, _ptr(out), os_))
    return out


def fluence_projection(mask_vol, beams, supersample: bool = True, aperture_ready: bool = False, device: int = 0):
    """Binary conformal fluence maps of the beams through a mask volume
    (an inputs.Volume whose density holds the mask); list of [fy, fx]."""
    lib = load_library()
    m = np.ascontiguousarray(mask_vol.density, np.float32)
    eb = to_ee_beams(beams)
    out = np.zeros(sum(int(b.fmap_size[0]) * int(b.fmap_size[1]) for b in beams), np.float32)
    _raise_status(lib, lib.ee_fluence_projection(int(device), C.byref(_frame_of(mask_vol)), _ptr(m), eb, len(beams),
                                                 int(bool(supersample)), int(bool(aperture_ready)), _ptr(out)))
    res, o = [], 0
    for b in beams:
        n = int(b.fmap_size[0]) * int(b.fmap_size[1])
        res.append(out[o:o + n].reshape(int(b.fmap_size[1]), int(b.fmap_size[0])))
        o += n
    return res


def beam_source(beam):
    """Source position and direction of a beam (BEAM::reconfigure)."""
    lib = load_library()
    eb = to_ee_beams([beam])
    s = (C.c_float * 3)()
    d = (C.c_float * 3)()
    st = lib.ee_beam_source(eb, s, d)
    if st:
        raise EEError(st, lib.ee_last_error().decode())
    return np.array(list(s)), np.array(list(d))


# ------------------------------------------------ kernel tables (dsa files) --
DSA_NRADII, DSA_NANGLES, DSA_NCATEGORIES = 24, 48, 5


def read_spectrum_file(path: str, capacity: int = 64):
    """Spectrum file (ee_read_spectrum_file): energy, fluence (normalised to
    unit sum), mu, mu_en as float32 arrays and the kernel file names."""
    lib = load_library()
    a = [np.zeros(capacity, np.float32) for _ in range(4)]
    stride = 256
    names = C.create_string_buffer(capacity * stride)
    n = C.c_int(0)
    _raise_status(lib, lib.ee_read_spectrum_file(os.fsencode(path), capacity, *[_ptr(x) for x in a], names, stride,
                                                 C.byref(n)))
    k = n.value
    nm = [names.raw[i * stride:(i + 1) * stride].split(b"\0", 1)[0].decode() for i in range(k)]
    return a[0][:k].copy(), a[1][:k].copy(), a[2][:k].copy(), a[3][:k].copy(), nm


def read_mono_kernel(path: str) -> np.ndarray:
    """dsa point-kernel file (ee_read_mono_kernel): [5][48][24] float32."""
    out = np.zeros((DSA_NCATEGORIES, DSA_NANGLES, DSA_NRADII), np.float32)
    lib = load_library()
    _raise_status(lib, lib.ee_read_mono_kernel(os.fsencode(path), _ptr(out)))
    return out


def read_kernel_radii(path: str) -> np.ndarray:
    """radii.dat (ee_read_kernel_radii): the 24 radial boundaries [cm]."""
    out = np.zeros(DSA_NRADII, np.float32)
    lib = load_library()
    _raise_status(lib, lib.ee_read_kernel_radii(os.fsencode(path), _ptr(out)))
    return out


def cumulative_kernel(energy, fluence, mu, mono, ntheta: int = 8, nphi: int = 6, device: int = 0) -> dict:
    """The cumulative kernel tables on the GPU (ee_cumulative_kernel).
    mono: [nE][5][48][24].  Returns cum_total [ntheta][24], cum_weights
    [5][ntheta][24], poly_total [48][24], poly_weights [5][48][24], conv_theta
    and conv_phi (degrees, nphi*ntheta/2)."""
    lib = load_library()
    e, f, m = (np.ascontiguousarray(x, np.float32) for x in (energy, fluence, mu))
    k = np.ascontiguousarray(mono, np.float32)
    n = len(e)
    if k.shape != (n, DSA_NCATEGORIES, DSA_NANGLES, DSA_NRADII) or len(f) != n or len(m) != n:
        raise ValueError("mono must be [nE][5][48][24] with nE spectrum entries")
    nang = nphi * (ntheta // 2)
    out = dict(cum_total=np.zeros((ntheta, DSA_NRADII), np.float32),
               cum_weights=np.zeros((DSA_NCATEGORIES, ntheta, DSA_NRADII), np.float32),
               poly_total=np.zeros((DSA_NANGLES, DSA_NRADII), np.float32),
               poly_weights=np.zeros((DSA_NCATEGORIES, DSA_NANGLES, DSA_NRADII), np.float32),
               conv_theta=np.zeros(max(nang, 1), np.float32), conv_phi=np.zeros(max(nang, 1), np.float32))
    _raise_status(lib, lib.ee_cumulative_kernel(int(device), n, _ptr(e), _ptr(f), _ptr(m), _ptr(k), int(ntheta),
                                                int(nphi), *[_ptr(out[x]) for x in ("cum_total", "cum_weights",
                                                                                    "poly_total", "poly_weights",
                                                                                    "conv_theta", "conv_phi")]))
    return out


def fit_exp_kernel(radii, cum_total):
    """Per-cone double-exponential fit of a cumulative table
    (ee_fit_exp_kernel): params [ntheta][4] = (A, a, B, b) and the maximum
    fit error of each cone relative to its table maximum."""
    lib = load_library()
    r = np.ascontiguousarray(radii, np.float32)
    K = np.ascontiguousarray(cum_total, np.float32)
    nt = K.shape[0]
    params = np.zeros((nt, 4), np.float32)
    err = np.zeros(nt, np.float32)
    _raise_status(lib, lib.ee_fit_exp_kernel(nt, K.shape[1], _ptr(r), _ptr(K), _ptr(params), _ptr(err)))
    return params, err


def physics_from_kernel_files(spectrum_path: str, kernel_dir: str, ntheta: int = 8, nphi: int = 6,
                              spacing_cm: float = 0.25, penumbra_cm: float = 1.0, device: int = 0):
    """inputs.Physics from a spectrum file and its dsa point kernels (the
    files in kernel_dir, with radii.dat): the cumulative table built on the
    GPU, the double-exponential fit of it for the exp fast path."""
    from . import inputs
    energy, fluence, mu, mu_en, names = read_spectrum_file(spectrum_path)
    mono = np.stack([read_mono_kernel(os.path.join(kernel_dir, n)) for n in names])
    radii = read_kernel_radii(os.path.join(kernel_dir, "radii.dat"))
    t = cumulative_kernel(energy, fluence, mu, mono, ntheta, nphi, device)
    params, _ = fit_exp_kernel(radii, t["cum_total"])
    return inputs.Physics(energy=energy, fluence=fluence, mu=mu, mu_en=mu_en, ntheta=ntheta, nphi=nphi,
                          radii=radii.astype(np.float64), exp_params=params.astype(np.float64),
                          cumkern=t["cum_total"].astype(np.float64), theta_deg=t["conv_theta"].astype(np.float64),
                          phi_deg=t["conv_phi"].astype(np.float64), rev_latspacing=spacing_cm,
                          rev_longspacing=spacing_cm, penumbra=penumbra_cm)
