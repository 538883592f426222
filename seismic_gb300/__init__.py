"""seismic_gb300: GB300-native acoustic wave-equation engine (libswave).

Python mirror of the C-ABI in include/swave.h, shaped after the reference's
operator plug-in interface (propagator_acoustic, libs/libwave/Propagator.f90)
and its drivers (RTM_to_memory, BORN_to_memory, LSRTM_to_memory,
compute_fct_gdt, l_bfgs).  All compute runs in libswave.so's CUDA kernels;
importing this package on a machine where the library cannot be loaded
raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

# Status codes (sw_status).
SW_OK, SW_BAD_PARAM, SW_OOM_ADMISSION, SW_TIMEOUT, SW_NUMERIC, SW_CUDA_ERR, SW_UNSUPPORTED = range(7)
STATUS_NAMES = {0: "SW_OK", 1: "SW_BAD_PARAM", 2: "SW_OOM_ADMISSION", 3: "SW_TIMEOUT",
                4: "SW_NUMERIC", 5: "SW_CUDA_ERR", 6: "SW_UNSUPPORTED"}
# Procedure selectors of propagator_acoustic.
FD_FORWARD, FD_ADJOINT = 0, 1
INJ_NONE, INJ_SINC, INJ_SIMPLE, INJ_LSRTM_SINC = 0, 1, 2, 3
EXT_NONE, EXT_SINC, EXT_SIMPLE_AFWI, EXT_LSRTM_SINC, EXT_SINC_AFWI = 0, 1, 2, 3, 4
IMG_NONE, IMG_RTM, IMG_LSRTM, IMG_AFWI, IMG_BORN, IMG_AFWI_RHO = 0, 1, 2, 3, 4, 5
# Data norms (invparam%dat_nrm_type).
NRM_L1, NRM_L2, NRM_CAUCHY, NRM_HYPERBOLIC, NRM_HUBER = 1, 2, 3, 4, 12


class SwGenpar(C.Structure):
    """sw_genpar: the GeneralParam fields the propagation path reads."""
    _fields_ = [("twoD", C.c_int), ("nz", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("dz", C.c_float), ("dx", C.c_float), ("dy", C.c_float),
                ("oz", C.c_float), ("ox", C.c_float), ("oy", C.c_float),
                ("dt", C.c_float), ("nt", C.c_int), ("ntaper", C.c_int), ("lsinc", C.c_int),
                ("snapi", C.c_int), ("surf_type", C.c_int), ("shot_type", C.c_int),
                ("rec_type", C.c_int), ("fmax", C.c_float)]


class SwPropDesc(C.Structure):
    _fields_ = [("g", SwGenpar), ("tmin", C.c_int), ("tmax", C.c_int), ("tstep", C.c_int),
                ("fd_scheme", C.c_int), ("injection", C.c_int), ("extraction", C.c_int),
                ("extract_wave", C.c_int), ("imaging", C.c_int)]


_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)


class SwPropIO(C.Structure):
    _fields_ = [("vel", _fp), ("nsou", C.c_int), ("sou_coord", _fp), ("sou_trace", _fp),
                ("nrec", C.c_int), ("rec_coord", _fp), ("rec_trace", _fp), ("wave", _fp),
                ("image", _fp), ("illum", _fp), ("ref", _fp), ("final_u2", _fp),
                ("rho", _fp), ("image2", _fp)]


class SwFwiShot(C.Structure):
    _fields_ = [("sou_coord", C.c_float * 3), ("nrec", C.c_int), ("rec_coord", _fp),
                ("dobs", _fp), ("mute", _fp), ("resid", _fp)]


class SwFwiDesc(C.Structure):
    _fields_ = [("g", SwGenpar), ("aperture_x", C.c_float), ("aperture_y", C.c_float),
                ("illu_pow", C.c_float), ("smooth_rect1", C.c_int), ("smooth_rect2", C.c_int),
                ("smooth_rect3", C.c_int), ("smooth_doz", C.c_int), ("smooth_dox", C.c_int),
                ("smooth_doy", C.c_int), ("checkpoint_snaps", C.c_int),
                ("dat_nrm_type", C.c_int), ("dat_thresh", C.c_float),
                ("revolve_slots", C.c_int)]


class SwRegDesc(C.Structure):
    """sw_reg_desc: the SparseRegParam fields of compute_fct_gdt_reg."""
    _fields_ = [("nz", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("wantreg", C.c_int),
                ("wantlog", C.c_int), ("derivdx", C.c_int), ("derivdy", C.c_int),
                ("derivdz", C.c_int), ("log_z_plus", C.c_int), ("ntaperz", C.c_int),
                ("ntaperx", C.c_int), ("ntapery", C.c_int), ("mod_nrm_type", C.c_int),
                ("hin_nrm_type", C.c_int), ("compute_eps", C.c_int), ("compute_eps_log", C.c_int),
                ("ratio", C.c_float), ("ratio_log", C.c_float), ("zweight", _fp)]


class SwRegState(C.Structure):
    _fields_ = [("eps", C.c_float), ("eps_log", C.c_float), ("mod_thresh", C.c_float),
                ("hin_thresh", C.c_float)]


def reg_desc(nz, nx, ny=1, wantreg=False, wantlog=False, derivdx=False, derivdy=False,
             derivdz=False, log_z_plus=False, taperz=10, taperx=10, tapery=0,
             model_nrm_type=NRM_CAUCHY, hinge_nrm_type=NRM_L2, compute_eps=False,
             compute_eps_log=False, ratio=10.0, ratio_log=10.0):
    """A sw_reg_desc with Init_SparseRegularization's defaults
    (Sparse_regularization.f90:51-79)."""
    d = SwRegDesc()
    d.nz, d.nx, d.ny = nz, nx, ny
    d.wantreg, d.wantlog = int(wantreg), int(wantlog)
    d.derivdx, d.derivdy, d.derivdz, d.log_z_plus = map(int, (derivdx, derivdy, derivdz,
                                                             log_z_plus))
    d.ntaperz, d.ntaperx, d.ntapery = taperz, taperx, tapery
    d.mod_nrm_type, d.hin_nrm_type = model_nrm_type, hinge_nrm_type
    d.compute_eps, d.compute_eps_log = int(compute_eps), int(compute_eps_log)
    d.ratio, d.ratio_log = ratio, ratio_log
    return d


class SwWindow(C.Structure):
    _fields_ = [("oxw", C.c_float), ("oyw", C.c_float), ("endx", C.c_float),
                ("endy", C.c_float), ("nxw", C.c_int), ("nyw", C.c_int)]


class SwShot(C.Structure):
    _fields_ = [("sou_coord", C.c_float * 3), ("nrec", C.c_int), ("rec_coord", _fp),
                ("data", _fp), ("nt", C.c_int)]


# LBFGSOC's and MCSRCHOC's saved scalars, in the order of the reference's
# LbfgsDat.dat / McsrchDat.dat lines (nlinv_lbfgs.f:277-281, 725-730).
LBFGS_OC_LINES = (("gtol", "one", "zero", "gnorm", "stp1", "ftol", "stpmin"),
                  ("stpmax", "stp", "ys", "yy", "sq", "yr", "beta", "xnorm"),
                  ("mp", "lp", "iter", "nfun", "point", "ispt", "iypt", "maxfev", "info"),
                  ("bound", "npt", "cp", "i", "nfev", "inmc", "iycn", "iscn"),
                  ("finish",))
MCSRCH_OC_LINES = (("infoc", "j"), ("brackt", "stage1"),
                   ("dg", "dgm", "dginit", "dgtest", "dgx", "dgxm", "dgy", "dgym"),
                   ("finit", "ftest1", "fm", "fx", "fxm", "fy", "fym", "stx", "sty"),
                   ("stmin", "stmax", "width", "width1"))
_OC_INTS = {"mp", "lp", "iter", "nfun", "point", "ispt", "iypt", "maxfev", "info", "bound",
            "npt", "cp", "i", "nfev", "inmc", "iycn", "iscn", "finish", "infoc", "j", "brackt",
            "stage1"}


class SwLbfgsOcState(C.Structure):
    """sw_lbfgs_oc_state: the out-of-core L-BFGS's saved scalars."""
    _fields_ = [(nm, C.c_int if nm in _OC_INTS else C.c_double)
                for line in LBFGS_OC_LINES + MCSRCH_OC_LINES for nm in line]


class SwLbfgsOcDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("nparam", C.c_int), ("xmin", _dp),
                ("xmax", _dp), ("lbfgs_type", C.c_int), ("bound_type", C.c_int),
                ("stp1_opt", C.c_int), ("step_init", C.c_double), ("eps", C.c_double),
                ("xtol", C.c_double)]


class SwTuning(C.Structure):
    _fields_ = [("step_kernel", C.c_int), ("tile_z", C.c_int), ("tile_x", C.c_int),
                ("tile_y", C.c_int), ("graph_chunk", C.c_int), ("use_graph", C.c_int)]


class SwStats(C.Structure):
    _fields_ = [("launches_total", C.c_uint64), ("launches_step", C.c_uint64),
                ("points_updated", C.c_uint64), ("step_kernel_ms", C.c_double),
                ("step_kernel_timed", C.c_uint64), ("step_bytes", C.c_uint64),
                ("steps_forward", C.c_uint64), ("steps_backward", C.c_uint64),
                ("ckpt_advances", C.c_uint64), ("cnn_conv_ms", C.c_double),
                ("cnn_conv_timed", C.c_uint64), ("cnn_conv_bytes", C.c_uint64),
                ("cnn_conv_flops", C.c_uint64)]


# Every symbol of include/swave.h with its signature.
_SIGS = {
    "sw_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "sw_ctx_destroy": (C.c_int, [C.c_void_p]),
    "sw_last_error": (C.c_char_p, [C.c_void_p]),
    "sw_version": (C.c_char_p, []),
    "sw_vel_check": (C.c_int, [C.POINTER(SwGenpar), _fp, _fp, _fp]),
    "sw_propagate": (C.c_int, [C.c_void_p, C.POINTER(SwPropDesc), C.POINTER(SwPropIO)]),
    "sw_modeling": (C.c_int, [C.c_void_p, C.POINTER(SwGenpar), _fp, _fp, _fp, C.c_int, _fp, _fp, _fp]),
    "sw_modeling_noalloc": (C.c_int, [C.POINTER(SwGenpar), _fp, _fp, _fp, C.c_int, _fp, _fp]),
    "sw_cnn_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_uint64,
                                C.POINTER(C.c_void_p)]),
    "sw_cnn_destroy": (C.c_int, [C.c_void_p]),
    "sw_cnn_num_weights": (C.c_int, [C.c_void_p]),
    "sw_cnn_get_weights": (C.c_int, [C.c_void_p, _fp]),
    "sw_cnn_set_weights": (C.c_int, [C.c_void_p, _fp]),
    "sw_cnn_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _fp, _fp]),
    "sw_cnn_train_step": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _fp, _fp, C.c_float,
                                    C.POINTER(C.c_double)]),
    "sw_cnn_gradient": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp,
                                  C.POINTER(C.c_double)]),
    "sw_cnn_create3d": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_uint64,
                                  C.POINTER(C.c_void_p)]),
    "sw_cnn_forward3d": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _fp, _fp]),
    "sw_cnn_gradient3d": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp,
                                    _fp, C.POINTER(C.c_double)]),
    "sw_cnn_train_step3d": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _fp, _fp,
                                      C.c_float, C.POINTER(C.c_double)]),
    "sw_rtm": (C.c_int, [C.c_void_p, C.POINTER(SwGenpar), _fp, _fp, _fp, C.c_int, _fp, _fp, _fp, _fp]),
    "sw_born": (C.c_int, [C.c_void_p, C.POINTER(SwGenpar), _fp, _fp, _fp, _fp, C.c_int, _fp, _fp]),
    "sw_lsrtm": (C.c_int, [C.c_void_p, C.POINTER(SwGenpar), _fp, _fp, _fp, C.c_int, _fp, _fp, _fp, _fp]),
    "sw_born_wavelet": (C.c_int, [_fp, C.c_int, C.c_float]),
    "sw_fwi_fct_gdt": (C.c_int, [C.c_void_p, C.POINTER(SwFwiDesc), _fp, _fp, C.c_int,
                                 C.POINTER(SwFwiShot), _fp, _dp, _fp, _fp]),
    "sw_fwi_regularize": (C.c_int, [C.c_void_p, C.POINTER(SwRegDesc), C.POINTER(SwRegState),
                                    C.c_int, _fp, _fp, _dp, _fp]),
    "sw_lbfgs_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, _fp,
                                  C.c_int, C.c_int, _dp, C.POINTER(C.c_void_p)]),
    "sw_lbfgs_destroy": (C.c_int, [C.c_void_p]),
    "sw_lbfgs_step": (C.c_int, [C.c_void_p, _dp, C.c_double, _dp, C.c_double, C.c_double,
                                C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sw_lbfgs_diag": (C.c_int, [C.c_void_p, _dp]),
    "sw_lbfgs_oc_step": (C.c_int, [C.c_void_p, C.POINTER(SwLbfgsOcDesc), _dp, C.c_double, _dp,
                                   _dp, _dp, C.POINTER(SwLbfgsOcState), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int)]),
    "sw_rtm_job_create": (C.c_int, [C.c_void_p, C.POINTER(SwGenpar), C.c_float, C.c_float, _fp,
                                    _fp, C.c_int, C.POINTER(SwShot), C.POINTER(C.c_void_p)]),
    "sw_rtm_job_set_batch": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "sw_rtm_job_run": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "sw_rtm_job_model": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(_fp)]),
    "sw_rtm_job_admit": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "sw_rtm_job_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]),
    "sw_rtm_job_result": (C.c_int, [C.c_void_p, _fp, _fp, _fp]),
    "sw_rtm_job_reset": (C.c_int, [C.c_void_p]),
    "sw_rtm_job_destroy": (C.c_int, [C.c_void_p]),
    "sw_ctx_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(SwTuning)]),
    "sw_ctx_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(SwTuning)]),
    "sw_ctx_get_stats": (C.c_int, [C.c_void_p, C.POINTER(SwStats)]),
    "sw_ctx_reset_stats": (C.c_int, [C.c_void_p]),
    "sw_ctx_set_boundary": (C.c_int, [C.c_void_p, C.c_int]),
    "sw_rho_wavelet": (C.c_int, [_fp, C.c_int, C.c_int]),
    "sw_bandpass": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                              C.c_int, C.c_int, C.c_int, _fp]),
    "sw_mute_mask": (C.c_int, [C.c_int, C.c_int, C.c_float, C.c_float, _fp, _fp, C.c_float,
                               C.c_float, C.c_float, C.c_float, C.c_float, _fp]),
    "sw_shot_window": (C.c_int, [C.POINTER(SwGenpar), C.c_float, C.c_float, _fp, C.c_int, _fp,
                                 C.POINTER(SwWindow)]),
    "sw_window_extract": (C.c_int, [C.POINTER(SwGenpar), C.POINTER(SwWindow), _fp, _fp]),
    "sw_window_scatter_add": (C.c_int, [C.POINTER(SwGenpar), C.POINTER(SwWindow), _fp, _fp]),
    "sw_ctx_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
}

_lib = None


class SwaveError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load_library(path: str | None = None) -> C.CDLL:
    """Loads libswave.so (built by build.py).  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libswave.so not found at {p}: run seismic_gb300.build.build_library()")
    lib = C.CDLL(p)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _f32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_fp)


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def make_genpar(nz, nx, ny=1, dz=10.0, dx=10.0, dy=1.0, oz=0.0, ox=0.0, oy=0.0, dt=1e-3,
                nt=1000, ntaper=20, lsinc=7, snapi=4, twoD=None, fmax=30.0) -> SwGenpar:
    """GeneralParam defaults follow read_3D_params (libs/libwave/ReadParam.f90:18-53)."""
    if twoD is None:
        twoD = ny == 1
    return SwGenpar(int(twoD), nz, nx, ny, dz, dx, dy if not twoD else 1.0, oz, ox, oy, dt, nt,
                    ntaper, lsinc, snapi, 0, 0, 0, fmax)


def padded_shape(g: SwGenpar) -> tuple[int, int, int]:
    """(n3p, n2p, n1p) of the padded arrays u(nmin1-4:nmax1+4, ...); the top
    padding follows shot_type and surf_type (ExtractPadModel.f90:228-234)."""
    nmin1 = -g.ntaper + 1
    if g.shot_type > 0:
        nmin1 = -(g.ntaper + g.lsinc // 2 + 2) + 1
    if g.surf_type > 0:
        nmin1 = -g.lsinc + 1
    n1p = (g.nz + g.ntaper + 4) - (nmin1 - 4) + 1
    n2p = g.nx + 2 * g.ntaper + 8
    n3p = 1 if g.twoD else g.ny + 2 * g.ntaper + 8
    return (n3p, n2p, n1p)


class Context:
    """One CUDA stream + device buffers (sw_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        code = self.lib.sw_ctx_create(device, C.byref(h))
        if code != SW_OK:
            raise SwaveError(code, "sw_ctx_create failed (is a CUDA device visible?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.sw_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, code: int):
        if code != SW_OK:
            raise SwaveError(code, (self.lib.sw_last_error(self.h) or b"").decode())

    # -- instrumentation -------------------------------------------------
    def stats(self) -> dict:
        s = SwStats()
        self._check(self.lib.sw_ctx_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in SwStats._fields_}

    def reset_stats(self):
        self._check(self.lib.sw_ctx_reset_stats(self.h))

    def tuning(self) -> dict:
        t = SwTuning()
        self._check(self.lib.sw_ctx_get_tuning(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in SwTuning._fields_}

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        t = SwTuning(**cur)
        self._check(self.lib.sw_ctx_set_tuning(self.h, C.byref(t)))

    def set_boundary(self, mode: int):
        """0: Higdon absorbing boundary (reference); 1: rigid (exact-adjoint mode)."""
        self._check(self.lib.sw_ctx_set_boundary(self.h, int(mode)))

    def set_profiling(self, on: bool):
        self._check(self.lib.sw_ctx_set_profiling(self.h, int(bool(on))))

    # -- propagator_acoustic ----------------------------------------------
    def propagate(self, desc: SwPropDesc, vel, sou_coord=None, sou_trace=None, rec_coord=None,
                  rec_trace=None, wave=None, image=None, illum=None, ref=None, final_u2=None,
                  rho=None, image2=None):
        """sw_propagate; array arguments are modified in place like the reference."""
        io = SwPropIO()
        vel = _f32(vel)
        io.vel = fptr(vel)
        keep = [vel]
        if sou_coord is not None:
            sc, st = _f32(sou_coord), _f32(sou_trace)
            keep += [sc, st]
            io.nsou, io.sou_coord, io.sou_trace = sc.size // 3, fptr(sc), fptr(st)
        if rec_coord is not None:
            rc = _f32(rec_coord)
            keep.append(rc)
            io.nrec, io.rec_coord, io.rec_trace = rc.size // 3, fptr(rc), fptr(rec_trace)
        io.wave, io.image, io.illum = fptr(wave), fptr(image), fptr(illum)
        if ref is not None:
            ref = _f32(ref)
            keep.append(ref)
        io.ref = fptr(ref)
        io.final_u2 = fptr(final_u2)
        if rho is not None:
            rho = _f32(rho)
            keep.append(rho)
        io.rho = fptr(rho)
        io.image2 = fptr(image2)
        self._check(self.lib.sw_propagate(self.h, C.byref(desc), C.byref(io)))

    def bandpass(self, traces, dt: float, flo: float = 0.0, fhi: float = 20.0, nplo: int = 14,
                 nphi: int = 14, phase: int = 0) -> np.ndarray:
        """sw_bandpass of a (ntr, nt) array; returns the filtered copy."""
        t = _f32(traces).copy()
        ntr, nt = t.shape
        self._check(self.lib.sw_bandpass(self.h, ntr, nt, dt, flo, fhi, nplo, nphi, phase,
                                         fptr(t)))
        return t

    # -- drivers -----------------------------------------------------------
    def modeling(self, g: SwGenpar, vel, sou_coord, wavelet, rec_coord, final_u2=False):
        vel, sc, w, rc = _f32(vel), _f32(sou_coord), _f32(wavelet), _f32(rec_coord)
        nrec = rc.size // 3
        data = np.zeros((nrec, g.nt), np.float32)
        fu = np.zeros(padded_shape(g), np.float32) if final_u2 else None
        self._check(self.lib.sw_modeling(self.h, C.byref(g), fptr(vel), fptr(sc), fptr(w), nrec,
                                         fptr(rc), fptr(data), fptr(fu)))
        return (data, fu) if final_u2 else data

    def rtm(self, g, vel, sou_coord, wavelet, rec_coord, data):
        vel, sc, w, rc, d = _f32(vel), _f32(sou_coord), _f32(wavelet), _f32(rec_coord), _f32(data)
        n = g.nz * g.nx * g.ny
        image, illum = np.zeros(n, np.float32), np.zeros(n, np.float32)
        self._check(self.lib.sw_rtm(self.h, C.byref(g), fptr(vel), fptr(sc), fptr(w), rc.size // 3,
                                    fptr(rc), fptr(d), fptr(image), fptr(illum)))
        return image, illum

    def lsrtm(self, g, vel, sou_coord, wavelet, rec_coord, data):
        vel, sc, w, rc, d = _f32(vel), _f32(sou_coord), _f32(wavelet), _f32(rec_coord), _f32(data)
        n = g.nz * g.nx * g.ny
        image, illum = np.zeros(n, np.float32), np.zeros(n, np.float32)
        self._check(self.lib.sw_lsrtm(self.h, C.byref(g), fptr(vel), fptr(sc), fptr(w),
                                      rc.size // 3, fptr(rc), fptr(d), fptr(image), fptr(illum)))
        return image, illum

    def born(self, g, vel, ref, sou_coord, wavelet, rec_coord):
        vel, r, sc, w, rc = _f32(vel), _f32(ref), _f32(sou_coord), _f32(wavelet), _f32(rec_coord)
        nrec = rc.size // 3
        data = np.zeros((nrec, g.nt), np.float32)
        self._check(self.lib.sw_born(self.h, C.byref(g), fptr(vel), fptr(r), fptr(sc), fptr(w),
                                     nrec, fptr(rc), fptr(data)))
        return data

    def fwi_fct_gdt(self, desc: SwFwiDesc, vel, wavelet, shots, vpmask=None, want_resid=False):
        """compute_fct_gdt.  shots: list of dicts(sou=(z,x,y), rec=(n,3), dobs=(n,nt), mute=...)."""
        g = desc.g
        vel, w = _f32(vel), _f32(wavelet)
        arr = (SwFwiShot * len(shots))()
        keep = []
        resids = []
        for i, s in enumerate(shots):
            rc, dob = _f32(s["rec"]), _f32(s["dobs"])
            mu = _f32(s["mute"]) if s.get("mute") is not None else None
            keep += [rc, dob, mu]
            arr[i].sou_coord[:] = [float(v) for v in s["sou"]]
            arr[i].nrec = rc.size // 3
            arr[i].rec_coord, arr[i].dobs, arr[i].mute = fptr(rc), fptr(dob), fptr(mu)
            r = np.zeros((rc.size // 3, g.nt), np.float32) if want_resid else None
            resids.append(r)
            arr[i].resid = fptr(r)
        n = g.nz * g.nx * g.ny
        grad, illum = np.zeros(n, np.float32), np.zeros(n, np.float32)
        f = C.c_double(0.0)
        m = _f32(vpmask) if vpmask is not None else None
        self._check(self.lib.sw_fwi_fct_gdt(self.h, C.byref(desc), fptr(vel), fptr(w), len(shots),
                                            arr, fptr(m), C.byref(f), fptr(grad), fptr(illum)))
        return (f.value, grad, illum, resids) if want_resid else (f.value, grad, illum)

    def lbfgs_oc_step(self, desc: SwLbfgsOcDesc, x: np.ndarray, f: float, g, w: np.ndarray,
                      diag: np.ndarray, state: SwLbfgsOcState, iflag: int,
                      myinfo: int = 0) -> tuple[int, int]:
        """sw_lbfgs_oc_step: one LBFGSOC call; x, w, diag (float64) and state
        are updated in place; returns (iflag, myinfo)."""
        fl, mi = C.c_int(iflag), C.c_int(myinfo)
        self._check(self.lib.sw_lbfgs_oc_step(self.h, C.byref(desc), dptr(x), float(f),
                                              dptr(np.ascontiguousarray(g, np.float64)),
                                              dptr(w), dptr(diag), C.byref(state), C.byref(fl),
                                              C.byref(mi)))
        return fl.value, mi.value

    def fwi_regularize(self, desc: SwRegDesc, state: SwRegState, eval_, vel, f, grad,
                       vpmask=None, zweight=None):
        """compute_fct_gdt_reg's terms: returns (f, grad) after the sparse and
        logistic regularisation and the mask; state is updated in place."""
        vel = _f32(vel)
        g = np.array(grad, np.float32, copy=True).ravel()
        m = _f32(vpmask) if vpmask is not None else None
        zw = _f32(zweight) if zweight is not None else None
        desc.zweight = fptr(zw)
        fd = C.c_double(f)
        try:
            self._check(self.lib.sw_fwi_regularize(self.h, C.byref(desc), C.byref(state),
                                                   int(eval_), fptr(vel), fptr(m), C.byref(fd),
                                                   fptr(g)))
        finally:
            desc.zweight = None
        return fd.value, g


def make_shots(shots) -> tuple:
    """sw_shot array from dicts(sou=(z,x,y), rec=(n,3), data=(n,nt)); returns (array, keep)."""
    arr = (SwShot * len(shots))()
    keep = []
    for i, s in enumerate(shots):
        rc = _f32(s["rec"])
        d = _f32(s["data"]) if s.get("data") is not None else None
        keep += [rc, d]
        arr[i].sou_coord[:] = [float(v) for v in s["sou"]]
        arr[i].nrec = rc.size // 3
        arr[i].rec_coord, arr[i].data = fptr(rc), fptr(d)
        arr[i].nt = int(d.shape[-1]) if d is not None and d.ndim == 2 else int(s["nt"])
    return arr, keep


class RTMJob:
    """Multi-shot RTM (sw_rtm_job_*): windows, HBM admission, stacking."""

    def __init__(self, ctx: Context, model: SwGenpar, vel, wavelet, shots, aperture_x=0.0,
                 aperture_y=0.0):
        self.ctx = ctx
        self.g = model
        arr, keep = make_shots(shots)
        v, w = _f32(vel), _f32(wavelet)
        h = C.c_void_p()
        ctx._check(ctx.lib.sw_rtm_job_create(ctx.h, C.byref(model), aperture_x, aperture_y,
                                             fptr(v), fptr(w), len(shots), arr, C.byref(h)))
        self.h = h
        self.nshot = len(shots)
        self._nrec = [np.asarray(x["rec"]).size // 3 for x in shots]
        self._nt = [int(arr[i].nt) for i in range(len(shots))]

    def model(self, first: int = 0, count: int | None = None) -> list:
        """Batched forward modelling of shots [first, first+count)."""
        count = self.nshot - first if count is None else count
        outs = [np.zeros((self._nrec[q], self._nt[q]), np.float32) for q in range(first, first + count)]
        ptrs = (_fp * count)(*[fptr(o) for o in outs])
        self.ctx._check(self.ctx.lib.sw_rtm_job_model(self.h, first, count, ptrs))
        return outs

    def set_batch(self, max_shots: int, mem_fraction: float = 0.85):
        self.ctx._check(self.ctx.lib.sw_rtm_job_set_batch(self.h, max_shots, mem_fraction))

    def run(self, first: int = 0, count: int | None = None):
        count = self.nshot - first if count is None else count
        self.ctx._check(self.ctx.lib.sw_rtm_job_run(self.h, first, count))

    def admit(self, first: int = 0, modeling: bool = False) -> int:
        """Shots from `first` that one batch takes now (sw_rtm_job_admit)."""
        n = C.c_int()
        self.ctx._check(self.ctx.lib.sw_rtm_job_admit(self.h, first, int(modeling), C.byref(n)))
        return n.value

    def info(self) -> tuple[int, int]:
        b, p = C.c_int(), C.c_uint64()
        self.ctx._check(self.ctx.lib.sw_rtm_job_info(self.h, C.byref(b), C.byref(p)))
        return b.value, p.value

    def result(self, normalised: bool = True):
        n = self.g.nz * self.g.nx * self.g.ny
        im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
        nm = np.zeros(n, np.float32) if normalised else None
        self.ctx._check(self.ctx.lib.sw_rtm_job_result(self.h, fptr(im), fptr(il), fptr(nm)))
        return (im, il, nm) if normalised else (im, il)

    def reset(self):
        self.ctx._check(self.ctx.lib.sw_rtm_job_reset(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sw_rtm_job_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lbfgs_oc_desc(n: int, m: int = 5, nparam: int = 1, xmin=None, xmax=None,
                  lbfgs_type: int = 1, bound_type: int = 1, stp1_opt: int = 1,
                  step_init: float = 999999.0, eps: float = 1.0e-20,
                  xtol: float = float(np.finfo(np.float64).eps)) -> tuple:
    """sw_lbfgs_oc_desc (and the bound arrays it points at, to keep alive)."""
    lo = np.ascontiguousarray(np.zeros(nparam) if xmin is None else xmin, np.float64)
    hi = np.ascontiguousarray(np.zeros(nparam) if xmax is None else xmax, np.float64)
    d = SwLbfgsOcDesc(n, m, nparam, dptr(lo), dptr(hi), lbfgs_type, bound_type, stp1_opt,
                      step_init, eps, xtol)
    return d, (lo, hi)


class LBFGS:
    """Reverse-communication L-BFGS (LBFGS, libs/libinv/lbfgs.f) on the device."""

    def __init__(self, ctx: Context, n: int, m: int = 5, xmin=1500.0, xmax=4500.0, mask=None,
                 bound_type: int = 2, freeze_soft: bool = True, xinit=None):
        self.ctx = ctx
        mask = np.ones(n, np.float32) if mask is None else _f32(mask)
        xinit = np.zeros(n) if xinit is None else np.ascontiguousarray(xinit, np.float64)
        self._keep = (mask, xinit)
        h = C.c_void_p()
        ctx._check(ctx.lib.sw_lbfgs_create(ctx.h, n, m, xmin, xmax, fptr(mask), bound_type,
                                           int(freeze_soft), dptr(xinit), C.byref(h)))
        self.h = h
        self.iflag = C.c_int(0)
        self.myinfo = C.c_int(0)

    def step(self, x: np.ndarray, f: float, g: np.ndarray, eps=1e-20, xtol=np.finfo(float).eps):
        self.myinfo.value = 0
        self.ctx._check(self.ctx.lib.sw_lbfgs_step(self.h, dptr(x), float(f),
                                                   dptr(np.ascontiguousarray(g, np.float64)),
                                                   eps, xtol, C.byref(self.iflag),
                                                   C.byref(self.myinfo)))
        return self.iflag.value, self.myinfo.value

    def diag(self) -> np.ndarray:
        out = np.zeros(8)
        self.ctx._check(self.ctx.lib.sw_lbfgs_diag(self.h, dptr(out)))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.sw_lbfgs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def vel_check(g: SwGenpar, vel) -> tuple[int, float, float]:
    lib = load_library()
    v = _f32(vel)
    a, b = C.c_float(), C.c_float()
    code = lib.sw_vel_check(C.byref(g), fptr(v), C.byref(a), C.byref(b))
    return code, a.value, b.value


def shot_window(model: SwGenpar, aperture_x: float, aperture_y: float, sou_coord,
                rec_coord) -> tuple[SwWindow, SwGenpar]:
    """The shot's window (sw_shot_window) and the window's genpar."""
    lib = load_library()
    s, r = _f32(sou_coord), _f32(rec_coord)
    w = SwWindow()
    code = lib.sw_shot_window(C.byref(model), aperture_x, aperture_y, fptr(s), r.size // 3,
                              fptr(r), C.byref(w))
    if code != SW_OK:
        raise SwaveError(code, "sw_shot_window")
    g = SwGenpar.from_buffer_copy(model)
    g.nx, g.ny, g.ox, g.oy = w.nxw, w.nyw, w.oxw, w.oyw
    return w, g


def window_extract(model: SwGenpar, w: SwWindow, big) -> np.ndarray:
    lib = load_library()
    b = _f32(big)
    out = np.zeros((w.nyw, w.nxw, model.nz), np.float32)
    code = lib.sw_window_extract(C.byref(model), C.byref(w), fptr(b), fptr(out))
    if code != SW_OK:
        raise SwaveError(code, "sw_window_extract")
    return out if not model.twoD else out[0]


def window_scatter_add(model: SwGenpar, w: SwWindow, small, big: np.ndarray) -> np.ndarray:
    """big += the window columns inside the model (in place; big float32)."""
    lib = load_library()
    s = _f32(small)
    assert big.dtype == np.float32 and big.flags.c_contiguous
    code = lib.sw_window_scatter_add(C.byref(model), C.byref(w), fptr(s), fptr(big))
    if code != SW_OK:
        raise SwaveError(code, "sw_window_scatter_add")
    return big


class CNN:
    """sw_cnn_*: the convolutional gradient preconditioner on the tensor cores."""

    def __init__(self, ctx: "Context", channels=(2, 32, 32, 32, 1), seed: int = 0,
                 three_d: bool = False):
        """three_d: 3 x 3 x 3 kernels on (ny, nx, nz) volumes instead of 3 x 3
        kernels on (nx, nz) images."""
        self.ctx = ctx
        self.channels = list(channels)
        self.three_d = bool(three_d)
        ch = (C.c_int * len(channels))(*channels)
        h = C.c_void_p()
        create = ctx.lib.sw_cnn_create3d if three_d else ctx.lib.sw_cnn_create
        ctx._check(create(ctx.h, len(channels) - 1, ch, seed, C.byref(h)))
        self.h = h

    @property
    def num_weights(self) -> int:
        return self.ctx.lib.sw_cnn_num_weights(self.h)

    def get_weights(self) -> np.ndarray:
        w = np.zeros(self.num_weights, np.float32)
        self.ctx._check(self.ctx.lib.sw_cnn_get_weights(self.h, fptr(w)))
        return w

    def set_weights(self, w) -> None:
        w = _f32(w)
        assert w.size == self.num_weights
        self.ctx._check(self.ctx.lib.sw_cnn_set_weights(self.h, fptr(w)))

    def forward(self, x) -> np.ndarray:
        """x: (channels[0], nx, nz) planar image stack (z fastest), or
        (channels[0], ny, nx, nz) for a 3 x 3 x 3 network."""
        x = _f32(x)
        if self.three_d:
            c, ny, nx, nz = x.shape
            out = np.zeros((ny, nx, nz), np.float32)
            self.ctx._check(self.ctx.lib.sw_cnn_forward3d(self.h, nz, nx, ny, fptr(x), fptr(out)))
            return out
        c, nx, nz = x.shape
        out = np.zeros((nx, nz), np.float32)
        self.ctx._check(self.ctx.lib.sw_cnn_forward(self.h, nz, nx, fptr(x), fptr(out)))
        return out

    def gradient(self, x, target) -> tuple[np.ndarray, float]:
        """Gradient of the batch-mean loss (packed like the weights) and that
        loss; x: (batch, channels[0], [ny,] nx, nz), target: (batch, [ny,] nx, nz)."""
        x, t = _f32(x), _f32(target)
        g = np.zeros(self.num_weights, np.float32)
        loss = C.c_double()
        if self.three_d:
            b, c, ny, nx, nz = x.shape
            self.ctx._check(self.ctx.lib.sw_cnn_gradient3d(self.h, b, nz, nx, ny, fptr(x), fptr(t),
                                                           fptr(g), C.byref(loss)))
        else:
            b, c, nx, nz = x.shape
            self.ctx._check(self.ctx.lib.sw_cnn_gradient(self.h, b, nz, nx, fptr(x), fptr(t),
                                                         fptr(g), C.byref(loss)))
        return g, loss.value

    def train_step(self, x, target, lr: float = 1e-3) -> float:
        """x: (batch, channels[0], [ny,] nx, nz); target: (batch, [ny,] nx, nz)."""
        x, t = _f32(x), _f32(target)
        loss = C.c_double()
        if self.three_d:
            b, c, ny, nx, nz = x.shape
            self.ctx._check(self.ctx.lib.sw_cnn_train_step3d(self.h, b, nz, nx, ny, fptr(x),
                                                             fptr(t), float(lr), C.byref(loss)))
        else:
            b, c, nx, nz = x.shape
            self.ctx._check(self.ctx.lib.sw_cnn_train_step(self.h, b, nz, nx, fptr(x), fptr(t),
                                                           float(lr), C.byref(loss)))
        return loss.value

    def close(self):
        if self.h:
            self.ctx.lib.sw_cnn_destroy(self.h)
            self.h = None


def modeling_noalloc(g: SwGenpar, vel, sou_coord, wavelet, rec_coord) -> np.ndarray:
    """sw_modeling_noalloc: 2D shot modelling on the current device that
    allocates no device memory (results equal Context.modeling).  Raises
    SwaveError with SW_OOM_ADMISSION when the run exceeds the library's fixed
    32 MiB scratch array, and with SW_UNSUPPORTED for a free surface or
    mirror sources / receivers (surf_type, shot_type, rec_type other than 0)."""
    lib = load_library()
    vel, sc, w, rc = _f32(vel), _f32(sou_coord), _f32(wavelet), _f32(rec_coord)
    nrec = rc.size // 3
    data = np.zeros((nrec, g.nt), np.float32)
    code = lib.sw_modeling_noalloc(C.byref(g), fptr(vel), fptr(sc), fptr(w), nrec, fptr(rc),
                                   fptr(data))
    if code != SW_OK:
        raise SwaveError(code, "sw_modeling_noalloc")
    return data


def mute_mask(nt: int, dt: float, sou_coord, rec_coord, ot: float = 0.0, v0: float = 1500.0,
              v1: float = 10000.0, t0: float = 0.0, t1: float = 40.0,
              tramp: float = 0.5) -> np.ndarray:
    """sw_mute_mask: (nrec, nt) mute mask of one gather (reference defaults)."""
    lib = load_library()
    s, r = _f32(sou_coord), _f32(rec_coord)
    m = np.zeros((r.size // 3, nt), np.float32)
    code = lib.sw_mute_mask(r.size // 3, nt, dt, ot, fptr(s), fptr(r), v0, v1, t0, t1, tramp,
                            fptr(m))
    if code != SW_OK:
        raise SwaveError(code, "sw_mute_mask")
    return m


def rho_wavelet(w, lsinc: int = 7) -> np.ndarray:
    """readsou's half-sample shift of the wavelet for the density path."""
    lib = load_library()
    w = _f32(w).copy()
    code = lib.sw_rho_wavelet(fptr(w), w.size, lsinc)
    if code != SW_OK:
        raise SwaveError(code, "sw_rho_wavelet")
    return w


def born_wavelet(w, dt: float) -> np.ndarray:
    lib = load_library()
    w = _f32(w).copy()
    code = lib.sw_born_wavelet(fptr(w), w.size, dt)
    if code != SW_OK:
        raise SwaveError(code, "sw_born_wavelet")
    return w
