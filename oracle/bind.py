"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py.  Parity status of the oracle: unpinned (see
oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_lib = None


def _types():
    from seismic_gb300 import SwFwiDesc, SwFwiShot, SwGenpar, SwPropDesc, SwPropIO
    return SwGenpar, SwPropDesc, SwPropIO, SwFwiDesc, SwFwiShot


class OrPropIO64(C.Structure):
    _fields_ = [("vel", _dp), ("nsou", C.c_int), ("sou_coord", _dp), ("sou_trace", _dp),
                ("nrec", C.c_int), ("rec_coord", _dp), ("rec_trace", _dp), ("wave", _dp),
                ("image", _dp), ("illum", _dp), ("ref", _dp), ("final_u2", _dp),
                ("rho", _dp), ("image2", _dp)]


def load(build_if_missing: bool = True) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from seismic_gb300.build import build_oracle
        build_oracle()
    lib = C.CDLL(LIB_PATH)
    G, D, IO, FD, FS = _types()
    g, d = C.POINTER(G), C.POINTER(D)
    sig = {
        "oracle_propagate_f32": [d, C.POINTER(IO)],
        "oracle_propagate_f64": [d, C.POINTER(OrPropIO64)],
        "oracle_modeling_f32": [g, _fp, _fp, _fp, C.c_int, _fp, _fp, _fp],
        "oracle_modeling_f64": [g, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp],
        "oracle_rtm_f32": [g, _fp, _fp, _fp, C.c_int, _fp, _fp, _fp, _fp],
        "oracle_rtm_f64": [g, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp, _dp],
        "oracle_born_f32": [g, _fp, _fp, _fp, _fp, C.c_int, _fp, _fp],
        "oracle_born_f64": [g, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp],
        "oracle_lsrtm_f32": [g, _fp, _fp, _fp, C.c_int, _fp, _fp, _fp, _fp],
        "oracle_lsrtm_f64": [g, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp, _dp],
        "oracle_born_wavelet": [_fp, C.c_int, C.c_float],
        "oracle_rho_wavelet": [_fp, C.c_int, C.c_int],
        "oracle_mute_mask": [C.c_int, C.c_int, C.c_float, C.c_float, _fp, _fp, C.c_float,
                             C.c_float, C.c_float, C.c_float, C.c_float, _fp],
        "oracle_bandpass": [_fp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                            C.c_int, C.c_int],
        "oracle_vel_check": [g, _fp, _fp, _fp],
        "oracle_fwi_fct_gdt": [C.POINTER(FD), _fp, _fp, C.c_int, C.POINTER(FS), _fp, _dp, _fp, _fp],
        "oracle_fwi_regularize": [C.c_void_p, C.c_void_p, C.c_int, _fp, _fp, _dp, _fp],
        "oracle_data_norm": [C.c_int, C.c_float, C.c_int, C.c_int, _fp, _fp, _fp, _fp, _dp],
        "oracle_rtm_job": [g, C.c_float, C.c_float, _fp, _fp, C.c_int, C.c_void_p, _fp, _fp, _fp],
        "oracle_stencil_f64": [g, C.c_int, _dp, _dp, _dp],
        "oracle_stencil_rho_f64": [g, _dp, _dp, _dp, _dp],
        "oracle_triangle2": [_fp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                             C.c_int, C.c_int],
        "oracle_lbfgs_step": [C.c_void_p, _dp, C.c_double, _dp, C.c_double, C.c_double,
                              C.POINTER(C.c_int), C.POINTER(C.c_int)],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    from seismic_gb300 import SwLbfgsOcDesc, SwLbfgsOcState
    lib.oracle_lbfgs_oc_step.argtypes = [C.POINTER(SwLbfgsOcDesc), _dp, C.c_double, _dp, _dp,
                                         _dp, C.POINTER(SwLbfgsOcState), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]
    lib.oracle_lbfgs_oc_step.restype = C.c_int
    lib.oracle_mksinc.argtypes = [_fp, C.c_int, C.c_float]
    lib.oracle_mksinc.restype = None
    lib.oracle_lbfgs_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _fp, C.c_int,
                                        C.c_int, _dp]
    lib.oracle_lbfgs_create.restype = C.c_void_p
    lib.oracle_lbfgs_destroy.argtypes = [C.c_void_p]
    lib.oracle_lbfgs_destroy.restype = None
    lib.oracle_lbfgs_diag.argtypes = [C.c_void_p, _dp]
    lib.oracle_lbfgs_diag.restype = None
    _lib = lib
    return lib


def _f(a):
    a = np.ascontiguousarray(a, np.float32)
    return a, a.ctypes.data_as(_fp)


def _d(a):
    a = np.ascontiguousarray(a, np.float64)
    return a, a.ctypes.data_as(_dp)


def _chk(code, what):
    if code != 0:
        raise RuntimeError(f"oracle {what} failed with status {code}")


def modeling(g, vel, sou, wavelet, rec, final_u2=False, f64=False):
    lib = load()
    from seismic_gb300 import padded_shape
    nrec = np.asarray(rec).size // 3
    if f64:
        v, pv = _d(vel); s, ps = _d(sou); w, pw = _d(wavelet); r, pr = _d(rec)
        data = np.zeros((nrec, g.nt)); fu = np.zeros(padded_shape(g)) if final_u2 else None
        _chk(lib.oracle_modeling_f64(C.byref(g), pv, ps, pw, nrec, pr, data.ctypes.data_as(_dp),
                                     fu.ctypes.data_as(_dp) if fu is not None else None), "modeling")
    else:
        v, pv = _f(vel); s, ps = _f(sou); w, pw = _f(wavelet); r, pr = _f(rec)
        data = np.zeros((nrec, g.nt), np.float32)
        fu = np.zeros(padded_shape(g), np.float32) if final_u2 else None
        _chk(lib.oracle_modeling_f32(C.byref(g), pv, ps, pw, nrec, pr, data.ctypes.data_as(_fp),
                                     fu.ctypes.data_as(_fp) if fu is not None else None), "modeling")
    return (data, fu) if final_u2 else data


def rtm(g, vel, sou, wavelet, rec, data, f64=False):
    lib = load()
    n = g.nz * g.nx * g.ny
    if f64:
        v, pv = _d(vel); s, ps = _d(sou); w, pw = _d(wavelet); r, pr = _d(rec); d, pd = _d(data)
        im, il = np.zeros(n), np.zeros(n)
        _chk(lib.oracle_rtm_f64(C.byref(g), pv, ps, pw, r.size // 3, pr, pd,
                                im.ctypes.data_as(_dp), il.ctypes.data_as(_dp)), "rtm")
        return im, il
    v, pv = _f(vel); s, ps = _f(sou); w, pw = _f(wavelet); r, pr = _f(rec); d, pd = _f(data)
    im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
    _chk(lib.oracle_rtm_f32(C.byref(g), pv, ps, pw, r.size // 3, pr, pd, im.ctypes.data_as(_fp),
                            il.ctypes.data_as(_fp)), "rtm")
    return im, il


def lsrtm(g, vel, sou, wavelet, rec, data, f64=False):
    lib = load()
    n = g.nz * g.nx * g.ny
    if f64:
        v, pv = _d(vel); s, ps = _d(sou); w, pw = _d(wavelet); r, pr = _d(rec); d, pd = _d(data)
        im, il = np.zeros(n), np.zeros(n)
        _chk(lib.oracle_lsrtm_f64(C.byref(g), pv, ps, pw, r.size // 3, pr, pd,
                                  im.ctypes.data_as(_dp), il.ctypes.data_as(_dp)), "lsrtm")
    else:
        v, pv = _f(vel); s, ps = _f(sou); w, pw = _f(wavelet); r, pr = _f(rec); d, pd = _f(data)
        im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
        _chk(lib.oracle_lsrtm_f32(C.byref(g), pv, ps, pw, r.size // 3, pr, pd,
                                  im.ctypes.data_as(_fp), il.ctypes.data_as(_fp)), "lsrtm")
    return im, il


def born(g, vel, ref, sou, wavelet, rec, f64=False):
    lib = load()
    nrec = np.asarray(rec).size // 3
    if f64:
        v, pv = _d(vel); f, pf = _d(ref); s, ps = _d(sou); w, pw = _d(wavelet); r, pr = _d(rec)
        data = np.zeros((nrec, g.nt))
        _chk(lib.oracle_born_f64(C.byref(g), pv, pf, ps, pw, nrec, pr, data.ctypes.data_as(_dp)),
             "born")
    else:
        v, pv = _f(vel); f, pf = _f(ref); s, ps = _f(sou); w, pw = _f(wavelet); r, pr = _f(rec)
        data = np.zeros((nrec, g.nt), np.float32)
        _chk(lib.oracle_born_f32(C.byref(g), pv, pf, ps, pw, nrec, pr, data.ctypes.data_as(_fp)),
             "born")
    return data


def propagate(desc, vel, sou_coord=None, sou_trace=None, rec_coord=None, rec_trace=None,
              wave=None, image=None, illum=None, ref=None, final_u2=None, rho=None,
              image2=None):
    lib = load()
    _, _, IO, _, _ = _types()
    io = IO()
    keep = []
    v, io.vel = _f(vel); keep.append(v)
    if sou_coord is not None:
        a, io.sou_coord = _f(sou_coord); b, io.sou_trace = _f(sou_trace); keep += [a, b]
        io.nsou = a.size // 3
    if rec_coord is not None:
        a, io.rec_coord = _f(rec_coord); keep.append(a)
        io.nrec = a.size // 3
        io.rec_trace = rec_trace.ctypes.data_as(_fp)
    for name, arr in (("wave", wave), ("image", image), ("illum", illum), ("final_u2", final_u2),
                      ("image2", image2)):
        if arr is not None:
            assert arr.dtype == np.float32 and arr.flags["C_CONTIGUOUS"]
            setattr(io, name, arr.ctypes.data_as(_fp))
    if ref is not None:
        a, io.ref = _f(ref); keep.append(a)
    if rho is not None:
        a, io.rho = _f(rho); keep.append(a)
    _chk(lib.oracle_propagate_f32(C.byref(desc), C.byref(io)), "propagate")


def fwi_fct_gdt(desc, vel, wavelet, shots, vpmask=None):
    lib = load()
    _, _, _, _, FS = _types()
    arr = (FS * len(shots))()
    keep = []
    for i, s in enumerate(shots):
        rc, prc = _f(s["rec"]); dob, pdo = _f(s["dobs"])
        keep += [rc, dob]
        arr[i].sou_coord[:] = [float(v) for v in s["sou"]]
        arr[i].nrec = rc.size // 3
        arr[i].rec_coord, arr[i].dobs = prc, pdo
        if s.get("mute") is not None:
            mu, pmu = _f(s["mute"]); keep.append(mu); arr[i].mute = pmu
        if s.get("resid") is not None:   # float32 (nrec, nt) array filled in place
            arr[i].resid = s["resid"].ctypes.data_as(_fp)
    g = desc.g
    n = g.nz * g.nx * g.ny
    grad, illum = np.zeros(n, np.float32), np.zeros(n, np.float32)
    f = C.c_double()
    v, pv = _f(vel); w, pw = _f(wavelet)
    m, pm = (_f(vpmask) if vpmask is not None else (None, None))
    _chk(lib.oracle_fwi_fct_gdt(C.byref(desc), pv, pw, len(shots), arr, pm, C.byref(f),
                                grad.ctypes.data_as(_fp), illum.ctypes.data_as(_fp)), "fwi")
    return f.value, grad, illum


def fwi_regularize(desc, state, eval_, vel, f, grad, vpmask=None, zweight=None):
    """compute_fct_gdt_reg's terms on the CPU; desc/state are the
    seismic_gb300 SwRegDesc/SwRegState (state updated in place)."""
    lib = load()
    v, pv = _f(vel)
    g = np.array(grad, np.float32, copy=True).ravel()
    m, pm = (_f(vpmask) if vpmask is not None else (None, None))
    zw, pz = (_f(zweight) if zweight is not None else (None, None))
    desc.zweight = pz
    fd = C.c_double(f)
    try:
        _chk(lib.oracle_fwi_regularize(C.byref(desc), C.byref(state), int(eval_), pv, pm,
                                       C.byref(fd), g.ctypes.data_as(_fp)), "fwi_regularize")
    finally:
        desc.zweight = None
    return fd.value, g


def data_norm(ntype, thresh, dobs, dmod, mute=None):
    """Compute_OF_RES_ADJ of one gather: returns (misfit, adjoint source,
    residual) for (nrec, nt) float32 traces."""
    lib = load()
    dobs = np.ascontiguousarray(dobs, np.float32)
    adj = np.array(dmod, np.float32, copy=True, order="C")
    res = np.zeros_like(adj)
    nrec, nt = adj.shape
    mu, pmu = (_f(mute) if mute is not None else (None, None))
    f = C.c_double()
    _chk(lib.oracle_data_norm(int(ntype), float(thresh), nrec, nt, dobs.ctypes.data_as(_fp), pmu,
                              adj.ctypes.data_as(_fp), res.ctypes.data_as(_fp), C.byref(f)),
         "data_norm")
    return f.value, adj, res


def rtm_job(model, vel, wavelet, shots, aperture_x=0.0, aperture_y=0.0):
    """Stacked RTM over shots (dicts as for seismic_gb300.make_shots)."""
    lib = load()
    from seismic_gb300 import make_shots
    arr, keep = make_shots(shots)
    n = model.nz * model.nx * model.ny
    im, il, nm = (np.zeros(n, np.float32) for _ in range(3))
    v, pv = _f(vel); w, pw = _f(wavelet)
    _chk(lib.oracle_rtm_job(C.byref(model), aperture_x, aperture_y, pv, pw, len(shots),
                            C.cast(arr, C.c_void_p), im.ctypes.data_as(_fp),
                            il.ctypes.data_as(_fp), nm.ctypes.data_as(_fp)), "rtm_job")
    return im, il, nm


def set_rigid(on: bool) -> None:
    """Skip the Higdon boundary in every propagation (exact-adjoint mode)."""
    lib = load()
    lib.oracle_set_rigid.argtypes = [C.c_int]
    lib.oracle_set_rigid.restype = None
    lib.oracle_set_rigid(int(bool(on)))


def stencil_f64(g, vel, u2, adjoint=False):
    """Applies the FD stencil once to a padded field u2 (shape padded_shape(g))."""
    lib = load()
    v, pv = _d(vel)
    a, pa = _d(u2)
    out = np.zeros_like(a)
    _chk(lib.oracle_stencil_f64(C.byref(g), int(adjoint), pv, pa, out.ctypes.data_as(_dp)),
         "stencil")
    return out


def stencil_rho_f64(g, vel, rho, u2):
    """Applies the variable-density operator once to a padded field u2."""
    lib = load()
    v, pv = _d(vel)
    r, pr = _d(rho)
    a, pa = _d(u2)
    out = np.zeros_like(a)
    _chk(lib.oracle_stencil_rho_f64(C.byref(g), pv, pr, pa, out.ctypes.data_as(_dp)),
         "stencil_rho")
    return out


def bandpass(traces, dt, flo=0.0, fhi=20.0, nplo=14, nphi=14, phase=0):
    """bandpass of a (ntr, nt) array (returns a filtered float32 copy)."""
    lib = load()
    t = np.ascontiguousarray(traces, np.float32).copy()
    ntr, nt = t.shape
    _chk(lib.oracle_bandpass(t.ctypes.data_as(_fp), ntr, nt, dt, flo, fhi, nplo, nphi, phase),
         "bandpass")
    return t


def mksinc(lsinc: int, shift: float) -> np.ndarray:
    lib = load()
    out = np.zeros(lsinc, np.float32)
    lib.oracle_mksinc(out.ctypes.data_as(_fp), lsinc, shift)
    return out


def triangle2(uu, n1, n2, n3, rect1, rect2, rect3, doz, dox, doy):
    lib = load()
    u = np.ascontiguousarray(uu, np.float32).copy()
    _chk(lib.oracle_triangle2(u.ctypes.data_as(_fp), n1, n2, n3, rect1, rect2, rect3, doz, dox,
                              doy), "triangle2")
    return u


class LBFGS:
    def __init__(self, n, m=5, xmin=1500.0, xmax=4500.0, mask=None, bound_type=2,
                 freeze_soft=True, xinit=None):
        lib = load()
        self.lib = lib
        self.mask = np.ones(n, np.float32) if mask is None else np.ascontiguousarray(mask, np.float32)
        self.xinit = np.zeros(n) if xinit is None else np.ascontiguousarray(xinit, np.float64)
        self.h = lib.oracle_lbfgs_create(n, m, xmin, xmax, self.mask.ctypes.data_as(_fp),
                                         bound_type, int(freeze_soft),
                                         self.xinit.ctypes.data_as(_dp))
        self.iflag = C.c_int(0)
        self.myinfo = C.c_int(0)

    def step(self, x, f, g, eps=1e-20, xtol=np.finfo(float).eps):
        self.myinfo.value = 0
        gg = np.ascontiguousarray(g, np.float64)
        _chk(self.lib.oracle_lbfgs_step(self.h, x.ctypes.data_as(_dp), float(f),
                                        gg.ctypes.data_as(_dp), eps, xtol, C.byref(self.iflag),
                                        C.byref(self.myinfo)), "lbfgs")
        return self.iflag.value, self.myinfo.value

    def diag(self):
        out = np.zeros(8)
        self.lib.oracle_lbfgs_diag(self.h, out.ctypes.data_as(_dp))
        return out

    def __del__(self):
        try:
            self.lib.oracle_lbfgs_destroy(self.h)
        except Exception:
            pass


def mute_mask(nt, dt, sou, rec, ot=0.0, v0=1500.0, v1=10000.0, t0=0.0, t1=40.0, tramp=0.5):
    """MuteParam_compute_mask (Mute.f90:50-95,172-219) of one gather."""
    lib = load()
    s, ps = _f(sou)
    r, pr = _f(rec)
    m = np.zeros((r.size // 3, nt), np.float32)
    _chk(lib.oracle_mute_mask(r.size // 3, nt, C.c_float(dt), C.c_float(ot), ps, pr,
                              C.c_float(v0), C.c_float(v1), C.c_float(t0), C.c_float(t1),
                              C.c_float(tramp), m.ctypes.data_as(_fp)), "mute_mask")
    return m


def freeze_x(x, xmin, xmax, mask, soft, xinit):
    """FREEZE_X (libs/libinv/lbfgs.f:1-40) on an FP64 vector, in place:
    TYPE (soft) clips every entry to [xmin, xmax]; otherwise entries whose
    mask is neither 0 nor 2 are clipped and the others reset to xinit."""
    if soft:
        np.maximum(xmin, x, out=x)
        np.minimum(xmax, x, out=x)
        return x
    m = np.asarray(mask, np.float32).ravel()
    free = (m != 0) & (m != 2)
    x[free] = np.minimum(xmax, np.maximum(xmin, x[free]))
    x[~free] = np.asarray(xinit, np.float64).ravel()[~free]
    return x


def l_bfgs(fctgdt, x, niter, neval, xmin, xmax, vpmask=None, const_type=2, freeze_soft=True,
           vpinit=None, msave=5):
    """l_bfgs (libs/libwave/Inversion.f90:29-189) over the oracle's LBFGS
    (lbfgs.f restated in swave_oracle.cpp).

    fctgdt(x, eval) -> (f: float (FP64), g: float32 array): the objective
    and gradient at the FP32 model x on evaluation `eval` (invparam%eval).
    At evaluation 0 the scalings g0 = max(x) / (100 max|g|) (FP32) and
    f0 = max(x)^2 / |f| (FP64) are fixed and then applied to every
    evaluation (Inversion.f90:118-125: f and g are scaled differently, a
    quirk kept as is); LBFGS receives the scaled f and minus the scaled g
    (gd = -dble(g), :130).  After each completed iteration the saved model
    goes through FREEZE_X when const_type = 2 (:140).  The loop ends after
    niter iterations, neval evaluations or when LBFGS returns iflag <= 0;
    in the last two cases the model of the last completed iteration is
    returned (:177-182).

    Returns (x, history) with history the values the reference writes to
    its 'function' file: f0*f at evaluation 0, then the scaled f of every
    completed iteration; plus the saved models of the iterations.
    """
    x = np.ascontiguousarray(x, np.float32).ravel().copy()
    n = x.size
    mask = np.ones(n, np.float32) if vpmask is None else np.ascontiguousarray(vpmask, np.float32).ravel()
    vpinit = x.astype(np.float64) if vpinit is None else np.ascontiguousarray(vpinit, np.float64).ravel()
    lb = LBFGS(n, msave, float(xmin), float(xmax), mask=mask, bound_type=const_type,
               freeze_soft=freeze_soft, xinit=vpinit)
    xsave = x.astype(np.float64)
    eval_, count, cont, found = 0, 0, True, False
    g0, f0 = np.float32(0), 0.0
    history, models = [], []
    while cont and not found:
        fd, g = fctgdt(x, eval_)
        g = np.asarray(g, np.float32).ravel()
        if eval_ == 0:
            mx = np.float32(x.max())
            g0 = np.float32(mx / (np.float32(100) * np.float32(np.abs(g).max())))
            f0 = float(np.float64(mx * mx)) / abs(fd)
            history.append(np.float32(f0 * fd))
        g = (g0 * g).astype(np.float32)
        fd = f0 * fd
        xd = x.astype(np.float64)
        gd = -g.astype(np.float64)
        xdsave = xd.copy()
        iflag, myinfo = lb.step(xd, fd, gd, eps=1.0e-20, xtol=np.finfo(np.float64).eps)
        x = xd.astype(np.float32)
        if myinfo == 1:
            if const_type == 2:
                freeze_x(xdsave, float(xmin), float(xmax), mask, freeze_soft, vpinit)
            xsave = xdsave
            count += 1
            found = count >= niter
            models.append(xdsave.astype(np.float32))
            history.append(np.float32(fd))
        if iflag <= 0:
            cont = False
        eval_ += 1
        if eval_ >= neval:
            cont = False
    if not cont:
        x = xsave.astype(np.float32)
    return x, np.array(history, np.float32), models


def lbfgs_oc_step(desc, x, f, g, w, diag, state, iflag, myinfo=0):
    """LBFGSOC / LBFGSOLD (nlinv_lbfgs.f:31-613,1066-1636), one call: x, w,
    diag (float64) and state (seismic_gb300.SwLbfgsOcState) updated in
    place; returns (iflag, myinfo)."""
    lib = load()
    fl, mi = C.c_int(iflag), C.c_int(myinfo)
    gg = np.ascontiguousarray(g, np.float64)
    _chk(lib.oracle_lbfgs_oc_step(C.byref(desc), x.ctypes.data_as(_dp), float(f),
                                  gg.ctypes.data_as(_dp), w.ctypes.data_as(_dp),
                                  diag.ctypes.data_as(_dp), C.byref(state), C.byref(fl),
                                  C.byref(mi)), "lbfgs_oc")
    return fl.value, mi.value
