"""Seeded golden cases: the inputs, and how to run one through either the
oracle's bindings or a libswave context (both take the same arguments).

The fixtures hold the inputs as well as the outputs, so a check never
depends on how the inputs were generated (NumPy's RNG or exp/sin may change
between versions and machines).
"""
from __future__ import annotations

import json

import numpy as np

import seismic_gb300 as sw
from seismic_gb300 import synth

GENPAR_FIELDS = [f for f, _ in sw.SwGenpar._fields_]
FWI_FIELDS = [f for f, _ in sw.SwFwiDesc._fields_ if f != "g"]


def _genpar_json(g) -> str:
    return json.dumps({f: getattr(g, f) for f in GENPAR_FIELDS})


def genpar_from(js: str):
    g = sw.SwGenpar()
    for k, v in json.loads(js).items():
        setattr(g, k, v)
    return g


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _model(nz, nx, ny, d, seed):
    rng = np.random.default_rng(seed)
    z = np.arange(nz)[None, None, :] * d
    x = np.arange(nx)[None, :, None] * d
    y = np.arange(ny)[:, None, None] * d
    v = (1750.0 + 1.1 * z + 120.0 * np.sin(x / 160.0) * np.cos(y / 140.0)
         + 35 * rng.standard_normal((ny, nx, nz)))
    return _f32(v[0] if ny == 1 else v)


def make_inputs() -> dict[str, dict]:
    """name -> input arrays (with "genpar" as JSON, "kind" as the operator)."""
    out = {}
    d, dt = 10.0, 1.5e-3
    # 2D: modeling (traces + final wavefield), RTM, Born + LSRTM.
    g2 = sw.make_genpar(44, 60, 1, dz=d, dx=d, dt=dt, nt=260, ntaper=10, lsinc=7, snapi=4)
    vel2 = _model(44, 60, 1, d, 1)
    sou2 = _f32([20.3, 291.7, 0.0])
    rec2 = np.zeros((30, 3), np.float32)
    rec2[:, 0] = d + 2.3
    rec2[:, 1] = np.linspace(3.0, 587.0, 30)
    w2 = _f32(synth.ricker(12.0, dt, g2.nt))
    base2 = {"genpar": _genpar_json(g2), "vel": vel2, "sou": sou2, "rec": rec2, "wavelet": w2}
    out["modeling2d"] = dict(base2, kind="modeling")
    rng = np.random.default_rng(21)
    out["rtm2d"] = dict(base2, kind="rtm",
                        data=_f32(rng.standard_normal((30, g2.nt)) * 1e-2))
    refl = _f32(rng.standard_normal(vel2.shape) * (rng.random(vel2.shape) < 0.05))
    out["born2d"] = dict(base2, kind="born", ref=refl,
                         wavelet=_f32(sw.born_wavelet(w2, g2.dt)))
    out["lsrtm2d"] = dict(base2, kind="lsrtm", wavelet=_f32(sw.born_wavelet(w2, g2.dt)),
                          data=_f32(rng.standard_normal((30, g2.nt)) * 1e-2))
    # 3D: modeling and RTM.
    g3 = sw.make_genpar(24, 28, 20, dz=d, dx=d, dy=d, dt=dt, nt=90, ntaper=8, lsinc=7,
                        snapi=3, twoD=False)
    vel3 = _model(24, 28, 20, d, 2)
    rx, ry = np.meshgrid(np.arange(2, 26, 3) * d, np.arange(2, 18, 4) * d, indexing="ij")
    rec3 = np.zeros((rx.size, 3), np.float32)
    rec3[:, 0] = d + 1.1
    rec3[:, 1] = rx.ravel()
    rec3[:, 2] = ry.ravel()
    base3 = {"genpar": _genpar_json(g3), "vel": vel3, "sou": _f32([30.4, 142.0, 98.5]),
             "rec": rec3, "wavelet": _f32(synth.ricker(12.0, dt, g3.nt))}
    out["modeling3d"] = dict(base3, kind="modeling")
    out["rtm3d"] = dict(base3, kind="rtm",
                        data=_f32(rng.standard_normal((rec3.shape[0], g3.nt)) * 1e-2))
    # 2D FWI objective and gradient over two shots with trace mutes.
    g4 = sw.make_genpar(40, 72, 1, dz=d, dx=d, dt=dt, nt=220, ntaper=10, lsinc=7, snapi=4)
    fwi = {"genpar": _genpar_json(g4), "kind": "fwi", "vel": _model(40, 72, 1, d, 3),
           "wavelet": _f32(synth.ricker(12.0, dt, g4.nt)),
           "desc": json.dumps({"aperture_x": 60.0, "aperture_y": 0.0, "illu_pow": 1.0,
                               "smooth_rect1": 3, "smooth_rect2": 4, "smooth_rect3": 1,
                               "smooth_doz": 1, "smooth_dox": 1, "smooth_doy": 0,
                               "checkpoint_snaps": 0}),
           "vpmask": _f32(np.r_[np.zeros(40 * 3), np.ones(40 * 69)])}
    for i, sx in enumerate((205.0, 455.0)):
        rec = np.zeros((34, 3), np.float32)
        rec[:, 0] = d + 2.0
        rec[:, 1] = np.linspace(20.0, 690.0, 34)
        fwi[f"shot{i}_sou"] = _f32([21.0, sx, 0.0])
        fwi[f"shot{i}_rec"] = rec
        fwi[f"shot{i}_dobs"] = _f32(rng.standard_normal((34, g4.nt)) * 1e-2)
        fwi[f"shot{i}_mute"] = _f32(rng.random((34, g4.nt)) > 0.1)
    out["fwi2d"] = fwi
    # Variable density (withRho): 2D modelling and the rho-v AFWI imaging
    # condition, 3D modelling (below).
    g5 = sw.make_genpar(52, 70, 1, dz=d, dx=d, dt=dt, nt=200, ntaper=10, lsinc=7, snapi=4)
    vel5 = _model(52, 70, 1, d, 4)
    rho5 = _f32(1.8 + 0.0008 * np.arange(52)[None, :] * d + 0.15 * rng.random(vel5.shape))
    rec5 = np.zeros((35, 3), np.float32)
    rec5[:, 0] = d + 2.3
    rec5[:, 1] = np.linspace(4.0, 686.0, 35)
    base5 = {"genpar": _genpar_json(g5), "vel": vel5, "rho": rho5, "sou": _f32([24.1, 333.3, 0.0]),
             "rec": rec5, "wavelet": _f32(sw.rho_wavelet(synth.ricker(12.0, dt, g5.nt), 7))}
    out["rho_modeling2d"] = dict(base5, kind="rho_modeling")
    out["rho_afwi2d"] = dict(base5, kind="rho_afwi",
                             data=_f32(rng.standard_normal((35, g5.nt)) * 1e-2))
    # A free surface between grid rows (sinc mirror) with a mirror source.
    g6 = sw.make_genpar(44, 60, 1, dz=d, dx=d, dt=dt, nt=260, ntaper=10, lsinc=7, snapi=4)
    g6.surf_type, g6.shot_type, g6.rec_type, g6.oz = 1, 1, 0, -4.0
    rec6 = rec2.copy()
    rec6[:, 0] = 20.7
    out["surface_modeling2d"] = dict(base2, kind="surface_modeling", genpar=_genpar_json(g6),
                                     sou=_f32([20.4, 291.7, 0.0]), rec=rec6)
    rho3 = _f32(1.8 + 0.15 * rng.random(vel3.shape))
    out["rho_modeling3d"] = dict(base3, kind="rho_modeling", rho=rho3,
                                 wavelet=_f32(sw.rho_wavelet(base3["wavelet"], 7)))
    # The AFWI imaging condition (second time difference of the snapshots).
    out["afwi2d"] = dict(base2, kind="afwi",
                         data=_f32(rng.standard_normal((30, g2.nt)) * 1e-2))
    # Born and LSRTM in 3D.
    refl3 = _f32(rng.standard_normal(vel3.shape) * (rng.random(vel3.shape) < 0.05))
    wb3 = _f32(sw.born_wavelet(base3["wavelet"], g3.dt))
    out["born3d"] = dict(base3, kind="born", ref=refl3, wavelet=wb3)
    out["lsrtm3d"] = dict(base3, kind="lsrtm", wavelet=wb3,
                          data=_f32(rng.standard_normal((rec3.shape[0], g3.nt)) * 1e-2))
    return out


def _prop_desc(g, forward: bool, **kw):
    d = sw.SwPropDesc()
    d.g = g
    d.tmin, d.tmax, d.tstep = (1, g.nt, 1) if forward else (g.nt, 1, -1)
    d.fd_scheme = sw.FD_FORWARD
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def run(api, inp: dict) -> dict[str, np.ndarray]:
    """Run one case through `api` (the oracle bindings or a Context)."""
    kind = str(inp["kind"])
    g = genpar_from(str(inp["genpar"]))
    vel, w = inp["vel"], inp["wavelet"]
    if kind == "modeling":
        if not g.twoD:   # the 3D final wavefield would dominate the fixture size
            return {"out_data": api.modeling(g, vel, inp["sou"], w, inp["rec"])}
        data, fu = api.modeling(g, vel, inp["sou"], w, inp["rec"], final_u2=True)
        return {"out_data": data, "out_final_u2": fu}
    if kind == "rtm":
        im, il = api.rtm(g, vel, inp["sou"], w, inp["rec"], inp["data"])
        return {"out_image": im, "out_illum": il}
    if kind == "born":
        return {"out_data": api.born(g, vel, inp["ref"], inp["sou"], w, inp["rec"])}
    if kind == "lsrtm":
        im, il = api.lsrtm(g, vel, inp["sou"], w, inp["rec"], inp["data"])
        return {"out_image": im, "out_illum": il}
    if kind == "fwi":
        desc = sw.SwFwiDesc()
        desc.g = g
        for k, v in json.loads(str(inp["desc"])).items():
            setattr(desc, k, v)
        shots = [{"sou": inp[f"shot{i}_sou"], "rec": inp[f"shot{i}_rec"],
                  "dobs": inp[f"shot{i}_dobs"], "mute": inp[f"shot{i}_mute"]}
                 for i in range(2)]
        f, grad, illum = api.fwi_fct_gdt(desc, vel, w, shots, vpmask=inp["vpmask"])
        return {"out_misfit": np.array([f], np.float64), "out_gradient": grad,
                "out_illum": illum}
    if kind in ("rho_modeling", "surface_modeling"):
        data = np.zeros((inp["rec"].shape[0], g.nt), np.float32)
        api.propagate(_prop_desc(g, True, injection=sw.INJ_SINC, extraction=sw.EXT_SINC), vel,
                      inp["sou"], w, inp["rec"], data, rho=inp.get("rho"))
        return {"out_data": data}
    if kind == "afwi":
        n = vel.size
        wave = np.zeros((g.nt // g.snapi) * n, np.float32)
        api.propagate(_prop_desc(g, True, injection=sw.INJ_SINC, extract_wave=1), vel,
                      inp["sou"], w, wave=wave)
        im, il = np.zeros(n, np.float32), np.zeros(n, np.float32)
        api.propagate(_prop_desc(g, False, injection=sw.INJ_SINC, imaging=sw.IMG_AFWI), vel,
                      inp["rec"], np.array(inp["data"]), wave=wave, image=im, illum=il)
        return {"out_image": im, "out_illum": il}
    if kind == "rho_afwi":
        n = vel.size
        wave = np.zeros((g.nt // g.snapi) * n, np.float32)
        api.propagate(_prop_desc(g, True, injection=sw.INJ_SINC, extract_wave=1), vel,
                      inp["sou"], w, wave=wave, rho=inp["rho"])
        im, im2, il = (np.zeros(n, np.float32) for _ in range(3))
        api.propagate(_prop_desc(g, False, injection=sw.INJ_SINC, imaging=sw.IMG_AFWI_RHO), vel,
                      inp["rec"], np.array(inp["data"]), wave=wave, image=im, illum=il,
                      rho=inp["rho"], image2=im2)
        return {"out_image": im, "out_image2": im2, "out_illum": il}
    raise ValueError(kind)
