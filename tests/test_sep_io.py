"""SEP dataset and parameter I/O of the command-line programs (cli/sep.c,
through ctypes) and of seismic_gb300.sep, and the programs' argument
checks that stop them before any GPU work."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from seismic_gb300 import sep


@pytest.fixture(scope="module")
def built():
    from seismic_gb300.build import build_cli
    return build_cli()


@pytest.fixture(scope="module")
def lib(built):
    L = C.CDLL(built["libswsep.so"])
    L.sep_init.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    L.sep_open_in.restype = C.c_void_p
    L.sep_open_in.argtypes = [C.c_char_p]
    L.sep_open_out.restype = C.c_void_p
    L.sep_open_out.argtypes = [C.c_char_p]
    for f in ("sep_hdr_int", "sep_hdr_float"):
        getattr(L, f).argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
    L.sep_read.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_size_t]
    L.sep_write.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_size_t]
    L.sep_put_int.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    L.sep_put_float.argtypes = [C.c_void_p, C.c_char_p, C.c_float]
    L.sep_close.argtypes = [C.c_void_p]
    L.sep_error.restype = C.c_char_p
    L.sep_par_str.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t]
    L.sep_par_int.argtypes = [C.c_char_p, C.c_void_p]
    L.sep_par_float.argtypes = [C.c_char_p, C.c_void_p]
    L.sep_par_bool.argtypes = [C.c_char_p, C.c_void_p]
    L.sep_exist.argtypes = [C.c_char_p]
    return L


def _init(lib, *words):
    argv = (C.c_char_p * (len(words) + 1))(b"prog", *[w.encode() for w in words])
    assert lib.sep_init(len(words) + 1, argv) == 0


def _read_all(lib, tag, n):
    f = lib.sep_open_in(tag.encode())
    assert f, lib.sep_error()
    buf = (C.c_float * n)()
    assert lib.sep_read(f, buf, n) == 0, lib.sep_error()
    hdr = {}
    for k in ("n1", "n2", "n3"):
        v = C.c_int(-7)
        hdr[k] = v.value if lib.sep_hdr_int(f, k.encode(), C.byref(v)) == 1 else None
    d1 = C.c_float()
    hdr["d1"] = d1.value if lib.sep_hdr_float(f, b"d1", C.byref(d1)) == 1 else None
    lib.sep_close(f)
    return np.frombuffer(buf, np.float32).copy(), hdr


@pytest.mark.parametrize("fmt", ["xdr_float", "native_float"])
def test_c_reads_python_written(lib, tmp_path, fmt):
    a = np.random.default_rng(0).standard_normal((3, 5, 7)).astype(np.float32)
    p = str(tmp_path / "v.H")
    sep.write(p, a, {"d1": 0.5, "o1": 0.0}, data_format=fmt)
    _init(lib, f"vel={p}")
    got, hdr = _read_all(lib, "vel", a.size)
    np.testing.assert_array_equal(got, a.ravel())
    assert (hdr["n1"], hdr["n2"], hdr["n3"], hdr["d1"]) == (7, 5, 3, 0.5)


def test_c_reads_samples_embedded_after_the_header(lib, tmp_path):
    """in=stdin (or no in=): samples follow the 0x0c 0x04 marker."""
    a = np.arange(10, dtype=np.float32)
    p = tmp_path / "w.H"
    p.write_bytes(b"prog:\n\tn1=10 d1=0.002\n\tdata_format=native_float in=stdin\n\x0c\x04" +
                  a.astype("<f4").tobytes())
    _init(lib, f"stdin={p}")
    got, hdr = _read_all(lib, "in", 10)
    np.testing.assert_array_equal(got, a)
    assert hdr["n1"] == 10 and abs(hdr["d1"] - 0.002) < 1e-9
    np.testing.assert_array_equal(sep.read(str(p))[0], a)


def test_python_reads_c_written(lib, tmp_path):
    p = str(tmp_path / "out.H")
    _init(lib, f"data={p}")
    f = lib.sep_open_out(b"data")
    assert f, lib.sep_error()
    a = np.random.default_rng(1).standard_normal((4, 9)).astype(np.float32)
    buf = (C.c_float * a.size)(*a.ravel())
    assert lib.sep_write(f, buf, a.size) == 0
    lib.sep_put_int(f, b"n1", 9)
    lib.sep_put_int(f, b"n2", 4)
    lib.sep_put_float(f, b"d1", 0.004)
    assert lib.sep_close(f) == 0
    got, h = sep.read(p)
    np.testing.assert_array_equal(got, a)
    assert h["data_format"] == "xdr_float" and float(h["d1"]) == pytest.approx(0.004)
    assert open(p + "@", "rb").read(4) == a.astype(">f4").tobytes()[:4]


def test_datapath_places_the_samples(lib, tmp_path):
    d = tmp_path / "dp"
    d.mkdir()
    p = str(tmp_path / "o.H")
    _init(lib, f"data={p}", f"datapath={d}/")
    f = lib.sep_open_out(b"data")
    buf = (C.c_float * 2)(1.0, 2.0)
    lib.sep_write(f, buf, 2)
    lib.sep_put_int(f, b"n1", 2)
    lib.sep_close(f)
    assert os.path.exists(d / "o.H@")
    np.testing.assert_array_equal(sep.read(p)[0], [1.0, 2.0])


def test_parameters_last_wins_par_files_and_logicals(lib, tmp_path):
    par = tmp_path / "p.par"
    par.write_text("fmax=20 ntaper=11\nTask='MIG' twoD=.true.\n")
    _init(lib, "fmax=30", f"par={par}", "fmax=16", "withRho=n", 'keygx="4"')
    v = C.c_float()
    assert lib.sep_par_float(b"fmax", C.byref(v)) == 1 and v.value == 16.0
    i = C.c_int()
    assert lib.sep_par_int(b"ntaper", C.byref(i)) == 1 and i.value == 11
    assert lib.sep_par_int(b"keygx", C.byref(i)) == 1 and i.value == 4
    assert lib.sep_par_bool(b"twoD", C.byref(i)) == 1 and i.value == 1
    assert lib.sep_par_bool(b"withRho", C.byref(i)) == 1 and i.value == 0
    assert lib.sep_par_int(b"missing", C.byref(i)) == 0
    assert lib.sep_par_bool(b"fmax", C.byref(i)) == -1
    s = C.create_string_buffer(16)
    assert lib.sep_par_str(b"Task", s, 16) == 1 and s.value == b"MIG"
    assert lib.sep_exist(b"keygx") == 1 and lib.sep_exist(b"vel") == 0


def _write_shot(tmp_path, nt=50, ntr=6, nz=30, nx=40, traces_nt=None):
    w = np.zeros(nt, np.float32)
    w[3] = 1.0
    sep.write(str(tmp_path / "w.H"), w, {"d1": 0.001, "o1": 0.0})
    sep.write(str(tmp_path / "t.H"), np.zeros((ntr, traces_nt or nt), np.float32), {"d1": 0.001})
    keys = np.zeros((ntr, 6), np.float32)
    keys[:, 0] = 195.0                                # sx
    keys[:, 1] = np.linspace(50, 350, ntr)            # gx
    keys[:, 4] = 10.0                                 # selev
    keys[:, 5] = 12.0                                 # gelev
    sep.write(str(tmp_path / "k.H"), keys)
    sep.write(str(tmp_path / "v.H"), np.full((nx, nz), 2000.0, np.float32),
              {"d1": 10.0, "d2": 10.0, "o1": 0.0, "o2": 0.0})
    return dict(stdin=tmp_path / "w.H", traces=tmp_path / "t.H", coordfile=tmp_path / "k.H",
                vel=tmp_path / "v.H", keysx=1, keygx=2, keysy=3, keygy=4, keyselev=5,
                keygelev=6, twoD=1, data=tmp_path / "d.H")


def _run(built, exe, **params):
    r = subprocess.run(sep.command(built[exe], **params), capture_output=True, text=True,
                       timeout=60)
    return r.returncode, r.stderr


@pytest.mark.parametrize("drop,msg", [("traces", "need traces file"),
                                      ("coordfile", "need coordfile"),
                                      ("keygx", "need keygx"),
                                      ("vel", "need vel file")])
def test_modeling_program_rejects_missing_inputs(built, tmp_path, drop, msg):
    p = _write_shot(tmp_path)
    p.pop(drop)
    rc, err = _run(built, "Acoustic_modeling_sep.x", **p)
    assert rc == 1 and msg in err, err


def test_programs_reject_inconsistent_or_unbuilt_options(built, tmp_path):
    p = _write_shot(tmp_path, traces_nt=40)
    rc, err = _run(built, "Acoustic_modeling_sep.x", **p)
    assert rc == 1 and "nt traces and sources are different" in err
    p = _write_shot(tmp_path)
    rc, err = _run(built, "3DRTM.x", **p, withRho=1, image=tmp_path / "i.H")
    assert rc == 1 and "need rho file" in err
    rc, err = _run(built, "3DRTM.x", **p, withRho=1, LSRTM=1, image=tmp_path / "i.H")
    assert rc == 1 and "withRho=1 with LSRTM=1" in err
    rc, err = _run(built, "3DBORNMOD.x", **p)
    assert rc == 1 and "need reflectivity file" in err
    far = dict(p, aperture_x=100)                     # every key 5000 m: off the model
    sep.write(str(tmp_path / "k2.H"), np.full((6, 6), 5000.0, np.float32))
    far["coordfile"] = tmp_path / "k2.H"
    rc, err = _run(built, "Acoustic_modeling_sep.x", **far)
    assert rc == 1 and "outside velocity model" in err, err


def test_afwi_program_rejects_inv_and_trace_count(built, tmp_path):
    p = _write_shot(tmp_path)
    p.pop("data")
    rc, err = _run(built, "2DAFWI.x", **p, Task="FOO")
    assert rc == 1 and "expected MOD, MIG or INV" in err
    sep.write(str(tmp_path / "t3.H"), np.zeros((3, 50), np.float32), {"d1": 0.001})
    rc, err = _run(built, "2DAFWI.x", **dict(p, traces=tmp_path / "t3.H"), Task="MIG",
                   image=tmp_path / "i.H")
    assert rc == 1 and "different from n2" in err, err
