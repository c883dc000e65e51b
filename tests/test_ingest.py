"""Catalogue ingest of the host program (CPU): the ASCII reader's semantics
(io/read_ascii.c:533-1142: header lines, comments, blank lines, formatter,
expressions, selection, total weight in file order) are the same for every
number of host threads; numbers convert exactly as strtod; NumPy .npy
catalogues give the same records as the ASCII file of the same values."""
import ctypes
import math
import os
import random
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HOST = os.path.join(ROOT, "powspec_gb300", "host")


class Cat(ctypes.Structure):
    _fields_ = [("fname", ctypes.c_char_p), ("skip", ctypes.c_long), ("comment", ctypes.c_char),
                ("fmtr", ctypes.c_char_p), ("pos", ctypes.c_char_p * 3),
                ("wcomp", ctypes.c_char_p), ("sel", ctypes.c_char_p), ("nthread", ctypes.c_int),
                ("survey", ctypes.c_int), ("wfkp", ctypes.c_char_p), ("nz", ctypes.c_char_p),
                ("sumw2", ctypes.POINTER(ctypes.c_double)), ("sumw2n", ctypes.POINTER(ctypes.c_double))]


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("host") / "libpshost.so")
    srcs = [os.path.join(HOST, f) for f in ("ps_read.c", "ps_expr.c")]
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-shared", "-fPIC", "-pthread", "-I" + HOST,
                    "-o", out] + srcs + ["-lm"], check=True)
    lib = ctypes.CDLL(out)
    for name in ("psh_read_ascii", "psh_read_npy"):
        f = getattr(lib, name)
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(Cat), ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                      ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_double),
                      ctypes.c_bool]
    lib.psh_strtod.restype = ctypes.c_double
    lib.psh_strtod.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
    return lib


LIBC = ctypes.CDLL(None)
LIBC.strtod.restype = ctypes.c_double
LIBC.strtod.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
LIBC.free.argtypes = [ctypes.c_void_p]


def read(host, path, fmtr="%lf %lf %lf", pos=("$1", "$2", "$3"), wcomp=None, sel=None, skip=0,
         comment=b"#", nthread=1, npy=False):
    c = Cat(str(path).encode(), skip, comment, fmtr.encode() if fmtr else None,
            (ctypes.c_char_p * 3)(*[p.encode() for p in pos]),
            wcomp.encode() if wcomp else None, sel.encode() if sel else None, nthread)
    ptr = ctypes.POINTER(ctypes.c_double)()
    n = ctypes.c_size_t()
    w = ctypes.c_double()
    rc = (host.psh_read_npy if npy else host.psh_read_ascii)(ctypes.byref(c), ctypes.byref(ptr),
                                                            ctypes.byref(n), ctypes.byref(w), False)
    if rc:
        return rc, None, None
    a = np.ctypeslib.as_array(ptr, (n.value, 4)).copy() if n.value else np.zeros((0, 4))
    LIBC.free(ptr)
    return 0, a, w.value


def _strings(rng):
    out = ["0", "-0", "+0.0", "-0.000", "1", "1.", ".5", "-.5", "1e5", "1E-5", "1e", "1e+",
           "1.e3", "00012.50", "0.000000000000000000000123", "123456789012345678901234",
           "9007199254740993", "9007199254740992", "1e22", "1e23", "4.9e-324", "1e-400",
           "1.7976931348623157e308", "1e309", "inf", "-Infinity", "nan", "0x1p3", "-0X1.8p1",
           "1.5x", "3.14159 rest", "2e-22", "1234567890123456789e-22", "12345678901234567890",
           "0.1", "0.2", "0.3", "7e-10", "1e0000000000000000005", "1e+0000000000000000000000400"]
    for _ in range(20000):
        k = rng.randrange(6)
        v = rng.uniform(-1, 1) * 10 ** rng.uniform(-30, 30)
        if k == 0:
            s = "%.*f" % (rng.randrange(0, 12), v)
        elif k == 1:
            s = "%.*e" % (rng.randrange(0, 18), v)
        elif k == 2:
            s = "%.*g" % (rng.randrange(1, 18), v)
        elif k == 3:
            s = repr(v)
        elif k == 4:
            s = str(rng.randrange(-10 ** rng.randrange(1, 21), 10 ** rng.randrange(1, 21)))
        else:
            s = "%.*f" % (rng.randrange(0, 7), rng.uniform(0, 2000))
        out.append(s)
    return out


def test_number_conversion_equals_strtod(host):
    rng = random.Random(5)
    for s in _strings(rng):
        b = s.encode()
        e1, e2 = ctypes.c_char_p(), ctypes.c_char_p()
        buf = ctypes.create_string_buffer(b)
        v1 = host.psh_strtod(ctypes.cast(buf, ctypes.c_char_p), ctypes.byref(e1))
        v2 = LIBC.strtod(ctypes.cast(buf, ctypes.c_char_p), ctypes.byref(e2))
        used1 = ctypes.cast(e1, ctypes.c_void_p).value - ctypes.addressof(buf)
        used2 = ctypes.cast(e2, ctypes.c_void_p).value - ctypes.addressof(buf)
        assert used1 == used2, s
        if math.isnan(v2):
            assert math.isnan(v1), s
        else:
            assert np.float64(v1).tobytes() == np.float64(v2).tobytes(), s


def _catalogue(rng, n):
    """Lines with a leading-blank / CRLF / comment / blank-line mix, a string
    column and four numbers; returns the text and the records it holds."""
    lines, recs = ["header one", "header two # not a comment here"], []
    for i in range(n):
        x, y, z = (rng.uniform(0, 1000) for _ in range(3))
        w = rng.uniform(0.1, 3)
        sx, sy, sz = ("%.*f" % (rng.randrange(2, 10), v) for v in (x, y, z))
        sw = "%.6g" % w
        lead = rng.choice(["", " ", "\t", "   "])
        end = rng.choice(["", " ", "\r"])
        lines.append("%s%s id%d %s %s %s%s" % (lead, sx, i, sy, sz, sw, end))
        recs.append((float(sx), float(sy), float(sz), float(sw)))
        r = rng.random()
        if r < 0.02:
            lines.append("# comment %d" % i)
        elif r < 0.04:
            lines.append(rng.choice(["", "   ", "\t", "\r"]))
        elif r < 0.05:
            lines.append("  # indented comment")
    return "\n".join(lines), np.array(recs)


@pytest.mark.parametrize("trailing", ["", "\n"])
def test_ascii_same_records_for_every_thread_count(host, tmp_path, trailing):
    rng = random.Random(11)
    text, recs = _catalogue(rng, 30000)
    p = tmp_path / "cat.txt"
    p.write_text(text + trailing)
    sel = "$4 < 2.5 && $1 >= 10"
    keep = (recs[:, 3] < 2.5) & (recs[:, 0] >= 10)
    expect = np.column_stack([recs[keep, 0], recs[keep, 1] * 2, recs[keep, 2], recs[keep, 3]])
    base = None
    for nt in (1, 2, 3, 7, 16, 61):
        rc, a, w = read(host, p, fmtr="%lf %*s %lf %lf %lf", pos=("$1", "$2*2", "$3"),
                        wcomp="$4", sel=sel, skip=2, nthread=nt)
        assert rc == 0
        if base is None:
            base = (a, w)
            assert np.array_equal(a, expect)
            wsum = 0.0
            for v in expect[:, 3]:
                wsum += v  # file order
            assert w == wsum
        else:
            assert np.array_equal(a, base[0]) and w == base[1], nt


def test_ascii_skip_and_width_and_literals(host, tmp_path):
    p = tmp_path / "w.txt"
    # skip counts lines of any kind; a width limits a field; literals match
    p.write_text("1 2 3\n\n# c\n(1.5,2.5,3.5) 123456\n  (4,5,6) 987654\n(7,8,9) 1")
    for nt in (1, 2, 5):
        rc, a, w = read(host, p, fmtr="(%lf,%lf,%lf) %3lf", wcomp="$4", skip=1, nthread=nt)
        assert rc == 0
        assert a.tolist() == [[1.5, 2.5, 3.5, 123.0], [4, 5, 6, 987.0], [7, 8, 9, 1.0]]
        assert w == 123.0 + 987.0 + 1.0
    # every line skipped
    rc, a, w = read(host, p, fmtr="(%lf,%lf,%lf)", skip=100, nthread=3)
    assert rc == 0 and a.shape == (0, 4) and w == 0


@pytest.mark.parametrize("nthread", [1, 2, 4, 9])
def test_ascii_error_names_the_first_bad_line(host, tmp_path, capfd, nthread):
    lines = ["%d %d %d" % (i, i, i) for i in range(5000)]
    lines[1234] = "1 2 x"
    lines[4321] = "oops"
    p = tmp_path / "bad.txt"
    p.write_text("\n".join(lines) + "\n")
    rc, _, _ = read(host, p, nthread=nthread)
    assert rc == -6
    err = capfd.readouterr().err
    assert "line 1235 of" in err and "(field 5)" in err
    assert "1 2 x\n    ^" in err


def test_ascii_empty_file_and_missing_file(host, tmp_path, capfd):
    p = tmp_path / "empty.txt"
    p.write_text("")
    assert read(host, p, nthread=4)[0] == 0
    assert read(host, tmp_path / "nope.txt")[0] == -3
    assert "cannot open" in capfd.readouterr().err


@pytest.mark.parametrize("dtype", ["<f8", ">f8", "<f4", "<i4", ">i8"])
@pytest.mark.parametrize("order", ["C", "F"])
def test_npy_records_equal_ascii_records(host, tmp_path, dtype, order):
    rng = np.random.default_rng(3)
    n = 20000
    v = rng.random((n, 5)) * 1000
    if dtype[1] == "i":
        v = np.floor(v)
    arr = np.asarray(v.astype(dtype), order=order)
    p = tmp_path / "cat.npy"
    np.save(p, arr)
    txt = tmp_path / "cat.txt"
    np.savetxt(txt, arr.astype(np.float64), fmt="%.17g")
    kw = dict(pos=("$2", "$3+1", "$1"), wcomp="$5/100", sel="$4 > 100")
    rc, a, w = read(host, p, fmtr=None, npy=True, nthread=6, **kw)
    assert rc == 0
    rc2, b, w2 = read(host, txt, fmtr="%lf %lf %lf %lf %lf", nthread=3, **kw)
    assert rc2 == 0
    assert np.array_equal(a, b) and w == w2
    f = arr.astype(np.float64)
    keep = f[:, 3] > 100
    assert np.array_equal(a[:, 0], f[keep, 1]) and np.array_equal(a[:, 3], f[keep, 4] / 100)


def test_npy_one_column_and_errors(host, tmp_path, capfd):
    p = tmp_path / "one.npy"
    np.save(p, np.arange(10.0))
    rc, a, w = read(host, p, fmtr=None, pos=("$1", "$1", "$1"), npy=True)
    assert rc == 0 and a[:, 0].tolist() == list(np.arange(10.0)) and w == 10
    rc, _, _ = read(host, p, fmtr=None, pos=("$1", "$2", "$1"), npy=True)
    assert rc == -5 and "column 2" in capfd.readouterr().err
    np.save(tmp_path / "h.npy", np.zeros((4, 3), np.float16))
    assert read(host, tmp_path / "h.npy", fmtr=None, npy=True)[0] == -3
    assert "dtype" in capfd.readouterr().err
    raw = (tmp_path / "one.npy").read_bytes()
    (tmp_path / "short.npy").write_bytes(raw[:-8])
    assert read(host, tmp_path / "short.npy", fmtr=None, pos=("$1", "$1", "$1"), npy=True)[0] == -3
    assert "shorter" in capfd.readouterr().err
    (tmp_path / "t.npy").write_text("1 2 3\n")
    assert read(host, tmp_path / "t.npy", fmtr=None, npy=True)[0] == -3


@pytest.mark.parametrize("nthread", [1, 5])
def test_survey_weights_and_sums(host, tmp_path, nthread):
    """Survey catalogues (io/read_ascii.c:880-895): record weight wc * wfkp;
    W = sum wc, sum (wc wfkp)^2 and sum wc wfkp^2 nz, in file order."""
    rng = np.random.default_rng(9)
    n = 20000
    v = np.column_stack([rng.random((n, 3)) * 500, rng.uniform(0.5, 1.5, n),
                         rng.uniform(1e-4, 3e-4, n)])
    p = tmp_path / "s.txt"
    np.savetxt(p, v, fmt="%.10g")
    w2, w2n = ctypes.c_double(), ctypes.c_double()
    c = Cat(str(p).encode(), 0, b"#", b"%lf %lf %lf %lf %lf",
            (ctypes.c_char_p * 3)(b"$1", b"$2", b"$3"), b"$4", b"$5 > 1.2e-4", nthread,
            1, b"1/(1+$5*10000)", b"$5", ctypes.pointer(w2), ctypes.pointer(w2n))
    ptr = ctypes.POINTER(ctypes.c_double)()
    cnt = ctypes.c_size_t()
    w = ctypes.c_double()
    assert host.psh_read_ascii(ctypes.byref(c), ctypes.byref(ptr), ctypes.byref(cnt),
                               ctypes.byref(w), False) == 0
    a = np.ctypeslib.as_array(ptr, (cnt.value, 4)).copy()
    LIBC.free(ptr)
    f = np.loadtxt(p)
    f = f[f[:, 4] > 1.2e-4]
    wc, wf, nz = f[:, 3], 1 / (1 + f[:, 4] * 10000), f[:, 4]
    assert np.array_equal(a[:, :3], f[:, :3])
    assert np.allclose(a[:, 3], wc * wf, rtol=1e-15, atol=0)
    s = s2 = s2n = 0.0
    for x, y, z in zip(wc, wf, nz):  # file order
        s += x
        s2 += (x * y) ** 2
        s2n += x * y * y * z
    assert w.value == pytest.approx(s, rel=1e-14)
    assert w2.value == pytest.approx(s2, rel=1e-13) and w2n.value == pytest.approx(s2n, rel=1e-13)


class Cosmo(ctypes.Structure):
    _fields_ = [("omega_m", ctypes.c_double), ("omega_l", ctypes.c_double),
                ("omega_k", ctypes.c_double), ("eos_w", ctypes.c_double), ("err", ctypes.c_double),
                ("widx", ctypes.c_double), ("order", ctypes.c_int),
                ("x", ctypes.c_double * 32), ("w", ctypes.c_double * 32),
                ("tz", ctypes.POINTER(ctypes.c_double)), ("td", ctypes.POINTER(ctypes.c_double)),
                ("typp", ctypes.POINTER(ctypes.c_double)), ("ntab", ctypes.c_size_t)]


@pytest.fixture(scope="module")
def cnvt(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cnvt") / "libpscnvt.so")
    srcs = [os.path.join(HOST, f) for f in ("ps_cnvt.c", "ps_read.c", "ps_expr.c")]
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-shared", "-fPIC", "-pthread", "-I" + HOST,
                    "-o", out] + srcs + ["-lm"], check=True)
    lib = ctypes.CDLL(out)
    lib.psh_cosmo_init.argtypes = [ctypes.POINTER(Cosmo), ctypes.c_char_p, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_bool]
    lib.psh_cosmo_distance.restype = ctypes.c_double
    lib.psh_cosmo_distance.argtypes = [ctypes.POINTER(Cosmo), ctypes.c_double]
    lib.psh_cosmo_convert.argtypes = [ctypes.POINTER(Cosmo), ctypes.c_void_p, ctypes.c_size_t,
                                      ctypes.c_int]
    lib.psh_cosmo_free.argtypes = [ctypes.POINTER(Cosmo)]
    return lib


@pytest.mark.parametrize("om,ol,w", [(0.31, 0.69, -1.0), (0.3, 0.6, -0.9)])
def test_comoving_distance_quadrature(cnvt, om, ol, w):
    """Gauss-Legendre quadrature of c/(100 km/s) / E(z) at the order that
    converges to CMVDST_ERR on the redshift range (src/cnvt_coord.c:295-400),
    against adaptive quadrature; then (RA, Dec, z) -> Cartesian."""
    integrate = pytest.importorskip("scipy.integrate")
    c = Cosmo(om, ol, 1 - om - ol, w, 1e-8, 0.0, 0)
    assert cnvt.psh_cosmo_init(ctypes.byref(c), None, 0.0, 2.0, False) == 0
    assert 4 <= c.order <= 32
    wi = 3 * (1 + w)

    def e(z):
        z1 = 1 + z
        return np.sqrt(om * z1 ** 3 + (1 - om - ol) * z1 ** 2 + ol * z1 ** wi)

    for z in (0.0, 0.1, 0.57, 1.3, 2.0):
        ref = integrate.quad(lambda t: 2997.92458 / e(t), 0, z, epsabs=0, epsrel=1e-13)[0]
        assert cnvt.psh_cosmo_distance(ctypes.byref(c), z) == pytest.approx(ref, rel=1e-9, abs=1e-12)
    rng = np.random.default_rng(2)
    rec = np.column_stack([rng.uniform(0, 360, 5000), rng.uniform(-90, 90, 5000),
                           rng.uniform(0, 2, 5000), np.ones(5000)])
    out = rec.copy()
    cnvt.psh_cosmo_convert(ctypes.byref(c), out.ctypes.data, len(out), 3)
    d = np.array([cnvt.psh_cosmo_distance(ctypes.byref(c), z) for z in rec[:, 2]])
    ra, dec = np.radians(rec[:, 0]), np.radians(rec[:, 1])
    assert np.allclose(out[:, 0], d * np.cos(dec) * np.cos(ra), rtol=1e-13, atol=1e-9)
    assert np.allclose(out[:, 2], d * np.sin(dec), rtol=1e-13, atol=1e-9)


def test_comoving_distance_table_spline(cnvt, tmp_path):
    """Z_CMVDST_CNVT: a natural cubic spline through the (z, D) samples."""
    interpolate = pytest.importorskip("scipy.interpolate")
    z = np.linspace(0.0, 1.5, 37) ** 1.3
    d = 3000 * z / (1 + 0.3 * z)
    p = tmp_path / "zd.txt"
    np.savetxt(p, np.column_stack([z, d]), fmt="%.17g", header="z D")
    c = Cosmo()
    assert cnvt.psh_cosmo_init(ctypes.byref(c), str(p).encode(), 0.0, 0.0, False) == 0
    sp = interpolate.CubicSpline(z, d, bc_type="natural")
    for zz in np.linspace(0, z[-1] * 0.999, 50):
        assert cnvt.psh_cosmo_distance(ctypes.byref(c), zz) == pytest.approx(float(sp(zz)), rel=1e-12)
    assert np.isinf(cnvt.psh_cosmo_distance(ctypes.byref(c), z[-1] + 0.1))
    cnvt.psh_cosmo_free(ctypes.byref(c))
