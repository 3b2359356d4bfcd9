"""The double-float primitives of the complex128 gate kernels
(qcware_unitair_gb300/csrc/dfloat.cuh), compiled for the host from the same
header and checked against exact rational arithmetic (fractions.Fraction):

* df_split keeps a double to 2^-48 relative, with hi the double rounded to
  a float and the rounding of lo unbiased;
* df_entry splits a double exactly;
* df_join rounds a renormalised pair to the nearest double (1 ulp);
* the gate forms (full, real, RX, diagonal) of one amplitude pair stay
  within a few 2^-47 of the exact product;
* the squared norm of a gate's output carries no bias against the exact
  product (a product that rounds its smallest terms away with a fixed
  sign would shrink every gate by about 2^-48 and drift the norm of deep
  circuits; an unbiased one stays within sampling noise of zero)."""
import ctypes
import math
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "qcware_unitair_gb300" / "csrc"
SRC = Path(__file__).resolve().parent / "native" / "dfloat_host.cpp"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("dfh") / "libdfh.so"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                    f"-I{CSRC}", str(SRC), "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    L.dfh_split.argtypes = [ctypes.c_double, fp]
    L.dfh_entry.argtypes = [ctypes.c_double, fp]
    L.dfh_join.argtypes = [ctypes.c_float, ctypes.c_float]
    L.dfh_join.restype = ctypes.c_double
    L.dfh_fast2.argtypes = [ctypes.c_float, ctypes.c_float, fp]
    L.dfh_gate.argtypes = [dp, dp, ctypes.c_int, dp]
    return L


def _f32(n):
    return (ctypes.c_float * n)()


def _values(rng, count, lo_exp, hi_exp):
    mag = np.exp2(rng.uniform(lo_exp, hi_exp, count))
    sign = rng.choice([-1.0, 1.0], count)
    return mag * sign * rng.uniform(1.0, 2.0, count)


def test_split_accuracy_and_shape(lib):
    rng = np.random.default_rng(1)
    out = _f32(2)
    errs = []
    for x in list(_values(rng, 3000, -40, 60)) + [1.0, -1.0, 0.5,
                                                   1 / math.sqrt(2)]:
        lib.dfh_split(float(x), out)
        hi, lo = out[0], out[1]
        # hi: x rounded to a float; lo: the remainder, rounded
        assert hi == float(np.float32(x))
        err = (Fraction(hi) + Fraction(lo) - Fraction(float(x))) / \
            Fraction(float(x))
        assert abs(err) <= Fraction(1, 2 ** 48)
        errs.append(float(err))
    # rounding to nearest: the signed error averages out
    assert abs(np.mean(errs)) < 2.0 ** -52


def test_split_zero_and_tiny(lib):
    out = _f32(2)
    for x, want in [(0.0, 0.0), (-0.0, 0.0), (1e-300, 0.0), (2.0 ** -127,
                                                              0.0)]:
        lib.dfh_split(x, out)
        assert out[0] == want and out[1] == 0.0
    # between 2^-126 and 2^-80: hi only
    lib.dfh_split(2.0 ** -100 * 1.2345, out)
    assert out[1] == 0.0 and abs(out[0] / (2.0 ** -100 * 1.2345) - 1) < 2e-7


def test_entry_is_exact(lib):
    rng = np.random.default_rng(2)
    out = _f32(3)
    for x in list(_values(rng, 2000, -74, 100)) + [1.0, -1 / math.sqrt(2),
                                                   math.cos(0.35), 0.0]:
        lib.dfh_entry(float(x), out)
        assert Fraction(out[0]) + Fraction(out[1]) + Fraction(out[2]) == \
            Fraction(float(x))
    lib.dfh_entry(2.0 ** -80, out)
    assert (out[0], out[1], out[2]) == (0.0, 0.0, 0.0)


def _nearest_double_err(got, exact):
    """|got - exact| in ulps of exact's binade."""
    if exact == 0:
        return abs(got)
    ulp = math.ulp(float(exact))
    return abs(Fraction(got) - exact) / Fraction(ulp)


def test_join_rounds_pairs(lib):
    rng = np.random.default_rng(3)
    out = _f32(2)
    worst = 0
    for _ in range(4000):
        a = np.float32(rng.uniform(-1, 1) * 2.0 ** rng.integers(-30, 30))
        b = np.float32(a * rng.uniform(-1, 1) * 2.0 ** -rng.integers(20, 40))
        lib.dfh_fast2(float(a), float(b), out)
        hi, lo = out[0], out[1]
        exact = Fraction(hi) + Fraction(lo)
        assert exact == Fraction(float(a)) + Fraction(float(b))
        got = lib.dfh_join(hi, lo)
        worst = max(worst, _nearest_double_err(got, exact))
    # powers of two with a lower low word (the half-ulp binade below)
    for k in range(-20, 20):
        for lo in (-2.0 ** (k - 30), -2.0 ** (k - 25) * 1.5,
                   2.0 ** (k - 26)):
            hi = np.float32(2.0 ** k)
            exact = Fraction(float(hi)) + Fraction(float(np.float32(lo)))
            got = lib.dfh_join(float(hi), float(np.float32(lo)))
            worst = max(worst, _nearest_double_err(got, exact))
    assert worst <= 1
    assert lib.dfh_join(0.0, 0.0) == 0.0


FORMS = {0: "full", 1: "real", 2: "rx", 3: "diag", 4: "rdiag", 5: "idiag"}


def _matrix(rng, form):
    th = rng.uniform(0, 2 * math.pi)
    if form == 0:
        q, _ = np.linalg.qr(rng.normal(size=(2, 2)) +
                            1j * rng.normal(size=(2, 2)))
        return q
    if form == 1:
        c, s = math.cos(th), math.sin(th)
        return np.array([[c, -s], [s, c]], dtype=complex)
    if form == 2:
        c, s = math.cos(th), math.sin(th)
        return np.array([[c, -1j * s], [-1j * s, c]])
    if form == 3:
        return np.diag(np.exp(1j * rng.uniform(0, 6.3, 2)))
    if form == 4:
        return np.diag([math.cos(th), -math.sin(th)]).astype(complex)
    return np.diag([1j * math.cos(th), -1j * math.sin(th)])


@pytest.mark.parametrize("form", sorted(FORMS))
def test_gate_forms_vs_exact(lib, form):
    rng = np.random.default_rng(10 + form)
    dp = ctypes.c_double * 8
    signed = []
    for _ in range(1500):
        m = _matrix(rng, form)
        a = (rng.normal(size=2) + 1j * rng.normal(size=2)) * \
            2.0 ** rng.integers(-20, 10)
        mv = dp(*[v for z in m.reshape(-1) for v in (z.real, z.imag)])
        av = dp(*[v for z in a for v in (z.real, z.imag)])
        yv = dp()
        lib.dfh_gate(mv, av, form, yv)
        F = Fraction
        mr = [[(F(float(m[i, j].real)), F(float(m[i, j].imag)))
               for j in range(2)] for i in range(2)]
        ar = [(F(float(z.real)), F(float(z.imag))) for z in a]
        scale = F(max(abs(a[0]), abs(a[1])))
        for i in range(2):
            re = sum(mr[i][j][0] * ar[j][0] - mr[i][j][1] * ar[j][1]
                     for j in range(2))
            im = sum(mr[i][j][0] * ar[j][1] + mr[i][j][1] * ar[j][0]
                     for j in range(2))
            for got, want in ((yv[2 * i], re), (yv[2 * i + 1], im)):
                err = (F(got) - want) / scale
                assert abs(err) <= F(1, 2 ** 44), (FORMS[form], float(err))
                if want != 0:
                    signed.append(float((F(got) - want) / abs(want)))
    assert len(signed) > 0


def test_4x4_rows_vs_exact(lib):
    rng = np.random.default_rng(20)
    d32 = ctypes.c_double * 32
    d8 = ctypes.c_double * 8
    lib.dfh_gate4.argtypes = [d32, d8, d8]
    F = Fraction
    signed = []
    for _ in range(400):
        q, _ = np.linalg.qr(rng.normal(size=(4, 4)) +
                            1j * rng.normal(size=(4, 4)))
        a = rng.normal(size=4) + 1j * rng.normal(size=4)
        y = d8()
        lib.dfh_gate4(d32(*[v for z in q.reshape(-1)
                            for v in (z.real, z.imag)]),
                      d8(*[v for z in a for v in (z.real, z.imag)]), y)
        scale = F(float(np.abs(a).max()))
        for i in range(4):
            re = sum(F(q[i, j].real) * F(a[j].real) -
                     F(q[i, j].imag) * F(a[j].imag) for j in range(4))
            im = sum(F(q[i, j].real) * F(a[j].imag) +
                     F(q[i, j].imag) * F(a[j].real) for j in range(4))
            for got, want in ((y[2 * i], re), (y[2 * i + 1], im)):
                assert abs((F(got) - want) / scale) <= F(1, 2 ** 43)
                if abs(want) > scale / 8:
                    signed.append(float((F(got) - want) / abs(want)))
    assert abs(np.mean(signed)) < 2.0 ** -49


@pytest.mark.parametrize("form", [0, 1])
def test_gate_norm_has_no_bias(lib, form):
    """Mean relative change of |y|^2 against the exact product over 4,000
    random gates, in units of 2^-53: the per-gate spread is about 27, so
    the sampling error of the mean is about 0.43; a rounding bias of the
    kind described above shows as -39."""
    rng = np.random.default_rng(30 + form)
    dp = ctypes.c_double * 8
    F = Fraction
    dn = []
    for _ in range(4000):
        m = _matrix(rng, form)
        a = (rng.normal(size=2) + 1j * rng.normal(size=2)) * 0.01
        y = dp()
        lib.dfh_gate(dp(*[v for z in m.reshape(-1) for v in (z.real, z.imag)]),
                     dp(*[v for z in a for v in (z.real, z.imag)]), form, y)
        mr = [[(F(float(m[i, j].real)), F(float(m[i, j].imag)))
               for j in range(2)] for i in range(2)]
        ar = [(F(float(z.real)), F(float(z.imag))) for z in a]
        exact = []
        for i in range(2):
            exact.append(sum(mr[i][j][0] * ar[j][0] - mr[i][j][1] * ar[j][1]
                             for j in range(2)))
            exact.append(sum(mr[i][j][0] * ar[j][1] + mr[i][j][1] * ar[j][0]
                             for j in range(2)))
        n_ex = sum(e * e for e in exact)
        n_got = sum(F(y[i]) ** 2 for i in range(4))
        dn.append(float((n_got - n_ex) / n_ex) / 2.0 ** -53)
    assert abs(np.mean(dn)) < 2.5, np.mean(dn)


def test_8x8_rows_vs_exact_and_unbiased(lib):
    """df_rowD<8> (3-qubit operators): within a few 2^-47 of the exact
    product, and no bias in the squared norm of the output."""
    rng = np.random.default_rng(40)
    d128 = ctypes.c_double * 128
    d16 = ctypes.c_double * 16
    lib.dfh_gate8.argtypes = [d128, d16, d16]
    F = Fraction
    dn = []
    for _ in range(300):
        q, _ = np.linalg.qr(rng.normal(size=(8, 8)) +
                            1j * rng.normal(size=(8, 8)))
        a = (rng.normal(size=8) + 1j * rng.normal(size=8)) * 0.01
        y = d16()
        lib.dfh_gate8(d128(*[v for z in q.reshape(-1)
                             for v in (z.real, z.imag)]),
                      d16(*[v for z in a for v in (z.real, z.imag)]), y)
        scale = F(float(np.abs(a).max()))
        exact = []
        for i in range(8):
            re = sum(F(q[i, j].real) * F(a[j].real) -
                     F(q[i, j].imag) * F(a[j].imag) for j in range(8))
            im = sum(F(q[i, j].real) * F(a[j].imag) +
                     F(q[i, j].imag) * F(a[j].real) for j in range(8))
            for got, want in ((y[2 * i], re), (y[2 * i + 1], im)):
                assert abs((F(got) - want) / scale) <= F(1, 2 ** 43)
            exact += [re, im]
        n_ex = sum(e * e for e in exact)
        n_got = sum(F(y[i]) ** 2 for i in range(16))
        dn.append(float((n_got - n_ex) / n_ex) / 2.0 ** -53)
    # spread about 39 per output norm: the mean of 300 is within +-2.3 (one
    # sigma); a fixed-sign rounding shows as about -39
    assert abs(np.mean(dn)) < 10.0, np.mean(dn)


def test_sincos_vs_high_precision(lib):
    """df_sincos (apply_phase's phase factor for float64 angles) against
    50-digit values: a few 2^-47 absolute at most, for angles up to 2^20,
    multiples of pi/2 and tiny angles."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    d2 = ctypes.c_double * 2
    lib.dfh_sincos.argtypes = [ctypes.c_double, d2]
    rng = np.random.default_rng(50)
    vals = (list(rng.uniform(-7, 7, 800)) +
            list(rng.uniform(-2.0 ** 20, 2.0 ** 20, 800)) +
            list(rng.uniform(-1e-3, 1e-3, 100)) +
            [k * math.pi / 2 for k in range(-40, 41)] +
            [0.0, 1e-30, -1e-30, 2.0 ** 20 - 1, math.pi / 4] +
            [k * math.pi / 2 + d for k in (1, 3, 1000, 654321)
             for d in (1e-9, -1e-9, 1e-15)])
    worst = 0.0
    for x in vals:
        o = d2()
        lib.dfh_sincos(float(x), o)
        xs = mpmath.mpf(float(x))
        worst = max(worst, abs(float(o[0] - mpmath.sin(xs))),
                    abs(float(o[1] - mpmath.cos(xs))))
    assert worst <= 2.0 ** -45, worst
