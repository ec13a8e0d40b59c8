"""The device libsvm reader's number conversion (libirwls_gb300/csrc/
numparse.cuh: exact strtod and strtol restated for the GPU) compiled for the
host and checked bit for bit against the C library, without a GPU: random
decimals of every shape (signs, leading zeros, points, exponents, 1 to 26
digits, trailing text), the shortest and long representations of random
doubles including subnormals, 17-19-digit truncations of the exact midpoints
between adjacent doubles, overflow and underflow edges, and strtol with
overflow. Decimals of more than 19 digits within their truncation interval
of a rounding boundary, hexadecimal numbers and NaN payloads are reported as
not converted; everything else must equal the C library's value and end."""
import ctypes as C
import math
import os
import random
import shutil
import struct
import subprocess
import tempfile
from decimal import Decimal, getcontext

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "libirwls_gb300", "csrc")
SHIM = r"""
#include "numparse.cuh"
extern "C" double np_strtod(const char *s, int len, int *end, int *unsup) {
    double v;
    *end = dev_strtod(s, 0, len, &v, unsup);
    return v;
}
extern "C" int np_strtol(const char *s, int len, int *end) { return dev_strtol(s, 0, len, end); }
"""


@pytest.fixture(scope="module")
def np_lib():
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    d = tempfile.mkdtemp()
    src, so = os.path.join(d, "shim.cpp"), os.path.join(d, "np.so")
    with open(src, "w") as f:
        f.write(SHIM)
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, "-o", so, src], check=True)
    lib = C.CDLL(so)
    lib.np_strtod.restype = C.c_double
    lib.np_strtod.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.np_strtol.restype = C.c_int
    lib.np_strtol.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int)]
    yield lib
    shutil.rmtree(d)


LIBC = C.CDLL(None)
LIBC.strtod.restype = C.c_double
LIBC.strtod.argtypes = [C.c_char_p, C.POINTER(C.c_char_p)]
LIBC.strtol.restype = C.c_long
LIBC.strtol.argtypes = [C.c_char_p, C.POINTER(C.c_char_p), C.c_int]


def _bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def _check_strtod(lib, s, stats):
    b = s.encode()
    buf = C.create_string_buffer(b)
    endp = C.c_char_p()
    ref = LIBC.strtod(buf, C.byref(endp))
    ref_end = C.cast(endp, C.c_void_p).value - C.cast(buf, C.c_void_p).value
    e, u = C.c_int(), C.c_int()
    got = lib.np_strtod(b, len(b), C.byref(e), C.byref(u))
    if u.value:
        stats["unsupported"] += 1
        return
    same = (math.isnan(ref) and math.isnan(got)) or _bits(ref) == _bits(got)
    assert same and e.value == ref_end, (s, ref, got, ref_end, e.value)
    stats["checked"] += 1


def _strings(rng):
    digits = lambda k: "".join(rng.choice("0123456789") for _ in range(k))
    for _ in range(40000):
        d = digits(rng.randint(0, 26))
        if rng.random() < 0.3:
            d = "0" * rng.randint(1, 5) + d
        if rng.random() < 0.6 and d:
            k = rng.randint(0, len(d))
            d = d[:k] + "." + d[k:]
        ex = ""
        if rng.random() < 0.5:
            ex = rng.choice("eE") + rng.choice(["", "+", "-"]) + str(rng.randint(0, 400))
            if rng.random() < 0.05:
                ex = rng.choice(["e", "e+", "E-"])
        yield rng.choice(["", "-", "+", " ", "\t-"]) + d + ex + rng.choice(["", "", "x", " 3", "\n", ":"])
    for _ in range(40000):
        if rng.random() < 0.5:
            x = struct.unpack("<d", struct.pack("<Q", rng.getrandbits(63)))[0]
        else:
            x = rng.uniform(-1, 1) * 10 ** rng.randint(-30, 30)
        if math.isnan(x) or math.isinf(x):
            continue
        fmt = rng.choice(["%r", "%.17g", "%.16g", "%.20g", "%.25e", "%.6f", "%.12e", "%.19g"])
        yield repr(x) if fmt == "%r" else fmt % x
    getcontext().prec = 2000
    for _ in range(4000):
        xb = rng.getrandbits(62) | (rng.getrandbits(1) << 62)
        x = struct.unpack("<d", struct.pack("<Q", xb))[0]
        y = struct.unpack("<d", struct.pack("<Q", xb + 1))[0]
        if math.isinf(y) or math.isnan(y) or math.isnan(x):
            continue
        mid = (Decimal(x) + Decimal(y)) / 2
        yield format(mid, "e")
        for nd in (17, 18, 19):
            yield format(mid, ".%de" % (nd - 1))
    yield from ["inf", "-INF", "Infinity", "nan", "-nan", "infin", "in", "na", "0x1p3", "0x", "0xg", "1e", ".", "+",
                "", "1e309", "-1e309", "1e-400", "4.9406564584124654e-324", "2.4703282292062327e-324",
                "2.4703282292062328e-324", "1.7976931348623157e308", "1.7976931348623159e308",
                "2.2250738585072011e-308", "9007199254740993", "9007199254740992.5", "1" * 30,
                "0." + "0" * 400 + "1"]


def test_strtod_equals_the_c_library(np_lib):
    stats = {"checked": 0, "unsupported": 0}
    for s in _strings(random.Random(1)):
        _check_strtod(np_lib, s, stats)
    assert stats["checked"] > 70000
    assert stats["unsupported"] < 0.1 * stats["checked"]


def test_strtol_equals_the_c_library(np_lib):
    rng = random.Random(2)
    for _ in range(30000):
        s = (rng.choice(["", " ", "-", "+", "\t"]) + "".join(rng.choice("0123456789") for _ in range(rng.randint(0, 22)))
             + rng.choice(["", "x", " ", ":"]))
        b = s.encode()
        buf = C.create_string_buffer(b)
        endp = C.c_char_p()
        ref = C.c_int(LIBC.strtol(buf, C.byref(endp), 10) & 0xffffffff).value
        ref_end = C.cast(endp, C.c_void_p).value - C.cast(buf, C.c_void_p).value
        e = C.c_int()
        assert (np_lib.np_strtol(b, len(b), C.byref(e)), e.value) == (ref, ref_end), s
