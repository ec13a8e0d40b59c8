"""The libsvm reader on the GPU (irwls_parse_libsvm / readTrainFileGPU,
libirwls_gb300/csrc/dev_parse.cu) against the reference's reader:

- the golden reader fixtures: the reference's own parse of two files, with
  the rows laid out from pass 1's entry counts and written by one pass 2;
- randomised files (tabs, repeated and trailing blanks, CRLF, exponents,
  17-digit and subnormal values, signs, ragged and dense rows) against the
  host readTrainFile, field by field and bit for bit, class-mean rows
  included;
- the device strtod against the C library's on random and hard strings;
- the reference's format errors (reported with their line), a line longer
  than the reference's line buffer, numbers the reader does not convert, and
  the empty file.
"""
import ctypes as C
import math
import os
import random
import struct
import tempfile

import numpy as np
import pytest

import harness as H
from libirwls_gb300 import _abi, load

pytestmark = pytest.mark.gpu

LIBC = C.CDLL(None)
LIBC.strtod.restype = C.c_double
LIBC.strtod.argtypes = [C.c_char_p, C.POINTER(C.c_char_p)]


def _lib():
    lib = load()
    lib.irwls_parse_libsvm.restype = C.c_int
    lib.irwls_parse_libsvm.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(_abi.SvmDataset)]
    lib.irwls_parse_doubles.restype = C.c_longlong
    lib.irwls_parse_doubles.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                        C.c_longlong]
    lib.readTrainFileGPU.restype = _abi.SvmDataset
    lib.readTrainFileGPU.argtypes = [C.c_char_p]
    return lib


def _parse(lib, text):
    ds = _abi.SvmDataset()
    rc = lib.irwls_parse_libsvm(text, len(text), C.byref(ds))
    return rc, ds


def _fields(ds):
    rows, y, q = _abi.dataset_rows(ds, ds.l + 2)
    return ds.l, ds.sparse, ds.maxdim, rows, y, q


def _same(a, b):
    la, sa, ma, ra, ya, qa = _fields(a)
    lb, sb, mb, rb, yb, qb = _fields(b)
    assert (la, sa, ma) == (lb, sb, mb)
    assert len(ra) == len(rb)
    for (ia, va), (ib, vb) in zip(ra, rb):
        assert np.array_equal(ia, ib)
        assert np.array_equal(va.view(np.int64), vb.view(np.int64))
    assert np.array_equal(ya.view(np.int64), yb.view(np.int64))
    assert np.array_equal(qa.view(np.int64), qb.view(np.int64))


def _host(lib, text):
    with tempfile.NamedTemporaryFile(suffix=".libsvm", delete=False) as f:
        f.write(text)
        path = f.name
    try:
        return lib.readTrainFile(path.encode()), path
    except BaseException:
        os.unlink(path)
        raise


@pytest.mark.parametrize("key", ["dense", "onehot"])
def test_golden_files(key):
    lib = _lib()
    g = np.load(os.path.join(H.GOLDEN, "reader.npz"))
    n0 = lib.irwls_kernel_launches()
    rc, ds = _parse(lib, g[key + "_text"].tobytes())
    assert rc == 0, lib.irwls_last_error_message()
    # one pass 2: the rows laid out from pass 1's counts (newline count and
    # write, pass 1, pass 2, the sparse flag)
    assert lib.irwls_kernel_launches() - n0 == 5
    assert ds.l == int(g[key + "_l"]) and ds.sparse == int(g[key + "_sparse"])
    assert ds.maxdim == int(g[key + "_maxdim"])
    rows, y, q = _abi.dataset_rows(ds, ds.l + 2)
    lens = g[key + "_lens"]
    assert [len(r[0]) for r in rows] == list(lens)
    assert np.array_equal(np.concatenate([r[0] for r in rows]), g[key + "_idx"])
    assert np.array_equal(np.concatenate([r[1] for r in rows]), g[key + "_val"])
    assert np.array_equal(y, g[key + "_y"]) and np.array_equal(q, g[key + "_q"])
    lib.freeDataset(ds)


def _value(rng):
    k = rng.random()
    if k < 0.3:
        return repr(rng.uniform(-3, 3))
    if k < 0.45:
        return "%.6g" % rng.uniform(-1e4, 1e4)
    if k < 0.55:
        return str(rng.randint(-5, 5))
    if k < 0.65:
        return "%.3e" % (rng.uniform(-1, 1) * 10 ** rng.randint(-300, 300))
    if k < 0.7:
        return repr(struct.unpack("<d", struct.pack("<Q", rng.getrandbits(52)))[0])  # subnormal
    if k < 0.8:
        return "%.17g" % rng.gauss(0, 1)
    if k < 0.9:
        return "0.%s" % "".join(rng.choice("0123456789") for _ in range(rng.randint(1, 18)))
    return rng.choice(["1", "0", "-0", "1.", ".5", "+2", "1E3", "2e-05"])


def _file(rng, n, d, dense):
    lines = []
    for _ in range(n):
        lab = rng.choice(["1", "-1", "+1", "-1.0", "1.0", "1", "-1"])
        idx = list(range(1, d + 1)) if dense else sorted(rng.sample(range(1, d + 1), rng.randint(0, min(d, 12))))
        sep = lambda: rng.choice([" ", " ", " ", "\t", "  ", " \t"])
        parts = [lab] + ["%d:%s" % (i, _value(rng)) for i in idx]
        line = parts[0] + "".join(sep() + p for p in parts[1:])
        # a row without entries followed by "\r" is a format error for the reference
        line += rng.choice(["", "", " ", "\t", "\r"] if idx else ["", " ", "\t"])
        lines.append(line)
    return ("\n".join(lines) + rng.choice(["\n", ""])).encode()


@pytest.mark.parametrize("seed,n,d,dense", [(1, 3000, 40, False), (2, 2000, 12, True), (3, 500, 300, False),
                                            (4, 1, 5, True), (5, 4000, 60, False)])
def test_random_files_equal_host_reader(seed, n, d, dense):
    lib = _lib()
    text = _file(random.Random(seed), n, d, dense)
    n0 = lib.irwls_kernel_launches()
    rc, dev = _parse(lib, text)
    assert rc == 0, lib.irwls_last_error_message()
    assert lib.irwls_kernel_launches() - n0 == 5  # pass 1's counts were pass 2's on every line
    host, path = _host(lib, text)
    try:
        _same(dev, host)
        gpu = lib.readTrainFileGPU(path.encode())
        _same(gpu, host)
        lib.freeDataset(gpu)
    finally:
        os.unlink(path)
    lib.freeDataset(dev)
    lib.freeDataset(host)


def test_strtod_matches_the_c_library():
    lib = _lib()
    rng = random.Random(11)
    strs = []
    for _ in range(60000):
        k = rng.random()
        if k < 0.4:
            x = struct.unpack("<d", struct.pack("<Q", rng.getrandbits(63)))[0]
            if math.isnan(x) or math.isinf(x):
                continue
            strs.append(rng.choice(["%r", "%.17g", "%.16g", "%.19g", "%.12e"]) % x if rng.random() < 0.8 else repr(x))
        else:
            d = "".join(rng.choice("0123456789") for _ in range(rng.randint(1, 25)))
            if rng.random() < 0.6:
                p = rng.randint(0, len(d))
                d = d[:p] + "." + d[p:]
            if rng.random() < 0.5:
                d += rng.choice("eE") + rng.choice(["", "+", "-"]) + str(rng.randint(0, 350))
            strs.append(rng.choice(["", "-", "+"]) + d)
    strs += ["inf", "-Infinity", "nan", "1e309", "2.4703282292062328e-324", "1.7976931348623158e308", "", "abc"]
    text = ("\n".join(strs) + "\n").encode()
    out = (C.c_double * len(strs))()
    st = (C.c_int * len(strs))()
    n = lib.irwls_parse_doubles(text, len(text), out, st, len(strs))
    assert n == len(strs)
    checked = 0
    for i, s in enumerate(strs):
        b = C.create_string_buffer(s.encode())
        end = C.c_char_p()
        ref = LIBC.strtod(b, C.byref(end))
        consumed = C.cast(end, C.c_void_p).value - C.cast(b, C.c_void_p).value
        if st[i] == 2:
            continue
        if consumed == 0:
            assert st[i] == -1, s
            continue
        assert st[i] == (0 if consumed == len(s) else 1), s
        if math.isnan(ref):
            assert math.isnan(out[i]), s
        else:
            assert struct.pack("<d", ref) == struct.pack("<d", out[i]), (s, ref, out[i])
        checked += 1
    assert checked > 0.95 * len(strs)


@pytest.mark.parametrize("text,line", [(b"1 1:0.5\n-1 2:0.1 1:0.3\n", 2), (b"1 1:0.5\n\n", 2),
                                       (b"1 1:x\n", 1), (b"+1 3:1 4a:2\n", 1), (b"1 3:\n", 1), (b"one 1:2\n", 1)])
def test_format_errors(text, line):
    lib = _lib()
    rc, _ = _parse(lib, text)
    assert rc == -20
    assert ("line %d" % line).encode() in lib.irwls_last_error_message()


def test_unsupported_and_too_long():
    lib = _lib()
    assert _parse(lib, b"1 1:0x1p3\n")[0] == -21
    long_line = b"1" + b"".join(b" %d:1" % k for k in range(1, 30000)) + b"\n"
    assert len(long_line) > 99999
    assert _parse(lib, long_line)[0] == -22


def test_empty_file():
    lib = _lib()
    rc, ds = _parse(lib, b"")
    assert rc == 0
    host, path = _host(lib, b"")
    try:
        assert ds.l == host.l == 0
        _same(ds, host)
    finally:
        os.unlink(path)
