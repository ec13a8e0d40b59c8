"""The interval step of the device reader's decimal conversion
(np_interval_round in libirwls_gb300/csrc/numparse.cuh, with the table of
libirwls_gb300/csrc/pow5_table.cuh), compiled for the host, without a GPU:

- the committed table is the generator's output, and every entry satisfies
  T_q <= 5^q 2^(127 - E_q) < T_q + 1 with 2^127 <= T_q < 2^128, checked here
  with integer arithmetic of its own;
- wherever the step answers, its double is w 10^q rounded to nearest even
  (exact rationals: Python's integer division rounds correctly), over random
  w of every length and q across the whole table, and at the subnormal,
  overflow and tie edges;
- it answers for all but a tiny fraction of random inputs, and declines the
  exact ties that the interval cannot settle;
- dec_to_double (Clinger's path, the step, big integers) equals exact
  rounding on the same inputs.
"""
import ctypes as C
import io
import os
import random
import re
import shutil
import subprocess
import sys
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "libirwls_gb300", "csrc")
SHIM = r"""
#include "numparse.cuh"
extern "C" int np_step(unsigned long long w, int q, double *out) { return np_interval_round(w, q, out) ? 1 : 0; }
extern "C" double np_dec(unsigned long long w, int q) { return dec_to_double(w, q); }
"""


@pytest.fixture(scope="module")
def lib():
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    d = tempfile.mkdtemp()
    src, so = os.path.join(d, "shim.cpp"), os.path.join(d, "np.so")
    with open(src, "w") as f:
        f.write(SHIM)
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, "-o", so, src], check=True)
    h = C.CDLL(so)
    h.np_step.restype = C.c_int
    h.np_step.argtypes = [C.c_ulonglong, C.c_int, C.POINTER(C.c_double)]
    h.np_dec.restype = C.c_double
    h.np_dec.argtypes = [C.c_ulonglong, C.c_int]
    yield h
    shutil.rmtree(d)


def exact(w, q):
    """w 10^q rounded to nearest even."""
    try:
        return float(w * 10 ** q) if q >= 0 else w / 10 ** -q
    except OverflowError:
        return float("inf")


def step(lib, w, q):
    out = C.c_double()
    return out.value if lib.np_step(w, q, C.byref(out)) else None


def test_table_is_generated_and_exact():
    sys.path.insert(0, CSRC)
    try:
        import gen_pow5
    finally:
        sys.path.pop(0)
    buf = io.StringIO()
    gen_pow5.main(buf)
    with open(os.path.join(CSRC, "pow5_table.cuh")) as f:
        text = f.read()
    assert text == buf.getvalue()
    host = text[text.index("NP_POW5_H[651][2]"):text.index("NP_POW5_H_E")]
    ents = [(int(a, 16) << 64) | int(b, 16) for a, b in re.findall(r"\{0x([0-9a-f]+)ULL, 0x([0-9a-f]+)ULL\}", host)]
    es = [int(v) for v in re.findall(r"-?\d+", text[text.index("NP_POW5_H_E[651] = {") + 20:text.index("};", text.index("NP_POW5_H_E"))])]
    assert len(ents) == len(es) == 651
    for k, (t, e) in enumerate(zip(ents, es)):
        q = k - 342
        assert 1 << 127 <= t < 1 << 128
        s = 127 - e
        if q >= 0:
            num, den = 5 ** q * (1 << max(s, 0)), 1 << max(-s, 0)
        else:
            num, den = 1 << s, 5 ** -q
        assert t * den <= num < (t + 1) * den, q  # T <= 5^q 2^s < T + 1


def _random_cases(rng, n):
    for _ in range(n):
        bits = rng.randint(1, 64)
        w = rng.getrandbits(bits) | (1 << (bits - 1))
        q = rng.randint(-342, 308)
        yield w, q


def test_step_is_exact_where_it_answers(lib):
    rng = random.Random(5)
    answered = total = 0
    for w, q in _random_cases(rng, 200000):
        r = step(lib, w, q)
        total += 1
        if r is None:
            continue
        answered += 1
        assert r == exact(w, q) or (r != r and exact(w, q) != exact(w, q)), (w, q, r, exact(w, q))
    assert answered >= 0.999 * total, (answered, total)


def test_step_edges(lib):
    cases = []
    # 17-19 digit decimals around the subnormal range, the normal minimum and the overflow edge
    for s in ["2.4703282292062327e-324", "2.4703282292062328e-324", "4.9406564584124654e-324",
              "2.2250738585072011e-308", "2.2250738585072012e-308", "2.2250738585072014e-308",
              "1.7976931348623157e308", "1.7976931348623158e308", "1.7976931348623159e308",
              "9.9999999999999999e-343", "1.0000000000000001e308", "4.4501477170144023e-308",
              "8.9884656743115795e307", "1.0e-320", "3.0e-324", "2.5e-324"]:
        mant, ex = s.split("e")
        ip, fp = mant.split(".")
        cases.append((int(ip + fp), int(ex) - len(fp)))
    # every double's neighbourhood: 17 and 19 significant digits of random doubles
    rng = random.Random(9)
    for _ in range(20000):
        x = abs(rng.choice([rng.uniform(0, 1), rng.gauss(0, 1) * 10 ** rng.randint(-300, 300),
                            5e-324 * rng.randint(1, 1 << 52)]))
        if x == 0.0:
            continue
        for digits in (17, 19):
            m, e = ("%.*e" % (digits - 1, x)).split("e")
            cases.append((int(m.replace(".", "")), int(e) - (digits - 1)))
    for w, q in cases:
        if not (-342 <= q <= 308):
            continue
        r = step(lib, w, q)
        if r is not None:
            assert r == exact(w, q), (w, q, r, exact(w, q))
        assert lib.np_dec(w, q) == exact(w, q), (w, q)


def test_exact_ties_are_declined_or_rounded_to_even(lib):
    # w 10^q exactly halfway between two doubles
    rng = random.Random(3)
    for _ in range(3000):
        m = rng.getrandbits(52) | (1 << 52)
        e = rng.randint(-60, 60)
        # the midpoint (2m + 1) 2^(e - 1) written as w 10^q with q <= 0: w = (2m + 1) 5^k, 2^-k scaled
        if e - 1 >= 0:
            w, q = (2 * m + 1) << (e - 1), 0
        else:
            k = 1 - e
            w, q = (2 * m + 1) * 5 ** k, -k
        if w >= 1 << 64:
            continue
        r = step(lib, w, q)
        want = exact(w, q)
        assert r is None or r == want, (w, q)
        assert lib.np_dec(w, q) == want
