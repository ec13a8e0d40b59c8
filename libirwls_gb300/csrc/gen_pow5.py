"""Writes pow5_table.cuh: for every decimal exponent q in [-342, 308], the
128-bit T_q = floor(5^q 2^(127 - E_q)) with E_q = floor(log2 5^q), so that
2^127 <= T_q < 2^128 and 5^q 2^(127 - E_q) lies in [T_q, T_q + 1). The table
is exact: Python integers, no floating point. Run from this directory:

    python gen_pow5.py > pow5_table.cuh
"""
import sys

QMIN, QMAX = -342, 308


def entry(q):
    """(T_q, E_q)."""
    if q >= 0:
        v = 5 ** q
        e = v.bit_length() - 1
        t = v << (127 - e) if e <= 127 else v >> (e - 127)
    else:
        d = 5 ** -q  # not a power of two, so log2(1 / d) lies strictly between two integers
        e = -d.bit_length()
        t = (1 << (127 - e)) // d
    assert 1 << 127 <= t < 1 << 128
    return t, e


def main(out=sys.stdout):
    w = out.write
    w("// pow5_table.cuh -- generated by gen_pow5.py; do not edit.\n")
    w("// NP_POW5[q - NP_POW5_QMIN] = {high 64 bits, low 64 bits} of\n")
    w("// T_q = floor(5^q 2^(127 - E_q)), 2^127 <= T_q < 2^128, and\n")
    w("// NP_POW5_E[q - NP_POW5_QMIN] = E_q = floor(log2 5^q), for q in [%d, %d].\n" % (QMIN, QMAX))
    w("#pragma once\n#include <stdint.h>\n\n")
    w("#define NP_POW5_QMIN (%d)\n#define NP_POW5_QMAX %d\n\n" % (QMIN, QMAX))
    rows = [entry(q) for q in range(QMIN, QMAX + 1)]
    for space, name in (("static const", "NP_POW5_H"), ("__device__ static const", "NP_POW5_D")):
        if space.startswith("__device__"):
            w("#ifdef __CUDACC__\n")
        w("%s uint64_t %s[%d][2] = {\n" % (space, name, len(rows)))
        for t, _ in rows:
            w("    {0x%016xULL, 0x%016xULL},\n" % (t >> 64, t & ((1 << 64) - 1)))
        w("};\n")
        w("%s int16_t %s_E[%d] = {\n" % (space, name, len(rows)))
        for k in range(0, len(rows), 12):
            w("    " + ", ".join("%d" % e for _, e in rows[k:k + 12]) + ",\n")
        w("};\n")
        if space.startswith("__device__"):
            w("#endif\n")
        w("\n")


if __name__ == "__main__":
    main()
