"""The text rules of the GPU Matrix Market conversion (mtx_parse.h), built for
the host and checked against the C library: atoi, (float)strtod and strtok
on seeded random and hand-picked tokens -- decimal text with up to 900
digits, exponents over the whole double range, subnormals, halfway cases,
hexadecimal floats, infinities, NaNs and junk.  No GPU."""
import ctypes as C
import os
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("mtx") / "libmtxh.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "dbd_gb300", "csrc"),
                    os.path.join(HERE, "helpers", "mtx_parse_harness.cpp"), "-o", out], check=True)
    h = C.CDLL(out)
    h.mh_atoi.argtypes = [C.c_char_p, C.c_int]
    h.mh_atoi.restype = C.c_int
    h.mh_value.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int)]
    h.mh_value.restype = C.c_float
    h.mh_decimal_double.argtypes = [C.c_char_p, C.c_int]
    h.mh_decimal_double.restype = C.c_double
    h.mh_tokens.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]
    h.mh_tokens.restype = C.c_int
    return h


@pytest.fixture(scope="module")
def libc():
    c = C.CDLL(None)
    c.strtod.argtypes = [C.c_char_p, C.c_void_p]
    c.strtod.restype = C.c_double
    c.atoi.argtypes = [C.c_char_p]
    c.atoi.restype = C.c_int
    return c


def f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def f64_bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def ref_float_bits(libc, s):
    d = libc.strtod(s, None)
    b = f64_bits(d)
    if (b & 0x7FF0000000000000) == 0x7FF0000000000000 and (b & 0xFFFFFFFFFFFFF):
        return 0xFFC00000 if b >> 63 else 0x7FC00000  # (float) of a NaN: its sign, the default payload
    with np.errstate(over="ignore"):
        return f32_bits(float(np.float32(np.float64(d))))


def decimal_tokens(rng, n):
    out = []
    for _ in range(n):
        nd = int(rng.choice([1, 2, 5, 9, 15, 16, 17, 18, 19, 20, 25, 40, 120]))
        digits = "".join(rng.choice(list("0123456789"), nd))
        if rng.random() < 0.3:
            digits = "0" * int(rng.integers(1, 30)) + digits
        if rng.random() < 0.6:
            k = int(rng.integers(0, len(digits) + 1))
            digits = digits[:k] + "." + digits[k:]
        s = ("-" if rng.random() < 0.3 else ("+" if rng.random() < 0.1 else "")) + digits
        r = rng.random()
        if r < 0.5:
            s += rng.choice(["e", "E"]) + str(int(rng.integers(-360, 330)))
        elif r < 0.6:
            s += "e" + rng.choice(["+", "-"]) + str(int(rng.integers(0, 40)))
        out.append(s)
    return out


def special_tokens():
    return [
        "0", "-0", "+0", "0.0", "-0.0e10", ".5", "5.", ".", "-", "+", "e5", "1e", "1e+", "1e-", "1.5e3x", "1,5",
        "inf", "-inf", "INF", "Infinity", "-infinity", "infx", "in", "nan", "-nan", "NaN", "nan(123)", "nanx", "na",
        "0x", "0x1", "-0x1p-1074", "0x1p-1075", "0x1.8p-1075", "0x1p-1076", "0x1.fffffffffffffp1023",
        "0x1.fffffffffffff8p1023", "0x1.00000000000008p0", "0x1.00000000000018p0", "0x.8p1", "0X1P+3", "0x1p",
        "0x123456789abcdef0123p-40", "0xg", "0x.", "1e-400", "1e400", "-1e400", "2.4703282292062327e-324",
        "2.4703282292062328e-324", "4.9406564584124654e-324", "2.2250738585072011e-308", "2.2250738585072014e-308",
        "1.7976931348623157e308", "1.7976931348623158e308", "1.7976931348623159e308", "9007199254740993",
        "9007199254740995", "1.00000000000000011102230246251565404236316680908203125",
        "1.00000000000000011102230246251565404236316680908203124", "0.1", "3.4028235677973366e38", "1.4e-45",
        "7.006492321624085e-46", "7.006492321624086e-46", "\n1.5", "\r2.5\r\n", "1.5\n", " 3", "\x0b4",
        "1" * 900 + "e-890", "0." + "0" * 500 + "1" * 400 + "e480", "123456789012345678901234567890",
    ]


def test_values_match_strtod(harness, libc):
    rng = np.random.default_rng(11)
    toks = special_tokens() + decimal_tokens(rng, 20000)
    slow_seen = 0
    for t in toks:
        b = t.encode()
        sl = C.c_int()
        got = f32_bits(harness.mh_value(b, len(b), C.byref(sl)))
        slow_seen += sl.value
        assert got == ref_float_bits(libc, b), (t, hex(got), hex(ref_float_bits(libc, b)))
    assert slow_seen > 1000  # the exact path was exercised, not only the fast one


def test_exact_decimal_conversion_matches_strtod(harness, libc):
    rng = np.random.default_rng(12)
    # Tokens with digits (those the exact path is given).
    specials = [x for x in special_tokens() if x[:1] in "0123456789.+-" and "x" not in x.lower() and any(c.isdigit() for c in x)]
    for t in decimal_tokens(rng, 20000) + specials:
        b = t.encode()
        got = f64_bits(harness.mh_decimal_double(b, len(b)))
        ref = f64_bits(libc.strtod(b, None))
        if (ref & 0x7FF0000000000000) == 0x7FF0000000000000 and (ref & 0xFFFFFFFFFFFFF):
            continue
        assert got == ref, (t, hex(got), hex(ref))


def test_atoi(harness, libc):
    rng = np.random.default_rng(13)
    toks = ["0", "-0", "+7", "2147483647", "2147483648", "-2147483648", "-2147483649", "4294967296",
            "9223372036854775807", "9223372036854775808", "-9223372036854775808", "-9223372036854775809",
            "99999999999999999999999", "-99999999999999999999999", "\n12", "\r\n", "", "x", "12x", "+-3", "-+3",
            "0012", "1e5", "\x0c9"]
    for _ in range(5000):
        nd = int(rng.integers(1, 25))
        toks.append(("-" if rng.random() < 0.4 else "") + "".join(rng.choice(list("0123456789"), nd)))
    for t in toks:
        b = t.encode()
        assert harness.mh_atoi(b, len(b)) == libc.atoi(b), t


def test_tokens_like_strtok(harness):
    def strtok(s):
        out, i = [], 0
        while True:
            while i < len(s) and s[i] in "\t, ":
                i += 1
            if i >= len(s) or s[i] == "\0":
                return out
            j = i
            while j < len(s) and s[j] not in "\t, \0":
                j += 1
            out.append((i, j - i))
            if j < len(s) and s[j] == "\0":
                return out
            i = j + 1
    for line in ["1 2 3\n", "1\t2,3\n", "  ,,1,,2\t\t3 \n", "1 2 \n", "\n", "   ", "1", "1 2\x003 4", ",,,",
                 "12 34 5.5e-3\r\n", "a b c d e f"]:
        b = line.encode()
        off = (C.c_int * 8)()
        ln = (C.c_int * 8)()
        k = harness.mh_tokens(b, len(b), off, ln, 8)
        assert [(off[i], ln[i]) for i in range(k)] == strtok(line), line
