// mtx_parse.h -- the text rules of the reference's Matrix Market / .dat
// reader (make_CSR, ZIP:dbd/src/readInput.cpp:48-176) as functions that run
// on the device (k_mtx.cu) and on the host (a CPU test checks them against
// the C library's atoi and strtod):
//
//  * strtok(line, "\t, ") tokens;
//  * atoi: strtol's white space, sign and digits, saturation to the range of
//    a 64-bit long, truncation to int;
//  * (float)atof: the text correctly rounded to double (decimal, hexadecimal,
//    infinities, NaNs), then to float.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define MTX_HD __host__ __device__ __forceinline__
#else
#define MTX_HD inline
#endif

namespace dbd {
namespace mtx {

constexpr int kDecDigits = 800;    // digits the exact decimal conversion keeps

// ---- the few intrinsics, on either side --------------------------------

MTX_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

MTX_HD double bits_to_double(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
#endif
}

MTX_HD uint64_t double_bits(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    memcpy(&b, &d, sizeof(b));
    return b;
#endif
}

MTX_HD float bits_to_float(uint32_t b) {
#ifdef __CUDA_ARCH__
    return __int_as_float((int)b);
#else
    float f;
    memcpy(&f, &b, sizeof(f));
    return f;
#endif
}

// IEEE operations rounded to nearest (the host's defaults).
MTX_HD double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}

MTX_HD double div_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

// 10^e, 0 <= e <= 22: a product of exact powers of ten, each partial
// product a power of ten below 10^23 and so exact too.
MTX_HD double pow10_exact(int e) {
    double r = 1.0, p = 10.0;
    for (; e; e >>= 1, p = mul_rn(p, p))
        if (e & 1) r = mul_rn(r, p);
    return r;
}

// Bits of a power-of-two step for a decimal exponent dp = 1..8: 2^n <= 10^dp,
// so a scaling step never jumps past the target range.
MTX_HD int pow2_step(int dp) {
    switch (dp) {
        case 0: return 1;
        case 1: return 3;
        case 2: return 6;
        case 3: return 9;
        case 4: return 13;
        case 5: return 16;
        case 6: return 19;
        case 7: return 23;
        default: return 26;
    }
}


// ---- tokens and integers -------------------------------------------------

MTX_HD bool is_delim(char c) { return c == '\t' || c == ',' || c == ' '; }
// isspace() of the C locale: ' ', \t, \n, \v, \f, \r.
MTX_HD bool is_space(char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

// One strtok(piece, "\t, ") step over [s, e): the piece ends at e or at a
// NUL byte.  Returns false when no token is left.
MTX_HD bool next_tok(const char *&s, const char *e, const char *&ts, const char *&te) {
    while (s < e && *s && is_delim(*s)) ++s;
    if (s >= e || !*s) return false;
    ts = s;
    while (s < e && *s && !is_delim(*s)) ++s;
    te = s;
    if (s < e && *s) ++s;  // strtok overwrites the delimiter and resumes after it
    return true;
}

// atoi: strtol's white space, sign and digits; saturation to the range of a
// 64-bit long; truncation to int.
MTX_HD int32_t parse_atoi(const char *p, const char *e) {
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    uint64_t v = 0;
    bool big = false;
    for (; p < e && *p >= '0' && *p <= '9'; ++p) {
        const uint64_t d = (uint64_t)(*p - '0');
        if (!big && v > (0xFFFFFFFFFFFFFFFFull - d) / 10) big = true;
        if (!big) v = v * 10 + d;
    }
    int64_t r;
    if (neg) r = (big || v > 0x8000000000000000ull) ? INT64_MIN : (int64_t)(0 - v);
    else r = (big || v > 0x7FFFFFFFFFFFFFFFull) ? INT64_MAX : (int64_t)v;
    return (int32_t)(uint32_t)(uint64_t)r;
}

// ---- values: (float)strtod(token) ----------------------------------------

MTX_HD bool ieq(char c, char lower) { return c == lower || c == lower - 32; }

MTX_HD int hex_val(char c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'f') return c - 'a' + 10;
    if (c >= 'A' && c <= 'F') return c - 'A' + 10;
    return -1;
}

// m * 2^e2 (plus a nonzero tail below m's last bit when sticky) rounded to
// the nearest double, ties to even; subnormals and overflow included.
MTX_HD double binary_to_double(uint64_t m, bool sticky, int64_t e2, bool neg) {
    if (m == 0) return neg ? -0.0 : 0.0;
    const int lz = clz64(m);
    m <<= lz;
    e2 -= lz;
    const int64_t E = e2 + 63;  // exponent of the leading bit
    uint64_t bits;
    if (E > 1023) {
        bits = 0x7FF0000000000000ull;
    } else {
        // Bits to drop: 11 for a normal result, more below the normal range.
        const int64_t shift = E >= -1022 ? 11 : 11 + (-1022 - E);
        uint64_t keep, rem, half;
        if (shift <= 63) {
            keep = m >> shift;
            rem = m & ((1ull << shift) - 1);
            half = 1ull << (shift - 1);
        } else if (shift == 64) {
            keep = 0;
            rem = m;
            half = 1ull << 63;
        } else {
            keep = 0;
            rem = 0;  // below half of the smallest subnormal: rounds to zero
            half = 1;
            sticky = false;
        }
        if (rem > half || (rem == half && (sticky || (keep & 1)))) ++keep;
        // A normal result carries its rounding overflow into the exponent
        // (and into infinity); a subnormal one into the smallest normal.
        bits = E >= -1022 ? ((uint64_t)(E + 1023) << 52) + keep - (1ull << 52) : keep;
    }
    if (neg) bits |= 0x8000000000000000ull;
    return bits_to_double(bits);
}

// Result of the fast scan of one value token.
struct ValueScan {
    float v;
    bool slow;  // the exact decimal conversion must finish it
};

// Digits of a decimal mantissa (value = 0.d0 d1 ... * 10^dp), the exact
// conversion of Go's strconv package (decimal.go, "simple decimal
// conversion" as Nigel Tao describes it for Wuffs): the decimal is scaled by
// powers of two, exactly, until it lies in [1/2, 1), and 53 bits are then
// read off with round-half-even; digits beyond kDecDigits only mark the
// value as truncated (above a halfway point).
struct Decimal {
    uint8_t d[kDecDigits + 24];
    int nd;
    int dp;
    bool trunc;
};

MTX_HD void dec_trim(Decimal &a) {
    while (a.nd > 0 && a.d[a.nd - 1] == 0) --a.nd;
    if (a.nd == 0) a.dp = 0;
}

// a /= 2^k, k <= 60.
MTX_HD void dec_rshift(Decimal &a, int k) {
    int r = 0, w = 0;
    uint64_t n = 0;
    for (; (n >> k) == 0; ++r) {
        if (r >= a.nd) {
            if (n == 0) {
                a.nd = 0;
                return;
            }
            while ((n >> k) == 0) {
                n *= 10;
                ++r;
            }
            break;
        }
        n = n * 10 + a.d[r];
    }
    a.dp -= r - 1;
    const uint64_t mask = (1ull << k) - 1;
    for (; r < a.nd; ++r) {
        const uint64_t dig = n >> k;
        n &= mask;
        a.d[w++] = (uint8_t)dig;
        n = n * 10 + a.d[r];
    }
    while (n > 0) {
        const uint64_t dig = n >> k;
        n &= mask;
        if (w < kDecDigits) a.d[w++] = (uint8_t)dig;
        else if (dig > 0) a.trunc = true;
        n *= 10;
    }
    a.nd = w;
    dec_trim(a);
}

// a *= 2^k, k <= 60: digits are produced from the right into room kept
// behind the number (the product has at most 20 more digits), then moved
// to the front.
MTX_HD void dec_lshift(Decimal &a, int k) {
    int w = a.nd + 20;
    uint64_t n = 0;
    for (int r = a.nd - 1; r >= 0; --r) {
        n += (uint64_t)a.d[r] << k;
        const uint64_t q = n / 10;
        a.d[--w] = (uint8_t)(n - 10 * q);
        n = q;
    }
    while (n > 0) {
        const uint64_t q = n / 10;
        a.d[--w] = (uint8_t)(n - 10 * q);
        n = q;
    }
    const int len = a.nd + 20 - w;
    const int delta = len - a.nd;
    int keep = len < kDecDigits ? len : kDecDigits;
    for (int i = 0; i < keep; ++i) a.d[i] = a.d[w + i];
    for (int i = keep; i < len; ++i)
        if (a.d[w + i]) a.trunc = true;
    a.nd = keep;
    a.dp += delta;
    dec_trim(a);
}

MTX_HD void dec_shift(Decimal &a, int k) {
    if (a.nd == 0) return;
    for (; k > 60; k -= 60) dec_lshift(a, 60);
    for (; k < -60; k += 60) dec_rshift(a, 60);
    if (k > 0) dec_lshift(a, k);
    else if (k < 0) dec_rshift(a, -k);
}

MTX_HD bool dec_round_up(const Decimal &a, int nd) {
    if (nd < 0 || nd >= a.nd) return false;
    if (a.d[nd] == 5 && nd + 1 == a.nd) {  // exactly halfway: ties to even (or up past a truncated tail)
        if (a.trunc) return true;
        return nd > 0 && (a.d[nd - 1] & 1);
    }
    return a.d[nd] >= 5;
}

MTX_HD uint64_t dec_rounded_integer(const Decimal &a) {
    if (a.dp > 20) return 0xFFFFFFFFFFFFFFFFull;
    uint64_t n = 0;
    int i = 0;
    for (; i < a.dp && i < a.nd; ++i) n = n * 10 + a.d[i];
    for (; i < a.dp; ++i) n *= 10;
    if (dec_round_up(a, a.dp)) ++n;
    return n;
}

MTX_HD double dec_to_double(Decimal &a, bool neg) {
    const uint64_t signbit = neg ? 0x8000000000000000ull : 0;
    const uint64_t inf = 0x7FF0000000000000ull | signbit;
    if (a.nd == 0) return bits_to_double(signbit);
    if (a.dp > 310) return bits_to_double(inf);
    if (a.dp < -330) return bits_to_double(signbit);
    int exp = 0;
    while (a.dp > 0) {
        const int n = a.dp >= 9 ? 27 : pow2_step(a.dp);
        dec_shift(a, -n);
        exp += n;
    }
    // Up to [1/2, 1): a step of 2^n <= 10^-dp keeps the value below 1.
    while (a.dp < 0 || (a.dp == 0 && a.d[0] < 5)) {
        const int n = a.dp == 0 ? (a.d[0] < 2 ? 2 : 1) : (-a.dp >= 9 ? 27 : pow2_step(-a.dp));
        dec_shift(a, n);
        exp -= n;
    }
    --exp;  // [1/2, 1) to [1, 2)
    if (exp < -1022) {
        const int n = -1022 - exp;
        dec_shift(a, -n);
        exp += n;
    }
    if (exp + 1023 >= 2047) return bits_to_double(inf);
    dec_shift(a, 53);
    uint64_t mant = dec_rounded_integer(a);
    if (mant == (2ull << 52)) {
        mant >>= 1;
        ++exp;
        if (exp + 1023 >= 2047) return bits_to_double(inf);
    }
    if (!(mant & (1ull << 52))) exp = -1023;  // subnormal
    const uint64_t bits = (mant & ((1ull << 52) - 1)) | ((uint64_t)((exp + 1023) & 0x7FF) << 52) | signbit;
    return bits_to_double(bits);
}

MTX_HD float to_float(double d) {
    // (float) of a NaN keeps its sign with the default quiet NaN payload.
    const uint64_t b = double_bits(d);
    if ((b & 0x7FF0000000000000ull) == 0x7FF0000000000000ull && (b & 0x000FFFFFFFFFFFFFull))
        return bits_to_float((b >> 63) ? 0xFFC00000u : 0x7FC00000u);
#ifdef __CUDA_ARCH__
    return __double2float_rn(d);
#else
    return (float)d;
#endif
}

// The exponent digits after 'e'/'p' at q (a sign and at least one digit, or
// nothing is taken); saturates far beyond any finite result.
MTX_HD bool scan_exponent(const char *&q, const char *e, int64_t *ex) {
    const char *t = q + 1;
    bool neg = false;
    if (t < e && (*t == '+' || *t == '-')) neg = *t++ == '-';
    if (!(t < e && *t >= '0' && *t <= '9')) return false;
    int64_t v = 0;
    for (; t < e && *t >= '0' && *t <= '9'; ++t)
        if (v < 100000000) v = v * 10 + (*t - '0');
    *ex = neg ? -v : v;
    q = t;
    return true;
}

// (float)strtod of the token [p, e).  Decimal text with at most 19
// significant digits, a mantissa of at most 2^53 and a decimal exponent
// within +-22 is exact in one IEEE multiply or divide (Clinger's fast path);
// other decimal text is marked slow.  Hexadecimal text, infinities and NaNs
// are converted here.
MTX_HD ValueScan parse_value_fast(const char *p, const char *e) {
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    ValueScan r{0.f, false};
    if (p < e && ieq(*p, 'i')) {
        if (p + 2 < e && ieq(p[1], 'n') && ieq(p[2], 'f')) r.v = bits_to_float(neg ? 0xFF800000u : 0x7F800000u);
        return r;
    }
    if (p < e && ieq(*p, 'n')) {
        if (p + 2 < e && ieq(p[1], 'a') && ieq(p[2], 'n')) r.v = bits_to_float(neg ? 0xFFC00000u : 0x7FC00000u);
        return r;
    }
    if (p + 1 < e && p[0] == '0' && ieq(p[1], 'x')) {
        const char *q = p + 2;
        const bool digits = (q < e && hex_val(*q) >= 0) || (q + 1 < e && *q == '.' && hex_val(q[1]) >= 0);
        if (digits) {
            uint64_t m = 0;
            bool sticky = false, dot = false;
            int64_t e2 = 0;
            for (; q < e; ++q) {
                if (*q == '.') {
                    if (dot) break;
                    dot = true;
                    continue;
                }
                const int h = hex_val(*q);
                if (h < 0) break;
                if ((m >> 60) == 0) {
                    m = m * 16 + (uint64_t)h;
                    if (dot) e2 -= 4;
                } else {
                    if (h) sticky = true;
                    if (!dot) e2 += 4;
                }
            }
            int64_t ex = 0;
            if (q < e && ieq(*q, 'p') && scan_exponent(q, e, &ex)) e2 += ex;
            r.v = to_float(binary_to_double(m, sticky, e2, neg));
            return r;
        }
        // "0x" without hex digits reads as the 0 before the x.
        r.v = neg ? -0.f : 0.f;
        return r;
    }
    uint64_t m = 0;
    int nd = 0;
    int64_t e10 = 0;
    bool any = false, dot = false, dropped = false;
    const char *q = p;
    for (; q < e; ++q) {
        const char c = *q;
        if (c == '.') {
            if (dot) break;
            dot = true;
            continue;
        }
        if (c < '0' || c > '9') break;
        any = true;
        if (c == '0' && nd == 0) {
            if (dot) --e10;
            continue;
        }
        if (nd < 19) {
            m = m * 10 + (uint64_t)(c - '0');
            ++nd;
            if (dot) --e10;
        } else {
            if (c != '0') dropped = true;
            if (!dot) ++e10;
        }
    }
    if (!any) return r;  // no conversion: 0.0
    int64_t ex = 0;
    if (q < e && ieq(*q, 'e') && scan_exponent(q, e, &ex)) e10 += ex;
    if (m == 0) {
        r.v = neg ? -0.f : 0.f;
        return r;
    }
    if (!dropped && m <= (1ull << 53) && e10 >= -22 && e10 <= 22) {
        double d = (double)m;
        d = e10 >= 0 ? mul_rn(d, pow10_exact((int)e10)) : div_rn(d, pow10_exact((int)-e10));
        r.v = to_float(neg ? -d : d);
        return r;
    }
    r.slow = true;
    return r;
}

// The exact conversion of a decimal token (one the fast path marked slow).
MTX_HD float parse_value_exact(const char *p, const char *e, Decimal &a) {
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    a.nd = 0;
    a.dp = 0;
    a.trunc = false;
    bool dot = false, nonzero = false;
    const char *q = p;
    for (; q < e; ++q) {
        const char c = *q;
        if (c == '.') {
            if (dot) break;
            dot = true;
            continue;
        }
        if (c < '0' || c > '9') break;
        if (c == '0' && !nonzero) {
            if (dot) --a.dp;
            continue;
        }
        nonzero = true;
        if (!dot) ++a.dp;
        if (a.nd < kDecDigits) a.d[a.nd++] = (uint8_t)(c - '0');
        else if (c != '0') a.trunc = true;
    }
    int64_t ex = 0;
    if (q < e && ieq(*q, 'e') && scan_exponent(q, e, &ex)) {
        int64_t dp = (int64_t)a.dp + ex;
        dp = dp > 100000 ? 100000 : (dp < -100000 ? -100000 : dp);
        a.dp = (int)dp;
    }
    dec_trim(a);
    return to_float(dec_to_double(a, neg));
}


}  // namespace mtx
}  // namespace dbd
