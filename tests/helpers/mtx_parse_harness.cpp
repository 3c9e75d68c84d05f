// Host build of the Matrix Market text rules that the GPU conversion runs
// (dbd_gb300/csrc/mtx_parse.h), for tests/test_mtx_parse.py to compare with
// the C library's atoi and strtod.
#include "mtx_parse.h"

using namespace dbd::mtx;

extern "C" {

int mh_atoi(const char *s, int n) { return parse_atoi(s, s + n); }

// (float)atof by the path the device takes: the fast scan, then the exact
// conversion for the values it marks slow.  *slow tells which.
float mh_value(const char *s, int n, int *slow) {
    const ValueScan r = parse_value_fast(s, s + n);
    *slow = r.slow ? 1 : 0;
    if (!r.slow) return r.v;
    static Decimal a;
    return parse_value_exact(s, s + n, a);
}

// The exact decimal conversion to double alone (no float rounding), for any
// decimal text, so that it can be checked against strtod bit for bit.
double mh_decimal_double(const char *s, int n) {
    static Decimal a;
    const char *p = s, *e = s + n;
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
    return dec_to_double(a, neg);
}

// The tokens of one line piece, as strtok(piece, "\t, ") gives them: their
// offsets and lengths (at most max), and the count.
int mh_tokens(const char *s, int n, int *off, int *len, int max) {
    const char *p = s, *e = s + n, *ts, *te;
    int k = 0;
    while (k < max && next_tok(p, e, ts, te)) {
        off[k] = (int)(ts - s);
        len[k] = (int)(te - ts);
        ++k;
    }
    return k;
}

}  // extern "C"
