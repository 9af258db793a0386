// df_host_check.cu -- the integer-pipe FP64 -> double-float split of df.cuh
// (f64_to_df) compiled for the host: hi must be the nearest float to v (ties
// away from zero), lo must be v - hi (exact in FP64) rounded to nearest
// float, and both flush to zero below 2^-126.  Random values over the FP32
// exponent range plus bit patterns at rounding ties and mantissa carries.
// Also the error bounds of the double-float operations (operator+, add_lazy,
// operator*) and of an 8-point butterfly of lazy sums.  Prints "split OK"
// and exits 0 when every value agrees.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "df.cuh"

using namespace topo;

static double ulp32(float h) {
    int e;
    frexpf(fabsf(h), &e);
    return ldexp(1.0, e - 24);
}

int main() {
    unsigned long long s = 0x2545F4914F6CDD1Dull;
    auto next = [&]() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return s;
    };
    long bad = 0, n = 0;
    auto check = [&](double v) {
        n++;
        const df d = f64_to_df(v);
        if (fabs(v) < ldexp(1.0, -126)) {
            if (d.hi != 0.0f || d.lo != 0.0f) bad++;
            return;
        }
        if (fabs(v) >= ldexp(1.0, 127)) return;
        const double r = v - (double)d.hi;  // exact
        const double hu = ulp32(d.hi);
        if (fabs(r) > hu / 2 || (fabs(r) == hu / 2 && fabs((double)d.hi) < fabs(v))) {
            bad++;
            return;
        }
        float lref = (float)r;
        if (fabs(r) < ldexp(1.0, -126)) lref = 0.0f;
        if (!(d.lo == lref)) bad++;
    };
    for (int i = 0; i < 2000000; i++) {
        const double m = (double)(next() >> 11) / 9007199254740992.0 * 2.0 - 1.0;
        check(ldexp(m, (int)(next() % 260) - 130));
    }
    for (int i = 0; i < 1000000; i++) {
        unsigned long long b = next();
        const unsigned long long e = 897 + next() % 254;
        b = (b & 0x800FFFFFFFFFFFFFull) | (e << 52);
        const int mode = (int)(next() % 4);
        if (mode == 0) b = (b & ~0x1FFFFFFFull) | 0x10000000ull;  // exact tie
        if (mode == 1) b |= 0x000FFFFFE0000000ull;                  // carry into the exponent
        if (mode == 2) b &= ~0x1FFFFFFFull;                         // lo = 0
        double v;
        memcpy(&v, &b, 8);
        check(v);
    }
    const double edges[] = {0.0, -0.0, 1.0, -1.0, 0.1, 1e-30, 1e30, 3.0000000000000004, 1.0000000596046448};
    for (double v : edges) check(v);
    printf("checked %ld, mismatches %ld\n", n, bad);

    // double-float arithmetic: the absolute error of operator+, add_lazy
    // (no renormalisation) and operator* stays within a few 2^-48 of the
    // operands, also for chains of lazy sums with cancellation (the mode
    // transforms); references in long double (64-bit significand)
    long arith_bad = 0;
    auto rnd = [&](int emin, int erange) {
        const double m = (double)(next() >> 11) / 9007199254740992.0 * 2.0 - 1.0;
        return ldexp(m, emin + (int)(next() % (unsigned)erange));
    };
    auto val = [](df a) { return (long double)a.hi + (long double)a.lo; };
    for (int i = 0; i < 200000; i++) {
        const df a = f64_to_df(rnd(-8, 16)), b = f64_to_df(rnd(-8, 16));
        const long double sa = fabsl(val(a)) + fabsl(val(b));
        const long double e1 = fabsl(val(a + b) - (val(a) + val(b))), e2 = fabsl(val(add_lazy(a, b)) - (val(a) + val(b)));
        if (e1 > ldexpl(sa, -46) || e2 > ldexpl(sa, -46)) arith_bad++;
        const long double e3 = fabsl(val(a * b) - val(a) * val(b));
        if (e3 > ldexpl(fabsl(val(a) * val(b)), -45)) arith_bad++;
        // an 8-point butterfly of lazy sums (mode transform) against the exact transform
        df v[8];
        long double w[8], mag = 0.0L;
        for (int L = 0; L < 8; L++) {
            v[L] = f64_to_df(1.0 + rnd(-20, 8));  // near-equal values: heavy cancellation
            w[L] = val(v[L]);
            mag += fabsl(w[L]);
        }
        for (int st = 0; st < 3; st++) {
            const int bit = 1 << st;
            for (int L = 0; L < 8; L++) {
                if (L & bit) continue;
                const df a0 = v[L], a1 = v[L | bit];
                v[L] = add_lazy(a0, a1);
                v[L | bit] = add_lazy(a1, -a0);
                const long double w0 = w[L], w1 = w[L | bit];
                w[L] = w0 + w1;
                w[L | bit] = w1 - w0;
            }
        }
        for (int L = 0; L < 8; L++)
            if (fabsl(val(v[L]) - w[L]) > ldexpl(mag, -45)) arith_bad++;
    }
    printf("double-float arithmetic mismatches %ld\n", arith_bad);
    if (bad == 0 && arith_bad == 0) printf("split OK\n");
    return (bad || arith_bad) ? 1 : 0;
}
