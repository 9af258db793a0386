// df_host_check.cu -- the integer-pipe FP64 -> double-float split of df.cuh
// (f64_to_df) compiled for the host: hi must be the nearest float to v (ties
// away from zero), lo must be v - hi (exact in FP64) rounded to nearest
// float, and both flush to zero below 2^-126.  Random values over the FP32
// exponent range plus bit patterns at rounding ties and mantissa carries.
// Prints "split OK" and exits 0 when every value agrees.
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
    if (bad == 0) printf("split OK\n");
    return bad ? 1 : 0;
}
