// The double-float FP64 arithmetic's conversions (split_double and
// join_double in tope-fft_gb300/csrc/fft_arith.cuh) on the host, against
// exact references:
//   - split_double(v, delta): hi must be v * 2^-delta truncated to 24
//     significant bits and lo the next 23 bits, exactly (both built here from
//     v's bits with the 6 lowest mantissa bits cleared); values more than
//     2^100 below 2^delta, zeros and FP64 subnormals give (0, 0);
//   - join_double(hi, lo, delta): must equal (hi + lo) * 2^delta rounded to
//     the nearest double (ties to even), computed in binary128 (exact for the
//     sums that can matter) and rounded once, for normalised and
//     unnormalised pairs (|lo| up to 2^30 |hi|, opposite signs, cancellation,
//     powers of two with a negative remainder, FP32-subnormal parts, zeros)
//     and for deltas that reach FP64's subnormal and overflow ranges, on
//     both the fast path and the general one (join_double_any).
// Prints one line per check; exit status 0 when all pass.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "cuda_runtime.h"
#include "fft_arith.cuh"

using namespace tfft;

static uint64_t rng = 0x5EED5EEDull;
static uint64_t next()
{
    rng += 0x9E3779B97F4A7C15ull;
    uint64_t z = rng;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double dbits(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t bitsd(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static float fbits(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t bitsf(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static __float128 pow2q(int k)
{
    __float128 r = 1, b = k >= 0 ? 2 : 0.5;
    for (int n = k >= 0 ? k : -k; n; n >>= 1, b *= b)
        if (n & 1) r *= b;
    return r;
}

/* the join's exact reference: (hi + lo) * 2^delta rounded once to double */
static double join_ref(float hi, float lo, int delta)
{
    const __float128 q = ((__float128)hi + (__float128)lo) * pow2q(delta);
    return (double)q;
}

/* fast-path condition of join_double, restated: s >= 2^-71, finite, and a
 * result exponent inside FP64's normal range with a margin */
static bool fast_path(float hi, float lo, int delta)
{
    const float s = hi + lo;
    const int es = (int)((bitsf(s) >> 23) & 0xff);
    const int bexp = es + 896 + delta;
    return es >= 56 && es != 255 && bexp >= 2 && bexp <= 2045;
}

static long ulps(double a, double b)
{
    int64_t x = (int64_t)bitsd(a), y = (int64_t)bitsd(b);
    if (x < 0) x = INT64_MIN - x;
    if (y < 0) y = INT64_MIN - y;
    const int64_t d = x - y;
    return (long)(d < 0 ? -d : d);
}

static int check_split()
{
    long bad = 0, n = 0, zeros = 0;
    for (int it = 0; it < 2000000; it++) {
        const uint64_t r = next();
        const int delta = (int)(next() % 2000) - 1000;
        /* exponent E = e - 1023 - delta in -110 .. 40, some zeros/subnormals */
        int E = (int)(next() % 151) - 110;
        int e = E + 1023 + delta;
        if (it % 97 == 0) e = 0;
        if (e < 0 || e > 2046) continue;
        const uint64_t v = (r & 0x800fffffffffffffull) | ((uint64_t)e << 52);
        float hi, lo;
        split_double(dbits(v), delta, hi, lo);
        n++;
        float rh = 0.f, rl = 0.f;
        if (e != 0 && e - 1023 - delta >= -100) {
            const double w = dbits(v & ~0x3full); /* 6 lowest mantissa bits cleared */
            const double hw = dbits(bitsd(w) & ~0x1fffffffull); /* top 24 significant bits */
            /* scale by 2^-delta through the exponent field (exact, both normal as floats) */
            const int sh = -delta;
            rh = (float)(double)((__float128)hw * pow2q(sh));
            rl = (float)(double)(((__float128)w - (__float128)hw) * pow2q(sh));
        } else {
            zeros++;
        }
        if (bitsf(hi) != bitsf(rh) || bitsf(lo) != bitsf(rl)) {
            if (bad < 5)
                printf("  split mismatch v=%a delta=%d: (%a, %a) expected (%a, %a)\n", dbits(v), delta, hi, lo,
                       rh, rl);
            bad++;
        }
    }
    printf("%s split_double: %ld values (%ld to zero), %ld mismatches\n", bad ? "FAIL" : "ok  ", n, zeros, bad);
    return bad == 0;
}

static float rand_float(int emin, int emax)
{
    const int e = emin + (int)(next() % (uint64_t)(emax - emin + 1));
    const uint32_t m = (uint32_t)next() & 0x7fffffu;
    const uint32_t sgn = (uint32_t)(next() & 1) << 31;
    if (e <= 0) return fbits(sgn | m); /* FP32 subnormal */
    return fbits(sgn | ((uint32_t)e << 23) | m);
}

static int check_join()
{
    long n = 0, fast = 0, bad_fast = 0, bad_any = 0, any = 0;
    for (int it = 0; it < 4000000; it++) {
        float hi, lo;
        const int kind = it % 8;
        const int eh = 1 + (int)(next() % 254);
        hi = rand_float(eh, eh);
        switch (kind) {
        case 0: /* normalised: lo below an ulp of hi */
            lo = rand_float(eh - 24 - (int)(next() % 30), eh - 24);
            break;
        case 1: /* unnormalised, lo comparable to or larger than hi */
            lo = rand_float(eh - 10, eh + 30 > 254 ? 254 : eh + 30);
            break;
        case 2: /* cancellation */
            lo = -hi * (1.0f + ((float)(next() % 1000) - 500.f) * 0x1p-23f);
            break;
        case 3: /* a power of two with a remainder of the other sign */
            hi = fbits((bitsf(hi) & 0xff800000u));
            lo = fbits(((bitsf(hi) & 0x80000000u) ^ 0x80000000u) |
                       (bitsf(rand_float(eh - 40, eh - 24)) & 0x7fffffffu));
            break;
        case 4: /* tiny remainder, possibly an FP32 subnormal */
            lo = rand_float(-20, 30);
            break;
        case 5: /* zero parts */
            lo = 0.f;
            if (next() & 1) hi = 0.f, lo = rand_float(1, 254);
            break;
        case 6: /* ties: lo exactly half an FP64 unit of hi (after the shift to 53 bits) */
            lo = fbits((bitsf(hi) & 0x80000000u) | ((uint32_t)(eh > 53 ? eh - 53 : 1) << 23));
            break;
        default: /* both random over the whole range */
            lo = rand_float(0, 254);
            break;
        }
        /* deltas: mostly small, some near FP64's ends */
        int delta = (int)(next() % 64) - 32;
        if (it % 16 == 0) delta = (int)(next() % 2200) - 1100;
        if (!(hi == hi) || !(lo == lo) || __builtin_isinf(hi) || __builtin_isinf(lo) ||
            __builtin_isinf(hi + lo))
            continue;
        const double got = join_double(hi, lo, delta), ref = join_ref(hi, lo, delta);
        n++;
        const bool fp = fast_path(hi, lo, delta);
        const long d = ulps(got, ref);
        if (fp) {
            fast++;
            if (bitsd(got) != bitsd(ref)) {
                if (bad_fast < 5)
                    printf("  fast-path mismatch hi=%a lo=%a delta=%d: %a expected %a\n", hi, lo, delta, got, ref);
                bad_fast++;
            }
        } else {
            any++;
            if (bitsd(got) != bitsd(ref) && !(got == 0 && ref == 0)) {
                if (bad_any < 5)
                    printf("  general-path mismatch hi=%a lo=%a delta=%d: %a expected %a (%ld ulp)\n", hi, lo, delta,
                           got, ref, d);
                bad_any++;
            }
        }
    }
    printf("%s join_double: %ld pairs, %ld on the fast path (%ld not exact), %ld general (%ld not exact)\n",
           (bad_fast || bad_any) ? "FAIL" : "ok  ", n, fast, bad_fast, any, bad_any);
    return bad_fast == 0 && bad_any == 0;
}

int main()
{
    bool ok = check_split();
    ok = check_join() && ok;
    return ok ? 0 : 1;
}
