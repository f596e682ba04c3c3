// The tensor form's stage arithmetic (tope-fft_gb300/csrc/fft_tc_split.cuh)
// run on the host: the same split, matrix and join functions the kernel
// uses, with the tensor cores' products formed here (FP16 operands rounded
// with _Float16; D_hi summed exactly in double and required to be an integer
// below 2^24, so that FP32 accumulation in any order is exact; D_lo summed in
// FP32 in K order).  Single rows are checked against a long-double DFT-16 of
// the same (twiddled) rows; whole lines of 2^8 .. 2^12 points run the
// kernel's Stockham stages (index arithmetic of fft_tc.cuh stage16, its
// first stage of radix 2^(log2 L mod 4) through the pass code's double-float
// butterflies, and the renormalising read after it) and are checked against
// a long-double DFT, for uniform data, a 1e6 pulse and a pure tone (whose
// first-stage sums cancel exactly).  Prints one line per check; exit status
// 0 when all pass.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cuda_runtime.h"
#include "fft_pass.cuh"
#include "fft_tc_split.cuh"

using namespace tfft;

static double fp16(double v) { return (double)(_Float16)v; }

static double B[tcs::kNB][32][32]; /* [matrix][n][k], FP16 values */
static long double Fx[32][32];    /* exact F */

static uint64_t rng = 0x70E0F0F7ull;
static double urand() /* uniform [-1, 1) */
{
    rng += 0x9E3779B97F4A7C15ull;
    uint64_t z = rng;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return 2.0 * ((double)(z >> 11) * 0x1p-53) - 1.0;
}

static int fails = 0;
static void check(bool ok, const char *what, double v)
{
    std::printf("%s %s %.3e\n", ok ? "ok  " : "FAIL", what, v);
    if (!ok) fails++;
}

/* D_hi, D_lo of one row from its pieces X[3][32] (the kernel's products) */
static void tc_products(const double (&X)[3][32], float (&dh)[32], float (&dl)[32])
{
    for (int n = 0; n < 32; n++) {
        double hi = 0;
        for (int k = 0; k < 32; k++) hi += X[0][k] * B[0][n][k];
        float lo = 0.f;
        for (int q = 1; q < tcs::kNB; q++)
            for (int k = 0; k < 32; k++)
                lo = (float)((double)lo + X[tcs::prod_a(q)][k] * B[tcs::prod_b(q)][n][k]);
        dh[n] = (float)hi; /* exact: an integer below 2^24 */
        dl[n] = lo;
    }
}

struct dfc {
    df2 r, i;
};

/* one radix-16 stage of a line of L points after NS points were combined:
 * the kernel's stage16 on the host */
static void tc_line_stage(std::vector<dfc> &a, int L, int NS, const std::vector<float4> &tw,
                          bool renorm)
{
    const int TPL = L / 16;
    std::vector<dfc> out(L);
    for (int j = 0; j < TPL; j++) {
        dfc v[16];
        for (int q = 0; q < 16; q++) v[q] = a[j + q * TPL];
        if (renorm)
            for (int q = 0; q < 16; q++) {
                two_sum(v[q].r.h, v[q].r.l, v[q].r.h, v[q].r.l);
                two_sum(v[q].i.h, v[q].i.l, v[q].i.h, v[q].i.l);
            }
        float m = 0;
        for (int q = 0; q < 16; q++)
            m = std::fmax(m, std::fmax(std::fabs(v[q].r.h) + std::fabs(v[q].r.l),
                                       std::fabs(v[q].i.h) + std::fabs(v[q].i.l)));
        if (NS > 1) m *= 1.4375f;
        const int sexp = tcs::scale_exp(m);
        const float sc = tcs::pow2f(sexp);
        const int k = j & (NS - 1);
        double X[3][32];
        for (int r = 0; r < 16; r++) {
            float pr[3], pi[3];
            if (NS > 1 && r > 0)
                tcs::split_tw(v[r].r, v[r].i, tw[(size_t)(r * k) * (L / (NS * 16))], sc, pr, pi);
            else
                tcs::split_plain(v[r].r, v[r].i, sc, pr, pi);
            for (int i = 0; i < 3; i++) {
                X[i][2 * r] = fp16(pr[i]);
                X[i][2 * r + 1] = fp16(pi[i]);
            }
        }
        float dh[32], dl[32];
        tc_products(X, dh, dl);
        const float sh = tcs::pow2f(-sexp - tcs::kFB), sl = tcs::pow2f(-sexp - tcs::kFB - tcs::kLoShift);
        const int o = (j / NS) * NS * 16 + k;
        for (int r = 0; r < 16; r++)
            out[o + r * NS] = dfc{tcs::join_d(dh[2 * r], dl[2 * r], sh, sl),
                                  tcs::join_d(dh[2 * r + 1], dl[2 * r + 1], sh, sl)};
    }
    a.swap(out);
}

/* a whole line: first stage of radix 2^(log2 L mod 4) in long double (the
 * CUDA-core double-float stage), then the tensor stages; returns the
 * double-float result's rel-L2 against a long-double DFT of the input */
static double tc_line(int lg, int kind)
{
    const int L = 1 << lg;
    const long double PI = 3.14159265358979323846264338327950288L;
    std::vector<float4> tw(L);
    for (int m = 0; m < L; m++) {
        const long double c = cosl(2 * PI * m / L), s = -sinl(2 * PI * m / L);
        const float ch = (float)c, sh = (float)s;
        tw[m] = make_float4(ch, (float)(c - ch), sh, (float)(s - sh));
    }
    std::vector<float> xr(L), xi(L);
    for (int p = 0; p < L; p++) {
        xr[p] = (float)urand();
        xi[p] = (float)urand();
        if (kind == 1) xr[p] += (float)(1e6 * std::exp(-0.5 * (p - L / 2) * (p - L / 2) / 16.0));
        if (kind == 2) { /* a tone: its first-stage sums cancel exactly */
            const long double ang = 2 * PI * (long double)((p * 37) % L) / L;
            xr[p] = (float)cosl(ang);
            xi[p] = (float)sinl(ang);
        }
    }
    std::vector<dfc> a(L);
    for (int p = 0; p < L; p++) a[p] = dfc{df2{xr[p], 0.f}, df2{xi[p], 0.f}};
    const int lr0 = lg % 4;
    int ns = 1;
    if (lr0) {
        /* the kernel's first stage: the double-float butterflies of the
         * CUDA-core pass code (fft_pass.cuh), which leave sums unnormalised */
        const int R = 1 << lr0, m = L / R;
        std::vector<dfc> out(L);
        for (int j = 0; j < m; j++) {
            ArithDF32::C c[8];
            for (int q = 0; q < R; q++) {
                c[q].r = a[j + q * m].r;
                c[q].i = a[j + q * m].i;
            }
            if (R == 2) dft<ArithDF32, 2>(c);
            else if (R == 4) dft<ArithDF32, 4>(c);
            else dft<ArithDF32, 8>(c);
            for (int kk = 0; kk < R; kk++) out[j * R + kk] = dfc{c[kk].r, c[kk].i};
        }
        a.swap(out);
        ns = R;
    }
    for (bool first = true; ns < L; ns *= 16, first = false) tc_line_stage(a, L, ns, tw, first && lr0);
    long double e2 = 0, r2 = 0;
    for (int k = 0; k < L; k++) {
        long double sr = 0, si = 0;
        for (int p = 0; p < L; p++) {
            const long double ang = -2 * PI * (long double)(((long long)p * k) % L) / L;
            const long double c = cosl(ang), s = sinl(ang);
            sr += xr[p] * c - xi[p] * s;
            si += xr[p] * s + xi[p] * c;
        }
        const long double gr = (long double)a[k].r.h + a[k].r.l, gi = (long double)a[k].i.h + a[k].i.l;
        e2 += (gr - sr) * (gr - sr) + (gi - si) * (gi - si);
        r2 += sr * sr + si * si;
    }
    return (double)sqrtl(e2 / r2);
}

int main()
{
    /* matrices */
    bool exact = true, normal = true;
    int nonzero_sub = 0;
    for (int n = 0; n < 32; n++)
        for (int k = 0; k < 32; k++) {
            const long double ang = 2.0L * 3.14159265358979323846264338327950288L *
                                    (long double)(((n >> 1) * (k >> 1)) & 15) / 16.0L;
            const double c = (double)cosl(ang), s = (double)sinl(ang);
            Fx[n][k] = (n & 1) == 0 ? ((k & 1) ? sinl(ang) : cosl(ang))
                                    : ((k & 1) ? cosl(ang) : -sinl(ang));
            double b[tcs::kNB];
            tcs::b_values(tcs::dft16_entry(n, k, c, s), b);
            for (int m = 0; m < tcs::kNB; m++) {
                B[m][n][k] = fp16(b[m]);
                if (m < 5 && B[m][n][k] != b[m]) exact = false;
                if (m < 5 && b[m] != 0 && std::fabs(b[m]) < 0x1p-14) normal = false;
                if (m == 5 && b[m] != 0 && std::fabs(b[m]) < 0x1p-14) nonzero_sub++;
            }
        }
    check(exact, "B0..B4 exact in FP16", 0);
    check(normal, "B0..B4 free of FP16 subnormals", 0);
    double rowsum = 0;
    for (int n = 0; n < 32; n++) {
        double r = 0;
        for (int k = 0; k < 32; k++) r += std::fabs(B[0][n][k]);
        rowsum = std::fmax(rowsum, r);
    }
    check(513.0 * rowsum < 0x1p24, "513 * max row sum of |F0| below 2^24", 513.0 * rowsum);
    /* the represented matrix (pieces recombined) against F */
    double ferr = 0;
    for (int n = 0; n < 32; n++)
        for (int k = 0; k < 32; k++) {
            /* F 2^10 = F0 + 2^-11 F1 + 2^-22 F2, B2 = F1 2^-3, B5 = F2 2^-14 */
            const long double f =
                ((long double)B[0][n][k] + (long double)B[2][n][k] * 0x1p-8L +
                 (long double)B[5][n][k] * 0x1p-8L) / 1024.0L;
            ferr = std::fmax(ferr, (double)fabsl(f - Fx[n][k]));
        }
    check(ferr < 0x1p-33, "F0 + F1 + F2 represent F within 2^-33", ferr);

    /* rows: uniform, wide dynamic range, a spike, zeros; plain and twiddled */
    double worst = 0, worst_tw = 0;
    double max_x0 = 0, max_x1 = 0, max_dhi = 0;
    bool ints = true, dhi_int = true;
    for (int row = 0; row < 20000; row++) {
        const int kind = row % 5;
        const bool tw = (row / 5) % 2;
        df2 xr[16], xi[16];
        for (int p = 0; p < 16; p++) {
            double a = urand(), b = urand();
            if (kind == 1) { a *= std::ldexp(1.0, (int)(urand() * 60)); b *= std::ldexp(1.0, (int)(urand() * 60)); }
            if (kind == 2) { if (p == 5) a = 1e6; }
            if (kind == 3) { a *= 1e-30; b *= 1e-30; }
            if (kind == 4 && p > 2) { a = 0; b = 0; }
            /* a double-float value: hi FP32, lo the FP32 of the rest */
            const float ah = (float)a, bh = (float)b;
            xr[p] = df2{ah, (float)((a - ah) * (kind == 0 ? 1.0 : 0.0))};
            xi[p] = df2{bh, (float)((b - bh) * (kind == 0 ? 1.0 : 0.0))};
        }
        /* twiddles W^(p t) of a 256-point table, FP64-accurate (hi, lo) */
        float4 w[16];
        long double wre[16], wim[16];
        const int tt = 1 + row % 97;
        for (int p = 0; p < 16; p++) {
            const long double ang = -2.0L * 3.14159265358979323846264338327950288L *
                                    (long double)((p * tt) % 256) / 256.0L;
            wre[p] = cosl(ang);
            wim[p] = sinl(ang);
            const float rh = (float)wre[p], ih = (float)wim[p];
            w[p] = make_float4(rh, (float)(wre[p] - rh), ih, (float)(wim[p] - ih));
        }
        /* the kernel's bound and scale */
        float m = 0;
        for (int p = 0; p < 16; p++)
            m = std::fmax(m, std::fmax(std::fabs(xr[p].h) + std::fabs(xr[p].l),
                                       std::fabs(xi[p].h) + std::fabs(xi[p].l)));
        if (tw) m *= 1.4375f;
        const int sexp = tcs::scale_exp(m);
        const float sc = tcs::pow2f(sexp);
        double X[3][32];
        long double v[32];
        for (int p = 0; p < 16; p++) {
            float pr[3], pi[3];
            const long double vr = (long double)xr[p].h + xr[p].l, vi = (long double)xi[p].h + xi[p].l;
            if (tw && p > 0) {
                tcs::split_tw(xr[p], xi[p], w[p], sc, pr, pi);
                const long double wr = (long double)w[p].x + w[p].y, wi = (long double)w[p].z + w[p].w;
                v[2 * p] = vr * wr - vi * wi;
                v[2 * p + 1] = vr * wi + vi * wr;
            } else {
                tcs::split_plain(xr[p], xi[p], sc, pr, pi);
                v[2 * p] = vr;
                v[2 * p + 1] = vi;
            }
            for (int i = 0; i < 3; i++) {
                X[i][2 * p] = fp16(pr[i]);
                X[i][2 * p + 1] = fp16(pi[i]);
            }
            for (int i = 0; i < 2; i++)
                if (X[i][2 * p] != pr[i] || X[i][2 * p + 1] != pi[i] ||
                    X[i][2 * p] != std::rint(X[i][2 * p]) || X[i][2 * p + 1] != std::rint(X[i][2 * p + 1]))
                    ints = false;
            max_x0 = std::fmax(max_x0, std::fmax(std::fabs(pr[0]), std::fabs(pi[0])));
            max_x1 = std::fmax(max_x1, std::fmax(std::fabs(pr[1]), std::fabs(pi[1])));
        }
        /* the products of the tensor stage */
        double err2 = 0, ref2 = 0;
        for (int n = 0; n < 32; n++) {
            double dhi = 0, dabs = 0;
            for (int k = 0; k < 32; k++) {
                dhi += X[0][k] * B[0][n][k];
                dabs += std::fabs(X[0][k] * B[0][n][k]);
            }
            if (dhi != std::rint(dhi) || dabs >= 0x1p24) dhi_int = false;
            max_dhi = std::fmax(max_dhi, dabs);
            float dlo = 0.f;
            for (int q = 1; q < tcs::kNB; q++)
                for (int k = 0; k < 32; k++)
                    dlo = (float)((double)dlo + X[tcs::prod_a(q)][k] * B[tcs::prod_b(q)][n][k]);
            const long double y = ((long double)dhi * tcs::pow2f(-sexp - tcs::kFB) +
                                   (long double)dlo * tcs::pow2f(-sexp - tcs::kFB - tcs::kLoShift));
            long double yx = 0;
            for (int k = 0; k < 32; k++) yx += Fx[n][k] * v[k];
            err2 += (double)((y - yx) * (y - yx));
            ref2 += (double)(yx * yx);
        }
        const double e = ref2 > 0 ? std::sqrt(err2 / ref2) : std::sqrt(err2);
        if (tw) worst_tw = std::fmax(worst_tw, e);
        else worst = std::fmax(worst, e);
    }
    check(ints, "x0, x1 are FP16 integers", 0);
    check(max_x0 <= 513, "|x0| <= 513", max_x0);
    check(max_x1 <= 2048, "|x1| <= 2048", max_x1);
    check(dhi_int, "D_hi an integer sum below 2^24 (exact in FP32)", max_dhi);
    check(worst < 2e-9, "worst row rel-L2, no twiddle", worst);
    check(worst_tw < 2e-9, "worst row rel-L2, twiddled", worst_tw);
    /* whole lines: two tensor stages after a first stage of radix 1, 2, 4
     * or 8 (256 .. 2048 points) and three (4096), uniform, with a 1e6 pulse
     * and a pure tone */
    const int lgs[5] = {8, 9, 10, 11, 12};
    for (int li = 0; li < 5; li++)
        for (int kind = 0; kind < 3; kind++) {
            char what[96];
            std::snprintf(what, sizeof what, "line 2^%d %s: rel-L2 before the FP32 store",
                          lgs[li], kind == 2 ? "one tone" : kind ? "with 1e6 pulse" : "uniform");
            const double e = tc_line(lgs[li], kind);
            check(e < 1e-8, what, e);
        }
    std::printf("B5 entries below the FP16 normal range: %d\n", nonzero_sub);
    return fails ? 1 : 0;
}
