// Runs the auxiliary kernels (fft_aux.cu: twiddle and four-step tables,
// real-data steps, Bluestein pieces, the exact-index DFT) on the host through
// the stand-in header, via the library's own tfft_* entry points, and prints
// the error of each against a long-double evaluation of its definition:
//   case <i> <what> err=<error> tol=<gate>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fft_arith.cuh"
#include "tfft_abi.h"

thread_local uint3v threadIdx;
uint3v blockIdx;
dim3 blockDim, gridDim;
std::barrier<> *g_cta_bar;
std::barrier<> *g_warp_bar[32];
unsigned g_warp_val[32][32];
emu_graph *g_capture;

using LD = long double;
using CLD = std::complex<LD>;
static const LD PI = 3.141592653589793238462643383279502884L;

static CLD wpow(long long m, long long n)
{
    const LD a = -2.0L * PI * (LD)(m % n) / (LD)n;
    return CLD(cosl(a), sinl(a));
}
static CLD c(double2 v) { return CLD(v.x, v.y); }
static CLD c(float2 v) { return CLD(v.x, v.y); }
static CLD c(float4 v) { return CLD((LD)v.x + (LD)v.y, (LD)v.z + (LD)v.w); }

static std::vector<CLD> dft(const std::vector<CLD> &x, int dir)
{
    const long long n = (long long)x.size();
    std::vector<CLD> y(n);
    for (long long k = 0; k < n; k++) {
        CLD s = 0;
        for (long long j = 0; j < n; j++) {
            CLD w = wpow(j * k, n);
            s += x[j] * (dir ? w : std::conj(w));
        }
        y[k] = dir ? s : s / (LD)n;
    }
    return y;
}

static double rel(const std::vector<CLD> &a, const std::vector<CLD> &b)
{
    LD num = 0, den = 0;
    for (size_t i = 0; i < a.size(); i++) {
        num += std::norm(a[i] - b[i]);
        den += std::norm(b[i]);
    }
    return (double)sqrtl(num / den);
}

static void report(int id, const char *what, double err, double tol)
{
    std::printf("case %d %s err=%.3e tol=%.1e\n", id, what, err, tol);
}

int main(int argc, char **argv)
{
    const int only = argc > 1 ? std::atoi(argv[1]) : -1;
    auto want = [&](int i) { return only < 0 || only == i; };
    if (want(0)) { /* W_L^m for a length that is not a power of two (FP64) */
        const int L = 1000;
        std::vector<double2> t(L);
        tfft_table_any(t.data(), L, TFFT_ARITH_F64, nullptr);
        double e = 0;
        for (int m = 0; m < L; m++) e = std::max(e, (double)std::abs(c(t[m]) - wpow(m, L)));
        report(0, "table_any_f64", e, 2.3e-16);
    }
    if (want(1)) { /* the same as (hi, lo) float pairs */
        const int L = 1001;
        std::vector<float4> t(L);
        tfft_table_any(t.data(), L, TFFT_ARITH_DF64, nullptr);
        double e = 0;
        for (int m = 0; m < L; m++) e = std::max(e, (double)std::abs(c(t[m]) - wpow(m, L)));
        report(1, "table_any_df", e, 1e-14);
    }
    if (want(2)) { /* two-level four-step tables for N = 10^6 */
        const long long N = 1000000;
        const int shift = 10;
        std::vector<double2> lo(1 << shift), hi((N + (1 << shift) - 1) >> shift);
        tfft_fourstep_tables(hi.data(), lo.data(), N, shift, TFFT_ARITH_F64, nullptr);
        double e = 0;
        for (long long m = 0; m < N; m += 997)
            e = std::max(e, (double)std::abs(c(hi[m >> shift]) * c(lo[m & ((1 << shift) - 1)]) -
                                             wpow(m, N)));
        report(2, "fourstep_any", e, 5e-16);
    }
    for (int f32 = 0; f32 < 2; f32++) { /* R2C post-step and C2R pre-step */
        const int id = 3 + f32;
        if (!want(id)) continue;
        const long long n = 24, m = n / 2, rows = 3;
        int shift = 0;
        while ((1LL << (2 * shift)) < n) shift++;
        const long long nhi = (m >> shift) + 1;
        const int arith = f32 ? TFFT_ARITH_DF32 : TFFT_ARITH_F64;
        std::vector<float4> hi32(nhi), lo32(1 << shift);
        std::vector<double2> hi64(nhi), lo64(1 << shift);
        void *hi = f32 ? (void *)hi32.data() : (void *)hi64.data();
        void *lo = f32 ? (void *)lo32.data() : (void *)lo64.data();
        tfft_real_tables(hi, lo, n, shift, arith, nullptr);
        std::vector<CLD> want_spec, got_spec, want_z, got_z;
        std::vector<double2> z64(m * rows), x64((m + 1) * rows), zz64(m * rows);
        std::vector<float2> z32(m * rows), x32((m + 1) * rows), zz32(m * rows);
        for (long long r = 0; r < rows; r++) {
            std::vector<CLD> reals(n), packed(m);
            for (long long j = 0; j < n; j++) reals[j] = sin(0.7 * (double)(j + 5 * r) + 0.2);
            for (long long j = 0; j < m; j++) packed[j] = CLD(reals[2 * j].real(), reals[2 * j + 1].real());
            std::vector<CLD> Z = dft(packed, 1), X = dft(reals, 1);
            for (long long k = 0; k < m; k++) {
                z64[r * m + k] = make_double2((double)Z[k].real(), (double)Z[k].imag());
                z32[r * m + k] = make_float2((float)Z[k].real(), (float)Z[k].imag());
                want_z.push_back(CLD((double)Z[k].real(), (double)Z[k].imag()));
            }
            for (long long k = 0; k <= m; k++) want_spec.push_back(X[k]);
        }
        if (f32) tfft_r2c_post(z32.data(), x32.data(), hi, lo, shift, m, rows, arith, nullptr);
        else tfft_r2c_post(z64.data(), x64.data(), hi, lo, shift, m, rows, arith, nullptr);
        for (long long i = 0; i < (m + 1) * rows; i++) got_spec.push_back(f32 ? c(x32[i]) : c(x64[i]));
        const double e1 = rel(got_spec, want_spec);
        /* and back: the spectrum gives the packed transform again */
        if (f32) tfft_c2r_pre(x32.data(), zz32.data(), hi, lo, shift, m, rows, arith, nullptr);
        else tfft_c2r_pre(x64.data(), zz64.data(), hi, lo, shift, m, rows, arith, nullptr);
        for (long long i = 0; i < m * rows; i++) got_z.push_back(f32 ? c(zz32[i]) : c(zz64[i]));
        const double e2 = rel(got_z, want_z);
        report(id, f32 ? "real_steps_f32" : "real_steps_f64", std::max(e1, e2), f32 ? 2e-7 : 5e-16);
    }
    if (want(5)) { /* Bluestein pieces around an exact cyclic convolution */
        const long long n = 7, m = 16, rows = 2;
        std::vector<double2> chirp(n), b(m), x(n * rows), w(m * rows), out(n * rows);
        tfft_bluestein_tables(chirp.data(), b.data(), n, m, nullptr);
        std::vector<CLD> want_all, got_all;
        std::vector<CLD> B(m);
        for (long long k = 0; k < m; k++) B[k] = c(b[k]);
        std::vector<CLD> Bh = dft(B, 1);
        std::vector<double2> bh(m);
        for (long long k = 0; k < m; k++) bh[k] = make_double2((double)Bh[k].real(), (double)Bh[k].imag());
        for (long long i = 0; i < n * rows; i++) x[i] = make_double2(cos(1.3 * i), sin(0.4 * i * i));
        tfft_bluestein_pre(x.data(), chirp.data(), w.data(), n, m, 0, rows, nullptr);
        /* stand-in for the sub-plan: forward DFT, pointwise, inverse DFT */
        for (long long r = 0; r < rows; r++) {
            std::vector<CLD> v(m);
            for (long long k = 0; k < m; k++) v[k] = c(w[r * m + k]);
            v = dft(v, 1);
            for (long long k = 0; k < m; k++) w[r * m + k] = make_double2((double)v[k].real(), (double)v[k].imag());
        }
        tfft_pointwise(w.data(), bh.data(), m, rows, nullptr);
        for (long long r = 0; r < rows; r++) {
            std::vector<CLD> v(m);
            for (long long k = 0; k < m; k++) v[k] = c(w[r * m + k]);
            v = dft(v, 0);
            for (long long k = 0; k < m; k++) w[r * m + k] = make_double2((double)v[k].real(), (double)v[k].imag());
        }
        tfft_bluestein_post(w.data(), chirp.data(), out.data(), n, m, 0, 1.0, rows, nullptr);
        for (long long r = 0; r < rows; r++) {
            std::vector<CLD> v(n);
            for (long long k = 0; k < n; k++) v[k] = c(x[r * n + k]);
            v = dft(v, 1);
            for (long long k = 0; k < n; k++) {
                want_all.push_back(v[k]);
                got_all.push_back(c(out[r * n + k]));
            }
        }
        report(5, "bluestein_pieces", rel(got_all, want_all), 1e-15);
    }
    if (want(6)) { /* exact-index DFT kernel, forward and inverse, 3 rows of 7 */
        const int n = 7;
        const long long rows = 3;
        std::vector<double2> tw(n), x(n * rows), y(n * rows);
        tfft_dft_table(tw.data(), n, nullptr);
        for (long long i = 0; i < n * rows; i++) x[i] = make_double2(sin(0.9 * i), cos(0.2 * i + 1));
        double e = 0;
        for (int dir = 1; dir >= 0; dir--) {
            tfft_launch_dft(x.data(), y.data(), tw.data(), n, dir, rows, nullptr);
            std::vector<CLD> got, ref;
            for (long long r = 0; r < rows; r++) {
                std::vector<CLD> v(n);
                for (int k = 0; k < n; k++) v[k] = c(x[r * n + k]);
                v = dft(v, dir);
                for (int k = 0; k < n; k++) {
                    ref.push_back(v[k]);
                    got.push_back(c(y[r * n + k]));
                }
            }
            e = std::max(e, rel(got, ref));
        }
        report(6, "dft_kernel", e, 1e-15);
    }
    return 0;
}
