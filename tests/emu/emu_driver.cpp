// Runs the library's pass kernels (fft_pass.cuh, fft_mixed.cuh) on the host,
// one std::thread per CUDA thread of a CTA and one CTA after another, through
// the stand-in header tests/emu/cuda_runtime.h.  Each case transforms a few
// lines and prints the relative L2 error against a long-double DFT of the
// same lines, with the same conjugations, scale and four-step factor:
//   case <i> <kernel> rel=<error> tol=<gate>
#include "fft_mixed.cuh"

#include <complex>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <thread>
#include <vector>

thread_local uint3v threadIdx;
uint3v blockIdx;
std::barrier<> *g_cta_bar;
std::barrier<> *g_warp_bar[32];
unsigned g_warp_val[32][32];
emu_graph *g_capture;
namespace tfft {
alignas(16) unsigned char smem_raw[1 << 18];
}

using LD = long double;
using CLD = std::complex<LD>;

static CLD wpow(long long m, long long n)
{
    const LD a = -2.0L * 3.141592653589793238462643383279502884L * (LD)(m % n) / (LD)n;
    return CLD(cosl(a), sinl(a));
}

#if defined(__SANITIZE_ADDRESS__)
#include <sanitizer/asan_interface.h>
#endif

/* bytes of dynamic shared memory the current launch asked for: under
 * AddressSanitizer the rest of the buffer is poisoned, so an access past the
 * launch's allocation is reported */
static size_t g_smem_bytes = sizeof(tfft::smem_raw);

static void smem_limit(size_t bytes)
{
    g_smem_bytes = bytes;
#if defined(__SANITIZE_ADDRESS__)
    __asan_unpoison_memory_region(tfft::smem_raw, sizeof(tfft::smem_raw));
    __asan_poison_memory_region(tfft::smem_raw + bytes, sizeof(tfft::smem_raw) - bytes);
#endif
}

/* one CTA at a time, all of its threads at once */
template <class K>
static void run_grid(K kernel, const tfft_pass &p, long long blocks, int threads)
{
    for (long long blk = 0; blk < blocks; blk++) {
        blockIdx.x = (unsigned)blk;
        std::barrier<> cta(threads);
        g_cta_bar = &cta;
        std::vector<std::unique_ptr<std::barrier<>>> wb;
        for (int w = 0; w * 32 < threads; w++) {
            wb.emplace_back(new std::barrier<>(std::min(32, threads - 32 * w)));
            g_warp_bar[w] = wb.back().get();
        }
        std::vector<std::thread> th;
        for (int x = 0; x < threads; x++)
            th.emplace_back([&, x] {
                threadIdx.x = (unsigned)x;
                kernel(p);
            });
        for (auto &t : th) t.join();
    }
}

/* table entries in an arithmetic's layout: double2, or (hi, lo) float pairs */
static void put(double2 *t, long long i, CLD w) { t[i] = make_double2((double)w.real(), (double)w.imag()); }
static void put(float4 *t, long long i, CLD w)
{
    const float rh = (float)w.real(), ih = (float)w.imag();
    t[i] = make_float4(rh, (float)(w.real() - rh), ih, (float)(w.imag() - ih));
}
static CLD get(double2 v) { return CLD(v.x, v.y); }
static CLD get(float2 v) { return CLD(v.x, v.y); }
static void set(double2 &v, CLD c) { v = make_double2((double)c.real(), (double)c.imag()); }
static void set(float2 &v, CLD c) { v = make_float2((float)c.real(), (float)c.imag()); }

struct Spec {
    long long L, B, lines;
    bool rows;          /* elements of a line contiguous (else lines contiguous) */
    int post;           /* 0 none, 1 two-level table, 2 whole table */
    bool conj;          /* conj on load and store with scale 1/L: an inverse */
    double magnitude;   /* input scale */
    long long n1 = 1;   /* groups of `lines` lines along the grid's second dimension */
    int level = 0;      /* four-step factor from the line index (0) or the group (1),
                           as in the middle pass of a three-pass line */
};

template <class A, class Launch>
static double run_case(const Spec &s, Launch launch)
{
    using Store = typename A::Store;
    using TW = typename A::TW;
    const long long L = s.L, lines = s.lines, grp = L * lines, tot = grp * s.n1;
    const long long N = L * (s.level ? s.n1 : lines); /* t * k < N for every factor */
    std::vector<Store> in(tot), out(tot);
    std::vector<CLD> x(tot);
    for (long long e = 0; e < tot; e++) {
        const double re = s.magnitude * sin(0.37 * (double)e + 1.0);
        const double im = s.magnitude * cos(0.11 * (double)e * (double)e + 0.3);
        set(in[e], CLD(re, im));
        x[e] = get(in[e]); /* the stored (possibly FP32-rounded) input */
    }
    std::vector<TW> tw(L), hi, lo, whole;
    for (long long m = 0; m < L; m++) put(tw.data(), m, wpow(m, L));
    tfft_pass p;
    std::memset(&p, 0, sizeof p);
    p.b_tile = (int)s.B;
    p.arith = A::kId;
    p.scale = s.conj ? 1.0 / (double)L : 1.0;
    p.conj_in = p.conj_out = s.conj;
    p.in = in.data();
    p.out = out.data();
    p.n[0] = lines;
    p.n[1] = s.n1;
    p.n[2] = 1;
    p.is[1] = p.os[1] = grp;
    p.is[0] = p.os[0] = s.rows ? L : 1;
    p.ies = p.oes = s.rows ? 1 : lines;
    p.tw = tw.data();
    int shift = 0;
    if (s.post) {
        p.post_tw = 1;
        p.tw_level = s.level;
        p.tw_n = N;
        if (s.post == 2) {
            whole.resize(N);
            for (long long m = 0; m < N; m++) put(whole.data(), m, wpow(m, N));
            p.tw_hi = whole.data();
            p.tw_lo = nullptr;
        } else {
            int lg = 0;
            while ((1LL << lg) < N) lg++;
            shift = (lg + 1) / 2;
            const long long nlo = 1LL << shift, nhi = (N + nlo - 1) >> shift;
            lo.resize(nlo);
            hi.resize(nhi);
            for (long long i = 0; i < nlo; i++) put(lo.data(), i, wpow(i, N));
            for (long long h = 0; h < nhi; h++) put(hi.data(), h, wpow(h << shift, N));
            p.tw_shift = shift;
            p.tw_hi = hi.data();
            p.tw_lo = lo.data();
        }
    }
    launch(p);
    LD num = 0, den = 0;
    for (long long h = 0; h < s.n1; h++)
        for (long long g = 0; g < lines; g++)
            for (long long k = 0; k < L; k++) {
                CLD acc = 0;
                for (long long j = 0; j < L; j++) {
                    CLD v = x[h * grp + (s.rows ? g * L + j : j * lines + g)];
                    if (s.conj) v = std::conj(v);
                    acc += v * wpow(j * k, L);
                }
                if (s.post) acc *= wpow((s.level ? h : g) * k, N);
                if (s.conj) acc = std::conj(acc) / (LD)L;
                const CLD got = get(out[h * grp + (s.rows ? g * L + k : k * lines + g)]);
                num += std::norm(got - acc);
                den += std::norm(acc);
            }
    return (double)sqrtl(num / den);
}

template <class A>
static void mixed(int id, const Spec &s, double tol)
{
    unsigned char rad[TFFT_MAX_RADICES];
    int nr = 0;
    long long t = s.L;
    while (t % 8 == 0) { rad[nr++] = 8; t /= 8; }
    if (t % 4 == 0) { rad[nr++] = 4; t /= 4; }
    if (t % 2 == 0) { rad[nr++] = 2; t /= 2; }
    for (int pr : {3, 5, 7, 11, 13})
        while (t % pr == 0) { rad[nr++] = (unsigned char)pr; t /= pr; }
    const double e = run_case<A>(s, [&](tfft_pass &p) {
        p.len = (int)s.L;
        p.nrad = nr;
        std::memcpy(p.radix, rad, nr);
        smem_limit(tfft::mixed_smem_bytes((int)(s.L * s.B), (int)sizeof(typename A::S)));
        run_grid(tfft::mixed_kernel<A>, p, (s.lines + s.B - 1) / s.B * s.n1, tfft::kMixedThreads);
    });
    std::printf("case %d mixed_kernel<%d> L=%lld B=%lld rel=%.3e tol=%.1e\n", id, A::kId, s.L, s.B,
                e, tol);
}

template <class A, int LOG_L, int B, int EPT>
static void pass(int id, const Spec &s, double tol)
{
    const double e = run_case<A>(s, [&](tfft_pass &p) {
        p.log_l = LOG_L;
        p.ept = EPT == 16 ? 0 : EPT;
        smem_limit(tfft::pass_smem_bytes<A, LOG_L, B, EPT>());
        run_grid(tfft::pass_kernel<A, LOG_L, B, EPT>, p, (s.lines + B - 1) / B * s.n1,
                 tfft::Shape<LOG_L, EPT>::TPL * B);
    });
    std::printf("case %d pass_kernel<%d,%d,%d,%d> rel=%.3e tol=%.1e\n", id, A::kId, LOG_L, B, EPT,
                e, tol);
}

int main(int argc, char **argv)
{
    using namespace tfft;
    const int only = argc > 1 ? std::atoi(argv[1]) : -1;
    auto want = [&](int i) { return only < 0 || only == i; };
    if (want(0)) mixed<ArithF64>(0, {400, 4, 30, true, 0, false, 1.0}, 1e-14);
    if (want(1)) mixed<ArithF64>(1, {400, 4, 30, false, 0, false, 1.0}, 1e-14);
    if (want(2)) mixed<ArithF64>(2, {1000, 2, 8, false, 1, false, 1.0}, 1e-14);
    if (want(3)) mixed<ArithF64>(3, {1001, 1, 2, true, 0, true, 1.0}, 1e-14);
    if (want(4)) mixed<ArithDF64>(4, {250, 8, 16, true, 0, false, 1e-280}, 1e-13);
    if (want(5)) mixed<ArithF32>(5, {60, 32, 64, true, 0, false, 1.0}, 3e-7);
    if (want(6)) mixed<ArithDF32>(6, {125, 16, 20, false, 2, false, 1.0}, 1e-7);
    if (want(7)) pass<ArithF64, 6, 2, 4>(7, {64, 2, 64, false, 2, false, 1.0}, 1e-14);
    if (want(8)) pass<ArithF64, 10, 4, 16>(8, {1024, 4, 8, true, 0, false, 1.0}, 1e-14);
    if (want(9)) pass<ArithDF64, 8, 8, 16>(9, {256, 8, 16, false, 1, false, 1.0}, 1e-13);
    if (want(10)) pass<ArithF32, 9, 8, 16>(10, {512, 8, 16, true, 0, false, 1.0}, 3e-7);
    if (want(11)) pass<ArithDF64, 12, 2, 16>(11, {4096, 2, 2, true, 0, true, 1e300}, 1e-13);
    /* the middle pass of a three-pass line: 3 groups, factor W_N^(group * k) */
    if (want(12)) mixed<ArithF64>(12, {243, 2, 3, false, 1, false, 1.0, 3, 1}, 1e-14);
    if (want(13)) mixed<ArithDF64>(13, {81, 4, 5, true, 2, true, 1.0, 3, 1}, 1e-13);
    if (want(14)) pass<ArithF64, 8, 2, 16>(14, {256, 2, 3, false, 1, false, 1.0, 4, 1}, 1e-14);
    /* double-float lines of three and four stages: the stages after the
     * first run as a loop with the stage index at run time */
    if (want(15)) pass<ArithDF32, 9, 8, 16>(15, {512, 8, 16, true, 1, false, 1.0}, 1e-7);
    if (want(16)) pass<ArithDF64, 11, 2, 16>(16, {2048, 2, 4, false, 0, true, 1.0}, 1e-13);
    return 0;
}
