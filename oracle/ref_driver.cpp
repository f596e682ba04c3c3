/*
 * Host driver for the reference's own OpenCL kernels compiled as C++
 * (TEST INFRASTRUCTURE ONLY).  oracle/ref_build.sh rewrites the reference's
 * src/kernels{1,2,3}D.cl into oracle/_ref/k{1,2,3}d.cpp (a textual rewrite
 * at build time; nothing of the reference is committed) and compiles this
 * file into oracle/_ref/librefemu.so.
 *
 * Each NDRange runs as an OpenMP loop over work-items, in the reference's
 * host order:
 *   plan  src/fft1d.c:234-300, src/fft2d.c:201-317, src/fft3d.c:287-472
 *         (twiddle table, bit-reversal table)
 *   exec  src/fft1d.c:12-146, src/fft2d.c:12-199, src/fft3d.c:12-285
 *         (swap, stage loop per axis, divide on inverse)
 * so its results are what a CPU OpenCL runtime would produce for the same
 * kernels (up to the host libm's cos/sin).
 */
#include "ref_shim.h"

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <omp.h>

namespace refshim {
thread_local size_t gid[3];
thread_local size_t gsize[3];
}

namespace k1 {
#include "k1d.cpp"
}
namespace k2 {
#include "k2d.cpp"
}
namespace k3 {
#include "k3d.cpp"
}

/* Run f over a 3D NDRange (x fastest). */
template <class F>
static void ndrange(size_t gx, size_t gy, size_t gz, F f)
{
    int64_t total = (int64_t)gx * gy * gz;
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < total; t++) {
        refshim::gsize[0] = gx;
        refshim::gsize[1] = gy;
        refshim::gsize[2] = gz;
        refshim::gid[0] = (size_t)(t % gx);
        refshim::gid[1] = (size_t)((t / gx) % gy);
        refshim::gid[2] = (size_t)(t / ((int64_t)gx * gy));
        f();
    }
}

static int ilog2(int n)
{
    if (n < 1) return -1;
    int l = 0;
    while ((1 << l) < n) l++;
    return (1 << l) == n ? l : -1;
}

static int radix_of(int lg) { return lg % 3 == 0 ? 8 : lg % 2 == 0 ? 4 : 2; }
static int stages_of(int lg, int r) { return r == 8 ? lg / 3 : r == 4 ? lg / 2 : lg; }

extern "C" {

void refemu_set_threads(int n)
{
    if (n > 0) omp_set_num_threads(n);
}

int refemu_num_threads(void) { return omp_get_max_threads(); }

/* twid1D over n/4 work-items (src/fft1d.c:238-258) */
void refemu_twiddles(int n, double *tw)
{
    ndrange((size_t)(n / 4), 1, 1, [&] { k1::twid1D((double2 *)tw, n); });
}

/* reverse2 over n/2 work-items with the full log (src/fft1d.c:286-300) */
void refemu_bitrev(int log2n, int *rev)
{
    int n = 1 << log2n;
    ndrange((size_t)(n / 2), 1, 1, [&] { k1::reverse2(rev, log2n); });
}

/* reference DFT kernel (src/kernels1D.cl:549-573), out-of-place */
void refemu_dft(double *data, double *scratch, int n, int dir)
{
    ndrange((size_t)n, 1, 1, [&] { k1::DFT(data, scratch, n, (unsigned)dir); });
}

/* Full 1D plan + exec.  Returns 0, or -1 for an unsupported size. */
int refemu_exec_1d(double *d, int n, int dir)
{
    int lg = ilog2(n);
    if (n == 2) { /* host path, src/fft1d.c:16-28 */
        double hr = d[0], hi = d[1];
        d[0] += d[2]; d[1] += d[3];
        d[2] = hr - d[2]; d[3] = hi - d[3];
        if (dir == 0) { d[0] /= 2; d[2] /= 2; }
        return 0;
    }
    if (lg < 2) return -1;
    int r = radix_of(lg), S = stages_of(lg, r);
    int *rev = (int *)malloc(sizeof(int) * n);
    double *tw = (double *)malloc(sizeof(double) * 2 * (n / 4));
    ndrange((size_t)(n / 4), 1, 1, [&] { k1::twid1D((double2 *)tw, n); });
    ndrange((size_t)(n / 2), 1, 1, [&] { k1::reverse2(rev, lg); });
    ndrange((size_t)n, 1, 1, [&] { k1::swap1D(d, rev); });
    for (int s = 1; s <= S; s++) {
        if (r == 8) ndrange((size_t)(n / 8), 1, 1, [&] { k1::DIT8C2C(d, (double2 *)tw, n, s, dir); });
        else if (r == 4) ndrange((size_t)(n / 4), 1, 1, [&] { k1::DIT4C2C(d, (double2 *)tw, n, s, dir); });
        else ndrange((size_t)(n / 2), 1, 1, [&] { k1::DIT2C2C(d, (double2 *)tw, n, s, dir); });
    }
    if (dir == 0) ndrange((size_t)n, 1, 1, [&] { k1::divide1D((double2 *)d, n); });
    free(rev);
    free(tw);
    return 0;
}

struct AxisTables {
    int n, lg, r, S;
    int *rev;
    double *tw;
};

static AxisTables make_axis(int n, bool use2d)
{
    AxisTables a;
    a.n = n;
    a.lg = ilog2(n);
    a.r = radix_of(a.lg);
    a.S = stages_of(a.lg, a.r);
    a.rev = (int *)malloc(sizeof(int) * n);
    a.tw = (double *)malloc(sizeof(double) * 2 * (n / 4 + 1));
    if (use2d) {
        ndrange((size_t)(n / 4), 1, 1, [&] { k2::twiddles((double2 *)a.tw, n); });
        ndrange((size_t)(n / 2), 1, 1, [&] { k2::reverse(a.rev, a.lg); });
    } else {
        ndrange((size_t)(n / 4), 1, 1, [&] { k3::twiddles((double2 *)a.tw, n); });
        ndrange((size_t)(n / 2), 1, 1, [&] { k3::reverse(a.rev, a.lg); });
    }
    return a;
}

static void free_axis(AxisTables &a)
{
    free(a.rev);
    free(a.tw);
}

/* 2D: src/fft2d.c:136-199.  Axis lengths must be powers of two >= 4 (the
 * reference divides by n/4 == 0 for length 2). */
int refemu_exec_2d(double *d, int x, int y, int dir)
{
    if (ilog2(x) < 2 || ilog2(y) < 2) return -1;
    AxisTables ax = make_axis(x, true), ay = make_axis(y, true);
    /* X axis, type 1 */
    ndrange(x, y, 1, [&] { k2::swapkernel(d, x, y, ax.rev, ay.rev, 1); });
    for (int s = 1; s <= ax.S; s++) {
        if (ax.r == 8) ndrange(x / 8, y, 1, [&] { k2::DIT8C2C(d, (double2 *)ax.tw, x, y, s, dir, 1); });
        else if (ax.r == 4) ndrange(x / 4, y, 1, [&] { k2::DIT4C2C(d, (double2 *)ax.tw, x, y, s, dir, 1); });
        else ndrange(x / 2, y, 1, [&] { k2::DIT2C2C(d, (double2 *)ax.tw, x, y, s, dir, 1); });
    }
    /* Y axis, type 2 */
    ndrange(x, y, 1, [&] { k2::swapkernel(d, x, y, ax.rev, ay.rev, 2); });
    for (int s = 1; s <= ay.S; s++) {
        if (ay.r == 8) ndrange(x, y / 8, 1, [&] { k2::DIT8C2C(d, (double2 *)ay.tw, x, y, s, dir, 2); });
        else if (ay.r == 4) ndrange(x, y / 4, 1, [&] { k2::DIT4C2C(d, (double2 *)ay.tw, x, y, s, dir, 2); });
        else ndrange(x, y / 2, 1, [&] { k2::DIT2C2C(d, (double2 *)ay.tw, x, y, s, dir, 2); });
    }
    if (dir == 0) ndrange(x, y, 1, [&] { k2::divide((double2 *)d, x, y); });
    free_axis(ax);
    free_axis(ay);
    return 0;
}

/* 3D: src/fft3d.c:216-285. */
int refemu_exec_3d(double *d, int x, int y, int z, int dir)
{
    if (ilog2(x) < 2 || ilog2(y) < 2 || ilog2(z) < 2) return -1;
    AxisTables ax = make_axis(x, false), ay = make_axis(y, false), az = make_axis(z, false);
    AxisTables *axes[3] = {&ax, &ay, &az};
    for (int type = 1; type <= 3; type++) {
        AxisTables &a = *axes[type - 1];
        ndrange(x, y, z, [&] { k3::swapkernel(d, x, y, z, ax.rev, ay.rev, az.rev, type); });
        size_t gx = x, gy = y, gz = z;
        size_t *g = type == 1 ? &gx : type == 2 ? &gy : &gz;
        *g /= a.r;
        for (int s = 1; s <= a.S; s++) {
            if (a.r == 8) ndrange(gx, gy, gz, [&] { k3::DIT8C2C(d, (double2 *)a.tw, x, y, z, s, dir, type); });
            else if (a.r == 4) ndrange(gx, gy, gz, [&] { k3::DIT4C2C(d, (double2 *)a.tw, x, y, z, s, dir, type); });
            else ndrange(gx, gy, gz, [&] { k3::DIT2C2C(d, (double2 *)a.tw, x, y, z, s, dir, type); });
        }
    }
    if (dir == 0) ndrange(x, y, z, [&] { k3::divide((double2 *)d, x, y, z); });
    free_axis(ax);
    free_axis(ay);
    free_axis(az);
    return 0;
}

/* The 3D swap kernel alone along one axis (type 1..3): the bit-reversal
 * permutation, for bit-exact comparison of permutation kernels. */
int refemu_swap_3d(double *d, int x, int y, int z, int type)
{
    if (ilog2(x) < 1 || ilog2(y) < 1 || ilog2(z) < 1) return -1;
    int *rx = (int *)malloc(sizeof(int) * x), *ry = (int *)malloc(sizeof(int) * y),
        *rz = (int *)malloc(sizeof(int) * z);
    ndrange(x / 2, 1, 1, [&] { k3::reverse(rx, ilog2(x)); });
    ndrange(y / 2, 1, 1, [&] { k3::reverse(ry, ilog2(y)); });
    ndrange(z / 2, 1, 1, [&] { k3::reverse(rz, ilog2(z)); });
    ndrange(x, y, z, [&] { k3::swapkernel(d, x, y, z, rx, ry, rz, type); });
    free(rx);
    free(ry);
    free(rz);
    return 0;
}

} /* extern "C" */
