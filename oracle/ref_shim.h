/*
 * Host shim that lets the reference's OpenCL C kernel source compile as C++
 * (TEST INFRASTRUCTURE ONLY: used to build oracle/_ref/librefemu.so, the
 * reference's own kernels executed on host cores).
 *
 * Provides the OpenCL vector types the kernels use (double2/4/8/16 with
 * positional constructors and the .x/.y/.s0... members), the work-item query
 * functions backed by per-thread NDRange coordinates, and the math names.
 */
#ifndef TOPEFFT_REF_SHIM_H
#define TOPEFFT_REF_SHIM_H
#include <cmath>
#include <cstddef>

namespace refshim {
extern thread_local size_t gid[3];
extern thread_local size_t gsize[3];
}

static inline size_t get_global_id(int d) { return refshim::gid[d]; }
static inline size_t get_global_size(int d) { return refshim::gsize[d]; }

using std::cos;
using std::sin;
using std::pow;
using std::exp2;
using std::log2;

struct double2 {
    double x, y;
    double2() : x(0), y(0) {}
    double2(double a, double b) : x(a), y(b) {}
    double2 &operator/=(double s) { x /= s; y /= s; return *this; }
};

struct double4 {
    double x, y, z, w;
    double4() : x(0), y(0), z(0), w(0) {}
    double4(double a, double b, double c, double d) : x(a), y(b), z(c), w(d) {}
};

struct double8 {
    double s0, s1, s2, s3, s4, s5, s6, s7;
    double8() : s0(0), s1(0), s2(0), s3(0), s4(0), s5(0), s6(0), s7(0) {}
    double8(double a0, double a1, double a2, double a3, double a4, double a5,
            double a6, double a7)
        : s0(a0), s1(a1), s2(a2), s3(a3), s4(a4), s5(a5), s6(a6), s7(a7) {}
};

struct double16 {
    double s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf;
    double16() { s0 = s1 = s2 = s3 = s4 = s5 = s6 = s7 = s8 = s9 = sa = sb = sc = sd = se = sf = 0; }
    double16(double a0, double a1, double a2, double a3, double a4, double a5,
             double a6, double a7, double a8, double a9, double aa, double ab,
             double ac, double ad, double ae, double af)
        : s0(a0), s1(a1), s2(a2), s3(a3), s4(a4), s5(a5), s6(a6), s7(a7),
          s8(a8), s9(a9), sa(aa), sb(ab), sc(ac), sd(ad), se(ae), sf(af) {}
};

#endif
