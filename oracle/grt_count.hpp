/*
 * grt_count.hpp -- an operation-counting complex type for the oracle.
 *
 * TEST INFRASTRUCTURE ONLY (the measurement of the roofline's algorithmic
 * work): oracle/op_count.cpp builds grt_oracle.c as C++ with GRTO_COUNT
 * defined, which replaces the oracle's C99 `double _Complex` by this type.
 * Every complex operation adds its conventional cost to a per-thread tally:
 *   complex multiply 6, add / subtract 2, divide 11 (also real / complex),
 *   real x complex 2, complex / real 2, real +- complex 1,
 *   exp, sqrt and log of a complex argument 20 each (counted where the
 *   oracle's c_exp / c_sqrt / c_log are called; their real internals are
 *   not counted again),
 *   negation, conjugation, real and imaginary parts, |z| (only compared,
 *   never combined) 0.
 * Real (double) arithmetic is not counted: in the per-(w,k) evaluation it is
 * limited to k^2 and the layer thicknesses.  Code between GRTO_COUNT_PAUSE
 * and GRTO_COUNT_RESUME is not counted (per-frequency quantities the oracle
 * recomputes at every wavenumber).  The values are exactly the FP64 oracle's.
 */
#ifndef GRT_COUNT_HPP_
#define GRT_COUNT_HPP_

#include <cmath>

struct grto_tally {
    long long flops;
    int paused;
};
extern thread_local grto_tally grto_cnt;
static inline void grto_count(long long n)
{
    if (!grto_cnt.paused) grto_cnt.flops += n;
}

struct cplx {
    double re, im;
    cplx() = default;
    constexpr cplx(double r) : re(r), im(0.0) {}
    constexpr cplx(double r, double i) : re(r), im(i) {}
};

static inline double creal(cplx a) { return a.re; }
static inline double cimag(cplx a) { return a.im; }
static inline cplx conj(cplx a) { return cplx(a.re, -a.im); }
static inline double cabs(cplx a) { return std::hypot(a.re, a.im); }

static inline bool operator==(cplx a, cplx b) { return a.re == b.re && a.im == b.im; }
static inline bool operator!=(cplx a, cplx b) { return !(a == b); }
static inline cplx operator-(cplx a) { return cplx(-a.re, -a.im); }
static inline cplx operator+(cplx a, cplx b) { grto_count(2); return cplx(a.re + b.re, a.im + b.im); }
static inline cplx operator-(cplx a, cplx b) { grto_count(2); return cplx(a.re - b.re, a.im - b.im); }
static inline cplx operator*(cplx a, cplx b)
{
    grto_count(6);
    return cplx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline cplx cdiv_(cplx a, cplx b)
{
    /* Smith's algorithm: the quotient the C99 type gives to rounding */
    if (std::fabs(b.re) >= std::fabs(b.im)) {
        const double t = b.im / b.re, d = b.re + b.im * t;
        return cplx((a.re + a.im * t) / d, (a.im - a.re * t) / d);
    }
    const double t = b.re / b.im, d = b.re * t + b.im;
    return cplx((a.re * t + a.im) / d, (a.im * t - a.re) / d);
}
static inline cplx operator/(cplx a, cplx b) { grto_count(11); return cdiv_(a, b); }

static inline cplx operator+(cplx a, double s) { grto_count(1); return cplx(a.re + s, a.im); }
static inline cplx operator+(double s, cplx a) { grto_count(1); return cplx(a.re + s, a.im); }
static inline cplx operator-(cplx a, double s) { grto_count(1); return cplx(a.re - s, a.im); }
static inline cplx operator-(double s, cplx a) { grto_count(1); return cplx(s - a.re, -a.im); }
static inline cplx operator*(cplx a, double s) { grto_count(2); return cplx(a.re * s, a.im * s); }
static inline cplx operator*(double s, cplx a) { grto_count(2); return cplx(a.re * s, a.im * s); }
static inline cplx operator/(cplx a, double s) { grto_count(2); return cplx(a.re / s, a.im / s); }
static inline cplx operator/(double s, cplx b) { grto_count(11); return cdiv_(cplx(s), b); }

static inline cplx &operator+=(cplx &a, cplx b) { return a = a + b; }
static inline cplx &operator-=(cplx &a, cplx b) { return a = a - b; }
static inline cplx &operator*=(cplx &a, cplx b) { return a = a * b; }
static inline cplx &operator/=(cplx &a, cplx b) { return a = a / b; }

/* the imaginary unit: i * x and i / x build a value without arithmetic */
struct grto_imag_unit {};
static const grto_imag_unit I = {};
static inline cplx operator*(double s, grto_imag_unit) { return cplx(0.0, s); }
static inline cplx operator*(grto_imag_unit, double s) { return cplx(0.0, s); }
static inline cplx operator/(grto_imag_unit, double s) { return cplx(0.0, 1.0 / s); }

#define GRTO_COUNT_PAUSE (grto_cnt.paused++)
#define GRTO_COUNT_RESUME (grto_cnt.paused--)
#define GRTO_COUNT_FN(n) grto_count(n)

#endif
