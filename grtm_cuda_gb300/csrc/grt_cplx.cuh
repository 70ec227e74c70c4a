// grt_cplx.cuh -- complex scalars and 2x2 complex matrices for the GRT
// kernels, templated on the real type (float for the product path, double for
// the FP64 GPU check path).  Plain structs, all in registers.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#define GRT_HD __host__ __device__ __forceinline__

namespace grt {

template <typename R>
struct C {
    R x, y;
};

template <typename R> GRT_HD C<R> mk(R x, R y) { return C<R>{x, y}; }
template <typename R> GRT_HD C<R> operator+(C<R> a, C<R> b) { return {a.x + b.x, a.y + b.y}; }
template <typename R> GRT_HD C<R> operator-(C<R> a, C<R> b) { return {a.x - b.x, a.y - b.y}; }
template <typename R> GRT_HD C<R> operator-(C<R> a) { return {-a.x, -a.y}; }
template <typename R> GRT_HD C<R> operator*(C<R> a, C<R> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename R> GRT_HD C<R> operator*(C<R> a, R s) { return {a.x * s, a.y * s}; }
template <typename R> GRT_HD C<R> operator*(R s, C<R> a) { return {a.x * s, a.y * s}; }
template <typename R> GRT_HD C<R> operator+(C<R> a, R s) { return {a.x + s, a.y}; }
template <typename R> GRT_HD C<R> operator+(R s, C<R> a) { return {a.x + s, a.y}; }
template <typename R> GRT_HD C<R> operator-(R s, C<R> a) { return {s - a.x, -a.y}; }
template <typename R> GRT_HD C<R> operator-(C<R> a, R s) { return {a.x - s, a.y}; }
template <typename R> GRT_HD C<R> conj(C<R> a) { return {a.x, -a.y}; }
template <typename R> GRT_HD R abs2(C<R> a) { return a.x * a.x + a.y * a.y; }

// 1/b, scaled so that |b|^2 neither overflows nor underflows
template <typename R> GRT_HD C<R> rcp(C<R> b)
{
    R s = fabs(b.x) > fabs(b.y) ? fabs(b.x) : fabs(b.y);
    R is = R(1) / s;
    C<R> t = {b.x * is, b.y * is};
    R d = is / (t.x * t.x + t.y * t.y);
    return {t.x * d, -t.y * d};
}
template <typename R> GRT_HD C<R> operator/(C<R> a, C<R> b) { return a * rcp(b); }
template <typename R> GRT_HD C<R> operator/(C<R> a, R s) { return a * (R(1) / s); }
template <typename R> GRT_HD C<R> operator/(R s, C<R> b) { return s * rcp(b); }

GRT_HD float gexp(float x) { return expf(x); }
GRT_HD double gexp(double x) { return exp(x); }
GRT_HD void gsincos(float x, float *s, float *c) { sincosf(x, s, c); }
GRT_HD void gsincos(double x, double *s, double *c) { sincos(x, s, c); }
GRT_HD float gsqrt(float x) { return sqrtf(x); }
GRT_HD double gsqrt(double x) { return sqrt(x); }
GRT_HD float ghypot(float x, float y) { return hypotf(x, y); }
GRT_HD double ghypot(double x, double y) { return hypot(x, y); }

template <typename R> GRT_HD R cabs_(C<R> a) { return ghypot(a.x, a.y); }

// exp(z) = e^x (cos y, sin y)
template <typename R> GRT_HD C<R> cexp_(C<R> z)
{
    R e = gexp(z.x), s, c;
    gsincos(z.y, &s, &c);
    return {e * c, e * s};
}

// principal square root (Re >= 0), cancellation-free form
template <typename R> GRT_HD C<R> csqrt_(C<R> z)
{
    // |z| without hypot's scaling: arguments here are k^2 - (w/c)^2, far from overflow
    R m = gsqrt(z.x * z.x + z.y * z.y);
    if (m == R(0)) return {R(0), R(0)};
    if (z.x >= R(0)) {
        R t = gsqrt((m + z.x) * R(0.5));
        return {t, z.y / (R(2) * t)};
    }
    R t = gsqrt((m - z.x) * R(0.5));
    return {fabs(z.y) / (R(2) * t), z.y >= R(0) ? t : -t};
}

// (exp(y) - 1) / y for |y| < 1/2 by its Taylor series
template <typename R> GRT_HD C<R> expm1_over_small(C<R> y)
{
    // 1 + y/2 + y^2/6 + ... ; 14 terms reach double precision at |y| = 1/2
    const int nt = sizeof(R) == 4 ? 8 : 15;
    C<R> s = {R(1), R(0)};
    C<R> t = {R(1), R(0)};
    for (int n = 2; n <= nt; n++) {
        t = t * y * (R(1) / R(n));
        s = s + t;
    }
    return s;
}

// ---- operand tiles of the tensor-core wavenumber GEMM (shared by the GRT
// kernel, which writes them, and the GEMM, which reads them)
constexpr int kTileK = 8;          // k per tile (one TF32 MMA K step)
constexpr int kTileRows = 128;     // 64 frequencies x (re, im)
// byte offset of element (row, k) in a K-major, no-swizzle core-matrix tile:
// 8-row x 16-byte core matrices ordered (row block, k block), 2 k blocks per row block
__host__ __device__ constexpr unsigned kt_tile_off(int row, int k)
{
    return (unsigned)((((row >> 3) * (kTileK / 4) + (k >> 2)) * 128) + (row & 7) * 16 + (k & 3) * 4);
}
// The 3xBF16 form of the same tiles: 16 k per tile (one kind::f16 MMA K
// step), 8 bf16 per 16-byte core-matrix row, 2 k blocks per row block; a
// tile is 4 KB in both forms.
constexpr int kTileK16 = 16;
__host__ __device__ constexpr unsigned kt_tile_off16(int row, int k)
{
    return (unsigned)((((row >> 3) * 2 + (k >> 3)) * 128) + (row & 7) * 16 + (k & 7) * 2);
}
// FP32 -> BF16 bits, round to nearest even; and the split x = hi + lo + O(2^-17 |x|)
__device__ __forceinline__ unsigned short bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_val(unsigned short b) { return __bfloat162float(__ushort_as_bfloat16(b)); }
__device__ __forceinline__ void bf16_split(float x, unsigned short &hi, unsigned short &lo)
{
    hi = bf16_bits(x);
    lo = bf16_bits(x - bf16_val(hi));
}

// FP32 -> TF32, round to nearest (ties away from zero)
__device__ __forceinline__ float tf32_rna(float x)
{
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

template <typename R>
struct M2 {
    C<R> a, b, c, d;  // [[a, b], [c, d]]
};

template <typename R> GRT_HD M2<R> m2(C<R> a, C<R> b, C<R> c, C<R> d) { return {a, b, c, d}; }
template <typename R> GRT_HD M2<R> operator*(const M2<R> &p, const M2<R> &q)
{
    return {p.a * q.a + p.b * q.c, p.a * q.b + p.b * q.d, p.c * q.a + p.d * q.c, p.c * q.b + p.d * q.d};
}
template <typename R> GRT_HD M2<R> operator+(const M2<R> &p, const M2<R> &q)
{
    return {p.a + q.a, p.b + q.b, p.c + q.c, p.d + q.d};
}
template <typename R> GRT_HD M2<R> operator-(const M2<R> &p, const M2<R> &q)
{
    return {p.a - q.a, p.b - q.b, p.c - q.c, p.d - q.d};
}
template <typename R> GRT_HD M2<R> operator*(const M2<R> &p, C<R> s) { return {p.a * s, p.b * s, p.c * s, p.d * s}; }
template <typename R> GRT_HD M2<R> operator*(const M2<R> &p, R s) { return {p.a * s, p.b * s, p.c * s, p.d * s}; }
template <typename R> GRT_HD M2<R> eye2() { return {{R(1), R(0)}, {R(0), R(0)}, {R(0), R(0)}, {R(1), R(0)}}; }
template <typename R> GRT_HD M2<R> zero2() { return {{R(0), R(0)}, {R(0), R(0)}, {R(0), R(0)}, {R(0), R(0)}}; }
// I - p
template <typename R> GRT_HD M2<R> eye_minus(const M2<R> &p) { return {R(1) - p.a, -p.b, -p.c, R(1) - p.d}; }
template <typename R> GRT_HD M2<R> eye_plus(const M2<R> &p) { return {R(1) + p.a, p.b, p.c, R(1) + p.d}; }
template <typename R> GRT_HD M2<R> minus_eye(const M2<R> &p) { return {p.a - R(1), p.b, p.c, p.d - R(1)}; }
// inverse given the determinant
template <typename R> GRT_HD M2<R> inv_det(const M2<R> &p, C<R> det)
{
    C<R> id = rcp(det);
    return {p.d * id, -(p.b * id), -(p.c * id), p.a * id};
}
template <typename R> GRT_HD M2<R> inv(const M2<R> &p) { return inv_det(p, p.a * p.d - p.b * p.c); }
// upper-triangular left/right products (phase matrices have c = 0)
template <typename R> GRT_HD M2<R> ut_mul_left(const M2<R> &u, const M2<R> &q)
{
    return {u.a * q.a + u.b * q.c, u.a * q.b + u.b * q.d, u.d * q.c, u.d * q.d};
}
template <typename R> GRT_HD M2<R> ut_mul_right(const M2<R> &q, const M2<R> &u)
{
    return {q.a * u.a, q.a * u.b + q.b * u.d, q.c * u.a, q.c * u.b + q.d * u.d};
}
template <typename R> GRT_HD void mv2(const M2<R> &p, C<R> x0, C<R> x1, C<R> *y0, C<R> *y1)
{
    *y0 = p.a * x0 + p.b * x1;
    *y1 = p.c * x0 + p.d * x1;
}

}  // namespace grt
