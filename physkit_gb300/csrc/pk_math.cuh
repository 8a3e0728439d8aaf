// pk_math.cuh — scalar-generic vector, quaternion and 3x3 math for the world-step kernels.
//
// Semantics follow the reference's algebra layer (include/physkit/algebra/lin_alg.h): Hamilton
// quaternions constructed w-first (lin_alg.h:428-432), quat*vec by the two-cross-product form
// (lin_alg.h:493-499), normalized() leaves a zero vector unchanged. Every reduction runs left to
// right; the FP64 translation unit is compiled with -fmad=false so that each operation rounds
// exactly as written.
#pragma once

#include <cmath>

#include <cstdint>

#if defined(__CUDACC__)
#define PK_HD __host__ __device__ __forceinline__
#else
#define PK_HD inline
#endif

namespace pk
{

template <class T> struct V3
{
    T x, y, z;
};
template <class T> struct Qt
{
    T w, x, y, z;
};
template <class T> struct M3
{
    T m[9]; // row-major
};

template <class T> PK_HD V3<T> mk(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> PK_HD V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> PK_HD V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> PK_HD V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> PK_HD V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> PK_HD V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> PK_HD V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> PK_HD T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> PK_HD V3<T> cross(V3<T> a, V3<T> b)
{ return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
template <class T> PK_HD T sqnorm(V3<T> a) { return dot(a, a); }

PK_HD double pk_sqrt(double x)
{
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(x);
#else
    return __builtin_sqrt(x);
#endif
}
PK_HD float pk_sqrt(float x)
{
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return __builtin_sqrtf(x);
#endif
}

// Inverse trigonometric functions of the platform's math library (they only pick a search
// neighbourhood; results never depend on their last bits).
PK_HD double pk_acos(double x) { return acos(x); }
PK_HD float pk_acos(float x) { return acosf(x); }
PK_HD double pk_atan2(double y, double x) { return atan2(y, x); }
PK_HD float pk_atan2(float y, float x) { return atan2f(y, x); }

template <class T> PK_HD T norm(V3<T> a) { return pk_sqrt(sqnorm(a)); }
template <class T> PK_HD V3<T> normalized(V3<T> a)
{
    T n2 = sqnorm(a);
    if (n2 > T(0)) return a / pk_sqrt(n2);
    return a;
}

template <class T> PK_HD T tmin(T a, T b) { return (b < a) ? b : a; } // std::min
template <class T> PK_HD T tmax(T a, T b) { return (a < b) ? b : a; } // std::max
template <class T> PK_HD T tabs(T a) { return a < T(0) ? -a : a; }

template <class T> PK_HD Qt<T> qmul(Qt<T> a, Qt<T> b)
{
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z, a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x};
}
template <class T> PK_HD Qt<T> conj(Qt<T> q) { return {q.w, -q.x, -q.y, -q.z}; }
template <class T> PK_HD V3<T> rotate(Qt<T> q, V3<T> v)
{
    V3<T> u{q.x, q.y, q.z};
    V3<T> uv = cross(u, v);
    uv = uv + uv;
    return v + q.w * uv + cross(u, uv);
}
template <class T> PK_HD Qt<T> qnormalized(Qt<T> q)
{
    T n2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w; // storage order x,y,z,w
    if (n2 > T(0))
    {
        T n = pk_sqrt(n2);
        return {q.w / n, q.x / n, q.y / n, q.z / n};
    }
    return q;
}

template <class T> PK_HD M3<T> to_matrix(Qt<T> q)
{
    T tx = T(2) * q.x, ty = T(2) * q.y, tz = T(2) * q.z;
    T twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    T txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    T tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    M3<T> r;
    r.m[0] = T(1) - (tyy + tzz);
    r.m[1] = txy - twz;
    r.m[2] = txz + twy;
    r.m[3] = txy + twz;
    r.m[4] = T(1) - (txx + tzz);
    r.m[5] = tyz - twx;
    r.m[6] = txz - twy;
    r.m[7] = tyz + twx;
    r.m[8] = T(1) - (txx + tyy);
    return r;
}
template <class T> PK_HD M3<T> transpose(const M3<T> &a)
{
    M3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[3 * i + j] = a.m[3 * j + i];
    return r;
}
template <class T> PK_HD M3<T> matmul(const M3<T> &a, const M3<T> &b)
{
    M3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}
template <class T> PK_HD V3<T> matvec(const T *m, V3<T> v)
{
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
// Adjugate inverse; det expanded along row 0.
template <class T> PK_HD M3<T> inverse(const M3<T> &a)
{
    const T *m = a.m;
    T c00 = m[4] * m[8] - m[5] * m[7];
    T c01 = m[5] * m[6] - m[3] * m[8];
    T c02 = m[3] * m[7] - m[4] * m[6];
    T c10 = m[2] * m[7] - m[1] * m[8];
    T c11 = m[0] * m[8] - m[2] * m[6];
    T c12 = m[1] * m[6] - m[0] * m[7];
    T c20 = m[1] * m[5] - m[2] * m[4];
    T c21 = m[2] * m[3] - m[0] * m[5];
    T c22 = m[0] * m[4] - m[1] * m[3];
    T det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    M3<T> r;
    r.m[0] = c00 / det;
    r.m[1] = c10 / det;
    r.m[2] = c20 / det;
    r.m[3] = c01 / det;
    r.m[4] = c11 / det;
    r.m[5] = c21 / det;
    r.m[6] = c02 / det;
    r.m[7] = c12 / det;
    r.m[8] = c22 / det;
    return r;
}

// Sine and cosine evaluated identically on host and device: Cody-Waite reduction by pi/2 (three-part
// split of pi/2 with 30-bit leading parts, exact k*P1 and k*P2 for |k| < 2^23) followed by Taylor
// polynomials on [-pi/4, pi/4] in Horner form (to x^19 and x^18). Accuracy ~1 ulp.
PK_HD void sincos_det(double x, double *s, double *c)
{
    const double two_over_pi = 0.6366197723675814;
    const double p1 = 1.570796325802803;
    const double p2 = 9.920935791635221e-10;
    const double p3 = 5.170182981794105e-19;
#if defined(__CUDA_ARCH__)
    double k = rint(x * two_over_pi);
#else
    double k = __builtin_nearbyint(x * two_over_pi);
#endif
    double r = x - k * p1;
    r = r - k * p2;
    r = r - k * p3;
    double r2 = r * r;
    double ps = -1.0 / 121645100408832000.0;
    ps = ps * r2 + 1.0 / 355687428096000.0;
    ps = ps * r2 - 1.0 / 1307674368000.0;
    ps = ps * r2 + 1.0 / 6227020800.0;
    ps = ps * r2 - 1.0 / 39916800.0;
    ps = ps * r2 + 1.0 / 362880.0;
    ps = ps * r2 - 1.0 / 5040.0;
    ps = ps * r2 + 1.0 / 120.0;
    ps = ps * r2 - 1.0 / 6.0;
    double sr = r + r * (r2 * ps);
    double pc = 1.0 / 6402373705728000.0;
    pc = pc * r2 - 1.0 / 20922789888000.0;
    pc = pc * r2 + 1.0 / 87178291200.0;
    pc = pc * r2 - 1.0 / 479001600.0;
    pc = pc * r2 + 1.0 / 3628800.0;
    pc = pc * r2 - 1.0 / 40320.0;
    pc = pc * r2 + 1.0 / 720.0;
    pc = pc * r2 - 1.0 / 24.0;
    pc = pc * r2 + 0.5;
    double cr = 1.0 - r2 * pc;
    long long q = static_cast<long long>(k);
    switch (static_cast<int>(q & 3))
    {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
    }
}
PK_HD void sincos_det(float x, float *s, float *c)
{
#if defined(__CUDA_ARCH__)
    sincosf(x, s, c);
#else
    double sd, cd;
    sincos_det(static_cast<double>(x), &sd, &cd);
    *s = static_cast<float>(sd);
    *c = static_cast<float>(cd);
#endif
}

PK_HD bool signbit_of(double z)
{
#if defined(__CUDA_ARCH__)
    return signbit(z);
#else
    return __builtin_signbit(z);
#endif
}
PK_HD bool signbit_of(float z)
{
#if defined(__CUDA_ARCH__)
    return signbit(z);
#else
    return __builtin_signbit(z);
#endif
}

// std::copysign(1, z): -1 when the sign bit of z is set (also for -0), else +1.
template <class T> PK_HD T copysign_one(T z) { return signbit_of(z) ? T(-1) : T(1); }

template <class T> struct Aabb
{
    V3<T> mn, mx;
};
template <class T> PK_HD bool aabb_contains(const Aabb<T> &a, const Aabb<T> &o)
{
    return (o.mn.x >= a.mn.x && o.mx.x <= a.mx.x) && (o.mn.y >= a.mn.y && o.mx.y <= a.mx.y) &&
           (o.mn.z >= a.mn.z && o.mx.z <= a.mx.z);
}
template <class T> PK_HD bool aabb_intersects(const Aabb<T> &a, const Aabb<T> &o)
{
    return (a.mn.x <= o.mx.x && a.mx.x >= o.mn.x) && (a.mn.y <= o.mx.y && a.mx.y >= o.mn.y) &&
           (a.mn.z <= o.mx.z && a.mx.z >= o.mn.z);
}

} // namespace pk
