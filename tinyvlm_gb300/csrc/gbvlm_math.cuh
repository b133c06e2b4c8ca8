// Device math shared by the gbvlm kernels: 3-vectors, the Biot-Savart
// straight-segment law in reference order (for the per-operator parity
// kernels) and the factored "relative-vector" form used by the tiled
// assembly, wake and roll-up kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbvlm {

// vlm/include/vlm_types.hpp:22-24 and vlm_backend_cpu_kernels.ispc:9-12
constexpr float PI_F = 3.141593f;
constexpr float EPS_F = 1.19209e-07f;
constexpr float RCUT_SQ = 1e-10f;   // |r1 x r2|^2 cut-off (both precisions)
constexpr float RCUT_NORM_F = 1e-5f; // |r1|, |r2| cut-off, float kernels
constexpr double RCUT_NORM_D = 1e-10; // |r1|, |r2| cut-off, double kernels

template <class T> struct V3 { T x, y, z; };

template <class T> __host__ __device__ __forceinline__ V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> __host__ __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> __host__ __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __host__ __device__ __forceinline__ V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> __host__ __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __host__ __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> __host__ __device__ __forceinline__ T len2(V3<T> a) { return a.x * a.x + a.y * a.y + a.z * a.z; }

template <class T> __device__ __forceinline__ T dsqrt(T x);
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }

template <class T> struct Prec;
template <> struct Prec<float> {
    static constexpr float rcut_norm = RCUT_NORM_F;
    __device__ static float fourpi() { return 4.0f * PI_F; }
};
template <> struct Prec<double> {
    static constexpr double rcut_norm = RCUT_NORM_D;
    // the reference's double kernel still forms 4*pi as the float product
    __device__ static double fourpi() { return (double)(4.0f * PI_F); }
};

// Katz-Plotkin eq. 10.115 in the reference's evaluation order
// (vlm_backend_cpu_kernels.ispc:69-89 float, :383-402 double).
template <class T>
__device__ __forceinline__ V3<T> biosavart_ref(V3<T> c, V3<T> a, V3<T> b, T sigma) {
    V3<T> r0 = b - a, r1 = c - a, r2 = c - b;
    V3<T> cr = cross(r1, r2);
    T r1n = dsqrt(len2(r1)), r2n = dsqrt(len2(r2));
    T sq = len2(cr);
    if (sq < (T)RCUT_SQ || r1n < Prec<T>::rcut_norm || r2n < Prec<T>::rcut_norm) return {0, 0, 0};
    T sm = sigma * sigma * len2(r0);
    T coeff = (dot(r0, r1) * r2n - dot(r0, r2) * r1n) / (Prec<T>::fourpi() * dsqrt(sq * sq + sm * sm) * r1n * r2n);
    return coeff * cr;
}

// Segment plus its y=0 image (ispc:91-102).
template <class T>
__device__ __forceinline__ void symmetry_ref(V3<T>& inf, V3<T> c, V3<T> a, V3<T> b, T sigma) {
    V3<T> s = biosavart_ref(c, a, b, sigma);
    inf.x += s.x; inf.y += s.y; inf.z += s.z;
    c.y = -c.y;
    V3<T> m = biosavart_ref(c, a, b, sigma);
    inf.x += m.x; inf.y -= m.y; inf.z += m.z;
}

template <class T>
__device__ __forceinline__ V3<T> ring_velocity_ref(V3<T> c, V3<T> v0, V3<T> v1, V3<T> v2, V3<T> v3_, T sigma) {
    V3<T> inf{0, 0, 0};
    symmetry_ref(inf, c, v0, v1, sigma);
    symmetry_ref(inf, c, v1, v2, sigma);
    symmetry_ref(inf, c, v2, v3_, sigma);
    symmetry_ref(inf, c, v3_, v0, sigma);
    return inf;
}

// ---------------------------------------------------------------------------
// Factored form.  For an evaluation point p and a lattice vertex v the kernel
// keeps r = p - v and |r|; a segment A->B with a = p - A, b = p - B and the
// segment vector r0 = B - A (taken from the vertex coordinates) gives
// a x b = r0 x a, and eq. 10.115's factor r0.(a/|a| - b/|b|) / |a x b|^2
// equals (|a|+|b|) / (|a||b| (|a||b| + a.b)).  When a.b < 0 the last factor
// is rewritten with |a x b|^2 = (|a||b| - a.b)(|a||b| + a.b), so neither the
// far field (a ~ b) nor points beside a long segment (a ~ -b) cancel:
//   k = (|a|+|b|) / (|a||b| (|a||b| + a.b))          a.b >= 0
//   k = (|a|+|b|) (|a||b| - a.b) / (|a||b| |a x b|^2)  a.b <  0
//   v(A->B) = k (r0 x a) / (4 pi)
// The cut-offs are the reference's.  Vertices are shared by the rings around
// them and a segment by its two rings, so a ring costs two vertex terms and
// three segment terms instead of eight segment evaluations.
// ---------------------------------------------------------------------------
template <class T> struct Rel { T x, y, z, n; };

template <class T> __device__ __forceinline__ T fast_len(T n2);
template <> __device__ __forceinline__ float fast_len<float>(float n2) { return n2 * rsqrtf(n2 + 1e-37f); }
template <> __device__ __forceinline__ double fast_len<double>(double n2) { return sqrt(n2); }

template <class T> __device__ __forceinline__ T fast_div(T a, T b);
template <> __device__ __forceinline__ float fast_div<float>(float a, float b) { return __fdividef(a, b); }
template <> __device__ __forceinline__ double fast_div<double>(double a, double b) { return a / b; }

// a + b where the two cannot cancel (both non-negative, or the result is
// only used when they are): plain addition; the float pair skips its
// renormalisation (its value stays in v without it)
template <class T> __device__ __forceinline__ T add_nc(T a, T b) { return a + b; }
template <class T> __device__ __forceinline__ T sub_nc(T a, T b) { return a - b; }

template <class T>
__device__ __forceinline__ Rel<T> make_rel(T x, T y, T z) {
    Rel<T> r;
    r.x = x; r.y = y; r.z = z;
    r.n = fast_len<T>(add_nc(add_nc(x * x, y * y), z * z));
    return r;
}

// scalar k with v(A->B) = k * (r0 x a) / (4 pi); the cross product is returned in c.
// DCUT: the double kernel's |r1|, |r2| cut-off (1e-10) in T's arithmetic: the
// batched mixed-precision path solves the FP64 system, whose near field is
// not cut at the float kernel's 1e-5 (a wing with panels smaller than 1e-4
// -- the tip strips of a finely cosine-spaced elliptic wing -- differs there)
template <class T, bool SIGMA, bool DCUT = false>
__device__ __forceinline__ T seg_coeff(const Rel<T>& a, const Rel<T>& b, T r0x, T r0y, T r0z, T sigma2, T& cx,
                                       T& cy, T& cz) {
    cx = r0y * a.z - r0z * a.y;
    cy = r0z * a.x - r0x * a.z;
    cz = r0x * a.y - r0y * a.x;
    const T sq = add_nc(add_nc(cx * cx, cy * cy), cz * cz);
    const T ab = a.x * b.x + a.y * b.y + a.z * b.z;
    const T nab = a.n * b.n;
    const T sum = add_nc(a.n, b.n);
    constexpr T rcut = DCUT ? (T)RCUT_NORM_D : Prec<T>::rcut_norm;
    const bool cut = (sq < (T)RCUT_SQ) | (a.n < rcut) | (b.n < rcut);
    const bool pos = ab >= (T)0;
    // |ab| <= nab: nab - ab cannot cancel when it is used (ab < 0), nor nab + ab (ab >= 0)
    T num = pos ? sum : sum * sub_nc(nab, ab);
    T den = pos ? nab * add_nc(nab, ab) : nab * sq;
    if (SIGMA) {
        // reference core smoothing: sq -> sqrt(sq^2 + (sigma^2 |r0|^2)^2)
        const T sm = sigma2 * (r0x * r0x + r0y * r0y + r0z * r0z);
        const T sc = dsqrt<T>(sq * sq + sm * sm);
        num = num * sq;
        den = den * sc;
    }
    const T k = fast_div<T>(num, den);
    return cut ? (T)0 : k;
}

// 4*pi * (velocity of segment A->B) . nrm
template <class T, bool SIGMA, bool DCUT = false>
__device__ __forceinline__ T seg_normal(const Rel<T>& a, const Rel<T>& b, T r0x, T r0y, T r0z, T nx, T ny, T nz,
                                        T sigma2) {
    T cx, cy, cz;
    const T k = seg_coeff<T, SIGMA, DCUT>(a, b, r0x, r0y, r0z, sigma2, cx, cy, cz);
    return k * (cx * nx + cy * ny + cz * nz);
}

// 4*pi * velocity vector of segment A->B (for wake roll-up)
template <class T, bool SIGMA>
__device__ __forceinline__ V3<T> seg_vec(const Rel<T>& a, const Rel<T>& b, T r0x, T r0y, T r0z, T sigma2) {
    T cx, cy, cz;
    const T k = seg_coeff<T, SIGMA>(a, b, r0x, r0y, r0z, sigma2, cx, cy, cz);
    return V3<T>{k * cx, k * cy, k * cz};
}

// Double-float difference (p_hi + p_lo) - (v_hi + v_lo): the hi difference is
// exact or rounded relative to the result, so r keeps float accuracy
// relative to |r| even far from the origin.
__device__ __forceinline__ float df_sub(float ph, float pl, float vh, float vl) {
    return (ph - vh) + (pl - vl);
}

// Kahan-Babuska (Neumaier) compensated accumulation in double.
struct CSum {
    double s = 0.0, c = 0.0;
    __device__ __forceinline__ void add(double x) {
        double t = s + x;
        c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
        s = t;
    }
    __device__ __forceinline__ double value() const { return s + c; }
};

// ---------------------------------------------------------------------------
// Float-pair arithmetic: x = v + e held as two floats (Dekker's double-length
// arithmetic; Knuth's TwoSum and an FMA-exact product), about 44 significant
// bits evaluated on the fp32 pipes.  Sums are renormalised (a difference
// whose float parts cancel exactly keeps its value in v, so later products
// see it), products are left with |e| of a few ulp(v).  The intrinsics keep
// every rounding as written (no contraction).  Used where the float AIC must
// be corrected toward its FP64 value (the refinement residual of the batched
// solver).
// ---------------------------------------------------------------------------
struct Fe {
    float v, e;
    Fe() = default;
    __host__ __device__ constexpr Fe(float a, float b) : v(a), e(b) {}
    __host__ __device__ constexpr Fe(float a) : v(a), e(0.f) {}
    __host__ __device__ constexpr Fe(int a) : v((float)a), e(0.f) {}
    __host__ __device__ constexpr Fe(double a) : v((float)a), e((float)(a - (double)(float)a)) {}
};

__device__ __forceinline__ Fe fe_fast2sum(float s, float t) {  // |s| >= |t| or s == 0
    const float h = __fadd_rn(s, t);
    return Fe(h, __fsub_rn(t, __fsub_rn(h, s)));
}
__device__ __forceinline__ Fe operator+(Fe a, Fe b) {
    const float s = __fadd_rn(a.v, b.v);
    const float bb = __fsub_rn(s, a.v);
    const float err = __fadd_rn(__fsub_rn(a.v, __fsub_rn(s, bb)), __fsub_rn(b.v, bb));  // a.v + b.v - s exactly
    return fe_fast2sum(s, __fadd_rn(err, __fadd_rn(a.e, b.e)));
}
__device__ __forceinline__ Fe operator-(Fe a) { return Fe(-a.v, -a.e); }
template <> __device__ __forceinline__ Fe add_nc<Fe>(Fe a, Fe b) {
    const float s = __fadd_rn(a.v, b.v);
    const float bb = __fsub_rn(s, a.v);
    const float err = __fadd_rn(__fsub_rn(a.v, __fsub_rn(s, bb)), __fsub_rn(b.v, bb));
    return Fe(s, __fadd_rn(err, __fadd_rn(a.e, b.e)));
}
template <> __device__ __forceinline__ Fe sub_nc<Fe>(Fe a, Fe b) { return add_nc<Fe>(a, Fe(-b.v, -b.e)); }
__device__ __forceinline__ Fe operator-(Fe a, Fe b) { return a + (-b); }
__device__ __forceinline__ Fe operator*(Fe a, Fe b) {
    const float p = __fmul_rn(a.v, b.v);
    float t = __fmaf_rn(a.v, b.v, -p);  // a.v*b.v - p exactly
    t = __fmaf_rn(a.v, b.e, t);
    t = __fmaf_rn(a.e, b.v, t);
    return Fe(p, t);
}
__device__ __forceinline__ Fe& operator+=(Fe& a, Fe b) { return a = a + b; }
// comparisons of the pair's value (v first; e breaks ties)
__device__ __forceinline__ bool operator<(Fe a, Fe b) { return a.v < b.v || (a.v == b.v && a.e < b.e); }
__device__ __forceinline__ bool operator>=(Fe a, Fe b) { return !(a < b); }

template <> struct Prec<Fe> {
    static constexpr double rcut_norm = RCUT_NORM_D;  // (a scalar: device code may read it)
};
template <> __device__ __forceinline__ Fe fast_len<Fe>(Fe n2) {
    // s = sqrt(v) to a few ulp, then one Newton correction from the exact
    // residual v - s^2 (plus e): sqrt(v + e) = s + (v - s^2 + e) / (2 s)
    const float r = rsqrtf(n2.v + 1e-37f);
    const float s = __fmul_rn(n2.v, r);
    const float d = __fadd_rn(__fmaf_rn(-s, s, n2.v), n2.e);
    return Fe(s, __fmul_rn(__fmul_rn(d, 0.5f), r));
}
template <> __device__ __forceinline__ Fe dsqrt<Fe>(Fe x) { return fast_len<Fe>(x); }
template <> __device__ __forceinline__ Fe fast_div<Fe>(Fe a, Fe b) {
    // q to a few ulp, then the correction (a - q b) / b from the FMA residual
    const float rb = __fdividef(1.0f, b.v);
    const float q = __fmul_rn(a.v, rb);
    const float r = __fadd_rn(__fmaf_rn(-q, b.v, a.v), __fmaf_rn(-q, b.e, a.e));
    return Fe(q, __fmul_rn(r, rb));
}

}  // namespace gbvlm
