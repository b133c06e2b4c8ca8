// Harmonic-balance VLM (lib/libhbvlm3.cpp:262-552 and lib/libhbvlm.cpp:230-468)
// in double on the device.
//
// The circulation is expanded in 2H+1 Fourier coefficients per panel
// (scaled orthonormal basis).  One fixed-point map (libhbvlm3.cpp:349-410):
// for every time instance s, the lifting surface's wake gamma is rebuilt
// from its trailing-edge coefficients and its influence (over the
// pre-generated kinematic wake) is subtracted from the instance's
// -V.n right-hand side; the (n x N) RHS is multiplied by the DFT matrix and
// solved with the AIC factored once.  Anderson acceleration
// (vlm/src/vlm_solvers.cpp:6-115, type II, history m, least squares by
// Householder QR like LAPACK dgels) iterates the map to a fixed point, on
// the device: iterate, residuals and histories stay in device memory and
// the host reads one residual norm per iteration.  The
// instance geometry, normals and -V.n do not depend on gamma and are
// computed once per run.
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gbvlm_internal.h"
#include "gbvlm_math.cuh"

namespace gbvlm {

__global__ void k_gather_te(const double* X, int64_t n, int64_t off, int64_t ns, int32_t N, double* te) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= ns * N) return;
    const int64_t i = g % ns, h = g / ns;
    te[i + h * ns] = X[off + i + h * n];
}

// Y (n x N) = R (n x N) . D (N x N), all column-major
__global__ void k_rdft(const double* R, const double* D, int64_t n, int32_t N, double* Y) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= n * N) return;
    const int64_t r = g % n, j = g / n;
    double s = 0;
    for (int32_t k = 0; k < N; k++) s += R[r + k * n] * D[k + j * N];
    Y[g] = s;
}

// The wake transforms of the libhbvlm kinematic chains (libhbvlm3.cpp:559-641,
// libhbvlm.cpp:470-515) at the steps t = i dt, evaluated on the device:
// free stream (-sigma t, 0, 0), heave (0, 0, -h(t)), pitch theta(t) about
// (px, 0, 0) and, when the lifting surface is the flap, a control rotation
// beta(t) about (qx, 0, 0) after the pitch.  h, theta, beta are Fourier
// series sum_k c_k cos(w t k) + s_k sin(w t k) of their coefficient rows.
// Parameters per set (HB_CHAIN_HEAD + 3 (2H+1) doubles): sigma, omega, dt,
// px, qx, flap, then the heave, pitch and control rows.  Writes the
// lifting surface's transform (column-major) at Tall[(i nsurf + m) 16].
constexpr int HB_CHAIN_HEAD = 6;

__device__ __forceinline__ void hb_rot_y(double px, double a, double& r00, double& r02, double& t0, double& t2) {
    double sn, cs;
    sincos(a, &sn, &cs);
    const double c1 = 1.0 - cs;
    r00 = 1.0 - c1;
    r02 = sn;
    t0 = px - r00 * px;
    t2 = 0.0 - (-sn) * px;
}

__global__ void k_hb_chain(const double* prm, int H, int64_t rows, int32_t nsurf, int32_t m, double* Tall) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const int U = 2 * H + 1;
    const double sigma = prm[0], omega = prm[1], dt = prm[2], px = prm[3], qx = prm[4];
    const bool flap = prm[5] != 0.0;
    const double* rh = prm + HB_CHAIN_HEAD;
    const double* rp = rh + U;
    const double* rc = rp + U;
    const double t = (double)i * dt;
    double h = rh[0] + 0.0 * t, th = rp[0] + 0.0 * t, be = rc[0] + 0.0 * t;
    for (int k = 0; k < H; k++) {
        double sn, cs;
        sincos((t * omega) * (double)(k + 1), &sn, &cs);
        h = (h + cs * rh[2 * k + 1]) + sn * rh[2 * k + 2];
        th = (th + cs * rp[2 * k + 1]) + sn * rp[2 * k + 2];
        be = (be + cs * rc[2 * k + 1]) + sn * rc[2 * k + 2];
    }
    double a00, a02, t0, t2;
    hb_rot_y(px, th, a00, a02, t0, t2);
    const double a03 = t0 + t * (-sigma), a23 = t2 + (-h);
    double M[16] = {0};
    M[5] = M[15] = 1.0;  // (1, 1), (3, 3)
    if (!flap) {
        M[0] = a00, M[8] = a02, M[12] = a03;   // row 0: (0,0), (0,2), (0,3)
        M[2] = -a02, M[10] = a00, M[14] = a23; // row 2
    } else {
        double b00, b02, u0, u2;
        hb_rot_y(qx, be, b00, b02, u0, u2);
        const double b20 = -b02;
        const double r0[3] = {a00, a02, a03}, r2[3] = {-a02, a00, a23};
        for (int rr = 0; rr < 2; rr++) {
            const double* ar = rr == 0 ? r0 : r2;
            const int row = rr == 0 ? 0 : 2;
            M[row] = ar[0] * b00 + ar[1] * b20;
            M[8 + row] = ar[0] * b02 + ar[1] * b00;
            M[12 + row] = (ar[0] * u0 + ar[1] * u2) + ar[2];
        }
    }
    double* o = Tall + 16 * ((int64_t)i * nsurf + m);
    for (int e = 0; e < 16; e++) o[e] = M[e];
}

// wake pre-generation in one launch (libhbvlm3.cpp:307-319): wake row
// nwv-1-i = T(i dt) applied to the trailing-edge vertices, every step i
__global__ void k_pregen_wake(const double* Tall, int32_t nsurf, int32_t m, const double* vinit, int64_t ns, int64_t nc,
                              int64_t max_t, double* wake) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t n1 = ns + 1;
    if (g >= n1 * max_t) return;
    const int64_t j = g % n1, i = g / n1;
    const double* T = Tall + 16 * ((size_t)i * nsurf + m);
    const int64_t nv = n1 * (nc + 1), te = j + nc * n1;
    const double x[4] = {vinit[te], vinit[nv + te], vinit[2 * nv + te], vinit[3 * nv + te]};
    const int64_t wl = n1 * max_t, row = max_t - 1 - i;
    for (int c = 0; c < 4; c++) {
        double acc = 0;
        for (int k = 0; k < 4; k++) acc += x[k] * T[c + 4 * k];
        wake[c * wl + j + row * n1] = acc;
    }
}

// ---------------------------------------------------------------------------
// The map's wake term as a precomputed linear operator.  The wake geometry
// (pre-generated once) and each instance's collocation points and normals do
// not change while Anderson iterates, and the wake gamma is linear in the
// trailing-edge Fourier coefficients te (i, c): gamma(j, i) = sum_c te(i, c)
// basis(j, c), with basis(j, 0) = 1/sqrt(N) and cos / sin (w k (t - (j -
// start + 1) dt)) sqrt(2/N) for harmonic k.  So the influence of instance q's
// wake on target p is sum_{i,c} Mq(p, i, c) te(i, c) with
//   Mq(p, i, c) = sum_j ring(p, j, i) basis_q(j, c),
// ring(p, j, i) = 4 pi (v . n) of the unit ring (row j, span i) and its mirror.
// The double Biot-Savart sums (the map's whole cost, and fp64 is a small
// fraction of the fp32 rate on this part) then run once per solve instead of
// once per map; each map reduces to the small contraction k_hb_rhs.
// ---------------------------------------------------------------------------
constexpr int WOP_THREADS = 64;  // two warps: the idle warps of a wider block cost registers
constexpr int WOP_NMAX = 32;  // Fourier coefficients a launch accumulates per thread (more: several launches)
constexpr int HB_NMAX = 2 * 64 + 1;  // time instances at most (64 harmonics)

// one instance of one parameter set (column)
struct WopInst {
    const double* colloc[GBVLM_MAX_SURFACES];
    const double* normals[GBVLM_MAX_SURFACES];
    const double* rhs_vel;  // -V.n of the instance (n)
    const double* wake;     // the column's lifting wake vertices, 4 planes of (wns+1) x nwv
    double* basis;          // (it x N) row-major
    int64_t it;             // active wake rows
    int64_t nwv;            // the column's wake vertex rows
    int64_t rps;            // wake rows per slice of k_wake_operator
    int64_t np0;            // panels of surface 0 (the origin is its first collocation point)
    double t;               // instance time
    double omega, dt;       // the column's map parameters
};

struct WopArgs {
    const WopInst* inst;
    int32_t nsurf, N, H;
    int64_t poff[GBVLM_MAX_SURFACES + 1];
    int64_t wns;
    double* partial;  // [slice][instance][n * wns][N]
    const float* wshift;       // k_wake_shift's output
    const int64_t* wshift_off; // per instance, into wshift
    float* basis_f2;           // the basis rows as float pairs, 2 floats per entry of the double rows
    const double* basis0;      // start of the double basis rows
    int32_t c0;                // the first Fourier coefficient this launch accumulates
};

// ---------------------------------------------------------------------------
// Float-pair ("double-single") arithmetic for the operator's ring values:
// a value is the unevaluated sum h + l of two floats, carried through the
// error-free transformations of Knuth (two-sum), Dekker (fast two-sum) and
// the fused multiply-add product, as in the double-double library of Hida,
// Li and Bailey but on float pairs.  About 48 significant bits, on the fp32
// pipe: GB300 issues fp32 arithmetic many times faster than fp64.  Division
// and square root take the float quotient / root and correct it with the
// residual formed in pairs (Karp and Markstein).  Every operation is written
// with the _rn intrinsics so that no contraction changes an error term.
// ---------------------------------------------------------------------------
struct F2 {
    float h, l;
};
__device__ __forceinline__ F2 f2_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return F2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ F2 f2_fast(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return F2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    F2 s = f2_two_sum(a.h, b.h);
    const F2 t = f2_two_sum(a.l, b.l);
    s = f2_fast(s.h, __fadd_rn(s.l, t.h));
    return f2_fast(s.h, __fadd_rn(s.l, t.l));
}
__device__ __forceinline__ F2 f2_neg(F2 a) { return F2{-a.h, -a.l}; }
__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) { return f2_add(a, f2_neg(b)); }
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return f2_fast(p, e);
}
__device__ __forceinline__ F2 f2_mulf(F2 a, float b) {
    const float p = __fmul_rn(a.h, b);
    const float e = __fmaf_rn(a.l, b, __fmaf_rn(a.h, b, -p));
    return f2_fast(p, e);
}
__device__ __forceinline__ F2 f2_div(F2 a, F2 b) {
    const float q1 = __fdiv_rn(a.h, b.h);
    F2 r = f2_sub(a, f2_mulf(b, q1));
    const float q2 = __fdiv_rn(r.h, b.h);
    r = f2_sub(r, f2_mulf(b, q2));
    const float q3 = __fdiv_rn(r.h, b.h);
    return f2_add(f2_fast(q1, q2), F2{q3, 0.f});
}
__device__ __forceinline__ F2 f2_sqrt(F2 a) {
    if (!(a.h > 0.f)) return F2{0.f, 0.f};
    const float x = __fsqrt_rn(a.h);
    const F2 d = f2_sub(a, f2_mul(F2{x, 0.f}, F2{x, 0.f}));
    return f2_add(F2{x, 0.f}, F2{__fdiv_rn(d.h, __fmul_rn(2.f, x)), 0.f});
}
__device__ __forceinline__ F2 f2_of(double x) {
    const float h = __double2float_rn(x);
    return F2{h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double f2_dbl(F2 a) { return (double)a.h + (double)a.l; }

// basis_q(j, c) for the active rows of every instance (grid y: instance),
// the same phases as k_gamma_wake in the operator library
__global__ void k_hb_basis(WopArgs a) {
    const WopInst& I = a.inst[blockIdx.y];
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // j - start
    if (r >= I.it) return;
    const double omega = I.omega, dt = I.dt;
    const int32_t U = a.N;
    const double s0 = 1.0 / sqrt((double)U), s2 = sqrt(2.0 / (double)U);
    double* b = I.basis + r * U;
    float* bf = a.basis_f2 + (b - a.basis0) * 2;
    auto put = [&](int c, double v) {
        b[c] = v;
        const F2 f = f2_of(v);
        bf[2 * c] = f.h;
        bf[2 * c + 1] = f.l;
    };
    put(0, s0);
    for (int32_t h = 0; h < a.H; h++) {
        const double wk = omega * (double)(h + 1);
        const double ph = wk * (I.t - (double)(r + 1) * dt);
        double sn, cs;
        sincos(ph, &sn, &cs);
        put(2 * h + 1, cs * s2);
        put(2 * h + 2, sn * s2);
    }
}

struct RelF2 {
    F2 x, y, z, n;
};
__device__ __forceinline__ RelF2 rel_f2(F2 px, F2 py, F2 pz, F2 vx, F2 vy, F2 vz) {
    RelF2 r;
    r.x = f2_sub(px, vx);
    r.y = f2_sub(py, vy);
    r.z = f2_sub(pz, vz);
    r.n = f2_sqrt(f2_add(f2_add(f2_mul(r.x, r.x), f2_mul(r.y, r.y)), f2_mul(r.z, r.z)));
    return r;
}
// seg_normal of the operator library (4 pi (v(A->B) . n), no core) in float pairs
__device__ __forceinline__ F2 seg_normal_f2(const RelF2& a, const RelF2& b, F2 nx, F2 ny, F2 nz) {
    const F2 r0x = f2_sub(a.x, b.x), r0y = f2_sub(a.y, b.y), r0z = f2_sub(a.z, b.z);  // B - A
    const F2 cx = f2_sub(f2_mul(r0y, a.z), f2_mul(r0z, a.y));
    const F2 cy = f2_sub(f2_mul(r0z, a.x), f2_mul(r0x, a.z));
    const F2 cz = f2_sub(f2_mul(r0x, a.y), f2_mul(r0y, a.x));
    const F2 sq = f2_add(f2_add(f2_mul(cx, cx), f2_mul(cy, cy)), f2_mul(cz, cz));
    if (sq.h < RCUT_SQ || a.n.h < (float)RCUT_NORM_D || b.n.h < (float)RCUT_NORM_D) return F2{0.f, 0.f};
    const F2 ab = f2_add(f2_add(f2_mul(a.x, b.x), f2_mul(a.y, b.y)), f2_mul(a.z, b.z));
    const F2 nab = f2_mul(a.n, b.n), sum = f2_add(a.n, b.n);
    F2 num, den;
    if (ab.h >= 0.f) {
        num = sum;
        den = f2_mul(nab, f2_add(nab, ab));
    } else {
        num = f2_mul(sum, f2_sub(nab, ab));
        den = f2_mul(nab, sq);
    }
    const F2 cn = f2_add(f2_add(f2_mul(cx, nx), f2_mul(cy, ny)), f2_mul(cz, nz));
    return f2_mul(f2_div(num, den), cn);
}

// the wake of each instance's set relative to the instance's origin (its
// first collocation point), as float pairs: 6 planes (x h, x l, y h, ...)
// of (wns+1) x nwv; the relative vectors of the operator are then
// differences of small numbers near the wing and lose no accuracy
__global__ void k_wake_shift(const WopInst* inst, int64_t wns, float* out, const int64_t* off) {
    const WopInst& I = inst[blockIdx.y];
    const int64_t nv = (wns + 1) * I.nwv;
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nv) return;
    float* o = out + off[blockIdx.y];
    const double O[3] = {I.colloc[0][0], I.colloc[0][I.np0], I.colloc[0][2 * I.np0]};
    for (int c = 0; c < 3; c++) {
        const F2 f = f2_of(I.wake[c * nv + v] - O[c]);
        o[(2 * c) * nv + v] = f.h;
        o[(2 * c + 1) * nv + v] = f.l;
    }
}

// one thread per (target p, wake span i) of instance blockIdx.y over the
// rows of slice blockIdx.z: the ring values along the rows in float pairs,
// each line's spanwise segment shared by the two rings it bounds
__global__ void __launch_bounds__(WOP_THREADS) k_wake_operator(WopArgs a) {
    const WopInst& I = a.inst[blockIdx.y];
    const int64_t n = a.poff[a.nsurf], npairs = n * a.wns;
    const int64_t g = blockIdx.x * (int64_t)WOP_THREADS + threadIdx.x;
    if (g >= npairs) return;
    const int64_t p = g / a.wns, i = g - p * a.wns;
    int m = 0;
    while (p >= a.poff[m + 1]) m++;
    const int64_t pl = p - a.poff[m], np = a.poff[m + 1] - a.poff[m];
    const double O[3] = {I.colloc[0][0], I.colloc[0][I.np0], I.colloc[0][2 * I.np0]};
    const double px = I.colloc[m][pl], py = I.colloc[m][np + pl], pz = I.colloc[m][2 * np + pl];
    const F2 Px = f2_of(px - O[0]), Py = f2_of(py - O[1]), Pz = f2_of(pz - O[2]);
    const F2 Qy = f2_of(-py - O[1]);  // the mirror point's y
    const F2 nx = f2_of(I.normals[m][pl]), ny = f2_of(I.normals[m][np + pl]), nz = f2_of(I.normals[m][2 * np + pl]);
    const F2 mny = f2_neg(ny);
    const int64_t start = I.nwv - 1 - I.it;
    const int64_t j0 = start + (int64_t)blockIdx.z * I.rps;
    const int64_t j1 = min(j0 + I.rps, I.nwv - 1);
    const int nco = a.N - a.c0;  // coefficients of this launch (at most WOP_NMAX used)
    F2 acc[WOP_NMAX];
#pragma unroll
    for (int c = 0; c < WOP_NMAX; c++) acc[c] = F2{0.f, 0.f};
    if (j0 < j1) {
        const int64_t n1 = a.wns + 1, nv = n1 * I.nwv;
        const float* W = a.wshift + a.wshift_off[blockIdx.y];
        auto V = [&](int64_t row, int64_t k, F2& x, F2& y, F2& z) {
            const int64_t o = k + row * n1;
            x = F2{W[o], W[nv + o]};
            y = F2{W[2 * nv + o], W[3 * nv + o]};
            z = F2{W[4 * nv + o], W[5 * nv + o]};
        };
        F2 x0, y0, z0, x1, y1, z1;
        V(j0, i, x0, y0, z0);
        V(j0, i + 1, x1, y1, z1);
        RelF2 A0 = rel_f2(Px, Py, Pz, x0, y0, z0), A1 = rel_f2(Px, Py, Pz, x1, y1, z1);
        RelF2 B0 = rel_f2(Px, Qy, Pz, x0, y0, z0), B1 = rel_f2(Px, Qy, Pz, x1, y1, z1);
        F2 Ta = seg_normal_f2(A0, A1, nx, ny, nz), Tb = seg_normal_f2(B0, B1, nx, mny, nz);
        for (int64_t j = j0; j < j1; j++) {
            F2 x3, y3, z3, x2, y2, z2;  // line j + 1: v3 = (j + 1, i), v2 = (j + 1, i + 1)
            V(j + 1, i, x3, y3, z3);
            V(j + 1, i + 1, x2, y2, z2);
            const RelF2 A3 = rel_f2(Px, Py, Pz, x3, y3, z3), A2 = rel_f2(Px, Py, Pz, x2, y2, z2);
            const RelF2 B3 = rel_f2(Px, Qy, Pz, x3, y3, z3), B2 = rel_f2(Px, Qy, Pz, x2, y2, z2);
            const F2 Na = seg_normal_f2(A3, A2, nx, ny, nz), Nb = seg_normal_f2(B3, B2, nx, mny, nz);
            F2 val = f2_add(f2_sub(f2_add(Ta, seg_normal_f2(A1, A2, nx, ny, nz)), Na), seg_normal_f2(A3, A0, nx, ny, nz));
            val = f2_add(val, f2_add(f2_sub(f2_add(Tb, seg_normal_f2(B1, B2, nx, mny, nz)), Nb),
                                     seg_normal_f2(B3, B0, nx, mny, nz)));
            const float* br = a.basis_f2 + (I.basis - a.basis0 + (j - start) * a.N + a.c0) * 2;
#pragma unroll
            for (int c = 0; c < WOP_NMAX; c++)
                if (c < nco) acc[c] = f2_add(acc[c], f2_mul(val, F2{br[2 * c], br[2 * c + 1]}));
            A0 = A3, A1 = A2, B0 = B3, B1 = B2;
            Ta = Na, Tb = Nb;
        }
    }
    double* out = a.partial + (((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * npairs + g) * a.N + a.c0;
#pragma unroll
    for (int c = 0; c < WOP_NMAX; c++)
        if (c < nco) out[c] = f2_dbl(acc[c]);
}

// M = sum over slices of the partial operators, in slice order
__global__ void k_wake_operator_sum(const double* partial, int64_t slices, int64_t len, double* M) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= len) return;
    double s = 0;
    for (int64_t k = 0; k < slices; k++) s += partial[k * len + e];
    M[e] = s;
}

// One map's right-hand sides and their DFT, one block per target p and
// column blockIdx.y: R(p, q) = -V.n_q(p) - sum_{i,c} Mq(p, i, c) te(i, c) /
// (4 pi), with te read from the column's iterate X (n x N) at the lifting
// surface's trailing-edge row; then Y(p, k) = sum_q R(p, q) D(q, k).
constexpr int HBR_THREADS = 128;
__global__ void __launch_bounds__(HBR_THREADS) k_hb_rhs(const WopInst* inst, const double* M, const double* X,
                                                        int64_t n, int64_t te_off, int64_t wns, int32_t N,
                                                        const double* D, double* Y) {
    __shared__ double R[HB_NMAX];
    const int64_t p = blockIdx.x, col = blockIdx.y;
    inst += col * N;
    M += col * (int64_t)N * n * wns * N;
    X += col * n * N;
    D += col * (int64_t)N * N;
    Y += col * n * N;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t K = wns * N;
    const double inv4pi = 1.0 / (double)(4.0f * PI_F);
    for (int q = wid; q < N; q += HBR_THREADS / 32) {
        const double* mq = M + ((int64_t)q * n + p) * K;
        double s = 0;
        for (int64_t e = lane; e < K; e += 32) {
            const int64_t i = e / N, c = e - i * N;
            s += mq[e] * X[te_off + i + c * n];
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) R[q] = inst[q].rhs_vel[p] - s * inv4pi;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < N; k += HBR_THREADS) {
        double y = 0;
        for (int q = 0; q < N; q++) y += R[q] * D[q + (int64_t)k * N];
        Y[p + (int64_t)k * n] = y;
    }
}

// ---------------------------------------------------------------------------
// Loads at the force instances (libhbvlm3.cpp:428-550) for every instance of
// every parameter set in one launch, one 512-thread block per (set,
// instance).  Per panel, as the operator library's kernels compute it: the
// displaced vertices (k_displace), normal and area (k_mesh_metrics), the
// circulation and its rate from the Fourier coefficients (one DFT row), the
// chordwise gamma delta (the wing's trailing edge subtracted from the flap's
// first row when coupled), -(dT/dt) at the undisplaced collocation point, and
// the unsteady Joukowski force (k_forces).  The sums per surface (area, CL,
// the mean aerodynamic chord and CM_y about each reference point) are
// compensated and strided over the block exactly as k_reduce sums them, and
// combined over the surfaces as the host does for one instance.
// ---------------------------------------------------------------------------
constexpr int HBL_THREADS = 512;

struct LoadsArgs {
    int32_t nsurf, N, coupled;
    int64_t n;
    int64_t ns[GBVLM_MAX_SURFACES], nc[GBVLM_MAX_SURFACES], poff[GBVLM_MAX_SURFACES + 1];
    const double* vinit[GBVLM_MAX_SURFACES];
    const double* colloc_h[GBVLM_MAX_SURFACES];
    const double *C, *D, *DD, *T, *Td, *fs, *ref_a, *ref_b;
    double* out;  // per set 3 x N
};

__device__ __forceinline__ double hbl_block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(HBL_THREADS) k_hb_loads(LoadsArgs a) {
    __shared__ double sh[32];
    const int64_t e = blockIdx.x, c = e / a.N, q = e - c * a.N;
    const int N = a.N, tid = threadIdx.x;
    const double* Cc = a.C + c * a.n * N;
    const double* Dr = a.D + c * (int64_t)N * N + q;   // row q: Dr[j * N]
    const double* DDr = a.DD + c * (int64_t)N * N + q;
    const double* fs = a.fs + 3 * e;
    auto gam = [&](const double* row, int64_t p) {
        double v = 0;
        for (int j = 0; j < N; j++) v += Cc[p + (int64_t)j * a.n] * row[(int64_t)j * N];
        return v;
    };
    double la[3] = {-fs[2], 0.0, fs[0]};
    const double ll = sqrt(la[0] * la[0] + la[2] * la[2]);
    la[0] /= ll;
    la[2] /= ll;
    const double v2 = fs[0] * fs[0] + fs[1] * fs[1] + fs[2] * fs[2];
    const double* ra = a.ref_a + 3 * e;
    const double* rb = a.ref_b ? a.ref_b + 3 * e : nullptr;
    double cl = 0, ta = 0, tm = 0, cm = 0, cmb_out = 0;
    for (int m = 0; m < a.nsurf; m++) {
        const int64_t ns = a.ns[m], nc = a.nc[m], np = ns * nc, nv = (ns + 1) * (nc + 1), po = a.poff[m];
        const double* vin = a.vinit[m];
        const double* tr = a.T + 16 * (e * a.nsurf + m);
        const double* td = a.Td + 16 * (e * a.nsurf + m);
        auto vert = [&](int64_t r) {
            const double x[4] = {vin[r], vin[nv + r], vin[2 * nv + r], vin[3 * nv + r]};
            double o[3];
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
                double acc = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) acc += x[k] * tr[cc + 4 * k];
                o[cc] = acc;
            }
            return V3<double>{o[0], o[1], o[2]};
        };
        const bool prev = a.coupled && m > 0 && a.ns[m - 1] == ns;
        const bool with_b = m == 1 && rb != nullptr;
        CSum s_area, s_cl, s_cm, s_cmb, s_mac0, s_mac1;
        for (int64_t p = tid; p < np; p += HBL_THREADS) {
            const int64_t i = p % ns, j = p / ns;
            const int64_t ia = i + j * (ns + 1), ib = ia + 1, ic = ib + (ns + 1), id = ia + (ns + 1);
            const V3<double> v0 = vert(ia), v1 = vert(ib), v2p = vert(ic), v3 = vert(id);
            const V3<double> nn = cross(v3 - v1, v2p - v0);
            const double l = sqrt(len2(nn));
            const V3<double> nor{nn.x / l, nn.y / l, nn.z / l};
            const V3<double> f = v3 - v0, bb = v2p - v0, ee = v1 - v0;
            const double ar = 0.5 * (sqrt(len2(cross(f, bb))) + sqrt(len2(cross(bb, ee))));
            const double gp = gam(Dr, po + p);
            double gd = gp;
            if (j > 0) gd -= gam(Dr, po + p - ns);
            else if (prev) gd -= gam(Dr, po - ns + i);
            const double dg = gam(DDr, po + p);
            const double* ch = a.colloc_h[m];
            const double x = ch[p], y = ch[np + p], z = ch[2 * np + p];
            double vel[3];
            for (int r = 0; r < 3; r++) vel[r] = -(td[r] * x + td[r + 4] * y + td[r + 8] * z + td[r + 12]);
            const V3<double> V{vel[0], vel[1], vel[2]};
            V3<double> F = (1.0 * gd) * cross(V, v1 - v0);
            F = F + (1.0 * dg * ar) * nor;
            s_area.add(ar);
            s_mac1.add(ar);
            s_cl.add(F.x * la[0] + F.y * la[1] + F.z * la[2]);
            const double lx = 0.5 * (v0.x + v1.x) - ra[0], lz = 0.5 * (v0.z + v1.z) - ra[2];
            s_cm.add(lz * F.x - lx * F.z);
            if (with_b) {
                const double bx = 0.5 * (v0.x + v1.x) - rb[0], bz = 0.5 * (v0.z + v1.z) - rb[2];
                s_cmb.add(bz * F.x - bx * F.z);
            }
        }
        const int64_t last = nc * (ns + 1);
        for (int64_t i = tid; i < ns; i += HBL_THREADS) {
            const V3<double> l0 = vert(i), l1 = vert(i + 1), t0 = vert(last + i), t1 = vert(last + i + 1);
            const V3<double> d0 = l0 - t0, d1 = l1 - t1, d3 = l1 - l0;
            const double c0 = sqrt(len2(d0)), c1 = sqrt(len2(d1));
            s_mac0.add(0.5 * (c0 * c0 + c1 * c1) * sqrt(len2(d3)));
        }
        const double area = hbl_block_sum(s_area.value(), sh);
        const double rcl = hbl_block_sum(s_cl.value(), sh);
        const double mac0 = hbl_block_sum(s_mac0.value(), sh), mac1 = hbl_block_sum(s_mac1.value(), sh);
        const double rcm = hbl_block_sum(s_cm.value(), sh);
        const double rcmb = with_b ? hbl_block_sum(s_cmb.value(), sh) : 0.0;
        if (tid == 0) {
            const double clm = rcl / (0.5 * 1.0 * v2 * area);
            const double mac = mac0 / mac1;
            const double d = 0.5 * 1.0 * v2 * area * mac;
            cl += clm * area;
            ta += area;
            tm += mac;
            cm += (rcm / d) * area * mac;
            if (with_b) cmb_out = rcmb / d;
        }
    }
    if (tid == 0) {
        double* o = a.out + c * 3 * N;
        o[q] = cl / ta;
        o[N + q] = cm / (ta * tm);
        o[2 * N + q] = cmb_out;
    }
}

// Instance geometry of every instance of every set in one launch (grid y:
// instance): per panel the displaced vertices (k_displace), collocation
// point and normal at zero angle of attack (k_mesh_metrics), and -V.n with
// V = -(dT/dt) applied to the undisplaced collocation point (k_vel_dual,
// k_rhs_velocities).  The instance buffer holds colloc (3n), normals (3n)
// and -V.n (n) per instance, each surface's planes at 3 poff[m].
struct GeomArgs {
    int32_t nsurf;
    int64_t n;
    int64_t ns[GBVLM_MAX_SURFACES], nc[GBVLM_MAX_SURFACES], poff[GBVLM_MAX_SURFACES + 1];
    const double* vinit[GBVLM_MAX_SURFACES];
    const double* colloc_h[GBVLM_MAX_SURFACES];
    const double *T, *Td;
    double* inst;  // per instance 7 n
};

__global__ void k_hb_geom(GeomArgs a) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, e = blockIdx.y;
    if (g >= a.n) return;
    int m = 0;
    while (m + 1 < a.nsurf && g >= a.poff[m + 1]) m++;
    const int64_t ns = a.ns[m], nc = a.nc[m], np = ns * nc, nv = (ns + 1) * (nc + 1), p = g - a.poff[m];
    const int64_t i = p % ns, j = p / ns;
    const double* vin = a.vinit[m];
    const double* tr = a.T + 16 * (e * a.nsurf + m);
    const double* td = a.Td + 16 * (e * a.nsurf + m);
    auto vert = [&](int64_t r) {
        const double x[4] = {vin[r], vin[nv + r], vin[2 * nv + r], vin[3 * nv + r]};
        double o[3];
#pragma unroll
        for (int cc = 0; cc < 3; cc++) {
            double acc = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) acc += x[k] * tr[cc + 4 * k];
            o[cc] = acc;
        }
        return V3<double>{o[0], o[1], o[2]};
    };
    const int64_t ia = i + j * (ns + 1), ib = ia + 1, ic = ib + (ns + 1), id = ia + (ns + 1);
    const V3<double> v0 = vert(ia), v1 = vert(ib), v2 = vert(ic), v3 = vert(id);
    const V3<double> nn = cross(v3 - v1, v2 - v0);
    const double l = sqrt(len2(nn));
    const V3<double> nor{nn.x / l, nn.y / l, nn.z / l};
    const V3<double> ch = 0.5 * (((v2 + v3) - v0) - v1);
    const V3<double> cp = 0.5 * (v0 + v1) + 0.5 * ch;
    const double* c0 = a.colloc_h[m];
    const double x = c0[p], y = c0[np + p], z = c0[2 * np + p];
    double vel[3];
    for (int r = 0; r < 3; r++) vel[r] = -(td[r] * x + td[r + 4] * y + td[r + 8] * z + td[r + 12]);
    double* base = a.inst + e * 7 * a.n;
    double* col = base + 3 * a.poff[m];
    double* nrm = base + 3 * a.n + 3 * a.poff[m];
    col[p] = cp.x;
    col[np + p] = cp.y;
    col[2 * np + p] = cp.z;
    nrm[p] = nor.x;
    nrm[np + p] = nor.y;
    nrm[2 * np + p] = nor.z;
    base[6 * a.n + g] = 0.0 + -(vel[0] * nor.x + vel[1] * nor.y + vel[2] * nor.z);
}

// X (n x cols) = Ainv (n x n) . Y (n x cols), column-major, one thread per
// entry with the sum over k in order: the map's solve for the AIC of a small
// lattice, whose inverse is formed once from its LU factors
constexpr int64_t HB_INV_MAX = 2048;  // largest n whose inverse is kept (32 MiB)
__global__ void k_hb_inv_apply(const double* Ainv, const double* Y, int64_t n, int64_t cols, double* X) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n * cols) return;
    const int64_t r = e % n, j = e / n;
    const double* y = Y + j * n;
    double s = 0;
    for (int64_t k = 0; k < n; k++) s += Ainv[r + k * n] * y[k];
    X[e] = s;
}

// device buffer, grown on demand
template <class T>
struct Buf {
    T* p = nullptr;
    size_t cap = 0;
    int grow(size_t cnt) {
        cnt = std::max<size_t>(cnt, 1);
        if (cap >= cnt) return GBVLM_OK;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        GB_CUDA(cudaMalloc((void**)&p, sizeof(T) * cnt));
        cap = cnt;
        return GBVLM_OK;
    }
    ~Buf() {
        if (p) cudaFree(p);
    }
};
using DBuf = Buf<double>;

// one time instance of one column; pointers into the batch buffers
struct Inst {
    int64_t t_steps = 0;
    double t = 0;
    std::vector<double*> colloc, normals, gwake;
    double* rhs_vel = nullptr;
};

// one parameter set (for instance a finite-difference Jacobian column):
// its wake, its instances and its map parameters
struct HbCol {
    int64_t max_t = 0;
    std::vector<gbvlm_dims> dims;  // nwv = max_t
    std::vector<double*> wake;     // per surface; only the lifting surface's is built
    std::vector<Inst> inst;        // N
};

struct HbState {
    int32_t nsurf = 0, wake_surf = 0, N = 0, K = 0;
    std::vector<gbvlm_dims> dims;
    std::vector<int32_t> lifting;
    int64_t n = 0;
    std::vector<int64_t> poff;
    std::vector<void*> allocs;
    std::vector<double*> vinit, verts, colloc_h, normals, areas;
    double* lhs = nullptr;
    gbvlm_lu lu = nullptr;
    bool aic_ready = false;
    DBuf ainv;  // the AIC's inverse when n <= HB_INV_MAX
    std::vector<HbCol> cols;
    // batch buffers: per instance colloc, normals (3n each) and -V.n (n);
    // the lifting wake's gammas for the per-map sums; wakes; transforms and
    // rates of every instance; iterate, map output and right-hand sides
    // (K x n x N); DFT matrices (K x N x N); trailing-edge coefficients
    DBuf inst_buf, gwake_buf, wake_buf, tw_buf, tdev, tddev, Xin, Xout, R, D, te, chain_buf;
    // the wake operator (k_wake_operator): instance table (host copy and
    // device), basis rows, partial sums and the operators
    std::vector<WopInst> wtab;
    WopInst* d_wop = nullptr;
    size_t d_wop_cap = 0;
    DBuf wop_basis, wop_part, wop_M;
    Buf<float> wop_basis_f2, wop_shift;
    Buf<int64_t> wop_shift_off;
    bool wop_valid = false;
    // inputs and outputs of k_hb_loads
    DBuf ld_C, ld_D, ld_DD, ld_T, ld_Td, ld_fs, ld_ra, ld_rb, ld_out;
    // Anderson state of every set, and the Anderson loop as a graph (a
    // while node), rebuilt when its arguments change
    DBuf aa_buf;
    cudaGraph_t aa_graph = nullptr;
    cudaGraphExec_t aa_exec = nullptr;
    cudaStream_t aa_cap = nullptr;
    std::vector<char> aa_key;

    ~HbState() {
        if (aa_exec) cudaGraphExecDestroy(aa_exec);
        if (aa_graph) cudaGraphDestroy(aa_graph);
        if (aa_cap) cudaStreamDestroy(aa_cap);
        if (lu) gbvlm_lu_destroy(lu);
        for (void* p : allocs) cudaFree(p);
        if (d_wop) cudaFree(d_wop);
    }

    // the loop can be a graph when a map is k_hb_rhs + k_hb_inv_apply
    bool anderson_graph_ok() const { return use_wop() && n <= HB_INV_MAX; }

    int alloc(double** p, size_t cnt) {
        GB_CUDA(cudaMalloc((void**)p, sizeof(double) * (cnt > 0 ? cnt : 1)));
        GB_CUDA(cudaMemset(*p, 0, sizeof(double) * (cnt > 0 ? cnt : 1)));
        allocs.push_back(*p);
        return GBVLM_OK;
    }
    std::vector<const double*> C(const std::vector<double*>& v) const { return {v.begin(), v.end()}; }

    int init(int32_t ns_, const gbvlm_dims* d, const double* const* vh, const int32_t* lift) {
        nsurf = ns_;
        dims.assign(d, d + ns_);
        lifting.assign(lift, lift + ns_);
        int nl = 0;
        for (int m = 0; m < nsurf; m++)
            if (lifting[m]) {
                wake_surf = m;
                nl++;
            }
        GB_REQUIRE(nl == 1, "harmonic balance needs exactly one lifting surface (its wake carries the TE gamma)");
        poff.assign(nsurf + 1, 0);
        int rc;
        for (int m = 0; m < nsurf; m++) {
            const int64_t np = dims[m].ns * dims[m].nc, nv = (dims[m].ns + 1) * (dims[m].nc + 1);
            poff[m + 1] = poff[m] + np;
            double* p;
            if ((rc = alloc(&p, 4 * nv))) return rc;
            vinit.push_back(p);
            GB_CUDA(cudaMemcpy(p, vh[m], sizeof(double) * 4 * nv, cudaMemcpyHostToDevice));
            if ((rc = alloc(&p, 4 * nv))) return rc;
            verts.push_back(p);
            for (auto* vec : {&colloc_h, &normals}) {
                if ((rc = alloc(&p, 3 * np))) return rc;
                vec->push_back(p);
            }
            if ((rc = alloc(&p, np))) return rc;
            areas.push_back(p);
        }
        n = poff[nsurf];
        if ((rc = alloc(&lhs, n * n))) return rc;
        if ((rc = gbvlm_lu_create(&lu))) return rc;
        return gbvlm_lu_init(lu, n);
    }

    // libhbvlm3.cpp:266-300: metrics at the undisplaced pose, the AIC
    // without wake and its factors.  The meshes are fixed once created, so
    // this runs at the first prepare only.
    int aic(cudaStream_t st) {
        if (aic_ready) return GBVLM_OK;
        gbvlm_stream s = (gbvlm_stream)st;
        int rc;
        for (int m = 0; m < nsurf; m++) {
            const int64_t nv = (dims[m].ns + 1) * (dims[m].nc + 1);
            GB_CUDA(cudaMemcpyAsync(verts[m], vinit[m], sizeof(double) * 4 * nv, cudaMemcpyDeviceToDevice, st));
        }
        if ((rc = gbvlm_mesh_metrics_f64(0.0, nsurf, dims.data(), C(verts).data(), colloc_h.data(), normals.data(),
                                         areas.data(), s)))
            return rc;
        GB_CUDA(cudaMemsetAsync(lhs, 0, sizeof(double) * n * n, st));
        if ((rc = gbvlm_lhs_assemble_f64(lhs, n, nsurf, dims.data(), C(colloc_h).data(), C(normals).data(),
                                         C(verts).data(), nullptr, 0, 0.0, s)))
            return rc;
        if ((rc = gbvlm_lu_factor_f64(lu, lhs, n, n, s))) return rc;
        if (n <= HB_INV_MAX) {  // A^-1 from the factors: the identity solved for
            if ((rc = ainv.grow(n * n))) return rc;
            std::vector<double> I((size_t)(n * n), 0.0);
            for (int64_t i = 0; i < n; i++) I[i + i * n] = 1.0;
            GB_CUDA(cudaMemcpyAsync(ainv.p, I.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice, st));
            if ((rc = gbvlm_lu_solve_f64(lu, lhs, n, n, ainv.p, n, n, s))) return rc;
            GB_CUDA(cudaStreamSynchronize(st));
        }
        aic_ready = true;
        return GBVLM_OK;
    }

    // K parameter sets (libhbvlm3.cpp:307-319 and 363-393 without the gamma
    // part, per set): the lifting wake pre-generated over max_t[c] steps,
    // then per instance the displaced geometry and -V.n.  Nothing here
    // synchronises per instance: every transform is uploaded once.
    // wake_T: per set its wake transforms (HOST), or chain: per set the
    // chain parameters of k_hb_chain (HOST, K x (HB_CHAIN_HEAD + 3 (2H+1)))
    int prepare(int32_t K_, int32_t harmonics, const int64_t* max_t, const double* const* wake_T, const double* chain,
                const int64_t* t_steps, const double* times, const double* Th, const double* Tdh, const double* dft,
                cudaStream_t st) {
        int rc;
        if ((rc = aic(st))) return rc;
        K = K_;
        N = 2 * harmonics + 1;
        wop_valid = false;
        const gbvlm_dims& W = dims[wake_surf];
        const int64_t wn1 = W.ns + 1;
        cols.assign(K, HbCol());
        int64_t wake_tot = 0, tw_tot = 0, gw_tot = 0;
        for (int c = 0; c < K; c++) {
            GB_REQUIRE(max_t[c] >= 2, "column %d: max_t_steps %lld < 2", c, (long long)max_t[c]);
            GB_REQUIRE(chain || wake_T[c] != nullptr, "column %d: wake transforms are null", c);
            wake_tot += 4 * wn1 * max_t[c];
            tw_tot += 16 * nsurf * max_t[c];
            gw_tot += (int64_t)N * W.ns * (max_t[c] - 1);
        }
        const int64_t ninst = (int64_t)K * N;
        if ((rc = wake_buf.grow(wake_tot)) || (rc = tw_buf.grow(tw_tot)) || (rc = gwake_buf.grow(gw_tot)) ||
            (rc = inst_buf.grow(ninst * 7 * n)) || (rc = tdev.grow(ninst * nsurf * 16)) ||
            (rc = tddev.grow(ninst * nsurf * 16)) || (rc = D.grow(ninst * N)) || (rc = Xin.grow(ninst * n)) ||
            (rc = Xout.grow(ninst * n)) || (rc = R.grow(ninst * n)) || (rc = te.grow(ninst * W.ns)))
            return rc;
        // wakes (only the lifting surface's: the others shed none)
        const int64_t cstride = HB_CHAIN_HEAD + 3 * (int64_t)N;
        if (chain) {
            if ((rc = chain_buf.grow(K * cstride))) return rc;
            GB_CUDA(cudaMemcpyAsync(chain_buf.p, chain, sizeof(double) * K * cstride, cudaMemcpyHostToDevice, st));
        }
        int64_t wo = 0, two = 0;
        for (int c = 0; c < K; c++) {
            HbCol& col = cols[c];
            col.max_t = max_t[c];
            col.dims = dims;
            for (auto& d : col.dims) d.nwv = col.max_t;
            col.wake.assign(nsurf, nullptr);
            col.wake[wake_surf] = wake_buf.p + wo;
            double* Tall = tw_buf.p + two;
            if (chain) {
                k_hb_chain<<<(unsigned)cdiv(col.max_t, 128), 128, 0, st>>>(chain_buf.p + c * cstride, harmonics,
                                                                          col.max_t, nsurf, wake_surf, Tall);
                GB_LAUNCH_CHECK();
            } else {
                GB_CUDA(cudaMemcpyAsync(Tall, wake_T[c], sizeof(double) * 16 * nsurf * col.max_t,
                                        cudaMemcpyHostToDevice, st));
            }
            const int64_t cnt = wn1 * col.max_t;
            k_pregen_wake<<<(unsigned)cdiv(cnt, 128), 128, 0, st>>>(Tall, nsurf, wake_surf, vinit[wake_surf], W.ns,
                                                                     W.nc, col.max_t, col.wake[wake_surf]);
            GB_LAUNCH_CHECK();
            wo += 4 * wn1 * col.max_t;
            two += 16 * nsurf * col.max_t;
        }
        // instances
        GB_CUDA(cudaMemcpyAsync(tdev.p, Th, sizeof(double) * ninst * nsurf * 16, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(tddev.p, Tdh, sizeof(double) * ninst * nsurf * 16, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(D.p, dft, sizeof(double) * ninst * N, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemsetAsync(gwake_buf.p, 0, sizeof(double) * std::max<int64_t>(gw_tot, 1), st));
        {
            GeomArgs ga;
            memset(&ga, 0, sizeof(ga));
            ga.nsurf = nsurf;
            ga.n = n;
            for (int m = 0; m < nsurf; m++) {
                ga.ns[m] = dims[m].ns;
                ga.nc[m] = dims[m].nc;
                ga.poff[m] = poff[m];
                ga.vinit[m] = vinit[m];
                ga.colloc_h[m] = colloc_h[m];
            }
            ga.poff[nsurf] = poff[nsurf];
            ga.T = tdev.p;
            ga.Td = tddev.p;
            ga.inst = inst_buf.p;
            k_hb_geom<<<dim3((unsigned)cdiv(n, 128), (unsigned)ninst), 128, 0, st>>>(ga);
            GB_LAUNCH_CHECK();
        }
        int64_t gwo = 0;
        for (int c = 0; c < K; c++) {
            HbCol& col = cols[c];
            col.inst.assign(N, Inst());
            for (int q = 0; q < N; q++) {
                const int64_t e = (int64_t)c * N + q;
                Inst& I = col.inst[q];
                I.t_steps = t_steps[e];
                I.t = times[e];
                GB_REQUIRE(I.t_steps >= 0 && I.t_steps <= col.max_t - 1,
                           "column %d instance %d: t_steps %lld outside the wake", c, q, (long long)I.t_steps);
                double* base = inst_buf.p + e * 7 * n;
                I.colloc.resize(nsurf);
                I.normals.resize(nsurf);
                I.gwake.assign(nsurf, nullptr);
                for (int m = 0; m < nsurf; m++) {
                    I.colloc[m] = base + 3 * poff[m];
                    I.normals[m] = base + 3 * n + 3 * poff[m];
                }
                I.rhs_vel = base + 6 * n;
                I.gwake[wake_surf] = gwake_buf.p + gwo;
                gwo += W.ns * (col.max_t - 1);
            }
        }
        // the operator's instance table and basis rows
        int64_t rows = 0;
        for (const HbCol& col : cols)
            for (const Inst& I : col.inst) rows += std::max<int64_t>(I.t_steps, 1);
        if ((rc = wop_basis.grow(rows * N)) || (rc = wop_basis_f2.grow(2 * rows * N))) return rc;
        if (d_wop_cap < (size_t)ninst) {
            if (d_wop) cudaFree(d_wop);
            d_wop = nullptr;
            d_wop_cap = 0;
            GB_CUDA(cudaMalloc((void**)&d_wop, sizeof(WopInst) * ninst));
            d_wop_cap = ninst;
        }
        wtab.assign(ninst, WopInst());
        int64_t off = 0;
        for (int c = 0; c < K; c++)
            for (int q = 0; q < N; q++) {
                const Inst& I = cols[c].inst[q];
                WopInst& w = wtab[(int64_t)c * N + q];
                memset(&w, 0, sizeof(w));
                for (int m = 0; m < nsurf; m++) {
                    w.colloc[m] = I.colloc[m];
                    w.normals[m] = I.normals[m];
                }
                w.rhs_vel = I.rhs_vel;
                w.wake = cols[c].wake[wake_surf];
                w.basis = wop_basis.p + off * N;
                w.it = I.t_steps;
                w.nwv = cols[c].max_t;
                w.np0 = dims[0].ns * dims[0].nc;
                w.t = I.t;
                off += std::max<int64_t>(I.t_steps, 1);
            }
        GB_CUDA(cudaStreamSynchronize(st));
        return GBVLM_OK;
    }

    // the wake term through the precomputed operator unless
    // GBVLM_HB_DIRECT=1 asks for the per-map Biot-Savart sums
    bool use_wop() const {
        const char* e = getenv("GBVLM_HB_DIRECT");
        return !(e && e[0] == '1');
    }

    // basis rows, ring values contracted with them per slice of wake rows,
    // and the slice sums, for every instance of every column (each with its
    // column's omega and dt)
    int build_wop(const double* omega, const double* dt, cudaStream_t st) {
        const gbvlm_dims& W = dims[wake_surf];
        const int64_t ninst = (int64_t)K * N;
        const int64_t npairs = n * W.ns, xb = cdiv(npairs, WOP_THREADS);
        // each instance's rows in about `hbvlm.waves` waves' worth of slices
        // of one instance (at least `hbvlm.min_rows` rows each): its partial
        // sums, and so its result, do not depend on the other sets of the batch
        const TuneParams tp = tune();
        const int64_t slices = std::max<int64_t>(1, cdiv(tp.hbvlm_waves * sm_count(), xb));
        int64_t max_it = 1;
        for (int64_t e = 0; e < ninst; e++) {
            wtab[e].omega = omega[e / N];
            wtab[e].dt = dt[e / N];
            wtab[e].rps = std::max<int64_t>(tp.hbvlm_min_rows, cdiv(wtab[e].it, slices));
            max_it = std::max(max_it, wtab[e].it);
        }
        const int64_t zs = std::min(slices, cdiv(max_it, tp.hbvlm_min_rows));
        GB_CUDA(cudaMemcpyAsync(d_wop, wtab.data(), sizeof(WopInst) * ninst, cudaMemcpyHostToDevice, st));
        WopArgs a;
        a.inst = d_wop;
        a.nsurf = nsurf;
        a.N = N;
        a.H = (N - 1) / 2;
        for (int m = 0; m <= nsurf; m++) a.poff[m] = poff[m];
        a.wns = W.ns;
        const int64_t len = ninst * npairs * N;
        int rc;
        if ((rc = wop_part.grow((size_t)(zs * len))) || (rc = wop_M.grow((size_t)len))) return rc;
        a.partial = wop_part.p;
        a.basis_f2 = wop_basis_f2.p;
        a.basis0 = wop_basis.p;
        // each instance's wake relative to its origin, as float pairs
        std::vector<int64_t> soff(ninst);
        int64_t stot = 0, maxv = 1;
        for (int64_t e = 0; e < ninst; e++) {
            soff[e] = stot;
            const int64_t nv = (W.ns + 1) * wtab[e].nwv;
            stot += 6 * nv;
            maxv = std::max(maxv, nv);
        }
        if ((rc = wop_shift.grow((size_t)stot)) || (rc = wop_shift_off.grow((size_t)ninst))) return rc;
        GB_CUDA(cudaMemcpyAsync(wop_shift_off.p, soff.data(), sizeof(int64_t) * ninst, cudaMemcpyHostToDevice, st));
        k_wake_shift<<<dim3((unsigned)cdiv(maxv, 256), (unsigned)ninst), 256, 0, st>>>(d_wop, W.ns, wop_shift.p,
                                                                                       wop_shift_off.p);
        GB_LAUNCH_CHECK();
        a.wshift = wop_shift.p;
        a.wshift_off = wop_shift_off.p;
        k_hb_basis<<<dim3((unsigned)cdiv(max_it, 128), (unsigned)ninst), 128, 0, st>>>(a);
        GB_LAUNCH_CHECK();
        for (a.c0 = 0; a.c0 < N; a.c0 += WOP_NMAX) {  // the ring values again for each block of coefficients
            k_wake_operator<<<dim3((unsigned)xb, (unsigned)ninst, (unsigned)zs), WOP_THREADS, 0, st>>>(a);
            GB_LAUNCH_CHECK();
        }
        k_wake_operator_sum<<<(unsigned)cdiv(len, 256), 256, 0, st>>>(wop_part.p, zs, len, wop_M.p);
        GB_LAUNCH_CHECK();
        wop_valid = true;
        return GBVLM_OK;
    }

    // one fixed-point map of every column on device buffers Xin -> Xout
    // (libhbvlm3.cpp:349-410); omega and dt per column
    int map_dev(const double* omega, const double* dt, cudaStream_t st) {
        gbvlm_stream s = (gbvlm_stream)st;
        int rc;
        const int32_t harmonics = (N - 1) / 2;
        const gbvlm_dims& W = dims[wake_surf];
        const int64_t te_off = poff[wake_surf] + (W.nc - 1) * W.ns;
        if (use_wop()) {
            bool same = wop_valid;
            for (int c = 0; c < K && same; c++)
                same = wtab[(int64_t)c * N].omega == omega[c] && wtab[(int64_t)c * N].dt == dt[c];
            if (!same && (rc = build_wop(omega, dt, st))) return rc;
            double* Y = n <= HB_INV_MAX ? R.p : Xout.p;
            k_hb_rhs<<<dim3((unsigned)n, (unsigned)K), HBR_THREADS, 0, st>>>(d_wop, wop_M.p, Xin.p, n, te_off, W.ns,
                                                                             N, D.p, Y);
            GB_LAUNCH_CHECK();
            if (n <= HB_INV_MAX) {
                const int64_t cols = (int64_t)K * N;
                k_hb_inv_apply<<<(unsigned)cdiv(n * cols, 128), 128, 0, st>>>(ainv.p, R.p, n, cols, Xout.p);
                GB_LAUNCH_CHECK();
                return GBVLM_OK;
            }
        } else {
            for (int c = 0; c < K; c++) {
                HbCol& col = cols[c];
                const double* Xc = Xin.p + (int64_t)c * n * N;
                double* tec = te.p + (int64_t)c * W.ns * N;
                double* Rc = R.p + (int64_t)c * n * N;
                k_gather_te<<<(unsigned)cdiv(W.ns * N, 128), 128, 0, st>>>(Xc, n, te_off, W.ns, N, tec);
                GB_LAUNCH_CHECK();
                for (int q = 0; q < N; q++) {
                    Inst& I = col.inst[q];
                    if ((rc = gbvlm_gamma_wake_from_coeffs_f64(I.gwake[wake_surf], W.ns, col.max_t - 1, tec,
                                                                harmonics, I.t, omega[c], dt[c], I.t_steps, s)))
                        return rc;
                    double* rcol = Rc + (int64_t)q * n;
                    GB_CUDA(cudaMemcpyAsync(rcol, I.rhs_vel, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
                    if ((rc = gbvlm_rhs_assemble_wake_influence_f64(rcol, nsurf, col.dims.data(), C(I.gwake).data(),
                                                                    C(I.colloc).data(), C(I.normals).data(),
                                                                    C(col.wake).data(), lifting.data(),
                                                                    (int32_t)I.t_steps, 0.0, s)))
                        return rc;
                }
                k_rdft<<<(unsigned)cdiv(n * N, 128), 128, 0, st>>>(Rc, D.p + (int64_t)c * N * N, n, N,
                                                                   Xout.p + (int64_t)c * n * N);
                GB_LAUNCH_CHECK();
            }
        }
        return gbvlm_lu_solve_f64(lu, lhs, n, n, Xout.p, n, (int64_t)K * N, s);
    }
};

// ---------------------------------------------------------------------------
// Anderson acceleration on the device (vlm/src/vlm_solvers.cpp:6-115): the
// iterate, residuals and the m-column histories X (iterate steps) and G
// (residual steps) stay in device memory; one CTA solves the small least
// squares min |G[:, :mk] gam - g| by Householder QR (reflector columns in
// a work copy of G, the right-hand side reflected alongside, then back
// substitution) and forms the next iterate; the host reads one norm per
// iteration.  Columns are L = n * N long (a few hundred to a few thousand).
// ---------------------------------------------------------------------------
constexpr int AA_THREADS = 512;

__device__ double aa_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();  // sh free (previous sum read)
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];
    return r;
}

// sum over one warp, every lane gets it
__device__ __forceinline__ double aa_wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// x_new = x + g - sum_j (X_j + G_j) gam_j with gam the least-squares
// coefficients of G[:, :mk]; X[:, slot] = x_new - x; x = x_new (in place).
// The CTA copies G[:, :mk] and g into shared memory (or, when they do not
// fit, into the global work buffers) and runs the Householder QR there:
// for each column j, warp 0 forms the reflector (its norm, the new pivot,
// v^T v = 2 |a| (|a| + |a_j|)), then the warps reflect the later columns
// and the right-hand side in parallel, one column per warp at a time.  The
// QR runs in float pairs on the fp32 pipe (one CTA's fp64 units made it a
// 68 us step); the least-squares coefficients and the new iterate are
// formed in double.
constexpr int AA_STEP_THREADS = 256;

// Per column c = blockIdx.x (its state at buf + c * stride: g (L), the
// histories X and G (L x m each), the QR work copy W (L x m) and its
// right-hand side b (L)); columns with act[c] == 0 are left as they are.
struct AaCol {
    double *g, *X, *G, *W, *b;
};
__device__ __forceinline__ AaCol aa_col(double* buf, int64_t L, int m) {
    double* g = buf + (int64_t)blockIdx.x * L * (3 * m + 2);
    return AaCol{g, g + L, g + L + L * m, g + L + 2 * L * m, g + L + 3 * L * m};
}

__global__ void __launch_bounds__(AA_STEP_THREADS) k_anderson_step(int64_t L, int m, int mk, int slot, double* buf,
                                                                   double* xall, const int* act, int use_smem,
                                                                   const int* kdev) {
    if (!act[blockIdx.x]) return;
    if (kdev) {  // the iteration k from device memory (the loop's graph): mk = min(m, k), slot = k mod m
        const int k = *kdev;
        mk = min(m, k);
        slot = k % m;
    }
    extern __shared__ double aa_sm[];
    __shared__ double gam[16];
    __shared__ F2 gamf[16], diag[16];
    __shared__ F2 s_nrm, s_rvv;
    const AaCol cs = aa_col(buf, L, m);
    double* X = cs.X;
    const double* G = cs.G;
    const double* g = cs.g;
    double* x = xall + (int64_t)blockIdx.x * L;
    // the QR's work copy of G[:, :mk] and its right-hand side, as float pairs
    F2* W = reinterpret_cast<F2*>(use_smem ? aa_sm : cs.W);
    F2* b = reinterpret_cast<F2*>(use_smem ? aa_sm + L * mk : cs.b);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    for (int64_t e = tid; e < L * mk; e += blockDim.x) W[e] = f2_of(G[e]);
    for (int64_t i = tid; i < L; i += blockDim.x) b[i] = f2_of(g[i]);
    // dot products over rows j..L-1: four partial sums per lane, reduced
    // down the warp and broadcast from lane 0
    auto dot = [&](const F2* u, const F2* w, int j) {
        F2 t0{0.f, 0.f}, t1{0.f, 0.f}, t2{0.f, 0.f}, t3{0.f, 0.f};
        int64_t i = j + lane;
        for (; i + 96 < L; i += 128) {
            t0 = f2_add(t0, f2_mul(u[i], w[i]));
            t1 = f2_add(t1, f2_mul(u[i + 32], w[i + 32]));
            t2 = f2_add(t2, f2_mul(u[i + 64], w[i + 64]));
            t3 = f2_add(t3, f2_mul(u[i + 96], w[i + 96]));
        }
        for (; i < L; i += 32) t0 = f2_add(t0, f2_mul(u[i], w[i]));
        F2 t = f2_add(f2_add(t0, t1), f2_add(t2, t3));
        for (int o = 16; o > 0; o >>= 1)
            t = f2_add(t, F2{__shfl_down_sync(0xffffffffu, t.h, o), __shfl_down_sync(0xffffffffu, t.l, o)});
        return F2{__shfl_sync(0xffffffffu, t.h, 0), __shfl_sync(0xffffffffu, t.l, 0)};
    };
    __syncthreads();
    for (int j = 0; j < mk; j++) {
        F2* wj = W + (int64_t)j * L;
        if (wid == 0) {
            const F2 nrm = f2_sqrt(dot(wj, wj, j));
            if (lane == 0) {
                s_nrm = nrm;
                diag[j] = F2{0.f, 0.f};
                if (nrm.h != 0.f) {
                    const F2 a0 = wj[j];
                    const F2 alpha = a0.h > 0.f ? f2_neg(nrm) : nrm;
                    wj[j] = f2_sub(a0, alpha);
                    diag[j] = alpha;
                    const F2 aa = a0.h < 0.f ? f2_neg(a0) : a0;
                    s_rvv = f2_div(F2{1.f, 0.f}, f2_mulf(f2_mul(nrm, f2_add(nrm, aa)), 2.f));
                }
            }
        }
        __syncthreads();
        if (s_nrm.h != 0.f) {  // uniform
            const F2 rvv = s_rvv;
            for (int t = wid; t < mk - j; t += nw) {  // the later columns, then the right-hand side
                F2* wc = t < mk - j - 1 ? W + (int64_t)(j + 1 + t) * L : b;
                const F2 f = f2_mulf(f2_mul(dot(wj, wc, j), rvv), 2.f);
                for (int64_t i = j + lane; i < L; i += 32) wc[i] = f2_sub(wc[i], f2_mul(f, wj[i]));
            }
        }
        __syncthreads();
    }
    if (tid == 0)
        for (int j = mk - 1; j >= 0; j--) {
            F2 sj = b[j];
            for (int c = j + 1; c < mk; c++) sj = f2_sub(sj, f2_mul(W[j + (int64_t)c * L], gamf[c]));
            gamf[j] = diag[j].h != 0.f ? f2_div(sj, diag[j]) : F2{0.f, 0.f};
            gam[j] = f2_dbl(gamf[j]);
        }
    __syncthreads();
    for (int64_t i = tid; i < L; i += blockDim.x) {
        double v = x[i] + g[i];
        for (int j = 0; j < mk; j++) v -= (X[i + (int64_t)L * j] + G[i + (int64_t)L * j]) * gam[j];
        X[i + (int64_t)L * slot] = v - x[i];
        x[i] = v;
    }
}

// after a map: g_new = f(x) - x; G[:, slot] = g_new - g (slot < 0: none);
// g = g_new; *norm = |g|
__global__ void __launch_bounds__(AA_THREADS) k_anderson_post(int64_t L, int m, int slot, const double* fxall,
                                                              const double* xall, double* buf, double* norm,
                                                              const int* act, const int* kdev) {
    if (!act[blockIdx.x]) return;
    if (kdev) slot = *kdev % m;
    __shared__ double sh[32];
    const AaCol cs = aa_col(buf, L, m);
    double* g = cs.g;
    double* G = cs.G;
    const double* fx = fxall + (int64_t)blockIdx.x * L;
    const double* x = xall + (int64_t)blockIdx.x * L;
    double t = 0;
    for (int64_t i = threadIdx.x; i < L; i += blockDim.x) {
        const double gn = fx[i] - x[i];
        if (slot >= 0) G[i + (int64_t)L * slot] = gn - g[i];
        g[i] = gn;
        t += gn * gn;
    }
    const double s2 = aa_sum(t, sh);
    if (threadIdx.x == 0) norm[blockIdx.x] = sqrt(s2);
}

// the first step (vlm_solvers.cpp:49-66): X[:, 0] = g, x = f(x); grid y: column
__global__ void k_anderson_first(int64_t L, int m, const double* fxall, double* xall, double* buf) {
    const int64_t c = blockIdx.y;
    const double* g = buf + c * L * (3 * m + 2);
    double* X = const_cast<double*>(g) + L;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L; i += (int64_t)gridDim.x * blockDim.x) {
        X[i] = g[i];
        xall[c * L + i] = fxall[c * L + i];
    }
}

// the loop's test (vlm_solvers.cpp:68-70) per column: a column whose
// residual norm is no longer above tol stops at iteration k; ctl[0] = the
// number still iterating
__global__ void k_anderson_check(int K, const double* norm, double tol, int k, int* act, int* iters, int* ctl) {
    int live = 0;
    for (int c = threadIdx.x; c < K; c += blockDim.x) {
        if (act[c] && !(norm[c] > tol)) {
            act[c] = 0;
            iters[c] = k;
        }
        live += act[c];
    }
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if (threadIdx.x == 0) ctl[0] = live;
}

// The loop's test inside its graph: ctl[0] = k (incremented first when
// `advance`), then k_anderson_check's test, and the while node continues
// while some set iterates and k < max_iter
__global__ void k_anderson_graph_test(int K, const double* norm, double tol, int max_iter, int* act, int* iters,
                                      int* ctl, int advance, cudaGraphConditionalHandle loop) {
    const int k = ctl[0] + (advance ? 1 : 0);
    int live = 0;
    for (int c = threadIdx.x; c < K; c += blockDim.x) {
        if (act[c] && !(norm[c] > tol)) {
            act[c] = 0;
            iters[c] = k;
        }
        live += act[c];
    }
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    __syncwarp();
    if (threadIdx.x == 0) {
        ctl[0] = k;
        ctl[1] = live;
        cudaGraphSetConditional(loop, (live > 0 && k < max_iter) ? 1u : 0u);
    }
}

// columns still iterating after max_iter steps report max_iter
__global__ void k_anderson_finish(int K, int k, const int* act, int* iters, const int* kdev) {
    if (kdev) k = *kdev;
    for (int c = threadIdx.x; c < K; c += blockDim.x)
        if (act[c]) iters[c] = k;
}

__global__ void k_fill_i32(int* p, int n, int v) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = v;
}

// The Anderson loop of gbvlm_hbvlm_solve_batch as one graph: a test node
// (k = 1), then a while node whose body is the step, the map (k_hb_rhs,
// k_hb_inv_apply), the residual update and the next test, which sets the
// loop condition on the device.  k lives in ctl[0]; nothing returns to the
// host until the loop ends.
static int anderson_graph(HbState& S, int K, int64_t L, int m, int max_iter, double tol, double* buf, double* dnorm,
                          int* act, int* iters, int* ctl, int use_smem, size_t smem) {
    const gbvlm_dims& W = S.dims[S.wake_surf];
    const int64_t te_off = S.poff[S.wake_surf] + (W.nc - 1) * W.ns;
    struct Key {
        const void* p[12];
        int64_t v[8];
        double tol;
    } key;
    memset(&key, 0, sizeof(key));
    const void* ps[12] = {buf, dnorm, act, iters, ctl, S.d_wop, S.wop_M.p, S.Xin.p, S.D.p, S.R.p, S.ainv.p, S.Xout.p};
    memcpy(key.p, ps, sizeof(ps));
    const int64_t vs[8] = {K, L, m, max_iter, use_smem, (int64_t)smem, S.n, S.N};
    memcpy(key.v, vs, sizeof(vs));
    key.tol = tol;
    if (S.aa_exec && S.aa_key.size() == sizeof(key) && memcmp(S.aa_key.data(), &key, sizeof(key)) == 0)
        return GBVLM_OK;
    if (S.aa_exec) cudaGraphExecDestroy(S.aa_exec);
    if (S.aa_graph) cudaGraphDestroy(S.aa_graph);
    S.aa_exec = nullptr;
    S.aa_graph = nullptr;
    S.aa_key.clear();
    if (!S.aa_cap) GB_CUDA(cudaStreamCreateWithFlags(&S.aa_cap, cudaStreamNonBlocking));
    GB_CUDA(cudaGraphCreate(&S.aa_graph, 0));
    cudaGraphConditionalHandle loop;
    GB_CUDA(cudaGraphConditionalHandleCreate(&loop, S.aa_graph, 0, cudaGraphCondAssignDefault));
    cudaGraphNode_t nh, nw;
    {
        int adv = 0;
        void* args[] = {&K, &dnorm, &tol, &max_iter, &act, &iters, &ctl, &adv, &loop};
        cudaKernelNodeParams kp = {};
        kp.func = (void*)k_anderson_graph_test;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(32);
        kp.kernelParams = args;
        GB_CUDA(cudaGraphAddKernelNode(&nh, S.aa_graph, nullptr, 0, &kp));
    }
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    GB_CUDA(cudaGraphAddNode(&nw, S.aa_graph, &nh, nullptr, 1, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    cudaStream_t cs = S.aa_cap;
    GB_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const int64_t cols = (int64_t)K * S.N;
    k_anderson_step<<<K, AA_STEP_THREADS, use_smem ? smem : 0, cs>>>(L, m, 0, 0, buf, S.Xin.p, act, use_smem, ctl);
    k_hb_rhs<<<dim3((unsigned)S.n, (unsigned)K), HBR_THREADS, 0, cs>>>(S.d_wop, S.wop_M.p, S.Xin.p, S.n, te_off, W.ns,
                                                                       S.N, S.D.p, S.R.p);
    k_hb_inv_apply<<<(unsigned)cdiv(S.n * cols, 128), 128, 0, cs>>>(S.ainv.p, S.R.p, S.n, cols, S.Xout.p);
    k_anderson_post<<<K, AA_THREADS, 0, cs>>>(L, m, 0, S.Xout.p, S.Xin.p, buf, dnorm, act, ctl);
    k_anderson_graph_test<<<1, 32, 0, cs>>>(K, dnorm, tol, max_iter, act, iters, ctl, 1, loop);
    const cudaError_t le = cudaGetLastError();
    cudaGraph_t got = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cs, &got);
    GB_CUDA(le);
    GB_CUDA(e);
    GB_CUDA(cudaGraphInstantiate(&S.aa_exec, S.aa_graph, 0));
    S.aa_key.assign((const char*)&key, (const char*)&key + sizeof(key));
    return GBVLM_OK;
}

}  // namespace gbvlm

using namespace gbvlm;

struct gbvlm_hbvlm_s {
    HbState st;
};

extern "C" {

int gbvlm_hbvlm_create(gbvlm_hbvlm* out, int32_t nsurf, const gbvlm_dims* dims, const double* const* verts_init,
                       const int32_t* lifting) {
    GB_REQUIRE(out && dims && verts_init && lifting, "null argument");
    GB_REQUIRE(nsurf >= 1 && nsurf <= GBVLM_MAX_SURFACES, "nsurf=%d outside [1, %d]", nsurf, GBVLM_MAX_SURFACES);
    auto* h = new gbvlm_hbvlm_s();
    int rc = h->st.init(nsurf, dims, verts_init, lifting);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return GBVLM_OK;
}

int gbvlm_hbvlm_destroy(gbvlm_hbvlm h) {
    delete h;
    return GBVLM_OK;
}

int gbvlm_hbvlm_prepare(gbvlm_hbvlm h, int32_t harmonics, int64_t max_t_steps, const double* wake_transforms,
                        const int64_t* t_steps, const double* times, const double* transforms,
                        const double* dtransforms, const double* dft, gbvlm_stream stream) {
    return gbvlm_hbvlm_prepare_batch(h, 1, harmonics, &max_t_steps, &wake_transforms, t_steps, times, transforms,
                                     dtransforms, dft, stream);
}

int gbvlm_hbvlm_prepare_batch(gbvlm_hbvlm h, int32_t K, int32_t harmonics, const int64_t* max_t_steps,
                              const double* const* wake_transforms, const int64_t* t_steps, const double* times,
                              const double* transforms, const double* dtransforms, const double* dft,
                              gbvlm_stream stream) {
    GB_REQUIRE(h && max_t_steps && wake_transforms && t_steps && times && transforms && dtransforms && dft,
               "null argument");
    GB_REQUIRE(harmonics >= 0 && harmonics <= 64, "harmonics %d outside [0, 64]", harmonics);
    GB_REQUIRE(K >= 1 && (int64_t)K * (2 * harmonics + 1) <= 65535, "K=%d: K (2H+1) must be in [1, 65535]", K);
    return h->st.prepare(K, harmonics, max_t_steps, wake_transforms, nullptr, t_steps, times, transforms, dtransforms,
                         dft, to_cuda(stream));
}

int gbvlm_hbvlm_prepare_batch_chain(gbvlm_hbvlm h, int32_t K, int32_t harmonics, const int64_t* max_t_steps,
                                    const double* chain, const int64_t* t_steps, const double* times,
                                    const double* transforms, const double* dtransforms, const double* dft,
                                    gbvlm_stream stream) {
    GB_REQUIRE(h && max_t_steps && chain && t_steps && times && transforms && dtransforms && dft, "null argument");
    GB_REQUIRE(harmonics >= 0 && harmonics <= 64, "harmonics %d outside [0, 64]", harmonics);
    GB_REQUIRE(K >= 1 && (int64_t)K * (2 * harmonics + 1) <= 65535, "K=%d: K (2H+1) must be in [1, 65535]", K);
    return h->st.prepare(K, harmonics, max_t_steps, nullptr, chain, t_steps, times, transforms, dtransforms, dft,
                         to_cuda(stream));
}

int gbvlm_hbvlm_map(gbvlm_hbvlm h, const double* x_in, double* x_out, double omega, double dt, gbvlm_stream stream) {
    GB_REQUIRE(h && x_in && x_out && h->st.N > 0, "map before prepare");
    HbState& S = h->st;
    GB_REQUIRE(S.K == 1, "map needs a single parameter set (prepared K=%d)", S.K);
    cudaStream_t st = to_cuda(stream);
    GB_CUDA(cudaMemcpyAsync(S.Xin.p, x_in, sizeof(double) * S.n * S.N, cudaMemcpyHostToDevice, st));
    int rc = S.map_dev(&omega, &dt, st);
    if (rc) return rc;
    GB_CUDA(cudaMemcpyAsync(x_out, S.Xout.p, sizeof(double) * S.n * S.N, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    return GBVLM_OK;
}

int gbvlm_hbvlm_solve(gbvlm_hbvlm h, double* x, double omega, double dt, int32_t max_iter, double tol, int32_t m,
                      int32_t* iters, gbvlm_stream stream) {
    GB_REQUIRE(h && h->st.K == 1, "solve needs a single parameter set");
    return gbvlm_hbvlm_solve_batch(h, 1, x, &omega, &dt, max_iter, tol, m, iters, stream);
}

int gbvlm_hbvlm_solve_batch(gbvlm_hbvlm h, int32_t K, double* x, const double* omega, const double* dt,
                            int32_t max_iter, double tol, int32_t m, int32_t* iters, gbvlm_stream stream) {
    GB_REQUIRE(h && x && omega && dt && h->st.N > 0, "solve before prepare");
    GB_REQUIRE(K == h->st.K, "K=%d differs from the prepared %d parameter sets", K, h->st.K);
    GB_REQUIRE(m >= 1 && m <= 16 && max_iter >= 2, "history m in [1, 16], max_iter >= 2");
    HbState& S = h->st;
    cudaStream_t st = to_cuda(stream);
    const int64_t L = S.n * S.N;
    // device state: the iterates live in the map's input S.Xin; per column
    // g, the histories X and G, the QR work copy of G and its right-hand
    // side; then the residual norms and the loop's flags
    const size_t per = (size_t)L * (3 * m + 2);
    int rc = S.aa_buf.grow(per * K + K + (2 * K + 4 + 1) / 2);
    if (rc) return rc;
    double* buf = S.aa_buf.p;
    double* dnorm = buf + per * K;
    int* act = (int*)(dnorm + K);
    int* d_iters = act + K;
    int* ctl = d_iters + K;
    int* hctl = (int*)host_scratch(sizeof(int));
    auto check = [&](const char* what) {
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? GBVLM_OK : cuda_fail(e, what, __FILE__, __LINE__);
    };
    auto map = [&]() { return S.map_dev(omega, dt, st); };  // S.Xin -> S.Xout, every column
    const unsigned g1 = (unsigned)std::min<int64_t>(cdiv(L, 256), 1024);
    if (cudaMemcpyAsync(S.Xin.p, x, sizeof(double) * L * K, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(buf, 0, sizeof(double) * per * K, st) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "Anderson setup", __FILE__, __LINE__);
    k_fill_i32<<<1, 256, 0, st>>>(act, K, 1);
    k_fill_i32<<<1, 256, 0, st>>>(d_iters, K, 0);
    // vlm_solvers.cpp:49-66: g0 = f(x0) - x0; X0 = g0; x1 = f(x0); g1 = f(x1) - x1; G0 = g1 - g0
    if ((rc = map())) return rc;
    k_anderson_post<<<K, AA_THREADS, 0, st>>>(L, m, -1, S.Xout.p, S.Xin.p, buf, dnorm, act, nullptr);
    k_anderson_first<<<dim3(g1, K), 256, 0, st>>>(L, m, S.Xout.p, S.Xin.p, buf);
    if ((rc = check("Anderson")) || (rc = map())) return rc;
    k_anderson_post<<<K, AA_THREADS, 0, st>>>(L, m, 0, S.Xout.p, S.Xin.p, buf, dnorm, act, nullptr);
    if ((rc = check("Anderson"))) return rc;
    // the QR's columns in shared memory when m of them and g fit
    const size_t smem = sizeof(double) * (size_t)L * (m + 1);
    const int use_smem = smem <= 200 * 1024 ? 1 : 0;
    if (use_smem && cudaFuncSetAttribute(k_anderson_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                        cudaSuccess)
        return cuda_fail(cudaGetLastError(), "cudaFuncSetAttribute", __FILE__, __LINE__);
    int k = 1;
    if (S.anderson_graph_ok()) {  // the whole loop on the device
        k_fill_i32<<<1, 32, 0, st>>>(ctl, 1, 1);
        if ((rc = anderson_graph(S, K, L, m, max_iter, tol, buf, dnorm, act, d_iters, ctl, use_smem, smem)))
            return rc;
        GB_CUDA(cudaGraphLaunch(S.aa_exec, st));
        k = max_iter;  // the host loop below does not run
    }
    while (k < max_iter) {
        k_anderson_check<<<1, 32, 0, st>>>(K, dnorm, tol, k, act, d_iters, ctl);
        if (cudaMemcpyAsync(hctl, ctl, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return cuda_fail(cudaGetLastError(), "Anderson norm", __FILE__, __LINE__);
        if (*hctl == 0) break;
        const int mk = std::min(m, k), slot = k % m;
        k_anderson_step<<<K, AA_STEP_THREADS, use_smem ? smem : 0, st>>>(L, m, mk, slot, buf, S.Xin.p, act,
                                                                          use_smem, nullptr);
        if ((rc = check("Anderson")) || (rc = map())) return rc;
        k_anderson_post<<<K, AA_THREADS, 0, st>>>(L, m, slot, S.Xout.p, S.Xin.p, buf, dnorm, act, nullptr);
        if ((rc = check("Anderson"))) return rc;
        k++;
    }
    k_anderson_finish<<<1, 256, 0, st>>>(K, k, act, d_iters, S.anderson_graph_ok() ? ctl : nullptr);
    std::vector<int> hit(K);
    if (cudaMemcpyAsync(x, S.Xin.p, sizeof(double) * L * K, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(hit.data(), d_iters, sizeof(int) * K, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "cudaMemcpyAsync", __FILE__, __LINE__);
    if (iters)
        for (int c = 0; c < K; c++) iters[c] = hit[c];
    return GBVLM_OK;
}

// libhbvlm3.cpp:428-550: loads at the force instances.  coeffs (n x N),
// dft / ddft (N x N), per instance transforms/rates (N x nsurf x 16),
// freestream (N x 3), ref_a / ref_b (N x 3; ref_b may be NULL).  out: 3 x N
// row-major [cl; cm_y about ref_a (multibody); cm_y of surface 1 about ref_b].
int gbvlm_hbvlm_loads(gbvlm_hbvlm h, const double* coeffs, const double* dft, const double* ddft,
                      const double* transforms, const double* dtransforms, const double* freestream,
                      const double* ref_a, const double* ref_b, int32_t coupled_te, double* out, gbvlm_stream stream) {
    return gbvlm_hbvlm_loads_batch(h, 1, coeffs, dft, ddft, transforms, dtransforms, freestream, ref_a, ref_b,
                                   coupled_te, out, stream);
}

int gbvlm_hbvlm_loads_batch(gbvlm_hbvlm h, int32_t K, const double* coeffs, const double* dft, const double* ddft,
                            const double* transforms, const double* dtransforms, const double* freestream,
                            const double* ref_a, const double* ref_b, int32_t coupled_te, double* out,
                            gbvlm_stream stream) {
    GB_REQUIRE(h && coeffs && dft && ddft && transforms && dtransforms && freestream && ref_a && out, "null argument");
    HbState& S = h->st;
    GB_REQUIRE(S.N > 0 && S.aic_ready, "loads before prepare");
    GB_REQUIRE(K >= 1 && (int64_t)K * S.N <= 2147483647, "bad K=%d", K);
    cudaStream_t st = to_cuda(stream);
    const int64_t N = S.N, ninst = (int64_t)K * N, nt = ninst * S.nsurf * 16;
    int rc;
    if ((rc = S.ld_C.grow(ninst * S.n)) || (rc = S.ld_D.grow(ninst * N)) || (rc = S.ld_DD.grow(ninst * N)) ||
        (rc = S.ld_T.grow(nt)) || (rc = S.ld_Td.grow(nt)) || (rc = S.ld_fs.grow(ninst * 3)) ||
        (rc = S.ld_ra.grow(ninst * 3)) || (rc = S.ld_rb.grow(ninst * 3)) || (rc = S.ld_out.grow(ninst * 3)))
        return rc;
    GB_CUDA(cudaMemcpyAsync(S.ld_C.p, coeffs, sizeof(double) * ninst * S.n, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(S.ld_D.p, dft, sizeof(double) * ninst * N, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(S.ld_DD.p, ddft, sizeof(double) * ninst * N, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(S.ld_T.p, transforms, sizeof(double) * nt, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(S.ld_Td.p, dtransforms, sizeof(double) * nt, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(S.ld_fs.p, freestream, sizeof(double) * ninst * 3, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(S.ld_ra.p, ref_a, sizeof(double) * ninst * 3, cudaMemcpyHostToDevice, st));
    if (ref_b) GB_CUDA(cudaMemcpyAsync(S.ld_rb.p, ref_b, sizeof(double) * ninst * 3, cudaMemcpyHostToDevice, st));
    LoadsArgs a;
    memset(&a, 0, sizeof(a));
    a.nsurf = S.nsurf;
    a.N = (int32_t)N;
    a.coupled = coupled_te ? 1 : 0;
    a.n = S.n;
    for (int m = 0; m < S.nsurf; m++) {
        a.ns[m] = S.dims[m].ns;
        a.nc[m] = S.dims[m].nc;
        a.poff[m] = S.poff[m];
        a.vinit[m] = S.vinit[m];
        a.colloc_h[m] = S.colloc_h[m];
    }
    a.poff[S.nsurf] = S.poff[S.nsurf];
    a.C = S.ld_C.p;
    a.D = S.ld_D.p;
    a.DD = S.ld_DD.p;
    a.T = S.ld_T.p;
    a.Td = S.ld_Td.p;
    a.fs = S.ld_fs.p;
    a.ref_a = S.ld_ra.p;
    a.ref_b = ref_b ? S.ld_rb.p : nullptr;
    a.out = S.ld_out.p;
    k_hb_loads<<<(unsigned)ninst, HBL_THREADS, 0, st>>>(a);
    GB_LAUNCH_CHECK();
    GB_CUDA(cudaMemcpyAsync(out, S.ld_out.p, sizeof(double) * ninst * 3, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    return GBVLM_OK;
}

}  // extern "C"
