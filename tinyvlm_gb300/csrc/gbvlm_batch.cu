// Batched steady VLM: many single-surface cases of uneven size, each with
// several angles of attack, solved in one CUDA graph.
//
// Per system (one AIC):
//   geometry  (double)  wake ring 100 u_inf chords along the freestream of
//                       the system's geometry angle, collocation points with
//                       the high-AoA factor, normals, areas
//                       (vlm/src/vlm.cpp:97-116, vlm_backend_cpu.cpp:391-433);
//                       positions stored as float hi/lo pairs
//   assembly  (float)   AIC from relative vectors formed in double-float, so
//                       input rounding does not enter (vlm_backend_cpu.cpp:84-148);
//                       the double kernel's cut-offs (ispc:393), since the
//                       path solves the FP64 system
//   factor    (float)   variable-size batched LU (gbvlm_lu.cu)
//   solve     (float + double refinement) residual b - A x in double against
//                       an unfactored copy of A
//   loads     (double)  Joukowski forces, CL, CM (compensated sums), Trefftz
//                       CDi (vlm_backend_cpu.cpp:276-362, ispc:273-323)
//
// Two ways to map angles to systems:
//   GBVLM_BATCH_EXACT : one system per (case, alpha) with the reference's
//                       alpha-dependent geometry (VLM::run semantics);
//   GBVLM_BATCH_SHARED: one system per case, geometry at alpha = 0 (wake
//                       along +x, collocation factor 1/2), every alpha a
//                       right-hand side V_inf(alpha) of the same AIC.
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "gbvlm_internal.h"
#include "gbvlm_lu.h"
#include "gbvlm_math.cuh"
#include "gbvlm_walk.cuh"

namespace gbvlm {

// device description of one system (all pointers into the batch arena)
struct SysDesc {
    int64_t ns, nc, n;
    int32_t case_id, nrhs;
    int32_t rhs_off;        // first solve index of this system (alphas / outputs)
    double alpha_geom;      // angle that shapes the geometry
    const float* vinit;     // case vertices (4, nc+1, ns+1) float, quarter-chord shifted
    float* vh;              // wing vertex hi (3 planes)
    float* vl;              // wing vertex lo
    float* wh;              // wake vertex hi (3 planes, 2 rows)
    float* wl;
    float* ch;              // colloc hi (3 planes)
    float* cl_;             // colloc lo
    float* nrm;             // normals float (3 planes)
    double* area;           // panel areas
    double* vd;             // wing vertices double (3 planes)
    double* wd;             // wake vertices double (3 planes, 2 rows) in the wake's frame (x along the wake;
                            // the Trefftz influence only)
    double* nrmd;           // normals double
    float* A;               // AIC (factored in place)
    float* A2;              // unfactored copy (refinement), may be null
    float* Alo;             // A64 - A2, the stored AIC's correction (FP64 residual plans), may be null
    int32_t* ipiv;
    float* X;               // float rhs / solutions (n x nrhs)
    double* B;              // double rhs (n x nrhs)
    double* Xd;             // double solution
    double* R;              // double residual
    double* K;              // Trefftz influence (ns x ns) of unit wake gammas
};

struct BatchArgs {
    SysDesc* sys;
    int32_t nsys;
    const double* alphas;   // per solve
    double u_inf, rho, beta;
    double ref[3];
    double* out;            // per solve in the caller's order: cl, cdi, cmx, cmy, cmz
    float* gamma_out;       // per solve, n floats at goff[solve] (the caller's order; may be null)
    const int64_t* goff;
    const int32_t* uidx;    // batch solve -> the caller's solve index
    int32_t* bad;           // per system: 1 if its case's vertices hold a non-finite coordinate
};

__device__ __forceinline__ void split_hl(double x, float& h, float& l) {
    h = (float)x;
    l = (float)(x - (double)h);
}

// ---------------------------------------------------------------------------
// geometry: one block per system
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_batch_geom(BatchArgs a) {
    SysDesc& S = a.sys[blockIdx.x];
    const int64_t ns = S.ns, nc = S.nc, nv = (ns + 1) * (nc + 1), np = ns * nc;
    const double al = S.alpha_geom;
    int bad = 0;
    for (int64_t v = threadIdx.x; v < nv; v += blockDim.x) {
        for (int k = 0; k < 3; k++) {
            double x = (double)S.vinit[k * nv + v];
            bad |= !isfinite(x);
            S.vd[k * nv + v] = x;
            split_hl(x, S.vh[k * nv + v], S.vl[k * nv + v]);
        }
    }
    // a case with a non-finite coordinate is reported by gbvlm_batch_results
    // (its solves come out non-finite; the other cases are unaffected)
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) a.bad[blockIdx.x] = bad;
    // the angle's double trigonometry once per block (long on the fp64 units)
    __shared__ double s_trig[5];
    if (threadIdx.x == 0) {
        const double sa = sin(al), ca = cos(al);
        s_trig[0] = 100.0 * a.u_inf * ca;
        s_trig[1] = 100.0 * a.u_inf * sa;
        s_trig[2] = (al < (double)EPS_F) ? 0.5 : 0.5 * (al / (sa + (double)EPS_F));
        s_trig[3] = ca;
        s_trig[4] = sa;
    }
    __syncthreads();
    // wake (vlm.cpp:104-114 seen from the displaced wing): row 0 = trailing
    // edge, row 1 = trailing edge + 100 u (cos a, 0, sin a)
    const double dx = s_trig[0], dz = s_trig[1], ca = s_trig[3], sa = s_trig[4];
    const int64_t wl = 2 * (ns + 1);
    for (int64_t i = threadIdx.x; i <= ns; i += blockDim.x) {
        const int64_t te = i + nc * (ns + 1);
        double x = S.vinit[te], y = S.vinit[nv + te], z = S.vinit[2 * nv + te];
        double w0[3] = {x, y, z}, w1[3] = {x + dx, y, z + dz};
        for (int k = 0; k < 3; k++) {
            split_hl(w0[k], S.wh[k * wl + i], S.wl[k * wl + i]);
            split_hl(w1[k], S.wh[k * wl + (ns + 1) + i], S.wl[k * wl + (ns + 1) + i]);
        }
        // the Trefftz copy turned about y by -a, so the wake runs along x: a
        // point's offsets across the 100-chord trailing legs are then small
        // coordinates of their own, which keep float precision when the
        // Trefftz kernel rounds its relative vectors (in the wing's frame
        // they are differences of ~50-chord coordinates; identity at a = 0)
        for (int r = 0; r < 2; r++) {
            const double* q = r ? w1 : w0;
            const int64_t o = r * (ns + 1) + i;
            S.wd[o] = fma(ca, q[0], sa * q[2]);
            S.wd[wl + o] = q[1];
            S.wd[2 * wl + o] = fma(ca, q[2], -(sa * q[0]));
        }
    }
    __syncthreads();
    const double factor = s_trig[2];
    const double* v = S.vd;
    for (int64_t p = threadIdx.x; p < np; p += blockDim.x) {
        const int64_t i = p % ns, j = p / ns;
        const int64_t ia = i + j * (ns + 1), ib = ia + 1, ic = ib + (ns + 1), id = ia + (ns + 1);
        V3<double> v0{v[ia], v[nv + ia], v[2 * nv + ia]}, v1{v[ib], v[nv + ib], v[2 * nv + ib]};
        V3<double> v2{v[ic], v[nv + ic], v[2 * nv + ic]}, v3_{v[id], v[nv + id], v[2 * nv + id]};
        V3<double> nn = cross(v3_ - v1, v2 - v0);
        double l = sqrt(len2(nn));
        V3<double> n{nn.x / l, nn.y / l, nn.z / l};
        S.nrmd[p] = n.x; S.nrmd[np + p] = n.y; S.nrmd[2 * np + p] = n.z;
        S.nrm[p] = (float)n.x; S.nrm[np + p] = (float)n.y; S.nrm[2 * np + p] = (float)n.z;
        V3<double> f = v3_ - v0, b = v2 - v0, e = v1 - v0;
        S.area[p] = 0.5 * (sqrt(len2(cross(f, b))) + sqrt(len2(cross(b, e))));
        V3<double> ch = 0.5 * (((v2 + v3_) - v0) - v1);
        V3<double> cp = 0.5 * (v0 + v1) + factor * ch;
        split_hl(cp.x, S.ch[p], S.cl_[p]);
        split_hl(cp.y, S.ch[np + p], S.cl_[np + p]);
        split_hl(cp.z, S.ch[2 * np + p], S.cl_[2 * np + p]);
    }
}

// ---------------------------------------------------------------------------
// assembly: tiles (system, 128-row block, chordwise ring row, span chunk)
// ---------------------------------------------------------------------------
constexpr int BA_THREADS = 128;
// rings per span chunk: a template parameter (64, 128 or 256) chosen per
// plan from the tuning table (batch.assembly_span), 128 by default

struct HL {
    float h, l;
};

// Walk a strip of rings with double-float positions (top/bot: hi planes at
// topH[k*BA_W], lo planes at topL[k*BA_W]); f(ring, 4*pi*(v.n + v'.n')).
// seg[0][k]: the chordwise segment top(k) -> bot(k); seg[1][k], k >= 1: the
// top segment top(k-1) -> top(k); seg[2][k], k >= 1: the bottom segment
// bot(k) -> bot(k-1) (the tile's, formed once per block in shared memory)
template <int BA_W, class F>
__device__ __forceinline__ void strip_hl(const float* topH, const float* topL, const float* botH, const float* botL,
                                         const float4 (*seg)[BA_W], int nvs, HL px, HL py, HL pz, float nx, float ny,
                                         float nz, F&& f) {
    auto rel = [&](const float* H, const float* L, int sl, bool mir) {
        const float y = mir ? df_sub(-py.h, -py.l, H[BA_W + sl], L[BA_W + sl]) : df_sub(py.h, py.l, H[BA_W + sl], L[BA_W + sl]);
        return make_rel<float>(df_sub(px.h, px.l, H[sl], L[sl]), y, df_sub(pz.h, pz.l, H[2 * BA_W + sl], L[2 * BA_W + sl]));
    };
    Rel<float> A0 = rel(topH, topL, 0, false), A3 = rel(botH, botL, 0, false);
    Rel<float> B0 = rel(topH, topL, 0, true), B3 = rel(botH, botL, 0, true);
    const float4 l0 = seg[0][0];
    float Ca = seg_normal<float, false, true>(A0, A3, l0.x, l0.y, l0.z, nx, ny, nz, 0.f);
    float Cb = seg_normal<float, false, true>(B0, B3, l0.x, l0.y, l0.z, nx, -ny, nz, 0.f);
    for (int k = 1; k < nvs; k++) {
        const Rel<float> A1 = rel(topH, topL, k, false), A2 = rel(botH, botL, k, false);
        const Rel<float> B1 = rel(topH, topL, k, true), B2 = rel(botH, botL, k, true);
        const float4 c4 = seg[0][k], t4 = seg[1][k], b4 = seg[2][k];
        const float cx = c4.x, cy = c4.y, cz = c4.z;  // v1 -> v2
        const float tx = t4.x, ty = t4.y, tz = t4.z;  // v0 -> v1
        const float bx = b4.x, by = b4.y, bz = b4.z;  // v2 -> v3
        const float Cra = seg_normal<float, false, true>(A1, A2, cx, cy, cz, nx, ny, nz, 0.f);
        const float Crb = seg_normal<float, false, true>(B1, B2, cx, cy, cz, nx, -ny, nz, 0.f);
        float val = seg_normal<float, false, true>(A0, A1, tx, ty, tz, nx, ny, nz, 0.f) + Cra +
                    seg_normal<float, false, true>(A2, A3, bx, by, bz, nx, ny, nz, 0.f) - Ca;
        val += seg_normal<float, false, true>(B0, B1, tx, ty, tz, nx, -ny, nz, 0.f) + Crb +
               seg_normal<float, false, true>(B2, B3, bx, by, bz, nx, -ny, nz, 0.f) - Cb;
        f(k - 1, val);
        A0 = A1; A3 = A2; B0 = B1; B3 = B2; Ca = Cra; Cb = Crb;
    }
}

// The wake rings behind a trailing-edge ring row, span rings [s0, s1): each
// one's value is added to the wing ring's unscaled value already stored at
// colA (Kutta condition, vlm_backend_cpu.cpp:121-139 with iteration = 1), and
// the sum is scaled and stored in A and the A2 copy.
__device__ __forceinline__ void te_wake(const SysDesc& S, int64_t s0, int64_t s1, HL px, HL py, HL pz, float nx,
                                        float ny, float nz, float* colA, float* colB) {
    const int64_t ns = S.ns, n = S.n;
    const float k4 = 1.0f / (4.0f * PI_F);
    const int64_t wl = 2 * (ns + 1);
    for (int64_t s = s0; s < s1; s++) {
        // wake ring: v0=(s,TE) v1=(s+1,TE) v2=(s+1,far) v3=(s,far)
        float Qh[4][3], Ql[4][3];
        const int64_t idx[4] = {s, s + 1, (ns + 1) + s + 1, (ns + 1) + s};
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                Qh[q][k] = S.wh[k * wl + idx[q]];
                Ql[q][k] = S.wl[k * wl + idx[q]];
            }
        float val = 0.f;
#pragma unroll
        for (int mir = 0; mir < 2; mir++) {
            Rel<float> R[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float y = mir ? df_sub(-py.h, -py.l, Qh[q][1], Ql[q][1]) : df_sub(py.h, py.l, Qh[q][1], Ql[q][1]);
                R[q] = make_rel<float>(df_sub(px.h, px.l, Qh[q][0], Ql[q][0]), y, df_sub(pz.h, pz.l, Qh[q][2], Ql[q][2]));
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int e = (q + 1) & 3;
                const float rx = df_sub(Qh[e][0], Ql[e][0], Qh[q][0], Ql[q][0]);
                const float ry = df_sub(Qh[e][1], Ql[e][1], Qh[q][1], Ql[q][1]);
                const float rz = df_sub(Qh[e][2], Ql[e][2], Qh[q][2], Ql[q][2]);
                val += seg_normal<float, false, true>(R[q], R[e], rx, ry, rz, nx, mir ? -ny : ny, nz, 0.f);
            }
        }
        float* dst = colA + (s - s0) * n;
        const float tot = (*dst + val) * k4;
        *dst = tot;
        if (colB) colB[(s - s0) * n] = tot;
    }
}

__device__ __forceinline__ int find_sys(const int64_t* pfx, int cnt, int64_t b) {
    int lo = 0, hi = cnt - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pfx[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// tile0: the first tile of this launch (a size group's systems are a
// contiguous range of tiles)
template <int BA_SPAN>
__global__ void __launch_bounds__(BA_THREADS, 8) k_batch_assemble(BatchArgs a, const int64_t* tpfx, int64_t tile0) {
    constexpr int BA_W = BA_SPAN + 1;
    __shared__ float sw[2][2][3 * BA_W];  // [row][hi/lo][plane*W + s]
    __shared__ float4 sseg[3][BA_W];      // the strip's segment vectors (strip_hl)
    const int64_t tile = tile0 + blockIdx.x;
    const int si = find_sys(tpfx, a.nsys, tile);
    const SysDesc& S = a.sys[si];
    const int64_t ns = S.ns, nc = S.nc, n = S.n;
    const int64_t nchunk = (ns + BA_SPAN - 1) / BA_SPAN, nrb = (n + BA_THREADS - 1) / BA_THREADS;
    int64_t t = tile - tpfx[si];
    const int64_t rb = t % nrb;
    t /= nrb;
    const int64_t z = t % nchunk, c = t / nchunk;
    const int64_t s0 = z * BA_SPAN, s1 = min(s0 + (int64_t)BA_SPAN, ns);
    const int nvs = (int)(s1 - s0 + 1);
    const int64_t nv = (ns + 1) * (nc + 1);
    for (int e = threadIdx.x; e < 2 * 3 * nvs; e += BA_THREADS) {
        const int r = e / (3 * nvs), rem = e - r * 3 * nvs, k = rem / nvs, sl = rem - k * nvs;
        const int64_t vi = k * nv + (s0 + sl) + (c + r) * (ns + 1);
        sw[r][0][k * BA_W + sl] = S.vh[vi];
        sw[r][1][k * BA_W + sl] = S.vl[vi];
    }
    __syncthreads();
    // segment vectors from the double-float positions, once per tile
    for (int e = threadIdx.x; e < 3 * nvs; e += BA_THREADS) {
        const int t = e / nvs, k = e - t * nvs;
        // t = 0: top(k) -> bot(k); 1: top(k-1) -> top(k); 2: bot(k) -> bot(k-1)
        const int r1 = t == 0 ? 1 : (t == 1 ? 0 : 1), k1 = t == 2 ? k - 1 : k;
        const int r0 = t == 0 ? 0 : (t == 1 ? 0 : 1), k0 = t == 1 ? k - 1 : k;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k1 >= 0 && k0 >= 0) {
            v.x = df_sub(sw[r1][0][k1], sw[r1][1][k1], sw[r0][0][k0], sw[r0][1][k0]);
            v.y = df_sub(sw[r1][0][BA_W + k1], sw[r1][1][BA_W + k1], sw[r0][0][BA_W + k0], sw[r0][1][BA_W + k0]);
            v.z = df_sub(sw[r1][0][2 * BA_W + k1], sw[r1][1][2 * BA_W + k1], sw[r0][0][2 * BA_W + k0],
                         sw[r0][1][2 * BA_W + k0]);
        }
        sseg[t][k] = v;
    }
    __syncthreads();
    const int64_t i = rb * BA_THREADS + threadIdx.x;
    if (i >= n) return;
    const HL px{S.ch[i], S.cl_[i]}, py{S.ch[n + i], S.cl_[n + i]}, pz{S.ch[2 * n + i], S.cl_[2 * n + i]};
    const float nx = S.nrm[i], ny = S.nrm[n + i], nz = S.nrm[2 * n + i];
    const float k4 = 1.0f / (4.0f * PI_F);
    float* colA = S.A + i + (c * ns + s0) * n;
    float* colB = S.A2 ? S.A2 + i + (c * ns + s0) * n : nullptr;
    const bool te = (c == nc - 1);
    if (!te) {
        strip_hl<BA_W>(sw[0][0], sw[0][1], sw[1][0], sw[1][1], sseg, nvs, px, py, pz, nx, ny, nz, [&](int kk, float v) {
            const float val = v * k4;
            colA[(int64_t)kk * n] = val;
            if (colB) colB[(int64_t)kk * n] = val;
        });
        return;
    }
    // trailing-edge ring row: wing ring plus the wake ring behind it (Kutta
    // condition, vlm_backend_cpu.cpp:121-139 with iteration = 1)
    strip_hl<BA_W>(sw[0][0], sw[0][1], sw[1][0], sw[1][1], sseg, nvs, px, py, pz, nx, ny, nz,
                   [&](int kk, float v) { colA[(int64_t)kk * n] = v; });
    te_wake(S, s0, s1, px, py, pz, nx, ny, nz, colA, colB);
}

// Tiles of R chordwise ring rows (system, 128-point block, R ring rows, span
// chunk).  The rows' R + 1 vertex lines are walked together along the span:
// a spanwise segment of a line inside the tile is evaluated once (forward,
// vertex k-1 -> k) and enters the ring above the line with + and the ring
// below it with -, and each vertex's distances to the point are formed once
// for the rings on both sides of it.  Per ring: (2R + 1) / R segment pairs
// (direct and mirror) and (R + 1) / R vertex distances, against 3 and 2 for
// one row per tile.  Ring value in the order of strip_hl: top + right - bottom
// - left, then the mirror image's four terms.  Up to three rows the kernel
// fits 64 registers and 8 CTAs per SM; four rows take 34 KB of shared
// memory (6 CTAs).
template <int BA_SPAN, int R>
__global__ void __launch_bounds__(BA_THREADS, R <= 3 ? 8 : 6) k_batch_assemble_rows(BatchArgs a, const int64_t* tpfx, int64_t tile0) {
    constexpr int BA_W = BA_SPAN + 1;
    __shared__ float sw[R + 1][2][3 * BA_W];  // [line][hi/lo][plane*W + s]
    __shared__ float4 sspan[R + 1][BA_W];     // line l: vertex k-1 -> k (k >= 1)
    __shared__ float4 schord[R][BA_W];        // ring row r: line r -> line r+1 at vertex k
    const int64_t tile = tile0 + blockIdx.x;
    const int si = find_sys(tpfx, a.nsys, tile);
    const SysDesc& S = a.sys[si];
    const int64_t ns = S.ns, nc = S.nc, n = S.n;
    const int64_t nchunk = (ns + BA_SPAN - 1) / BA_SPAN, nrb = (n + BA_THREADS - 1) / BA_THREADS;
    int64_t t = tile - tpfx[si];
    const int64_t rb = t % nrb;
    t /= nrb;
    const int64_t z = t % nchunk, c0 = (t / nchunk) * R;
    const int rows = (int)min((int64_t)R, nc - c0);  // ring rows of this tile
    const int64_t s0 = z * BA_SPAN, s1 = min(s0 + (int64_t)BA_SPAN, ns);
    const int nvs = (int)(s1 - s0 + 1);
    const int64_t nv = (ns + 1) * (nc + 1);
    for (int e = threadIdx.x; e < (rows + 1) * 3 * nvs; e += BA_THREADS) {
        const int l = e / (3 * nvs), rem = e - l * 3 * nvs, k = rem / nvs, sl = rem - k * nvs;
        const int64_t vi = k * nv + (s0 + sl) + (c0 + l) * (ns + 1);
        sw[l][0][k * BA_W + sl] = S.vh[vi];
        sw[l][1][k * BA_W + sl] = S.vl[vi];
    }
    __syncthreads();
    // segment vectors from the double-float positions, once per tile
    for (int e = threadIdx.x; e < (2 * rows + 1) * nvs; e += BA_THREADS) {
        const int q = e / nvs, k = e - q * nvs;
        const bool span = q <= rows;  // q <= rows: line q's spanwise segment; else row q - rows - 1's chordwise
        const int l0 = span ? q : q - rows - 1, l1 = span ? q : l0 + 1, k0 = span ? k - 1 : k;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k0 >= 0) {
            v.x = df_sub(sw[l1][0][k], sw[l1][1][k], sw[l0][0][k0], sw[l0][1][k0]);
            v.y = df_sub(sw[l1][0][BA_W + k], sw[l1][1][BA_W + k], sw[l0][0][BA_W + k0], sw[l0][1][BA_W + k0]);
            v.z = df_sub(sw[l1][0][2 * BA_W + k], sw[l1][1][2 * BA_W + k], sw[l0][0][2 * BA_W + k0],
                         sw[l0][1][2 * BA_W + k0]);
        }
        if (span) sspan[q][k] = v;
        else schord[q - rows - 1][k] = v;
    }
    __syncthreads();
    const int64_t i = rb * BA_THREADS + threadIdx.x;
    if (i >= n) return;
    const HL px{S.ch[i], S.cl_[i]}, py{S.ch[n + i], S.cl_[n + i]}, pz{S.ch[2 * n + i], S.cl_[2 * n + i]};
    const float nx = S.nrm[i], ny = S.nrm[n + i], nz = S.nrm[2 * n + i];
    const float k4 = 1.0f / (4.0f * PI_F);
    const int te_row = (c0 + rows == nc) ? rows - 1 : -1;  // the trailing-edge ring row, if in the tile
    auto rel = [&](int l, int sl, bool mir) {
        const float* H = sw[l][0];
        const float* L = sw[l][1];
        const float y = mir ? df_sub(-py.h, -py.l, H[BA_W + sl], L[BA_W + sl]) : df_sub(py.h, py.l, H[BA_W + sl], L[BA_W + sl]);
        return make_rel<float>(df_sub(px.h, px.l, H[sl], L[sl]), y, df_sub(pz.h, pz.l, H[2 * BA_W + sl], L[2 * BA_W + sl]));
    };
    Rel<float> A[R + 1], B[R + 1];  // the lines' distances at the previous vertex (direct, mirror)
    float Ca[R], Cb[R];             // the rows' left chordwise segments
#pragma unroll
    for (int l = 0; l <= R; l++)
        if (l <= rows) {
            A[l] = rel(l, 0, false);
            B[l] = rel(l, 0, true);
        }
#pragma unroll
    for (int r = 0; r < R; r++)
        if (r < rows) {
            const float4 cv = schord[r][0];
            Ca[r] = seg_normal<float, false, true>(A[r], A[r + 1], cv.x, cv.y, cv.z, nx, ny, nz, 0.f);
            Cb[r] = seg_normal<float, false, true>(B[r], B[r + 1], cv.x, cv.y, cv.z, nx, -ny, nz, 0.f);
        }
    float* col0 = S.A + i + (c0 * ns + s0) * n;
    float* colB0 = S.A2 ? S.A2 + i + (c0 * ns + s0) * n : nullptr;
    for (int k = 1; k < nvs; k++) {
        float Sp = 0.f, Spm = 0.f;  // the line above's spanwise segment (direct, mirror)
#pragma unroll
        for (int l = 0; l <= R; l++) {
            if (l <= rows) {
                const Rel<float> An = rel(l, k, false), Bn = rel(l, k, true);
                const float4 sv = sspan[l][k];
                const float Sc = seg_normal<float, false, true>(A[l], An, sv.x, sv.y, sv.z, nx, ny, nz, 0.f);
                const float Scm = seg_normal<float, false, true>(B[l], Bn, sv.x, sv.y, sv.z, nx, -ny, nz, 0.f);
                A[l] = An;
                B[l] = Bn;
                if (l >= 1) {
                    const int r = l - 1;
                    const float4 cv = schord[r][k];
                    const float Cr = seg_normal<float, false, true>(A[r], A[l], cv.x, cv.y, cv.z, nx, ny, nz, 0.f);
                    const float Crm = seg_normal<float, false, true>(B[r], B[l], cv.x, cv.y, cv.z, nx, -ny, nz, 0.f);
                    float val = Sp + Cr - Sc - Ca[r];
                    val += Spm + Crm - Scm - Cb[r];
                    Ca[r] = Cr;
                    Cb[r] = Crm;
                    const int64_t off = ((int64_t)r * ns + (k - 1)) * n;
                    if (r == te_row) {
                        col0[off] = val;  // unscaled: te_wake adds the wake ring
                    } else {
                        col0[off] = val * k4;
                        if (colB0) colB0[off] = val * k4;
                    }
                }
                Sp = Sc;
                Spm = Scm;
            }
        }
    }
    if (te_row >= 0) {
        const int64_t off = (int64_t)te_row * ns * n;
        te_wake(S, s0, s1, px, py, pz, nx, ny, nz, col0 + off, colB0 ? colB0 + off : nullptr);
    }
}

// The correction Alo = A - A2 of the stored float AIC, A evaluated in
// float-pair arithmetic (about 44 bits: the FP64 system's AIC to far below
// float rounding) by the same strip walk over the same tiles as
// k_batch_assemble, with the double kernel's cut-offs.  The refinement
// residual b - (A2 + Alo) x then measures the FP64 system, so the refined
// circulations converge to its solution instead of the float-rounded one's.
// Reads A2, which the tile's k_batch_assemble launch has written.
template <int BA_SPAN>
__global__ void __launch_bounds__(BA_THREADS, 4) k_batch_assemble_lo(BatchArgs a, const int64_t* tpfx, int64_t tile0) {
    constexpr int BA_W = BA_SPAN + 1;
    __shared__ Fe sw[2][3 * BA_W];  // [row][plane*W + s]
    const int64_t tile = tile0 + blockIdx.x;
    const int si = find_sys(tpfx, a.nsys, tile);
    const SysDesc& S = a.sys[si];
    const int64_t ns = S.ns, nc = S.nc, n = S.n;
    const int64_t nchunk = (ns + BA_SPAN - 1) / BA_SPAN, nrb = (n + BA_THREADS - 1) / BA_THREADS;
    int64_t t = tile - tpfx[si];
    const int64_t rb = t % nrb;
    t /= nrb;
    const int64_t z = t % nchunk, c = t / nchunk;
    const int64_t s0 = z * BA_SPAN, s1 = min(s0 + (int64_t)BA_SPAN, ns);
    const int nvs = (int)(s1 - s0 + 1);
    const int64_t nv = (ns + 1) * (nc + 1);
    for (int e = threadIdx.x; e < 2 * 3 * nvs; e += BA_THREADS) {
        const int r = e / (3 * nvs), rem = e - r * 3 * nvs, k = rem / nvs, sl = rem - k * nvs;
        const int64_t vi = k * nv + (s0 + sl) + (c + r) * (ns + 1);
        sw[r][k * BA_W + sl] = Fe(S.vh[vi], S.vl[vi]);
    }
    __syncthreads();
    // the strip's segment vectors once per tile (strip_normal's SEG layout)
    __shared__ V3<Fe> sseg[3 * BA_W];
    for (int e = threadIdx.x; e < 3 * nvs; e += BA_THREADS) {
        const int t = e / nvs, k = e - t * nvs;
        const int r1 = t == 1 ? 0 : 1, k1 = t == 2 ? k - 1 : k;
        const int r0 = t == 2 ? 1 : 0, k0 = t == 1 ? k - 1 : k;
        V3<Fe> v{Fe(0), Fe(0), Fe(0)};
        if (k1 >= 0 && k0 >= 0)
            v = V3<Fe>{sw[r1][k1] - sw[r0][k0], sw[r1][BA_W + k1] - sw[r0][BA_W + k0],
                       sw[r1][2 * BA_W + k1] - sw[r0][2 * BA_W + k0]};
        sseg[t * BA_W + k] = v;
    }
    __syncthreads();
    const int64_t i = rb * BA_THREADS + threadIdx.x;
    if (i >= n) return;
    const Fe px(S.ch[i], S.cl_[i]), py(S.ch[n + i], S.cl_[n + i]), pz(S.ch[2 * n + i], S.cl_[2 * n + i]);
    const Fe nx(S.nrmd[i]), ny(S.nrmd[n + i]), nz(S.nrmd[2 * n + i]);
    const Fe k4(1.0 / (double)(4.0f * PI_F));
    const float* colB = S.A2 + i + (c * ns + s0) * n;
    float* colL = S.Alo + i + (c * ns + s0) * n;
    const bool te = (c == nc - 1);
    const int64_t wl = 2 * (ns + 1);
    strip_normal<Fe, false, true, true>(sw[0], sw[1], BA_W, nvs, px, py, pz, nx, ny, nz, Fe(0), [&](int kk, Fe v) {
        if (te) {
            // the wake ring behind this trailing-edge ring (Kutta condition)
            const int64_t s = s0 + kk;
            const int64_t idx[4] = {s, s + 1, (ns + 1) + s + 1, (ns + 1) + s};
            V3<Fe> q[4];
#pragma unroll
            for (int m = 0; m < 4; m++)
                q[m] = V3<Fe>{Fe(S.wh[idx[m]], S.wl[idx[m]]), Fe(S.wh[wl + idx[m]], S.wl[wl + idx[m]]),
                              Fe(S.wh[2 * wl + idx[m]], S.wl[2 * wl + idx[m]])};
            v += ring_normal_full<Fe, false, true>(px, py, pz, nx, ny, nz, q, Fe(0));
        }
        const Fe tot = v * k4;
        const float a2 = colB[(int64_t)kk * n];
        colL[(int64_t)kk * n] = __fadd_rn(__fsub_rn(tot.v, a2), tot.e);
    }, sseg);
}

// ---------------------------------------------------------------------------
// right-hand sides: b = -V_inf(alpha).n in double, float copy into X
// grid: (blocks over max n, systems)
// ---------------------------------------------------------------------------
__device__ __forceinline__ V3<double> freestream_d(double u, double al, double be) {
    return {u * cos(al) * cos(be), -(u * cos(al) * sin(be)), u * sin(al)};
}

// the system's free-stream vectors are formed once per block (double cos and
// sin are long on this part's fp64 units), not once per panel
__global__ void k_batch_rhs(BatchArgs a) {
    __shared__ double sv[64][3];  // a system has at most 64 right-hand sides
    const SysDesc& S = a.sys[blockIdx.y];
    if ((int64_t)blockIdx.x * blockDim.x >= S.n) return;  // uniform over the block
    for (int q = threadIdx.x; q < S.nrhs; q += blockDim.x) {
        const V3<double> V = freestream_d(a.u_inf, a.alphas[S.rhs_off + q], a.beta);
        sv[q][0] = V.x;
        sv[q][1] = V.y;
        sv[q][2] = V.z;
    }
    __syncthreads();
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= S.n) return;
    const double nx = S.nrmd[p], ny = S.nrmd[S.n + p], nz = S.nrmd[2 * S.n + p];
    for (int q = 0; q < S.nrhs; q++) {
        const double b = -(sv[q][0] * nx + sv[q][1] * ny + sv[q][2] * nz);
        S.B[p + q * S.n] = b;
        S.X[p + q * S.n] = (float)b;
        S.Xd[p + q * S.n] = 0.0;
    }
}

// x (double) += x_float ; grid (blocks over n, systems)
__global__ void k_batch_accum(BatchArgs a) {
    const SysDesc& S = a.sys[blockIdx.y];
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= S.n) return;
    for (int q = 0; q < S.nrhs; q++) S.Xd[p + q * S.n] += (double)S.X[p + q * S.n];
}

// R = B - A2 Xd (B - (A2 + Alo) Xd in FP64 residual plans); X = (float)R.
// One thread per row, tiles (system, row
// block).  The products of the float matrix A2 with the double solution Xd
// are accumulated in double-float arithmetic on the fp32 units (Xd split as
// hi + lo floats, each product a*hi exact through an FMA, running sums
// (sh, sl) kept with a compensated addition): about 2^-44 relative per term,
// where the fp64 units of this part run at a small fraction of the fp32 rate.
constexpr int RS_THREADS = 64;
constexpr int RS_MAXRHS = 8;  // (the inner loop reads them as two float4)
constexpr int RS_CB = 8;  // columns of Xd staged per step
constexpr int RS_ROWS = 2;  // rows per thread

// (sh, sl) += a * (xh + xl); XL = false: xl is zero
template <bool XL>
__device__ __forceinline__ void df_mac(float& sh, float& sl, float a, float xh, float xl) {
    const float p = __fmul_rn(a, xh);
    const float pe = __fmaf_rn(a, xh, -p);  // a*xh - p exactly
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));  // sh + p - s exactly
    sh = s;
    sl = XL ? __fmaf_rn(a, xl, __fadd_rn(sl, __fadd_rn(e, pe))) : __fadd_rn(sl, __fadd_rn(e, pe));
}

// LO: the plan keeps the correction Alo of the stored AIC; its products with
// the hi part of Xd join the low-order sums (Alo is about 2^-24 of A, so
// the float product is exact to far below the residual's accuracy).
// XL = false: Xd holds float values (the first sweep: Xd = 0 + the float
// solve), so its lo part is zero and its products are left out.
template <bool LO, bool XL>
__global__ void __launch_bounds__(RS_THREADS) k_batch_residual(BatchArgs a, const int64_t* rpfx) {
    __shared__ __align__(16) float xh[RS_CB][RS_MAXRHS];
    __shared__ __align__(16) float xl[RS_CB][RS_MAXRHS];
    const int si = find_sys(rpfx, a.nsys, blockIdx.x);
    const SysDesc& S = a.sys[si];
    // RS_ROWS rows per thread, RS_THREADS apart: each staged value of X is
    // read once from shared memory for all of them
    const int64_t r0 = (blockIdx.x - rpfx[si]) * (RS_THREADS * RS_ROWS) + threadIdx.x;
    const int64_t n = S.n;
    bool rv[RS_ROWS];
    const float* arow[RS_ROWS];
    const float* lrow[RS_ROWS];
#pragma unroll
    for (int k = 0; k < RS_ROWS; k++) {
        const int64_t r = r0 + k * RS_THREADS;
        rv[k] = r < n;
        arow[k] = S.A2 + (rv[k] ? r : 0);
        lrow[k] = LO ? S.Alo + (rv[k] ? r : 0) : nullptr;
    }
    // grid.y: blocks of RS_MAXRHS right-hand sides
    for (int q0 = blockIdx.y * RS_MAXRHS; q0 < S.nrhs; q0 += RS_MAXRHS * gridDim.y) {
        const int nq = min(RS_MAXRHS, S.nrhs - q0);
        float sh[RS_ROWS][RS_MAXRHS], sl[RS_ROWS][RS_MAXRHS];
#pragma unroll
        for (int k = 0; k < RS_ROWS; k++)
#pragma unroll
            for (int q = 0; q < RS_MAXRHS; q++) sh[k][q] = sl[k][q] = 0.f;
        for (int64_t c0 = 0; c0 < n; c0 += RS_CB) {
            __syncthreads();
            for (int e = threadIdx.x; e < RS_CB * RS_MAXRHS; e += RS_THREADS) {
                const int cc = e / RS_MAXRHS, q = e % RS_MAXRHS;
                const double v = (c0 + cc < n && q < nq) ? S.Xd[(c0 + cc) + (q0 + q) * n] : 0.0;
                const float h = (float)v;
                xh[cc][q] = h;
                if (XL) xl[cc][q] = (float)(v - (double)h);
            }
            __syncthreads();
            if (rv[0]) {
                const int cn = (int)min((int64_t)RS_CB, n - c0);
                float av[RS_ROWS][RS_CB], lv[RS_ROWS][RS_CB];
#pragma unroll
                for (int k = 0; k < RS_ROWS; k++)
#pragma unroll
                    for (int cc = 0; cc < RS_CB; cc++) {
                        av[k][cc] = (cc < cn && rv[k]) ? arow[k][(c0 + cc) * n] : 0.f;
                        if (LO) lv[k][cc] = (cc < cn && rv[k]) ? lrow[k][(c0 + cc) * n] : 0.f;
                    }
#pragma unroll
                for (int cc = 0; cc < RS_CB; cc++) {
                    // the 8 hi and 8 lo values of column cc as four 16-byte broadcasts
                    const float4 h0 = *reinterpret_cast<const float4*>(&xh[cc][0]);
                    const float4 h1 = *reinterpret_cast<const float4*>(&xh[cc][4]);
                    const float hh[RS_MAXRHS] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
                    float ll[RS_MAXRHS] = {};
                    if (XL) {
                        const float4 l0 = *reinterpret_cast<const float4*>(&xl[cc][0]);
                        const float4 l1 = *reinterpret_cast<const float4*>(&xl[cc][4]);
                        ll[0] = l0.x, ll[1] = l0.y, ll[2] = l0.z, ll[3] = l0.w;
                        ll[4] = l1.x, ll[5] = l1.y, ll[6] = l1.z, ll[7] = l1.w;
                    }
#pragma unroll
                    for (int k = 0; k < RS_ROWS; k++)
#pragma unroll
                        for (int q = 0; q < RS_MAXRHS; q++) {
                            df_mac<XL>(sh[k][q], sl[k][q], av[k][cc], hh[q], ll[q]);
                            if (LO) sl[k][q] = __fmaf_rn(lv[k][cc], hh[q], sl[k][q]);
                        }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < RS_ROWS; k++) {
            if (!rv[k]) continue;
            const int64_t r = r0 + k * RS_THREADS;
#pragma unroll
            for (int q = 0; q < RS_MAXRHS; q++) {
                if (q < nq) {
                    const double res = S.B[r + (q0 + q) * n] - ((double)sh[k][q] + (double)sl[k][q]);
                    S.R[r + (q0 + q) * n] = res;
                    S.X[r + (q0 + q) * n] = (float)res;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// loads: one block per solve.  Forces F = rho dgamma (V x dl) on the bound
// segment (vlm_backend_cpu.cpp:276-297), CL/CM (:323-362), Trefftz CDi
// (ispc:273-323).  The geometry differences are formed in double, the force
// and moment terms in float (this part's fp64 rate is a small fraction of its
// fp32 rate) and summed in double.
// ---------------------------------------------------------------------------
// threads per solve: 64 for batches of small systems (most of a block would
// idle; measured faster on 24-2048 panels), 256 once a system exceeds 4096
constexpr int LD_THREADS_SMALL = 64, LD_THREADS_LARGE = 256;

// Trefftz influence matrix of one system: K[j, jj] = -(induced velocity of
// the trailing legs of wake ring jj with unit gamma, plus mirror, at the
// centre of wake ring j) . n_j * |dl_j| / (4 pi); CDi = gamma^T K gamma / (|V|^2 S)
// (ispc:273-323).  grid: (blocks over ns*ns, systems)
__global__ void k_batch_trefftz_k(BatchArgs a) {
    const SysDesc& S = a.sys[blockIdx.y];
    const int64_t ns = S.ns, e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ns * ns) return;
    const int64_t j = e % ns, jj = e / ns;
    const double* w = S.wd;
    const int64_t wl = 2 * (ns + 1);
    auto WP = [&](int64_t idx) { return V3<double>{w[idx], w[wl + idx], w[2 * wl + idx]}; };
    const V3<double> q0 = WP(j), q1 = WP(j + 1), q2 = WP((ns + 1) + j + 1), q3 = WP((ns + 1) + j);
    const V3<double> c = 0.25 * (((q0 + q1) + q2) + q3);
    V3<double> nn = cross(q3 - q1, q2 - q0);
    nn = (1.0 / sqrt(len2(nn))) * nn;
    const V3<double> w0 = WP(jj), w1 = WP(jj + 1), w2 = WP((ns + 1) + jj + 1), w3 = WP((ns + 1) + jj);
    const V3<double> cm_{c.x, -c.y, c.z};
    // ring jj's two streamwise segments at c and at its mirror image: relative
    // vectors and segment vectors formed in double and rounded to float, the
    // segment law in float (the fp64 units of this part are slow).  The wake
    // vertices are in the wake's frame (x along the trailing legs), so the
    // offsets across a leg, which the cross product takes, are coordinates
    // of their own and keep float precision; a rotation about y leaves K
    // (a normal velocity) and the mirror image in y as they are
    auto rel = [](V3<double> p, V3<double> q) {
        return make_rel<float>((float)(p.x - q.x), (float)(p.y - q.y), (float)(p.z - q.z));
    };
    const V3<double> s12 = w2 - w1, s30 = w0 - w3;
    auto seg = [&](V3<double> p, V3<double> a, V3<double> b, V3<double> r0) {
        return seg_vec<float, false>(rel(p, a), rel(p, b), (float)r0.x, (float)r0.y, (float)r0.z, 0.f);
    };
    const V3<float> t = seg(c, w1, w2, s12) + seg(c, w3, w0, s30);
    const V3<float> tm = seg(cm_, w1, w2, s12) + seg(cm_, w3, w0, s30);
    const V3<double> sv{(double)t.x + tm.x, (double)t.y - tm.y, (double)t.z + tm.z};
    S.K[j + jj * ns] = -dot(sv, nn) / (4.0 * (double)PI_F) * sqrt(len2(q1 - q0));
}

template <int LD_THREADS>
__global__ void __launch_bounds__(LD_THREADS) k_batch_loads(BatchArgs a, const int32_t* solve_sys, int32_t want_gamma) {
    const int32_t sol = blockIdx.x;
    const int32_t si = solve_sys[sol];
    const SysDesc& S = a.sys[si];
    const int q = sol - S.rhs_off;
    const int64_t ns = S.ns, nc = S.nc, n = S.n, nv = (ns + 1) * (nc + 1);
    const double al = a.alphas[sol];
    const V3<double> V = freestream_d(a.u_inf, al, a.beta);
    V3<double> L{-V.z, 0.0, V.x};
    const double ll = sqrt(len2(L));
    L = (1.0 / ll) * L;
    const double* x = S.Xd + q * n;
    const double* v = S.vd;
    // per panel: the bound-vortex vector and lever arm formed in double and
    // rounded to float, the Joukowski force and its moment in float, sums in
    // double (float terms: ~1e-7 relative each; plain double sums of at most
    // a few thousand terms per thread keep ~1e-13 relative)
    const float Vx = (float)V.x, Vy = (float)V.y, Vz = (float)V.z;
    const float Lx = (float)L.x, Lz = (float)L.z;
    double cl = 0, cmx = 0, cmy = 0, cmz = 0, ar = 0;
    for (int64_t p = threadIdx.x; p < n; p += LD_THREADS) {
        const int64_t i = p % ns, j = p / ns;
        const double g = x[p], gd = (j > 0) ? g - x[p - ns] : g;
        const int64_t ia = i + j * (ns + 1), ib = ia + 1;
        const double ax = v[ia], ay = v[nv + ia], az = v[2 * nv + ia];
        const double bx = v[ib], by = v[nv + ib], bz = v[2 * nv + ib];
        const float dx = (float)(bx - ax), dy = (float)(by - ay), dz = (float)(bz - az);
        const float mx = (float)(0.5 * (ax + bx) - a.ref[0]), my = (float)(0.5 * (ay + by) - a.ref[1]),
                    mz = (float)(0.5 * (az + bz) - a.ref[2]);
        const float rg = (float)(a.rho * gd);
        const float Fx = rg * (Vy * dz - Vz * dy), Fy = rg * (Vz * dx - Vx * dz), Fz = rg * (Vx * dy - Vy * dx);
        cl += (double)(Fx * Lx + Fz * Lz);  // L has no y component
        cmx += (double)(my * Fz - mz * Fy);
        cmy += (double)(mz * Fx - mx * Fz);
        cmz += (double)(mx * Fy - my * Fx);
        ar += S.area[p];
        if (want_gamma && a.gamma_out) a.gamma_out[a.goff[sol] + p] = (float)g;
    }
    // MAC numerator over spanwise stations (vlm_backend_cpu.cpp:443-468)
    const int64_t last = nc * (ns + 1);
    double mac = 0;
    for (int64_t i = threadIdx.x; i < ns; i += LD_THREADS) {
        double c0 = sqrt((v[i] - v[last + i]) * (v[i] - v[last + i]) + (v[nv + i] - v[nv + last + i]) * (v[nv + i] - v[nv + last + i]) +
                         (v[2 * nv + i] - v[2 * nv + last + i]) * (v[2 * nv + i] - v[2 * nv + last + i]));
        double c1 = sqrt((v[i + 1] - v[last + i + 1]) * (v[i + 1] - v[last + i + 1]) +
                         (v[nv + i + 1] - v[nv + last + i + 1]) * (v[nv + i + 1] - v[nv + last + i + 1]) +
                         (v[2 * nv + i + 1] - v[2 * nv + last + i + 1]) * (v[2 * nv + i + 1] - v[2 * nv + last + i + 1]));
        double w = sqrt((v[i + 1] - v[i]) * (v[i + 1] - v[i]) + (v[nv + i + 1] - v[nv + i]) * (v[nv + i + 1] - v[nv + i]) +
                        (v[2 * nv + i + 1] - v[2 * nv + i]) * (v[2 * nv + i + 1] - v[2 * nv + i]));
        mac += 0.5 * (c0 * c0 + c1 * c1) * w;
    }
    // Trefftz drag: gamma_TE^T K gamma_TE (the wake carries the TE gamma)
    double cd = 0;
    const double* gte = x + (nc - 1) * ns;
    for (int64_t e = threadIdx.x; e < ns * ns; e += LD_THREADS) {
        const int64_t j = e % ns, jj = e / ns;
        cd += gte[j] * S.K[e] * gte[jj];
    }
    // the seven sums in one pass: each reduced down its warp, then the warps'
    // partial sums added in warp order by thread 0
    __shared__ double sh7[7][LD_THREADS / 32];
    double vals[7] = {cl, cmx, cmy, cmz, ar, mac, cd};
#pragma unroll
    for (int k = 0; k < 7; k++)
        for (int o = 16; o > 0; o >>= 1) vals[k] += __shfl_down_sync(0xffffffffu, vals[k], o);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < 7; k++) sh7[k][threadIdx.x >> 5] = vals[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[7];
        for (int k = 0; k < 7; k++) {
            t[k] = 0;
            for (int w = 0; w < LD_THREADS / 32; w++) t[k] += sh7[k][w];
        }
        const double s_cl = t[0], s_x = t[1], s_y = t[2], s_z = t[3], s_ar = t[4], s_mac = t[5], s_cd = t[6];
        const double v2 = len2(V);
        const double macv = s_mac / s_ar;
        double* o = a.out + 5 * (int64_t)a.uidx[sol];
        o[0] = s_cl / (0.5 * a.rho * v2 * s_ar);
        o[1] = s_cd / (v2 * s_ar);
        const double d = 0.5 * a.rho * v2 * s_ar * macv;
        o[2] = s_x / d;
        o[3] = s_y / d;
        o[4] = s_z / d;
    }
}

}  // namespace gbvlm

using namespace gbvlm;

// ===========================================================================
// host object
// ===========================================================================
struct gbvlm_batch_s {
    int32_t ncases = 0, nsys = 0, nsolve = 0, mode = 0, refine = 1;
    TuneParams tp;                    // launch shapes, copied from the tuning table at creation
    std::vector<gbvlm_dims> dims;
    std::vector<int32_t> nalpha;
    std::vector<int64_t> case_voff;   // float offsets of case vertices in the input buffer
    std::vector<int64_t> solve_n;     // n per solve
    std::vector<int64_t> goff;        // gamma offsets per solve
    int64_t vin_floats = 0, gamma_floats = 0;
    std::vector<SysDesc> sys;         // sorted by n descending
    std::vector<int32_t> solve_sys;   // solve -> system (sorted index)
    std::vector<int32_t> solve_order; // solve index in user order -> solve index in batch order
    void* arena = nullptr;
    size_t arena_bytes = 0;
    float* d_vin = nullptr;
    double* d_alpha = nullptr;   // per solve (batch order)
    double* d_out = nullptr;     // per solve x5 (the caller's order)
    float* d_gamma = nullptr;
    int64_t* d_goff = nullptr;
    int32_t* d_uidx = nullptr;   // batch solve -> the caller's solve
    int32_t* d_bad = nullptr;    // per system: non-finite input vertices
    void* status = nullptr;      // pinned: error words and pivot flags read back with the results
    SysDesc* d_sys = nullptr;
    int32_t* d_solve_sys = nullptr;
    int64_t* d_tpfx = nullptr;   // assembly tiles
    int64_t* d_tpfx_rows = nullptr;  // float assembly tiles of asm_rows ring rows (asm_rows > 1)
    int asm_rows = 1;
    int64_t* d_rpfx = nullptr;   // residual tiles
    int64_t assembly_tiles = 0, residual_tiles = 0;
    std::vector<int64_t> tpfx_host;   // assembly tile prefix over the sorted systems
    int64_t gtile[4][2] = {};         // per size group: first tile, tiles
    int64_t gtile_rows[4][2] = {};    // the same over the float assembly's tiles of asm_rows rows
    int64_t assembly_tiles_rows = 0;
    std::vector<int64_t> tpfx_rows_host;
    int64_t maxn = 0;
    // the sorted systems in size groups, each factored by its own plan on its
    // own stream (graph branch), so the long step chain of the largest
    // systems runs beside the shorter chains of the others
    static constexpr int MAX_GROUPS = 4;
    int ngroups = 0;
    LuPlan plans[MAX_GROUPS];
    cudaStream_t side[MAX_GROUPS] = {};
    cudaEvent_t fork = nullptr, join[MAX_GROUPS] = {};
    // FP64 residual plans: the AIC correction of each size group on its own
    // low-priority branch, after the group's assembly and beside its
    // factorisation; joined before the first refinement residual
    bool fp64_residual = false;
    cudaStream_t lo_side = nullptr;
    cudaEvent_t asm_done[MAX_GROUPS] = {}, lo_join = nullptr;
    // the plan's device memory is stream-ordered on `mem` (dev_alloc), so
    // creating and destroying a plan does not synchronise the device while
    // other streams run; `done` marks the end of the last enqueued work, and
    // the releases wait for it
    cudaStream_t mem = nullptr;
    cudaEvent_t done = nullptr;
    size_t status_bytes = 0;
    LuBatch<float> lub;
    TrsFlow flow;  // triangular solves of all systems (unless GBVLM_TRS_FLOW=0: one CTA per system)
    bool use_flow = true;
    double u_inf = 1, rho = 1, beta = 0, ref[3] = {0, 0, 0};
    int32_t want_gamma = 0;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double interactions = 0, lu_flops = 0;
    int64_t launches = 0;
    ~gbvlm_batch_s() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
        if (mem && done) cudaStreamWaitEvent(mem, done, 0);  // releases after the last enqueued work
        dev_free(arena, mem);
        pinned_give(status, status_bytes);
        for (int g = 0; g < MAX_GROUPS; g++) {
            plans[g].release();
            if (side[g]) cudaStreamDestroy(side[g]);
            if (join[g]) cudaEventDestroy(join[g]);
            if (asm_done[g]) cudaEventDestroy(asm_done[g]);
        }
        flow.release();
        if (lo_side) cudaStreamDestroy(lo_side);
        if (lo_join) cudaEventDestroy(lo_join);
        if (fork) cudaEventDestroy(fork);
        if (done) cudaEventDestroy(done);
        if (mem) cudaStreamDestroy(mem);  // returns at once; the stream goes when its frees are done
    }
};

constexpr int MAX_GROUPS_B = 3;  // size-group boundaries (gbvlm_batch_s::MAX_GROUPS - 1)

// serial_lu: factor the size groups one after another on `st` (kernel timing
// without the groups' launches overlapping)
// the assembly kernel of the plan's span chunk over `tiles` tiles from tile0
template <int SPAN>
static void launch_assemble_rows(int rows, unsigned tiles, int64_t tile0, const BatchArgs& a, const int64_t* tpfx,
                                 cudaStream_t st) {
    switch (rows) {
        case 2: k_batch_assemble_rows<SPAN, 2><<<tiles, BA_THREADS, 0, st>>>(a, tpfx, tile0); break;
        case 3:
            if constexpr (SPAN <= 128) k_batch_assemble_rows<SPAN, 3><<<tiles, BA_THREADS, 0, st>>>(a, tpfx, tile0);
            break;
        default:
            if constexpr (SPAN <= 128) k_batch_assemble_rows<SPAN, 4><<<tiles, BA_THREADS, 0, st>>>(a, tpfx, tile0);
            break;
    }
}

// the float assembly's tiles: one ring row each (k_batch_assemble), or
// asm_rows rows (k_batch_assemble_rows, its own tile prefix)
static cudaError_t launch_assemble(gbvlm_batch h, unsigned tiles, int64_t tile0, const BatchArgs& a, cudaStream_t st) {
    if (h->asm_rows > 1) {
        switch (h->tp.batch_assembly_span) {
            case 64: launch_assemble_rows<64>(h->asm_rows, tiles, tile0, a, h->d_tpfx_rows, st); break;
            case 256: launch_assemble_rows<256>(h->asm_rows, tiles, tile0, a, h->d_tpfx_rows, st); break;
            default: launch_assemble_rows<128>(h->asm_rows, tiles, tile0, a, h->d_tpfx_rows, st); break;
        }
        return cudaGetLastError();
    }
    switch (h->tp.batch_assembly_span) {
        case 64: k_batch_assemble<64><<<tiles, BA_THREADS, 0, st>>>(a, h->d_tpfx, tile0); break;
        case 256: k_batch_assemble<256><<<tiles, BA_THREADS, 0, st>>>(a, h->d_tpfx, tile0); break;
        default: k_batch_assemble<128><<<tiles, BA_THREADS, 0, st>>>(a, h->d_tpfx, tile0); break;
    }
    return cudaGetLastError();
}

static cudaError_t launch_assemble_lo(gbvlm_batch h, unsigned tiles, int64_t tile0, const BatchArgs& a,
                                      cudaStream_t st) {
    switch (h->tp.batch_assembly_span) {
        case 64: k_batch_assemble_lo<64><<<tiles, BA_THREADS, 0, st>>>(a, h->d_tpfx, tile0); break;
        case 256: k_batch_assemble_lo<256><<<tiles, BA_THREADS, 0, st>>>(a, h->d_tpfx, tile0); break;
        default: k_batch_assemble_lo<128><<<tiles, BA_THREADS, 0, st>>>(a, h->d_tpfx, tile0); break;
    }
    return cudaGetLastError();
}

static int batch_enqueue(gbvlm_batch h, cudaStream_t st, cudaEvent_t* ev = nullptr, bool serial_lu = false) {
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st); };
    int64_t nlaunch = 0;
    for (int g = 0; g < h->ngroups; g++) nlaunch += lu_plan_launches(h->plans[g], 4);
    int32_t mr = 0;
    for (auto& s : h->sys) mr = std::max(mr, s.nrhs);
    const int64_t solves = h->use_flow ? trs_flow_launches(mr, h->flow.groups) : (mr + 7) / 8;
    // geometry, Trefftz, the groups' assemblies, RHS, the factorisations, the
    // solves and accumulations, the refinement sweeps, the loads
    h->launches = 3 + h->ngroups * (h->fp64_residual ? 2 : 1) + nlaunch + solves + 1 +
                  (int64_t)h->refine * (1 + solves + 1) + 1;
    BatchArgs a;
    a.sys = h->d_sys;
    a.nsys = h->nsys;
    a.alphas = h->d_alpha;
    a.u_inf = h->u_inf;
    a.rho = h->rho;
    a.beta = h->beta;
    for (int k = 0; k < 3; k++) a.ref[k] = h->ref[k];
    a.out = h->d_out;
    a.gamma_out = h->d_gamma;
    a.goff = h->d_goff;
    a.uidx = h->d_uidx;
    a.bad = h->d_bad;
    // staged: every phase after the previous one on `st` (stage timing, or
    // kernel timing without the groups' launches overlapping); otherwise each
    // size group's assembly and factorisation run on its own branch, group 0
    // (the largest systems, the critical path) at high priority, with the
    // Trefftz kernel and the right-hand sides on the main stream beside them
    const bool staged = ev != nullptr || serial_lu;
    auto trefftz = [&]() {
        int64_t maxns = 1;
        for (auto& S : h->sys) maxns = std::max(maxns, S.ns);
        dim3 gk((unsigned)cdiv(maxns * maxns, 128), (unsigned)h->nsys);
        k_batch_trefftz_k<<<gk, 128, 0, st>>>(a);
        return cudaGetLastError();
    };
    mark(0);
    k_batch_geom<<<h->nsys, 256, 0, st>>>(a);
    GB_LAUNCH_CHECK();
    if (staged) GB_CUDA(trefftz());
    mark(1);
    if (staged) {
        GB_CUDA(launch_assemble(h, (unsigned)(h->asm_rows > 1 ? h->assembly_tiles_rows : h->assembly_tiles), 0, a, st));
        if (h->fp64_residual) GB_CUDA(launch_assemble_lo(h, (unsigned)h->assembly_tiles, 0, a, st));
    }
    mark(2);
    dim3 gp((unsigned)cdiv(h->maxn, 256), (unsigned)h->nsys);  // one thread per row of every system
    if (staged) {
        k_batch_rhs<<<gp, 256, 0, st>>>(a);
        GB_LAUNCH_CHECK();
    }
    mark(3);
    if (staged) {
        for (int g = 0; g < h->ngroups; g++) {
            int rc = lu_batch_factor<float>(h->lub, h->plans[g], st, !serial_lu);
            if (rc) return rc;
        }
    } else {
        GB_CUDA(cudaEventRecord(h->fork, st));
        for (int g = 0; g < h->ngroups; g++) {
            GB_CUDA(cudaStreamWaitEvent(h->side[g], h->fork, 0));
            if (h->gtile[g][1] > 0) {
                const int64_t(&gt)[2] = h->asm_rows > 1 ? h->gtile_rows[g] : h->gtile[g];
                GB_CUDA(launch_assemble(h, (unsigned)gt[1], gt[0], a, h->side[g]));
                if (h->fp64_residual) {
                    GB_CUDA(cudaEventRecord(h->asm_done[g], h->side[g]));
                    GB_CUDA(cudaStreamWaitEvent(h->lo_side, h->asm_done[g], 0));
                    GB_CUDA(launch_assemble_lo(h, (unsigned)h->gtile[g][1], h->gtile[g][0], a, h->lo_side));
                }
            }
            int rc = lu_batch_factor<float>(h->lub, h->plans[g], h->side[g], true);
            if (rc) return rc;
            GB_CUDA(cudaEventRecord(h->join[g], h->side[g]));
        }
        GB_CUDA(trefftz());
        k_batch_rhs<<<gp, 256, 0, st>>>(a);
        GB_LAUNCH_CHECK();
        for (int gi = 0; gi < h->ngroups; gi++) GB_CUDA(cudaStreamWaitEvent(st, h->join[gi], 0));
        if (h->fp64_residual) GB_CUDA(cudaEventRecord(h->lo_join, h->lo_side));
    }
    int rc = GBVLM_OK;
    mark(4);
    int32_t maxrhs = 0;
    for (auto& s : h->sys) maxrhs = std::max(maxrhs, s.nrhs);
    auto solve = [&]() {
        return h->use_flow ? trs_flow_solve(h->lub, h->flow, maxrhs, st)
                           : lu_batch_solve<float>(h->lub, h->nsys, maxrhs, h->maxn, st,
                                                   h->plans[0].tc_passes ? h->plans[0].d_err : nullptr);
    };
    rc = solve();
    if (rc) return rc;
    k_batch_accum<<<gp, 256, 0, st>>>(a);
    GB_LAUNCH_CHECK();
    if (h->fp64_residual && !staged && h->refine > 0) GB_CUDA(cudaStreamWaitEvent(st, h->lo_join, 0));
    for (int it = 0; it < h->refine; it++) {
        const dim3 rg((unsigned)h->residual_tiles, (unsigned)cdiv(maxrhs, RS_MAXRHS));
        if (h->fp64_residual) {
            if (it == 0) k_batch_residual<true, false><<<rg, RS_THREADS, 0, st>>>(a, h->d_rpfx);
            else k_batch_residual<true, true><<<rg, RS_THREADS, 0, st>>>(a, h->d_rpfx);
        } else {
            if (it == 0) k_batch_residual<false, false><<<rg, RS_THREADS, 0, st>>>(a, h->d_rpfx);
            else k_batch_residual<false, true><<<rg, RS_THREADS, 0, st>>>(a, h->d_rpfx);
        }
        GB_LAUNCH_CHECK();
        rc = solve();
        if (rc) return rc;
        k_batch_accum<<<gp, 256, 0, st>>>(a);
        GB_LAUNCH_CHECK();
    }
    mark(5);
    {
        // the loads block: by the largest system, or the tuned width
        const int64_t lt = h->tp.batch_loads_threads ? h->tp.batch_loads_threads
                                                     : (h->maxn > 4096 ? LD_THREADS_LARGE : LD_THREADS_SMALL);
        if (lt == 32)
            k_batch_loads<32><<<h->nsolve, 32, 0, st>>>(a, h->d_solve_sys, h->want_gamma);
        else if (lt == 64)
            k_batch_loads<64><<<h->nsolve, 64, 0, st>>>(a, h->d_solve_sys, h->want_gamma);
        else if (lt == 128)
            k_batch_loads<128><<<h->nsolve, 128, 0, st>>>(a, h->d_solve_sys, h->want_gamma);
        else
            k_batch_loads<256><<<h->nsolve, 256, 0, st>>>(a, h->d_solve_sys, h->want_gamma);
        GB_LAUNCH_CHECK();
    }
    mark(6);
    return GBVLM_OK;
}

extern "C" {

int gbvlm_batch_create(gbvlm_batch* out, int32_t ncases, const gbvlm_dims* dims, const int32_t* nalpha, int32_t mode,
                       int32_t refine_iters) {
    return gbvlm_batch_create_ex(out, ncases, dims, nalpha, mode, refine_iters, 0);
}

int gbvlm_batch_create_ex(gbvlm_batch* out, int32_t ncases, const gbvlm_dims* dims, const int32_t* nalpha,
                          int32_t mode, int32_t refine_iters, int32_t flags) {
    GB_REQUIRE(out && dims && nalpha && ncases >= 1, "bad batch arguments");
    GB_REQUIRE(mode == GBVLM_BATCH_EXACT || mode == GBVLM_BATCH_SHARED, "unknown batch mode %d", mode);
    GB_REQUIRE(refine_iters >= 0 && refine_iters <= 8, "refine_iters outside [0, 8]");
    GB_REQUIRE((flags & ~GBVLM_BATCH_FP64_RESIDUAL) == 0, "unknown batch flags 0x%x", (unsigned)flags);
    const bool fp64_residual = (flags & GBVLM_BATCH_FP64_RESIDUAL) != 0;
    GB_REQUIRE(!fp64_residual || refine_iters >= 1, "GBVLM_BATCH_FP64_RESIDUAL needs refine_iters >= 1");
    const TuneParams tp = tune();
    GB_REQUIRE(tp.batch_group_hi > tp.batch_group_lo, "batch.group_hi (%lld) must exceed batch.group_lo (%lld)",
               (long long)tp.batch_group_hi, (long long)tp.batch_group_lo);
    GB_REQUIRE(tp.batch_group_mid == 0 || (tp.batch_group_hi > tp.batch_group_mid && tp.batch_group_mid > tp.batch_group_lo),
               "batch.group_mid (%lld) must be 0 or between batch.group_lo and batch.group_hi",
               (long long)tp.batch_group_mid);
    auto* h = new gbvlm_batch_s();
    h->tp = tp;
    h->fp64_residual = fp64_residual;
    h->ncases = ncases;
    h->mode = mode;
    h->refine = refine_iters;
    h->dims.assign(dims, dims + ncases);
    h->nalpha.assign(nalpha, nalpha + ncases);
    struct Proto {
        int32_t case_id;
        int64_t n;
        int32_t nrhs;
        int32_t first_user_solve;
    };
    std::vector<Proto> protos;
    int32_t user_solve = 0;
    for (int c = 0; c < ncases; c++) {
        if (dims[c].ns < 1 || dims[c].nc < 1 || nalpha[c] < 1 || nalpha[c] > 64) {
            delete h;
            set_error("case %d: bad sizes (ns=%lld nc=%lld nalpha=%d)", c, (long long)dims[c].ns,
                      (long long)dims[c].nc, nalpha[c]);
            return GBVLM_ERR_ARG;
        }
        h->case_voff.push_back(h->vin_floats);
        h->vin_floats += 4 * (dims[c].ns + 1) * (dims[c].nc + 1);
        const int64_t n = dims[c].ns * dims[c].nc;
        if (mode == GBVLM_BATCH_SHARED) {
            protos.push_back({c, n, nalpha[c], user_solve});
        } else {
            for (int q = 0; q < nalpha[c]; q++) protos.push_back({c, n, 1, user_solve + q});
        }
        user_solve += nalpha[c];
    }
    h->nsolve = user_solve;
    std::vector<int> order(protos.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return protos[x].n > protos[y].n; });
    h->nsys = (int32_t)protos.size();
    // arena layout
    size_t bytes = 0;
    auto reserve = [&](size_t b) {
        size_t o = bytes;
        bytes += (b + 255) / 256 * 256;
        return o;
    };
    struct Off {
        size_t vh, vl, wh, wl, ch, cl, nrm, area, vd, wd, nrmd, A, A2, Alo, ipiv, perm, X, B, Xd, R, K;
    };
    std::vector<Off> offs(h->nsys);
    const size_t o_vin = reserve(sizeof(float) * h->vin_floats);
    for (int k = 0; k < h->nsys; k++) {
        const Proto& P = protos[order[k]];
        const gbvlm_dims& d = dims[P.case_id];
        const int64_t nv = (d.ns + 1) * (d.nc + 1), n = P.n, wv = 2 * (d.ns + 1);
        Off& o = offs[k];
        o.vh = reserve(sizeof(float) * 3 * nv);
        o.vl = reserve(sizeof(float) * 3 * nv);
        o.wh = reserve(sizeof(float) * 3 * wv);
        o.wl = reserve(sizeof(float) * 3 * wv);
        o.ch = reserve(sizeof(float) * 3 * n);
        o.cl = reserve(sizeof(float) * 3 * n);
        o.nrm = reserve(sizeof(float) * 3 * n);
        o.area = reserve(sizeof(double) * n);
        o.vd = reserve(sizeof(double) * 3 * nv);
        o.wd = reserve(sizeof(double) * 3 * wv);
        o.nrmd = reserve(sizeof(double) * 3 * n);
        o.A = reserve(sizeof(float) * n * n);
        o.A2 = refine_iters > 0 ? reserve(sizeof(float) * n * n) : (size_t)-1;
        o.Alo = fp64_residual ? reserve(sizeof(float) * n * n) : (size_t)-1;
        o.ipiv = reserve(sizeof(int32_t) * n);
        o.perm = reserve(sizeof(int32_t) * n);
        o.X = reserve(sizeof(float) * n * P.nrhs);
        o.B = reserve(sizeof(double) * n * P.nrhs);
        o.Xd = reserve(sizeof(double) * n * P.nrhs);
        o.R = reserve(sizeof(double) * n * P.nrhs);
        o.K = reserve(sizeof(double) * d.ns * d.ns);
        h->interactions += (double)n * (double)n + (double)n * d.ns;
        h->lu_flops += 2.0 / 3.0 * (double)n * n * n;
    }
    const size_t o_alpha = reserve(sizeof(double) * h->nsolve);
    const size_t o_out = reserve(sizeof(double) * 5 * h->nsolve);
    // gamma per solve in batch order
    std::vector<int32_t> solve_sys;
    std::vector<int64_t> goff;
    int64_t gtot = 0;
    for (int k = 0; k < h->nsys; k++) {
        for (int q = 0; q < protos[order[k]].nrhs; q++) {
            solve_sys.push_back(k);
            goff.push_back(gtot);
            gtot += protos[order[k]].n;
        }
    }
    h->gamma_floats = gtot;
    const size_t o_gamma = reserve(sizeof(float) * gtot);
    const size_t o_goff = reserve(sizeof(int64_t) * goff.size());
    const size_t o_sys = reserve(sizeof(SysDesc) * h->nsys);
    const size_t o_ssys = reserve(sizeof(int32_t) * solve_sys.size());
    const size_t o_uidx = reserve(sizeof(int32_t) * solve_sys.size());
    const size_t o_bad = reserve(sizeof(int32_t) * h->nsys);
    // tile prefix tables
    // ring rows per float assembly tile: at most 4, at most 2 with 256-ring span chunks (shared memory)
    h->asm_rows = (int)std::min<int64_t>(h->tp.batch_assembly_rows, h->tp.batch_assembly_span > 128 ? 2 : 4);
    std::vector<int64_t> tpfx(h->nsys + 1, 0), tpfx_rows(h->nsys + 1, 0), rpfx(h->nsys + 1, 0);
    for (int k = 0; k < h->nsys; k++) {
        const gbvlm_dims& d = dims[protos[order[k]].case_id];
        const int64_t n = protos[order[k]].n;
        const int64_t per_row = cdiv(n, BA_THREADS) * cdiv(d.ns, h->tp.batch_assembly_span);
        tpfx[k + 1] = tpfx[k] + per_row * d.nc;
        tpfx_rows[k + 1] = tpfx_rows[k] + per_row * cdiv(d.nc, (int64_t)h->asm_rows);
        rpfx[k + 1] = rpfx[k] + cdiv(n, RS_THREADS * RS_ROWS);
    }
    h->assembly_tiles = tpfx[h->nsys];
    h->tpfx_host = tpfx;
    h->assembly_tiles_rows = tpfx_rows[h->nsys];
    h->tpfx_rows_host = tpfx_rows;
    h->residual_tiles = rpfx[h->nsys];
    const size_t o_tpfx = reserve(sizeof(int64_t) * tpfx.size());
    const size_t o_tpfx_rows = reserve(sizeof(int64_t) * tpfx_rows.size());
    const size_t o_rpfx = reserve(sizeof(int64_t) * rpfx.size());
    // LU tables
    const size_t o_lun = reserve(sizeof(int64_t) * h->nsys);
    const size_t o_luA = reserve(sizeof(float*) * h->nsys);
    const size_t o_lup = reserve(sizeof(int32_t*) * h->nsys);
    const size_t o_luinfo = reserve(sizeof(int32_t) * h->nsys);
    const size_t o_luX = reserve(sizeof(float*) * h->nsys);
    const size_t o_lurhs = reserve(sizeof(int32_t) * h->nsys);
    const size_t o_luperm = reserve(sizeof(int32_t*) * h->nsys);
    const size_t o_lumv = reserve(sizeof(int32_t) * 64 * h->nsys);
    cudaError_t e = cudaStreamCreateWithFlags(&h->mem, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = dev_alloc(&h->arena, bytes, h->mem);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "batch arena", __FILE__, __LINE__);
    }
    h->arena_bytes = bytes;
    char* base = (char*)h->arena;
    h->d_vin = (float*)(base + o_vin);
    h->d_alpha = (double*)(base + o_alpha);
    h->d_out = (double*)(base + o_out);
    h->d_gamma = (float*)(base + o_gamma);
    h->d_goff = (int64_t*)(base + o_goff);
    h->d_sys = (SysDesc*)(base + o_sys);
    h->d_solve_sys = (int32_t*)(base + o_ssys);
    h->d_uidx = (int32_t*)(base + o_uidx);
    h->d_bad = (int32_t*)(base + o_bad);
    h->d_tpfx = (int64_t*)(base + o_tpfx);
    h->d_tpfx_rows = (int64_t*)(base + o_tpfx_rows);
    h->d_rpfx = (int64_t*)(base + o_rpfx);
    // system descriptors
    h->sys.resize(h->nsys);
    std::vector<int64_t> lun(h->nsys);
    std::vector<float*> luA(h->nsys), luX(h->nsys);
    std::vector<int32_t*> lup(h->nsys), lperm(h->nsys);
    std::vector<int32_t> lurhs(h->nsys);
    int32_t rhs_off = 0;
    h->solve_order.assign(h->nsolve, 0);
    for (int k = 0; k < h->nsys; k++) {
        const Proto& P = protos[order[k]];
        const gbvlm_dims& d = dims[P.case_id];
        const Off& o = offs[k];
        SysDesc& S = h->sys[k];
        memset(&S, 0, sizeof(S));
        S.ns = d.ns;
        S.nc = d.nc;
        S.n = P.n;
        S.case_id = P.case_id;
        S.nrhs = P.nrhs;
        S.rhs_off = rhs_off;
        for (int q = 0; q < P.nrhs; q++) h->solve_order[P.first_user_solve + q] = rhs_off + q;
        rhs_off += P.nrhs;
        S.vinit = h->d_vin + h->case_voff[P.case_id];
        S.vh = (float*)(base + o.vh);
        S.vl = (float*)(base + o.vl);
        S.wh = (float*)(base + o.wh);
        S.wl = (float*)(base + o.wl);
        S.ch = (float*)(base + o.ch);
        S.cl_ = (float*)(base + o.cl);
        S.nrm = (float*)(base + o.nrm);
        S.area = (double*)(base + o.area);
        S.vd = (double*)(base + o.vd);
        S.wd = (double*)(base + o.wd);
        S.nrmd = (double*)(base + o.nrmd);
        S.A = (float*)(base + o.A);
        S.A2 = o.A2 == (size_t)-1 ? nullptr : (float*)(base + o.A2);
        S.Alo = o.Alo == (size_t)-1 ? nullptr : (float*)(base + o.Alo);
        S.ipiv = (int32_t*)(base + o.ipiv);
        S.X = (float*)(base + o.X);
        S.B = (double*)(base + o.B);
        S.Xd = (double*)(base + o.Xd);
        S.R = (double*)(base + o.R);
        S.K = (double*)(base + o.K);
        lun[k] = P.n;
        luA[k] = S.A;
        lup[k] = S.ipiv;
        lperm[k] = (int32_t*)(base + o.perm);
        luX[k] = S.X;
        lurhs[k] = P.nrhs;
        h->maxn = std::max(h->maxn, P.n);
    }
    // outputs in the caller's order: circulations packed by the caller's solve
    // index, so the results copy straight into the caller's buffers
    std::vector<int32_t> uidx(h->nsolve);
    {
        int64_t uoff = 0;
        for (int32_t u = 0; u < h->nsolve; u++) {
            const int32_t b = h->solve_order[u];
            uidx[b] = u;
            goff[b] = uoff;
            uoff += h->sys[solve_sys[b]].n;
        }
    }
    h->solve_sys = solve_sys;
    h->goff = goff;
    int rc = GBVLM_OK;
    auto up = [&](void* dst, const void* src, size_t b) {
        if (rc == GBVLM_OK && b) {
            cudaError_t ee = cudaMemcpy(dst, src, b, cudaMemcpyHostToDevice);
            if (ee != cudaSuccess) rc = cuda_fail(ee, "cudaMemcpy(batch tables)", __FILE__, __LINE__);
        }
    };
    up(h->d_sys, h->sys.data(), sizeof(SysDesc) * h->nsys);
    up(h->d_solve_sys, solve_sys.data(), sizeof(int32_t) * solve_sys.size());
    up(h->d_goff, goff.data(), sizeof(int64_t) * goff.size());
    up(h->d_uidx, uidx.data(), sizeof(int32_t) * uidx.size());
    up(h->d_tpfx, tpfx.data(), sizeof(int64_t) * tpfx.size());
    up(h->d_tpfx_rows, tpfx_rows.data(), sizeof(int64_t) * tpfx_rows.size());
    up(h->d_rpfx, rpfx.data(), sizeof(int64_t) * rpfx.size());
    up(base + o_lun, lun.data(), sizeof(int64_t) * h->nsys);
    up(base + o_luA, luA.data(), sizeof(float*) * h->nsys);
    up(base + o_lup, lup.data(), sizeof(int32_t*) * h->nsys);
    up(base + o_luX, luX.data(), sizeof(float*) * h->nsys);
    up(base + o_lurhs, lurhs.data(), sizeof(int32_t) * h->nsys);
    up(base + o_luperm, lperm.data(), sizeof(int32_t*) * h->nsys);
    if (rc == GBVLM_OK) {
        cudaError_t ee = cudaMemset(base + o_luinfo, 0, sizeof(int32_t) * h->nsys);
        if (ee != cudaSuccess) rc = cuda_fail(ee, "cudaMemset", __FILE__, __LINE__);
    }
    if (rc) {
        delete h;
        return rc;
    }
    h->lub.n = (const int64_t*)(base + o_lun);
    h->lub.ld = (const int64_t*)(base + o_lun);  // leading dimension = n
    h->lub.A = (float* const*)(base + o_luA);
    h->lub.ipiv = (int32_t* const*)(base + o_lup);
    h->lub.info = (int32_t*)(base + o_luinfo);
    h->lub.X = (float* const*)(base + o_luX);
    h->lub.ldx = (const int64_t*)(base + o_lun);
    h->lub.nrhs = (const int32_t*)(base + o_lurhs);
    h->lub.perm = (int32_t* const*)(base + o_luperm);
    h->lub.mv = (int32_t*)(base + o_lumv);
    // size groups: n > hi, lo < n <= hi, n <= lo (by default 1024 and 384;
    // with batch.group_mid, lo < n <= hi splits at mid; empty groups dropped)
    {
        int64_t bounds[MAX_GROUPS_B] = {h->tp.batch_group_hi, h->tp.batch_group_lo, 0};
        int nb = 2;
        if (h->tp.batch_group_mid > 0) {
            bounds[1] = h->tp.batch_group_mid;
            bounds[2] = h->tp.batch_group_lo;
            nb = 3;
        }
        int i0 = 0;
        int greatest = 0, least = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        for (int g = 0; g <= nb && rc == GBVLM_OK; g++) {
            int i1 = i0;
            while (i1 < h->nsys && (g == nb || lun[i1] > bounds[g])) i1++;
            if (i1 == i0) continue;
            const int gi = h->ngroups++;
            h->gtile[gi][0] = h->tpfx_host[i0];
            h->gtile[gi][1] = h->tpfx_host[i1] - h->tpfx_host[i0];
            h->gtile_rows[gi][0] = h->tpfx_rows_host[i0];
            h->gtile_rows[gi][1] = h->tpfx_rows_host[i1] - h->tpfx_rows_host[i0];
            std::vector<int64_t> ns(lun.begin() + i0, lun.begin() + i1);
            h->plans[gi].mem = h->mem;
            rc = lu_plan_build(h->plans[gi], ns, 0, i0);
            if (rc == GBVLM_OK) {
                cudaError_t ee = cudaStreamCreateWithPriority(&h->side[gi], cudaStreamNonBlocking,
                                                              gi == 0 ? greatest : least);
                if (ee == cudaSuccess) ee = cudaEventCreateWithFlags(&h->join[gi], cudaEventDisableTiming);
                if (ee == cudaSuccess && fp64_residual)
                    ee = cudaEventCreateWithFlags(&h->asm_done[gi], cudaEventDisableTiming);
                if (ee != cudaSuccess) rc = cuda_fail(ee, "batch streams", __FILE__, __LINE__);
            }
            i0 = i1;
        }
        if (rc == GBVLM_OK) {
            cudaError_t ee = cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming);
            if (ee == cudaSuccess && fp64_residual)
                ee = cudaStreamCreateWithPriority(&h->lo_side, cudaStreamNonBlocking, least);
            if (ee == cudaSuccess && fp64_residual) ee = cudaEventCreateWithFlags(&h->lo_join, cudaEventDisableTiming);
            if (ee != cudaSuccess) rc = cuda_fail(ee, "batch streams", __FILE__, __LINE__);
        }
    }
    if (rc == GBVLM_OK) {
        // every system and every block of 8 right-hand sides in one dataflow
        // launch; GBVLM_TRS_FLOW=0 selects the per-system solves (k_trsolve,
        // or 128-row blocks on the tensor cores for one large system)
        // (beyond the dataflow solve's limits the plan keeps the per-system solves)
        const char* fe = getenv("GBVLM_TRS_FLOW");
        int32_t mr = 1;
        for (auto& sy : h->sys) mr = std::max(mr, sy.nrhs);
        h->use_flow = !(fe && fe[0] == '0') && trs_flow_fits(h->nsys, (mr + 7) / 8);
        h->flow.mem = h->mem;
        if (h->use_flow) rc = trs_flow_build(h->flow, lun, 0, (mr + 7) / 8);
    }
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return GBVLM_OK;
}

int gbvlm_batch_destroy(gbvlm_batch h) {
    delete h;
    return GBVLM_OK;
}

int gbvlm_batch_info(gbvlm_batch h, int64_t* nsolve, int64_t* nsys, int64_t* gamma_floats, double* interactions,
                     double* lu_flops, int64_t* arena_bytes) {
    GB_REQUIRE(h, "null batch");
    if (nsolve) *nsolve = h->nsolve;
    if (nsys) *nsys = h->nsys;
    if (gamma_floats) *gamma_floats = h->gamma_floats;
    if (interactions) *interactions = h->interactions;
    if (lu_flops) *lu_flops = h->lu_flops;
    if (arena_bytes) *arena_bytes = (int64_t)h->arena_bytes;
    return GBVLM_OK;
}

int gbvlm_batch_launches(gbvlm_batch h, int64_t* out) {
    GB_REQUIRE(h && out, "null argument");
    GB_REQUIRE(h->exec != nullptr || h->launches > 0, "run the batch first");
    *out = h->launches;
    return GBVLM_OK;
}

int gbvlm_batch_set_inputs(gbvlm_batch h, const float* verts, const double* alphas, double u_inf, double rho,
                           const double* ref_pt, gbvlm_stream stream) {
    GB_REQUIRE(h && verts && alphas, "null argument");
    GB_REQUIRE(u_inf > 0 && rho > 0, "u_inf and rho must be positive");
    for (int32_t u = 0; u < h->nsolve; u++)
        GB_REQUIRE(isfinite(alphas[u]), "alpha %d is not finite", u);
    cudaStream_t st = to_cuda(stream);
    // conditions baked into the graph: rebuild it if they change
    const double r[3] = {ref_pt ? ref_pt[0] : 0, ref_pt ? ref_pt[1] : 0, ref_pt ? ref_pt[2] : 0};
    if (u_inf != h->u_inf || rho != h->rho || r[0] != h->ref[0] || r[1] != h->ref[1] || r[2] != h->ref[2]) {
        h->u_inf = u_inf;
        h->rho = rho;
        for (int k = 0; k < 3; k++) h->ref[k] = r[k];
        if (h->exec) {
            cudaGraphExecDestroy(h->exec);
            h->exec = nullptr;
        }
    }
    GB_CUDA(cudaMemcpyAsync(h->d_vin, verts, sizeof(float) * h->vin_floats, cudaMemcpyDefault, st));
    // alphas in user order -> batch order; geometry angles live in the descriptors
    std::vector<double> al(h->nsolve);
    for (int32_t u = 0; u < h->nsolve; u++) al[h->solve_order[u]] = alphas[u];
    bool geom_changed = false;
    for (auto& S : h->sys) {
        const double g = (h->mode == GBVLM_BATCH_EXACT) ? al[S.rhs_off] : 0.0;
        if (g != S.alpha_geom) {
            S.alpha_geom = g;
            geom_changed = true;
        }
    }
    if (geom_changed) {
        GB_CUDA(cudaStreamSynchronize(st));
        GB_CUDA(cudaMemcpy(h->d_sys, h->sys.data(), sizeof(SysDesc) * h->nsys, cudaMemcpyHostToDevice));
    }
    GB_CUDA(cudaMemcpyAsync(h->d_alpha, al.data(), sizeof(double) * h->nsolve, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaStreamSynchronize(st));  // `al` is a host temporary
    return GBVLM_OK;
}

int gbvlm_batch_run_eager(gbvlm_batch h, int32_t want_gamma, gbvlm_stream stream) {
    GB_REQUIRE(h, "null batch");
    h->want_gamma = want_gamma ? 1 : 0;
    if (h->exec) {  // a captured graph bakes want_gamma in
        cudaGraphExecDestroy(h->exec);
        h->exec = nullptr;
    }
    int rc = batch_enqueue(h, to_cuda(stream));
    if (rc == GBVLM_OK) GB_CUDA(cudaEventRecord(h->done, to_cuda(stream)));
    return rc;
}

int gbvlm_batch_run(gbvlm_batch h, int32_t want_gamma, gbvlm_stream stream) {
    GB_REQUIRE(h, "null batch");
    cudaStream_t st = to_cuda(stream);
    if (want_gamma != h->want_gamma && h->exec) {
        cudaGraphExecDestroy(h->exec);
        h->exec = nullptr;
    }
    h->want_gamma = want_gamma ? 1 : 0;
    if (!h->exec) {
        if (!h->cap) GB_CUDA(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking));
        if (h->graph) {
            cudaGraphDestroy(h->graph);
            h->graph = nullptr;
        }
        GB_CUDA(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal));
        int rc = batch_enqueue(h, h->cap);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(h->cap, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        GB_CUDA(e);
        h->graph = g;
        GB_CUDA(cudaGraphInstantiate(&h->exec, h->graph, cudaGraphInstantiateFlagUseNodePriority));
    }
    GB_CUDA(cudaGraphLaunch(h->exec, st));
    GB_CUDA(cudaEventRecord(h->done, st));
    return GBVLM_OK;
}

int gbvlm_batch_profile(gbvlm_batch h, float* stage_ms, gbvlm_stream stream) {
    GB_REQUIRE(h && stage_ms, "null argument");
    cudaStream_t st = to_cuda(stream);
    cudaEvent_t ev[7];
    for (int k = 0; k < 7; k++) GB_CUDA(cudaEventCreate(&ev[k]));
    int rc = batch_enqueue(h, st, ev);
    if (rc == GBVLM_OK) {
        cudaEventRecord(h->done, st);
        cudaError_t e = cudaEventSynchronize(ev[6]);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventSynchronize", __FILE__, __LINE__);
        for (int k = 0; k < 6 && rc == GBVLM_OK; k++) {
            e = cudaEventElapsedTime(&stage_ms[k], ev[k], ev[k + 1]);
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventElapsedTime", __FILE__, __LINE__);
        }
    }
    for (int k = 0; k < 7; k++) cudaEventDestroy(ev[k]);
    return rc;
}

int gbvlm_batch_update_profile(gbvlm_batch h, double* out, gbvlm_stream stream) {
    GB_REQUIRE(h && out, "null argument");
    cudaStream_t st = to_cuda(stream);
    std::vector<cudaEvent_t> ev;
    for (int g = 0; g < h->ngroups; g++) h->plans[g].tc_events = &ev;
    int rc = batch_enqueue(h, st, nullptr, true);
    for (int g = 0; g < h->ngroups; g++) h->plans[g].tc_events = nullptr;
    double ms = 0;
    if (rc == GBVLM_OK) {
        cudaEventRecord(h->done, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
        for (size_t k = 0; k + 1 < ev.size() && rc == GBVLM_OK; k += 2) {
            float t = 0;
            e = cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventElapsedTime", __FILE__, __LINE__);
            ms += t;
        }
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (rc) return rc;
    out[0] = ms;
    out[1] = (double)(ev.size() / 2);
    out[2] = out[3] = 0;
    for (int g = 0; g < h->ngroups; g++) {
        out[2] += h->plans[g].tc_flops;
        out[3] += h->plans[g].tc_bytes;
    }
    return GBVLM_OK;
}

int gbvlm_batch_results(gbvlm_batch h, double* coeffs, float* gamma, gbvlm_stream stream) {
    GB_REQUIRE(h && coeffs, "null argument");
    GB_REQUIRE(!gamma || h->want_gamma, "gamma requested but the last run did not store it");
    cudaStream_t st = to_cuda(stream);
    constexpr int G = gbvlm_batch_s::MAX_GROUPS;
    // outputs are already in the caller's order: straight into the caller's buffers
    GB_CUDA(cudaMemcpyAsync(coeffs, h->d_out, sizeof(double) * 5 * h->nsolve, cudaMemcpyDeviceToHost, st));
    if (gamma)
        GB_CUDA(cudaMemcpyAsync(gamma, h->d_gamma, sizeof(float) * h->gamma_floats, cudaMemcpyDeviceToHost, st));
    // status words (bounded-wait errors of the LU plans and the triangular
    // solve, pivot flags) with the same synchronisation
    const size_t sbytes = sizeof(int32_t) * (G + 1 + 2 * (size_t)h->nsys);
    if (!h->status) {
        h->status = pinned_take(sbytes);
        if (!h->status) {
            set_error("no pinned host memory for the batch status words");
            return GBVLM_ERR_NOMEM;
        }
        h->status_bytes = sbytes;
    }
    int32_t* hs = (int32_t*)h->status;
    memset(hs, 0, sizeof(int32_t) * (G + 1));
    for (int g = 0; g < h->ngroups; g++)
        if (h->plans[g].d_err)
            GB_CUDA(cudaMemcpyAsync(hs + g, h->plans[g].d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    if (h->use_flow && h->flow.d_ctl)
        GB_CUDA(cudaMemcpyAsync(hs + G, h->flow.d_ctl + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(hs + G + 1, h->lub.info, sizeof(int32_t) * h->nsys, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(hs + G + 1 + h->nsys, h->d_bad, sizeof(int32_t) * h->nsys, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    for (int g = 0; g < h->ngroups; g++)
        if (hs[g]) {
            set_error("LU: a tensor-core update tile timed out waiting for its MMAs");
            return GBVLM_ERR_CUDA;
        }
    if (hs[G]) {
        set_error("triangular solve: a block timed out waiting for the blocks it depends on");
        return GBVLM_ERR_CUDA;
    }
    for (int k = 0; k < h->nsys; k++) {
        if (hs[G + 1 + h->nsys + k] != 0) {
            set_error("batch case %d: non-finite vertex coordinates (its solves are not valid)", h->sys[k].case_id);
            return GBVLM_ERR_ARG;
        }
    }
    for (int k = 0; k < h->nsys; k++) {
        if (hs[G + 1 + k] != 0) {
            set_error("batch system %d (case %d): exactly zero pivot at column %d", k, h->sys[k].case_id,
                      hs[G + 1 + k]);
            return GBVLM_ERR_SINGULAR;
        }
    }
    return GBVLM_OK;
}

}  // extern "C"
