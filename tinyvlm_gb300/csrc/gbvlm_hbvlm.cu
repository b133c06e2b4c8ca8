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

// g = C . row_s(D) : g[p] = sum_j C[p + j n] D[s + j N]
__global__ void k_dft_row(const double* C, const double* D, int64_t n, int32_t N, int32_t s, double* g) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    double v = 0;
    for (int32_t j = 0; j < N; j++) v += C[p + j * n] * D[s + j * N];
    g[p] = v;
}

// chordwise delta of one surface; with `prev_te` the first chordwise row
// also loses the previous surface's trailing-edge gamma (libhbvlm3.cpp:476-480)
__global__ void k_delta(const double* g, int64_t ns, int64_t nc, const double* prev_te, double* d) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= ns * nc) return;
    const int64_t i = p % ns, j = p / ns;
    double v = g[p];
    if (j > 0) v -= g[p - ns];
    else if (prev_te) v -= prev_te[i];
    d[p] = v;
}

template <class T>
__global__ void k_vel_dual(const double* Td, const double* c0, double* vel, int64_t np) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const double x = c0[p], y = c0[np + p], z = c0[2 * np + p];
    for (int r = 0; r < 3; r++) vel[r * np + p] = -(Td[r] * x + Td[r + 4] * y + Td[r + 8] * z + Td[r + 12]);
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
constexpr int WOP_THREADS = 128;
constexpr int WOP_NMAX = 32;  // Fourier coefficients a thread accumulates (harmonics <= 15)

struct WopInst {
    const double* colloc[GBVLM_MAX_SURFACES];
    const double* normals[GBVLM_MAX_SURFACES];
    const double* rhs_vel;  // -V.n of the instance (n)
    double* basis;          // (it x N) row-major
    int64_t it;             // active wake rows
    double t;               // instance time
};

struct WopArgs {
    const WopInst* inst;
    int32_t nsurf, N, H;
    int64_t poff[GBVLM_MAX_SURFACES + 1];
    const double* wake;  // lifting wake vertices, 4 planes of (ns+1) x nwv
    int64_t wns, nwv;
    int64_t rows_per_slice;
    double* partial;  // [slice][instance][n * wns][N]
};

// basis_q(j, c) for the active rows of every instance (grid y: instance),
// the same phases as k_gamma_wake in the operator library
__global__ void k_hb_basis(WopArgs a, double omega, double dt) {
    const WopInst& I = a.inst[blockIdx.y];
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // j - start
    if (r >= I.it) return;
    const int32_t U = a.N;
    const double s0 = 1.0 / sqrt((double)U), s2 = sqrt(2.0 / (double)U);
    double* b = I.basis + r * U;
    b[0] = s0;
    for (int32_t h = 0; h < a.H; h++) {
        const double wk = omega * (double)(h + 1);
        const double ph = wk * (I.t - (double)(r + 1) * dt);
        double sn, cs;
        sincos(ph, &sn, &cs);
        b[2 * h + 1] = cs * s2;
        b[2 * h + 2] = sn * s2;
    }
}

// one thread per (target p, wake span i) of instance blockIdx.y over the
// rows of slice blockIdx.z: the ring values along the rows, each line's
// spanwise segment shared by the two rings it bounds
__global__ void __launch_bounds__(WOP_THREADS) k_wake_operator(WopArgs a) {
    const WopInst& I = a.inst[blockIdx.y];
    const int64_t n = a.poff[a.nsurf], npairs = n * a.wns;
    const int64_t g = blockIdx.x * (int64_t)WOP_THREADS + threadIdx.x;
    if (g >= npairs) return;
    const int64_t p = g / a.wns, i = g - p * a.wns;
    int m = 0;
    while (p >= a.poff[m + 1]) m++;
    const int64_t pl = p - a.poff[m], np = a.poff[m + 1] - a.poff[m];
    const double px = I.colloc[m][pl], py = I.colloc[m][np + pl], pz = I.colloc[m][2 * np + pl];
    const double nx = I.normals[m][pl], ny = I.normals[m][np + pl], nz = I.normals[m][2 * np + pl];
    const int64_t start = a.nwv - 1 - I.it;
    const int64_t j0 = start + (int64_t)blockIdx.z * a.rows_per_slice;
    const int64_t j1 = min(j0 + a.rows_per_slice, a.nwv - 1);
    double acc[WOP_NMAX];
#pragma unroll
    for (int c = 0; c < WOP_NMAX; c++) acc[c] = 0.0;
    if (j0 < j1) {
        const int64_t n1 = a.wns + 1, wl = n1 * a.nwv;
        auto V = [&](int64_t row, int64_t k) {
            const int64_t o = k + row * n1;
            return V3<double>{a.wake[o], a.wake[wl + o], a.wake[2 * wl + o]};
        };
        // line j: v0 = (j, i), v1 = (j, i + 1)
        V3<double> v0 = V(j0, i), v1 = V(j0, i + 1);
        Rel<double> A0 = make_rel<double>(px - v0.x, py - v0.y, pz - v0.z);
        Rel<double> A1 = make_rel<double>(px - v1.x, py - v1.y, pz - v1.z);
        Rel<double> B0 = make_rel<double>(px - v0.x, -py - v0.y, pz - v0.z);
        Rel<double> B1 = make_rel<double>(px - v1.x, -py - v1.y, pz - v1.z);
        double Ta = seg_normal<double, false>(A0, A1, v1.x - v0.x, v1.y - v0.y, v1.z - v0.z, nx, ny, nz, 0.0);
        double Tb = seg_normal<double, false>(B0, B1, v1.x - v0.x, v1.y - v0.y, v1.z - v0.z, nx, -ny, nz, 0.0);
        for (int64_t j = j0; j < j1; j++) {
            // line j + 1: v3 = (j + 1, i), v2 = (j + 1, i + 1)
            const V3<double> v3 = V(j + 1, i), v2 = V(j + 1, i + 1);
            const Rel<double> A3 = make_rel<double>(px - v3.x, py - v3.y, pz - v3.z);
            const Rel<double> A2 = make_rel<double>(px - v2.x, py - v2.y, pz - v2.z);
            const Rel<double> B3 = make_rel<double>(px - v3.x, -py - v3.y, pz - v3.z);
            const Rel<double> B2 = make_rel<double>(px - v2.x, -py - v2.y, pz - v2.z);
            const double rx = v2.x - v1.x, ry = v2.y - v1.y, rz = v2.z - v1.z;  // v1 -> v2
            const double lx = v0.x - v3.x, ly = v0.y - v3.y, lz = v0.z - v3.z;  // v3 -> v0
            const double bx = v2.x - v3.x, by = v2.y - v3.y, bz = v2.z - v3.z;  // v3 -> v2: the next ring's top
            const double Na = seg_normal<double, false>(A3, A2, bx, by, bz, nx, ny, nz, 0.0);
            const double Nb = seg_normal<double, false>(B3, B2, bx, by, bz, nx, -ny, nz, 0.0);
            double val = Ta + seg_normal<double, false>(A1, A2, rx, ry, rz, nx, ny, nz, 0.0) - Na +
                         seg_normal<double, false>(A3, A0, lx, ly, lz, nx, ny, nz, 0.0);
            val += Tb + seg_normal<double, false>(B1, B2, rx, ry, rz, nx, -ny, nz, 0.0) - Nb +
                   seg_normal<double, false>(B3, B0, lx, ly, lz, nx, -ny, nz, 0.0);
            const double* br = I.basis + (j - start) * a.N;
#pragma unroll
            for (int c = 0; c < WOP_NMAX; c++)
                if (c < a.N) acc[c] += val * br[c];
            v0 = v3, v1 = v2;
            A0 = A3, A1 = A2, B0 = B3, B1 = B2;
            Ta = Na, Tb = Nb;
        }
    }
    double* out = a.partial + (((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * npairs + g) * a.N;
#pragma unroll
    for (int c = 0; c < WOP_NMAX; c++)
        if (c < a.N) out[c] = acc[c];
}

// M = sum over slices of the partial operators, in slice order
__global__ void k_wake_operator_sum(const double* partial, int64_t slices, int64_t len, double* M) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= len) return;
    double s = 0;
    for (int64_t k = 0; k < slices; k++) s += partial[k * len + e];
    M[e] = s;
}

// One map's right-hand sides and their DFT, one block per target p:
// R(p, q) = -V.n_q(p) - sum_{i,c} Mq(p, i, c) te(i, c) / (4 pi), with te
// read from the iterate X (n x N) at the lifting surface's trailing-edge
// row; then Y(p, k) = sum_q R(p, q) D(q, k).
constexpr int HBR_THREADS = 128;
__global__ void __launch_bounds__(HBR_THREADS) k_hb_rhs(const WopInst* inst, const double* M, const double* X,
                                                        int64_t n, int64_t te_off, int64_t wns, int32_t N,
                                                        const double* D, double* Y) {
    __shared__ double R[WOP_NMAX];
    const int64_t p = blockIdx.x;
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

struct Inst {
    int64_t t_steps = 0;
    double t = 0;
    std::vector<double*> colloc, normals;
    double* rhs_vel = nullptr;
    std::vector<double*> gwake;
};

struct HbState {
    int32_t nsurf = 0, wake_surf = 0, N = 0;
    std::vector<gbvlm_dims> dims;
    std::vector<int32_t> lifting;
    int64_t n = 0, max_t = 0;
    std::vector<int64_t> poff;
    std::vector<void*> allocs;
    std::vector<double*> vinit, verts, wake, colloc_h, colloc, normals, areas, vel, forces, gdelta, gdt, gam, trans;
    double *lhs = nullptr, *D = nullptr, *Xin = nullptr, *Xout = nullptr, *R = nullptr, *te = nullptr;
    gbvlm_lu lu = nullptr;
    std::vector<Inst> inst;
    // the wake operator (k_wake_operator): instance table, basis rows,
    // partial sums and the operators, built at the first map of a solve
    WopInst* d_wop = nullptr;
    double *wop_basis = nullptr, *wop_part = nullptr, *wop_M = nullptr;
    size_t wop_part_cap = 0, wop_M_cap = 0;
    bool wop_valid = false;
    double wop_omega = 0, wop_dt = 0;

    ~HbState() {
        if (lu) gbvlm_lu_destroy(lu);
        for (void* p : allocs) cudaFree(p);
        for (void* p : {(void*)d_wop, (void*)wop_basis, (void*)wop_part, (void*)wop_M})
            if (p) cudaFree(p);
    }

    // the wake term through the precomputed operator unless the harmonics
    // exceed what a thread accumulates (or GBVLM_HB_DIRECT=1 asks for the
    // per-map Biot-Savart sums)
    bool use_wop() const {
        if (N > WOP_NMAX) return false;
        const char* e = getenv("GBVLM_HB_DIRECT");
        return !(e && e[0] == '1');
    }

    static int grow(double** p, size_t* cap, size_t cnt) {
        if (*cap >= cnt) return GBVLM_OK;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *cap = 0;
        GB_CUDA(cudaMalloc((void**)p, sizeof(double) * cnt));
        *cap = cnt;
        return GBVLM_OK;
    }

    // basis rows, ring values contracted with them per slice of wake rows,
    // and the slice sums (for the map's omega and dt)
    int build_wop(double omega, double dt, cudaStream_t st) {
        const gbvlm_dims& W = dims[wake_surf];
        int64_t max_it = 1;
        for (const Inst& I : inst) max_it = std::max(max_it, I.t_steps);
        WopArgs a;
        a.inst = d_wop;
        a.nsurf = nsurf;
        a.N = N;
        a.H = (N - 1) / 2;
        for (int m = 0; m <= nsurf; m++) a.poff[m] = poff[m];
        a.wake = wake[wake_surf];
        a.wns = W.ns;
        a.nwv = max_t;
        const int64_t npairs = n * W.ns, xb = cdiv(npairs, WOP_THREADS);
        // about four waves of 152 SMs, at least 32 rows per slice
        int64_t slices = std::max<int64_t>(1, cdiv(4 * 152, xb * N));
        const int64_t rps = std::max<int64_t>(32, cdiv(max_it, slices));
        slices = std::max<int64_t>(1, cdiv(max_it, rps));
        a.rows_per_slice = rps;
        const int64_t len = (int64_t)N * npairs * N;
        int rc;
        if ((rc = grow(&wop_part, &wop_part_cap, (size_t)(slices * len)))) return rc;
        if ((rc = grow(&wop_M, &wop_M_cap, (size_t)len))) return rc;
        a.partial = wop_part;
        k_hb_basis<<<dim3((unsigned)cdiv(max_it, 128), (unsigned)N), 128, 0, st>>>(a, omega, dt);
        GB_LAUNCH_CHECK();
        k_wake_operator<<<dim3((unsigned)xb, (unsigned)N, (unsigned)slices), WOP_THREADS, 0, st>>>(a);
        GB_LAUNCH_CHECK();
        k_wake_operator_sum<<<(unsigned)cdiv(len, 256), 256, 0, st>>>(wop_part, slices, len, wop_M);
        GB_LAUNCH_CHECK();
        wop_valid = true;
        wop_omega = omega;
        wop_dt = dt;
        return GBVLM_OK;
    }

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
            for (auto* vec : {&colloc_h, &colloc, &normals, &vel, &forces}) {
                if ((rc = alloc(&p, 3 * np))) return rc;
                vec->push_back(p);
            }
            for (auto* vec : {&areas, &gdelta, &gdt, &gam}) {
                if ((rc = alloc(&p, np))) return rc;
                vec->push_back(p);
            }
            if ((rc = alloc(&p, 16))) return rc;
            trans.push_back(p);
        }
        n = poff[nsurf];
        if ((rc = alloc(&lhs, n * n))) return rc;
        if ((rc = gbvlm_lu_create(&lu))) return rc;
        return gbvlm_lu_init(lu, n);
    }

    int place(const double* Th, cudaStream_t st) {
        for (int m = 0; m < nsurf; m++)
            GB_CUDA(cudaMemcpyAsync(trans[m], Th + 16 * m, sizeof(double) * 16, cudaMemcpyHostToDevice, st));
        return gbvlm_displace_wing_f64(nsurf, dims.data(), C(trans).data(), verts.data(), C(vinit).data(),
                                       (gbvlm_stream)st);
    }

    // libhbvlm3.cpp:266-319: metrics at the undisplaced pose, AIC without wake, factor, wake pre-generation
    int prepare(int32_t harmonics, int64_t max_t_steps, const double* wake_T, cudaStream_t st) {
        gbvlm_stream s = (gbvlm_stream)st;
        N = 2 * harmonics + 1;
        max_t = max_t_steps;
        int rc;
        for (auto& d : dims) d.nwv = max_t;
        for (double* p : wake) cudaFree(p);
        wake.clear();
        for (int m = 0; m < nsurf; m++) {
            double* p;
            GB_CUDA(cudaMalloc((void**)&p, sizeof(double) * 4 * (dims[m].ns + 1) * max_t));
            GB_CUDA(cudaMemset(p, 0, sizeof(double) * 4 * (dims[m].ns + 1) * max_t));
            wake.push_back(p);
        }
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
        double* Tall = nullptr;
        GB_CUDA(cudaMalloc((void**)&Tall, sizeof(double) * 16 * nsurf * max_t));
        GB_CUDA(cudaMemcpyAsync(Tall, wake_T, sizeof(double) * 16 * nsurf * max_t, cudaMemcpyHostToDevice, st));
        for (int m = 0; m < nsurf; m++) {
            const int64_t cnt = (dims[m].ns + 1) * max_t;
            k_pregen_wake<<<(unsigned)cdiv(cnt, 128), 128, 0, st>>>(Tall, nsurf, m, vinit[m], dims[m].ns, dims[m].nc,
                                                                     max_t, wake[m]);
            GB_LAUNCH_CHECK();
        }
        GB_CUDA(cudaStreamSynchronize(st));
        cudaFree(Tall);
        wop_valid = false;
        return GBVLM_OK;
    }

    // per-instance geometry, -V.n and wake-gamma buffers (libhbvlm3.cpp:363-393 without the gamma part)
    int set_instances(const int64_t* t_steps, const double* times, const double* Th, const double* Tdh,
                      const double* dft, cudaStream_t st) {
        gbvlm_stream s = (gbvlm_stream)st;
        int rc;
        for (auto& I : inst) {
            for (double* p : I.colloc) cudaFree(p);
            for (double* p : I.normals) cudaFree(p);
            for (double* p : I.gwake) cudaFree(p);
            if (I.rhs_vel) cudaFree(I.rhs_vel);
        }
        inst.assign(N, Inst());
        if (!D && (rc = alloc(&D, N * N))) return rc;
        if (!Xin) {
            if ((rc = alloc(&Xin, n * N)) || (rc = alloc(&Xout, n * N)) || (rc = alloc(&R, n * N)) ||
                (rc = alloc(&te, dims[wake_surf].ns * N)))
                return rc;
        }
        GB_CUDA(cudaMemcpy(D, dft, sizeof(double) * N * N, cudaMemcpyHostToDevice));
        std::vector<double*> tdm(nsurf);
        for (int m = 0; m < nsurf; m++) {
            GB_CUDA(cudaMalloc((void**)&tdm[m], sizeof(double) * 16));
        }
        for (int q = 0; q < N; q++) {
            Inst& I = inst[q];
            I.t_steps = t_steps[q];
            I.t = times[q];
            GB_REQUIRE(I.t_steps >= 0 && I.t_steps <= max_t - 1, "instance %d: t_steps %lld outside the wake", q,
                       (long long)I.t_steps);
            if ((rc = place(Th + 16 * nsurf * q, st))) return rc;
            for (int m = 0; m < nsurf; m++) {
                const int64_t np = dims[m].ns * dims[m].nc;
                double *c, *nm, *gw;
                GB_CUDA(cudaMalloc((void**)&c, sizeof(double) * 3 * np));
                GB_CUDA(cudaMalloc((void**)&nm, sizeof(double) * 3 * np));
                GB_CUDA(cudaMalloc((void**)&gw, sizeof(double) * dims[m].ns * (max_t - 1)));
                GB_CUDA(cudaMemset(gw, 0, sizeof(double) * dims[m].ns * (max_t - 1)));
                I.colloc.push_back(c);
                I.normals.push_back(nm);
                I.gwake.push_back(gw);
            }
            if ((rc = gbvlm_mesh_metrics_f64(0.0, nsurf, dims.data(), C(verts).data(), I.colloc.data(),
                                             I.normals.data(), areas.data(), s)))
                return rc;
            for (int m = 0; m < nsurf; m++) {
                const int64_t np = dims[m].ns * dims[m].nc;
                GB_CUDA(cudaMemcpyAsync(tdm[m], Tdh + 16 * (nsurf * q + m), sizeof(double) * 16, cudaMemcpyHostToDevice, st));
                k_vel_dual<double><<<(unsigned)cdiv(np, 128), 128, 0, st>>>(tdm[m], colloc_h[m], vel[m], np);
                GB_LAUNCH_CHECK();
            }
            GB_CUDA(cudaMalloc((void**)&I.rhs_vel, sizeof(double) * n));
            GB_CUDA(cudaMemsetAsync(I.rhs_vel, 0, sizeof(double) * n, st));
            if ((rc = gbvlm_rhs_assemble_velocities_f64(I.rhs_vel, nsurf, dims.data(), C(I.normals).data(),
                                                        C(vel).data(), s)))
                return rc;
            GB_CUDA(cudaStreamSynchronize(st));
        }
        for (double* p : tdm) cudaFree(p);
        // the operator's instance table and basis rows
        wop_valid = false;
        int64_t rows = 0;
        for (const Inst& I : inst) rows += std::max<int64_t>(I.t_steps, 1);
        if (wop_basis) cudaFree(wop_basis);
        wop_basis = nullptr;
        GB_CUDA(cudaMalloc((void**)&wop_basis, sizeof(double) * rows * N));
        if (!d_wop) GB_CUDA(cudaMalloc((void**)&d_wop, sizeof(WopInst) * (2 * 64 + 1)));
        std::vector<WopInst> tab(N);
        int64_t off = 0;
        for (int q = 0; q < N; q++) {
            WopInst& w = tab[q];
            memset(&w, 0, sizeof(w));
            for (int m = 0; m < nsurf; m++) {
                w.colloc[m] = inst[q].colloc[m];
                w.normals[m] = inst[q].normals[m];
            }
            w.rhs_vel = inst[q].rhs_vel;
            w.basis = wop_basis + off * N;
            w.it = inst[q].t_steps;
            w.t = inst[q].t;
            off += std::max<int64_t>(inst[q].t_steps, 1);
        }
        GB_CUDA(cudaMemcpy(d_wop, tab.data(), sizeof(WopInst) * N, cudaMemcpyHostToDevice));
        return GBVLM_OK;
    }

    // one fixed-point map on device buffers Xin -> Xout (libhbvlm3.cpp:349-410)
    int map_dev(double omega, double dt, int32_t harmonics, cudaStream_t st) {
        gbvlm_stream s = (gbvlm_stream)st;
        int rc;
        const gbvlm_dims& W = dims[wake_surf];
        const int64_t te_off = poff[wake_surf] + (W.nc - 1) * W.ns;
        if (use_wop()) {
            if ((!wop_valid || omega != wop_omega || dt != wop_dt) && (rc = build_wop(omega, dt, st))) return rc;
            k_hb_rhs<<<(unsigned)n, HBR_THREADS, 0, st>>>(d_wop, wop_M, Xin, n, te_off, W.ns, N, D, Xout);
            GB_LAUNCH_CHECK();
            return gbvlm_lu_solve_f64(lu, lhs, n, n, Xout, n, N, s);
        }
        k_gather_te<<<(unsigned)cdiv(W.ns * N, 128), 128, 0, st>>>(Xin, n, te_off, W.ns, N, te);
        GB_LAUNCH_CHECK();
        for (int q = 0; q < N; q++) {
            Inst& I = inst[q];
            if ((rc = gbvlm_gamma_wake_from_coeffs_f64(I.gwake[wake_surf], W.ns, max_t - 1, te, harmonics, I.t, omega,
                                                        dt, I.t_steps, s)))
                return rc;
            double* col = R + (int64_t)q * n;
            GB_CUDA(cudaMemcpyAsync(col, I.rhs_vel, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            if ((rc = gbvlm_rhs_assemble_wake_influence_f64(col, nsurf, dims.data(), C(I.gwake).data(),
                                                            C(I.colloc).data(), C(I.normals).data(), C(wake).data(),
                                                            lifting.data(), (int32_t)I.t_steps, 0.0, s)))
                return rc;
        }
        k_rdft<<<(unsigned)cdiv(n * N, 128), 128, 0, st>>>(R, D, n, N, Xout);
        GB_LAUNCH_CHECK();
        return gbvlm_lu_solve_f64(lu, lhs, n, n, Xout, n, N, s);
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
// fit, into the global work buffers Wg, bg) and runs the Householder QR
// there: for each column j, warp 0 forms the reflector (its norm, the new
// pivot, v^T v = 2 |a| (|a| + |a_j|)), then the warps reflect the later
// columns and the right-hand side in parallel, one column per warp at a
// time.  fp64 runs at a small fraction of the fp32 rate on this part, so the
// work is spread over all four schedulers' fp64 units.
constexpr int AA_STEP_THREADS = 256;

__global__ void __launch_bounds__(AA_STEP_THREADS) k_anderson_step(int64_t L, int mk, int slot, double* X,
                                                                   const double* G, double* Wg, double* bg,
                                                                   const double* g, double* x, int use_smem) {
    extern __shared__ double aa_sm[];
    __shared__ double gam[16], diag[16];
    __shared__ double s_nrm, s_rvv;
    double* W = use_smem ? aa_sm : Wg;
    double* b = use_smem ? aa_sm + L * mk : bg;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    for (int64_t e = tid; e < L * mk; e += blockDim.x) W[e] = G[e];
    for (int64_t i = tid; i < L; i += blockDim.x) b[i] = g[i];
    // dot products over rows j..L-1, four partial sums per lane, warp-reduced
    auto dot = [&](const double* u, const double* w, int j) {
        double t0 = 0, t1 = 0, t2 = 0, t3 = 0;
        int64_t i = j + lane;
        for (; i + 96 < L; i += 128) {
            t0 += u[i] * w[i];
            t1 += u[i + 32] * w[i + 32];
            t2 += u[i + 64] * w[i + 64];
            t3 += u[i + 96] * w[i + 96];
        }
        for (; i < L; i += 32) t0 += u[i] * w[i];
        return aa_wsum((t0 + t1) + (t2 + t3));
    };
    __syncthreads();
    for (int j = 0; j < mk; j++) {
        double* wj = W + (int64_t)j * L;
        if (wid == 0) {
            const double nrm = sqrt(dot(wj, wj, j));
            if (lane == 0) {
                s_nrm = nrm;
                diag[j] = 0;
                if (nrm != 0) {
                    const double a0 = wj[j];
                    const double alpha = a0 > 0 ? -nrm : nrm;
                    wj[j] = a0 - alpha;
                    diag[j] = alpha;
                    s_rvv = 1.0 / (2.0 * nrm * (nrm + fabs(a0)));
                }
            }
        }
        __syncthreads();
        if (s_nrm != 0) {  // uniform
            const double rvv = s_rvv;
            for (int t = wid; t < mk - j; t += nw) {  // the later columns, then the right-hand side
                double* wc = t < mk - j - 1 ? W + (int64_t)(j + 1 + t) * L : b;
                const double f = 2.0 * dot(wj, wc, j) * rvv;
                for (int64_t i = j + lane; i < L; i += 32) wc[i] -= f * wj[i];
            }
        }
        __syncthreads();
    }
    if (tid == 0)
        for (int j = mk - 1; j >= 0; j--) {
            double sj = b[j];
            for (int c = j + 1; c < mk; c++) sj -= W[j + (int64_t)c * L] * gam[c];
            gam[j] = diag[j] != 0 ? sj / diag[j] : 0;
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
__global__ void __launch_bounds__(AA_THREADS) k_anderson_post(int64_t L, int slot, const double* fx, const double* x,
                                                              double* g, double* G, double* norm) {
    __shared__ double sh[32];
    double t = 0;
    for (int64_t i = threadIdx.x; i < L; i += blockDim.x) {
        const double gn = fx[i] - x[i];
        if (slot >= 0) G[i + (int64_t)L * slot] = gn - g[i];
        g[i] = gn;
        t += gn * gn;
    }
    const double s2 = aa_sum(t, sh);
    if (threadIdx.x == 0) *norm = sqrt(s2);
}

// the first step (vlm_solvers.cpp:49-66): X[:, 0] = g, x = f(x)
__global__ void k_anderson_first(int64_t L, const double* fx, double* x, const double* g, double* X) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L; i += (int64_t)gridDim.x * blockDim.x) {
        X[i] = g[i];
        x[i] = fx[i];
    }
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
    GB_REQUIRE(h && wake_transforms && t_steps && times && transforms && dtransforms && dft, "null argument");
    GB_REQUIRE(harmonics >= 0 && harmonics <= 64 && max_t_steps >= 2, "bad sizes");
    int rc = h->st.prepare(harmonics, max_t_steps, wake_transforms, to_cuda(stream));
    if (rc) return rc;
    return h->st.set_instances(t_steps, times, transforms, dtransforms, dft, to_cuda(stream));
}

int gbvlm_hbvlm_map(gbvlm_hbvlm h, const double* x_in, double* x_out, double omega, double dt, gbvlm_stream stream) {
    GB_REQUIRE(h && x_in && x_out && h->st.N > 0, "map before prepare");
    HbState& S = h->st;
    cudaStream_t st = to_cuda(stream);
    GB_CUDA(cudaMemcpyAsync(S.Xin, x_in, sizeof(double) * S.n * S.N, cudaMemcpyHostToDevice, st));
    int rc = S.map_dev(omega, dt, (S.N - 1) / 2, st);
    if (rc) return rc;
    GB_CUDA(cudaMemcpyAsync(x_out, S.Xout, sizeof(double) * S.n * S.N, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    return GBVLM_OK;
}

int gbvlm_hbvlm_solve(gbvlm_hbvlm h, double* x, double omega, double dt, int32_t max_iter, double tol, int32_t m,
                      int32_t* iters, gbvlm_stream stream) {
    GB_REQUIRE(h && x && h->st.N > 0, "solve before prepare");
    GB_REQUIRE(m >= 1 && m <= 16 && max_iter >= 2, "history m in [1, 16], max_iter >= 2");
    HbState& S = h->st;
    cudaStream_t st = to_cuda(stream);
    const int64_t L = S.n * S.N;
    const int32_t H = (S.N - 1) / 2;
    // device state: the iterate lives in the map's input S.Xin; g, the
    // histories X and G, the QR work copy of G and its right-hand side
    double* buf = nullptr;
    GB_CUDA(cudaMalloc((void**)&buf, sizeof(double) * ((size_t)L * (3 * m + 2) + 1)));
    double *g = buf, *X = g + L, *G = X + (size_t)L * m, *W = G + (size_t)L * m, *b = W + (size_t)L * m,
           *dnorm = b + L;
    double* hn = (double*)host_scratch(sizeof(double));
    int rc = GBVLM_OK;
    auto fail = [&](int r) {
        cudaFree(buf);
        return r;
    };
    auto map = [&]() { return S.map_dev(omega, dt, H, st); };  // S.Xin -> S.Xout
    const unsigned g1 = (unsigned)std::min<int64_t>(cdiv(L, 256), 1024);
    if (cudaMemcpyAsync(S.Xin, x, sizeof(double) * L, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaMemcpyAsync", __FILE__, __LINE__));
    if (cudaMemsetAsync(X, 0, sizeof(double) * (size_t)L * m * 2, st) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaMemsetAsync", __FILE__, __LINE__));
    // vlm_solvers.cpp:49-66: g0 = f(x0) - x0; X0 = g0; x1 = f(x0); g1 = f(x1) - x1; G0 = g1 - g0
    if ((rc = map())) return fail(rc);
    k_anderson_post<<<1, AA_THREADS, 0, st>>>(L, -1, S.Xout, S.Xin, g, G, dnorm);
    k_anderson_first<<<g1, 256, 0, st>>>(L, S.Xout, S.Xin, g, X);
    if ((rc = map())) return fail(rc);
    k_anderson_post<<<1, AA_THREADS, 0, st>>>(L, 0, S.Xout, S.Xin, g, G, dnorm);
    if (cudaGetLastError() != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "Anderson", __FILE__, __LINE__));
    // the QR's columns in shared memory when m of them and g fit
    const size_t smem = sizeof(double) * (size_t)L * (m + 1);
    const int use_smem = smem <= 200 * 1024 ? 1 : 0;
    if (use_smem && cudaFuncSetAttribute(k_anderson_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                        cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaFuncSetAttribute", __FILE__, __LINE__));
    int k = 1;
    while (k < max_iter) {
        if (cudaMemcpyAsync(hn, dnorm, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError(), "Anderson norm", __FILE__, __LINE__));
        if (!(*hn > tol)) break;
        const int mk = std::min(m, k), slot = k % m;
        k_anderson_step<<<1, AA_STEP_THREADS, use_smem ? smem : 0, st>>>(L, mk, slot, X, G, W, b, g, S.Xin,
                                                                          use_smem);
        if ((rc = map())) return fail(rc);
        k_anderson_post<<<1, AA_THREADS, 0, st>>>(L, slot, S.Xout, S.Xin, g, G, dnorm);
        if (cudaGetLastError() != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError(), "Anderson", __FILE__, __LINE__));
        k++;
    }
    if (cudaMemcpyAsync(x, S.Xin, sizeof(double) * L, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaMemcpyAsync", __FILE__, __LINE__));
    cudaFree(buf);
    if (iters) *iters = k;
    return GBVLM_OK;
}

// libhbvlm3.cpp:428-550: loads at the force instances.  coeffs (n x N),
// dft / ddft (N x N), per instance transforms/rates (N x nsurf x 16),
// freestream (N x 3), ref_a / ref_b (N x 3; ref_b may be NULL).  out: 3 x N
// row-major [cl; cm_y about ref_a (multibody); cm_y of surface 1 about ref_b].
int gbvlm_hbvlm_loads(gbvlm_hbvlm h, const double* coeffs, const double* dft, const double* ddft,
                      const double* transforms, const double* dtransforms, const double* freestream,
                      const double* ref_a, const double* ref_b, int32_t coupled_te, double* out, gbvlm_stream stream) {
    GB_REQUIRE(h && coeffs && dft && ddft && transforms && dtransforms && freestream && ref_a && out, "null argument");
    HbState& S = h->st;
    cudaStream_t st = to_cuda(stream);
    gbvlm_stream s = stream;
    const int N = S.N, ns = S.nsurf;
    int rc = GBVLM_OK;
    double *C, *Dd, *DDd, *td;
    GB_CUDA(cudaMalloc((void**)&C, sizeof(double) * S.n * N));
    GB_CUDA(cudaMalloc((void**)&Dd, sizeof(double) * N * N));
    GB_CUDA(cudaMalloc((void**)&DDd, sizeof(double) * N * N));
    GB_CUDA(cudaMalloc((void**)&td, sizeof(double) * 16 * ns));
    GB_CUDA(cudaMemcpy(C, coeffs, sizeof(double) * S.n * N, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(Dd, dft, sizeof(double) * N * N, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(DDd, ddft, sizeof(double) * N * N, cudaMemcpyHostToDevice));
    double* gfull;
    double* dgfull;
    GB_CUDA(cudaMalloc((void**)&gfull, sizeof(double) * S.n));
    GB_CUDA(cudaMalloc((void**)&dgfull, sizeof(double) * S.n));
    for (int q = 0; q < N && rc == 0; q++) {
        rc = S.place(transforms + 16 * ns * q, st);
        if (rc) break;
        rc = gbvlm_mesh_metrics_f64(0.0, ns, S.dims.data(), S.C(S.verts).data(), S.colloc.data(), S.normals.data(),
                                    S.areas.data(), s);
        if (rc) break;
        GB_CUDA(cudaMemcpyAsync(td, dtransforms + 16 * ns * q, sizeof(double) * 16 * ns, cudaMemcpyHostToDevice, st));
        k_dft_row<<<(unsigned)cdiv(S.n, 128), 128, 0, st>>>(C, Dd, S.n, N, q, gfull);
        k_dft_row<<<(unsigned)cdiv(S.n, 128), 128, 0, st>>>(C, DDd, S.n, N, q, dgfull);
        for (int m = 0; m < ns; m++) {
            const int64_t nsm = S.dims[m].ns, ncm = S.dims[m].nc, np = nsm * ncm;
            k_vel_dual<double><<<(unsigned)cdiv(np, 128), 128, 0, st>>>(td + 16 * m, S.colloc_h[m], S.vel[m], np);
            const double* prev = nullptr;
            if (coupled_te && m > 0 && S.dims[m - 1].ns == nsm) prev = gfull + S.poff[m] - nsm;  // TE row of surface m-1
            k_delta<<<(unsigned)cdiv(np, 128), 128, 0, st>>>(gfull + S.poff[m], nsm, ncm, prev, S.gdelta[m]);
            rc = gbvlm_forces_unsteady_f64(nsm, ncm, S.verts[m], S.gdelta[m], dgfull + S.poff[m], S.vel[m],
                                           S.areas[m], S.normals[m], S.forces[m], s);
            if (rc) break;
        }
        if (rc) break;
        const double* fs = freestream + 3 * q;
        double la[3] = {-fs[2], 0.0, fs[0]};
        const double ll = sqrt(la[0] * la[0] + la[2] * la[2]);
        la[0] /= ll;
        la[2] /= ll;
        double cl = 0, ta = 0, tm = 0, cm = 0;
        for (int m = 0; m < ns && rc == 0; m++) {
            const int64_t nsm = S.dims[m].ns, ncm = S.dims[m].nc;
            double area, clm, mac, cmm[3];
            if ((rc = gbvlm_sum_f64(S.areas[m], nsm * ncm, &area, s))) break;
            if ((rc = gbvlm_coeff_cl_f64(nsm, ncm, S.forces[m], la, fs, 1.0, area, &clm, s))) break;
            if ((rc = gbvlm_mesh_mac_f64(nsm, ncm, S.verts[m], S.areas[m], &mac, s))) break;
            if ((rc = gbvlm_coeff_cm_f64(nsm, ncm, S.forces[m], S.verts[m], ref_a + 3 * q, fs, 1.0, area, mac, cmm, s)))
                break;
            cl += clm * area;
            ta += area;
            tm += mac;
            cm += cmm[1] * area * mac;
            if (m == 1 && ref_b) {
                double cmb[3];
                if ((rc = gbvlm_coeff_cm_f64(nsm, ncm, S.forces[m], S.verts[m], ref_b + 3 * q, fs, 1.0, area, mac, cmb,
                                             s)))
                    break;
                out[2 * N + q] = cmb[1];
            }
        }
        out[q] = cl / ta;
        out[N + q] = cm / (ta * tm);
    }
    cudaFree(C);
    cudaFree(Dd);
    cudaFree(DDd);
    cudaFree(td);
    cudaFree(gfull);
    cudaFree(dgfull);
    return rc;
}

}  // extern "C"
