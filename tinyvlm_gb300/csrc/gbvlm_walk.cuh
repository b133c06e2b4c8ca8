// Ring and strip walkers of the Biot-Savart vortex-ring law, templated on
// the arithmetic type T (float, double, or the float pair Fe of
// gbvlm_math.cuh): the per-operator kernels, the batched assembly and its
// extended-precision correction evaluate the same walk.
#pragma once
#include "gbvlm_math.cuh"

namespace gbvlm {

template <class T>
__device__ __forceinline__ T inv_four_pi();
template <>
__device__ __forceinline__ float inv_four_pi<float>() { return 1.0f / (4.0f * PI_F); }
template <>
__device__ __forceinline__ double inv_four_pi<double>() { return 1.0 / (double)(4.0f * PI_F); }

// value of one full ring (4 vertices given) at point (px,py,pz) + mirror, dotted with normal (unscaled by 1/4pi)
template <class T, bool SIGMA, bool DCUT = false>
__device__ __forceinline__ T ring_normal_full(T px, T py, T pz, T nx, T ny, T nz, const V3<T>* q, T sigma2) {
    Rel<T> a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        a[k] = make_rel<T>(px - q[k].x, py - q[k].y, pz - q[k].z);
        b[k] = make_rel<T>(px - q[k].x, -py - q[k].y, pz - q[k].z);
    }
    T v = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int e = (k + 1) & 3;
        const T rx = q[e].x - q[k].x, ry = q[e].y - q[k].y, rz = q[e].z - q[k].z;
        v += seg_normal<T, SIGMA, DCUT>(a[k], a[e], rx, ry, rz, nx, ny, nz, sigma2);
        v += seg_normal<T, SIGMA, DCUT>(b[k], b[e], rx, ry, rz, nx, -ny, nz, sigma2);
    }
    return v;
}

// Walk the rings of one strip whose vertex lines sit in shared memory
// (top/bot: 3 planes W apart), local vertices 0..nvs-1; calls
// f(ring_index, 4*pi*(v.n + v_mirror.n_mirror)) for rings 0..nvs-2.
// SEG: the segment vectors come precomputed in seg[t * W + k] (shared by all
// evaluation points of a tile): t = 0 the chordwise segment top(k) -> bot(k),
// t = 1 the top segment top(k-1) -> top(k), t = 2 the bottom segment
// bot(k) -> bot(k-1); otherwise each walk forms them.
template <class T, bool SIGMA, bool DCUT = false, bool SEG = false, class F>
__device__ __forceinline__ void strip_normal(const T* top, const T* bot, int W, int nvs, T px, T py, T pz, T nx, T ny,
                                             T nz, T sg, F&& f, const V3<T>* seg = nullptr) {
    auto V = [&](const T* line, int sl) { return V3<T>{line[sl], line[W + sl], line[2 * W + sl]}; };
    V3<T> v0 = V(top, 0), v3 = V(bot, 0);
    Rel<T> A0 = make_rel<T>(px - v0.x, py - v0.y, pz - v0.z), A3 = make_rel<T>(px - v3.x, py - v3.y, pz - v3.z);
    Rel<T> B0 = make_rel<T>(px - v0.x, -py - v0.y, pz - v0.z), B3 = make_rel<T>(px - v3.x, -py - v3.y, pz - v3.z);
    const V3<T> l0 = SEG ? seg[0] : V3<T>{v3.x - v0.x, v3.y - v0.y, v3.z - v0.z};
    T Ca = seg_normal<T, SIGMA, DCUT>(A0, A3, l0.x, l0.y, l0.z, nx, ny, nz, sg);
    T Cb = seg_normal<T, SIGMA, DCUT>(B0, B3, l0.x, l0.y, l0.z, nx, -ny, nz, sg);
    for (int k = 1; k < nvs; k++) {
        const V3<T> v1 = V(top, k), v2 = V(bot, k);
        const Rel<T> A1 = make_rel<T>(px - v1.x, py - v1.y, pz - v1.z), A2 = make_rel<T>(px - v2.x, py - v2.y, pz - v2.z);
        const Rel<T> B1 = make_rel<T>(px - v1.x, -py - v1.y, pz - v1.z), B2 = make_rel<T>(px - v2.x, -py - v2.y, pz - v2.z);
        const V3<T> c3 = SEG ? seg[k] : V3<T>{v2.x - v1.x, v2.y - v1.y, v2.z - v1.z};          // right chordwise segment
        const V3<T> t3 = SEG ? seg[W + k] : V3<T>{v1.x - v0.x, v1.y - v0.y, v1.z - v0.z};      // top segment v0->v1
        const V3<T> b3 = SEG ? seg[2 * W + k] : V3<T>{v3.x - v2.x, v3.y - v2.y, v3.z - v2.z};  // bottom segment v2->v3
        const T cx = c3.x, cy = c3.y, cz = c3.z;
        const T tx = t3.x, ty = t3.y, tz = t3.z;
        const T bx = b3.x, by = b3.y, bz = b3.z;
        const T Cra = seg_normal<T, SIGMA, DCUT>(A1, A2, cx, cy, cz, nx, ny, nz, sg);
        const T Crb = seg_normal<T, SIGMA, DCUT>(B1, B2, cx, cy, cz, nx, -ny, nz, sg);
        T val = seg_normal<T, SIGMA, DCUT>(A0, A1, tx, ty, tz, nx, ny, nz, sg) + Cra +
                seg_normal<T, SIGMA, DCUT>(A2, A3, bx, by, bz, nx, ny, nz, sg) - Ca;
        val += seg_normal<T, SIGMA, DCUT>(B0, B1, tx, ty, tz, nx, -ny, nz, sg) + Crb +
               seg_normal<T, SIGMA, DCUT>(B2, B3, bx, by, bz, nx, -ny, nz, sg) - Cb;
        f(k - 1, val);
        A0 = A1; A3 = A2; B0 = B1; B3 = B2; Ca = Cra; Cb = Crb; v0 = v1; v3 = v2;
    }
}

// Same walk returning 4*pi times the full velocity of each ring (direct + mirror).
template <class T, bool SIGMA, class F>
__device__ __forceinline__ void strip_vec(const T* top, const T* bot, int W, int nvs, T px, T py, T pz, T sg, F&& f) {
    auto V = [&](const T* line, int sl) { return V3<T>{line[sl], line[W + sl], line[2 * W + sl]}; };
    V3<T> v0 = V(top, 0), v3 = V(bot, 0);
    Rel<T> A0 = make_rel<T>(px - v0.x, py - v0.y, pz - v0.z), A3 = make_rel<T>(px - v3.x, py - v3.y, pz - v3.z);
    Rel<T> B0 = make_rel<T>(px - v0.x, -py - v0.y, pz - v0.z), B3 = make_rel<T>(px - v3.x, -py - v3.y, pz - v3.z);
    V3<T> Ca = seg_vec<T, SIGMA>(A0, A3, v3.x - v0.x, v3.y - v0.y, v3.z - v0.z, sg);
    V3<T> Cb = seg_vec<T, SIGMA>(B0, B3, v3.x - v0.x, v3.y - v0.y, v3.z - v0.z, sg);
    for (int k = 1; k < nvs; k++) {
        const V3<T> v1 = V(top, k), v2 = V(bot, k);
        const Rel<T> A1 = make_rel<T>(px - v1.x, py - v1.y, pz - v1.z), A2 = make_rel<T>(px - v2.x, py - v2.y, pz - v2.z);
        const Rel<T> B1 = make_rel<T>(px - v1.x, -py - v1.y, pz - v1.z), B2 = make_rel<T>(px - v2.x, -py - v2.y, pz - v2.z);
        const T cx = v2.x - v1.x, cy = v2.y - v1.y, cz = v2.z - v1.z;
        const T tx = v1.x - v0.x, ty = v1.y - v0.y, tz = v1.z - v0.z;
        const T bx = v3.x - v2.x, by = v3.y - v2.y, bz = v3.z - v2.z;
        const V3<T> Cra = seg_vec<T, SIGMA>(A1, A2, cx, cy, cz, sg), Crb = seg_vec<T, SIGMA>(B1, B2, cx, cy, cz, sg);
        const V3<T> ra = seg_vec<T, SIGMA>(A0, A1, tx, ty, tz, sg) + Cra + seg_vec<T, SIGMA>(A2, A3, bx, by, bz, sg) - Ca;
        const V3<T> rb = seg_vec<T, SIGMA>(B0, B1, tx, ty, tz, sg) + Crb + seg_vec<T, SIGMA>(B2, B3, bx, by, bz, sg) - Cb;
        f(k - 1, V3<T>{ra.x + rb.x, ra.y - rb.y, ra.z + rb.z});
        A0 = A1; A3 = A2; B0 = B1; B3 = B2; Ca = Cra; Cb = Crb; v0 = v1; v3 = v2;
    }
}

}  // namespace gbvlm
