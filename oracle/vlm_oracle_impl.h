/*
 * Oracle (test infrastructure only): a plain-C restatement of the reference's
 * CPU backend for the vortex-lattice hot path.  Included twice by
 * vlm_oracle.c, once with T=float (suffix _f) and once with T=double
 * (suffix _d), so every routine exists in the reference's two precisions.
 *
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * use this code, as the checker.  The product path never links it.
 *
 * Each routine cites the reference file:line it restates (paths relative to
 * the tinyvlm project root).  Loop order and the left-to-right evaluation
 * order of every expression follow the reference so that the float variant
 * rounds like the reference's scalar code; vlm_oracle.c is compiled with
 * -ffp-contract=off so no FMA contraction changes that on any host.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

typedef struct { T x, y, z; } FN(vec3_);
#define V3 FN(vec3_)

static inline V3 FN(v3)(T x, T y, T z) { V3 r = {x, y, z}; return r; }
static inline V3 FN(vsub)(V3 a, V3 b) { return FN(v3)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 FN(vadd)(V3 a, V3 b) { return FN(v3)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 FN(vscale)(T s, V3 a) { return FN(v3)(s * a.x, s * a.y, s * a.z); }
static inline T FN(vdot)(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 FN(vcross)(V3 a, V3 b) {
    return FN(v3)(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline T FN(vlen2)(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline T FN(vlen)(V3 a) { return SQRT(FN(vlen2)(a)); }
static inline V3 FN(vnormalize)(V3 a) {
    T l = FN(vlen)(a);
    return FN(v3)(a.x / l, a.y / l, a.z / l);
}

/* Katz & Plotkin eq. 10.115 straight-segment velocity with the reference's
 * cut-offs and smoothing.  vlm_backend_cpu_kernels.ispc:69-89 (float, cut-off
 * RCUT2 on |r1|,|r2|) and :383-402 (double, cut-off RCUT on all three, and
 * 4*pi still formed as the float product 4.0f*PI_f). */
static inline V3 FN(biosavart)(V3 c, V3 a, V3 b, T sigma) {
    V3 r0 = FN(vsub)(b, a);
    V3 r1 = FN(vsub)(c, a);
    V3 r2 = FN(vsub)(c, b);
    V3 cr = FN(vcross)(r1, r2);
    T r1n = FN(vlen)(r1);
    T r2n = FN(vlen)(r2);
    T sq = FN(vlen2)(cr);
    if ((sq < (T)ORC_RCUT) || (r1n < (T)ORC_RCUT_NORM) || (r2n < (T)ORC_RCUT_NORM)) {
        return FN(v3)(0, 0, 0);
    }
    T smoother = sigma * sigma * FN(vlen2)(r0);
    T coeff = (FN(vdot)(r0, r1) * r2n - FN(vdot)(r0, r2) * r1n) /
              (ORC_FOURPI * SQRT(sq * sq + smoother * smoother) * r1n * r2n);
    return FN(vscale)(coeff, cr);
}

/* Segment plus its image in the y=0 symmetry plane.
 * vlm_backend_cpu_kernels.ispc:91-102 (float), :404-415 (double). */
static inline void FN(symmetry)(V3* inf, V3 c, V3 a, V3 b, T sigma) {
    V3 s = FN(biosavart)(c, a, b, sigma);
    inf->x += s.x; inf->y += s.y; inf->z += s.z;
    c.y = -c.y;
    V3 m = FN(biosavart)(c, a, b, sigma);
    inf->x += m.x; inf->y -= m.y; inf->z += m.z;
}

static inline V3 FN(ring_velocity)(V3 c, V3 v0, V3 v1, V3 v2, V3 v3, T sigma) {
    V3 inf = FN(v3)(0, 0, 0);
    FN(symmetry)(&inf, c, v0, v1, sigma);
    FN(symmetry)(&inf, c, v1, v2, sigma);
    FN(symmetry)(&inf, c, v2, v3, sigma);
    FN(symmetry)(&inf, c, v3, v0, sigma);
    return inf;
}

/* One influencing vortex ring (corner vertex at v, planes v_ld apart, rows
 * v_rld apart) on m collocation points: one AIC column.
 * vlm_backend_cpu_kernels.ispc:106-135 (float), :419-448 (double). */
void FN(orc_influence_)(int64_t m, T* lhs, const T* collocs, int64_t collocs_ld,
                        const T* v, int64_t v_ld, int64_t v_rld,
                        const T* normals, int64_t normals_ld, T sigma) {
    V3 v0 = FN(v3)(v[0 * v_ld], v[1 * v_ld], v[2 * v_ld]);
    V3 v1 = FN(v3)(v[0 * v_ld + 1], v[1 * v_ld + 1], v[2 * v_ld + 1]);
    V3 v2 = FN(v3)(v[0 * v_ld + v_rld + 1], v[1 * v_ld + v_rld + 1], v[2 * v_ld + v_rld + 1]);
    V3 v3 = FN(v3)(v[0 * v_ld + v_rld], v[1 * v_ld + v_rld], v[2 * v_ld + v_rld]);
    for (int64_t i = 0; i < m; i++) {
        V3 c = FN(v3)(collocs[0 * collocs_ld + i], collocs[1 * collocs_ld + i], collocs[2 * collocs_ld + i]);
        V3 n = FN(v3)(normals[0 * normals_ld + i], normals[1 * normals_ld + i], normals[2 * normals_ld + i]);
        V3 inf = FN(ring_velocity)(c, v0, v1, v2, v3, sigma);
        lhs[i] += FN(vdot)(inf, n);
    }
}

/* Induced velocity of the last `iteration` wake ring rows of one wake on one
 * collocation point, projected on its normal and subtracted from its RHS.
 * The float variant keeps at most 5000 rows.
 * vlm_backend_cpu_kernels.ispc:150-196 (float), :463-502 (double). */
void FN(orc_wake_influence_)(const T* colloc, int64_t colloc_ld, const T* normals, int64_t normals_ld,
                             const T* v, int64_t v_ld, int64_t v_m, int64_t v_n,
                             const T* gamma, T* rhs, T sigma, int32_t iteration) {
    V3 c = FN(v3)(colloc[0 * colloc_ld], colloc[1 * colloc_ld], colloc[2 * colloc_ld]);
    V3 vel = FN(v3)(0, 0, 0);
    int64_t end = v_m - 1;
    if (ORC_WAKE_WINDOW > 0 && iteration > ORC_WAKE_WINDOW) end = v_m - 1 - iteration + ORC_WAKE_WINDOW;
    for (int64_t i = v_m - iteration - 1; i < end; i++) {
        for (int64_t j = 0; j < v_n - 1; j++) {
            const int64_t i0 = (i + 0) * v_n + j, i1 = (i + 0) * v_n + j + 1;
            const int64_t i2 = (i + 1) * v_n + j + 1, i3 = (i + 1) * v_n + j;
            V3 a = FN(v3)(v[0 * v_ld + i0], v[1 * v_ld + i0], v[2 * v_ld + i0]);
            V3 b = FN(v3)(v[0 * v_ld + i1], v[1 * v_ld + i1], v[2 * v_ld + i1]);
            V3 d = FN(v3)(v[0 * v_ld + i2], v[1 * v_ld + i2], v[2 * v_ld + i2]);
            V3 e = FN(v3)(v[0 * v_ld + i3], v[1 * v_ld + i3], v[2 * v_ld + i3]);
            V3 ind = FN(ring_velocity)(c, a, b, d, e, sigma);
            vel = FN(vadd)(vel, FN(vscale)(gamma[i * (v_n - 1) + j], ind));
        }
    }
    V3 n = FN(v3)(normals[0 * normals_ld], normals[1 * normals_ld], normals[2 * normals_ld]);
    *rhs -= FN(vdot)(vel, n);
}

/* Velocity of the rings of one lattice (vertex rows [row0, row1], spanwise
 * n vertices) at point p, each ring weighted by its gamma (row-major over
 * ring rows, n-1 rings per row, ring row r at gamma[r*(n-1)]). */
static V3 FN(lattice_velocity)(V3 p, const T* v, int64_t v_ld, int64_t n, int64_t r0, int64_t r1,
                               const T* gamma, T sigma) {
    V3 vel = FN(v3)(0, 0, 0);
    for (int64_t i = r0; i < r1; i++) {
        for (int64_t j = 0; j < n - 1; j++) {
            const int64_t i0 = (i + 0) * n + j, i1 = (i + 0) * n + j + 1;
            const int64_t i2 = (i + 1) * n + j + 1, i3 = (i + 1) * n + j;
            V3 a = FN(v3)(v[0 * v_ld + i0], v[1 * v_ld + i0], v[2 * v_ld + i0]);
            V3 b = FN(v3)(v[0 * v_ld + i1], v[1 * v_ld + i1], v[2 * v_ld + i1]);
            V3 d = FN(v3)(v[0 * v_ld + i2], v[1 * v_ld + i2], v[2 * v_ld + i2]);
            V3 e = FN(v3)(v[0 * v_ld + i3], v[1 * v_ld + i3], v[2 * v_ld + i3]);
            V3 ind = FN(ring_velocity)(p, a, b, d, e, sigma);
            vel = FN(vadd)(vel, FN(vscale)(gamma[i * (n - 1) + j], ind));
        }
    }
    return vel;
}

/* Free-wake roll-up of one wake vertex: position + dt * (velocity induced by
 * all wing rings and the last `iteration` wake ring rows).  The reference
 * kernel exists but its caller is commented out.
 * vlm_backend_cpu_kernels.ispc:215-271. */
void FN(orc_rollup_)(const T* v_wake, int64_t v_wake_ld, int64_t v_wake_m, int64_t v_wake_n, int64_t v_wake_idx,
                     const T* v_wing, int64_t v_wing_ld, int64_t v_wing_m, int64_t v_wing_n,
                     T* rollup, int64_t rollup_ld, const T* gamma_wing, const T* gamma_wake,
                     T sigma, T dt, int32_t iteration) {
    V3 p = FN(v3)(v_wake[0 * v_wake_ld + v_wake_idx], v_wake[1 * v_wake_ld + v_wake_idx], v_wake[2 * v_wake_ld + v_wake_idx]);
    V3 a = FN(lattice_velocity)(p, v_wing, v_wing_ld, v_wing_n, 0, v_wing_m - 1, gamma_wing, sigma);
    V3 b = FN(lattice_velocity)(p, v_wake, v_wake_ld, v_wake_n, v_wake_m - iteration - 1, v_wake_m - 1, gamma_wake, sigma);
    V3 vel = FN(vadd)(a, b);
    rollup[0 * rollup_ld + v_wake_idx] = p.x + vel.x * dt;
    rollup[1 * rollup_ld + v_wake_idx] = p.y + vel.y * dt;
    rollup[2 * rollup_ld + v_wake_idx] = p.z + vel.z * dt;
}

/* Trefftz-plane induced drag sum over the first wake ring row (trailing
 * segments only).  The caller divides by |V|^2 S.
 * vlm_backend_cpu_kernels.ispc:273-323; normalisation from the commented
 * caller vlm_backend_cpu.cpp:364-369. */
T FN(orc_trefftz_cd_)(const T* v, int64_t v_ld, int64_t v_m, int64_t v_n, const T* gamma, T sigma) {
    T cd = 0;
    const int64_t i = v_m - 2;
    for (int64_t j = 0; j < v_n - 1; j++) {
        const int64_t i0 = (i + 0) * v_n + j, i1 = (i + 0) * v_n + j + 1;
        const int64_t i2 = (i + 1) * v_n + j + 1, i3 = (i + 1) * v_n + j;
        V3 a = FN(v3)(v[0 * v_ld + i0], v[1 * v_ld + i0], v[2 * v_ld + i0]);
        V3 b = FN(v3)(v[0 * v_ld + i1], v[1 * v_ld + i1], v[2 * v_ld + i1]);
        V3 d = FN(v3)(v[0 * v_ld + i2], v[1 * v_ld + i2], v[2 * v_ld + i2]);
        V3 e = FN(v3)(v[0 * v_ld + i3], v[1 * v_ld + i3], v[2 * v_ld + i3]);
        V3 c = FN(vscale)((T)0.25, FN(vadd)(FN(vadd)(FN(vadd)(a, b), d), e));
        V3 n = FN(vnormalize)(FN(vcross)(FN(vsub)(e, b), FN(vsub)(d, a)));
        V3 inf = FN(v3)(0, 0, 0);
        for (int64_t jj = 0; jj < v_n - 1; jj++) {
            const int64_t k0 = (i + 0) * v_n + jj, k1 = (i + 0) * v_n + jj + 1;
            const int64_t k2 = (i + 1) * v_n + jj + 1, k3 = (i + 1) * v_n + jj;
            V3 w0 = FN(v3)(v[0 * v_ld + k0], v[1 * v_ld + k0], v[2 * v_ld + k0]);
            V3 w1 = FN(v3)(v[0 * v_ld + k1], v[1 * v_ld + k1], v[2 * v_ld + k1]);
            V3 w2 = FN(v3)(v[0 * v_ld + k2], v[1 * v_ld + k2], v[2 * v_ld + k2]);
            V3 w3 = FN(v3)(v[0 * v_ld + k3], v[1 * v_ld + k3], v[2 * v_ld + k3]);
            V3 inf2 = FN(v3)(0, 0, 0);
            FN(symmetry)(&inf2, c, w1, w2, sigma);
            FN(symmetry)(&inf2, c, w3, w0, sigma);
            inf = FN(vadd)(inf, FN(vscale)(gamma[i * (v_n - 1) + jj], inf2));
        }
        T iv = FN(vdot)(inf, n);
        cd -= gamma[i * (v_n - 1) + j] * iv * FN(vlen)(FN(vsub)(b, a));
    }
    return cd;
}

/* ---------------------------------------------------------------------------
 * Backend operators.  Multi-surface arguments are host arrays with one
 * pointer per surface, mirroring the reference's MultiTensorView.  Per
 * surface m: wing vertices (ns+1, nc+1, 4), panel fields (ns, nc, 3) or
 * (ns, nc), wake vertices (ns+1, nwv, 4), wake gamma (ns, nwv-1); all
 * column-major (first index fastest) and contiguous.
 * ------------------------------------------------------------------------- */

/* AIC assembly with the Kutta wake coupling of `iteration` wake rows.
 * vlm_backend_cpu.cpp:84-148 (float), vlm_backend_cpud.cpp:27-91 (double). */
void FN(orc_lhs_assemble_)(T* lhs, int64_t ld, int32_t nsurf, const int64_t* ns, const int64_t* nc,
                           const int64_t* nwv, T* const* colloc, T* const* normals,
                           T* const* verts_wing, T* const* verts_wake, int32_t iteration, T sigma) {
    int64_t offset_j = 0;
    for (int32_t mj = 0; mj < nsurf; mj++) {
        int64_t offset_i = 0;
        const int64_t nsj = ns[mj], ncj = nc[mj];
        const int64_t vw_ld = (nsj + 1) * (ncj + 1);
        for (int32_t mi = 0; mi < nsurf; mi++) {
            const int64_t npi = ns[mi] * nc[mi];
            T* sec = lhs + offset_i + offset_j * ld;
            /* wing pass + last row: one column per wing ring */
            #pragma omp parallel for schedule(static)
            for (int64_t l = 0; l < nsj * ncj; l++) {
                FN(orc_influence_)(npi, sec + l * ld, colloc[mi], npi, verts_wing[mj] + l + l / nsj,
                                   vw_ld, nsj + 1, normals[mi], npi, sigma);
            }
            /* wake pass, `iteration` times, into the trailing-edge columns */
            const int64_t end_wing = (ncj - 1) * nsj;
            const int64_t wk_ld = (nsj + 1) * nwv[mj];
            for (int32_t c = 0; c < iteration; c++) {
                #pragma omp parallel for schedule(static)
                for (int64_t j = 0; j < nsj; j++) {
                    const T* vwk = verts_wake[mj] + j + (nwv[mj] - 2 - c) * (nsj + 1);
                    FN(orc_influence_)(npi, sec + (j + end_wing) * ld, colloc[mi], npi, vwk,
                                       wk_ld, nsj + 1, normals[mi], npi, sigma);
                }
            }
            offset_i += npi;
        }
        offset_j += nsj * ncj;
    }
}

/* rhs[p] += -(V_p . n_p).  vlm_backend_cpu.cpp:156-179. */
void FN(orc_rhs_assemble_velocities_)(T* rhs, int32_t nsurf, const int64_t* ns, const int64_t* nc,
                                      T* const* normals, T* const* velocities) {
    int64_t offset = 0;
    for (int32_t m = 0; m < nsurf; m++) {
        const int64_t np = ns[m] * nc[m];
        const T* n = normals[m];
        const T* v = velocities[m];
        for (int64_t p = 0; p < np; p++) {
            rhs[offset + p] += -(v[p] * n[p] + v[np + p] * n[np + p] + v[2 * np + p] * n[2 * np + p]);
        }
        offset += np;
    }
}

/* vlm_backend_cpu.cpp:181-224 (float), vlm_backend_cpud.cpp:124-167. */
void FN(orc_rhs_assemble_wake_influence_)(T* rhs, int32_t nsurf, const int64_t* ns, const int64_t* nc,
                                          const int64_t* nwv, T* const* gamma_wake, T* const* colloc,
                                          T* const* normals, T* const* verts_wake,
                                          const int32_t* lifting, int32_t iteration, T sigma) {
    int64_t offset = 0;
    for (int32_t mi = 0; mi < nsurf; mi++) {
        const int64_t np = ns[mi] * nc[mi];
        #pragma omp parallel for schedule(dynamic, 16)
        for (int64_t idx = 0; idx < np; idx++) {
            for (int32_t mj = 0; mj < nsurf; mj++) {
                if (!lifting[mj]) continue;
                FN(orc_wake_influence_)(colloc[mi] + idx, np, normals[mi] + idx, np, verts_wake[mj],
                                        (ns[mj] + 1) * nwv[mj], nwv[mj], ns[mj] + 1, gamma_wake[mj],
                                        rhs + offset + idx, sigma, iteration);
            }
        }
        offset += np;
    }
}

/* Free-wake roll-up of every surface's wake: vertex rows [nwv-iteration, nwv)
 * move with the velocity of all wing rings and all lifting wakes.  Restates
 * kernel_rollup (vlm_backend_cpu_kernels.ispc:215-271) summed over surfaces;
 * the row range follows the commented caller vlm_backend_cpu.cpp:239-240.
 * Writes the moved positions to `rollup` (same layout as verts_wake), then
 * copies them back, as the commented caller does (:263-267). */
void FN(orc_wake_rollup_)(int32_t nsurf, const int64_t* ns, const int64_t* nc, const int64_t* nwv,
                          T* const* verts_wake, T* const* verts_wing, T* const* gamma_wing,
                          T* const* gamma_wake, T* const* rollup, const int32_t* lifting,
                          T sigma, T dt, int32_t iteration) {
    for (int32_t m = 0; m < nsurf; m++) {
        const int64_t n = ns[m] + 1, wk_ld = n * nwv[m];
        const int64_t begin = (nwv[m] - iteration) * n, end = nwv[m] * n;
        #pragma omp parallel for schedule(dynamic, 8)
        for (int64_t vi = begin; vi < end; vi++) {
            const T* vw = verts_wake[m];
            V3 p = FN(v3)(vw[vi], vw[wk_ld + vi], vw[2 * wk_ld + vi]);
            V3 vel = FN(v3)(0, 0, 0);
            for (int32_t k = 0; k < nsurf; k++) {
                const int64_t nk = ns[k] + 1;
                vel = FN(vadd)(vel, FN(lattice_velocity)(p, verts_wing[k], nk * (nc[k] + 1), nk, 0, nc[k],
                                                         gamma_wing[k], sigma));
                if (!lifting[k]) continue;
                vel = FN(vadd)(vel, FN(lattice_velocity)(p, verts_wake[k], nk * nwv[k], nk,
                                                         nwv[k] - iteration - 1, nwv[k] - 1,
                                                         gamma_wake[k], sigma));
            }
            rollup[m][vi] = p.x + vel.x * dt;
            rollup[m][wk_ld + vi] = p.y + vel.y * dt;
            rollup[m][2 * wk_ld + vi] = p.z + vel.z * dt;
        }
    }
    for (int32_t m = 0; m < nsurf; m++) {
        const int64_t n = ns[m] + 1, wk_ld = n * nwv[m];
        const int64_t begin = (nwv[m] - iteration) * n, end = nwv[m] * n;
        for (int k = 0; k < 3; k++)
            for (int64_t vi = begin; vi < end; vi++) verts_wake[m][k * wk_ld + vi] = rollup[m][k * wk_ld + vi];
    }
}

/* vlm_backend_cpu.cpp:276-297 (rho hard-coded to 1 at :282). */
void FN(orc_forces_steady_)(int64_t ns, int64_t nc, const T* verts_wing, const T* gamma_delta,
                            const T* velocities, T* forces) {
    const T rho = 1;
    const int64_t vld = (ns + 1) * (nc + 1), np = ns * nc;
    for (int64_t j = 0; j < nc; j++) {
        for (int64_t i = 0; i < ns; i++) {
            const int64_t p = i + j * ns, a = i + j * (ns + 1), b = a + 1;
            V3 V = FN(v3)(velocities[p], velocities[np + p], velocities[2 * np + p]);
            V3 v0 = FN(v3)(verts_wing[a], verts_wing[vld + a], verts_wing[2 * vld + a]);
            V3 v1 = FN(v3)(verts_wing[b], verts_wing[vld + b], verts_wing[2 * vld + b]);
            V3 f = FN(vscale)(rho * gamma_delta[p], FN(vcross)(V, FN(vsub)(v1, v0)));
            forces[p] = f.x; forces[np + p] = f.y; forces[2 * np + p] = f.z;
        }
    }
}

/* vlm_backend_cpu.cpp:299-321. */
void FN(orc_forces_unsteady_)(int64_t ns, int64_t nc, const T* verts_wing, const T* gamma_delta,
                              const T* dgamma_dt, const T* velocities, const T* areas,
                              const T* normals, T* forces) {
    FN(orc_forces_steady_)(ns, nc, verts_wing, gamma_delta, velocities, forces);
    const T rho = 1;
    const int64_t np = ns * nc;
    for (int64_t p = 0; p < np; p++) {
        V3 n = FN(v3)(normals[p], normals[np + p], normals[2 * np + p]);
        V3 f = FN(vscale)(rho * dgamma_dt[p] * areas[p], n);
        forces[p] += f.x; forces[np + p] += f.y; forces[2 * np + p] += f.z;
    }
}

/* vlm_backend_cpu.cpp:323-338. */
T FN(orc_coeff_cl_)(int64_t ns, int64_t nc, const T* forces, const T* lift_axis, const T* freestream,
                    T rho, T area) {
    const int64_t np = ns * nc;
    V3 la = FN(v3)(lift_axis[0], lift_axis[1], lift_axis[2]);
    V3 fs = FN(v3)(freestream[0], freestream[1], freestream[2]);
    T cl = 0;
    for (int64_t p = 0; p < np; p++) cl += FN(vdot)(FN(v3)(forces[p], forces[np + p], forces[2 * np + p]), la);
    return cl / ((T)0.5 * rho * FN(vlen2)(fs) * area);
}

/* vlm_backend_cpu.cpp:340-362.  out = cm (3 values). */
void FN(orc_coeff_cm_)(int64_t ns, int64_t nc, const T* forces, const T* verts_wing, const T* ref_pt,
                       const T* freestream, T rho, T area, T mac, T* out) {
    const int64_t np = ns * nc, vld = (ns + 1) * (nc + 1);
    V3 r = FN(v3)(ref_pt[0], ref_pt[1], ref_pt[2]);
    V3 fs = FN(v3)(freestream[0], freestream[1], freestream[2]);
    V3 cm = FN(v3)(0, 0, 0);
    for (int64_t j = 0; j < nc; j++) {
        for (int64_t i = 0; i < ns; i++) {
            const int64_t p = i + j * ns, a = i + j * (ns + 1), b = a + 1;
            V3 v0 = FN(v3)(verts_wing[a], verts_wing[vld + a], verts_wing[2 * vld + a]);
            V3 v1 = FN(v3)(verts_wing[b], verts_wing[vld + b], verts_wing[2 * vld + b]);
            V3 f = FN(v3)(forces[p], forces[np + p], forces[2 * np + p]);
            V3 lever = FN(vsub)(FN(vscale)((T)0.5, FN(vadd)(v0, v1)), r);
            cm = FN(vadd)(cm, FN(vcross)(lever, f));
        }
    }
    T d = (T)0.5 * rho * FN(vlen2)(fs) * area * mac;
    out[0] = cm.x / d; out[1] = cm.y / d; out[2] = cm.z / d;
}

/* Normals, areas and collocation points (with the high-AoA factor).
 * vlm_backend_cpu.cpp:391-433, vlm_backend_cpud.cpp:258-300. */
void FN(orc_mesh_metrics_)(T alpha_rad, int64_t ns, int64_t nc, const T* verts_wing, T* colloc,
                           T* normals, T* areas) {
    const int64_t vld = (ns + 1) * (nc + 1), np = ns * nc;
    const T factor = (alpha_rad < (T)ORC_EPS_F) ? (T)0.5
                   : (T)0.5 * (alpha_rad / (SIN(alpha_rad) + (T)ORC_EPS_F));
    for (int64_t j = 0; j < nc; j++) {
        for (int64_t i = 0; i < ns; i++) {
            const int64_t p = i + j * ns;
            const int64_t a = i + j * (ns + 1), b = a + 1, c = b + (ns + 1), d = a + (ns + 1);
            V3 v0 = FN(v3)(verts_wing[a], verts_wing[vld + a], verts_wing[2 * vld + a]);
            V3 v1 = FN(v3)(verts_wing[b], verts_wing[vld + b], verts_wing[2 * vld + b]);
            V3 v2 = FN(v3)(verts_wing[c], verts_wing[vld + c], verts_wing[2 * vld + c]);
            V3 v3 = FN(v3)(verts_wing[d], verts_wing[vld + d], verts_wing[2 * vld + d]);
            V3 n = FN(vnormalize)(FN(vcross)(FN(vsub)(v3, v1), FN(vsub)(v2, v0)));
            normals[p] = n.x; normals[np + p] = n.y; normals[2 * np + p] = n.z;
            V3 vf = FN(vsub)(v3, v0), vb = FN(vsub)(v2, v0), ve = FN(vsub)(v1, v0);
            areas[p] = (T)0.5 * (FN(vlen)(FN(vcross)(vf, vb)) + FN(vlen)(FN(vcross)(vb, ve)));
            V3 chord = FN(vscale)((T)0.5, FN(vsub)(FN(vsub)(FN(vadd)(v2, v3), v0), v1));
            V3 cp = FN(vadd)(FN(vscale)((T)0.5, FN(vadd)(v0, v1)), FN(vscale)(factor, chord));
            colloc[p] = cp.x; colloc[np + p] = cp.y; colloc[2 * np + p] = cp.z;
        }
    }
}

/* vlm_backend_cpu.cpp:506-523. */
T FN(orc_sum_)(int64_t n, const T* x) {
    T s = 0;
    for (int64_t i = 0; i < n; i++) s += x[i];
    return s;
}

/* Mean aerodynamic chord by the trapezoidal rule over spanwise stations.
 * vlm_backend_cpu.cpp:443-468. */
T FN(orc_mesh_mac_)(int64_t ns, int64_t nc, const T* verts_wing, const T* areas) {
    const int64_t vld = (ns + 1) * (nc + 1), last = nc * (ns + 1);
    T mac = 0;
    for (int64_t i = 0; i < ns; i++) {
        const T dx0 = verts_wing[i] - verts_wing[last + i];
        const T dy0 = verts_wing[vld + i] - verts_wing[vld + last + i];
        const T dz0 = verts_wing[2 * vld + i] - verts_wing[2 * vld + last + i];
        const T dx1 = verts_wing[i + 1] - verts_wing[last + i + 1];
        const T dy1 = verts_wing[vld + i + 1] - verts_wing[vld + last + i + 1];
        const T dz1 = verts_wing[2 * vld + i + 1] - verts_wing[2 * vld + last + i + 1];
        const T c0 = SQRT(dx0 * dx0 + dy0 * dy0 + dz0 * dz0);
        const T c1 = SQRT(dx1 * dx1 + dy1 * dy1 + dz1 * dz1);
        const T dx3 = verts_wing[i + 1] - verts_wing[i];
        const T dy3 = verts_wing[vld + i + 1] - verts_wing[vld + i];
        const T dz3 = verts_wing[2 * vld + i + 1] - verts_wing[2 * vld + i];
        const T width = SQRT(dx3 * dx3 + dy3 * dy3 + dz3 * dz3);
        mac += (T)0.5 * (c0 * c0 + c1 * c1) * width;
    }
    return mac / FN(orc_sum_)(ns * nc, areas);
}

/* Wake gamma of the last `iteration` columns from the trailing-edge Fourier
 * coefficients (scaled orthonormal basis).  gamma_wake (ns, ncols),
 * coeffs (ns, 2H+1).  vlm_backend_cpu.cpp:470-503, vlm_backend_cpud.cpp:337-370. */
void FN(orc_gamma_wake_from_coeffs_)(int64_t ns, int64_t ncols, T* gamma_wake, const T* coeffs,
                                     int32_t harmonics, T tn, T omega, T dt, int64_t iteration) {
    const int32_t unknowns = 2 * harmonics + 1;
    const T s0 = (T)1 / SQRT((T)unknowns);
    const T s2 = SQRT((T)2 / (T)unknowns);
    const int64_t start = ncols - iteration;
    for (int64_t j = start; j < ncols; j++) {
        for (int64_t i = 0; i < ns; i++) {
            T g = coeffs[i] * s0;
            for (int64_t h = 0; h < harmonics; h++) {
                const T wk = omega * (T)(h + 1);
                g += coeffs[i + (2 * h + 1) * ns] * COS(wk * (tn - (T)(j - start + 1) * dt)) * s2;
                g += coeffs[i + (2 * h + 2) * ns] * SIN(wk * (tn - (T)(j - start + 1) * dt)) * s2;
            }
            gamma_wake[i + j * ns] = g;
        }
    }
}

/* verts = verts_init . T^T for one surface (T column-major 4x4).
 * vlm_backend.cpp:50-69 (a BLAS gemm there). */
void FN(orc_displace_wing_)(int64_t nv, const T* transform, T* verts, const T* verts_init) {
    for (int64_t r = 0; r < nv; r++) {
        T in[4] = {verts_init[r], verts_init[nv + r], verts_init[2 * nv + r], verts_init[3 * nv + r]};
        for (int c = 0; c < 4; c++) {
            T acc = 0;
            for (int k = 0; k < 4; k++) acc += in[k] * transform[c + 4 * k];
            verts[c * nv + r] = acc;
        }
    }
}
