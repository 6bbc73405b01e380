/*
 * OpenMP C restatement of the reference's FDK and forward-projection kernels --
 * TEST INFRASTRUCTURE: the timed CPU baseline ("port") of bench.py and, built in
 * float64, the FP64 checker of results at benchmark sizes.
 *
 * It follows the reference's Taichi kernels loop for loop, parallel over the same
 * outer loops Taichi parallelises:
 *   cpu_weight     run_mgfbp.py:956-970   (flat/curved cosine weighting; full scans)
 *   cpu_filter     run_mgfbp.py:1030-1046 (direct O(nu^2) row convolution)
 *   cpu_fdk_bp     run_mgfbp.py:1062-1187 (axial view mode; per voxel, per view,
 *                                          global accumulate, break-to-zero rule)
 *   cpu_fp         run_mgfpj_v3.py:255-365 (one ray per (u, v, view), every step)
 * The arithmetic type is REAL: float (Taichi's default precision; the baseline) or,
 * compiled with -DREAL=double, float64 end to end (the checker; it reproduces the
 * float64 NumPy restatement in oracle/ to rounding, which tests/test_cpu_ref.py
 * checks).  Geometry comes in as int64 and double arrays (indices below) and is
 * converted to REAL once, as Taichi converts its Python-float fields.
 * Views can be restricted to [v0, v1), slices to [z0, z1) and the filtered
 * sinogram to a block of detector rows, so that bench.py can time a bounded sample
 * and check a slab of a benchmark-size result.
 * Nothing in the product links or calls this file.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL float
#endif
#define R(x) ((REAL)(x))

/* integer geometry */
enum { GI_NU, GI_NV, GI_VIEWS, GI_NX, GI_NZ, GI_CONE, GI_CURVED, GI_SHORT, GI_STEPS, GI_N };
/* floating-point geometry */
enum {
    GD_DU, GD_DV, GD_U0, GD_USTEP, GD_V0, GD_VSTEP, GD_PX, GD_PZ, GD_CX, GD_CY, GD_CZ, GD_SID, GD_SDD, GD_ROT,
    GD_SCAN, GD_STEP, GD_N
};

static inline REAL r_cos(REAL x) { return sizeof(REAL) == 8 ? (REAL)cos((double)x) : (REAL)cosf((float)x); }
static inline REAL r_sin(REAL x) { return sizeof(REAL) == 8 ? (REAL)sin((double)x) : (REAL)sinf((float)x); }
static inline REAL r_sqrt(REAL x) { return sizeof(REAL) == 8 ? (REAL)sqrt((double)x) : (REAL)sqrtf((float)x); }
static inline REAL r_floor(REAL x) { return sizeof(REAL) == 8 ? (REAL)floor((double)x) : (REAL)floorf((float)x); }
static inline REAL r_fabs(REAL x) { return sizeof(REAL) == 8 ? (REAL)fabs((double)x) : (REAL)fabsf((float)x); }
static inline REAL r_atan2(REAL y, REAL x) {
    return sizeof(REAL) == 8 ? (REAL)atan2((double)y, (double)x) : (REAL)atan2f((float)y, (float)x);
}

#define PI_REF R(3.1415926536)

int cpu_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int cpu_real_bytes(void) { return (int)sizeof(REAL); }

/* sgm [nv][views][nu] weighted in place (rows as given by nv, v0, v_step) */
void cpu_weight(const int64_t* gi, const double* gd, REAL* sgm) {
    const int nu = (int)gi[GI_NU], nv = (int)gi[GI_NV], views = (int)gi[GI_VIEWS];
    const REAL sdd = R(gd[GD_SDD]), u0 = R(gd[GD_U0]), us = R(gd[GD_USTEP]), v0 = R(gd[GD_V0]), vs = R(gd[GD_VSTEP]);
    const int curved = gi[GI_CURVED] != 0;
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < views; ++i)
        for (int j = 0; j < nu; ++j) {
            REAL u = u0 + j * us;
            for (int s = 0; s < nv; ++s) {
                REAL v = v0 + s * vs;
                REAL* p = sgm + ((int64_t)s * views + i) * nu + j;
                if (curved) *p = *p * sdd * r_cos(-u / sdd) * sdd / r_sqrt(sdd * sdd + v * v);
                else *p = (*p * sdd * sdd) / r_sqrt(sdd * sdd + u * u + v * v);
            }
        }
}

/* rows [r0, r1) of x [rows][nu] -> y [rows][nu]; y = du * sum_m x[m] h[k-m+nu-1] */
void cpu_filter(const int64_t* gi, const double* gd, const REAL* x, const REAL* h, REAL* y, int64_t r0, int64_t r1) {
    const int nu = (int)gi[GI_NU];
    const REAL du = R(gd[GD_DU]);
#pragma omp parallel for schedule(static)
    for (int64_t r = r0; r < r1; ++r) {
        const REAL* xr = x + r * nu;
        for (int k = 0; k < nu; ++k) {
            REAL acc = R(0);
            for (int m = 0; m < nu; ++m) acc += xr[m] * h[k + (nu - 1) - m];
            y[r * nu + k] = acc * du;
        }
    }
}

/* vol [z1-z0][nx][nx] (slices [z0, z1) of the volume) += contributions of views
 * [v0, v1); the caller zeroes vol; alive flags (same shape) start at 1 and record the
 * break-to-zero rule.  F holds detector rows [f_row0, f_row0 + f_rows) of the filtered
 * sinogram [nv][views][nu].  Axial view mode.  Returns the number of voxel-view
 * updates that needed a row outside that block (0 when the block covers the slab). */
int64_t cpu_fdk_bp(const int64_t* gi, const double* gd, const REAL* angles, const REAL* F, int f_row0, int f_rows,
                   REAL* vol, uint8_t* alive, int z0, int z1, int v0, int v1) {
    const int nx = (int)gi[GI_NX], nz = (int)gi[GI_NZ], nu = (int)gi[GI_NU], nv = (int)gi[GI_NV];
    const int views = (int)gi[GI_VIEWS];
    const int cone = gi[GI_CONE] != 0, curved = gi[GI_CURVED] != 0;
    const REAL sid = R(gd[GD_SID]), sdd = R(gd[GD_SDD]), rot = R(gd[GD_ROT]), px = R(gd[GD_PX]), pz = R(gd[GD_PZ]);
    const REAL cx = R(gd[GD_CX]), cy = R(gd[GD_CY]), cz = R(gd[GD_CZ]);
    const REAL u0 = R(gd[GD_U0]), us = R(gd[GD_USTEP]), vv0 = R(gd[GD_V0]), dv = R(gd[GD_DV]);
    const REAL tsa = r_fabs(R(gd[GD_SCAN]));
    REAL num_rounds = r_floor(tsa / (PI_REF * 2));
    REAL div = R(1) / (num_rounds * R(2));
    if (gi[GI_SHORT]) {
        REAL remain = tsa - num_rounds * 2 * PI_REF;
        div = R(1);
        if (tsa < 2 * PI_REF) div = R(1);
        else if (remain < PI_REF) div = R(1) / (num_rounds * R(2));
        else if (PI_REF < remain && remain < 2 * PI_REF) div = R(1) / (num_rounds * R(2) + R(1));
    }
    const REAL vsgn = gd[GD_VSTEP] > 0 ? R(1) : R(-1);
    /* per-view cos, sin and angular step: the values the reference evaluates per voxel
     * and view, evaluated once per view */
    REAL* tab = (REAL*)malloc(sizeof(REAL) * 3 * (size_t)(views > 0 ? views : 1));
    if (!tab) return -1;
    for (int j = 0; j < views; ++j) {
        tab[3 * j] = r_cos(angles[j] - rot);
        tab[3 * j + 1] = r_sin(angles[j] - rot);
        tab[3 * j + 2] = (j == views - 1) ? r_fabs(angles[views - 1] - angles[0]) / (views - 1)
                                          : r_fabs(angles[j + 1] - angles[j]);
    }
    int64_t misses = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 4) reduction(+ : misses)
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < nx; ++iy)
            for (int iz = z0; iz < z1; ++iz) {
                int64_t vi = ((int64_t)(iz - z0) * nx + iy) * nx + ix;
                if (!alive[vi]) continue;
                REAL xa = px * (ix - (nx - 1) / R(2)) + cx;
                REAL ya = -px * (iy - (nx - 1) / R(2)) + cy;
                REAL z = (iz - (nz - 1) / R(2)) * pz + cz;
                REAL x = xa * r_cos(rot) + ya * r_sin(rot);
                REAL y = -xa * r_sin(rot) + ya * r_cos(rot);
                REAL acc = vol[vi];
                for (int j = v0; j < v1; ++j) {
                    const REAL cb = tab[3 * j], sb = tab[3 * j + 1], dang = tab[3 * j + 2];
                    REAL L = sid - x * cb - y * sb;
                    REAL mag = sdd / L;
                    REAL t = -x * sb + y * cb;
                    REAL u = curved ? sdd * r_atan2(t, L) : mag * t;
                    REAL ui = (u - u0) / us;
                    if (ui < 0 || ui + 1 > nu - 1) {
                        acc = 0;
                        alive[vi] = 0;
                        break;
                    }
                    REAL uff = r_floor(ui);
                    int uf = (int)uff;
                    REAL ru = ui - uff;
                    REAL dw = curved ? R(1) / (L * L + t * t) : R(1) / (L * L);
                    if (cone) {
                        REAL vidx = (mag * z - vv0) / dv * vsgn;
                        REAL vff = r_floor(vidx);
                        int vf = (int)vff;
                        if (vf < 0 || vf + 1 > nv - 1) {
                            acc = 0;
                            alive[vi] = 0;
                            break;
                        }
                        if (vf < f_row0 || vf + 1 >= f_row0 + f_rows) {
                            ++misses;
                            continue;
                        }
                        REAL rv = vidx - vff;
                        const REAL* r0 = F + ((int64_t)(vf - f_row0) * views + j) * nu;
                        const REAL* r1 = F + ((int64_t)(vf + 1 - f_row0) * views + j) * nu;
                        REAL p0 = r0[uf] * (1 - ru) + r0[uf + 1] * ru;
                        REAL p1 = r1[uf] * (1 - ru) + r1[uf + 1] * ru;
                        acc += (sid * dw) * ((1 - rv) * p0 + rv * p1) * dang * div;
                    } else {
                        if (iz < f_row0 || iz >= f_row0 + f_rows) {
                            ++misses;
                            continue;
                        }
                        const REAL* r0 = F + ((int64_t)(iz - f_row0) * views + j) * nu;
                        acc += (sid * dw) * ((1 - ru) * r0[uf] + ru * r0[uf + 1]) * dang * div;
                    }
                }
                vol[vi] = acc;
            }
    free(tab);
    return misses;
}

/* out [nv][views][nu] for views [v0, v1) (flat detector, circular, no matrices). */
void cpu_fp(const int64_t* gi, const double* gd, const REAL* angles, const REAL* u_arr, const REAL* v_arr,
            const REAL* vol, REAL* out, int v0, int v1) {
    const int nx = (int)gi[GI_NX], nz = (int)gi[GI_NZ], nu = (int)gi[GI_NU], nv = (int)gi[GI_NV];
    const int views = (int)gi[GI_VIEWS];
    const int cone = gi[GI_CONE] != 0;
    const REAL sid = R(gd[GD_SID]), sdd = R(gd[GD_SDD]), px = R(gd[GD_PX]), pz = R(gd[GD_PZ]), step = R(gd[GD_STEP]);
    const REAL img_dimension = nx * px, image_dimension_z = nz * pz;
    const REAL l_min = sid - r_sqrt(2 * img_dimension * img_dimension + image_dimension_z * image_dimension_z) / R(2);
    const REAL vd = r_sqrt(2 * px * px + pz * pz);
    const REAL x0 = -(nx - R(1)) / R(2) * px + R(gd[GD_CX]);
    const REAL y0 = -(nx - R(1)) / R(2) * (-px) + R(gd[GD_CY]);
    const REAL z0 = -(nz - R(1)) / R(2) * pz + R(gd[GD_CZ]);
    const int K = (int)gi[GI_STEPS];
#pragma omp parallel for collapse(3) schedule(dynamic, 16)
    for (int j = v0; j < v1; ++j)
        for (int iv = 0; iv < nv; ++iv)
            for (int iu = 0; iu < nu; ++iu) {
                REAL dx = -(sdd - sid), dy = u_arr[iu], dz = v_arr[iv];
                REAL dist = r_sqrt((dx - sid) * (dx - sid) + dy * dy + dz * dz);
                REAL ux = (dx - sid) / dist, uy = dy / dist, uz = dz / dist;
                REAL cb = r_cos(angles[j]), sb = r_sin(angles[j]);
                REAL acc = R(0);
                for (int k = 0; k < K; ++k) {
                    REAL l = k * step * vd + l_min;
                    REAL x = sid + ux * l, y = uy * l, z = uz * l;
                    REAL xr = x * cb - y * sb, yr = y * cb + x * sb;
                    REAL xff = r_floor((xr - x0) / px), yff = r_floor((yr - y0) / (-px));
                    int xi = (int)xff, yi = (int)yff;
                    if (xi >= 0 && xi + 1 < nx && yi >= 0 && yi + 1 < nx) {
                        REAL xw = (xr - (xi * px + x0)) / px;
                        REAL yw = (yr - (yi * (-px) + y0)) / (-px);
                        int zi;
                        REAL zw = R(0);
                        if (cone) {
                            zi = (int)r_floor((z - z0) / pz);
                            if (!(zi >= 0 && zi + 1 < nz)) continue;
                            zw = (z - (zi * pz + z0)) / pz;
                        } else {
                            zi = iv;
                        }
                        const REAL* b = vol + ((int64_t)zi * nx + yi) * nx + xi;
                        REAL lo = (1 - xw) * (1 - yw) * b[0] + xw * (1 - yw) * b[1] + (1 - xw) * yw * b[nx] +
                                  xw * yw * b[nx + 1];
                        if (cone) {
                            const REAL* c = b + (int64_t)nx * nx;
                            REAL hi = (1 - xw) * (1 - yw) * c[0] + xw * (1 - yw) * c[1] + (1 - xw) * yw * c[nx] +
                                      xw * yw * c[nx + 1];
                            acc += ((1 - zw) * lo + zw * hi) * step * vd;
                        } else {
                            acc += lo * step * vd;
                        }
                    }
                }
                out[((int64_t)iv * views + j) * nu + iu] = acc;
            }
}

/* The IR driver's per-view voxel-driven "P^T" (run_mgfbp_iterative_recon_IRN_CGLS.py
 * :372-474, driven view by view as in :319-336): per voxel and view, the bilinear gather
 * times distance_factor * pixel size, distance_factor = |voxel - source| / max(|dx|,
 * |dy|) of the in-plane offsets; rows outside [0, nv-1) only skip the view; a u outside
 * [0, nu-1) in any view clears the voxel's flag (SetTruncatedRegionToZero :477-481 is
 * applied by the caller: vol *= flag).  Axial view mode, per-view image centre z
 * (cz_views).  vol and flag are slices [z0, z1); S holds detector rows [s_row0, s_row0 +
 * s_rows) of the sinogram [nv][views][nu].  Returns the number of updates that needed
 * a row outside that block. */
int64_t cpu_bp_unmatched(const int64_t* gi, const double* gd, const REAL* angles, const REAL* cz_views, const REAL* S,
                         int s_row0, int s_rows, REAL* vol, uint8_t* flag, int z0, int z1, int v0, int v1) {
    const int nx = (int)gi[GI_NX], nz = (int)gi[GI_NZ], nu = (int)gi[GI_NU], nv = (int)gi[GI_NV];
    const int views = (int)gi[GI_VIEWS];
    const int cone = gi[GI_CONE] != 0, curved = gi[GI_CURVED] != 0;
    const REAL sid = R(gd[GD_SID]), sdd = R(gd[GD_SDD]), rot = R(gd[GD_ROT]), px = R(gd[GD_PX]), pz = R(gd[GD_PZ]);
    const REAL cx = R(gd[GD_CX]), cy = R(gd[GD_CY]);
    const REAL u0 = R(gd[GD_U0]), us = R(gd[GD_USTEP]), vv0 = R(gd[GD_V0]), dv = R(gd[GD_DV]);
    const REAL vsgn = gd[GD_VSTEP] > 0 ? R(1) : R(-1);
    REAL* tab = (REAL*)malloc(sizeof(REAL) * 2 * (size_t)(views > 0 ? views : 1));
    if (!tab) return -1;
    for (int j = 0; j < views; ++j) {
        tab[2 * j] = r_cos(angles[j] - rot);
        tab[2 * j + 1] = r_sin(angles[j] - rot);
    }
    int64_t misses = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 4) reduction(+ : misses)
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < nx; ++iy) {
            const REAL xa = px * (ix - (nx - 1) / R(2)) + cx;
            const REAL ya = -px * (iy - (nx - 1) / R(2)) + cy;
            const REAL x = xa * r_cos(rot) + ya * r_sin(rot);
            const REAL y = -xa * r_sin(rot) + ya * r_cos(rot);
            for (int iz = z0; iz < z1; ++iz) {
                const int64_t vi = ((int64_t)(iz - z0) * nx + iy) * nx + ix;
                REAL acc = vol[vi];
                for (int j = v0; j < v1; ++j) {
                    const REAL z = (iz - (nz - 1) / R(2)) * pz + cz_views[j];
                    const REAL cb = tab[2 * j], sb = tab[2 * j + 1];
                    const REAL L = sid - x * cb - y * sb;
                    const REAL ax = r_fabs(x - sid * cb), ay = r_fabs(y - sid * sb);
                    const REAL dfac = r_sqrt((x - sid * cb) * (x - sid * cb) + (y - sid * sb) * (y - sid * sb) + z * z) /
                                      (ax > ay ? ax : ay);
                    const REAL mag = sdd / L;
                    const REAL t = -x * sb + y * cb;
                    const REAL u = curved ? sdd * r_atan2(t, L) : mag * t;
                    const REAL ui = (u - u0) / us;
                    if (ui < 0 || ui + 1 > nu - 1) {
                        flag[vi] = 0;
                        continue;
                    }
                    const REAL uff = r_floor(ui);
                    const int uf = (int)uff;
                    const REAL ru = ui - uff;
                    if (cone) {
                        const REAL vidx = (mag * z - vv0) / dv * vsgn;
                        const REAL vff = r_floor(vidx);
                        const int vf = (int)vff;
                        if (vf < 0 || vf + 1 > nv - 1) continue;
                        if (vf < s_row0 || vf + 1 >= s_row0 + s_rows) {
                            ++misses;
                            continue;
                        }
                        const REAL rv = vidx - vff;
                        const REAL* r0 = S + ((int64_t)(vf - s_row0) * views + j) * nu;
                        const REAL* r1 = S + ((int64_t)(vf + 1 - s_row0) * views + j) * nu;
                        const REAL p0 = r0[uf] * (1 - ru) + r0[uf + 1] * ru;
                        const REAL p1 = r1[uf] * (1 - ru) + r1[uf + 1] * ru;
                        acc += ((1 - rv) * p0 + rv * p1) * dfac * px;
                    } else {
                        if (iz < s_row0 || iz >= s_row0 + s_rows) {
                            ++misses;
                            continue;
                        }
                        const REAL* r0 = S + ((int64_t)(iz - s_row0) * views + j) * nu;
                        acc += ((1 - ru) * r0[uf] + ru * r0[uf + 1]) * dfac * px;
                    }
                }
                vol[vi] = acc;
            }
        }
    free(tab);
    return misses;
}
