/*
 * OpenMP C restatement of the reference's FDK and forward-projection kernels --
 * TEST INFRASTRUCTURE and the timed CPU baseline ("port") of bench.py.
 *
 * It follows the reference's Taichi kernels loop for loop, in float32 like Taichi's
 * default precision, parallel over the same outer loops Taichi parallelises:
 *   cpu_weight     run_mgfbp.py:956-970   (flat/curved cosine weight; full scans)
 *   cpu_filter     run_mgfbp.py:1030-1046 (direct O(nu^2) row convolution)
 *   cpu_fdk_bp     run_mgfbp.py:1062-1187 (axial view mode; per voxel, per view,
 *                                          global accumulate, break-to-zero rule)
 *   cpu_fp         run_mgfpj_v3.py:255-365 (one ray per (u, v, view), every step)
 * Views can be restricted to [v0, v1) so that bench.py can time a bounded sample.
 * Nothing in the product links or calls this file.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mandoct_gb300.h"

#define PI_REF 3.1415926536f

int cpu_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* sgm [nv][views][nu] weighted in place */
void cpu_weight(const mct_geom* g, float* sgm) {
    const int nu = g->nu, nv = g->nv, views = g->views;
    const float sdd = g->sdd;
    const int curved = (g->flags & MCT_CURVED) != 0;
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < views; ++i)
        for (int j = 0; j < nu; ++j) {
            float u = g->u0 + j * g->u_step;
            for (int s = 0; s < nv; ++s) {
                float v = g->v0 + s * g->v_step;
                float* p = sgm + ((int64_t)s * views + i) * nu + j;
                if (curved) *p = *p * sdd * cosf(-u / sdd) * sdd / sqrtf(sdd * sdd + v * v);
                else *p = (*p * sdd * sdd) / sqrtf(sdd * sdd + u * u + v * v);
            }
        }
}

/* rows [r0, r1) of x [rows][nu] -> y [rows][nu]; y = du * sum_m x[m] h[k-m+nu-1] */
void cpu_filter(const mct_geom* g, const float* x, const float* h, float* y, int64_t r0, int64_t r1) {
    const int nu = g->nu;
    const float du = g->du;
#pragma omp parallel for schedule(static)
    for (int64_t r = r0; r < r1; ++r) {
        const float* xr = x + r * nu;
        for (int k = 0; k < nu; ++k) {
            float acc = 0.0f;
            for (int m = 0; m < nu; ++m) acc += xr[m] * h[k + (nu - 1) - m];
            y[r * nu + k] = acc * du;
        }
    }
}

/* vol [nz][nx][nx] += contributions of views [v0, v1) (caller zeroes vol; alive
 * flags [nz*nx*nx] start at 1 and record the break-to-zero rule).  Axial only. */
void cpu_fdk_bp(const mct_geom* g, const float* angles, const float* F, float* vol, uint8_t* alive, int v0, int v1) {
    const int nx = g->nx, nz = g->nz, nu = g->nu, nv = g->nv, views = g->views;
    const int cone = (g->flags & MCT_CONE) != 0, curved = (g->flags & MCT_CURVED) != 0;
    const float sid = g->sid, sdd = g->sdd, rot = g->img_rot;
    const float tsa = fabsf(g->total_scan_angle);
    float num_rounds = floorf(tsa / (PI_REF * 2));
    float div = 1.0f / (num_rounds * 2.0f);
    if (g->flags & MCT_SHORT_SCAN) {
        float remain = tsa - num_rounds * 2 * PI_REF;
        div = 1.0f;
        if (tsa < 2 * PI_REF) div = 1.0f;
        else if (remain < PI_REF) div = 1.0f / (num_rounds * 2.0f);
        else if (PI_REF < remain && remain < 2 * PI_REF) div = 1.0f / (num_rounds * 2.0f + 1.0f);
    }
    const float vsgn = g->v_step > 0 ? 1.0f : -1.0f;
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < nx; ++iy)
            for (int iz = 0; iz < nz; ++iz) {
                int64_t vi = ((int64_t)iz * nx + iy) * nx + ix;
                if (!alive[vi]) continue;
                float xa = g->px * (ix - (nx - 1) / 2.0f) + g->cx;
                float ya = -g->px * (iy - (nx - 1) / 2.0f) + g->cy;
                float z = (iz - (nz - 1) / 2.0f) * g->pz + g->cz;
                float x = xa * cosf(rot) + ya * sinf(rot);
                float y = -xa * sinf(rot) + ya * cosf(rot);
                float acc = vol[vi];
                for (int j = v0; j < v1; ++j) {
                    float dang = (j == views - 1) ? fabsf(angles[views - 1] - angles[0]) / (views - 1)
                                                  : fabsf(angles[j + 1] - angles[j]);
                    float b = angles[j] - rot;
                    float cb = cosf(b), sb = sinf(b);
                    float L = sid - x * cb - y * sb;
                    float mag = sdd / L;
                    float t = -x * sb + y * cb;
                    float u = curved ? sdd * atan2f(t, L) : mag * t;
                    float ui = (u - g->u0) / g->u_step;
                    if (ui < 0 || ui + 1 > nu - 1) {
                        acc = 0;
                        alive[vi] = 0;
                        break;
                    }
                    int uf = (int)floorf(ui);
                    float ru = ui - uf;
                    float dw = curved ? 1.0f / (L * L + t * t) : 1.0f / (L * L);
                    if (cone) {
                        float vidx = (mag * z - g->v0) / g->dv * vsgn;
                        int vf = (int)floorf(vidx);
                        if (vf < 0 || vf + 1 > nv - 1) {
                            acc = 0;
                            alive[vi] = 0;
                            break;
                        }
                        float rv = vidx - vf;
                        const float* r0 = F + ((int64_t)vf * views + j) * nu;
                        const float* r1 = F + ((int64_t)(vf + 1) * views + j) * nu;
                        float p0 = r0[uf] * (1 - ru) + r0[uf + 1] * ru;
                        float p1 = r1[uf] * (1 - ru) + r1[uf + 1] * ru;
                        acc += (sid * dw) * ((1 - rv) * p0 + rv * p1) * dang * div;
                    } else {
                        const float* r0 = F + ((int64_t)iz * views + j) * nu;
                        acc += (sid * dw) * ((1 - ru) * r0[uf] + ru * r0[uf + 1]) * dang * div;
                    }
                }
                vol[vi] = acc;
            }
}

/* out [nv][views][nu] for views [v0, v1) (flat detector, circular, no matrices). */
void cpu_fp(const mct_geom* g, const float* angles, const float* u_arr, const float* v_arr, const float* vol,
            float* out, int v0, int v1) {
    const int nx = g->nx, nz = g->nz, nu = g->nu, nv = g->nv, views = g->views;
    const int cone = (g->flags & MCT_CONE) != 0;
    const float sid = g->sid, sdd = g->sdd, px = g->px, pz = g->pz, step = g->fp_step;
    const float img_dimension = nx * px, image_dimension_z = nz * pz;
    const float l_min = sid - sqrtf(2 * img_dimension * img_dimension + image_dimension_z * image_dimension_z) / 2.0f;
    const float vd = sqrtf(2 * px * px + pz * pz);
    const float x0 = -(nx - 1.0f) / 2.0f * px + g->cx;
    const float y0 = -(nx - 1.0f) / 2.0f * (-px) + g->cy;
    const float z0 = -(nz - 1.0f) / 2.0f * pz + g->cz;
    const int K = g->fp_steps;
#pragma omp parallel for collapse(3) schedule(dynamic, 16)
    for (int j = v0; j < v1; ++j)
        for (int iv = 0; iv < nv; ++iv)
            for (int iu = 0; iu < nu; ++iu) {
                float dx = -(sdd - sid), dy = u_arr[iu], dz = v_arr[iv];
                float dist = sqrtf((dx - sid) * (dx - sid) + dy * dy + dz * dz);
                float ux = (dx - sid) / dist, uy = dy / dist, uz = dz / dist;
                float cb = cosf(angles[j]), sb = sinf(angles[j]);
                float acc = 0.0f;
                for (int k = 0; k < K; ++k) {
                    float l = k * step * vd + l_min;
                    float x = sid + ux * l, y = uy * l, z = uz * l;
                    float xr = x * cb - y * sb, yr = y * cb + x * sb;
                    int xi = (int)floorf((xr - x0) / px);
                    int yi = (int)floorf((yr - y0) / (-px));
                    if (xi >= 0 && xi + 1 < nx && yi >= 0 && yi + 1 < nx) {
                        float xw = (xr - (xi * px + x0)) / px;
                        float yw = (yr - (yi * (-px) + y0)) / (-px);
                        int zi;
                        float zw = 0.0f;
                        if (cone) {
                            zi = (int)floorf((z - z0) / pz);
                            if (!(zi >= 0 && zi + 1 < nz)) continue;
                            zw = (z - (zi * pz + z0)) / pz;
                        } else {
                            zi = iv;
                        }
                        const float* b = vol + ((int64_t)zi * nx + yi) * nx + xi;
                        float lo = (1 - xw) * (1 - yw) * b[0] + xw * (1 - yw) * b[1] + (1 - xw) * yw * b[nx] + xw * yw * b[nx + 1];
                        if (cone) {
                            const float* c = b + (int64_t)nx * nx;
                            float hi = (1 - xw) * (1 - yw) * c[0] + xw * (1 - yw) * c[1] + (1 - xw) * yw * c[nx] +
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
