// Sinogram weighting shared by the weighting kernels (csrc/filter.cu) and the fused
// weighting + tensor-core operand split (csrc/filter_tc.cu): BHCorrection
// run_mgfbp.py:946-954 and WeightSgm :956-1011, one element at a time, the same
// operations in the same order wherever they run.
#pragma once
#include <cmath>

#include "common.cuh"

namespace mct {

struct WeightParams {
    int nu, nv, views, curved, short_scan, n_bh, view_begin;
    int64_t row_stride, view_stride;
    float u0, u_step, v0, v_step, sdd, scan;
    float num_rounds, remain;  // short-scan constants
};

// Parker / over-scan weight of one (view, column), run_mgfbp.py:971-1011.
__device__ __forceinline__ float parker(const WeightParams& p, float beta, float u) {
    const float PI = (float)kPI;
    float rot_dir = fabsf(p.scan) / p.scan;
    float gamma = p.curved ? ((-1.0f) * u / p.sdd) * rot_dir : atan2f(-u, p.sdd) * rot_dir;
    float gmax = p.remain - PI;
    float nr = p.num_rounds, ra = p.remain;
    float w = 0.0f;
    if (ra <= PI && nr == 0.0f) {
        w = 1.0f;
    } else if (ra <= PI && nr >= 1.0f) {
        if (0.0f <= beta && beta < ra) w = beta / ra;
        else if (ra <= beta && beta < 2 * PI * nr) w = 1.0f;
        else if (2 * PI * nr <= beta && beta <= (2 * PI * nr + ra)) w = (2 * PI * nr + ra - beta) / ra;
    } else if (PI < ra && ra <= 2 * PI) {
        if (0.0f <= beta && beta < (gmax - 2 * gamma)) {
            w = sinf(PI / 2 * beta / (gmax - 2 * gamma));
            w = w * w;
        } else if ((gmax - 2 * gamma) <= beta && beta < (PI * (2 * nr + 1) - 2 * gamma)) {
            w = 1.0f;
        } else if ((PI * (2 * nr + 1) - 2 * gamma) <= beta && beta <= (PI * (2 * nr + 1) + gmax)) {
            w = sinf(PI / 2 * (PI + gmax - (beta - PI * 2 * nr)) / (gmax + 2 * gamma));
            w = w * w;
        }
    } else {
        w = 1.0f;
    }
    return w;
}

// Distance factor's denominator and the curved detector's cosine (per row v, column u).
__device__ __forceinline__ float weight_den(const WeightParams& p, float u, float v) {
    const float sdd = p.sdd;
    return p.curved ? sqrtf(sdd * sdd + v * v) : sqrtf(sdd * sdd + u * u + v * v);
}
__device__ __forceinline__ float weight_cos(const WeightParams& p, float u) {
    return p.curved ? cosf((-1.0f) * u / p.sdd) : 0.0f;
}

// One weighted element: beam-hardening polynomial, cosine weight, Parker weight
// (beta = |angle - angle_0| of the element's view, used with short scans only).
__device__ __forceinline__ float weight_value(const WeightParams& p, float val, const float* __restrict__ bh, float u,
                                              float cs, float den, float beta) {
    if (p.n_bh > 0) {
        float acc = 0.0f, pw = val;
        for (int t = 0; t < p.n_bh; ++t) {
            acc += bh[t] * pw;
            pw *= val;
        }
        val = acc;
    }
    const float sdd = p.sdd;
    if (p.curved) val = val * sdd * cs * sdd / den;
    else val = (val * sdd * sdd) / den;
    if (p.short_scan) val *= parker(p, beta, u);
    return val;
}

inline WeightParams weight_params(const mct_geom* g, int64_t row_stride, int64_t view_stride, int n_bh) {
    WeightParams p{};
    p.nu = g->nu; p.nv = g->nv; p.views = g->views;
    p.view_begin = g->view_begin;  // angles is the whole scan's table (view-chunked FBP)
    p.curved = (g->flags & MCT_CURVED) != 0;
    p.short_scan = (g->flags & MCT_SHORT_SCAN) != 0;
    p.n_bh = n_bh;
    p.row_stride = row_stride; p.view_stride = view_stride;
    p.u0 = g->u0; p.u_step = g->u_step; p.v0 = g->v0; p.v_step = g->v_step;
    p.sdd = g->sdd; p.scan = g->total_scan_angle;
    const float PI = (float)kPI;
    p.num_rounds = floorf(fabsf(p.scan) / (PI * 2));
    p.remain = fabsf(p.scan) - p.num_rounds * PI * 2;
    return p;
}

}  // namespace mct
