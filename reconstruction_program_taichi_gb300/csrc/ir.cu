// Iterative-reconstruction kernels: the reference CGLS backprojector, TV operators,
// float64 reductions and fused CGLS vector updates.
//
// Reference code replaced (run_mgfbp_iterative_recon_IRN_CGLS.py):
// BackProjectionPixelDrivenPerView :372-474 + SetTruncatedRegionToZero :477-481,
// GenerateWR :234-243, TVPenaltyVal :245-254, Dt_W_D :267-286, and the NumPy vector
// algebra of TikhonovSol :188-232.
#include <cmath>

#include "common.cuh"

namespace mct {
namespace {

constexpr int UB_TX = 32, UB_TY = 8, UB_ZC = 8, UB_VCHUNK = 512;
constexpr int RED_BLOCKS = 152 * 4, RED_THREADS = 256;

struct UbParams {
    int nx, nz, nu, nv, views, cone, curved;
    float sid, sdd, img_rot, px;
    float u0, inv_ustep, v0, kv;
    float ex_x, ex_y, ey_x, ey_y, ez_x, ez_y;  // (x, y) per unit (ix, iy, iz), rotated
    float o_x, o_y;
    float zx, zy, zz, z0;                      // z (without the per-view centre) per unit index
};

// All views of the per-view backprojector, accumulated in registers in view order.
// SRC 0 reads the plain sinogram [nv][views][nu] (4 gathers per update); SRC 1 reads
// the packed bilinear coefficients of mct_pack_strided (one 16-byte float32 or 8-byte
// bf16 / float16 gather per update; the same bilinear value up to float32 rounding).
template <int SRC, typename QT, typename PT>
__global__ void __launch_bounds__(UB_TX* UB_TY)
bp_unmatched_kernel(UbParams p, const float* __restrict__ angles, const float* __restrict__ czv, float cz_const,
                    const float* __restrict__ sgm, const void* __restrict__ packed, float* __restrict__ vol,
                    const uint32_t* __restrict__ f16_max) {
    const int nq = p.nu - 1;  // packed: nv rows of nu-1 stencils per view
    __shared__ float4 tab[UB_VCHUNK];  // {cos b, sin b, cz_j, unused}
    const int ix = blockIdx.x * UB_TX + threadIdx.x;
    const int iy = blockIdx.y * UB_TY + threadIdx.y;
    const int zb = blockIdx.z * UB_ZC;
    const int tid = threadIdx.y * UB_TX + threadIdx.x;
    const bool active = ix < p.nx && iy < p.nx;
    const float bx = p.o_x + ix * p.ex_x + iy * p.ey_x + zb * p.ez_x;
    const float by = p.o_y + ix * p.ex_y + iy * p.ey_y + zb * p.ez_y;
    const float bz = p.z0 + ix * p.zx + iy * p.zy + zb * p.zz;
    const int64_t rowstride = (int64_t)p.views * p.nu;
    float acc[UB_ZC];
#pragma unroll
    for (int k = 0; k < UB_ZC; ++k) acc[k] = 0.0f;
    uint32_t trunc = 0;

    for (int jc = 0; jc < p.views; jc += UB_VCHUNK) {
        const int nvc = min(UB_VCHUNK, p.views - jc);
        __syncthreads();
        for (int q = tid; q < nvc; q += UB_TX * UB_TY) {
            float s, c;
            sincosf(angles[jc + q] - p.img_rot, &s, &c);
            tab[q] = make_float4(c, s, czv ? czv[jc + q] : cz_const, 0.0f);
        }
        __syncthreads();
        if (!active) continue;
        for (int q = 0; q < nvc; ++q) {
            const int j = jc + q;
            const float4 tb = tab[q];
            const float cb = tb.x, sb = tb.y;
            const float scb = p.sid * cb, ssb = p.sid * sb;
#pragma unroll
            for (int k = 0; k < UB_ZC; ++k) {
                if (zb + k >= p.nz) continue;
                const float x = fmaf((float)k, p.ez_x, bx);
                const float y = fmaf((float)k, p.ez_y, by);
                const float z = fmaf((float)k, p.zz, bz) + tb.z;
                const float L = p.sid - x * cb - y * sb;
                const float qx = x - scb, qy = y - ssb;
                const float aqx = fabsf(qx), aqy = fabsf(qy);
                const float dfac = sqrtf(qx * qx + qy * qy + z * z) / (aqx > aqy ? aqx : aqy);
                const float mag = p.sdd / L;
                const float t = -x * sb + y * cb;
                const float u = p.curved ? p.sdd * atan2f(t, L) : mag * t;
                const float ui = (u - p.u0) * p.inv_ustep;
                if (!(ui >= 0.0f && ui + 1.0f <= (float)(p.nu - 1))) {
                    trunc |= 1u << k;
                    continue;
                }
                const float uf = floorf(ui);
                const float ru = ui - uf;
                const int uc = (int)uf;
                const float w = dfac * p.px;
                if (p.cone) {
                    const float vi = (mag * z - p.v0) * p.kv;
                    const float vf = floorf(vi);
                    if (!(vf >= 0.0f && vf + 1.0f <= (float)(p.nv - 1))) continue;
                    const float rv = vi - vf;
                    if (SRC == 0) {
                        const float* s0 = sgm + (int64_t)(int)vf * rowstride + (int64_t)j * p.nu + uc;
                        const float a = __ldg(s0), b = __ldg(s0 + 1), c = __ldg(s0 + rowstride),
                                    d = __ldg(s0 + rowstride + 1);
                        const float p0 = a * (1 - ru) + b * ru;
                        const float p1 = c * (1 - ru) + d * ru;
                        acc[k] += ((1 - rv) * p0 + rv * p1) * w;
                    } else {
                        float2 lo, hi;
                        Quad<QT>::load(reinterpret_cast<const QT*>(packed) + ((int64_t)j * p.nv + (int)vf) * nq + uc, lo,
                                       hi);
                        const float2 s2 = __ffma2_rn(make_float2(ru, ru), hi, lo);
                        acc[k] += fmaf(rv, s2.y, s2.x) * w;
                    }
                } else {
                    if (SRC == 0) {
                        const float* s0 = sgm + (int64_t)(zb + k) * rowstride + (int64_t)j * p.nu + uc;
                        const float a = __ldg(s0), b = __ldg(s0 + 1);
                        acc[k] += ((1 - ru) * a + ru * b) * w;
                    } else {
                        const float2 pr =
                            Pair<PT>::load(reinterpret_cast<const PT*>(packed) + ((int64_t)j * p.nv + zb + k) * nq + uc);
                        acc[k] += fmaf(ru, pr.y, pr.x) * w;
                    }
                }
            }
        }
    }
    if (!active) return;
    const int64_t plane = (int64_t)p.nx * p.nx;
    const float unscale = IsF16<QT>::value ? ldexpf(1.0f, -f16_scale_exp(*f16_max)) : 1.0f;
#pragma unroll
    for (int k = 0; k < UB_ZC; ++k)
        if (zb + k < p.nz)
            vol[(zb + k) * plane + (int64_t)iy * p.nx + ix] = ((trunc >> k) & 1u) ? 0.0f : acc[k] * unscale;
}

// Axial view mode over packed coefficients.  For a voxel column (x, y) the rotation,
// the magnification, u, the truncation test and the in-plane distance to the source
// depend only on (x, y, view), so they are evaluated once per column and view; per
// slice remain v, one gather and the distance factor
//     sqrt(qx^2 + qy^2 + z^2) / max(|qx|, |qy|) * px
// (run_mgfbp_iterative_recon_IRN_CGLS.py:417-421) with the square root as d2 * rsqrt(d2).
// A column that leaves the detector in u in some view is all zero in the reference
// (SetTruncatedRegionToZero), so its thread stops there.  As in the FDK kernel, v and
// z are affine in the slice index, and the register budget lets the UA_ZC gathers of
// a view issue ahead of their arithmetic, which hides the gather latency.
constexpr int UA_ZC = 16;

// (D^T W D x)[i] of run_mgfbp_iterative_recon_IRN_CGLS.py:267-286: forward differences
// weighted by W, their transposed differences on the interior indices [1, n-2] of each
// axis (z only when nz > 2), 0 on the borders.
template <typename T>
__device__ __forceinline__ float dtwd_at(const T* __restrict__ x, const float* __restrict__ wr, int nx, int nz,
                                         int64_t i, int iz, int iy, int ix) {
    const int64_t plane = (int64_t)nx * nx;
    const float c = ldv(x, i);
    float r = 0.0f;
    if (iy >= 1 && iy <= nx - 2) {  // uxx = Ux[y] - Ux[y-1]
        const float ux_c = wr[i] * (ldv(x, i + nx) - c);
        const float ux_m = wr[i - nx] * (c - ldv(x, i - nx));
        r -= ux_c - ux_m;
    }
    if (ix >= 1 && ix <= nx - 2) {
        const float uy_c = wr[i] * (ldv(x, i + 1) - c);
        const float uy_m = wr[i - 1] * (c - ldv(x, i - 1));
        r -= uy_c - uy_m;
    }
    if (nz > 2 && iz >= 1 && iz <= nz - 2) {
        const float uz_c = wr[i] * (ldv(x, i + plane) - c);
        const float uz_m = wr[i - plane] * (c - ldv(x, i - plane));
        r -= uz_c - uz_m;
    }
    return r;
}

// value as stored in a volume of type T (bf16 iterates: rounded to nearest)
template <typename T>
__device__ __forceinline__ float stored(float v);
template <>
__device__ __forceinline__ float stored<float>(float v) { return v; }
template <>
__device__ __forceinline__ float stored<__nv_bfloat16>(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// CG epilogue of the backprojector (the operator application of one CGLS step):
// q = P^T p + s1 D^T W1 D d (+ s2 D^T W2 D d), and the block's float64 partial of <d, q>
// over the stored q.  d and q are volumes of the kernel's output type.
struct CgEpi {
    const void* d;
    const float* w1;
    const float* w2;
    float s1, s2;
    double* partials;  // one per block, in blockIdx order
};
// Resident blocks per SM that the register allocation targets: 3 (80 registers) for
// 8-byte operands and for 16-byte ones without the CG epilogue (with slices in pairs,
// 512x512x64 / 360 views float32 5.67 ms with 2 blocks of 128 registers, 5.44 ms with
// 3 blocks, bit-identical), 2 for 16-byte operands with the epilogue.
template <typename QT, bool EPI>
constexpr int ua_min_blocks() {
    return sizeof(QT) == 8 || !EPI ? 3 : 2;
}
template <bool CONE, typename QT, typename PT, typename OT = float, bool EPI = false>
__global__ void __launch_bounds__(UB_TX* UB_TY, ua_min_blocks<QT, EPI>())
bp_unmatched_axial_kernel(UbParams p, const float* __restrict__ angles, const float* __restrict__ czv, float cz_const,
                          const void* __restrict__ packed, OT* __restrict__ vol,
                          const uint32_t* __restrict__ f16_max, CgEpi epi = CgEpi{}) {
    const int nq = p.nu - 1;  // packed: nv rows of nu-1 coefficient sets per view
    __shared__ float4 tab[UB_VCHUNK];  // {cos b, sin b, cz_j, sid*cos b}
    __shared__ float tab_s[UB_VCHUNK];  // sid*sin b
    // a warp is 4 columns along x x 8 along y of the block's 32 x 8 (a view's gathers
    // then span fewer detector columns; 512x512x64 / 360 views: float32 6.01 -> 5.79 ms,
    // bf16 5.94 -> 5.91)
    constexpr int WX = 4;
    const int tid = threadIdx.y * UB_TX + threadIdx.x;
    const int wq = tid >> 5, lq = tid & 31;
    const int ix = blockIdx.x * UB_TX + (wq % (UB_TX / WX)) * WX + (lq % WX);
    const int iy = blockIdx.y * UB_TY + (wq / (UB_TX / WX)) * (32 / WX) + lq / WX;
    const int zb = blockIdx.z * UA_ZC;
    const bool active = ix < p.nx && iy < p.nx;
    // same expressions as the general kernel with the axial mode's zero z-terms
    const float x = p.o_x + ix * p.ex_x + iy * p.ey_x + zb * p.ez_x;
    const float y = p.o_y + ix * p.ex_y + iy * p.ey_y + zb * p.ez_y;
    const float bz = p.z0 + ix * p.zx + iy * p.zy + zb * p.zz;
    float acc[UA_ZC];
#pragma unroll
    for (int k = 0; k < UA_ZC; ++k) acc[k] = 0.0f;
    bool trunc = false;

    for (int jc = 0; jc < p.views; jc += UB_VCHUNK) {
        const int nvc = min(UB_VCHUNK, p.views - jc);
        __syncthreads();
        for (int q = tid; q < nvc; q += UB_TX * UB_TY) {
            float s, c;
            sincosf(angles[jc + q] - p.img_rot, &s, &c);
            tab[q] = make_float4(c, s, czv ? czv[jc + q] : cz_const, p.sid * c);
            tab_s[q] = p.sid * s;
        }
        __syncthreads();
        if (!active || trunc) continue;
        for (int q = 0; q < nvc; ++q) {
            const int j = jc + q;
            const float4 tb = tab[q];
            const float cb = tb.x, sb = tb.y;
            const float L = p.sid - x * cb - y * sb;
            const float qx = x - tb.w, qy = y - tab_s[q];
            const float aqx = fabsf(qx), aqy = fabsf(qy);
            const float mq = aqx > aqy ? aqx : aqy;
            const float rr = 1.0f / (L * mq);  // one reciprocal for sdd / L and px / max(|qx|, |qy|)
            const float mag = p.sdd * mq * rr;
            const float t = -x * sb + y * cb;
            const float u = p.curved ? p.sdd * atan2f(t, L) : mag * t;
            const float ui = (u - p.u0) * p.inv_ustep;
            if (!(ui >= 0.0f && ui + 1.0f <= (float)(p.nu - 1))) {
                trunc = true;
                break;
            }
            const float uf = floorf(ui);
            const float ru = ui - uf;
            const int uc = (int)uf;
            const float r2 = qx * qx + qy * qy;
            const float wpx = p.px * L * rr;
            if (CONE) {
                const QT* base = reinterpret_cast<const QT*>(packed) + (int64_t)j * p.nv * nq + uc;
                const float2 ru2 = make_float2(ru, ru);
                // slice k: z = zA + k zz, v index = vA + k vB
                const float zA = bz + tb.z;
                const float vA = (mag * zA - p.v0) * p.kv, vB = (mag * p.zz) * p.kv;
                const unsigned top = (unsigned)(p.nv - 2);  // rows [0, nv-2] hold a bilinear cell (nv >= 2)
                // Slices k and k+1 share each packed f32x2 operation (v, the row
                // fraction, z and the distance factor); every rounding is the scalar
                // loop's, so the sums are bit-identical to it (5.81 -> 5.68 ms float32,
                // 5.92 -> 5.62 ms bf16 at 512^2 x 64 / 360 views).
                const float2 vA2 = make_float2(vA, vA), vB2 = make_float2(vB, vB);
                const float2 zA2 = make_float2(zA, zA), zz2 = make_float2(p.zz, p.zz);
                const float2 r22 = make_float2(r2, r2), wpx2 = make_float2(wpx, wpx);
                static_assert(UA_ZC % 2 == 0, "slices are taken in pairs");
#pragma unroll
                for (int k = 0; k < UA_ZC; k += 2) {
                    const float2 kk = make_float2((float)k, (float)(k + 1));
                    const float2 vi = __ffma2_rn(kk, vB2, vA2);
                    const float vf0 = floorf(vi.x), vf1 = floorf(vi.y);
                    const unsigned vu0 = (unsigned)(int)vf0, vu1 = (unsigned)(int)vf1;  // negative rows wrap around
                    const float2 rv = __fadd2_rn(vi, make_float2(-vf0, -vf1));
                    float2 lo0, hi0, lo1, hi1;
                    Quad<QT>::load(base + min(vu0, top) * (unsigned)nq, lo0, hi0);
                    Quad<QT>::load(base + min(vu1, top) * (unsigned)nq, lo1, hi1);
                    const float2 s0 = __ffma2_rn(ru2, hi0, lo0), s1 = __ffma2_rn(ru2, hi1, lo1);
                    const float2 z = __ffma2_rn(kk, zz2, zA2);
                    const float2 d2 = __ffma2_rn(z, z, r22);
                    const float2 w = __fmul2_rn(__fmul2_rn(d2, make_float2(rsqrtf(d2.x), rsqrtf(d2.y))), wpx2);
                    // a row outside [0, nv-2] contributes nothing
                    acc[k] = fmaf(fmaf(rv.x, s0.y, s0.x), vu0 <= top ? w.x : 0.0f, acc[k]);
                    acc[k + 1] = fmaf(fmaf(rv.y, s1.y, s1.x), vu1 <= top ? w.y : 0.0f, acc[k + 1]);
                }
            } else {
                const PT* base = reinterpret_cast<const PT*>(packed) + ((int64_t)j * p.nv + zb) * nq + uc;
#pragma unroll
                for (int k = 0; k < UA_ZC; ++k) {
                    if (zb + k < p.nz) {
                        const float z = fmaf((float)k, p.zz, bz) + tb.z;
                        const float2 pr = Pair<PT>::load(base + k * nq);
                        const float d2 = fmaf(z, z, r2);
                        acc[k] += fmaf(ru, pr.y, pr.x) * (d2 * rsqrtf(d2) * wpx);
                    }
                }
            }
        }
    }
    const int64_t plane = (int64_t)p.nx * p.nx;
    const float unscale = IsF16<QT>::value ? ldexpf(1.0f, -f16_scale_exp(*f16_max)) : 1.0f;
    if constexpr (EPI) {
        // q = P^T p + s1 D^T W1 D d (+ s2 D^T W2 D d) in the order of the separate passes
        // (each term added to the stored value), then <d, q> of the stored q.  The
        // backprojection is stored first, as without the epilogue, and the terms are
        // added in a compact loop over the thread's own slices (a loop that indexes
        // acc[] at run time would move the accumulators to local memory, and an
        // unrolled stencil costs the main loop registers).
        const OT* d = static_cast<const OT*>(epi.d);
        double dsum = 0.0;
        if (active) {
#pragma unroll
            for (int k = 0; k < UA_ZC; ++k)
                if (zb + k < p.nz) stv(vol, (zb + k) * plane + (int64_t)iy * p.nx + ix, trunc ? 0.0f : acc[k] * unscale);
#pragma unroll 1
            for (int k = 0; k < UA_ZC && zb + k < p.nz; ++k) {
                const int64_t i = (zb + k) * plane + (int64_t)iy * p.nx + ix;
                float v = ldv(vol, i);  // this thread's own store
                if (epi.w1) v = __fadd_rn(__fmul_rn(epi.s1, dtwd_at(d, epi.w1, p.nx, p.nz, i, zb + k, iy, ix)), v);
                if (epi.w2) v = __fadd_rn(__fmul_rn(epi.s2, dtwd_at(d, epi.w2, p.nx, p.nz, i, zb + k, iy, ix)), v);
                stv(vol, i, v);
                dsum += (double)ldv(d, i) * (double)stored<OT>(v);
            }
        }
        // block sum over the 256 threads, then one partial per block
        __shared__ double red[UB_TX * UB_TY / 32];
        const int lane = tid & 31, w = tid >> 5;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dsum += __shfl_down_sync(0xffffffffu, dsum, o);
        if (lane == 0) red[w] = dsum;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
#pragma unroll
            for (int q = 0; q < UB_TX * UB_TY / 32; ++q) t += red[q];
            epi.partials[((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = t;
        }
        return;
    }
    if (!active) return;
#pragma unroll
    for (int k = 0; k < UA_ZC; ++k)
        if (zb + k < p.nz) stv(vol, (zb + k) * plane + (int64_t)iy * p.nx + ix, trunc ? 0.0f : acc[k] * unscale);
}

// Forward differences (y, x, z) with zero at the far edge; z only when nz > 2.
struct Grad {
    float gy, gx, gz;
};
template <typename T>
__device__ __forceinline__ Grad grad_at(const T* __restrict__ x, int nx, int nz, int iz, int iy, int ix) {
    const int64_t plane = (int64_t)nx * nx;
    const int64_t i = (int64_t)iz * plane + (int64_t)iy * nx + ix;
    const float c = ldv(x, i);
    Grad g;
    g.gy = (iy < nx - 1) ? ldv(x, i + nx) - c : 0.0f;
    g.gx = (ix < nx - 1) ? ldv(x, i + 1) - c : 0.0f;
    g.gz = (nz > 2 && iz < nz - 1) ? ldv(x, i + plane) - c : 0.0f;
    return g;
}

template <typename T>
__global__ void tv_weights_kernel(int nx, int nz, float beta, const T* __restrict__ x, float* __restrict__ wr) {
    const int64_t n = (int64_t)nz * nx * nx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % nx);
        const int iy = (int)((i / nx) % nx);
        const int iz = (int)(i / ((int64_t)nx * nx));
        Grad g = grad_at(x, nx, nz, iz, iy, ix);
        wr[i] = 1.0f / sqrtf(g.gy * g.gy + g.gx * g.gx + g.gz * g.gz + beta);
    }
}

// ADMM-TV splitting updates (run_mgfbp_iterative_recon_ADMM_CGLS.py:128-143), one pass:
// w = D x + p / rho per in-plane axis (Diff along y and x, 0 at the far edge);
// v = w where |w| = sqrt(wy^2 + wx^2) exceeds thr, else 0 (the reference's rule is a
// hard threshold: it multiplies w by (|w| - thr > 0) * |w| / |w|); p += rho * (D x - v).
__global__ void admm_shrink_kernel(int nx, int nz, const float* __restrict__ x, float rho, float thr,
                                   float* __restrict__ vy, float* __restrict__ vx, float* __restrict__ py,
                                   float* __restrict__ px) {
    const int64_t n = (int64_t)nz * nx * nx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % nx);
        const int iy = (int)((i / nx) % nx);
        const float c = x[i];
        const float dy = iy < nx - 1 ? x[i + nx] - c : 0.0f;
        const float dx = ix < nx - 1 ? x[i + 1] - c : 0.0f;
        const float wy = dy + py[i] / rho, wx = dx + px[i] / rho;
        const float t = sqrtf(wy * wy + wx * wx);
        const bool keep = (t - thr) > 0.0f && t != 0.0f;
        const float ny = keep ? wy : 0.0f, nx_ = keep ? wx : 0.0f;
        vy[i] = ny;
        vx[i] = nx_;
        py[i] = py[i] + rho * (dy - ny);
        px[i] = px[i] + rho * (dx - nx_);
    }
}

// Right-hand side of the ADMM x-step (FunctionY, :160-162):
// out = bpb + rho * (DiffT(vy, y) + DiffT(vx, x)) - (DiffT(py, y) + DiffT(px, x)), with
// DiffT(a)[i] = a[i-1] - a[i] on interior indices and 0 on the first and last.
__global__ void admm_rhs_kernel(int nx, int nz, const float* __restrict__ bpb, const float* __restrict__ vy,
                                const float* __restrict__ vx, const float* __restrict__ py,
                                const float* __restrict__ px, float rho, float* __restrict__ out) {
    const int64_t n = (int64_t)nz * nx * nx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % nx);
        const int iy = (int)((i / nx) % nx);
        const bool iny = iy >= 1 && iy <= nx - 2, inx = ix >= 1 && ix <= nx - 2;
        const float tvy = iny ? vy[i - nx] - vy[i] : 0.0f, tvx = inx ? vx[i - 1] - vx[i] : 0.0f;
        const float tpy = iny ? py[i - nx] - py[i] : 0.0f, tpx = inx ? px[i - 1] - px[i] : 0.0f;
        out[i] = bpb[i] + rho * (tvy + tvx) - (tpy + tpx);
    }
}

__device__ __forceinline__ double block_sum(double v);

// out = a*out_in + s * (D^T W D x), run_mgfbp_iterative_recon_IRN_CGLS.py:267-286.
// DOT: also the per-block float64 partial sums of x[i] * out[i] (the CG step's <d, q>
// while q is being written; out may alias out_in).
template <bool DOT, typename T = float>
__global__ void __launch_bounds__(256)
dtwd_kernel(int nx, int nz, const T* __restrict__ x, const float* __restrict__ wr, float s,
            const T* out_in, float a, T* out, double* __restrict__ partials) {
    const int64_t n = (int64_t)nz * nx * nx;
    const int64_t plane = (int64_t)nx * nx;
    double dsum = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % nx);
        const int iy = (int)((i / nx) % nx);
        const int iz = (int)(i / plane);
        const float c = ldv(x, i);
        const float r = dtwd_at(x, wr, nx, nz, i, iz, iy, ix);
        float v = s * r;
        if (a != 0.0f) v += a * ldv(out_in, i);
        stv(out, i, v);
        if (DOT) dsum += (double)c * (double)ldv(out, i);  // the stored value
    }
    if (DOT) {
        dsum = block_sum(dsum);
        if (threadIdx.x == 0) partials[blockIdx.x] = dsum;
    }
}

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double red[RED_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    v = (threadIdx.x < RED_THREADS / 32) ? red[threadIdx.x] : 0.0;
    if (w == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;  // valid in thread 0
}

// Per thread four independent float64 accumulators (the products of two float32 values
// are exact in float64, so each step is one DFMA): float64 has a fraction of the float32
// rate on this GPU, and one dependent chain per thread left the kernel at 10 % issue.
template <typename T = float>
__global__ void __launch_bounds__(RED_THREADS)
dot_partial_kernel(const T* __restrict__ a, const T* __restrict__ b, int64_t n, double* __restrict__ partials) {
    const int64_t stride = (int64_t)gridDim.x * RED_THREADS;
    int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (; i + 3 * stride < n; i += 4 * stride) {
        s0 = fma((double)ldv(a, i), (double)ldv(b, i), s0);
        s1 = fma((double)ldv(a, i + stride), (double)ldv(b, i + stride), s1);
        s2 = fma((double)ldv(a, i + 2 * stride), (double)ldv(b, i + 2 * stride), s2);
        s3 = fma((double)ldv(a, i + 3 * stride), (double)ldv(b, i + 3 * stride), s3);
    }
    for (; i < n; i += stride) s0 = fma((double)ldv(a, i), (double)ldv(b, i), s0);
    double s = (s0 + s1) + (s2 + s3);
    s = block_sum(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(RED_THREADS)
tv_partial_kernel(int nx, int nz, float beta, const float* __restrict__ x, double* __restrict__ partials) {
    const int64_t n = (int64_t)nz * nx * nx;
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * RED_THREADS) {
        const int ix = (int)(i % nx);
        const int iy = (int)((i / nx) % nx);
        const int iz = (int)(i / ((int64_t)nx * nx));
        Grad g = grad_at(x, nx, nz, iz, iy, ix);
        s += sqrt((double)g.gy * g.gy + (double)g.gx * g.gx + (double)g.gz * g.gz + (double)beta);
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(RED_THREADS)
finish_sum_kernel(const double* __restrict__ partials, int n, double* __restrict__ result) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += RED_THREADS) s += partials[i];
    s = block_sum(s);
    if (threadIdx.x == 0) *result = s;
}

// x += alpha d; r -= alpha q; partial sums of r^2 (alpha = rr/dq read on device)
template <typename T = float>
__global__ void __launch_bounds__(RED_THREADS)
cgls_update_kernel(int64_t n, const double* __restrict__ rr, const double* __restrict__ dq, T* __restrict__ x,
                   T* __restrict__ r, const T* __restrict__ d, const T* __restrict__ q,
                   double* __restrict__ partials) {
    const float alpha = (float)(*rr / *dq);
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)RED_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * RED_THREADS) {
        const float di = ldv(d, i);
        stv(x, i, ldv(x, i) + alpha * di);
        stv(r, i, ldv(r, i) - alpha * ldv(q, i));
        const float ri = ldv(r, i);  // the stored value
        s += (double)ri * (double)ri;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

template <typename T = float>
__global__ void cgls_direction_kernel(int64_t n, const double* __restrict__ rr, const double* __restrict__ rr_new,
                                      const T* __restrict__ r, T* __restrict__ d) {
    const float beta = (float)(*rr_new / *rr);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        stv(d, i, ldv(r, i) + beta * ldv(d, i));
}

inline int ew_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

}  // namespace
}  // namespace mct

using namespace mct;

template <typename QT, typename PT>
void launch_unmatched_packed(const mct_geom* g, const UbParams& p, const mct_tables* t, const void* packed,
                                    float* vol, const uint32_t* f16_max, cudaStream_t s) {
    dim3 block(UB_TX, UB_TY);
    if (g->view_mode == 1) {
        dim3 grid((g->nx + UB_TX - 1) / UB_TX, (g->nx + UB_TY - 1) / UB_TY, (g->nz + UA_ZC - 1) / UA_ZC);
        if (p.cone)
            bp_unmatched_axial_kernel<true, QT, PT><<<grid, block, 0, s>>>(p, t->angles, t->cz, g->cz, packed, vol,
                                                                           f16_max);
        else
            bp_unmatched_axial_kernel<false, QT, PT><<<grid, block, 0, s>>>(p, t->angles, t->cz, g->cz, packed, vol,
                                                                            f16_max);
    } else {
        dim3 grid((g->nx + UB_TX - 1) / UB_TX, (g->nx + UB_TY - 1) / UB_TY, (g->nz + UB_ZC - 1) / UB_ZC);
        bp_unmatched_kernel<1, QT, PT><<<grid, block, 0, s>>>(p, t->angles, t->cz, g->cz, nullptr, packed, vol,
                                                              f16_max);
    }
}

extern "C" {

static int unmatched_params(const mct_geom* g, UbParams& p);

int mct_bp_ref_unmatched(const mct_geom* g, const mct_tables* t, const float* sgm, float* vol, void* stream) {
    UbParams p{};
    MCT_TRY(unmatched_params(g, p));
    MCT_REQUIRE(t && t->angles && sgm && vol, "mct_bp_ref_unmatched: NULL buffer");
    dim3 block(UB_TX, UB_TY);
    dim3 grid((g->nx + UB_TX - 1) / UB_TX, (g->nx + UB_TY - 1) / UB_TY, (g->nz + UB_ZC - 1) / UB_ZC);
    bp_unmatched_kernel<0, float4, float2><<<grid, block, 0, as_stream(stream)>>>(p, t->angles, t->cz, g->cz, sgm,
                                                                                  nullptr, vol, nullptr);
    return launched("bp_unmatched_kernel");
}

int mct_bp_ref_unmatched_packed_out(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype,
                                    void* vol, int32_t vol_dtype, void* stream) {
    if (vol_dtype == MCT_F32)
        return mct_bp_ref_unmatched_packed(g, t, packed, dtype, static_cast<float*>(vol), stream);
    UbParams p{};
    MCT_TRY(unmatched_params(g, p));
    MCT_REQUIRE(vol_dtype == MCT_BF16, "mct_bp_ref_unmatched_packed_out: vol_dtype must be MCT_F32 or MCT_BF16");
    MCT_REQUIRE(t && t->angles && packed && vol, "mct_bp_ref_unmatched_packed_out: NULL buffer");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16 || dtype == MCT_F16,
                "mct_bp_ref_unmatched_packed_out: dtype must be MCT_F32, MCT_BF16 or MCT_F16");
    MCT_REQUIRE(g->view_mode == 1 && p.cone,
                "mct_bp_ref_unmatched_packed_out: bf16 output needs the axial view mode and cone beam");
    MCT_REQUIRE((int64_t)g->nv * (g->nu - 1) < ((int64_t)1 << 31), "mct_bp_ref_unmatched_packed_out: detector too large");
    cudaStream_t s = as_stream(stream);
    dim3 block(UB_TX, UB_TY);
    dim3 grid((g->nx + UB_TX - 1) / UB_TX, (g->nx + UB_TY - 1) / UB_TY, (g->nz + UA_ZC - 1) / UA_ZC);
    __nv_bfloat16* out = static_cast<__nv_bfloat16*>(vol);
    if (dtype == MCT_F32)
        bp_unmatched_axial_kernel<true, float4, float2, __nv_bfloat16><<<grid, block, 0, s>>>(
            p, t->angles, t->cz, g->cz, packed, out, nullptr);
    else if (dtype == MCT_BF16)
        bp_unmatched_axial_kernel<true, uint2, uint32_t, __nv_bfloat16><<<grid, block, 0, s>>>(
            p, t->angles, t->cz, g->cz, packed, out, nullptr);
    else
        bp_unmatched_axial_kernel<true, h16x4, h16x2, __nv_bfloat16><<<grid, block, 0, s>>>(
            p, t->angles, t->cz, g->cz, packed, out, f16_trailer(g, packed));
    return launched("bp_unmatched_kernel");
}

size_t mct_bp_cg_partials_size(const mct_geom* g) {
    if (!g || g->nx < 1 || g->nz < 1) return 0;
    return (size_t)((g->nx + UB_TX - 1) / UB_TX) * (size_t)((g->nx + UB_TY - 1) / UB_TY) *
           (size_t)((g->nz + UA_ZC - 1) / UA_ZC) * sizeof(double);
}

int mct_bp_ref_unmatched_packed_cg(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype,
                                   const void* d, const float* wr1, float s1, const float* wr2, float s2, void* q,
                                   int32_t vec_dtype, double* partials, double* dq, void* stream) {
    UbParams p{};
    MCT_TRY(unmatched_params(g, p));
    MCT_REQUIRE(t && t->angles && packed && d && q && partials && dq, "mct_bp_ref_unmatched_packed_cg: NULL buffer");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16 || dtype == MCT_F16,
                "mct_bp_ref_unmatched_packed_cg: dtype must be MCT_F32, MCT_BF16 or MCT_F16");
    MCT_REQUIRE(vec_dtype == MCT_F32 || vec_dtype == MCT_BF16,
                "mct_bp_ref_unmatched_packed_cg: vec_dtype must be MCT_F32 or MCT_BF16");
    MCT_REQUIRE(g->view_mode == 1 && p.cone,
                "mct_bp_ref_unmatched_packed_cg: the fused epilogue needs the axial view mode and cone beam");
    MCT_REQUIRE(wr1 || !wr2, "mct_bp_ref_unmatched_packed_cg: wr2 given without wr1");
    MCT_REQUIRE(q != d && q != (const void*)wr1 && q != (const void*)wr2 && q != packed,
                "mct_bp_ref_unmatched_packed_cg: q aliases an input");
    MCT_REQUIRE((int64_t)g->nv * (g->nu - 1) < ((int64_t)1 << 31), "mct_bp_ref_unmatched_packed_cg: detector too large");
    cudaStream_t s = as_stream(stream);
    dim3 block(UB_TX, UB_TY);
    dim3 grid((g->nx + UB_TX - 1) / UB_TX, (g->nx + UB_TY - 1) / UB_TY, (g->nz + UA_ZC - 1) / UA_ZC);
    const CgEpi e{d, wr1, wr2, s1, s2, partials};
    const uint32_t* fm = dtype == MCT_F16 ? f16_trailer(g, packed) : nullptr;
    auto go = [&](auto out_tag) {
        using OT = decltype(out_tag);
        OT* out = static_cast<OT*>(q);
        if (dtype == MCT_F32)
            bp_unmatched_axial_kernel<true, float4, float2, OT, true><<<grid, block, 0, s>>>(p, t->angles, t->cz, g->cz,
                                                                                           packed, out, nullptr, e);
        else if (dtype == MCT_BF16)
            bp_unmatched_axial_kernel<true, uint2, uint32_t, OT, true><<<grid, block, 0, s>>>(
                p, t->angles, t->cz, g->cz, packed, out, nullptr, e);
        else
            bp_unmatched_axial_kernel<true, h16x4, h16x2, OT, true><<<grid, block, 0, s>>>(p, t->angles, t->cz, g->cz,
                                                                                         packed, out, fm, e);
    };
    if (vec_dtype == MCT_F32) go(float{});
    else go(__nv_bfloat16{});
    MCT_TRY(launched("bp_unmatched_kernel"));
    finish_sum_kernel<<<1, RED_THREADS, 0, s>>>(partials, (int)(grid.x * grid.y * grid.z), dq);
    return launched("finish_sum_kernel");
}

int mct_bp_ref_unmatched_packed(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype, float* vol,
                                void* stream) {
    UbParams p{};
    MCT_TRY(unmatched_params(g, p));
    MCT_REQUIRE(t && t->angles && packed && vol, "mct_bp_ref_unmatched_packed: NULL buffer");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16 || dtype == MCT_F16,
                "mct_bp_ref_unmatched_packed: dtype must be MCT_F32, MCT_BF16 or MCT_F16");
    MCT_REQUIRE((int64_t)g->nv * (g->nu - 1) < ((int64_t)1 << 31), "mct_bp_ref_unmatched_packed: detector too large");
    cudaStream_t s = as_stream(stream);
    if (dtype == MCT_F32)
        launch_unmatched_packed<float4, float2>(g, p, t, packed, vol, nullptr, s);
    else if (dtype == MCT_BF16)
        launch_unmatched_packed<uint2, uint32_t>(g, p, t, packed, vol, nullptr, s);
    else
        launch_unmatched_packed<h16x4, h16x2>(g, p, t, packed, vol, f16_trailer(g, packed), s);
    return launched("bp_unmatched_kernel");
}

static int unmatched_params(const mct_geom* g, UbParams& p) {
    MCT_TRY(check_geom(g, "mct_bp_ref_unmatched"));
    MCT_TRY(check_whole_scan(g, "mct_bp_ref_unmatched"));
    MCT_REQUIRE(!(g->flags & MCT_PMATRIX), "mct_bp_ref_unmatched: projection-matrix geometry is not supported");
    const bool cone = (g->flags & MCT_CONE) != 0;
    MCT_REQUIRE(!cone || g->nv >= 2, "mct_bp_ref_unmatched: cone beam needs at least 2 rows");
    MCT_REQUIRE(cone || g->nz <= g->nv, "mct_bp_ref_unmatched: fan beam needs nz <= detector rows");
    MCT_REQUIRE(g->u_step != 0.0f, "mct_bp_ref_unmatched: zero detector spacing");
    p.nx = g->nx; p.nz = g->nz; p.nu = g->nu; p.nv = g->nv; p.views = g->views;
    p.cone = cone; p.curved = (g->flags & MCT_CURVED) != 0;
    p.sid = g->sid; p.sdd = g->sdd; p.img_rot = g->img_rot; p.px = g->px;
    p.u0 = g->u0; p.inv_ustep = (float)(1.0 / (double)g->u_step);
    p.v0 = g->v0;
    if (cone) {
        MCT_REQUIRE(g->v_step != 0.0f && g->dv != 0.0f, "mct_bp_ref_unmatched: zero row spacing");
        p.kv = (float)((g->v_step > 0 ? 1.0 : -1.0) / (double)g->dv);
    }
    // voxel coordinates, run_mgfbp_iterative_recon_IRN_CGLS.py:386-401 (z without the
    // per-view centre, which is added per view)
    const double nx = g->nx, nz = g->nz, px = g->px, pz = g->pz;
    const double cr = std::cos((double)g->img_rot), sr = std::sin((double)g->img_rot);
    double ax[3] = {0, 0, 0}, ay[3] = {0, 0, 0}, az[3] = {0, 0, 0}, a0[3] = {0, 0, 0};
    if (g->view_mode == 1) {
        ax[0] = px; a0[0] = -px * (nx - 1) / 2.0 + g->cx;
        ay[1] = -px; a0[1] = px * (nx - 1) / 2.0 + g->cy;
        az[2] = pz; a0[2] = -(nz - 1) / 2.0 * pz;
    } else if (g->view_mode == 2) {
        ax[0] = px; a0[0] = -px * (nx - 1) / 2.0 + g->cx;
        ay[2] = -px; a0[2] = px * (nx - 1) / 2.0;
        az[1] = -pz; a0[1] = (nz - 1) / 2.0 * pz + g->cy;
    } else {
        ay[2] = -px; a0[2] = px * (nx - 1) / 2.0;
        ax[1] = -px; a0[1] = px * (nx - 1) / 2.0 + g->cy;
        az[0] = pz; a0[0] = -(nz - 1) / 2.0 * pz + g->cx;
    }
    auto rx = [&](const double* a) { return (float)(a[0] * cr + a[1] * sr); };
    auto ry = [&](const double* a) { return (float)(-a[0] * sr + a[1] * cr); };
    p.ex_x = rx(ax); p.ex_y = ry(ax); p.ey_x = rx(ay); p.ey_y = ry(ay); p.ez_x = rx(az); p.ez_y = ry(az);
    p.o_x = rx(a0); p.o_y = ry(a0);
    p.zx = (float)ax[2]; p.zy = (float)ay[2]; p.zz = (float)az[2]; p.z0 = (float)a0[2];
    return MCT_OK;
}

int mct_tv_weights(const mct_geom* g, const float* x, float beta, float* wr, void* stream) {
    MCT_REQUIRE(g && x && wr && x != wr && g->nx >= 1 && g->nz >= 1, "mct_tv_weights: bad arguments");
    tv_weights_kernel<<<ew_grid(vol_elems(*g)), 256, 0, as_stream(stream)>>>(g->nx, g->nz, beta, x, wr);
    return launched("tv_weights_kernel");
}

int mct_admm_shrink(const mct_geom* g, const float* x, float rho, float threshold, float* vy, float* vx, float* py,
                    float* px, void* stream) {
    MCT_REQUIRE(g && x && vy && vx && py && px && g->nx >= 1 && g->nz >= 1 && rho != 0.0f,
                "mct_admm_shrink: bad arguments");
    admm_shrink_kernel<<<ew_grid(vol_elems(*g)), 256, 0, as_stream(stream)>>>(g->nx, g->nz, x, rho, threshold, vy, vx,
                                                                             py, px);
    return launched("admm_shrink_kernel");
}

int mct_admm_rhs(const mct_geom* g, const float* bpb, const float* vy, const float* vx, const float* py,
                 const float* px, float rho, float* out, void* stream) {
    MCT_REQUIRE(g && bpb && vy && vx && py && px && out && g->nx >= 1 && g->nz >= 1, "mct_admm_rhs: bad arguments");
    admm_rhs_kernel<<<ew_grid(vol_elems(*g)), 256, 0, as_stream(stream)>>>(g->nx, g->nz, bpb, vy, vx, py, px, rho,
                                                                          out);
    return launched("admm_rhs_kernel");
}

int mct_dtwd(const mct_geom* g, const float* x, const float* wr, float s, const float* out_in, float a, float* out,
             void* stream) {
    MCT_REQUIRE(g && x && wr && out && out != x && out != wr && g->nx >= 1 && g->nz >= 1, "mct_dtwd: bad arguments");
    MCT_REQUIRE(a == 0.0f || out_in, "mct_dtwd: out_in is NULL");
    dtwd_kernel<false><<<ew_grid(vol_elems(*g)), 256, 0, as_stream(stream)>>>(g->nx, g->nz, x, wr, s, out_in, a, out,
                                                                             nullptr);
    return launched("dtwd_kernel");
}

int mct_dtwd_dot(const mct_geom* g, const float* x, const float* wr, float s, const float* out_in, float a, float* out,
                 double* partials, double* dot, void* stream) {
    MCT_REQUIRE(g && x && wr && out && partials && dot && out != x && out != wr && g->nx >= 1 && g->nz >= 1,
                "mct_dtwd_dot: bad arguments");
    MCT_REQUIRE(a == 0.0f || out_in, "mct_dtwd_dot: out_in is NULL");
    static_assert(RED_THREADS == 256, "dtwd_kernel<true> reduces over blocks of 256 threads");
    cudaStream_t st = as_stream(stream);
    dtwd_kernel<true><<<RED_BLOCKS, RED_THREADS, 0, st>>>(g->nx, g->nz, x, wr, s, out_in, a, out, partials);
    MCT_TRY(launched("dtwd_kernel"));
    finish_sum_kernel<<<1, RED_THREADS, 0, st>>>(partials, RED_BLOCKS, dot);
    return launched("finish_sum_kernel");
}

size_t mct_reduce_scratch_size(void) { return (size_t)RED_BLOCKS * sizeof(double); }

int mct_tv_penalty(const mct_geom* g, const float* x, float beta, double* partials, double* result, void* stream) {
    MCT_REQUIRE(g && x && partials && result, "mct_tv_penalty: bad arguments");
    cudaStream_t s = as_stream(stream);
    tv_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(g->nx, g->nz, beta, x, partials);
    MCT_TRY(launched("tv_partial_kernel"));
    finish_sum_kernel<<<1, RED_THREADS, 0, s>>>(partials, RED_BLOCKS, result);
    return launched("finish_sum_kernel");
}

int mct_dot_f64(const float* a, const float* b, int64_t n, double* partials, double* result, void* stream) {
    MCT_REQUIRE(a && b && partials && result && n >= 0, "mct_dot_f64: bad arguments");
    cudaStream_t s = as_stream(stream);
    dot_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, b, n, partials);
    MCT_TRY(launched("dot_partial_kernel"));
    finish_sum_kernel<<<1, RED_THREADS, 0, s>>>(partials, RED_BLOCKS, result);
    return launched("finish_sum_kernel");
}

int mct_cgls_update(int64_t n, const double* rr, const double* dq, float* x, float* r, const float* d, const float* q,
                    double* partials, double* rr_new, void* stream) {
    MCT_REQUIRE(rr && dq && x && r && d && q && partials && rr_new && n >= 0, "mct_cgls_update: bad arguments");
    cudaStream_t s = as_stream(stream);
    cgls_update_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, rr, dq, x, r, d, q, partials);
    MCT_TRY(launched("cgls_update_kernel"));
    finish_sum_kernel<<<1, RED_THREADS, 0, s>>>(partials, RED_BLOCKS, rr_new);
    return launched("finish_sum_kernel");
}

int mct_cgls_direction(int64_t n, const double* rr, const double* rr_new, const float* r, float* d, void* stream) {
    MCT_REQUIRE(rr && rr_new && r && d && n >= 0, "mct_cgls_direction: bad arguments");
    cgls_direction_kernel<<<ew_grid(n), 256, 0, as_stream(stream)>>>(n, rr, rr_new, r, d);
    return launched("cgls_direction_kernel");
}

// ---- the same vector operations on float32 or bf16 volumes (bf16 iterate storage)

#define MCT_VEC_DTYPE(who, dt) MCT_REQUIRE((dt) == MCT_F32 || (dt) == MCT_BF16, "%s: vector dtype must be MCT_F32 or MCT_BF16", who)

int mct_tv_weights_t(const mct_geom* g, const void* x, int32_t x_dtype, float beta, float* wr, void* stream) {
    MCT_REQUIRE(g && x && wr && x != (const void*)wr && g->nx >= 1 && g->nz >= 1, "mct_tv_weights_t: bad arguments");
    MCT_VEC_DTYPE("mct_tv_weights_t", x_dtype);
    cudaStream_t s = as_stream(stream);
    if (x_dtype == MCT_F32)
        tv_weights_kernel<<<ew_grid(vol_elems(*g)), 256, 0, s>>>(g->nx, g->nz, beta, static_cast<const float*>(x), wr);
    else
        tv_weights_kernel<<<ew_grid(vol_elems(*g)), 256, 0, s>>>(g->nx, g->nz, beta,
                                                                 static_cast<const __nv_bfloat16*>(x), wr);
    return launched("tv_weights_kernel");
}

int mct_dtwd_t(const mct_geom* g, const void* x, const float* wr, float s, const void* out_in, float a, void* out,
               int32_t vec_dtype, double* partials, double* dot, void* stream) {
    MCT_REQUIRE(g && x && wr && out && out != x && out != (const void*)wr && g->nx >= 1 && g->nz >= 1,
                "mct_dtwd_t: bad arguments");
    MCT_REQUIRE(a == 0.0f || out_in, "mct_dtwd_t: out_in is NULL");
    MCT_REQUIRE((partials == nullptr) == (dot == nullptr), "mct_dtwd_t: partials and dot go together");
    MCT_VEC_DTYPE("mct_dtwd_t", vec_dtype);
    cudaStream_t st = as_stream(stream);
    const bool with_dot = dot != nullptr;
    const int grid = with_dot ? RED_BLOCKS : ew_grid(vol_elems(*g));
    if (vec_dtype == MCT_F32) {
        auto xx = static_cast<const float*>(x);
        auto oi = static_cast<const float*>(out_in);
        auto oo = static_cast<float*>(out);
        if (with_dot) dtwd_kernel<true, float><<<grid, 256, 0, st>>>(g->nx, g->nz, xx, wr, s, oi, a, oo, partials);
        else dtwd_kernel<false, float><<<grid, 256, 0, st>>>(g->nx, g->nz, xx, wr, s, oi, a, oo, nullptr);
    } else {
        auto xx = static_cast<const __nv_bfloat16*>(x);
        auto oi = static_cast<const __nv_bfloat16*>(out_in);
        auto oo = static_cast<__nv_bfloat16*>(out);
        if (with_dot) dtwd_kernel<true, __nv_bfloat16><<<grid, 256, 0, st>>>(g->nx, g->nz, xx, wr, s, oi, a, oo, partials);
        else dtwd_kernel<false, __nv_bfloat16><<<grid, 256, 0, st>>>(g->nx, g->nz, xx, wr, s, oi, a, oo, nullptr);
    }
    MCT_TRY(launched("dtwd_kernel"));
    if (!with_dot) return MCT_OK;
    finish_sum_kernel<<<1, RED_THREADS, 0, st>>>(partials, RED_BLOCKS, dot);
    return launched("finish_sum_kernel");
}

int mct_dot_f64_t(const void* a, const void* b, int64_t n, int32_t dtype, double* partials, double* result,
                  void* stream) {
    MCT_REQUIRE(a && b && partials && result && n >= 0, "mct_dot_f64_t: bad arguments");
    MCT_VEC_DTYPE("mct_dot_f64_t", dtype);
    cudaStream_t s = as_stream(stream);
    if (dtype == MCT_F32)
        dot_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(static_cast<const float*>(a),
                                                              static_cast<const float*>(b), n, partials);
    else
        dot_partial_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(static_cast<const __nv_bfloat16*>(a),
                                                              static_cast<const __nv_bfloat16*>(b), n, partials);
    MCT_TRY(launched("dot_partial_kernel"));
    finish_sum_kernel<<<1, RED_THREADS, 0, s>>>(partials, RED_BLOCKS, result);
    return launched("finish_sum_kernel");
}

int mct_cgls_update_t(int64_t n, int32_t dtype, const double* rr, const double* dq, void* x, void* r, const void* d,
                      const void* q, double* partials, double* rr_new, void* stream) {
    MCT_REQUIRE(rr && dq && x && r && d && q && partials && rr_new && n >= 0, "mct_cgls_update_t: bad arguments");
    MCT_VEC_DTYPE("mct_cgls_update_t", dtype);
    cudaStream_t s = as_stream(stream);
    if (dtype == MCT_F32)
        cgls_update_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, rr, dq, static_cast<float*>(x), static_cast<float*>(r),
                                                              static_cast<const float*>(d),
                                                              static_cast<const float*>(q), partials);
    else
        cgls_update_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(
            n, rr, dq, static_cast<__nv_bfloat16*>(x), static_cast<__nv_bfloat16*>(r),
            static_cast<const __nv_bfloat16*>(d), static_cast<const __nv_bfloat16*>(q), partials);
    MCT_TRY(launched("cgls_update_kernel"));
    finish_sum_kernel<<<1, RED_THREADS, 0, s>>>(partials, RED_BLOCKS, rr_new);
    return launched("finish_sum_kernel");
}

int mct_cgls_direction_t(int64_t n, int32_t dtype, const double* rr, const double* rr_new, const void* r, void* d,
                         void* stream) {
    MCT_REQUIRE(rr && rr_new && r && d && n >= 0, "mct_cgls_direction_t: bad arguments");
    MCT_VEC_DTYPE("mct_cgls_direction_t", dtype);
    cudaStream_t s = as_stream(stream);
    if (dtype == MCT_F32)
        cgls_direction_kernel<<<ew_grid(n), 256, 0, s>>>(n, rr, rr_new, static_cast<const float*>(r),
                                                         static_cast<float*>(d));
    else
        cgls_direction_kernel<<<ew_grid(n), 256, 0, s>>>(n, rr, rr_new, static_cast<const __nv_bfloat16*>(r),
                                                         static_cast<__nv_bfloat16*>(d));
    return launched("cgls_direction_kernel");
}

}  // extern "C"
