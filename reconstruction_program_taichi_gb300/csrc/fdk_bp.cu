// Pixel-driven FDK / fan-beam backprojection (run_mgfbp.py:1062-1187).
//
// Design (sm_103a):
//   * one thread owns one (x, y) column and ZC consecutive slices, accumulating every
//     view in registers (the reference does a global read-modify-write per view);
//   * the filtered sinogram is pre-packed so that the 2x2 bilinear stencil of a
//     detector position is ONE 16-byte (f32) or 8-byte (bf16) load;
//   * per-view cos/sin/weight tables (and projection matrices) live in shared memory;
//   * the slices of a column share x and y (z runs along the image's i_z axis in the
//     axial view mode and along i_y in the coronal and sagittal ones, whose columns
//     the kernel takes over (i_x, i_z)), so u, the distance weight and the
//     magnification are evaluated once per (column, view) and v is an affine
//     function of the slice index.
// Voxels that project outside the detector in any view are written as 0, as in the
// reference (the view loop "breaks" with the voxel set to 0).  In the cone-beam
// path an off-detector row index is redirected to the packed operand's NaN row, so the
// voxel's sum becomes NaN and is written as 0 without any per-slice bookkeeping (a
// voxel whose sum is NaN because the sinogram itself holds NaN is written as 0 too,
// where the reference would return NaN).
#include <cmath>

#include "common.cuh"

namespace mct {
namespace {

constexpr int BP_TX = 32, BP_TY = 8, BP_ZC = 16, BP_VCHUNK = 1024;
constexpr int BP_WX = 4;  // columns along x per warp (32 / BP_WX along y)
static_assert(BP_TX % BP_WX == 0 && BP_TY % (32 / BP_WX) == 0, "warps tile the block");
static_assert(BP_ZC % 2 == 0, "the 16-bit axial loop takes slices in pairs");
// Minimum resident blocks per SM, i.e. a register budget of 65536 / (256 * minb) per
// thread.  The axial kernel needs enough registers to issue all BP_ZC stencil gathers
// of a view before their arithmetic (that hides the gather latency): measured at
// 512x512x256 / 1080 views, float32 stencils run fastest with 128 registers (2
// blocks), bf16 stencils with 80 (3 blocks).  The general modes use 2.
template <int MODE, typename QT>
constexpr int bp_min_blocks() {
    return MODE == 0 && sizeof(QT) == 8 ? 3 : 2;
}

struct BpParams {
    int nx, nz, nu, nv, views, cone, curved;
    // the kernel's index frame: a thread owns column (ix, iy) with ix in [0, nx), iy in
    // [0, ncb), and slices iz in [0, nsl) at vol[iz * ss + iy * sb + ix].  Axial: (iy, iz)
    // are the image's (i_y, i_z); coronal and sagittal: the image's (i_z, i_y), so that
    // the slice axis is the one along z and x, y stay fixed per column
    int ncb, nsl;
    int64_t sb, ss;
    int view_begin, views_total, accumulate;  // view-chunked FBP (scan index of view 0, scan size)
    float sid, sdd, img_rot;
    float u0, inv_ustep;   // uidx = (u - u0) * inv_ustep
    float v0, kv;          // vidx = (mag*z - v0) * kv, kv = sign(v_step)/dv
    float div;             // redundancy factor
    // voxel centre of (ix, iy, iz) of the kernel's frame = P + ix*EX + iy*EY + iz*EZ (rotated)
    float px_x, px_y, px_z;  // EX
    float py_x, py_y, py_z;  // EY
    float pz_x, pz_y, pz_z;  // EZ
    float o_x, o_y, o_z;     // P
};

// Per-view table of a chunk of nvc views starting at jc: {cos b', sin b', weight, 0}
// with b' = b - img_rot and weight = delta-beta (run_mgfbp.py:1107-1111) x the
// redundancy factor x the float16 unscale.
__device__ __forceinline__ void fill_view_table(const BpParams& p, const float* __restrict__ angles, float4* tab,
                                                int jc, int nvc, int tid, int nthreads, float unscale) {
    for (int q = tid; q < nvc; q += nthreads) {
        const int jg = p.view_begin + jc + q;  // scan index (angles is the whole scan's table)
        const int vt = p.views_total;
        float s, c;
        sincosf(angles[jg] - p.img_rot, &s, &c);
        float db = (jg == vt - 1) ? fabsf(angles[vt - 1] - angles[0]) / (vt - 1) : fabsf(angles[jg + 1] - angles[jg]);
        tab[q] = make_float4(c, s, db * p.div * unscale, 0.0f);
    }
}

// MODE 0: cone beam in any view mode; flat or curved detector, no projection matrix
//         (u hoisted per column of the kernel's frame)
// MODE 1: fan beam in the coronal or sagittal view mode (per-voxel u)
// MODE 3: projection matrix geometry in any view mode (per-column matrix rows)
template <int MODE, bool CONE, typename QT, typename PT>
__global__ void __launch_bounds__(BP_TX* BP_TY, bp_min_blocks<MODE, QT>())
fdk_bp_kernel(BpParams p, const float* __restrict__ angles, const float* __restrict__ pmat,
              const void* __restrict__ packed, float* __restrict__ vol, const uint32_t* __restrict__ f16_max) {
    // views per chunk of the shared tables; with projection matrices the chunk's 3x4
    // matrices are staged too (12 floats a view), in chunks of a quarter the size
    constexpr int VCH = MODE == 3 ? BP_VCHUNK / 4 : BP_VCHUNK;
    __shared__ float4 tab[VCH];  // {cos b, sin b, dbeta*div, unused}
    __shared__ __align__(16) float pms[MODE == 3 ? 12 * VCH : 4];
    const int tid = threadIdx.y * BP_TX + threadIdx.x;
    // A warp is 4 columns along x x 8 along y of the block's 32 x 8: for one view its
    // columns project onto fewer detector columns than a row of 32 (about 4|sin| + 8|cos|
    // + 1 against 32|sin| + 1), so each gather touches fewer L1 lines.  At 512x512x256 /
    // 1080 views: 52.19 -> 50.22 ms (float32), 49.07 -> 47.17 ms (bf16); warps of 16 x 2
    // 51.62 / 48.50, 8 x 4 50.78 / 47.70; blocks of 16 x 16 or 8 x 32 no better.
    const int warp = tid >> 5, lane = tid & 31;
    const int ix = blockIdx.x * BP_TX + (warp % (BP_TX / BP_WX)) * BP_WX + (lane % BP_WX);
    const int iy = blockIdx.y * BP_TY + (warp / (BP_TX / BP_WX)) * (32 / BP_WX) + lane / BP_WX;
    const int zb = blockIdx.z * BP_ZC;
    const bool active = ix < p.nx && iy < p.ncb;
    const int nq = p.nu - 1;  // packed columns; packed rows per view: nv (cone: row nv-1 is NaN)

    // voxel centres of the ZC slices of this column: c_k = c0 + k * dc
    const float c0x = p.o_x + ix * p.px_x + iy * p.py_x + zb * p.pz_x;
    const float c0y = p.o_y + ix * p.px_y + iy * p.py_y + zb * p.pz_y;
    const float c0z = p.o_z + ix * p.px_z + iy * p.py_z + zb * p.pz_z;

    float acc[BP_ZC];
#pragma unroll
    for (int k = 0; k < BP_ZC; ++k) acc[k] = 0.0f;
    uint32_t dead = 0;  // bit k: slice zb+k projected off the detector in some view

    // float16 operands hold values scaled by 2^e: fold 2^-e (exact) into the view weight
    const float unscale = IsF16<QT>::value ? ldexpf(1.0f, -f16_scale_exp(*f16_max)) : 1.0f;
    for (int jc = 0; jc < p.views; jc += VCH) {
        const int nvc = min(VCH, p.views - jc);
        __syncthreads();
        fill_view_table(p, angles, tab, jc, nvc, tid, BP_TX * BP_TY, unscale);
        if (MODE == 3) {
            const float* src = pmat + 12 * (int64_t)(p.view_begin + jc);
            for (int q = tid; q < 12 * nvc; q += BP_TX * BP_TY) pms[q] = __ldg(src + q);
        }
        __syncthreads();
        if (!active || dead == 0xffffffffu) continue;

        for (int q = 0; q < nvc; ++q) {
            const int j = jc + q;
            const float4 tb = tab[q];
            const float cb = tb.x, sb = tb.y;
            if (MODE == 0) {
                // u is shared by the whole column (cone beam: axial fan beam has its own kernel)
                static_assert(MODE != 0 || CONE, "MODE 0 is the cone-beam kernel");
                const float L = p.sid - c0x * cb - c0y * sb;
                const float t = -c0x * sb + c0y * cb;
                const float rL = 1.0f / L;  // one reciprocal for the magnification and the flat distance weight
                const float mag = p.sdd * rL;
                const float u = p.curved ? p.sdd * atan2f(t, L) : mag * t;
                const float ui = (u - p.u0) * p.inv_ustep;
                if (!(ui >= 0.0f && ui + 1.0f <= (float)(p.nu - 1))) {  // NaN counts as off-detector
                    dead = 0xffffffffu;
                    break;
                }
                const float uf = floorf(ui);
                const float ru = ui - uf;
                const int uc = (int)uf;
                const float dw = p.curved ? 1.0f / (L * L + t * t) : rL * rL;
                const float w = (p.sid * dw) * tb.z;
                const float vA = (mag * c0z - p.v0) * p.kv;
                const float vB = (mag * p.pz_z) * p.kv;
                const QT* base = reinterpret_cast<const QT*>(packed) + (int64_t)j * p.nv * nq + uc;
                const float2 ru2 = make_float2(ru, ru);
                const unsigned nan_row = (unsigned)(p.nv - 1);
                if constexpr (sizeof(QT) == 8) {
                    // 16-bit operands: slices in pairs, row index and weight as f32x2
                    // (the same values; at 512x512x256 / 1080 views bf16 48.9 ms
                    // against 49.7, float32 53.6 against 52.3, so float32 keeps the
                    // scalar loop)
                    const float2 vA2 = make_float2(vA, vA), vB2 = make_float2(vB, vB);
#pragma unroll
                    for (int k = 0; k < BP_ZC; k += 2) {
                        const float2 vi = __ffma2_rn(make_float2((float)k, (float)(k + 1)), vB2, vA2);
                        const float vf0 = floorf(vi.x), vf1 = floorf(vi.y);
                        const unsigned vr0 = min((unsigned)(int)vf0, nan_row);
                        const unsigned vr1 = min((unsigned)(int)vf1, nan_row);
                        const float2 rv = __fadd2_rn(vi, make_float2(-vf0, -vf1));
                        float2 lo0, hi0, lo1, hi1;
                        Quad<QT>::load(base + vr0 * (unsigned)nq, lo0, hi0);
                        Quad<QT>::load(base + vr1 * (unsigned)nq, lo1, hi1);
                        const float2 s0 = __ffma2_rn(ru2, hi0, lo0), s1 = __ffma2_rn(ru2, hi1, lo1);
                        acc[k] = fmaf(w, fmaf(rv.x, s0.y, s0.x), acc[k]);
                        acc[k + 1] = fmaf(w, fmaf(rv.y, s1.y, s1.x), acc[k + 1]);
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < BP_ZC; ++k) {
                        const float vi = fmaf((float)k, vB, vA);
                        const float vf = floorf(vi);
                        // rows outside [0, nv-2] (negative ones wrap around) read the NaN row
                        const unsigned vr = min((unsigned)(int)vf, nan_row);
                        const float rv = vi - vf;
                        float2 lo, hi;
                        Quad<QT>::load(base + vr * (unsigned)nq, lo, hi);
                        const float2 s2 = __ffma2_rn(ru2, hi, lo);
                        acc[k] = fmaf(w, fmaf(rv, s2.y, s2.x), acc[k]);
                    }
                }
            } else if (MODE == 3) {
                // Projection matrices: in the kernel's frame x and y are fixed per column, so
                // the matrix rows are affine in the slice index and the distance weight does
                // not depend on z.  An untilted trajectory has no z term in the u and depth
                // rows (P2 = P10 = 0 up to rounding left by the matrix processing): when
                // 16 |B| < 2^-26 |A| for both, fmaf(k, B, A) rounds to A for every slice, so
                // u and the magnification are the column's (as in MODE 0) and taking them
                // once gives exactly the per-slice result.
                const float4* P = reinterpret_cast<const float4*>(pms + 12 * q);  // the view's matrix, staged
                const float4 r0 = P[0], r1 = P[1], r2 = P[2];
                const float P0 = r0.x, P1 = r0.y, P2 = r0.z, P3 = r0.w;
                const float P4 = r1.x, P5 = r1.y, P6 = r1.z, P7 = r1.w;
                const float P8 = r2.x, P9 = r2.y, P10 = r2.z, P11 = r2.w;
                const float dz = p.pz_z;
                const float Au = P0 * c0x + P1 * c0y + P2 * c0z + P3, Bu = P2 * dz;
                const float Av = P4 * c0x + P5 * c0y + P6 * c0z + P7, Bv = P6 * dz;
                const float Aw = P8 * c0x + P9 * c0y + P10 * c0z + P11, Bw = P10 * dz;
                const float L = p.sid - c0x * cb - c0y * sb;
                const float t = -c0x * sb + c0y * cb;
                const float dw = p.curved ? 1.0f / (L * L + t * t) : 1.0f / (L * L);
                const float w = (p.sid * dw) * tb.z;
                const unsigned nan_row = (unsigned)(p.nv - 1);  // rows outside [0, nv-2] read the NaN row
                const QT* view = reinterpret_cast<const QT*>(packed) + (int64_t)j * p.nv * nq;
                const float tiny = 0x1p-26f / (float)BP_ZC;
                if (fabsf(Bu) <= tiny * fabsf(Au) && fabsf(Bw) <= tiny * fabsf(Aw)) {
                    const float mag = 1.0f / Aw;
                    const float ui = Au * mag;
                    if (!(ui >= 0.0f && ui + 1.0f <= (float)(p.nu - 1))) {  // NaN counts as off-detector
                        dead = 0xffffffffu;
                        break;
                    }
                    const float uf = floorf(ui);
                    const float ru = ui - uf;
                    const QT* base = view + (int)uf;
                    const float2 ru2 = make_float2(ru, ru);
#pragma unroll
                    for (int k = 0; k < BP_ZC; ++k) {
                        const float vi = fmaf((float)k, Bv, Av) * mag;  // as in the per-slice branch
                        const float vf = floorf(vi);
                        const unsigned vr = min((unsigned)(int)vf, nan_row);
                        const float rv = vi - vf;
                        float2 lo, hi;
                        Quad<QT>::load(base + vr * (unsigned)nq, lo, hi);
                        const float2 s2 = __ffma2_rn(ru2, hi, lo);
                        acc[k] = fmaf(w, fmaf(rv, s2.y, s2.x), acc[k]);
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < BP_ZC; ++k) {
                        if ((dead >> k) & 1u) continue;
                        const float fk = (float)k;
                        const float mag = 1.0f / fmaf(fk, Bw, Aw);
                        const float ui = fmaf(fk, Bu, Au) * mag;
                        if (!(ui >= 0.0f && ui + 1.0f <= (float)(p.nu - 1))) {
                            dead |= 1u << k;
                            continue;
                        }
                        const float uf = floorf(ui);
                        const float ru = ui - uf;
                        const float vi = fmaf(fk, Bv, Av) * mag;
                        const float vf = floorf(vi);
                        const unsigned vr = min((unsigned)(int)vf, nan_row);
                        const float rv = vi - vf;
                        float2 lo, hi;
                        Quad<QT>::load(view + vr * (unsigned)nq + (int)uf, lo, hi);
                        const float2 s2 = __ffma2_rn(make_float2(ru, ru), hi, lo);
                        acc[k] = fmaf(w, fmaf(rv, s2.y, s2.x), acc[k]);
                    }
                }
            } else {
                // MODE 1 (fan beam, coronal or sagittal view mode): the voxel moves by
                // (pz_x, pz_y) per slice, so L and t are affine in k; slice k reads
                // detector row zb + k
                static_assert(MODE != 1 || !CONE, "cone beam takes MODE 0 or 3 in every view mode");
                const float L0 = p.sid - c0x * cb - c0y * sb, dL = -(p.pz_x * cb + p.pz_y * sb);
                const float t0 = -c0x * sb + c0y * cb, dt = -p.pz_x * sb + p.pz_y * cb;
#pragma unroll
                for (int k = 0; k < BP_ZC; ++k) {
                    if (zb + k >= p.nsl || (dead >> k) & 1u) continue;
                    const float L = fmaf((float)k, dL, L0);
                    const float t = fmaf((float)k, dt, t0);
                    const float rL = 1.0f / L;  // one reciprocal for the magnification and the flat distance weight
                    const float mag = p.sdd * rL;
                    const float u = p.curved ? p.sdd * atan2f(t, L) : mag * t;
                    const float ui = (u - p.u0) * p.inv_ustep;
                    if (!(ui >= 0.0f && ui + 1.0f <= (float)(p.nu - 1))) {
                        dead |= 1u << k;
                        continue;
                    }
                    const float uf = floorf(ui);
                    const float ru = ui - uf;
                    const int uc = (int)uf;
                    const float dw = p.curved ? 1.0f / (L * L + t * t) : rL * rL;
                    const float w = (p.sid * dw) * tb.z;
                    const float2 pr = Pair<PT>::load(reinterpret_cast<const PT*>(packed) + ((int64_t)j * p.nv + zb + k) * nq + uc);
                    acc[k] = fmaf(w, fmaf(ru, pr.y, pr.x), acc[k]);
                }
            }
        }
    }
    if (!active) return;
    float* out = vol + (int64_t)zb * p.ss + (int64_t)iy * p.sb + ix;
#pragma unroll
    for (int k = 0; k < BP_ZC; ++k) {
        if (zb + k < p.nsl) {
            const bool off_detector = ((dead >> k) & 1u) || acc[k] != acc[k];
            if (p.accumulate)  // a voxel off the detector in any chunk stays NaN until mct_fdk_bp_finish
                out[(int64_t)k * p.ss] = off_detector ? __int_as_float(0x7fffffff) : out[(int64_t)k * p.ss] + acc[k];
            else
                out[(int64_t)k * p.ss] = off_detector ? 0.0f : acc[k];
        }
    }
}

__global__ void nan_to_zero_kernel(int64_t n, float* __restrict__ v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (v[i] != v[i]) v[i] = 0.0f;
}

// Axial fan beam (one detector row per slice, run_mgfbp.py:1183-1187).  A 2D image
// has few voxels (256^2 at 720 views: 256 blocks of the kernel above, under two per
// SM, each thread walking every view), so here the views of a column are split over
// FB_G threads: block (32 x-voxels, FB_G view groups) for one image row and ZC slices
// (1 for a single slice, else 8), thread g taking views g, g + FB_G, ...  The group
// sums are added in a fixed order through shared memory (deterministic), and a column
// is off the detector if any group saw it off.  A view that sees the column off the
// detector does not stop the loop (its index is clamped and the column's result is
// discarded), so independent views can overlap; 1/L is taken once per view.
constexpr int FB_G = 8;
template <int ZC, typename PT>
__global__ void __launch_bounds__(32 * FB_G)
fdk_bp_fan_kernel(BpParams p, const float* __restrict__ angles, const void* __restrict__ packed,
                  float* __restrict__ vol, const uint32_t* __restrict__ f16_max) {
    static_assert(ZC <= FB_G, "each of the first ZC view groups finishes one slice");
    __shared__ float4 tab[BP_VCHUNK];
    __shared__ float part[FB_G][ZC][32];
    __shared__ int dead_g[FB_G][32];
    const int tx = threadIdx.x, g = threadIdx.y;
    const int ix = blockIdx.x * 32 + tx;
    const int iy = blockIdx.y;
    const int zb = blockIdx.z * ZC;
    const int tid = g * 32 + tx;
    const bool active = ix < p.nx;
    const int nq = p.nu - 1;
    const float c0x = p.o_x + ix * p.px_x + iy * p.py_x;
    const float c0y = p.o_y + ix * p.px_y + iy * p.py_y;
    float acc[ZC];
#pragma unroll
    for (int k = 0; k < ZC; ++k) acc[k] = 0.0f;
    bool dead = false;
    const float unscale = IsF16<PT>::value ? ldexpf(1.0f, -f16_scale_exp(*f16_max)) : 1.0f;
    const float umax = (float)(p.nu - 1);
    for (int jc = 0; jc < p.views; jc += BP_VCHUNK) {
        const int nvc = min(BP_VCHUNK, p.views - jc);
        __syncthreads();
        fill_view_table(p, angles, tab, jc, nvc, tid, 32 * FB_G, unscale);
        __syncthreads();
        if (!active || dead) continue;
        // views in flight per thread: a one-slice thread has one short dependent chain
        // per view (helical FBP, 140 slices of 512^2 x 720 views, bit-identical: 51.45
        // ms unrolled 2, 48.85 unrolled 4, 49.63 unrolled 8)
        constexpr int kViewUnroll = ZC == 1 ? 4 : 2;
#pragma unroll kViewUnroll
        for (int q = g; q < nvc; q += FB_G) {
            const int j = jc + q;
            const float4 tb = tab[q];
            const float cb = tb.x, sb = tb.y;
            const float L = p.sid - c0x * cb - c0y * sb;
            const float t = -c0x * sb + c0y * cb;
            const float r = 1.0f / L;
            const float mag = p.sdd * r;
            const float u = p.curved ? p.sdd * atan2f(t, L) : mag * t;
            const float ui = (u - p.u0) * p.inv_ustep;
            dead |= !(ui >= 0.0f && ui + 1.0f <= umax);  // NaN counts as off-detector
            const float uf = floorf(ui);
            const float ru = ui - uf;
            const int uc = min(max((int)uf, 0), p.nu - 2);
            const float dw = p.curved ? 1.0f / (L * L + t * t) : r * r;
            const float w = (p.sid * dw) * tb.z;
            const PT* base = reinterpret_cast<const PT*>(packed) + ((int64_t)j * p.nv + zb) * nq + uc;
#pragma unroll
            for (int k = 0; k < ZC; ++k) {
                if (ZC == 1 || zb + k < p.nz) {
                    const float2 pr = Pair<PT>::load(base + (int64_t)k * nq);
                    acc[k] = fmaf(w, fmaf(ru, pr.y, pr.x), acc[k]);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < ZC; ++k) part[g][k][tx] = acc[k];
    dead_g[g][tx] = dead;
    __syncthreads();
    const int k = g;  // the first ZC groups finish slice zb + g of their column
    if (!active || k >= ZC || zb + k >= p.nz) return;
    float sum = 0.0f;
    int any_dead = 0;
#pragma unroll
    for (int h = 0; h < FB_G; ++h) {
        sum += part[h][k][tx];
        any_dead |= dead_g[h][tx];
    }
    const bool off_detector = any_dead || sum != sum;
    float* out = vol + (int64_t)(zb + k) * p.nx * p.nx + (int64_t)iy * p.nx + ix;
    if (p.accumulate)  // a voxel off the detector in any chunk stays NaN until mct_fdk_bp_finish
        *out = off_detector ? __int_as_float(0x7fffffff) : *out + sum;
    else
        *out = off_detector ? 0.0f : sum;
}

template <int ZC>
void launch_bp_fan(const BpParams& p, const mct_geom* g, cudaStream_t s, const float* angles, const void* packed,
                   int dtype, float* vol, const uint32_t* f16_max) {
    dim3 grid((g->nx + 31) / 32, g->nx, (g->nz + ZC - 1) / ZC), block(32, FB_G);
    if (dtype == MCT_BF16)
        fdk_bp_fan_kernel<ZC, uint32_t><<<grid, block, 0, s>>>(p, angles, packed, vol, nullptr);
    else if (dtype == MCT_F16)
        fdk_bp_fan_kernel<ZC, h16x2><<<grid, block, 0, s>>>(p, angles, packed, vol, f16_max);
    else
        fdk_bp_fan_kernel<ZC, float2><<<grid, block, 0, s>>>(p, angles, packed, vol, nullptr);
}

template <int MODE, bool CONE>
void launch_bp(const BpParams& p, dim3 grid, dim3 block, cudaStream_t s, const float* angles, const float* pmat,
               const void* packed, int dtype, float* vol, const uint32_t* f16_max) {
    if (dtype == MCT_BF16)
        fdk_bp_kernel<MODE, CONE, uint2, uint32_t><<<grid, block, 0, s>>>(p, angles, pmat, packed, vol, nullptr);
    else if (dtype == MCT_F16)
        fdk_bp_kernel<MODE, CONE, h16x4, h16x2><<<grid, block, 0, s>>>(p, angles, pmat, packed, vol, f16_max);
    else
        fdk_bp_kernel<MODE, CONE, float4, float2><<<grid, block, 0, s>>>(p, angles, pmat, packed, vol, nullptr);
}

}  // namespace
}  // namespace mct

using namespace mct;

extern "C" int mct_fdk_bp(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype, float* vol,
                          void* stream) {
    MCT_TRY(check_geom(g, "mct_fdk_bp"));
    MCT_REQUIRE(t && t->angles && packed && vol, "mct_fdk_bp: NULL buffer");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16 || dtype == MCT_F16,
                "mct_fdk_bp: dtype must be MCT_F32, MCT_BF16 or MCT_F16");
    const bool cone = (g->flags & MCT_CONE) != 0;
    const bool pm = (g->flags & MCT_PMATRIX) != 0;
    MCT_REQUIRE(!pm || (cone && t->pmatrix), "mct_fdk_bp: projection matrices need cone beam and the table");
    MCT_REQUIRE(!cone || g->nv >= 2, "mct_fdk_bp: cone beam needs at least 2 detector rows");
    MCT_REQUIRE(cone || g->nz <= g->nv, "mct_fdk_bp: fan beam needs nz <= detector rows");
    MCT_REQUIRE(g->u_step != 0.0f, "mct_fdk_bp: zero detector spacing");
    MCT_REQUIRE((int64_t)g->nv * (g->nu - 1) < ((int64_t)1 << 31), "mct_fdk_bp: detector too large");
    BpParams p{};
    p.nx = g->nx; p.nz = g->nz; p.nu = g->nu; p.nv = g->nv; p.views = g->views;
    p.view_begin = g->view_begin;
    p.views_total = g->views_total > 0 ? g->views_total : g->views;
    p.accumulate = (g->flags & MCT_ACCUMULATE) != 0;
    p.cone = cone; p.curved = (g->flags & MCT_CURVED) != 0;
    p.sid = g->sid; p.sdd = g->sdd; p.img_rot = g->img_rot;
    p.u0 = g->u0; p.inv_ustep = (float)(1.0 / (double)g->u_step);
    p.v0 = g->v0;
    if (cone && !pm) {
        MCT_REQUIRE(g->v_step != 0.0f && g->dv != 0.0f, "mct_fdk_bp: zero row spacing");
        p.kv = (float)((g->v_step > 0 ? 1.0 : -1.0) / (double)g->dv);
    }
    p.div = (float)div_factor(*g);
    // voxel coordinates, run_mgfbp.py:1090-1104, as an affine map of (ix, iy, iz)
    const double nx = g->nx, nz = g->nz, px = g->px, pz = g->pz;
    const double cr = std::cos((double)g->img_rot), sr = std::sin((double)g->img_rot);
    double ax[3] = {0, 0, 0}, ay[3] = {0, 0, 0}, az[3] = {0, 0, 0}, a0[3] = {0, 0, 0};  // (xa, ya, z) per unit index
    if (g->view_mode == 1) {
        ax[0] = px; a0[0] = -px * (nx - 1) / 2.0 + g->cx;
        ay[1] = -px; a0[1] = px * (nx - 1) / 2.0 + g->cy;
        az[2] = pz; a0[2] = -(nz - 1) / 2.0 * pz + g->cz;
    } else if (g->view_mode == 2) {
        ax[0] = px; a0[0] = -px * (nx - 1) / 2.0 + g->cx;
        ay[2] = -px; a0[2] = px * (nx - 1) / 2.0 + g->cz;
        az[1] = -pz; a0[1] = (nz - 1) / 2.0 * pz + g->cy;
    } else {
        ay[2] = -px; a0[2] = px * (nx - 1) / 2.0 + g->cz;
        ax[1] = -px; a0[1] = px * (nx - 1) / 2.0 + g->cy;
        az[0] = pz; a0[0] = -(nz - 1) / 2.0 * pz + g->cx;
    }
    auto rot = [&](const double* a, float& x, float& y, float& z) {
        x = (float)(a[0] * cr + a[1] * sr);
        y = (float)(-a[0] * sr + a[1] * cr);
        z = (float)a[2];
    };
    // The kernel's frame.  In the coronal and sagittal view modes the image's i_y axis is
    // the one along z and its i_x, i_z axes lie in the (x, y) plane, so with cone beam the
    // kernel takes (i_x, i_z) as the column and i_y as the slice axis: x and y are then
    // fixed per column, as in the axial mode, and the same hoisted kernels apply (u, the
    // weight and the truncation test once per column and view, v affine in the slice).
    const int64_t plane = (int64_t)g->nx * g->nx;
    const bool permuted = cone && g->view_mode != 1;
    rot(ax, p.px_x, p.px_y, p.px_z);
    rot(permuted ? az : ay, p.py_x, p.py_y, p.py_z);
    rot(permuted ? ay : az, p.pz_x, p.pz_y, p.pz_z);
    rot(a0, p.o_x, p.o_y, p.o_z);
    p.ncb = permuted ? g->nz : g->nx;
    p.nsl = permuted ? g->nx : g->nz;
    p.sb = permuted ? plane : g->nx;
    p.ss = permuted ? g->nx : plane;
    dim3 block(BP_TX, BP_TY);
    dim3 grid((g->nx + BP_TX - 1) / BP_TX, (p.ncb + BP_TY - 1) / BP_TY, (p.nsl + BP_ZC - 1) / BP_ZC);
    MCT_REQUIRE(grid.y <= 65535 && grid.z <= 65535, "mct_fdk_bp: volume too large for the launch grid");
    cudaStream_t s = as_stream(stream);
    const uint32_t* fm = dtype == MCT_F16 ? f16_trailer(g, packed) : nullptr;
    if (pm) launch_bp<3, true>(p, grid, block, s, t->angles, t->pmatrix, packed, dtype, vol, fm);
    else if (cone) launch_bp<0, true>(p, grid, block, s, t->angles, nullptr, packed, dtype, vol, fm);
    else if (g->view_mode == 1) {
        MCT_REQUIRE(g->nx <= 65535, "mct_fdk_bp: fan beam images are at most 65535 pixels wide");
        if (g->nz == 1) launch_bp_fan<1>(p, g, s, t->angles, packed, dtype, vol, fm);
        else launch_bp_fan<8>(p, g, s, t->angles, packed, dtype, vol, fm);
    }
    else launch_bp<1, false>(p, grid, block, s, t->angles, nullptr, packed, dtype, vol, fm);
    return launched("fdk_bp_kernel");
}

extern "C" int mct_fdk_bp_finish(const mct_geom* g, float* vol, void* stream) {
    MCT_REQUIRE(g && vol && g->nx >= 1 && g->nz >= 1, "mct_fdk_bp_finish: bad arguments");
    const int64_t n = (int64_t)g->nz * g->nx * g->nx;
    const int64_t blocks = (n + 255) / 256;
    nan_to_zero_kernel<<<(int)(blocks < 152 * 32 ? blocks : 152 * 32), 256, 0, as_stream(stream)>>>(n, vol);
    return launched("nan_to_zero_kernel");
}
