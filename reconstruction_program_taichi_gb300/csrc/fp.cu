// Ray-driven trilinear forward projector, its exact adjoint, the effective ray map,
// binning/noise, and analytic ellipsoid projections.
//
// Reference kernels replaced: Mgfpj_v3.ForwardProjectionBilinear
// (run_mgfpj_v3.py:184-366), its masked copy in Mgfbp_ir
// (run_mgfbp_iterative_recon_IRN_CGLS.py:494-676), the effective-map agent (:679-833),
// BinSinogram / AddPossionNoise (run_mgfpj_v3.py:368-391).
//
// All views are projected in ONE launch (the reference launches once per view).
// A ray's sample positions are affine in the step index k, so each ray first clips
// its step range to the volume's bounding box (with a one-step margin) and then
// applies the reference's per-sample inside test exactly; samples outside the box
// contribute 0 in the reference too.
#include <cmath>
#include <type_traits>

#include "common.cuh"

namespace mct {
namespace {

struct FpParams {
    int nx, nz, nu, nv, views, K, cone, curved, pmat;
    float sid, sdd, cx, cy, cz;
    float stepvd, l_min, inv_px, inv_pz;
    float x0, y0, zoff;  // voxel (0,0) centre x, y; z0 = zoff + cz_view
    float zpv;
    // fp_kernel ray tiling: a block of 256 rays is 2^bcs detector columns x 2^vshift
    // views x 2^(8 - bcs - vshift) detector rows, a warp 2^wcs columns x 2^(5 - wcs)
    // of the block's (view, row) slots; blockIdx.y runs over 2^rs row tiles within
    // each view group (the block order is column tile, row tile, view group, row group)
    int vshift, bcs, wcs, rs;
};

struct Ray {
    float fx0, dfx, fy0, dfy, fz0, dfz;  // fractional voxel index = f0 + k*df
    int ks, ke;                          // clipped step range [ks, ke]
};

// Ray set-up shared by all ray kernels, following run_mgfpj_v3.py:221-324.
__device__ __forceinline__ bool setup_ray(const FpParams& p, int iu, int iv, int j, const float* __restrict__ angles,
                                          const float* __restrict__ u_arr, const float* __restrict__ v_arr,
                                          const float* __restrict__ czv, const float* __restrict__ pa,
                                          const float* __restrict__ pxs, bool clip_z, Ray& r) {
    float sb, cb;
    sincosf(angles[j], &sb, &cb);
    const float zj = p.zpv * (float)j;
    const float uval = u_arr[iu];
    float dx, dy;
    if (p.curved) {
        const float g = (-uval) / p.sdd;
        float sg, cg;
        sincosf(g, &sg, &cg);
        dx = -p.sdd * cg + p.sid;
        dy = -p.sdd * sg;
    } else {
        dx = -(p.sdd - p.sid);
        dy = uval;
    }
    const float dz = v_arr[iv] + zj;
    const float ex = dx - p.sid, ey = dy, ez = dz - zj;
    const float dist = sqrtf(ex * ex + ey * ey + ez * ez);
    float Ox, Oy, Oz, Dx, Dy, Dz;
    if (p.pmat) {
        float s0, c0;
        sincosf(angles[0], &s0, &c0);
        const float* A = pa + 9 * j;
        const float* xs = pxs + 3 * j;
        const float fu = (float)iu, fv = (float)iv;
        const float ax = A[0] * fu + A[1] * fv + A[2];
        const float ay = A[3] * fu + A[4] * fv + A[5];
        const float az = A[6] * fu + A[7] * fv + A[8];
        Ox = xs[0] * c0 - xs[1] * s0;
        Oy = xs[1] * c0 + xs[0] * s0;
        Oz = xs[2] + zj;
        Dx = (ax * c0 - ay * s0) / dist;
        Dy = (ay * c0 + ax * s0) / dist;
        Dz = az / dist;
    } else {
        const float ux = ex / dist, uy = ey / dist, uz = ez / dist;
        Ox = p.sid * cb;
        Oy = p.sid * sb;
        Oz = zj;
        Dx = ux * cb - uy * sb;
        Dy = uy * cb + ux * sb;
        Dz = uz;
    }
    const float z0 = p.zoff + (czv ? czv[j] : p.cz);
    r.fx0 = (Ox + p.l_min * Dx - p.x0) * p.inv_px;
    r.dfx = p.stepvd * Dx * p.inv_px;
    r.fy0 = (Oy + p.l_min * Dy - p.y0) * (-p.inv_px);
    r.dfy = p.stepvd * Dy * (-p.inv_px);
    r.fz0 = (Oz + p.l_min * Dz - z0) * p.inv_pz;
    r.dfz = p.stepvd * Dz * p.inv_pz;
    // clip k so that f in [0, n-1) on each axis (conservative by one step)
    float klo = -1.0f, khi = (float)p.K;
    auto clip = [&](float f0, float df, float n) -> bool {
        if (fabsf(df) < 1e-20f) return f0 >= 0.0f && f0 < n - 1.0f;
        float t1 = (0.0f - f0) / df, t2 = (n - 1.0f - f0) / df;
        klo = fmaxf(klo, fminf(t1, t2));
        khi = fminf(khi, fmaxf(t1, t2));
        return true;
    };
    bool any = clip(r.fx0, r.dfx, (float)p.nx) && clip(r.fy0, r.dfy, (float)p.nx);
    if (clip_z && p.cone) any = any && clip(r.fz0, r.dfz, (float)p.nz);
    if (!any || !(klo <= khi)) {
        r.ks = 0;
        r.ke = -1;
        return false;
    }
    r.ks = max(0, (int)floorf(klo) - 1);
    r.ke = min(p.K - 1, (int)ceilf(khi) + 1);
    return r.ks <= r.ke;
}

// Steps [kis, kie] whose sample lies at least 1e-3 voxel inside the box on every
// tested axis (and one more step in from both ends): for them the reference's inside
// test certainly passes, far beyond float rounding, so it can be skipped.
__device__ __forceinline__ void interior_range(const FpParams& p, const Ray& r, bool test_z, int& kis, int& kie) {
    const float eps = 1e-3f;
    float lo = -3.0e38f, hi = 3.0e38f;
    bool empty = false;
    auto axis = [&](float f0, float df, float n) {
        const float a = eps, b = n - 1.0f - eps;
        if (fabsf(df) < 1e-20f) {
            if (!(f0 >= a && f0 <= b)) empty = true;
            return;
        }
        const float t1 = (a - f0) / df, t2 = (b - f0) / df;
        lo = fmaxf(lo, fminf(t1, t2));
        hi = fminf(hi, fmaxf(t1, t2));
    };
    axis(r.fx0, r.dfx, (float)p.nx);
    axis(r.fy0, r.dfy, (float)p.nx);
    if (test_z) axis(r.fz0, r.dfz, (float)p.nz);
    lo = fmaxf(lo, (float)r.ks - 2.0f);
    hi = fminf(hi, (float)r.ke + 2.0f);
    if (empty || !(lo <= hi)) {
        kis = r.ke + 1;
        kie = r.ke;
        return;
    }
    kis = max(r.ks, (int)ceilf(lo) + 1);
    kie = min(r.ke, (int)floorf(hi) - 1);
    if (kis > kie) {
        kis = r.ke + 1;
        kie = r.ke;
    }
}

// Direction (in object x, y) along which neighbouring detector columns spread.
__device__ __forceinline__ bool spread_along_y(const FpParams& p, int j, const float* __restrict__ angles,
                                               const float* __restrict__ pa) {
    if (p.pmat) {
        float s0, c0;
        sincosf(angles[0], &s0, &c0);
        const float* A = pa + 9 * j;
        const float ex = A[0] * c0 - A[3] * s0, ey = A[3] * c0 + A[0] * s0;
        return fabsf(ey) > fabsf(ex);
    }
    float sb, cb;
    sincosf(angles[j], &sb, &cb);
    return fabsf(cb) > fabsf(sb);  // d(x, y)/du is (-sin b, cos b)
}

// Grid of every ray kernel: x = 32-column detector tiles, y = views, z = 8-row
// detector tiles.  Blocks are scheduled x, then y, then z, so the blocks resident at
// one time cover many views of the same detector rows; those rays cross only a thin
// z-slab of the volume, which then stays in L2 across views.  fp_kernel with copies
// instead takes tiles of 16 columns x 2^vshift consecutive views x 2^(4 - vshift)
// rows (x = column tiles, y = view groups, z = row tiles), each warp 4 columns x 8
// (view, row) slots; each ray's arithmetic is the same either way.
//
// One thread per ray (u, v) of view j.  vol is [z][y][x]; vol_t, when
// given, is the same volume as [z][x][y]: views whose detector columns spread along
// y read vol_t so that neighbouring rays touch consecutive addresses.  With ZP
// (cone beam, workspace given) the volume is read from copies zp_x ([z][y][x]) and
// zp_y ([z][x][y]): float32 quads (two adjacent 16-byte elements per cell reload) or
// 16-bit cells (the whole 2x2x2 trilinear cell in one 16-byte element), below.

// float32 quad copy, indexed in a (slow s, fast f) frame: (s, f) = (y, x) for views whose
// detector columns spread along x (copy cx, [z][y][x]) and (x, y) for the others (copy
// cy, [z][x][y]), so that neighbouring rays read neighbouring elements.  Element
// (z, s, f) holds the z-pairs of the voxel and of its neighbour along s,
//   {V(z, s, f), V(z+1, s, f), V(z, s+1, f), V(z+1, s+1, f)}    (16 bytes),
// and the neighbour along f is the next element: a cell reload is two adjacent 16-byte
// loads, and the f-differences are taken in registers (the same float32 subtraction a
// direct read would do).  Against a 32-byte element holding the whole cell (differences
// included) this halves the copies (32 instead of 64 bytes per voxel for both
// orientations), so twice the cells fit L1 and L2; with blocks of 8 consecutive views,
// whose rays cross nearly the same cells at the same step, the projector at
// 512x512x256 / 1080 views went 297.6 -> 267.3 ms (the 32-byte cells: 304-312 ms with
// 2-8 views per block, 297.6 with 8 rows of one view).
struct __align__(16) Quad16 {
    float v[4];
};

// bf16 cell copy: element (z, y, x) of either orientation holds the whole 2x2x2 cell
// whose lowest corner is voxel (z, y, x), as four bf16 pairs {lower, upper z-plane}:
//   .x = e00 = {V[z][y][x], V[z+1][y][x]}      .y = g00 = e01 - e00' (x+1 corner)
//   .z = e10 = {V[z][y+1][x], V[z+1][y+1][x]}  .w = g10 = e11 - e10' (x+1, y+1)
// (x, y as in the volume; e' is e rounded to bf16, so the x+1 corners are restored to
// the bf16 precision of the differences).  A reload is one 16-byte gather.
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&b);
}

// Resident blocks per SM that the register allocation of fp_kernel targets.  The
// float32 cone-beam path waits on L1 and needs its warps: with quad copies and the
// 16 x 16-view tiles, 5 blocks (48 registers) take 237.2 ms at 512x512x256 / 1080
// views, 4 blocks 240.2 ms (8-view tiles: 5 blocks 267.3, 4 blocks 273.8, 6 blocks,
// 40 registers with spills, 317.1); the fan-beam path keeps 40 registers (6 blocks).
// The 16-bit paths are issue-bound and gain from registers: 1 (80 registers, 3 blocks
// of 256) gives bf16 237.4 ms against 254.9 with 5 blocks (8-view tiles), float16
// 274.4 against 291.7; with the 16-column tiles 1 and 2 blocks are equal (224.0).
template <bool CONE, typename ZT>
struct FpMinBlocks {
    static constexpr int value = (std::is_same<ZT, uint4>::value || std::is_same<ZT, h16x8>::value) ? 1
                                 : CONE                                                             ? 5
                                                                                                    : 6;
};

template <bool CONE, bool ZP, typename ZT>
__global__ void __launch_bounds__(256, FpMinBlocks<CONE, ZT>::value)
fp_kernel(FpParams p, const float* __restrict__ angles, const float* __restrict__ u_arr,
          const float* __restrict__ v_arr, const float* __restrict__ czv, const float* __restrict__ pa,
          const float* __restrict__ pxs, const float* __restrict__ vol, const float* __restrict__ vol_t,
          const ZT* __restrict__ zp_x, const ZT* __restrict__ zp_y, const float* __restrict__ mask,
          float* __restrict__ sgm, const uint32_t* __restrict__ f16_max) {
    // ray of this thread: column tx and (view, row) slot ty of the block's tile, warps
    // of 2^wcs columns x 2^(5 - wcs) slots
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int gpr = p.bcs - p.wcs;  // log2 of the warps across the tile's columns
    const int tx = ((warp & ((1 << gpr) - 1)) << p.wcs) + (lane & ((1 << p.wcs) - 1));
    const int ty = ((warp >> gpr) << (5 - p.wcs)) + (lane >> p.wcs);
    const int iu = (blockIdx.x << p.bcs) + tx;
    const int vs = p.vshift;
    const int vg = blockIdx.y >> p.rs, rsub = blockIdx.y & ((1 << p.rs) - 1);  // view group, row tile in it
    const int iv = ((((int)blockIdx.z << p.rs) + rsub) << (8 - p.bcs - vs)) + (ty >> vs);
    const int j = (vg << vs) + (ty & ((1 << vs) - 1));
    if (iu >= p.nu || iv >= p.nv || j >= p.views) return;
    const int64_t oidx = ((int64_t)iv * p.views + j) * p.nu + iu;
    if (mask && mask[oidx] != 1.0f) {
        sgm[oidx] = 0.0f;
        return;
    }
    const int nx = p.nx;
    const bool tr = (ZP || vol_t != nullptr) && spread_along_y(p, j, angles, pa);
    // quad copies are addressed in their (slow, fast) frame: the ray's x and y swap for
    // the transposed copy, so the fast axis is always "x" below (both axes span
    // [0, nx - 1), so the clipping and inside tests are unchanged)
    constexpr bool kQuad = ZP && std::is_same<ZT, Quad16>::value;
    const float* __restrict__ V = tr ? vol_t : vol;
    const ZT* __restrict__ V2 = tr ? zp_y : zp_x;
    const int sx = (tr && !kQuad) ? nx : 1, sy = (tr && !kQuad) ? 1 : nx;
    const int plane = nx * nx;  // volumes below 2^31 voxels (checked on the host)
    Ray r;
    float acc = 0.0f;
    if (setup_ray(p, iu, iv, j, angles, u_arr, v_arr, czv, pa, pxs, true, r)) {
        if (kQuad && tr) {
            float t = r.fx0;
            r.fx0 = r.fy0;
            r.fy0 = t;
            t = r.dfx;
            r.dfx = r.dfy;
            r.dfy = t;
        }
        const float xmax = (float)(nx - 1), zmax = (float)(p.nz - 1);
        // Consecutive samples are 0.2 voxel diagonals apart, so most fall in the same
        // 2x2x2 cell as the previous one: the cell stays in registers (as corner values
        // and x-differences, lower and upper z-plane packed side by side) and is
        // reloaded only when the ray enters a new cell.
        int cell = -1;
        float2 e00 = make_float2(0.f, 0.f), e10 = e00, g00 = e00, g10 = e00;  // corners, x-differences
        auto load_cell = [&](int off) {
            if (off == cell) return;
            cell = off;
            if constexpr (kQuad) {
                const float4 q0 = __ldg(reinterpret_cast<const float4*>(V2 + off));
                const float4 q1 = __ldg(reinterpret_cast<const float4*>(V2 + off + 1));
                e00 = make_float2(q0.x, q0.y);
                e10 = make_float2(q0.z, q0.w);
                g00 = __fadd2_rn(make_float2(q1.x, q1.y), make_float2(-q0.x, -q0.y));
                g10 = __fadd2_rn(make_float2(q1.z, q1.w), make_float2(-q0.z, -q0.w));
            } else if constexpr (ZP && std::is_same<ZT, uint4>::value) {
                const uint4 q = __ldg(V2 + off);
                e00 = bf16x2_to_float2(q.x);
                g00 = bf16x2_to_float2(q.y);
                e10 = bf16x2_to_float2(q.z);
                g10 = bf16x2_to_float2(q.w);
            } else if constexpr (ZP && std::is_same<ZT, h16x8>::value) {
                const uint4 q = __ldg(reinterpret_cast<const uint4*>(V2 + off));
                e00 = h16x2_to_float2(q.x);
                g00 = h16x2_to_float2(q.y);
                e10 = h16x2_to_float2(q.z);
                g10 = h16x2_to_float2(q.w);
            } else {
                const float* b = V + off;
                const float a00 = __ldg(b), a01 = __ldg(b + sx), a10 = __ldg(b + sy), a11 = __ldg(b + sx + sy);
                float c00 = 0.f, c01 = 0.f, c10 = 0.f, c11 = 0.f;
                if (CONE) {
                    const float* c = b + plane;
                    c00 = __ldg(c); c01 = __ldg(c + sx); c10 = __ldg(c + sy); c11 = __ldg(c + sx + sy);
                }
                e00 = make_float2(a00, c00);
                e10 = make_float2(a10, c10);
                g00 = __fadd2_rn(make_float2(a01, c01), make_float2(-a00, -c00));
                g10 = __fadd2_rn(make_float2(a11, c11), make_float2(-a10, -c10));
            }
        };
        // lower (.x) and upper (.y) z-plane bilinear values in packed f32x2 FMAs; per
        // lane this is exactly fmaf(xw, a01 - a00, a00) etc.
        auto interp = [&](float xw, float yw, float zw) -> float {
            const float2 xw2 = make_float2(xw, xw), yw2 = make_float2(yw, yw);
            const float2 l0 = __ffma2_rn(xw2, g00, e00);
            const float2 l1 = __ffma2_rn(xw2, g10, e10);
            const float2 pl = __ffma2_rn(yw2, __fadd2_rn(l1, make_float2(-l0.x, -l0.y)), l0);
            return CONE ? fmaf(zw, pl.y - pl.x, pl.x) : pl.x;
        };
        auto sample = [&](int k, bool check) {
            const float fk = (float)k;
            const float fx = fmaf(fk, r.dfx, r.fx0);
            const float fy = fmaf(fk, r.dfy, r.fy0);
            const float xf = floorf(fx), yf = floorf(fy);
            bool ok = true;
            int xi = (int)xf, yi = (int)yf, zi;
            if (check) {
                ok = xf >= 0.0f && xf < xmax && yf >= 0.0f && yf < xmax;
                xi = min(max(xi, 0), nx - 2);
                yi = min(max(yi, 0), nx - 2);
            }
            const float xw = fx - xf, yw = fy - yf;
            float zw = 0.0f;
            if (CONE) {
                const float fz = fmaf(fk, r.dfz, r.fz0);
                const float zf = floorf(fz);
                zi = (int)zf;
                if (check) {
                    ok = ok && zf >= 0.0f && zf < zmax;
                    zi = min(max(zi, 0), p.nz - 2);
                }
                zw = fz - zf;
            } else {
                zi = iv;
            }
            const int off = zi * plane + yi * sy + xi * sx;
            load_cell(off);
            const float val = interp(xw, yw, zw);
            if (check) acc += ok ? val : 0.0f;
            else acc += val;
        };
        // Interior samples (at least 1e-3 voxel inside on every axis).  With copies
        // the floors come from adding M = 1.5 * 2^23 rounded toward -infinity (exactly
        // M + floor(f) for |f| < 2^22), on the FMA pipe instead of the conversion unit
        // (which otherwise limits the 16-bit kernels), and the x and y coordinates
        // travel as one f32x2 pair: position, floor and weight are three packed
        // operations for both axes.  The element offset is summed in unsigned arithmetic
        // (the bias terms wrap, the total is the offset, below 2^31).
        constexpr bool kRoundFloor = ZP && !std::is_same<ZT, float2>::value;
        const float M = 12582912.0f;
        const unsigned MB = 0x4B400000u;  // bit pattern of M
        const unsigned obias = CONE ? MB * (unsigned)(plane + sy + sx) : MB * (unsigned)(sy + sx) - (unsigned)(iv * plane);
        const float2 dxy = make_float2(r.dfx, r.dfy), fxy0 = make_float2(r.fx0, r.fy0);
        const float2 M2 = make_float2(M, M), nM2 = make_float2(-M, -M);
        auto sample_fast = [&](float fk) {
            const float2 f = __ffma2_rn(make_float2(fk, fk), dxy, fxy0);  // fractional indices x, y
            const float2 m = __fadd2_rd(f, M2);                            // M + floor(f)
            const float2 fl = __fadd2_rn(m, nM2);                          // floor(f), exact
            const float2 w = __fadd2_rn(f, make_float2(-fl.x, -fl.y));     // weights, exact
            unsigned off = (unsigned)__float_as_int(m.x) * (unsigned)sx + (unsigned)__float_as_int(m.y) * (unsigned)sy - obias;
            float zw = 0.0f;
            if (CONE) {
                const float fz = fmaf(fk, r.dfz, r.fz0);
                const float mz = __fadd_rd(fz, M);
                zw = fz - (mz - M);
                off += (unsigned)__float_as_int(mz) * (unsigned)plane;
            }
            load_cell((int)off);
            acc += interp(w.x, w.y, zw);
        };
        int kis, kie;
        interior_range(p, r, CONE, kis, kie);
        for (int k = r.ks; k < kis; ++k) sample(k, true);
        if constexpr (kRoundFloor) {
            float fk = (float)kis;
            // unrolled 4 times for float32 quads, twice for 16-bit cells (at 512x512x256 /
            // 1080 views: float32 237.4 ms against 239.6 with 2; bf16 215.7 against 222.1
            // with 4)
            constexpr int kUnroll = kQuad ? 4 : 2;
#pragma unroll kUnroll
            for (int k = kis; k <= kie; ++k, fk += 1.0f) sample_fast(fk);
        } else {
#pragma unroll 4
            for (int k = kis; k <= kie; ++k) sample(k, false);
        }
        for (int k = max(kie + 1, kis); k <= r.ke; ++k) sample(k, true);
    }
    if constexpr (IsF16<ZT>::value) acc *= ldexpf(1.0f, -f16_scale_exp(*f16_max));  // float16 cells hold v * 2^e
    sgm[oidx] = acc * p.stepvd;
}

// Largest |v| of the volume as float bits into *maxbits (zeroed by the caller).
template <typename TIN>
__global__ void vol_absmax_kernel(int64_t n, const TIN* __restrict__ v, uint32_t* __restrict__ maxbits) {
    uint32_t m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, __float_as_uint(ldv(v, i)) & 0x7fffffffu);
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, m);
}

// 16-bit cell copies (layout above; float16 cells hold v * 2^e, see f16_scale_exp): cx[z][y][x] and cy[z][x][y] both hold the cell at
// voxel (z, y, x); corners outside the volume are 0 (no in-volume sample uses them).
// 32x32 tiles, the transposed copy through shared memory.
template <bool F16, typename TIN = float>
__global__ void cell16_kernel(int nx, int nz, const TIN* __restrict__ v, uint4* __restrict__ cx,
                              uint4* __restrict__ cy, const uint32_t* __restrict__ f16_max) {
    __shared__ uint4 tile[32][33];
    const int64_t plane = (int64_t)nx * nx;
    const int z = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const float sc = F16 ? ldexpf(1.0f, f16_scale_exp(*f16_max)) : 1.0f;
    auto at = [&](int zz, int yy, int xx) -> float {
        return (zz < nz && yy < nx && xx < nx) ? ldv(v, zz * plane + (int64_t)yy * nx + xx) * sc : 0.0f;
    };
    auto rb = [](float a) {
        return F16 ? __half2float(__float2half_rn(a)) : __bfloat162float(__float2bfloat16_rn(a));
    };
    auto pk = [](float lo, float hi) { return F16 ? pack_h16x2(lo, hi) : pack_bf16x2(lo, hi); };
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int y = y0 + i, x = x0 + threadIdx.x;
        if (y < nx && x < nx) {
            const float a0 = rb(at(z, y, x)), a1 = rb(at(z + 1, y, x));
            const float c0 = rb(at(z, y + 1, x)), c1 = rb(at(z + 1, y + 1, x));
            uint4 q;
            q.x = pk(a0, a1);
            q.y = pk(at(z, y, x + 1) - a0, at(z + 1, y, x + 1) - a1);
            q.z = pk(c0, c1);
            q.w = pk(at(z, y + 1, x + 1) - c0, at(z + 1, y + 1, x + 1) - c1);
            cx[z * plane + (int64_t)y * nx + x] = q;
            tile[i][threadIdx.x] = q;
        }
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int x = x0 + i, y = y0 + threadIdx.x;
        if (y < nx && x < nx) cy[z * plane + (int64_t)x * nx + y] = tile[threadIdx.x][i];
    }
}

// float32 quad copies (layout at Quad16): cx[z][y][x] = {V[z][y][x], V[z+1][y][x],
// V[z][y+1][x], V[z+1][y+1][x]} (fast axis x) and cy[z][x][y] = {V[z][y][x],
// V[z+1][y][x], V[z][y][x+1], V[z+1][y][x+1]} (fast axis y); corners outside the volume
// are 0 (no in-volume sample uses them).  32x32 tiles, the transposed copy through
// shared memory.
template <typename TIN = float>
__global__ void quad32_kernel(int nx, int nz, const TIN* __restrict__ v, float4* __restrict__ cx,
                              float4* __restrict__ cy) {
    __shared__ float4 tile[32][33];
    const int64_t plane = (int64_t)nx * nx;
    const int z = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    auto at = [&](int zz, int yy, int xx) -> float {
        return (zz < nz && yy < nx && xx < nx) ? ldv(v, zz * plane + (int64_t)yy * nx + xx) : 0.0f;
    };
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int y = y0 + i, x = x0 + threadIdx.x;
        if (y < nx && x < nx) {
            const float a0 = at(z, y, x), a1 = at(z + 1, y, x);
            cx[z * plane + (int64_t)y * nx + x] = make_float4(a0, a1, at(z, y + 1, x), at(z + 1, y + 1, x));
            tile[i][threadIdx.x] = make_float4(a0, a1, at(z, y, x + 1), at(z + 1, y, x + 1));
        }
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int x = x0 + i, y = y0 + threadIdx.x;
        if (y < nx && x < nx) cy[z * plane + (int64_t)x * nx + y] = tile[threadIdx.x][i];
    }
}

// vt[z][x][y] = v[z][y][x], 32x32 tiles through shared memory.
__global__ void transpose_xy_kernel(int nx, int nz, const float* __restrict__ v, float* __restrict__ vt) {
    __shared__ float tile[32][33];
    const int64_t plane = (int64_t)nx * nx;
    const int z = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int y = y0 + i, x = x0 + threadIdx.x;
        if (y < nx && x < nx) tile[i][threadIdx.x] = v[z * plane + (int64_t)y * nx + x];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int x = x0 + i, y = y0 + threadIdx.x;
        if (y < nx && x < nx) vt[z * plane + (int64_t)x * nx + y] = tile[threadIdx.x][i];
    }
}

// 16-byte vector reduction (sm_90 and later): four float adds at one aligned address,
// one L2 atomic request instead of four.
__device__ __forceinline__ void red_add_v4(float* q, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(q), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Exact transpose of fp_kernel: every in-volume sample scatters its trilinear weights
// times the ray value into the volume.  CELLS: the corner sums go to a cell-space
// buffer instead (per cell of the 2x2x2 stencil its 8 corner sums, z-low 4 then
// z-high 4, each group ordered (x,y) (x+1,y) (x,y+1) (x+1,y+1); fan beam: the 4 of the
// slice), one or two 16-byte reductions per flush; adjoint_gather_kernel then sums
// each voxel's corner entries from the cells that contain it.
template <bool CELLS>
__global__ void __launch_bounds__(256)
fp_adjoint_kernel(FpParams p, const float* __restrict__ angles, const float* __restrict__ u_arr,
                  const float* __restrict__ v_arr, const float* __restrict__ czv, const float* __restrict__ pa,
                  const float* __restrict__ pxs, const float* __restrict__ sgm, const float* __restrict__ mask,
                  float* __restrict__ vol) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.z * blockDim.y + threadIdx.y;
    const int j = blockIdx.y;
    if (iu >= p.nu || iv >= p.nv) return;
    const int64_t oidx = ((int64_t)iv * p.views + j) * p.nu + iu;
    if (mask && mask[oidx] != 1.0f) return;
    const float yv = sgm[oidx] * p.stepvd;
    if (yv == 0.0f) return;
    Ray r;
    if (!setup_ray(p, iu, iv, j, angles, u_arr, v_arr, czv, pa, pxs, true, r)) return;
    const int nx = p.nx;
    const int plane = nx * nx;
    // The 8 corner weights of consecutive samples in the same cell are summed in
    // registers and scattered once when the ray leaves the cell.
    int cell = -1;
    float s00 = 0.f, s01 = 0.f, s10 = 0.f, s11 = 0.f, t00 = 0.f, t01 = 0.f, t10 = 0.f, t11 = 0.f;
    auto flush = [&]() {
        if (cell < 0) return;
        if (CELLS) {
            float* c = vol + (int64_t)cell * (p.cone ? 8 : 4);
            red_add_v4(c, s00, s01, s10, s11);
            if (p.cone) red_add_v4(c + 4, t00, t01, t10, t11);
            s00 = s01 = s10 = s11 = t00 = t01 = t10 = t11 = 0.f;
            return;
        }
        float* b = vol + cell;
        atomicAdd(b, s00);
        atomicAdd(b + 1, s01);
        atomicAdd(b + nx, s10);
        atomicAdd(b + nx + 1, s11);
        if (p.cone) {
            float* c = b + plane;
            atomicAdd(c, t00);
            atomicAdd(c + 1, t01);
            atomicAdd(c + nx, t10);
            atomicAdd(c + nx + 1, t11);
        }
        s00 = s01 = s10 = s11 = t00 = t01 = t10 = t11 = 0.f;
    };
    for (int k = r.ks; k <= r.ke; ++k) {
        const float fk = (float)k;
        const float fx = fmaf(fk, r.dfx, r.fx0);
        const float fy = fmaf(fk, r.dfy, r.fy0);
        const float xf = floorf(fx), yf = floorf(fy);
        if (!(xf >= 0.0f && xf + 1.0f < (float)nx && yf >= 0.0f && yf + 1.0f < (float)nx)) continue;
        const float xw = fx - xf, yw = fy - yf;
        int zi;
        float zw = 0.0f;
        if (p.cone) {
            const float fz = fmaf(fk, r.dfz, r.fz0);
            const float zf = floorf(fz);
            if (!(zf >= 0.0f && zf + 1.0f < (float)p.nz)) continue;
            zi = (int)zf;
            zw = fz - zf;
        } else {
            zi = iv;
        }
        const int off = zi * plane + (int)yf * nx + (int)xf;
        if (off != cell) {
            flush();
            cell = off;
        }
        const float wl = p.cone ? (1.0f - zw) * yv : yv;
        const float w00 = (1.0f - xw) * (1.0f - yw), w01 = xw * (1.0f - yw);
        const float w10 = (1.0f - xw) * yw, w11 = xw * yw;
        s00 += w00 * wl;
        s01 += w01 * wl;
        s10 += w10 * wl;
        s11 += w11 * wl;
        if (p.cone) {
            const float wh = zw * yv;
            t00 += w00 * wh;
            t01 += w01 * wh;
            t10 += w10 * wh;
            t11 += w11 * wh;
        }
    }
    flush();
}

// vol[z][y][x] += the corner entries of the (up to) 8 cells that contain voxel
// (z, y, x), in a fixed order.  C = 8 (cone beam) or 4 (fan beam: one slice per cell).
template <int C>
__global__ void __launch_bounds__(256)
adjoint_gather_kernel(int nx, int nz, const float* __restrict__ cells, float* __restrict__ vol) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= nx || y >= nx || z >= nz) return;
    const int64_t plane = (int64_t)nx * nx;
    const int64_t v = z * plane + (int64_t)y * nx + x;
    float acc = 0.0f;
#pragma unroll
    for (int dz = 0; dz < C / 4; ++dz) {
        if (z - dz < 0) continue;
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            if (y - dy < 0) continue;
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
                if (x - dx < 0) continue;
                const int64_t c = v - dz * plane - (int64_t)dy * nx - dx;
                acc += __ldg(cells + c * C + dz * 4 + dy * 2 + dx);
            }
        }
    }
    vol[v] += acc;
}

// Effective ray map, run_mgfbp_iterative_recon_IRN_CGLS.py:749-833.
__global__ void __launch_bounds__(256)
emap_kernel(FpParams p, const float* __restrict__ angles, const float* __restrict__ u_arr,
            const float* __restrict__ v_arr, const float* __restrict__ czv, const float* __restrict__ pa,
            const float* __restrict__ pxs, float* __restrict__ mask) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.z * blockDim.y + threadIdx.y;
    const int j = blockIdx.y;
    if (iu >= p.nu || iv >= p.nv) return;
    const int64_t oidx = ((int64_t)iv * p.views + j) * p.nu + iu;
    float m = 1.0f;
    Ray r;
    if (p.cone && setup_ray(p, iu, iv, j, angles, u_arr, v_arr, czv, pa, pxs, false, r)) {
        const float h = (float)p.nx / 2.0f;
        for (int k = r.ks; k <= r.ke; ++k) {
            const float fk = (float)k;
            const float xf = floorf(fmaf(fk, r.dfx, r.fx0));
            const float yf = floorf(fmaf(fk, r.dfy, r.fy0));
            if (!(xf >= 0.0f && xf + 1.0f < (float)p.nx && yf >= 0.0f && yf + 1.0f < (float)p.nx)) continue;
            if ((xf - h) * (xf - h) + (yf - h) * (yf - h) < h * h) {
                const float zf = floorf(fmaf(fk, r.dfz, r.fz0));
                if (zf < 0.0f || zf + 1.0f >= (float)p.nz) {
                    m = 0.0f;
                    break;
                }
            }
        }
    }
    mask[oidx] = m;
}

// Number of in-volume trilinear samples (the forward projector's algorithmic work).
__global__ void __launch_bounds__(256)
fp_count_kernel(FpParams p, const float* __restrict__ angles, const float* __restrict__ u_arr,
                const float* __restrict__ v_arr, const float* __restrict__ czv, const float* __restrict__ pa,
                const float* __restrict__ pxs, const float* __restrict__ mask, unsigned long long* __restrict__ count) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.z * blockDim.y + threadIdx.y;
    const int j = blockIdx.y;
    unsigned long long c = 0;
    Ray r;
    if (iu < p.nu && iv < p.nv && !(mask && mask[((int64_t)iv * p.views + j) * p.nu + iu] != 1.0f) &&
        setup_ray(p, iu, iv, j, angles, u_arr, v_arr, czv, pa, pxs, true, r)) {
        for (int k = r.ks; k <= r.ke; ++k) {
            const float fk = (float)k;
            const float xf = floorf(fmaf(fk, r.dfx, r.fx0)), yf = floorf(fmaf(fk, r.dfy, r.fy0));
            if (!(xf >= 0.0f && xf + 1.0f < (float)p.nx && yf >= 0.0f && yf + 1.0f < (float)p.nx)) continue;
            if (p.cone) {
                const float zf = floorf(fmaf(fk, r.dfz, r.fz0));
                if (!(zf >= 0.0f && zf + 1.0f < (float)p.nz)) continue;
            }
            ++c;
        }
    }
    // warp-aggregate, one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Oversample binning + Gaussian-approximated photon noise, run_mgfpj_v3.py:368-391.
__global__ void bin_noise_kernel(int64_t n_out, int nu, int bin, float photons, uint64_t seed,
                                 const float* __restrict__ in, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_out; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t rowv = i / nu;
        const int c = (int)(i % nu);
        const float* src = in + rowv * (int64_t)nu * bin + (int64_t)c * bin;
        float s = 0.0f;
        for (int b = 0; b < bin; ++b) s += src[b];
        float val = s / (float)bin;
        if (photons > 0.0f) {
            uint64_t h1 = splitmix64(seed ^ (uint64_t)(2 * i));
            uint64_t h2 = splitmix64(seed ^ (uint64_t)(2 * i + 1) ^ 0x5851F42D4C957F2Dull);
            float u1 = ((h1 >> 40) + 1.0f) * (1.0f / 16777217.0f);
            float u2 = (h2 >> 40) * (1.0f / 16777216.0f);
            float g = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
            float t = photons * expf(-val);
            t = t + g * sqrtf(t);
            if (t <= 0.0f) t = 1e-6f;
            val = logf(photons / t);
        }
        out[i] = val;
    }
}

// Exact line integrals of rotated ellipsoids along the forward projector's rays.
__global__ void __launch_bounds__(256)
ellipsoid_kernel(FpParams p, const float* __restrict__ angles, const float* __restrict__ u_arr,
                 const float* __restrict__ v_arr, const float* __restrict__ ell, int n_ell,
                 float* __restrict__ sgm) {
    const int iu = blockIdx.x * blockDim.x + threadIdx.x;
    const int iv = blockIdx.z * blockDim.y + threadIdx.y;
    const int j = blockIdx.y;
    if (iu >= p.nu || iv >= p.nv) return;
    float sb, cb;
    sincosf(angles[j], &sb, &cb);
    const float zj = p.zpv * (float)j;
    const float uval = u_arr[iu];
    float dx, dy;
    if (p.curved) {
        float sg, cg;
        sincosf((-uval) / p.sdd, &sg, &cg);
        dx = -p.sdd * cg + p.sid;
        dy = -p.sdd * sg;
    } else {
        dx = -(p.sdd - p.sid);
        dy = uval;
    }
    const float ex = dx - p.sid, ey = dy, ez = v_arr[iv];
    const float dist = sqrtf(ex * ex + ey * ey + ez * ez);
    const double ux = ex / dist, uy = ey / dist, uz = ez / dist;
    // source and direction in the object frame (object rotated by +beta)
    const double Ox = p.sid * (double)cb, Oy = p.sid * (double)sb, Oz = zj;
    const double Dx = ux * cb - uy * sb, Dy = uy * cb + ux * sb, Dz = uz;
    double total = 0.0;
    for (int e = 0; e < n_ell; ++e) {
        const float* E = ell + 10 * e;
        const double cph = cos((double)E[6]), sph = sin((double)E[6]);
        const double qx = Ox - E[0], qy = Oy - E[1], qz = Oz - E[2];
        const double px_ = (qx * cph + qy * sph) / E[3], py_ = (-qx * sph + qy * cph) / E[4], pz_ = qz / E[5];
        const double dx_ = (Dx * cph + Dy * sph) / E[3], dy_ = (-Dx * sph + Dy * cph) / E[4], dz_ = Dz / E[5];
        const double a = dx_ * dx_ + dy_ * dy_ + dz_ * dz_;
        const double b = px_ * dx_ + py_ * dy_ + pz_ * dz_;
        const double c = px_ * px_ + py_ * py_ + pz_ * pz_ - 1.0;
        const double disc = b * b - a * c;
        if (disc > 0.0) total += E[9] * 2.0 * sqrt(disc) / a;
    }
    sgm[((int64_t)iv * p.views + j) * p.nu + iu] = (float)total;
}

int make_params(const mct_geom* g, FpParams& p, const char* who) {
    MCT_TRY(check_geom(g, who));
    MCT_TRY(check_whole_scan(g, who));
    p = FpParams{};
    p.nx = g->nx; p.nz = g->nz; p.nu = g->nu; p.nv = g->nv; p.views = g->views; p.K = g->fp_steps;
    p.cone = (g->flags & MCT_CONE) != 0;
    p.curved = (g->flags & MCT_CURVED) != 0;
    p.pmat = (g->flags & MCT_PMATRIX) != 0;
    MCT_REQUIRE(p.K >= 0, "%s: negative step count", who);
    MCT_REQUIRE(g->views <= 65535, "%s: at most 65535 views per launch", who);
    MCT_REQUIRE(p.cone || g->nz >= g->nv, "%s: fan beam needs one image slice per detector row", who);
    MCT_REQUIRE(!p.cone || g->pz > 0.0f, "%s: cone beam needs a positive voxel height", who);
    MCT_REQUIRE(g->px > 0.0f, "%s: pixel size must be positive", who);
    MCT_REQUIRE((int64_t)g->nz * g->nx * g->nx < ((int64_t)1 << 31), "%s: volume must have fewer than 2^31 voxels", who);
    p.sid = g->sid; p.sdd = g->sdd; p.cx = g->cx; p.cy = g->cy; p.cz = g->cz;
    // run_mgfpj_v3.py:210-239 in double, then rounded
    const double px = g->px, pz = p.cone ? g->pz : 0.0;
    const double img_dimension = g->nx * px, image_dimension_z = g->nz * (double)g->pz;
    const double vd = std::sqrt(2 * px * px + (double)g->pz * g->pz);
    p.stepvd = (float)(g->fp_step * vd);
    p.l_min = (float)(g->sid - std::sqrt(2 * img_dimension * img_dimension + image_dimension_z * image_dimension_z) / 2.0);
    p.inv_px = (float)(1.0 / px);
    p.inv_pz = p.cone ? (float)(1.0 / pz) : 0.0f;
    p.x0 = (float)(-(g->nx - 1.0) / 2.0 * px + g->cx);
    p.y0 = (float)(-(g->nx - 1.0) / 2.0 * (-px) + g->cy);
    p.zoff = (float)(-(g->nz - 1.0) / 2.0 * (double)g->pz);
    p.zpv = g->fp_z_per_view;
    p.vshift = 0;
    p.bcs = 5;  // 32 columns x 8 rows of one view, warps of 32 columns
    p.wcs = 5;
    p.rs = 0;
    return MCT_OK;
}

}  // namespace
}  // namespace mct

using namespace mct;

extern "C" {

size_t mct_fp_workspace_size(const mct_geom* g) {
    if (!g || g->nx < 1 || g->nz < 1) return 0;
    const size_t n = (size_t)g->nz * g->nx * g->nx;
    // cone beam: two float32 quad copies (16 bytes per voxel each); fan beam: one
    // transposed copy
    return (g->flags & MCT_CONE) ? 2 * n * sizeof(Quad16) : n * sizeof(float);
}

size_t mct_fp_storage_workspace_size(const mct_geom* g, int32_t dtype) {
    if (!g || g->nx < 1 || g->nz < 1) return 0;
    if (dtype == MCT_F32) return mct_fp_workspace_size(g);
    if (!(g->flags & MCT_CONE) || (dtype != MCT_BF16 && dtype != MCT_F16)) return 0;
    // two 16-bit cell copies (+16 bytes for the float16 scale's source maximum)
    return 2 * (size_t)g->nz * g->nx * g->nx * sizeof(uint4) + (dtype == MCT_F16 ? 16 : 0);
}

}  // extern "C"

namespace {
// The projector's launches with a float32 or bf16 volume (TIN); the bf16 volume is read
// only by the copy kernels, so it needs cone beam and a workspace.
template <typename TIN>
int fp_storage_impl(const mct_geom* g, const mct_tables* t, const TIN* vol_in, const float* mask, float* sgm,
                    void* workspace, int32_t dtype, void* stream) {
    const float* vol = reinterpret_cast<const float*>(vol_in);  // read as float32 only when TIN is float
    constexpr bool kIn32 = std::is_same<TIN, float>::value;
    FpParams p;
    MCT_TRY(make_params(g, p, "mct_fp"));
    MCT_REQUIRE(t && t->angles && t->u && t->v && vol && sgm, "mct_fp: NULL buffer");
    MCT_REQUIRE(kIn32 || (p.cone && workspace), "mct_fp: a bf16 volume needs cone beam and a workspace");
    MCT_REQUIRE(!p.pmat || (t->pmat_a && t->pmat_xs), "mct_fp: projection-matrix tables missing");
    MCT_REQUIRE(workspace != (void*)vol, "mct_fp: workspace aliases the volume");
    MCT_REQUIRE(((uintptr_t)workspace & 15) == 0, "mct_fp: workspace must be 16-byte aligned");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16 || dtype == MCT_F16,
                "mct_fp: dtype must be MCT_F32, MCT_BF16 or MCT_F16");
    MCT_REQUIRE(dtype == MCT_F32 || (p.cone && workspace), "mct_fp: 16-bit storage needs cone beam and a workspace");
    cudaStream_t s = as_stream(stream);
    if (g->nx < 2 || (p.cone && g->nz < 2)) {
        // no trilinear stencil fits inside the volume: every ray sums nothing, as in the
        // reference (its inside test fails for every sample)
        cudaError_t e = cudaMemsetAsync(sgm, 0, (size_t)sgm_elems(*g) * sizeof(float), s);
        if (e != cudaSuccess) {
            set_error("mct_fp: %s", cudaGetErrorString(e));
            return MCT_E_CUDA;
        }
        return MCT_OK;
    }
    dim3 tb(32, 8), tg((g->nx + 31) / 32, (g->nx + 31) / 32, g->nz);
    // Ray tiles with copies: 16 detector columns x 16 consecutive views of one row
    // (float32 quads) or 16 columns x 4 views x 4 rows (16-bit cells), warps of 4
    // columns x 8 (view, row) slots.  The rays of neighbouring views cross nearly the
    // same cells at the same step, so a compact warp touches fewer L1 lines per
    // reload than 32 columns of one view.  Measured at 512x512x256 / 1080 views
    // (float32 / bf16 ms): 32 columns x 8 views with warps of 32 columns 263.6 / 230.5,
    // of 8 x 4 248.1 / 223.3, of 4 x 8 244.7 / 223.5; 16 x 16 views with warps of
    // 4 x 8 237.2 / 224.0 (bf16 with 4 views x 4 rows: 222.2), 2 x 16 244.8 / 222.9,
    // 8 x 4 240.8 / 224.2; 8 x 32 views with warps of 2 x 16 245.4 / 226.9, 1 x 32
    // 255.9 / 227.1.  Short scans keep 4 views x 4 rows: float32 at 512x512x128 / 90
    // views 12.96 ms against 14.34 with 16 views (512x512x64 / 360 views: 21.55 against
    // 20.92).  Without copies: 32 columns x 8 rows of one view.
    // The 16-view tiles take 4 rows in turn per view group (row tile, then view group):
    // neighbouring rows' rays cross nearly the same cells, and the outer rows' slab (up
    // to ~50 planes) does not fit L2 across all views.  DRAM per launch at 512x512x256 /
    // 1080 views: 31.3 GB with one row at a time, 19.1 GB with 2 (236.3 ms), 12.8 GB
    // with 4 (237.8 ms against 237.6), 10.7 GB with 8 (238.7 ms); the 16-bit tiles already
    // span 4 rows (2 more in turn: 219.7 against 215.9 ms).
    if (p.cone && workspace) {
        p.vshift = (dtype == MCT_F32 && g->views >= 256) ? 4 : 2;
        p.bcs = 4;
        p.wcs = 2;
        p.rs = p.vshift == 4 ? 2 : 0;
    }
    const int vb = 1 << p.vshift, rb = 1 << (8 - p.bcs - p.vshift + p.rs), cb = 1 << p.bcs;
    dim3 block(32, 8), grid((g->nu + cb - 1) / cb, ((g->views + vb - 1) / vb) << p.rs, (g->nv + rb - 1) / rb);
    const size_t n = (size_t)g->nz * g->nx * g->nx;
    if (p.cone && workspace && dtype == MCT_BF16) {
        uint4* cx = static_cast<uint4*>(workspace);
        uint4* cy = cx + n;
        cell16_kernel<false><<<tg, tb, 0, s>>>(g->nx, g->nz, vol_in, cx, cy, nullptr);
        MCT_TRY(launched("cell16_kernel"));
        fp_kernel<true, true, uint4><<<grid, block, 0, s>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a, t->pmat_xs, vol,
                                                            nullptr, cx, cy, mask, sgm, nullptr);
    } else if (p.cone && workspace && dtype == MCT_F16) {
        uint4* cx = static_cast<uint4*>(workspace);
        uint4* cy = cx + n;
        uint32_t* vmax = reinterpret_cast<uint32_t*>(cy + n);
        cudaError_t e = cudaMemsetAsync(vmax, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) {
            set_error("mct_fp: %s", cudaGetErrorString(e));
            return MCT_E_CUDA;
        }
        const int64_t blocks = ((int64_t)n + 255) / 256;
        vol_absmax_kernel<<<(int)(blocks < 152 * 32 ? blocks : 152 * 32), 256, 0, s>>>((int64_t)n, vol_in, vmax);
        MCT_TRY(launched("vol_absmax_kernel"));
        cell16_kernel<true><<<tg, tb, 0, s>>>(g->nx, g->nz, vol_in, cx, cy, vmax);
        MCT_TRY(launched("cell16_kernel"));
        fp_kernel<true, true, h16x8><<<grid, block, 0, s>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a, t->pmat_xs, vol,
                                                            nullptr, reinterpret_cast<const h16x8*>(cx),
                                                            reinterpret_cast<const h16x8*>(cy), mask, sgm, vmax);
    } else if (p.cone && workspace) {
        Quad16* cx = static_cast<Quad16*>(workspace);
        Quad16* cy = cx + n;
        quad32_kernel<<<tg, tb, 0, s>>>(g->nx, g->nz, vol_in, reinterpret_cast<float4*>(cx),
                                        reinterpret_cast<float4*>(cy));
        MCT_TRY(launched("quad32_kernel"));
        fp_kernel<true, true, Quad16><<<grid, block, 0, s>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a, t->pmat_xs,
                                                             vol, nullptr, cx, cy, mask, sgm, nullptr);
    } else if constexpr (kIn32) {
        float* vt = static_cast<float*>(workspace);
        if (vt) {
            transpose_xy_kernel<<<tg, tb, 0, s>>>(g->nx, g->nz, vol, vt);
            MCT_TRY(launched("transpose_xy_kernel"));
        }
        if (p.cone)
            fp_kernel<true, false, float2><<<grid, block, 0, s>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a,
                                                                  t->pmat_xs, vol, vt, nullptr, nullptr, mask, sgm,
                                                                  nullptr);
        else
            fp_kernel<false, false, float2><<<grid, block, 0, s>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a,
                                                                   t->pmat_xs, vol, vt, nullptr, nullptr, mask, sgm,
                                                                   nullptr);
    }
    return launched("fp_kernel");
}
}  // namespace

extern "C" {

int mct_fp_storage(const mct_geom* g, const mct_tables* t, const float* vol, const float* mask, float* sgm,
                   void* workspace, int32_t dtype, void* stream) {
    return fp_storage_impl<float>(g, t, vol, mask, sgm, workspace, dtype, stream);
}

int mct_fp_storage_in(const mct_geom* g, const mct_tables* t, const void* vol, int32_t vol_dtype, const float* mask,
                      float* sgm, void* workspace, int32_t dtype, void* stream) {
    MCT_REQUIRE(vol_dtype == MCT_F32 || vol_dtype == MCT_BF16, "mct_fp_storage_in: vol_dtype must be MCT_F32 or MCT_BF16");
    if (vol_dtype == MCT_F32)
        return fp_storage_impl<float>(g, t, static_cast<const float*>(vol), mask, sgm, workspace, dtype, stream);
    return fp_storage_impl<__nv_bfloat16>(g, t, static_cast<const __nv_bfloat16*>(vol), mask, sgm, workspace, dtype,
                                          stream);
}

int mct_fp(const mct_geom* g, const mct_tables* t, const float* vol, const float* mask, float* sgm, void* workspace,
           void* stream) {
    return mct_fp_storage(g, t, vol, mask, sgm, workspace, MCT_F32, stream);
}

int mct_fp_adjoint(const mct_geom* g, const mct_tables* t, const float* sgm, const float* mask, float* vol,
                   void* stream) {
    FpParams p;
    MCT_TRY(make_params(g, p, "mct_fp_adjoint"));
    MCT_REQUIRE(t && t->angles && t->u && t->v && vol && sgm, "mct_fp_adjoint: NULL buffer");
    MCT_REQUIRE(!p.pmat || (t->pmat_a && t->pmat_xs), "mct_fp_adjoint: projection-matrix tables missing");
    dim3 block(32, 8), grid((g->nu + 31) / 32, g->views, (g->nv + 7) / 8);
    fp_adjoint_kernel<false><<<grid, block, 0, as_stream(stream)>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a,
                                                                    t->pmat_xs, sgm, mask, vol);
    return launched("fp_adjoint_kernel");
}

size_t mct_fp_adjoint_workspace_size(const mct_geom* g) {
    if (!g || g->nx < 1 || g->nz < 1) return 0;
    return (size_t)g->nz * g->nx * g->nx * ((g->flags & MCT_CONE) ? 32 : 16);
}

int mct_fp_adjoint_cells(const mct_geom* g, const mct_tables* t, const float* sgm, const float* mask, float* vol,
                         void* workspace, void* stream) {
    FpParams p;
    MCT_TRY(make_params(g, p, "mct_fp_adjoint_cells"));
    MCT_REQUIRE(t && t->angles && t->u && t->v && vol && sgm && workspace, "mct_fp_adjoint_cells: NULL buffer");
    MCT_REQUIRE(!p.pmat || (t->pmat_a && t->pmat_xs), "mct_fp_adjoint_cells: projection-matrix tables missing");
    MCT_REQUIRE(((uintptr_t)workspace & 15) == 0, "mct_fp_adjoint_cells: workspace must be 16-byte aligned");
    MCT_REQUIRE(g->nx <= 65535 * 8 && g->nz <= 65535, "mct_fp_adjoint_cells: at most 524280 x 524280 x 65535 voxels");
    cudaStream_t s = as_stream(stream);
    float* cells = static_cast<float*>(workspace);
    const int C = p.cone ? 8 : 4;
    MCT_REQUIRE(cudaMemsetAsync(cells, 0, mct_fp_adjoint_workspace_size(g), s) == cudaSuccess,
                "mct_fp_adjoint_cells: clearing the workspace failed");
    dim3 block(32, 8), grid((g->nu + 31) / 32, g->views, (g->nv + 7) / 8);
    fp_adjoint_kernel<true><<<grid, block, 0, s>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a, t->pmat_xs, sgm,
                                                   mask, cells);
    MCT_TRY(launched("fp_adjoint_kernel"));
    dim3 gb(32, 8), gg((g->nx + 31) / 32, (g->nx + 7) / 8, g->nz);
    if (C == 8)
        adjoint_gather_kernel<8><<<gg, gb, 0, s>>>(g->nx, g->nz, cells, vol);
    else
        adjoint_gather_kernel<4><<<gg, gb, 0, s>>>(g->nx, g->nz, cells, vol);
    return launched("adjoint_gather_kernel");
}

int mct_fp_count_samples(const mct_geom* g, const mct_tables* t, const float* mask, uint64_t* count, void* stream) {
    FpParams p;
    MCT_TRY(make_params(g, p, "mct_fp_count_samples"));
    MCT_REQUIRE(t && t->angles && t->u && t->v && count, "mct_fp_count_samples: NULL buffer");
    MCT_REQUIRE(!p.pmat || (t->pmat_a && t->pmat_xs), "mct_fp_count_samples: projection-matrix tables missing");
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint64_t), as_stream(stream));
    if (e != cudaSuccess) {
        set_error("mct_fp_count_samples: %s", cudaGetErrorString(e));
        return MCT_E_CUDA;
    }
    dim3 block(32, 8), grid((g->nu + 31) / 32, g->views, (g->nv + 7) / 8);
    fp_count_kernel<<<grid, block, 0, as_stream(stream)>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a, t->pmat_xs, mask,
                                                           (unsigned long long*)count);
    return launched("fp_count_kernel");
}

int mct_effective_map(const mct_geom* g, const mct_tables* t, float* mask, void* stream) {
    FpParams p;
    MCT_TRY(make_params(g, p, "mct_effective_map"));
    MCT_REQUIRE(t && t->angles && t->u && t->v && mask, "mct_effective_map: NULL buffer");
    MCT_REQUIRE(!p.pmat || (t->pmat_a && t->pmat_xs), "mct_effective_map: projection-matrix tables missing");
    dim3 block(32, 8), grid((g->nu + 31) / 32, g->views, (g->nv + 7) / 8);
    emap_kernel<<<grid, block, 0, as_stream(stream)>>>(p, t->angles, t->u, t->v, t->cz, t->pmat_a, t->pmat_xs, mask);
    return launched("emap_kernel");
}

int mct_bin_noise(const mct_geom* g, const float* in, int32_t bin, float photons, uint64_t seed, float* out,
                  void* stream) {
    MCT_TRY(check_geom(g, "mct_bin_noise"));
    MCT_REQUIRE(in && out && bin >= 1, "mct_bin_noise: bad arguments");
    MCT_REQUIRE(bin == 1 || in != out, "mct_bin_noise: binning cannot run in place");
    int64_t n = sgm_elems(*g);
    int64_t blocks = (n + 255) / 256;
    bin_noise_kernel<<<(int)(blocks < 152 * 64 ? (blocks < 1 ? 1 : blocks) : 152 * 64), 256, 0, as_stream(stream)>>>(
        n, g->nu, bin, photons, seed, in, out);
    return launched("bin_noise_kernel");
}

int mct_project_ellipsoids(const mct_geom* g, const mct_tables* t, const float* ell, int32_t n_ell, float* sgm,
                           void* stream) {
    FpParams p;
    MCT_TRY(make_params(g, p, "mct_project_ellipsoids"));
    MCT_REQUIRE(t && t->angles && t->u && t->v && ell && sgm && n_ell >= 0, "mct_project_ellipsoids: bad arguments");
    dim3 block(32, 8), grid((g->nu + 31) / 32, g->views, (g->nv + 7) / 8);
    ellipsoid_kernel<<<grid, block, 0, as_stream(stream)>>>(p, t->angles, t->u, t->v, ell, n_ell, sgm);
    return launched("ellipsoid_kernel");
}

}  // extern "C"
