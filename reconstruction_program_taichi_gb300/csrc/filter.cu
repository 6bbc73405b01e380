// Sinogram weighting, vertical Gaussian, Toeplitz row filter and BP operand packing.
//
// Reference kernels replaced (run_mgfbp.py): BHCorrection :946-954, WeightSgm
// :956-1011, ConvolveSgmAndKernel :1013-1046.
#include <cmath>

#include "common.cuh"
#include "weight.cuh"

namespace mct {
namespace {

// One block per (row, view) line of nu elements (grid-stride over lines), so the
// line's row, view and source offset are computed once per line, not per element.
__global__ void weight_kernel(WeightParams p, const float* __restrict__ in, const float* __restrict__ bh,
                              const float* __restrict__ angles, float* __restrict__ out) {
    const int64_t lines = (int64_t)p.nv * p.views;
    for (int64_t rj = blockIdx.x; rj < lines; rj += gridDim.x) {
        const int j = (int)(rj % p.views);
        const int r = (int)(rj / p.views);
        const float* src = in + r * p.row_stride + j * p.view_stride;
        float* dst = out + rj * p.nu;
        const float v = p.v0 + r * p.v_step;
        const float beta = p.short_scan ? fabsf(angles[p.view_begin + j] - angles[0]) : 0.0f;
        for (int c = threadIdx.x; c < p.nu; c += blockDim.x) {
            const float u = p.u0 + c * p.u_step;
            dst[c] = weight_value(p, src[c], bh, u, weight_cos(p, u), weight_den(p, u, v), beta);
        }
    }
}

// The same weighting with 16-byte accesses (nu, the strides and both pointers multiples
// of 4 floats): block = one detector row and WV views, thread = 4 columns.  The
// distance factor's square root (and the curved cosine) depend on (row, column) only,
// so each thread takes them once for its WV views; every element then goes through
// the same operations, in the same order, as in weight_kernel (identical results).
// 64-bit line division gone, WV independent 16-byte loads in flight per thread.
constexpr int WV = 8;
__global__ void __launch_bounds__(256)
weight4_kernel(WeightParams p, const float* __restrict__ in, const float* __restrict__ bh,
               const float* __restrict__ angles, float* __restrict__ out) {
    const int r = blockIdx.y;
    const int j0 = blockIdx.x * WV;
    const int nj = min(WV, p.views - j0);
    const float v = p.v0 + r * p.v_step;
    const int nu4 = p.nu >> 2;
    for (int c4 = threadIdx.x; c4 < nu4; c4 += blockDim.x) {
        float uu[4], cs[4], den[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float u = p.u0 + (4 * c4 + e) * p.u_step;
            uu[e] = u;
            cs[e] = weight_cos(p, u);
            den[e] = weight_den(p, u, v);
        }
#pragma unroll
        for (int jj = 0; jj < WV; ++jj) {
            if (jj < nj) {
                const int j = j0 + jj;
                const float4 x = *reinterpret_cast<const float4*>(in + r * p.row_stride + j * p.view_stride + 4 * c4);
                const float beta = p.short_scan ? fabsf(angles[p.view_begin + j] - angles[0]) : 0.0f;
                float o[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                for (int e = 0; e < 4; ++e) o[e] = weight_value(p, o[e], bh, uu[e], cs[e], den[e], beta);
                *reinterpret_cast<float4*>(out + ((int64_t)r * p.views + j) * p.nu + 4 * c4) =
                    make_float4(o[0], o[1], o[2], o[3]);
            }
        }
    }
}

__global__ void vgauss_kernel(int nu, int nv, int views, float dv, const float* __restrict__ in,
                              const float* __restrict__ g, float* __restrict__ out) {
    int64_t n = (int64_t)nv * views * nu;
    int64_t plane = (int64_t)views * nu;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(idx / plane);
        int64_t jk = idx % plane;
        float acc = 0.0f;
        int n0 = max(0, i - 10), n1 = min(nv - 1, i + 10);
        for (int m = n0; m <= n1; ++m) acc += in[m * plane + jk] * g[i + (nv - 1) - m];
        out[idx] = acc * dv;
    }
}

// ---------------------------------------------------------------- Toeplitz filter
// Y[R][k] = du * sum_m X[R][m] * h[k - m + nu - 1] for R = r*views + j, written to the
// view-major output F[j][r][k].  Block tile 128 rows x 128 columns, 32-deep m slices,
// 256 threads with an 8x8 register tile each.  Along m the Toeplitz operand is a
// sliding window of the taps, so each thread keeps 8 taps in registers and loads one
// new tap per m step.
constexpr int FBM = 128, FBN = 128, FBK = 32, FAPAD = 4;

__global__ void __launch_bounds__(256, 2)
toeplitz_filter_kernel(int nu, int nv, int views, float du, const float* __restrict__ X,
                       const float* __restrict__ h, float* __restrict__ F) {
    __shared__ __align__(16) float As[FBK][FBM + FAPAD];
    __shared__ float hs[FBN + FBK];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t rows = (int64_t)nv * views;
    const int64_t row0 = (int64_t)blockIdx.y * FBM;
    const int k0 = blockIdx.x * FBN;
    const int ntaps = 2 * nu - 1;

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) acc[i][jj] = 0.0f;

    for (int m0 = 0; m0 < nu; m0 += FBK) {
        // A tile: X[row0 .. +127][m0 .. +31] -> As[m][row]
#pragma unroll
        for (int it = 0; it < (FBM * FBK) / 256; ++it) {
            int e = tid + it * 256;
            int rr = e / FBK, mm = e % FBK;
            int64_t R = row0 + rr;
            int m = m0 + mm;
            As[mm][rr] = (R < rows && m < nu) ? X[R * nu + m] : 0.0f;
        }
        // taps window: hs[i] = h[base + i], base = k0 - m0 - (FBK-1) + nu - 1
        int base = k0 - m0 - (FBK - 1) + nu - 1;
        for (int i = tid; i < FBN + FBK; i += 256) {
            int hi = base + i;
            hs[i] = (hi >= 0 && hi < ntaps) ? h[hi] : 0.0f;
        }
        __syncthreads();
        float b[8];
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) b[jj] = hs[(FBK - 1) + tx * 8 + jj];
#pragma unroll
        for (int mm = 0; mm < FBK; ++mm) {
            if (mm > 0) {
#pragma unroll
                for (int jj = 7; jj > 0; --jj) b[jj] = b[jj - 1];
                b[0] = hs[(FBK - 1) + tx * 8 - mm];
            }
            float4 a0 = *reinterpret_cast<const float4*>(&As[mm][ty * 8]);
            float4 a1 = *reinterpret_cast<const float4*>(&As[mm][ty * 8 + 4]);
            float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) acc[i][jj] = fmaf(a[i], b[jj], acc[i][jj]);
        }
        __syncthreads();
    }
    // epilogue: scale by du, write view-major
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        int64_t R = row0 + ty * 8 + i;
        if (R >= rows) continue;
        int r = (int)(R / views), j = (int)(R % views);
        float* dst = F + ((int64_t)j * nv + r) * nu;
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
            int k = k0 + tx * 8 + jj;
            if (k < nu) dst[k] = acc[i][jj] * du;
        }
    }
}

// ---------------------------------------------------------------- packing
template <typename QT>
__device__ __forceinline__ QT make_quad(float a, float b, float c, float d);
template <>
__device__ __forceinline__ float4 make_quad<float4>(float a, float b, float c, float d) {
    return make_float4(a, b, c, d);
}
template <>
__device__ __forceinline__ uint2 make_quad<uint2>(float a, float b, float c, float d) {
    __nv_bfloat162 lo = __floats2bfloat162_rn(a, b);
    __nv_bfloat162 hi = __floats2bfloat162_rn(c, d);
    uint2 r;
    r.x = *reinterpret_cast<uint32_t*>(&lo);
    r.y = *reinterpret_cast<uint32_t*>(&hi);
    return r;
}
template <>
__device__ __forceinline__ h16x4 make_quad<h16x4>(float a, float b, float c, float d) {
    return h16x4{pack_h16x2(a, b), pack_h16x2(c, d)};
}
template <typename PT>
__device__ __forceinline__ PT make_pair(float a, float b);
template <>
__device__ __forceinline__ h16x2 make_pair<h16x2>(float a, float b) {
    return h16x2{pack_h16x2(a, b)};
}
template <>
__device__ __forceinline__ float2 make_pair<float2>(float a, float b) { return make_float2(a, b); }
template <>
__device__ __forceinline__ uint32_t make_pair<uint32_t>(float a, float b) {
    __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&p);
}

// The base value A as the packed type stores it (float32: A itself; bf16: A rounded).
template <typename QT>
__device__ __forceinline__ float stored_base(float a);
template <>
__device__ __forceinline__ float stored_base<float4>(float a) { return a; }
template <>
__device__ __forceinline__ float stored_base<uint2>(float a) { return __bfloat162float(__float2bfloat16_rn(a)); }
template <>
__device__ __forceinline__ float stored_base<float2>(float a) { return a; }
template <>
__device__ __forceinline__ float stored_base<uint32_t>(float a) { return __bfloat162float(__float2bfloat16_rn(a)); }
template <>
__device__ __forceinline__ float stored_base<h16x4>(float a) { return __half2float(__float2half_rn(a)); }
template <>
__device__ __forceinline__ float stored_base<h16x2>(float a) { return __half2float(__float2half_rn(a)); }

// Largest |F| over a strided [rows][views][cols] source, as float bits, into *maxbits
// (which the caller zeroes first); NaN counts as larger than every finite value.
__global__ void absmax_kernel(int nu, int nv, int views, int64_t rs, int64_t vs, const float* __restrict__ F,
                              uint32_t* __restrict__ maxbits) {
    const int64_t n = (int64_t)nv * views * nu;
    uint32_t m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % nu);
        const int64_t rj = i / nu;
        const int j = (int)(rj % views), r = (int)(rj / views);
        m = max(m, __float_as_uint(F[r * rs + j * vs + c]) & 0x7fffffffu);
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, m);
}

// Source element (view j, row r, column c) is F[r*rs + j*vs + c].
// cone: Q[j][r][c], r < nv, c < nu-1.  For r < nv-1 the bilinear coefficients of
// detector cell (r, c) (A = F(j,r,c), B = F(j,r,c+1), C = F(j,r+1,c), D = F(j,r+1,c+1)):
// {A', C-A', B-A', (D-C)-(B-A')} with A' = A as stored.  The differences are formed in
// float32 against the stored A', so with bf16 storage the corners B, C, D are
// reproduced to bf16 precision of the (small) differences and only A carries a full
// bf16 rounding error, weighted by (1-ru)(1-rv) in the interpolated value.
// Row nv-1 is all NaN: the backprojector sends every off-detector row there, so an
// off-detector voxel ends up NaN and is written as 0.
template <typename QT>
__global__ void pack_quad_kernel(int nu, int nv, int views, int64_t rs, int64_t vs, const float* __restrict__ F,
                                 QT* __restrict__ Q, const uint32_t* __restrict__ maxbits) {
    const int nq = nu - 1, rq = nv;
    const float sc = IsF16<QT>::value ? ldexpf(1.0f, f16_scale_exp(*maxbits)) : 1.0f;
    int64_t n = (int64_t)views * rq * nq;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int c = (int)(i % nq);
        int64_t jr = i / nq;
        int r = (int)(jr % rq);
        int j = (int)(jr / rq);
        if (r == nv - 1) {
            const float qn = __int_as_float(0x7fffffff);
            Q[i] = make_quad<QT>(qn, qn, qn, qn);
            continue;
        }
        const float* f = F + r * rs + j * vs + c;
        const float a = stored_base<QT>(f[0] * sc), b = f[1] * sc, cc = f[rs] * sc, d = f[rs + 1] * sc;
        const float bma = b - a, dmc = d - cc;
        Q[i] = make_quad<QT>(a, cc - a, bma, dmc - bma);
    }
}

// fan: P[j][r][c] = {A', F(j,r,c+1) - A'} with A' = F(j,r,c) as stored, c < nu-1
template <typename PT>
__global__ void pack_pair_kernel(int nu, int nv, int views, int64_t rs, int64_t vs, const float* __restrict__ F,
                                 PT* __restrict__ P, const uint32_t* __restrict__ maxbits) {
    const int nq = nu - 1;
    const float sc = IsF16<PT>::value ? ldexpf(1.0f, f16_scale_exp(*maxbits)) : 1.0f;
    int64_t n = (int64_t)views * nv * nq;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int c = (int)(i % nq);
        int64_t jr = i / nq;
        int r = (int)(jr % nv);
        int j = (int)(jr / nv);
        const float* f = F + r * rs + j * vs + c;
        const float a = stored_base<PT>(f[0] * sc);
        P[i] = make_pair<PT>(a, f[1] * sc - a);
    }
}

inline int grid_for(int64_t n, int block = 256) {
    int64_t b = (n + block - 1) / block;
    return (int)(b < 152 * 64 ? (b < 1 ? 1 : b) : 152 * 64);
}

}  // namespace
}  // namespace mct

using namespace mct;

extern "C" {

int mct_weight(const mct_geom* g, const mct_tables* t, const float* sgm, int64_t row_stride, int64_t view_stride,
               const float* bh_coeffs, int32_t n_bh, float* weighted, void* stream) {
    MCT_TRY(check_geom(g, "mct_weight"));
    MCT_REQUIRE(sgm && weighted, "mct_weight: NULL buffer");
    MCT_REQUIRE(n_bh >= 0 && (n_bh == 0 || bh_coeffs), "mct_weight: bad BH coefficients");
    bool short_scan = (g->flags & MCT_SHORT_SCAN) != 0;
    MCT_REQUIRE(!short_scan || (t && t->angles), "mct_weight: short scan needs the angle table");
    const WeightParams p = weight_params(g, row_stride, view_stride, n_bh);
    const bool vec4 = g->nu % 4 == 0 && row_stride % 4 == 0 && view_stride % 4 == 0 && g->nv <= 65535 &&
                      ((uintptr_t)sgm & 15) == 0 && ((uintptr_t)weighted & 15) == 0;
    if (vec4) {
        dim3 grid((g->views + WV - 1) / WV, g->nv);
        weight4_kernel<<<grid, 256, 0, as_stream(stream)>>>(p, sgm, bh_coeffs, t ? t->angles : nullptr, weighted);
        return launched("weight4_kernel");
    }
    const int64_t lines = (int64_t)g->nv * g->views;
    const int blocks = (int)(lines < 152 * 64 ? lines : 152 * 64);
    weight_kernel<<<blocks, 256, 0, as_stream(stream)>>>(p, sgm, bh_coeffs, t ? t->angles : nullptr, weighted);
    return launched("weight_kernel");
}

int mct_vgauss(const mct_geom* g, const float* weighted, const float* gauss_taps, float* out, void* stream) {
    MCT_TRY(check_geom(g, "mct_vgauss"));
    MCT_REQUIRE(weighted && gauss_taps && out && weighted != out, "mct_vgauss: bad buffers");
    int64_t n = sgm_elems(*g);
    vgauss_kernel<<<grid_for(n), 256, 0, as_stream(stream)>>>(g->nu, g->nv, g->views, g->dv, weighted, gauss_taps, out);
    return launched("vgauss_kernel");
}

int mct_filter(const mct_geom* g, const float* weighted, const float* taps, float* filtered, void* stream) {
    MCT_TRY(check_geom(g, "mct_filter"));
    MCT_REQUIRE(weighted && taps && filtered && weighted != filtered, "mct_filter: bad buffers");
    int64_t rows = (int64_t)g->nv * g->views;
    MCT_REQUIRE((rows + FBM - 1) / FBM < 2147483647LL, "mct_filter: too many rows");
    dim3 grid((g->nu + FBN - 1) / FBN, (unsigned)((rows + FBM - 1) / FBM));
    toeplitz_filter_kernel<<<grid, 256, 0, as_stream(stream)>>>(g->nu, g->nv, g->views, g->du, weighted, taps, filtered);
    return launched("toeplitz_filter_kernel");
}

size_t mct_packed_size(const mct_geom* g, int32_t dtype) {
    if (!g || g->nu < 2 || g->nv < 1 || g->views < 1) return 0;
    // cone: 4 coefficients per (view, row incl. the NaN row nv-1, col < nu-1); fan: 2
    const bool cone = (g->flags & MCT_CONE) != 0;
    if (cone && g->nv < 2) return 0;
    const size_t esz = (cone ? 2 : 1) * (dtype == MCT_F32 ? 8 : 4);
    const size_t body = (size_t)g->views * g->nv * (g->nu - 1) * esz;
    return dtype == MCT_F16 ? body + 16 : body;  // float16: the scale's source maximum behind the body
}

int mct_pack_strided(const mct_geom* g, const float* src, int64_t row_stride, int64_t view_stride, void* packed,
                     int32_t dtype, void* stream) {
    MCT_TRY(check_geom(g, "mct_pack"));
    MCT_REQUIRE(src && packed, "mct_pack: NULL buffer");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16 || dtype == MCT_F16,
                "mct_pack: dtype must be MCT_F32, MCT_BF16 or MCT_F16");
    MCT_REQUIRE(((uintptr_t)packed & 15) == 0, "mct_pack: packed buffer must be 16-byte aligned");
    cudaStream_t s = as_stream(stream);
    const int64_t rs = row_stride, vs = view_stride;
    const bool cone = (g->flags & MCT_CONE) != 0;
    MCT_REQUIRE(!cone || g->nv >= 2, "mct_pack: cone beam needs at least 2 detector rows");
    const int64_t n = (int64_t)g->views * g->nv * (g->nu - 1);
    uint32_t* maxbits = nullptr;
    if (dtype == MCT_F16) {
        maxbits = f16_trailer(g, packed);
        cudaError_t e = cudaMemsetAsync(maxbits, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) {
            set_error("mct_pack: %s", cudaGetErrorString(e));
            return MCT_E_CUDA;
        }
        absmax_kernel<<<grid_for(sgm_elems(*g)), 256, 0, s>>>(g->nu, g->nv, g->views, rs, vs, src, maxbits);
        MCT_TRY(launched("absmax_kernel"));
    }
    if (cone) {
        if (dtype == MCT_F32)
            pack_quad_kernel<float4><<<grid_for(n), 256, 0, s>>>(g->nu, g->nv, g->views, rs, vs, src, (float4*)packed,
                                                                 maxbits);
        else if (dtype == MCT_BF16)
            pack_quad_kernel<uint2><<<grid_for(n), 256, 0, s>>>(g->nu, g->nv, g->views, rs, vs, src, (uint2*)packed,
                                                                maxbits);
        else
            pack_quad_kernel<h16x4><<<grid_for(n), 256, 0, s>>>(g->nu, g->nv, g->views, rs, vs, src, (h16x4*)packed,
                                                                maxbits);
    } else {
        if (dtype == MCT_F32)
            pack_pair_kernel<float2><<<grid_for(n), 256, 0, s>>>(g->nu, g->nv, g->views, rs, vs, src, (float2*)packed,
                                                                 maxbits);
        else if (dtype == MCT_BF16)
            pack_pair_kernel<uint32_t><<<grid_for(n), 256, 0, s>>>(g->nu, g->nv, g->views, rs, vs, src,
                                                                   (uint32_t*)packed, maxbits);
        else
            pack_pair_kernel<h16x2><<<grid_for(n), 256, 0, s>>>(g->nu, g->nv, g->views, rs, vs, src, (h16x2*)packed,
                                                                maxbits);
    }
    return launched("pack_kernel");
}

int mct_pack(const mct_geom* g, const float* filtered, void* packed, int32_t dtype, void* stream) {
    if (!g) {
        set_error("mct_pack: geometry is NULL");
        return MCT_E_INVALID;
    }
    return mct_pack_strided(g, filtered, g->nu, (int64_t)g->nv * g->nu, packed, dtype, stream);
}

}  // extern "C"
