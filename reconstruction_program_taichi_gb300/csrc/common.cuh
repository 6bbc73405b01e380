// Shared helpers of the MandoCT GB300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>
#include <cstdio>

#include "../../include/mandoct_gb300.h"

namespace mct {

// The reference's pi (run_mgfbp.py:16).
constexpr double kPI = 3.1415926536;

void set_error(const char* fmt, ...);
void count_launches(uint64_t n);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Checks the launch that was just issued; counts it as one kernel of this library.
inline int launched(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return MCT_E_CUDA;
    }
    count_launches(1);
    return MCT_OK;
}

#define MCT_REQUIRE(cond, ...)          \
    do {                                \
        if (!(cond)) {                  \
            ::mct::set_error(__VA_ARGS__); \
            return MCT_E_INVALID;       \
        }                               \
    } while (0)

#define MCT_TRY(expr)              \
    do {                           \
        int _rc = (expr);          \
        if (_rc != MCT_OK) return _rc; \
    } while (0)

// Geometry validation shared by all entry points.
int check_geom(const mct_geom* g, const char* who);
int check_whole_scan(const mct_geom* g, const char* who);

inline int64_t vol_elems(const mct_geom& g) { return (int64_t)g.nz * g.nx * g.nx; }
inline int64_t sgm_elems(const mct_geom& g) { return (int64_t)g.nv * g.views * g.nu; }

// Redundancy factor of the backprojection (run_mgfbp.py:1072-1084), evaluated in
// double on the host.
double div_factor(const mct_geom& g);

__device__ __forceinline__ float bf16_to_f32(__nv_bfloat16 h) { return __bfloat162float(h); }

// Elements of float32 or bf16 volumes (bf16 iterate storage): loads widen to float32,
// stores round to nearest.
template <typename T>
__device__ __forceinline__ float ldv(const T* p, int64_t i);
template <>
__device__ __forceinline__ float ldv<float>(const float* p, int64_t i) { return p[i]; }
template <>
__device__ __forceinline__ float ldv<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) {
    return __bfloat162float(p[i]);
}
template <typename T>
__device__ __forceinline__ void stv(T* p, int64_t i, float v);
template <>
__device__ __forceinline__ void stv<float>(float* p, int64_t i, float v) { p[i] = v; }
template <>
__device__ __forceinline__ void stv<__nv_bfloat16>(__nv_bfloat16* p, int64_t i, float v) {
    p[i] = __float2bfloat16_rn(v);
}

// Read-only, L1-cached loads.
template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

// Loaders of the packed backprojection operand (see mct_pack).
//
// Cone beam: detector cell (r, c) with corners A = F[r][c], B = F[r][c+1],
// C = F[r+1][c], D = F[r+1][c+1] is stored in bilinear coefficient form
// {A, C-A, B-A, (D-C)-(B-A)} as float4 or 4 x bf16 (uint2) and returned as
// lo = {A, C-A}, hi = {B-A, (D-C)-(B-A)}.  The bilinear value at fractions (ru, rv) is
//     s = lo + ru*hi (one packed f32x2 FMA);  value = s.x + rv*s.y.
// Fan beam: the column pair {A, B-A} as float2 or 2 x bf16 (uint32); value = A + ru*(B-A).
// A bf16 word holds its first element in the low 16 bits.
__device__ __forceinline__ float2 bf16x2_to_float2(uint32_t w) {
    return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
}
// ---- float16 storage with a power-of-two scale.
// A float16 operand stores fp16(v * 2^e); e is chosen from the largest magnitude m of
// the source so that m * 2^e lies in [2^12, 2^13): differences of up to four values (the
// bilinear coefficients) stay below 2^15, inside fp16's range of 65504, and the
// relative precision is fp16's 2^-11 for every value down to 2^-12 of the largest.
// Readers multiply by 2^-e, which is exact.  m is reduced as float bits into a uint32
// (non-negative floats order like unsigned integers) stored behind the operand.
__device__ __forceinline__ int f16_scale_exp(uint32_t maxbits) {
    const float m = __uint_as_float(maxbits);
    if (!(m > 0.0f) || !(m <= 3.0e38f)) return 0;  // all zero, or inf/NaN in the source
    return 12 - ilogbf(m);
}
struct __align__(8) h16x4 {  // four fp16: bilinear coefficients of one cell
    uint32_t x, y;
};
struct h16x2 {  // two fp16: a column pair
    uint32_t v;
};
struct __align__(16) h16x8 {  // eight fp16: a trilinear cell (forward projection)
    uint32_t x, y, z, w;
};
__device__ __forceinline__ float2 h16x2_to_float2(uint32_t w) {
    __half2 h;
    *reinterpret_cast<uint32_t*>(&h) = w;
    return __half22float2(h);
}
__device__ __forceinline__ uint32_t pack_h16x2(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}
// The float16 operand's source maximum sits in the 16 bytes behind its body
// (mct_packed_size includes them).
inline uint32_t* f16_trailer(const mct_geom* g, const void* packed) {
    const bool cone = (g->flags & MCT_CONE) != 0;
    const size_t body = (size_t)g->views * g->nv * (g->nu - 1) * (cone ? 8 : 4);
    return reinterpret_cast<uint32_t*>(static_cast<char*>(const_cast<void*>(packed)) + body);
}
template <typename T>
struct IsF16 {
    static constexpr bool value = false;
};
template <>
struct IsF16<h16x4> {
    static constexpr bool value = true;
};
template <>
struct IsF16<h16x2> {
    static constexpr bool value = true;
};
template <>
struct IsF16<h16x8> {
    static constexpr bool value = true;
};

template <typename QT>
struct Quad;
template <>
struct Quad<float4> {
    static __device__ __forceinline__ void load(const float4* p, float2& lo, float2& hi) {
        const float4 q = __ldg(p);
        lo = make_float2(q.x, q.y);
        hi = make_float2(q.z, q.w);
    }
};
template <>
struct Quad<uint2> {
    static __device__ __forceinline__ void load(const uint2* p, float2& lo, float2& hi) {
        const uint2 q = __ldg(p);
        lo = bf16x2_to_float2(q.x);
        hi = bf16x2_to_float2(q.y);
    }
};
template <>
struct Quad<h16x4> {
    static __device__ __forceinline__ void load(const h16x4* p, float2& lo, float2& hi) {
        const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
        lo = h16x2_to_float2(q.x);
        hi = h16x2_to_float2(q.y);
    }
};
template <typename PT>
struct Pair;
template <>
struct Pair<h16x2> {
    static __device__ __forceinline__ float2 load(const h16x2* p) {
        return h16x2_to_float2(__ldg(reinterpret_cast<const uint32_t*>(p)));
    }
};
template <>
struct Pair<float2> {
    static __device__ __forceinline__ float2 load(const float2* p) { return __ldg(p); }
};
template <>
struct Pair<uint32_t> {
    static __device__ __forceinline__ float2 load(const uint32_t* p) { return bf16x2_to_float2(__ldg(p)); }
};

}  // namespace mct
