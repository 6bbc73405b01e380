// Shared helpers of the MandoCT GB300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
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

inline int64_t vol_elems(const mct_geom& g) { return (int64_t)g.nz * g.nx * g.nx; }
inline int64_t sgm_elems(const mct_geom& g) { return (int64_t)g.nv * g.views * g.nu; }

// Redundancy factor of the backprojection (run_mgfbp.py:1072-1084), evaluated in
// double on the host.
double div_factor(const mct_geom& g);

__device__ __forceinline__ float bf16_to_f32(__nv_bfloat16 h) { return __bfloat162float(h); }

// Read-only, L1-cached loads.
template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

// Loaders of the packed backprojection operand (see mct_pack): a 2x2 bilinear
// stencil {r c, r c+1, r+1 c, r+1 c+1} as float4 or 4 x bf16 (uint2), and a column
// pair {c, c+1} as float2 or 2 x bf16 (uint32).
template <typename QT>
struct Quad;
template <>
struct Quad<float4> {
    static __device__ __forceinline__ void load(const float4* p, float& a, float& b, float& c, float& d) {
        float4 q = __ldg(p);
        a = q.x; b = q.y; c = q.z; d = q.w;
    }
};
template <>
struct Quad<uint2> {
    static __device__ __forceinline__ void load(const uint2* p, float& a, float& b, float& c, float& d) {
        uint2 q = __ldg(p);
        a = __uint_as_float(q.x << 16);
        b = __uint_as_float(q.x & 0xffff0000u);
        c = __uint_as_float(q.y << 16);
        d = __uint_as_float(q.y & 0xffff0000u);
    }
};
template <typename PT>
struct Pair;
template <>
struct Pair<float2> {
    static __device__ __forceinline__ void load(const float2* p, float& a, float& b) {
        float2 q = __ldg(p);
        a = q.x; b = q.y;
    }
};
template <>
struct Pair<uint32_t> {
    static __device__ __forceinline__ void load(const uint32_t* p, float& a, float& b) {
        uint32_t q = __ldg(p);
        a = __uint_as_float(q << 16);
        b = __uint_as_float(q & 0xffff0000u);
    }
};

}  // namespace mct
