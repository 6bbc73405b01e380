// Toeplitz row filter on the 5th-generation tensor cores (tcgen05), split BF16.
//
// Y[R][k] = du * sum_m X[R][m] h[k-m+nu-1] is a GEMM  D[M x N] = A[M x K] B[K x N]
// with M = rows*views sinogram rows, N = K = nu.  Each float32 operand is split into
// bf16 hi + lo parts and D = A_hi B_hi + A_hi B_lo + A_lo B_hi is accumulated in
// float32 in tensor memory (the dropped A_lo B_lo term is ~2^-16 relative).
// Replaces the row convolution of Mgfbp.ConvolveSgmAndKernel (run_mgfbp.py:1030-1046).
//
// Operand layout.  A and B^T are stored pre-tiled in global memory exactly as one
// pipeline stage needs them in shared memory (tcgen05 canonical K-major layout, no
// swizzle): a 128x32 (A) or 256x32 (B^T) bf16 tile is one contiguous block of 8x8
// "core matrices" (8 rows x 16 bytes each); core (row group i, k group j) sits at
// byte (i*4 + j)*128.  So the K-direction core stride (LBO) is 128 B and the
// row-direction stride (SBO) is 512 B, and each stage is filled by plain bulk copies
// (cp.async.bulk, the TMA engine) of contiguous tiles.
//
// Kernel structure: 128 threads, two CTAs per SM (98 KiB of shared memory and 256
// tensor-memory columns each), so that one CTA's epilogue overlaps the other's MMAs
// (with one CTA per SM the tensor pipe idled during every epilogue: 29 % busy).
// Thread 0 issues the bulk copies of a 2-stage ring (48 KiB per stage),
// thread 32 issues tcgen05.mma (M=128, N=256, K=16; 3 products per K step) and
// commits each stage back to the producer; after the last stage all four warps read
// the 128x256 float32 accumulator from tensor memory (warp w owns lanes 32w..32w+31)
// and store du*D to the view-major output.  Every mbarrier wait is bounded (about 2 s
// of %globaltimer); a timeout sets an error flag, the kernel waits (bounded) for its
// own copies and MMAs, frees its tensor memory and returns; the host reports
// MCT_E_TIMEOUT on the next call that reads the flag.
#include <cmath>

#include "common.cuh"
#include "weight.cuh"

namespace mct {
namespace {

constexpr int TC_BM = 128, TC_BN = 256, TC_STAGES = 2;
constexpr int TC_TMEM_COLS = 256;
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;        // 2 s

// NS = number of bf16 parts each float32 operand is split into:
//   2: x = hi + lo, products hi*hi + hi*lo + lo*hi (~1e-5 relative; the mixed path);
//   3: x = hi + mid + lo, products of total order <= 2 (hi*hi, hi*mid, mid*hi, hi*lo,
//      lo*hi, mid*mid): the dropped terms are ~2^-24 relative; the result is within
//      ~1e-6 of float32 (the level of the tensor pipe's float32 accumulation).
// BK (K depth of one pipeline stage) keeps a stage small enough for two CTAs per SM.
template <int NS>
struct TcCfg;
template <>
struct TcCfg<2> {
    static constexpr int BK = 32, NPROD = 3;
};
template <>
struct TcCfg<3> {
    static constexpr int BK = 16, NPROD = 6;
};
template <int NS>
struct TcTiles {
    static constexpr int BK = TcCfg<NS>::BK;
    static constexpr int KG = BK / 8;                          // core matrices along K per row group
    static constexpr int SBO = KG * 128;                       // bytes between row groups
    static constexpr int A_TILE = TC_BM * BK * 2;
    static constexpr int B_TILE = TC_BN * BK * 2;
    static constexpr int STAGE = NS * (A_TILE + B_TILE);
    static constexpr int SMEM = TC_STAGES * STAGE + 2048;      // + 1 KiB alignment slack + barriers
    static_assert(2 * SMEM <= 228 * 1024, "two CTAs per SM");
};

struct TcDims {
    int64_t rows;    // M (sinogram rows)
    int nu;          // N = K
    int mb, kb, nb;  // tile counts along M, K, N
};

template <int NS>
inline TcDims tc_dims(int64_t rows, int nu) {
    TcDims d;
    d.rows = rows;
    d.nu = nu;
    d.mb = (int)((rows + TC_BM - 1) / TC_BM);
    d.kb = (nu + TcTiles<NS>::BK - 1) / TcTiles<NS>::BK;
    d.nb = (nu + TC_BN - 1) / TC_BN;
    return d;
}

// x as NS bf16 parts (bit patterns), largest first; each part is the bf16 rounding of
// what the previous parts leave
template <int NS>
__device__ __forceinline__ void split_parts(float x, uint32_t* out) {
    float r = x;
#pragma unroll
    for (int p = 0; p < NS; ++p) {
        const __nv_bfloat16 h = __float2bfloat16_rn(r);
        out[p] = (uint32_t)__bfloat16_as_ushort(h);
        r = r - __bfloat162float(h);
    }
}

// One 16-byte core-matrix row (8 bf16 along K) of every part of a tile.  Chunk i
// enumerates (tile, row group, k group kj, row r8) in storage order, so consecutive
// threads write consecutive 16-byte chunks.  ROWS = 128 (A) or 256 (B^T).
template <int NS, int ROWS>
__device__ __forceinline__ void tile_coords(int64_t i, int KB, int& r8, int& kj, int& gi, int& kb, int64_t& tb) {
    constexpr int KG = TcTiles<NS>::KG;
    r8 = (int)(i & 7);
    kj = (int)((i >> 3) % KG);
    const int64_t rest = (i >> 3) / KG;
    gi = (int)(rest % (ROWS / 8));
    const int64_t tile = rest / (ROWS / 8);
    kb = (int)(tile % KB);
    tb = tile / KB;
}

template <int NS>
__device__ __forceinline__ void store_parts(uint4* const* dst, int64_t i, const uint32_t (*v)[NS]) {
#pragma unroll
    for (int p = 0; p < NS; ++p)
        dst[p][i] = make_uint4(v[0][p] | (v[1][p] << 16), v[2][p] | (v[3][p] << 16), v[4][p] | (v[5][p] << 16),
                               v[6][p] | (v[7][p] << 16));
}

struct Parts {
    uint4* p[3];
};

template <int NS>
__global__ void split_a_kernel(const float* __restrict__ x, int64_t rows, int nu, int KB, int64_t n_chunks, Parts a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_chunks; i += (int64_t)gridDim.x * blockDim.x) {
        int r8, kj, mi, kb;
        int64_t mb;
        tile_coords<NS, TC_BM>(i, KB, r8, kj, mi, kb, mb);
        const int64_t R = mb * TC_BM + mi * 8 + r8;
        const int m0 = kb * TcTiles<NS>::BK + kj * 8;
        uint32_t v[8][NS];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int m = m0 + c;
            split_parts<NS>((R < rows && m < nu) ? x[R * nu + m] : 0.0f, v[c]);
        }
        store_parts<NS>(a.p, i, v);
    }
}

// split_a_kernel reading the raw sinogram and weighting each element on the way
// (weight_value, as the weighting kernels do), so the weighted float32 sinogram is never
// written: operand row R = r * views + j is detector row r of view j, as in the
// weighting kernels' output.
template <int NS>
__global__ void weight_split_a_kernel(WeightParams wp, const float* __restrict__ in, const float* __restrict__ bh,
                                      const float* __restrict__ angles, int64_t rows, int nu, int KB, int64_t n_chunks,
                                      Parts a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_chunks; i += (int64_t)gridDim.x * blockDim.x) {
        int r8, kj, mi, kb;
        int64_t mb;
        tile_coords<NS, TC_BM>(i, KB, r8, kj, mi, kb, mb);
        const int64_t R = mb * TC_BM + mi * 8 + r8;
        const int m0 = kb * TcTiles<NS>::BK + kj * 8;
        uint32_t v[8][NS];
        if (R < rows) {
            const int r = (int)(R / wp.views), j = (int)(R % wp.views);
            const float* src = in + r * wp.row_stride + j * wp.view_stride;
            const float vv = wp.v0 + r * wp.v_step;
            const float beta = wp.short_scan ? fabsf(angles[wp.view_begin + j] - angles[0]) : 0.0f;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int m = m0 + c;
                float x = 0.0f;
                if (m < nu) {
                    const float u = wp.u0 + m * wp.u_step;
                    x = weight_value(wp, __ldg(src + m), bh, u, weight_cos(wp, u), weight_den(wp, u, vv), beta);
                }
                split_parts<NS>(x, v[c]);
            }
        } else {
#pragma unroll
            for (int c = 0; c < 8; ++c) split_parts<NS>(0.0f, v[c]);
        }
        store_parts<NS>(a.p, i, v);
    }
}

// B^T element (n, k) = T[k][n] = h[n - k + nu - 1] (output column n, input column k),
// tiled like A with 256-row tiles.
template <int NS>
__global__ void build_b_kernel(const float* __restrict__ taps, int nu, int KB, int64_t n_chunks, Parts b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_chunks; i += (int64_t)gridDim.x * blockDim.x) {
        int r8, kj, ni, kb;
        int64_t nb;
        tile_coords<NS, TC_BN>(i, KB, r8, kj, ni, kb, nb);
        const int n = (int)nb * TC_BN + ni * 8 + r8;
        const int k0 = kb * TcTiles<NS>::BK + kj * 8;
        uint32_t v[8][NS];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int k = k0 + c;
            split_parts<NS>((n < nu && k < nu) ? taps[n - k + nu - 1] : 0.0f, v[c]);
        }
        store_parts<NS>(b.p, i, v);
    }
}

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait; returns false (and raises the error flag) after TC_WAIT_NS.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code) {
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > TC_WAIT_NS) {
            atomicExch(err, code);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    // start address >> 4 (bits 0-13), leading byte offset >> 4 (16-29), stride byte
    // offset >> 4 (32-45), fixed 0b001 (46-48), no swizzle (61-63 = 0)
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int NS>
__global__ void __launch_bounds__(128, 2)
tc_filter_kernel(TcDims d, int nv, int views, float du, Parts a, Parts b, float* __restrict__ F, int* __restrict__ err) {
    using T = TcTiles<NS>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1 KiB-aligned stage buffers: [A part 0..NS-1][B part 0..NS-1] per stage
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* ctrl = smem + TC_STAGES * T::STAGE;  // barriers and the TMEM address
    uint64_t* full = reinterpret_cast<uint64_t*>(ctrl);
    uint64_t* empty = full + TC_STAGES;
    uint64_t* done = empty + TC_STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nbk = blockIdx.x;  // N tile
    const int64_t mbk = blockIdx.y;  // M tile

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    bool ok = true;
    if (threadIdx.x == 0) {
        // producer: bulk copies of the A and B part tiles of every K block
        int issued = 0;
        for (int kb = 0; kb < d.kb && ok; ++kb) {
            const int s = kb % TC_STAGES;
            if (kb >= TC_STAGES) ok = mbar_wait(smem_u32(&empty[s]), ((kb / TC_STAGES) - 1) & 1, err, 1);
            if (!ok) break;
            unsigned char* st = smem + s * T::STAGE;
            const uint32_t bar = smem_u32(&full[s]);
            mbar_expect_tx(bar, T::STAGE);
            const int64_t at = mbk * d.kb + kb;
            const int64_t bt = (int64_t)nbk * d.kb + kb;
#pragma unroll
            for (int p = 0; p < NS; ++p) {
                bulk_g2s(smem_u32(st + p * T::A_TILE), a.p[p] + at * (T::A_TILE / 16), T::A_TILE, bar);
                bulk_g2s(smem_u32(st + NS * T::A_TILE + p * T::B_TILE), b.p[p] + bt * (T::B_TILE / 16), T::B_TILE,
                         bar);
            }
            issued = kb + 1;
        }
        // drain: the copies of the last issued block of every stage must have landed
        // before this CTA's shared memory is released (immediate on the normal path)
        for (int kb = (issued > TC_STAGES ? issued - TC_STAGES : 0); kb < issued; ++kb)
            mbar_wait(smem_u32(&full[kb % TC_STAGES]), (kb / TC_STAGES) & 1, err, 4);
    } else if (threadIdx.x == 32) {
        // MMA issuer: the products of total order <= 1 (NS = 2) or <= 2 (NS = 3)
        constexpr int NP = TcCfg<NS>::NPROD;
        constexpr int pa[6] = {0, 0, 1, 0, 2, 1};
        constexpr int pb[6] = {0, 1, 0, 2, 0, 1};
        const uint32_t idesc = idesc_bf16(TC_BM, TC_BN);
        for (int kb = 0; kb < d.kb && ok; ++kb) {
            const int s = kb % TC_STAGES;
            ok = mbar_wait(smem_u32(&full[s]), (kb / TC_STAGES) & 1, err, 2);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t st = smem_u32(smem + s * T::STAGE);
#pragma unroll
            for (int ks = 0; ks < T::BK / 16; ++ks) {
                const uint32_t off = ks * 256;  // two core matrices along K
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const uint64_t da = smem_desc(st + pa[q] * T::A_TILE + off, 128, T::SBO);
                    const uint64_t db = smem_desc(st + NS * T::A_TILE + pb[q] * T::B_TILE + off, 128, T::SBO);
                    mma_bf16(tmem, da, db, idesc, (kb | ks | q) != 0);
                }
            }
            mma_commit(smem_u32(&empty[s]));  // stage free once these MMAs complete
        }
        mma_commit(smem_u32(done));  // accumulator complete (or all issued MMAs drained)
    }
    __syncwarp();
    // epilogue: every warp waits for the accumulator, then reads its 32 lanes
    ok = mbar_wait(smem_u32(done), 0, err, 3);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // tcgen05.ld is warp-collective: decide per warp
    const bool go = __all_sync(0xffffffffu, ok && *(volatile int*)err == 0);
    if (go) {
        const int64_t R = mbk * TC_BM + warp * 32 + lane;
        const bool row_ok = R < d.rows;
        float* dst = nullptr;
        if (row_ok) {
            const int r = (int)(R / views), j = (int)(R % views);
            dst = F + ((int64_t)j * nv + r) * d.nu;
        }
        for (int c0 = 0; c0 < TC_BN; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (row_ok) {
                const int n0 = nbk * TC_BN + c0;
                if ((d.nu & 3) == 0 && n0 + 16 <= d.nu) {  // 16-byte aligned full chunk: vector stores
                    float4* q = reinterpret_cast<float4*>(dst + n0);
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        q[i] = make_float4(v[4 * i] * du, v[4 * i + 1] * du, v[4 * i + 2] * du, v[4 * i + 3] * du);
                } else {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (n0 + i < d.nu) dst[n0 + i] = v[i] * du;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
    }
}

// Workspace layout: [A parts][B parts][flag]
template <int NS>
size_t tc_workspace(const mct_geom* g, Parts* a, Parts* b, int** flag, void* ws) {
    using T = TcTiles<NS>;
    const TcDims d = tc_dims<NS>((int64_t)g->nv * g->views, g->nu);
    const size_t as = (size_t)d.mb * d.kb * T::A_TILE, bs = (size_t)d.nb * d.kb * T::B_TILE;
    if (ws) {
        unsigned char* p = static_cast<unsigned char*>(ws);
        for (int i = 0; i < NS; ++i) {
            a->p[i] = reinterpret_cast<uint4*>(p + i * as);
            b->p[i] = reinterpret_cast<uint4*>(p + NS * as + i * bs);
        }
        *flag = reinterpret_cast<int*>(p + NS * (as + bs));
    }
    return NS * (as + bs) + 256;
}

template <int NS>
int tc_prepare(const mct_geom* g, const float* taps, void* ws, cudaStream_t s) {
    Parts a{}, b{};
    int* flag;
    tc_workspace<NS>(g, &a, &b, &flag, ws);
    const TcDims d = tc_dims<NS>((int64_t)g->nv * g->views, g->nu);
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), s);
    if (e != cudaSuccess) {
        set_error("mct_filter_tc_prepare: %s", cudaGetErrorString(e));
        return MCT_E_CUDA;
    }
    const int64_t chunks = (int64_t)d.nb * d.kb * (TcTiles<NS>::B_TILE / 16);
    const int grid = (int)std::min<int64_t>((chunks + 255) / 256, 152 * 32);
    build_b_kernel<NS><<<grid, 256, 0, s>>>(taps, g->nu, d.kb, chunks, b);
    return launched("build_b_kernel");
}

// weighted: the weighted sinogram [nv][views][nu]; or, with wp, the raw sinogram
// (strides in wp), weighted while it is split.
template <int NS>
int tc_run(const mct_geom* g, const float* weighted, void* ws, float* filtered, cudaStream_t s,
           const WeightParams* wp = nullptr, const float* bh = nullptr, const float* angles = nullptr) {
    Parts a{}, b{};
    int* flag;
    tc_workspace<NS>(g, &a, &b, &flag, ws);
    const TcDims d = tc_dims<NS>((int64_t)g->nv * g->views, g->nu);
    MCT_REQUIRE(d.mb < 65535 * 32, "mct_filter_tc: too many rows");
    const int64_t chunks = (int64_t)d.mb * d.kb * (TcTiles<NS>::A_TILE / 16);
    const int grid = (int)std::min<int64_t>((chunks + 255) / 256, 152 * 32);
    if (wp) {
        weight_split_a_kernel<NS><<<grid, 256, 0, s>>>(*wp, weighted, bh, angles, d.rows, g->nu, d.kb, chunks, a);
        MCT_TRY(launched("weight_split_a_kernel"));
    } else {
        split_a_kernel<NS><<<grid, 256, 0, s>>>(weighted, d.rows, g->nu, d.kb, chunks, a);
        MCT_TRY(launched("split_a_kernel"));
    }
    // opt in to the large dynamic shared memory (per device, idempotent)
    cudaError_t e = cudaFuncSetAttribute(tc_filter_kernel<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         TcTiles<NS>::SMEM);
    if (e != cudaSuccess) {
        set_error("mct_filter_tc: cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        return MCT_E_CUDA;
    }
    dim3 grid2(d.nb, d.mb);
    tc_filter_kernel<NS><<<grid2, 128, TcTiles<NS>::SMEM, s>>>(d, g->nv, g->views, g->du, a, b, filtered, flag);
    return launched("tc_filter_kernel");
}

}  // namespace
}  // namespace mct

using namespace mct;

extern "C" {

size_t mct_filter_tc_workspace_size(const mct_geom* g, int32_t dtype) {
    if (!g || g->nu < 2 || g->nv < 1 || g->views < 1 || (dtype != MCT_F32 && dtype != MCT_BF16)) return 0;
    Parts a, b;
    int* f;
    return dtype == MCT_F32 ? tc_workspace<3>(g, &a, &b, &f, nullptr) : tc_workspace<2>(g, &a, &b, &f, nullptr);
}

int mct_filter_tc_prepare(const mct_geom* g, const float* taps, int32_t dtype, void* workspace, void* stream) {
    MCT_TRY(check_geom(g, "mct_filter_tc_prepare"));
    MCT_REQUIRE(taps && workspace, "mct_filter_tc_prepare: NULL buffer");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16, "mct_filter_tc_prepare: dtype must be MCT_F32 or MCT_BF16");
    MCT_REQUIRE(((uintptr_t)workspace & 1023) == 0, "mct_filter_tc_prepare: workspace must be 1 KiB aligned");
    return dtype == MCT_F32 ? tc_prepare<3>(g, taps, workspace, as_stream(stream))
                            : tc_prepare<2>(g, taps, workspace, as_stream(stream));
}

int mct_filter_tc(const mct_geom* g, const float* weighted, int32_t dtype, void* workspace, float* filtered,
                  void* stream) {
    MCT_TRY(check_geom(g, "mct_filter_tc"));
    MCT_REQUIRE(weighted && workspace && filtered, "mct_filter_tc: NULL buffer");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16, "mct_filter_tc: dtype must be MCT_F32 or MCT_BF16");
    MCT_REQUIRE(((uintptr_t)workspace & 1023) == 0, "mct_filter_tc: workspace must be 1 KiB aligned");
    return dtype == MCT_F32 ? tc_run<3>(g, weighted, workspace, filtered, as_stream(stream))
                            : tc_run<2>(g, weighted, workspace, filtered, as_stream(stream));
}

int mct_weight_filter(const mct_geom* g, const mct_tables* t, const float* sgm, int64_t row_stride,
                      int64_t view_stride, const float* bh_coeffs, int32_t n_bh, int32_t dtype, void* workspace,
                      float* filtered, void* stream) {
    MCT_TRY(check_geom(g, "mct_weight_filter"));
    MCT_REQUIRE(sgm && workspace && filtered, "mct_weight_filter: NULL buffer");
    MCT_REQUIRE(n_bh >= 0 && (n_bh == 0 || bh_coeffs), "mct_weight_filter: bad BH coefficients");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16, "mct_weight_filter: dtype must be MCT_F32 or MCT_BF16");
    MCT_REQUIRE(((uintptr_t)workspace & 1023) == 0, "mct_weight_filter: workspace must be 1 KiB aligned");
    const bool short_scan = (g->flags & MCT_SHORT_SCAN) != 0;
    MCT_REQUIRE(!short_scan || (t && t->angles), "mct_weight_filter: short scan needs the angle table");
    MCT_REQUIRE(row_stride >= 0 && view_stride >= 0, "mct_weight_filter: negative stride");
    const WeightParams wp = weight_params(g, row_stride, view_stride, n_bh);
    const float* angles = t ? t->angles : nullptr;
    cudaStream_t s = as_stream(stream);
    return dtype == MCT_F32 ? tc_run<3>(g, sgm, workspace, filtered, s, &wp, bh_coeffs, angles)
                            : tc_run<2>(g, sgm, workspace, filtered, s, &wp, bh_coeffs, angles);
}

// 0 if no tensor-core filter launch on this workspace has timed out, else MCT_E_TIMEOUT
// (synchronises the stream).
int mct_filter_tc_status(const mct_geom* g, int32_t dtype, void* workspace, void* stream) {
    MCT_REQUIRE(g && workspace, "mct_filter_tc_status: NULL argument");
    MCT_REQUIRE(dtype == MCT_F32 || dtype == MCT_BF16, "mct_filter_tc_status: dtype must be MCT_F32 or MCT_BF16");
    Parts a, b;
    int* flag;
    if (dtype == MCT_F32) tc_workspace<3>(g, &a, &b, &flag, workspace);
    else tc_workspace<2>(g, &a, &b, &flag, workspace);
    int h = 0;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("mct_filter_tc_status: %s", cudaGetErrorString(e));
        return MCT_E_CUDA;
    }
    if (h != 0) {
        set_error("mct_filter_tc: a pipeline wait timed out (stage %d)", h);
        return MCT_E_TIMEOUT;
    }
    return MCT_OK;
}

}  // extern "C"
