// Helical cone-beam to per-slice fan-beam rebinning (Mgfbp_helical.SinogramRebinning,
// run_mgfbp_helical.py:178-205), for every reconstructed slice in one launch.
//
// The reference rebins one slice at a time on the host loop (one kernel launch, one
// host round trip and one temporary file per slice).  Here one thread produces one
// element out[s][i][c] of the whole stack of rebinned fan sinograms; a warp covers 32
// consecutive detector columns of one (slice, view), so both the two source rows it
// reads and the element it writes are coalesced.
#include <cmath>

#include "common.cuh"

namespace mct {
namespace {

__global__ void helical_rebin_kernel(mct_helical h, const float* __restrict__ sgm, const float* __restrict__ z_pos,
                                     float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;   // rebinned view
    const int s = blockIdx.z;   // slice
    if (c >= h.nu) return;
    const float z = z_pos[s];
    // float32 throughout, as the reference's Taichi kernel computes
    const float view_idx_v_equal_0 = (z - h.det_offset_vertical / h.mag) / h.dis_per_view;
    const float view_begin = floorf(view_idx_v_equal_0 - 0.5f * (float)h.view_count + 0.5f);
    const float view_idx = view_begin + (float)i;
    float val = 0.0f;
    if (0.0f <= view_idx && view_idx <= (float)(h.views - 2)) {
        const float v_pos = (z - view_idx * h.dis_per_view) * h.mag - h.det_offset_vertical;
        const float v_idx = -v_pos / h.dv + ((float)h.nv - 1.0f) / 2.0f;
        const int64_t col = (int64_t)(int)view_idx * h.nu + c;
        const int64_t row_stride = (int64_t)h.views * h.nu;
        if (v_idx >= (float)(h.nv - 1)) {
            val = sgm[(int64_t)(h.nv - 1) * row_stride + col];
        } else if (v_idx <= 0.0f) {
            val = sgm[col];
        } else {
            const float vf = floorf(v_idx);
            const float w = v_idx - vf;
            const int r = (int)vf;
            const float d1 = sgm[(int64_t)r * row_stride + col], d2 = sgm[(int64_t)(r + 1) * row_stride + col];
            val = d1 * (1.0f - w) + d2 * w;
        }
        val *= h.sdd / sqrtf(h.sdd * h.sdd + v_pos * v_pos);
    }
    out[((int64_t)s * h.view_count + i) * h.nu + c] = val;
}

}  // namespace
}  // namespace mct

using namespace mct;

extern "C" int mct_helical_rebin(const mct_helical* h, const float* sgm, const float* z_pos, float* out,
                                 void* stream) {
    MCT_REQUIRE(h && sgm && z_pos && out, "mct_helical_rebin: NULL argument");
    MCT_REQUIRE(h->nu >= 1 && h->nv >= 1 && h->views >= 2 && h->view_count >= 1 && h->n_slices >= 1,
                "mct_helical_rebin: bad sizes nu=%d nv=%d views=%d view_count=%d slices=%d", h->nu, h->nv, h->views,
                h->view_count, h->n_slices);
    MCT_REQUIRE(h->view_count <= 65535 && h->n_slices <= 65535, "mct_helical_rebin: too many views or slices");
    MCT_REQUIRE(h->dv != 0.0f && h->dis_per_view != 0.0f && h->mag != 0.0f, "mct_helical_rebin: zero spacing");
    dim3 block(128), grid((h->nu + 127) / 128, h->view_count, h->n_slices);
    helical_rebin_kernel<<<grid, block, 0, as_stream(stream)>>>(*h, sgm, z_pos, out);
    return launched("helical_rebin_kernel");
}
