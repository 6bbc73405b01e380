// Library-level entry points: version, error text, launch counter, shared checks.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "common.cuh"

namespace mct {

static thread_local char g_err[512] = "";
static std::atomic<uint64_t> g_launches{0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int check_geom(const mct_geom* g, const char* who) {
    MCT_REQUIRE(g != nullptr, "%s: geometry is NULL", who);
    MCT_REQUIRE(g->nu >= 2 && g->views >= 1 && g->nv >= 1, "%s: bad detector size nu=%d nv=%d views=%d",
                who, g->nu, g->nv, g->views);
    MCT_REQUIRE(g->nx >= 2 && g->nz >= 1, "%s: bad image size nx=%d nz=%d", who, g->nx, g->nz);
    MCT_REQUIRE((int64_t)g->nu * g->nv * g->views < (int64_t)1 << 40, "%s: sinogram too large", who);
    MCT_REQUIRE(g->view_mode >= 1 && g->view_mode <= 3, "%s: view_mode must be 1, 2 or 3", who);
    MCT_REQUIRE(g->view_begin >= 0 && (g->views_total == 0 || g->view_begin + g->views <= g->views_total),
                "%s: view chunk [%d, %d) outside the scan's %d views", who, g->view_begin, g->view_begin + g->views,
                g->views_total);
    MCT_REQUIRE(g->views_total == 0 || g->views_total >= 2 || g->view_begin == 0, "%s: bad views_total", who);
    return MCT_OK;
}

double div_factor(const mct_geom& g) {
    const double PI = kPI;
    double tsa = std::fabs((double)g.total_scan_angle);
    double num_rounds = std::floor(tsa / (PI * 2));
    double div = 1.0;
    if (g.flags & MCT_SHORT_SCAN) {
        double remain = tsa - num_rounds * 2 * PI;
        if (tsa < 2 * PI) div = 1.0;
        else if (remain < PI) div = 1.0 / (num_rounds * 2.0);
        else if (PI < remain && remain < 2 * PI) div = 1.0 / (num_rounds * 2.0 + 1.0);
    } else {
        div = 1.0 / (num_rounds * 2.0);
    }
    return div;
}

// Entry points that do not take view chunks (everything but weighting and FDK
// backprojection) reject them.
int check_whole_scan(const mct_geom* g, const char* who) {
    MCT_REQUIRE(g->view_begin == 0 && (g->views_total == 0 || g->views_total == g->views),
                "%s: view-chunked geometry is only supported by mct_weight and mct_fdk_bp", who);
    return MCT_OK;
}

}  // namespace mct

extern "C" {

const char* mct_version(void) { return "mandoct-gb300 0.1 (sm_103a)"; }

const char* mct_last_error_string(void) { return mct::g_err; }

uint64_t mct_launch_count(void) { return mct::g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
