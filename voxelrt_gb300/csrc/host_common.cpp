// host_common.cpp - host code compiled into both libvrt.so and the host-only
// libvrt_synth.so: the thread-local error message, the sector-stream release and the
// camera builder.  Each library holds its own copy (and its own error message).

#include <cmath>
#include <cstdlib>
#include <string>

#include "../../include/vrt.h"

namespace vrt {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }

}  // namespace vrt

extern "C" {

void vrt_sector_stream_free(vrt_sector_stream* s) {
    if (!s) return;
    std::free(s->sector_idx);
    std::free(s->alloc_mask);
    std::free(s->bricks);
    std::free(s);
}

vrt_status vrt_camera_look_at(const double pos[3], const double target[3], double vfov_deg, uint32_t width,
                              uint32_t height, vrt_camera* out) {
    if (!pos || !target || !out || width == 0 || height == 0 || !(vfov_deg > 0.0 && vfov_deg < 180.0)) {
        vrt::set_error("bad camera arguments");
        return VRT_ERR_INVALID_ARG;
    }
    double f[3] = {target[0] - pos[0], target[1] - pos[1], target[2] - pos[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0.0)) {
        vrt::set_error("camera target equals position");
        return VRT_ERR_INVALID_ARG;
    }
    for (double& c : f) c /= fl;
    // right = forward x worldUp (y up); fall back to z when looking straight up/down
    double up[3] = {0.0, 1.0, 0.0};
    if (std::fabs(f[1]) > 0.999999) {
        up[1] = 0.0;
        up[2] = 1.0;
    }
    double r[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    double rl = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (double& c : r) c /= rl;
    double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    const double th = std::tan(vfov_deg * 0.5 * 3.14159265358979323846 / 180.0);
    const double aspect = (double)width / (double)height;
    for (int c = 0; c < 3; c++) {
        const double fp = std::floor(pos[c]);
        out->world_origin[c] = (int32_t)fp;
        out->origin[c] = (float)(pos[c] - fp);
        out->d0[c] = (float)(f[c] - r[c] * th * aspect + u[c] * th);
        out->du[c] = (float)(r[c] * (2.0 * th * aspect / width));
        out->dv[c] = (float)(-u[c] * (2.0 * th / height));
    }
    out->width = width;
    out->height = height;
    return VRT_OK;
}

}  // extern "C"
