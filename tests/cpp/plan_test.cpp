// plan_test.cpp - the batch planner of libvrt.so on the host, no GPU needed: the launch
// config fields left to the library, and the layout of views behind one tile queue.
// Links libvrt.so and calls its internal planner (vrt::normalize_batch_config,
// vrt::resolve_batch_defaults, vrt::plan_views); prints FAIL lines and exits non-zero
// on a mismatch.
#include <cstdio>
#include <vector>

#include "batch_internal.h"

using namespace vrt;

static int fails = 0;
#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c);       \
            fails++;                                                      \
        }                                                                 \
    } while (0)

static vrt_view make(uint32_t w, uint32_t h, uint32_t world = 0, uint32_t bounces = 0, uint32_t flags = 0) {
    vrt_view v{};
    v.cam.width = w;
    v.cam.height = h;
    v.cam.d0[2] = 1.0f;
    v.cam.du[0] = 1.0f / w;
    v.cam.dv[1] = 1.0f / h;
    v.world = world;
    v.n_bounces = bounces;
    v.flags = flags;
    if (flags & VRT_VIEW_SHADOW) v.sun_dir[1] = 1.0f;
    return v;
}

static uint64_t tiles_of(const vrt_view& v, uint32_t tw, uint32_t th) {
    return (uint64_t)((v.cam.width + tw - 1) / tw) * ((v.cam.height + th - 1) / th);
}

int main() {
    // a zeroed config: 8x8 tiles, 4 warps, 16-step rounds; refill and chunk left open
    vrt_batch_config cfg{};
    CHECK(normalize_batch_config(nullptr, cfg) == VRT_OK);
    CHECK(cfg.tile_w == 8 && cfg.tile_h == 8 && cfg.warps_per_block == 4 && cfg.inner_iters == 16);
    CHECK(cfg.refill_threshold == 0 && cfg.chunk_tiles == 0);
    vrt_batch_config bad{};
    bad.tile_w = 4;
    bad.tile_h = 4;
    CHECK(normalize_batch_config(&bad, cfg) == VRT_ERR_INVALID_ARG);
    bad = vrt_batch_config{};
    bad.refill_threshold = 33;
    CHECK(normalize_batch_config(&bad, cfg) == VRT_ERR_INVALID_ARG);

    // chunk size per launch: about eight fetches per warp, 1..16 tiles
    CHECK(auto_chunk_tiles(5513, 0) == 1);
    CHECK(auto_chunk_tiles(100, 4256) == 1);
    CHECK(auto_chunk_tiles(100000, 1000) == 12);
    CHECK(auto_chunk_tiles(5514240, 4256) == 16);

    // defaults follow the views: diffuse bounces refill below 28 and claim single tiles
    std::vector<vrt_view> cams = {make(1280, 720), make(64, 64, 0, 0, VRT_VIEW_SHADOW)};
    std::vector<vrt_view> bounce = {make(1280, 720, 0, 4)};
    vrt_batch_config c{};
    normalize_batch_config(nullptr, c);
    vrt_batch_config r = c;
    resolve_batch_defaults(r, cams.data(), (uint32_t)cams.size(), 1000);
    const uint64_t t = tiles_of(cams[0], 8, 8) + tiles_of(cams[1], 8, 8);
    CHECK(r.refill_threshold == 16 && r.chunk_tiles == auto_chunk_tiles(t, 1000));
    r = c;
    resolve_batch_defaults(r, bounce.data(), 1, 1000);
    CHECK(r.refill_threshold == 28 && r.chunk_tiles == 1);
    r = c;
    resolve_batch_defaults(r, nullptr, 0, 0);  // a resident launch before its views arrive
    CHECK(r.refill_threshold == 16 && r.chunk_tiles == 1);
    r = c;
    r.refill_threshold = 5;
    r.chunk_tiles = 3;
    resolve_batch_defaults(r, bounce.data(), 1, 1000);  // values a caller set are kept
    CHECK(r.refill_threshold == 5 && r.chunk_tiles == 3);

    // record planes per view: primary; sun; bounces; the renderer's whole path
    CHECK(view_record_count(make(10, 10)) == 100);
    CHECK(view_record_count(make(10, 10, 0, 0, VRT_VIEW_SHADOW)) == 200);
    CHECK(view_record_count(make(10, 10, 0, 4)) == 500);
    CHECK(view_record_count(make(10, 10, 0, 3, VRT_VIEW_SHADOW)) == 700);

    // queue and record layout: ragged views, 16x4 tiles, explicit chunk size
    std::vector<vrt_view> views = {make(64, 64), make(100, 37, 1, 0, VRT_VIEW_SHADOW), make(1280, 720, 0, 2),
                                   make(1, 1, 1)};
    vrt_batch_config lc{};
    lc.tile_w = 16;
    lc.tile_h = 4;
    lc.chunk_tiles = 4;
    lc.refill_threshold = 20;
    CHECK(normalize_batch_config(&lc, lc) == VRT_OK);
    LaunchPlan plan;
    CHECK(plan_views(views.data(), (uint32_t)views.size(), 2, lc, plan, 100) == VRT_OK);
    CHECK(plan.cfg.chunk_tiles == 4 && plan.cfg.refill_threshold == 20);
    CHECK(plan.tile_w_log2 == 4 && plan.tile_size_log2 == 6);
    uint64_t chunks = 0, records = 0;
    for (size_t i = 0; i < views.size(); i++) {
        const uint64_t tiles = tiles_of(views[i], 16, 4);
        CHECK(plan.chunk_base[i] == chunks);
        CHECK(plan.views[i].chunk_base == chunks);
        CHECK(plan.views[i].n_rays == tiles * 64);
        CHECK(plan.views[i].tiles_x == (views[i].cam.width + 15) / 16);
        CHECK(plan.views[i].out_base == records);
        chunks += (tiles + 3) / 4;
        records += view_record_count(views[i]);
    }
    CHECK(plan.chunk_base[views.size()] == chunks && plan.chunks == chunks && plan.records == records);
    CHECK(!plan.glsl && !plan.aniso && !plan.full);

    // left to the library: resolved in the plan
    LaunchPlan p2;
    CHECK(plan_views(bounce.data(), 1, 1, c, p2, 1000) == VRT_OK);
    CHECK(p2.cfg.refill_threshold == 28 && p2.cfg.chunk_tiles == 1 && p2.chunks == tiles_of(bounce[0], 8, 8));

    // refusals: a world outside the list, mixed traversal modes, a bad view
    LaunchPlan p3;
    CHECK(plan_views(views.data(), (uint32_t)views.size(), 1, lc, p3, 100) == VRT_ERR_INVALID_ARG);
    std::vector<vrt_view> mixed = {make(8, 8), make(8, 8, 0, 0, VRT_VIEW_GLSL)};
    CHECK(plan_views(mixed.data(), 2, 1, lc, p3, 100) == VRT_ERR_INVALID_ARG);
    std::vector<vrt_view> big = {make(20000, 8)};
    CHECK(plan_views(big.data(), 1, 1, lc, p3, 100) == VRT_ERR_INVALID_ARG);
    std::vector<vrt_view> deep = {make(8, 8, 0, 16)};
    CHECK(plan_views(deep.data(), 1, 1, lc, p3, 100) == VRT_ERR_INVALID_ARG);

    std::printf("%s: %d failures\n", fails ? "FAIL" : "ok", fails);
    return fails ? 1 : 0;
}
