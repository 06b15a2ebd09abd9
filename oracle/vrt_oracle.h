/*
 * vrt_oracle.h - CPU oracle for the brickmap traversal path.  TEST INFRASTRUCTURE:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as
 * the checker and the timed CPU baseline; the library never links it.
 *
 * It restates, as scalar per-ray C++, the reference CPU path:
 *   FlatVoxelStorage + SyncBuffers + UpdateOccupancy  src/VoxelRT/CpuRenderer.cpp:20-83
 *   GetInboundMask / GetVoxelMaterial                  src/VoxelRT/CpuRenderer.cpp:114-132
 *   GetStepPos / RayCast                               src/VoxelRT/CpuRenderer.cpp:135-224
 * with the SIMD primitive semantics of src/LibGlimpsw/SwRast/SIMD_AVX512.h:109,123
 * (floor2i, minps) and the ray-entry clip of src/VoxelRT/Shaders/VoxelTraversal.glsl:133-145.
 * Edits follow VoxelMap::RegionDispatchSIMD + GC (src/VoxelRT/VoxelMap.h:222-263).
 * Parity is pinned against the reference's own RayCast compiled in place
 * (oracle/ref_pin/, x86 only) through the committed fixtures in tests/golden/.
 * The GLSL mode (VRT_CAST_GLSL / VRT_VIEW_GLSL) restates the GPU renderer's rayCast
 * (src/VoxelRT/Shaders/VoxelTraversal.glsl:100-204); its parity is unpinned, as the
 * shader cannot run here.
 */
#ifndef VRT_ORACLE_H_
#define VRT_ORACLE_H_

#include <stdint.h>
#include "../include/vrt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_world ora_world;

/* Traversal counters summed over a batch: rays, GetStepPos calls, calls that
 * fetched a voxel-cell mask (brick bit set), hits. */
typedef struct ora_stats {
    uint64_t rays;
    uint64_t step_calls;
    uint64_t occ_fetches;
    uint64_t hits;
} ora_stats;

ora_world* ora_world_create(uint32_t sectors_x, uint32_t sectors_y, uint32_t sectors_z);
void ora_world_destroy(ora_world* w);
/* Same record semantics as vrt_world_sync_sectors. Returns 0 or -1 on a bad stream. */
int ora_world_sync(ora_world* w, uint32_t n, const int32_t* sector_idx, const uint64_t* alloc_mask,
                   const uint64_t* dirty_mask, const uint8_t* bricks);
uint64_t ora_world_sector_mask(const ora_world* w, int32_t sector_idx);
int ora_world_read_sector(const ora_world* w, int32_t sector_idx, uint64_t* mask, uint8_t* bricks);
uint8_t ora_world_get_voxel(const ora_world* w, int32_t x, int32_t y, int32_t z);
/* 8 cell masks of one brick as UpdateOccupancy derives them (0 if not allocated). */
int ora_world_brick_occupancy(const ora_world* w, int32_t bx, int32_t by, int32_t bz, uint64_t out[8]);
uint64_t ora_world_allocated_bricks(const ora_world* w);

/* Cast explicit rays. threads = 0 uses every hardware thread. stats may be NULL. */
int ora_cast(const ora_world* w, const vrt_ray* rays, uint64_t n, const vrt_cast_params* params,
             vrt_hit* hits, int threads, ora_stats* stats);
/* Camera rays of a view (the ray generation of vrt_camera). */
int ora_camera_rays(const vrt_camera* cam, vrt_ray* rays);
/* RayCellInteractionMaskLUT (GpuRenderer.cpp:193-210): 512 masks, entry idx + octant*64. */
int ora_ray_cell_lut(uint64_t* out);

/* mode: 0 = the reference CPU traversal, 1 = the GLSL mode (VRT_VIEW_GLSL), 3 = the GLSL
 * mode with anisotropic LODs (VRT_VIEW_GLSL_ANISO). */
int ora_render_view(const ora_world* w, const vrt_camera* cam, uint32_t max_iters, uint32_t mode, vrt_hit* hits,
                    int threads, ora_stats* stats);
/* Primary ray, then for every hit one shadow ray from hitPos + normal*0.01
 * (CpuRenderer.cpp:389) toward sun_dir.  shadow[i] for a primary miss is a miss
 * record with steps 0 and tag VRT_NO_RAY. */
int ora_render_view_shadow(const ora_world* w, const vrt_camera* cam, const float sun_dir[3],
                           uint32_t max_iters, uint32_t mode, vrt_hit* primary, vrt_hit* shadow, int threads,
                           ora_stats* stats);
/* Primary ray plus up to n_bounces diffuse bounces per pixel (CpuRenderer.cpp:342-393):
 * origin hitPos + normal*0.01, direction normalize(normal + s) with s uniform on the
 * unit sphere, drawn by rejection from the cube [-1,1]^3 with PCG32 seeded by
 * pixel ^ bounce (IEEE +,*,/,sqrt only, so the device reproduces it bit for bit).
 * hits has (n_bounces+1)*width*height records, bounce-major; a path stops at its
 * first miss and later records are VRT_NO_RAY misses. */
int ora_render_view_bounces(const ora_world* w, const vrt_camera* cam, uint32_t n_bounces,
                            uint32_t max_iters, uint32_t mode, vrt_hit* hits, int threads, ora_stats* stats);

/* The GPU renderer's per-pixel path with u_MaxBounces = n_bounces (1..15), VoxelRender.comp:51-86:
 * primary; sun ray from its hit; bounces 1..n (stop at the first miss), the first two each
 * followed by a sun ray.  Planes [primary][sun 0][bounce 1][sun 1][bounce 2][sun 2][bounce 3]..
 * [bounce n] (2 + n + min(n, 2) of them), VRT_NO_RAY where no ray was cast. */
int ora_render_view_path(const ora_world* w, const vrt_camera* cam, const float sun_dir[3], uint32_t n_bounces,
                         uint32_t max_iters, uint32_t mode, vrt_hit* hits, int threads, ora_stats* stats);
/* G-buffer of the primary hits (VoxelRender.comp:39-46,91-93): RGBA8 albedo + packed normal
 * and projected depth per pixel (vrt_render_gbuffer_device's contract); hits may be NULL. */
int ora_render_gbuffer(const ora_world* w, const vrt_camera* cam, uint32_t max_iters, uint32_t mode,
                       const uint32_t* palette, const float* proj, uint32_t* albedo_normal, float* depth, vrt_hit* hits,
                       int threads);

/* Picking ray cast (VoxelMap::RayCast, VoxelMap.cpp:125-170), double precision.
 * rays: 6 doubles each (origin, dir).  max_iters 0 = 1024. */
int ora_pick(const ora_world* w, const double* rays, uint64_t n, uint32_t max_iters, vrt_pick_hit* hits);

/* Apply sphere edits in order with the reference's region dispatch + empty-brick GC. */
int ora_world_edit(ora_world* w, const vrt_edit* edits, uint32_t n);

#ifdef __cplusplus
}
#endif
#endif
