/*
 * vrt.h - C ABI of the GB300 brickmap ray-traversal library (libvrt.so).
 *
 * The library replaces the storage-sync and traversal path of VoxelRT:
 *   - the device-layout storage that GpuVoxelStorage::SyncBuffers(VoxelMap&)
 *     (src/VoxelRT/GpuRenderer.cpp:45-167) and FlatVoxelStorage::SyncBuffers
 *     (src/VoxelRT/CpuRenderer.cpp:33-61) build from the host VoxelMap;
 *   - the mask re-derivation of UpdateOccupancy (src/VoxelRT/CpuRenderer.cpp:63-83,
 *     src/VoxelRT/Shaders/UpdateOccupancy.comp:9-34);
 *   - the traversal RayCast/GetStepPos (src/VoxelRT/CpuRenderer.cpp:135-224) and
 *     its GLSL twin rayCast (src/VoxelRT/Shaders/VoxelTraversal.glsl:162-204),
 *     driven per view as GpuRenderer::RenderFrame does (GpuRenderer.cpp:239-273);
 *   - the edit path VoxelMap::RegionDispatchSIMD + brick GC
 *     (src/VoxelRT/VoxelMap.h:222-263) and BrickSlotAllocator
 *     (src/VoxelRT/BrickSlotAllocator.cpp:5-94).
 *
 * Conventions (all fixed by the reference's indexers, src/VoxelRT/VoxelMap.h:60-102):
 *   - a brick is 8x8x8 u8 voxel ids, 0 = empty; voxel index x | z<<3 | y<<6;
 *   - a sector is 4x4x4 bricks; brick index bx | bz<<2 | by<<4 is the bit in the
 *     sector's 64-bit allocation mask;
 *   - sector indices passed to the ABI use the reference's WorldSectorIndexer
 *     packing (12-bit signed x, 12-bit signed z at bit 12, 8-bit signed y at bit
 *     24); sectors outside the world's extent are ignored, as SyncBuffers skips
 *     sectors outside its view (GpuRenderer.cpp:53-55, CpuRenderer.cpp:39-40).
 *
 * Errors are returned as vrt_status codes; nothing throws across the ABI.
 * vrt_last_error() returns a thread-local message for the last failure.
 *
 * Every function taking a `stream` takes a cudaStream_t passed as void*
 * (NULL = legacy default stream).  Functions with host buffers synchronise that
 * stream before returning; *_device variants are asynchronous on it.
 *
 * A call on a world, batch or server makes that object's device current while it
 * runs and gives the calling thread's current device back when it returns.
 */
#ifndef VRT_H_
#define VRT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VRT_ABI_VERSION 1

typedef enum vrt_status {
    VRT_OK = 0,
    VRT_ERR_INVALID_ARG = 1,     /* bad pointer, size or descriptor */
    VRT_ERR_OUT_OF_MEMORY = 2,   /* device or host allocation failed, or admission refused */
    VRT_ERR_QUEUE_TIMEOUT = 3,   /* a bounded device or host wait gave up */
    VRT_ERR_DEVICE = 4,          /* CUDA runtime error; see vrt_last_error() */
    VRT_ERR_NO_DEVICE = 5,       /* no CUDA device */
    VRT_ERR_SLOTS_EXHAUSTED = 6, /* brick pool full: BrickSlotAllocator.cpp:14-16 throws here */
    VRT_ERR_NOT_FOUND = 7,
    VRT_ERR_IO = 8,
    VRT_ERR_FORMAT = 9           /* malformed stream or file */
} vrt_status;

/* ---- layout constants (VoxelMap.h:100-102) ---- */
#define VRT_BRICK_DIM 8
#define VRT_BRICK_BYTES 512
#define VRT_SECTOR_DIM_BRICKS 4
#define VRT_SECTOR_DIM 32
/* Largest world: hit voxels are packed 11/10/11 bits (x | y<<11 | z<<21). */
#define VRT_MAX_WORLD_X 2048
#define VRT_MAX_WORLD_Y 1024
#define VRT_MAX_WORLD_Z 2048

#define VRT_DEFAULT_MAX_ITERS 128 /* CpuRenderer.cpp:185 */
#define VRT_MISS_VOXEL 0xFFFFFFFFu
#define VRT_MISS_FACE 0xFFu

/* Ray in the frame of an integer world origin (CpuRenderer.cpp:172: origin is
 * relative to worldOrigin; voxel = worldOrigin + floor(pos)). 32 bytes. */
typedef struct vrt_ray {
    float origin[3];
    float dir[3];
    uint32_t tag;      /* copied to vrt_hit.tag */
    uint32_t reserved; /* must be 0 */
} vrt_ray;

/* Hit record, 16 bytes.
 *   voxel    hit voxel in world coordinates packed x | y<<11 | z<<21, or VRT_MISS_VOXEL
 *   face     axis*2 + (dir[axis] < 0), axis = X if sideX==t, else Y if sideY==t, else Z
 *            (CpuRenderer.cpp:204-207); VRT_MISS_FACE on a miss
 *   material voxel id (u8), 0 on a miss
 *   steps    DDA iteration at which the ray left the active set (hit or out of
 *            bounds); max_iters when the iteration cap ran out
 *   t        hit distance min(sideX, sideY, sideZ) (CpuRenderer.cpp:204); +inf on a miss
 *   tag      vrt_ray.tag, or the pixel index y*width+x for camera rays          */
typedef struct vrt_hit {
    uint32_t voxel;
    uint8_t face;
    uint8_t material;
    uint16_t steps;
    float t;
    uint32_t tag;
} vrt_hit;

/* Hit record without its tag, 12 bytes: the per-ray output (voxel, face, material, steps,
 * t) in the fields and encoding of vrt_hit.  vrt_batch_run_packed delivers these: a
 * view's records are in pixel order, so a record's position gives the pixel its tag
 * would name.  A record whose ray was never cast (VRT_NO_RAY in vrt_hit.tag: the shadow
 * or bounce records after a path ended) keeps the miss fields with material
 * VRT_PACKED_NO_RAY; a miss that was cast always has material 0. */
typedef struct vrt_hit_packed {
    uint32_t voxel;
    uint8_t face;
    uint8_t material;
    uint16_t steps;
    float t;
} vrt_hit_packed;
#define VRT_PACKED_NO_RAY 0xFFu

typedef struct vrt_cast_params {
    int32_t world_origin[3]; /* FrameConstants::WorldOrigin (CpuRenderer.cpp:447) */
    uint32_t max_iters;      /* 0 = VRT_DEFAULT_MAX_ITERS (VRT_GLSL_MAX_ITERS in GLSL mode); at most 65535 */
    uint32_t flags;          /* 0, or VRT_CAST_GLSL with VRT_CAST_GLSL_COARSE and/or VRT_CAST_GLSL_ANISO */
} vrt_cast_params;

/* Traversal modes.  The default is the reference CPU traversal (CpuRenderer.cpp:135-224,
 * the pinned contract above).  The GLSL mode is the GPU renderer's rayCast
 * (Shaders/VoxelTraversal.glsl:100-204) with anisotropic LODs off:
 *   - a 4th level: where a sector holds no brick, the mask of its 4^3 group of sectors
 *     (bit set per non-empty sector, GpuRenderer.cpp:139-149) gives cells of 32, 64 or
 *     128 voxels;
 *   - each iteration first takes the side distances of the current voxel (the start
 *     voxel on iteration 0, which is therefore never tested), then
 *     tmin = min(sides) + 5 ulp (integer add on the bits; a NaN tmin stays NaN, as the
 *     bits of a NaN differ between platforms), pos = origin + tmin*dir,
 *     voxel = worldOrigin + floor(pos), bounds, getStepPos;
 *   - a hit reports t = the biased tmin and face = the first axis with tmin >= side;
 *     secondary rays start at pos + normal*0.01 with normal = -sign(dir) on every such
 *     axis (sign(0) = 0);
 *   - the iteration cap defaults to VRT_GLSL_MAX_ITERS.
 * The GPU renderer casts shadow and bounce rays with rayCastCoarse instead
 * (VoxelTraversal.glsl:206-240, VoxelRender.comp:56,74,81), and so do the secondary
 * rays of VRT_VIEW_GLSL views and casts with VRT_CAST_GLSL_COARSE:
 *   - the entry-clipped start replaces the ray origin: tStart, positions and the
 *     reported t count from it (rayCast keeps the origin and clips the start voxel);
 *   - tmin = min(sides) + 0.001 instead of + 5 ulp;
 *   - from iteration 31 on, an empty voxel whose 4^3 cell holds a solid voxel ends
 *     the ray as a hit on the cell's first solid voxel in mask order (x, then z, then
 *     y; getStepPos with coarse, findAnyOccupiedPos): that voxel and its material are
 *     reported;
 *   - the iteration cap is VRT_GLSL_COARSE_MAX_ITERS (or a smaller max_iters).
 * Entry clip, bounds (per axis, the world's extent) and the x86 min/floor rules are
 * shared with the default mode. */
#define VRT_CAST_GLSL 1u
#define VRT_CAST_GLSL_COARSE 2u
/* With VRT_CAST_GLSL (or on a view, VRT_VIEW_GLSL_ANISO with VRT_VIEW_GLSL): the GPU
 * renderer's anisotropic LODs (u_UseAnisotropicLods, off by default there;
 * VoxelTraversal.glsl:116-121): getStepPos restricts the occupancy mask of the level it
 * reads (4^3 cell, sector or sector group) to the cells ahead of the ray in its octant
 * (RayCellInteractionMaskLUT, GpuRenderer.cpp:193-210) before taking its LOD. */
#define VRT_CAST_GLSL_ANISO 4u
#define VRT_GLSL_MAX_ITERS 256
#define VRT_GLSL_COARSE_MAX_ITERS 96

/* Pinhole camera in the reference's split form: integer world origin plus a
 * fractional ray origin (GBuffer.h:79, CpuRenderer.cpp:447-448).  The ray of
 * pixel (px, py), u = px + 0.5, v = py + 0.5, has unnormalised direction
 * d0 + u*du + v*dv (each op rounded separately), multiplied per component by
 * r = 1/sqrt(l2), l2 = (x*x + y*y) + z*z, computed as: r = bits 0x5F3759DF -
 * (bits(l2) >> 1), then three times r = r * fma(-(0.5*l2), r*r, 1.5) (every op IEEE
 * round-to-nearest, so any machine reproduces the direction bit for bit; within 3 ulp
 * of unit length).  Build one with vrt_camera_look_at(). */
typedef struct vrt_camera {
    int32_t world_origin[3];
    float origin[3];
    float d0[3];
    float du[3];
    float dv[3];
    uint32_t width;
    uint32_t height;
} vrt_camera;

/* Marks records of rays that were never cast (shadow rays of missed pixels,
 * bounces after a path ended). */
#define VRT_NO_RAY 0xFFFFFFFFu

/* Sphere edit (the brush of Brush.cpp:10-31 with an exact integer sphere):
 * every voxel v with |v - center|^2 <= radius^2 (integer arithmetic) is set to
 * `material` (0 carves).  mode VRT_EDIT_REPLACE only overwrites non-empty voxels
 * (BrushAction::Replace, Brush.cpp:24-26).  Bricks are created for fills and
 * every empty brick in the edit's brick bounding box is freed afterwards
 * (VoxelMap.h:222-263).  Voxels outside the world are ignored. */
typedef struct vrt_edit {
    int32_t center[3];
    uint32_t radius;
    uint8_t material;
    uint8_t mode;
    uint16_t reserved; /* must be 0 */
} vrt_edit;

#define VRT_EDIT_FILL 0
#define VRT_EDIT_REPLACE 1

typedef struct vrt_world vrt_world;

typedef struct vrt_world_desc {
    uint32_t sectors_x, sectors_y, sectors_z; /* world extent in 32-voxel sectors */
    uint32_t brick_capacity;                  /* initial brick-pool slots; 0 = 4096; grows on demand */
    int32_t device;                           /* CUDA device ordinal */
    uint32_t flags;                           /* VRT_WORLD_* */
} vrt_world_desc;

/* Keep the world's brick table (the mask level every DDA step reads, 4 bytes per brick
 * position) persisting in L2: casts, view renders and batch launches whose batch holds
 * exactly one such world carry an L2 access-policy window over it on the caller's stream
 * (not on the legacy default stream, whose attributes cannot be set); the stream's own
 * window is restored after the launch.  Creating such a world raises this process's
 * persisting-L2 set-aside (cudaLimitPersistingL2CacheSize) to cover the table, up to the
 * device's maximum. */
#define VRT_WORLD_L2_PERSIST 1u

typedef struct vrt_world_stats {
    uint32_t sectors_x, sectors_y, sectors_z;
    uint32_t allocated_bricks;  /* FreeList::NumAllocated: live bricks */
    uint32_t brick_capacity;    /* slots in the device pool */
    uint32_t free_ranges;       /* FreeList::FreeRanges.size(): the gaps between live ranges and the tail */
    uint64_t device_bytes;      /* device memory held by the world */
    uint32_t compactions;       /* pool compactions so far: vrt_world_defrag, and edits that ran out of room */
    uint32_t reserved;
} vrt_world_stats;

/* ---- library ---- */
const char* vrt_last_error(void);
uint32_t vrt_abi_version(void);
int32_t vrt_sector_index(int32_t sx, int32_t sy, int32_t sz); /* WorldSectorIndexer::GetIndex */

/* ---- world storage (GpuVoxelStorage, GpuRenderer.cpp:17-167) ---- */
vrt_status vrt_world_create(const vrt_world_desc* desc, vrt_world** out);
vrt_status vrt_world_destroy(vrt_world* world);
vrt_status vrt_world_get_stats(const vrt_world* world, vrt_world_stats* out);

/* Sync dirty bricks into device storage, as SyncBuffers(VoxelMap&) does for each
 * DirtyLocs entry (GpuRenderer.cpp:52-166).  For sector i:
 *   alloc_mask[i]  the sector's full allocation mask (0 deletes the sector);
 *   dirty_mask[i]  bricks whose content is supplied (NULL = all of alloc_mask);
 *   bricks         popcount(alloc_mask[i] & dirty_mask[i]) x 512 bytes per sector, in
 *                  ascending bit order, sectors back to back (the cvox pack record
 *                  shape, VoxelMap.cpp:234-242).
 * Bricks that stay allocated but are not dirty keep their device content, even if
 * their slots move.  Brick occupancy masks are re-derived on the device. */
vrt_status vrt_world_sync_sectors(vrt_world* world, uint32_t n, const int32_t* sector_idx,
                                  const uint64_t* alloc_mask, const uint64_t* dirty_mask,
                                  const uint8_t* bricks, void* stream);

/* Apply sphere edits in order (VoxelMap::RegionDispatchSIMD + brick GC,
 * VoxelMap.h:222-263): bricks are allocated for fills, voxels written on the device,
 * cell masks re-derived, and bricks that became empty are freed, so the allocation
 * mask stays the set of non-empty bricks.
 * The whole edit runs on the device, allocation included (BrickSlotAllocator.cpp:5-94
 * allocates on the host): a sector that gains bricks takes a new slot range from a
 * device bump allocator, one that loses bricks shrinks in place.  The call enqueues the
 * work on `stream` after earlier work there and after the world's previous edit, and
 * returns without waiting for the device; traversals on other streams must be ordered
 * after it by the caller (edits land between frames), and vrt_world_wait waits for it
 * on the host.  The host reads the device's allocator state only when its own bound of
 * the bump pointer reaches the end of the pool; the call then compacts the pool first
 * (as vrt_world_defrag, growing it when the live bricks fill 3/4 of it) and returns
 * when that is done.  Host-side readers of the world (read_sector, save, stats) and
 * vrt_world_sync_sectors wait for earlier edits themselves. */
vrt_status vrt_world_edit(vrt_world* world, const vrt_edit* edits, uint32_t n, void* stream);

/* Wait on the host until the world's last edit has run on the device. */
vrt_status vrt_world_wait(vrt_world* world);

/* Defragment the brick pool: every live brick is packed from slot 0 in sector order
 * into a pool of `capacity` slots (0 = the current size; never fewer than the live
 * bricks), reclaiming the slots edits left behind; the reference leaves this as a TODO
 * (BrickSlotAllocator.cpp:14).  Content, masks and every traversal result are unchanged.
 * Returns when done (the pool is copied once; the old one is freed). */
vrt_status vrt_world_defrag(vrt_world* world, uint32_t capacity, void* stream);

/* Read one sector back: its allocation mask and popcount(mask) x 512 bytes. */
vrt_status vrt_world_read_sector(vrt_world* world, int32_t sector_idx, uint64_t* alloc_mask,
                                 uint8_t* bricks, size_t bricks_capacity, void* stream);

/* ---- world files (cvox v4: VoxelMap::Serialize/Deserialize, VoxelMap.cpp:205-273) ---- */
/* A sector stream in host memory (records as vrt_world_sync_sectors takes them). */
typedef struct vrt_sector_stream {
    uint32_t sectors_x, sectors_y, sectors_z;
    uint32_t n_sectors;   /* records */
    uint64_t n_bricks;    /* bricks in `bricks` */
    int32_t* sector_idx;  /* WorldSectorIndexer packing, ascending linear order */
    uint64_t* alloc_mask;
    uint8_t* bricks;      /* n_bricks x 512 */
} vrt_sector_stream;
void vrt_sector_stream_free(vrt_sector_stream* s);

/* Write / read a cvox v4 file from / into a sector stream.  Blobs are zstd frames:
 * written with stored blocks (any zstd decoder, the reference's included, reads
 * them); read natively when stored or RLE, through the system libzstd.so.1 when
 * compressed (VRT_ERR_FORMAT when that library is absent).  The palette is
 * written as default materials and ignored on reading (voxels are raw ids). */
vrt_status vrt_cvox_write(const char* path, uint32_t n, const int32_t* sector_idx, const uint64_t* alloc_mask,
                          const uint8_t* bricks);
vrt_status vrt_cvox_read(const char* path, vrt_sector_stream** out);
/* Device worlds to / from files (every allocated sector in ascending index order). */
vrt_status vrt_world_save_cvox(vrt_world* world, const char* path);
vrt_status vrt_world_load_cvox(vrt_world* world, const char* path, void* stream);

/* ---- traversal ---- */
/* Cast n explicit rays (host buffers): copies in, traverses, copies out. */
vrt_status vrt_cast(vrt_world* world, const vrt_ray* rays, uint32_t n, const vrt_cast_params* params,
                    vrt_hit* hits, void* stream);
/* Same with device pointers; asynchronous on stream. */
vrt_status vrt_cast_device(vrt_world* world, const vrt_ray* rays, uint32_t n,
                           const vrt_cast_params* params, vrt_hit* hits, void* stream);

/* Primary rays of one view, one launch (the per-view path, GpuRenderer.cpp:267-268).
 * hits: width*height records in row-major pixel order (host buffer). */
vrt_status vrt_render_view(vrt_world* world, const vrt_camera* cam, uint32_t max_iters,
                           vrt_hit* hits, void* stream);
vrt_status vrt_render_view_device(vrt_world* world, const vrt_camera* cam, uint32_t max_iters,
                                  vrt_hit* hits, void* stream);

/* Build a camera at `pos` looking at `target` (world voxel units), vertical field of
 * view in degrees, for a width x height image; computed in double on the host. */
vrt_status vrt_camera_look_at(const double pos[3], const double target[3], double vfov_deg,
                              uint32_t width, uint32_t height, vrt_camera* out);

/* ---- picking (VoxelMap::RayCast, VoxelMap.cpp:125-170) ---- */
/* The reference's scalar double-precision ray cast used for mouse picking and brush
 * placement: steps of 32/8/1 voxels from the sector map, brick presence and voxel
 * emptiness, a +1e-4 bias, no bounds test (sectors outside the world are empty). */
typedef struct vrt_pick_ray {
    double origin[3]; /* world voxel coordinates */
    double dir[3];
} vrt_pick_ray;

typedef struct vrt_pick_hit {
    double distance;  /* HitResult::Distance: biased tmin of the hit, -1 on a miss */
    int32_t voxel[3]; /* HitResult::VoxelPos */
    float normal[3];  /* HitResult::Normal: -sign(dir) on axes with tmin >= sideDist */
    float uv[2];      /* HitResult::UV */
    uint32_t iters;   /* iteration of the hit, max_iters on a miss */
    uint32_t reserved;
} vrt_pick_hit;

/* max_iters 0 = 1024 (VoxelMap.h:214).  Host buffers. */
vrt_status vrt_pick(vrt_world* world, const vrt_pick_ray* rays, uint32_t n, uint32_t max_iters, vrt_pick_hit* hits,
                    void* stream);

/* ---- views: primary rays plus secondary rays per pixel ---- */
/* A view is one RenderFrame of the reference's renderers: a primary ray per pixel
 * (VoxelRender.comp:27-30, CpuRenderer.cpp:326-333), then optionally
 *   - one shadow ray from hitPos + normal*0.01 toward sun_dir for every hit
 *     (VoxelRender.comp:51-61, origin offset as CpuRenderer.cpp:389), or
 *   - up to n_bounces diffuse bounces (CpuRenderer.cpp:342-393): origin
 *     hitPos + normal*0.01, direction normalize(normal + s), s uniform on the unit
 *     sphere by rejection from [-1,1]^3 with PCG32(initstate = pixel ^ bounce,
 *     initseq = 0x9E3779B97F4A7C15); a path ends at its first miss, or
 *   - with both VRT_VIEW_SHADOW and n_bounces > 0, the GPU renderer's whole path
 *     (VoxelRender.comp:51-86, u_MaxBounces = n_bounces): a sun ray toward sun_dir from
 *     the primary hit, then the bounces as above (bounce k from the hit of bounce k-1,
 *     not from a sun ray), the first two bounce hits each followed by a sun ray from
 *     them; a sun ray's hit or miss does not end the path.
 * Records are laid out per view as [primary w*h][shadow w*h], or
 * [primary w*h][bounce 1 w*h]...[bounce n w*h], or for the whole path
 * [primary][sun 0][bounce 1][sun 1][bounce 2][sun 2][bounce 3]...[bounce n]
 * (2 + n + min(n, 2) planes of w*h); rays never cast (shadow of a miss, bounces after
 * a miss) get a miss record with steps 0 and tag VRT_NO_RAY. */
typedef struct vrt_view {
    vrt_camera cam;
    uint32_t world;     /* index into the batch's world list */
    uint32_t max_iters; /* 0 = VRT_DEFAULT_MAX_ITERS */
    uint32_t n_bounces; /* 0..15 */
    uint32_t flags;     /* VRT_VIEW_SHADOW, VRT_VIEW_GLSL, VRT_VIEW_GLSL_ANISO */
    float sun_dir[3];
} vrt_view;

#define VRT_VIEW_SHADOW 1u
#define VRT_VIEW_GLSL 2u /* GLSL traversal mode (see VRT_CAST_GLSL); every view of a batch shares one mode */
#define VRT_VIEW_GLSL_ANISO 4u /* with VRT_VIEW_GLSL: anisotropic LODs (see VRT_CAST_GLSL_ANISO) */
#define VRT_MAX_BOUNCES 15u

/* One view with its secondary rays, one plain launch (thread per pixel, no
 * compaction).  `world` in the view is ignored.  Host / device record buffers
 * of vrt_view_records(view) entries. */
uint64_t vrt_view_records(const vrt_view* view);
vrt_status vrt_render_path(vrt_world* world, const vrt_view* view, vrt_hit* hits, void* stream);
vrt_status vrt_render_path_device(vrt_world* world, const vrt_view* view, vrt_hit* hits, void* stream);

/* ---- G-buffer of a view's primary hits (the consumer of the hits) ---- */
/* The headless G-buffer the reference's renderers write from each pixel's primary hit
 * (VoxelRender.comp:39-46,91-93, GBuffer.glsl:18-21; CpuRenderer.cpp:364-376), traced in
 * the view's traversal mode (its shadow and bounce fields are ignored):
 *   albedo_normal[p]  RGBA8: r, g, b = round-half-even(255 * c^2) of the hit material's
 *                     RGB565 color palette[material] & 0xFFFF (c = field/31, /63, /31 as
 *                     getMaterialColor computes them, each op rounded on its own), and
 *                     a = (n.x+1) | (n.y+1)<<2 | (n.z+1)<<4 with n the hit normal
 *                     (packGNormal; in the GLSL mode n may have several axes); on a miss
 *                     0x00FFFFFF (white; the shader leaves the normal unset there);
 *   depth[p]          projPos.z / projPos.w, projPos = proj * (hitPos / 16, 1) with proj
 *                     column-major 4x4 and hitPos the hit position in the ray frame (relative
 *                     to cam.world_origin), every op rounded on its own in the order
 *                     ((m[r]*x + m[4+r]*y) + m[8+r]*z) + m[12+r]; -1 on a miss.
 * palette: 256 Material words (the reference's Palette encodings); proj: 16 floats. */
vrt_status vrt_render_gbuffer(vrt_world* world, const vrt_view* view, const uint32_t* palette, const float* proj,
                              uint32_t* albedo_normal, float* depth, void* stream);
/* Device buffers, asynchronous; hits (may be NULL) also receives the primary records. */
vrt_status vrt_render_gbuffer_device(vrt_world* world, const vrt_view* view, const uint32_t* palette,
                                     const float* proj, uint32_t* albedo_normal, float* depth, vrt_hit* hits,
                                     void* stream);

/* ---- batched persistent traversal over many worlds and views ---- */
typedef struct vrt_batch_config {
    uint32_t tile_w, tile_h;   /* ray tile: 8x8, 16x4 or 32x1 (0,0 = 8x8) */
    uint32_t morton;           /* 1: Z-order inside 8x8 tiles */
    uint32_t warps_per_block;  /* 1..16 (0 = 4) */
    uint32_t blocks_per_sm;    /* 0 = as many as fit */
    uint32_t refill_threshold; /* refill idle lanes when fewer lanes are active (1..32; 0 = 28 for a
                                  launch with diffuse bounces, else 16) */
    uint32_t chunk_tiles;      /* tiles taken from the device queue per atomic (1..64; 0 = 1 for a
                                  launch with diffuse bounces, else chosen per launch: about
                                  eight fetches per warp, 1..16 tiles) */
    uint32_t inner_iters;      /* DDA iterations between refill checks (0 = 16) */
} vrt_batch_config;

typedef struct vrt_batch_stats {
    uint64_t rays_cast;   /* primary + secondary rays traversed by the last launch */
    uint64_t step_calls;  /* GetStepPos calls (vrt_batch_measure only) */
    uint64_t occ_fetches; /* calls that fetched a voxel-cell mask (vrt_batch_measure only) */
    uint64_t hits;        /* rays that hit (vrt_batch_measure only) */
} vrt_batch_stats;

typedef struct vrt_batch vrt_batch;

/* Worlds must outlive the batch; they may be re-synced between launches. */
vrt_status vrt_batch_create(vrt_world* const* worlds, uint32_t n_worlds, const vrt_view* views, uint32_t n_views,
                            const vrt_batch_config* cfg, vrt_batch** out);
vrt_status vrt_batch_destroy(vrt_batch* batch);
/* offsets[v] = first record of view v; offsets[n_views] = total records. */
vrt_status vrt_batch_output_layout(const vrt_batch* batch, uint64_t* offsets);
/* Persistent kernel over the device tile queue (queue reset included). */
vrt_status vrt_batch_launch(vrt_batch* batch, vrt_hit* hits_device, void* stream);
/* Same launch captured once into a CUDA graph and replayed. */
vrt_status vrt_batch_launch_graph(vrt_batch* batch, vrt_hit* hits_device, void* stream);
/* Baseline: one plain vrt_render_path launch per view. */
vrt_status vrt_batch_launch_per_view(vrt_batch* batch, vrt_hit* hits_device, void* stream);
/* New cameras for every view (same resolutions), copied to the device. */
vrt_status vrt_batch_update_cameras(vrt_batch* batch, const vrt_camera* cams, void* stream);
/* Host-buffer form; returns when the records are in hits_host.  The views are
 * traced in parts of about equal record count, back to back on `stream`, into a
 * batch-owned device buffer; each part's records are copied to hits_host as soon as
 * that part is done, so the host transfer overlaps the tracing of later parts
 * (pinned memory from vrt_host_alloc keeps the copies asynchronous). */
vrt_status vrt_batch_run(vrt_batch* batch, vrt_hit* hits_host, void* stream);
/* vrt_batch_run delivering 12-byte records (vrt_hit_packed, same order and count): 3/4 of
 * the bytes over the host link.  Each part's records are packed on the device once the
 * part is traced, and the packed part is copied to records_host as vrt_batch_run copies
 * the full one. */
vrt_status vrt_batch_run_packed(vrt_batch* batch, vrt_hit_packed* records_host, void* stream);
/* Counters of the last launch (synchronises the stream of that launch). */
vrt_status vrt_batch_get_stats(vrt_batch* batch, vrt_batch_stats* out);
/* One launch of the counting variant: fills step_calls/occ_fetches/hits. */
vrt_status vrt_batch_measure(vrt_batch* batch, vrt_hit* hits_device, void* stream, vrt_batch_stats* out);

/* Same traversal as vrt_batch_create + vrt_batch_launch, in one call that allocates
 * no memory: no counterpart in the reference.  For callers that cannot call
 * cudaMalloc once their frame loop runs (it may synchronise the device) or whose
 * host application owns all device memory.  The launch scratch (world table, view
 * table, tile-queue counter) lives in one fixed 152.5 KiB device array that every GPU
 * loading the library holds until the process exits, so a call takes at most 256
 * worlds and 1024 views (VRT_ERR_INVALID_ARG beyond).  The first call on a device
 * looks up that array's address and creates the event that guards the host tables;
 * make that first call before any stream capture begins.  All calls share the array: calls whose launches
 * overlap on the GPU race, so order them on one stream.  The world and view tables are staged in library-owned host tables,
 * so a call first waits on the host until the table copies of the previous call on
 * the same device have run.  The caller's current device is the same when the call
 * returns.  Records are laid out as for vrt_batch (views back to back). */
vrt_status vrt_render_views_static(vrt_world* const* worlds, uint32_t n_worlds, const vrt_view* views,
                                   uint32_t n_views, const vrt_batch_config* cfg, vrt_hit* hits_device,
                                   void* stream);

/* ---- pinned host memory (asynchronous copies for host-buffer calls) ---- */
vrt_status vrt_host_alloc(size_t bytes, void** out);
vrt_status vrt_host_free(void* ptr);

/* ---- request server: continuous batching over resident worlds ---- */
/* Render and edit requests are queued as they arrive.  A scheduler thread packs
 * the render requests at the head of the queue into one persistent launch per
 * in-flight slot (up to max_inflight launches overlap on the device, each on its
 * own stream), admitting a request only while the output records of admitted
 * requests fit the HBM budget; records are copied to the caller's host buffer
 * (pinned memory: see vrt_host_alloc).  An edit waits until the launches in flight
 * have finished and is applied before any later request starts, so every request
 * sees the world as of its place in the submission order (edits between frames,
 * as the reference applies them, Main.cpp:229-256). */
typedef struct vrt_server vrt_server;

typedef struct vrt_server_config {
    uint32_t max_inflight;          /* concurrent launches (0 = 2); launch mode only */
    uint32_t max_batch_requests;    /* requests per launch / per publish at most (0 = 256) */
    uint64_t hbm_budget_bytes;      /* output records in flight (0 = 1/4 of free HBM at creation) */
    vrt_batch_config batch;         /* persistent launch configuration */
    uint32_t flags;                 /* VRT_SERVE_RESIDENT or VRT_SERVE_LAUNCHES (0: see below) */
    uint32_t idle_us;               /* resident mode: how long an idle launch waits for work (0 = 500) */
} vrt_server_config;

/* Resident mode: one persistent launch stays on the device and takes the ray tiles of
 * requests published while it runs (through a mailbox word in mapped host memory that
 * the scheduler and the kernel update with system-scope atomics); a request is done
 * when the last of its pixels is finished (a per-view counter, then a flag in host
 * memory) and its records are copied back.  The launch ends when it has been idle for
 * idle_us, or is closed before an edit or a change of traversal mode.  Needs a device
 * with host-native atomics (GB300's coherent host link has them); VRT_ERR_INVALID_ARG
 * otherwise.
 * Launch mode (VRT_SERVE_LAUNCHES): each batch of queued requests is its own launch, up
 * to max_inflight of them overlapping on separate streams.
 * With neither flag the server runs in resident mode where the device has host-native
 * atomics and in launch mode elsewhere (vrt_server_stats.resident says which). */
#define VRT_SERVE_RESIDENT 1u
#define VRT_SERVE_LAUNCHES 2u

#define VRT_REQ_QUEUED 0u
#define VRT_REQ_RUNNING 1u
#define VRT_REQ_DONE 2u
#define VRT_REQ_FAILED 3u

typedef struct vrt_request_info {
    uint32_t state;      /* VRT_REQ_* */
    uint32_t kind;       /* 0 render, 1 edit */
    vrt_status status;   /* result of a finished request */
    uint32_t batch_size; /* requests in the launch that carried it */
    uint64_t rays;       /* records written (renders) */
    double submit_us, start_us, done_us; /* server clock, microseconds */
} vrt_request_info;

typedef struct vrt_server_stats {
    uint64_t renders_done, edits_done, rejected, launches;
    uint64_t records;
    double p50_us, p99_us, p999_us, max_us; /* render latency, submit -> records in host memory */
    double busy_seconds;                    /* wall time with at least one launch in flight */
    uint32_t resident;                      /* 1 in resident mode, 0 in launch mode */
    uint32_t reserved;
} vrt_server_stats;

vrt_status vrt_server_create(vrt_world* const* worlds, uint32_t n_worlds, const vrt_server_config* cfg,
                             vrt_server** out);
/* Waits (bounded by timeout_ms) for queued work, then stops the scheduler. */
vrt_status vrt_server_destroy(vrt_server* server, uint32_t timeout_ms);
/* hits_host: vrt_view_records(view) records, owned by the caller until the request is done. */
vrt_status vrt_server_submit_render(vrt_server* server, const vrt_view* view, vrt_hit* hits_host, uint64_t* ticket);
vrt_status vrt_server_submit_edit(vrt_server* server, uint32_t world, const vrt_edit* edits, uint32_t n,
                                  uint64_t* ticket);
/* Bounded wait for one request: VRT_ERR_QUEUE_TIMEOUT when it is not done in time. */
vrt_status vrt_server_wait(vrt_server* server, uint64_t ticket, uint32_t timeout_ms, vrt_request_info* info);
/* Bounded wait until every submitted request is done. */
vrt_status vrt_server_drain(vrt_server* server, uint32_t timeout_ms);
/* Latency percentiles over renders finished since the last reset. */
vrt_status vrt_server_get_stats(vrt_server* server, int reset, vrt_server_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* VRT_H_ */
