/*
 * vrt_synth.h - seeded synthetic worlds and ray sets (libvrt_synth.so, a host-only
 * library: it needs no GPU and links no CUDA; it also exports vrt_camera_look_at and
 * vrt_sector_stream_free of vrt.h, so that test and benchmark inputs can be built
 * without loading libvrt.so).
 *
 * The reference builds worlds with FastNoise2 terrain (src/VoxelRT/TerrainGenerator.cpp:5-34)
 * or by voxelizing meshes; neither is reproducible here, so benchmark and test
 * worlds come from these deterministic generators.  Noise is 2D/3D Perlin gradient
 * noise over a PCG lattice hash, evaluated in double with every op rounded on its
 * own, so x86 and arm64 hosts build identical worlds.  Output is a sector stream
 * in the record shape vrt_world_sync_sectors takes (the cvox pack shape,
 * VoxelMap.cpp:234-242), holding only non-empty bricks, as the terrain generator
 * keeps (TerrainGenerator.cpp:139-145).
 */
#ifndef VRT_SYNTH_H_
#define VRT_SYNTH_H_

#include "vrt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Heightfield terrain, optionally minus caves:
 *   solid(x,y,z) = y < base + amplitude * fbm2(x/scale, z/scale)   (octaves, lacunarity 2, gain 0.5)
 *                  and not (caves && fbm3(x/cave_scale, y/cave_scale, z/cave_scale) > cave_threshold)
 *   material     = 1 + min(3, y/32) */
typedef struct vrt_synth_terrain {
    uint32_t size[3];      /* voxels, multiples of 32 */
    double base, amplitude, scale;
    uint32_t octaves;
    uint64_t seed;
    uint32_t cave_octaves; /* 0 = no caves */
    double cave_scale, cave_threshold;
    uint64_t cave_seed;
} vrt_synth_terrain;

/* Message of the last failed call of this library on the calling thread. */
const char* vrt_synth_last_error(void);

/* threads = 0 uses every hardware thread. The stream is freed with vrt_sector_stream_free. */
vrt_status vrt_synth_terrain_world(const vrt_synth_terrain* desc, int threads, vrt_sector_stream** out);

/* Height of the terrain surface at column (x, z): base + amplitude * fbm2. */
double vrt_synth_terrain_height(const vrt_synth_terrain* desc, double x, double z);

/* A cubic world of edge `edge` voxels (multiple of 32) mixing, by seeded draws:
 * terrain (base 0.375*edge, amplitude 0.1875*edge, scale 128, 4 octaves), solid
 * spheres of radius 2..40 filling 0..20% of the volume, and uniform random voxels
 * at density 1..30%.  Spheres win over terrain, terrain over random voxels. */
vrt_status vrt_synth_mix_world(uint32_t edge, uint64_t seed, int threads, vrt_sector_stream** out);

/* n rays with origins uniform in [0,size) (world frame, world origin 0) and
 * directions uniform on the unit sphere (rejection from the cube, IEEE ops only),
 * ray i drawn from PCG32(initstate = i, initseq = seed); tag = i. */
vrt_status vrt_synth_random_rays(const uint32_t size[3], uint64_t seed, uint64_t first, uint64_t n, int threads,
                                 vrt_ray* out);

#ifdef __cplusplus
}
#endif
#endif
