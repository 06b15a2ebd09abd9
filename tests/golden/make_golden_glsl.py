"""Records tests/golden/refglsl.npz: the reference's own traversal shaders
(VoxelTraversal.glsl rayCast and rayCastCoarse, with and without anisotropic LODs),
compiled as C++ by oracle/glsl_pin/build_glsl.py, on seeded worlds and rays.  The pin
of the GLSL traversal mode: the shader cannot run here (no graphics stack), but its
source compiles on the host against a GLSL-subset header.

The shaders' buffers are filled as GpuVoxelStorage::SyncBuffers and
UpdateOccupancy.comp fill them (GpuRenderer.cpp:45-167):
  * BaseSlots[sector] = the sector's first slot (0-based), BrickMasks = its 64-bit
    allocation mask, sector index x + z*XZ + y*XZ*XZ;
  * SectorMasks[group] bit (x&3) + (z&3)*4 + (y&3)*16 per non-empty sector, group
    index gx + gz*XZ/4 + gy*(XZ/4)^2;
  * BrickData: 512 voxel ids per slot, voxel x + z*8 + y*64;
  * occupancy: 8 cell masks per slot, cell cx + cz*2 + cy*4, bit vx + vz*4 + vy*16;
  * RayCellInteractionMaskLUT from the oracle's restatement of
    GenerateRayCellInteractionMaskLUT (GpuRenderer.cpp:193-210), which
    tests/test_oracle_cpu.py checks against the forward box for all 512 entries;
  * Palette[i] encodes id i, so a hit's material is the voxel id.

Usage: python tests/golden/make_golden_glsl.py <reference checkout> (or $VRT_REFERENCE_DIR)
"""
import ctypes as C
import subprocess
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

SXZ, SY = 8, 4  # sectors the shader build is sized for: 256 x 128 x 256 voxels
MODES = ((False, False), (True, False), (False, True), (True, True))  # (coarse, aniso)
SUN = (np.array([0.3, 0.8, 0.5]) / np.linalg.norm([0.3, 0.8, 0.5])).astype(np.float32)


def glsl_world(kind: str, seed: int) -> np.ndarray:
    """(Y, Z, X) voxel ids of a 256 x 128 x 256 world."""
    rng = np.random.default_rng(seed)
    vol = np.zeros((SY * 32, SXZ * 32, SXZ * 32), np.uint8)
    if kind == "blobs":  # solid boxes far apart: empty sectors and groups between them
        for _ in range(40):
            y, z, x = rng.integers(0, vol.shape)
            vol[max(0, y - 6):y + 6, max(0, z - 6):z + 6, max(0, x - 6):x + 6] = rng.integers(1, 256)
    else:  # a terrain slab with caves and scattered voxels
        zz, xx = np.meshgrid(np.arange(vol.shape[1]), np.arange(vol.shape[2]), indexing="ij")
        h = 40 + 18 * np.sin(xx / 23.0 + seed) * np.cos(zz / 31.0) + 6 * np.sin((xx + zz) / 7.0)
        yy = np.arange(vol.shape[0])[:, None, None]
        vol[:] = np.where(yy < h[None], 1 + yy // 16, 0).astype(np.uint8)  # material by height band
        cave = rng.random(vol.shape) < 0.004
        vol[cave] = 0
        vol[rng.random(vol.shape) < 0.002] = rng.integers(1, 256)
        vol[:, 96:160, 96:160] = 0  # whole sectors carved empty
    return vol


def buffers(data):
    import oracle.oracle as ora
    base = np.zeros(SXZ * SXZ * SY, np.uint32)
    masks = np.zeros(SXZ * SXZ * SY, np.uint64)
    groups = np.zeros((SXZ // 4) * (SXZ // 4) * (SY // 4), np.uint64)
    slot = 0
    for idx, m in zip(data.sector_idx.tolist(), data.alloc_mask.tolist()):
        x, z, y = idx & 4095, (idx >> 12) & 4095, (idx >> 24) & 255
        s = x + z * SXZ + y * SXZ * SXZ
        base[s], masks[s] = slot, m
        slot += bin(m).count("1")
        if m:
            g = (x >> 2) + (z >> 2) * (SXZ // 4) + (y >> 2) * (SXZ // 4) ** 2
            groups[g] |= np.uint64(1) << np.uint64((x & 3) + (z & 3) * 4 + (y & 3) * 16)
    nb = data.n_bricks
    solid = data.bricks.reshape(nb, 8, 8, 8) != 0  # (n, y, z, x)
    cv = solid.reshape(nb, 2, 4, 2, 4, 2, 4).transpose(0, 1, 3, 5, 2, 4, 6)  # (n, cy, cz, cx, vy, vz, vx)
    bits = np.uint64(1) << np.arange(64, dtype=np.uint64)
    occ = (cv.reshape(nb, 8, 64).astype(np.uint64) * bits).sum(axis=2, dtype=np.uint64)
    return base, masks, groups, np.ascontiguousarray(data.bricks), occ, ora.ray_cell_lut()


def ray_sets(rng):
    """Camera-frame sets (fractional origin, integer world origin) and one world-frame set."""
    size = np.array([SXZ * 32, SY * 32, SXZ * 32], np.float64)
    sets = []
    for _ in range(2):
        eye = rng.uniform(size * 0.1, size * 0.9)
        d = rng.normal(size=(1500, 3)).astype(np.float32)
        d[rng.random(d.shape) < 0.02] = 0.0
        wo = np.floor(eye).astype(np.int32)
        sets.append((np.tile((eye - np.floor(eye)).astype(np.float32), (len(d), 1)), d, wo))
    o = rng.uniform(-0.2 * size, 1.2 * size, (1500, 3)).astype(np.float32)
    d = rng.normal(size=(1500, 3)).astype(np.float32)
    sets.append((o, d, np.zeros(3, np.int32)))
    return sets


def main(ref: str) -> None:
    subprocess.run([sys.executable, str(ROOT / "oracle" / "glsl_pin" / "build_glsl.py"), ref, str(SXZ), str(SY)],
                   check=True)
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / f"libglsl_ref_{SXZ}x{SY}.so"))
    from tests.helpers import dense_to_stream
    out = {"worlds": np.array(["blobs:11", "terrain:12"]), "sxz_sy": np.array([SXZ, SY], np.int32)}
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    for wi, spec in enumerate(out["worlds"]):
        kind, seed = str(spec).split(":")
        data = dense_to_stream(glsl_world(kind, int(seed)))
        base, masks, groups, bricks, occ, lut = buffers(data)
        lib.glsl_ref_load(p(base), p(masks), p(groups), p(bricks), C.c_uint64(data.n_bricks), p(occ), p(lut))
        for si, (org, d, wo) in enumerate(ray_sets(np.random.default_rng(100 + wi))):
            key = f"{wi}/{si}"
            out[f"{key}/origin"], out[f"{key}/dir"], out[f"{key}/wo"] = org, d, wo
            rays = np.ascontiguousarray(np.concatenate([org, d], axis=1), np.float32)
            n = len(rays)
            for coarse, aniso in MODES:
                hit = np.zeros(n, np.uint8)
                dist = np.zeros(n, np.float32)
                pos = np.zeros((n, 3), np.float32)
                nrm = np.zeros((n, 3), np.float32)
                iters = np.zeros(n, np.uint32)
                mat = np.zeros(n, np.uint32)
                lib.glsl_ref_cast(p(rays), C.c_uint32(n), p(wo), int(coarse), int(aniso), p(hit), p(dist), p(pos),
                                  p(nrm), p(iters), p(mat))
                m = f"{key}/{int(coarse)}{int(aniso)}"
                out[f"{m}/hit"], out[f"{m}/dist"], out[f"{m}/iters"] = hit, dist, iters
                out[f"{m}/mat"] = mat.astype(np.uint8)
                out[f"{m}/pos"] = pos
                out[f"{m}/normal"] = np.sign(nrm).astype(np.int8)
        # a view with shadow rays: the oracle's camera rays (the library's camera model), a
        # primary rayCast each and the renderer's shadow ray where it hits
        import voxelrt_gb300 as v
        from oracle.oracle import camera_rays
        rng = np.random.default_rng(200 + wi)
        size = np.array([SXZ * 32, SY * 32, SXZ * 32], np.float64)
        cam = v.look_at(rng.uniform(size * 0.2, size * 0.8), rng.uniform(size * 0.2, size * 0.8), 70.0, 64, 48)
        out[f"{wi}/cam"] = np.frombuffer(bytes(cam), np.uint8)
        cr = camera_rays(cam)
        rays = np.ascontiguousarray(np.concatenate([cr["origin"], cr["dir"]], axis=1), np.float32)
        wo = np.array(cam.world_origin[:], np.int32)
        n = len(rays)
        for aniso in (False, True):
            a = {k: np.zeros(n, t) for k, t in (("hit", np.uint8), ("dist", np.float32), ("iters", np.uint32),
                                                 ("mat", np.uint32), ("s_hit", np.uint8), ("s_dist", np.float32),
                                                 ("s_iters", np.uint32), ("s_mat", np.uint32))}
            pos, nrm = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
            lib.glsl_ref_shadow(p(rays), C.c_uint32(n), p(wo), p(SUN), int(aniso), p(a["hit"]), p(a["dist"]), p(pos),
                                p(nrm), p(a["iters"]), p(a["mat"]), p(a["s_hit"]), p(a["s_dist"]), p(a["s_iters"]),
                                p(a["s_mat"]))
            m = f"{wi}/view/{int(aniso)}"
            for k, arr in a.items():
                out[f"{m}/{k}"] = arr.astype(np.uint8) if k in ("mat", "s_mat") else arr
            out[f"{m}/pos"], out[f"{m}/normal"] = pos, np.sign(nrm).astype(np.int8)
    out["sun"] = SUN
    np.savez_compressed(ROOT / "tests" / "golden" / "refglsl.npz", **out)
    print("wrote tests/golden/refglsl.npz")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VRT_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: give the reference checkout as the argument or in $VRT_REFERENCE_DIR")
    main(ref)
