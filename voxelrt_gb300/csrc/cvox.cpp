// cvox.cpp - the reference's world file format, version 4 (VoxelMap::Serialize /
// Deserialize, src/VoxelRT/VoxelMap.cpp:205-273, framing of BinaryIO.cpp:8-64):
//
//   u64  magic "cvox" 04 00 00 00
//   u32  number of sectors
//   blob palette (256 x 16-byte Material)
//   then, until every sector is read: u32 raw pack size, blob pack
//   pack = records of { u32 WorldSectorIndexer index, u64 allocation mask,
//                       popcount(mask) x 512-byte bricks in bit order }, <= 16 MiB each
//   blob = u32 byte count + one zstd frame
//
// Frames are written with raw (stored) blocks, which every zstd decoder reads, so
// the reference loads these files.  On reading, raw and RLE blocks are decoded
// here; frames with compressed blocks (what the reference writes) are handed to
// the system's libzstd.so.1 when it can be loaded, and refused otherwise.

#include <dlfcn.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vrt_synth.h"
#include "vrt_internal.h"

namespace vrt {
void set_error(const std::string& msg);
}

namespace {

constexpr uint64_t kMagic = 0x00000004786f7663ull;  // "cvox" 04 00 00 00
constexpr uint32_t kMaxPack = 16u * 1024 * 1024;
constexpr uint32_t kZstdMagic = 0xFD2FB528u;
constexpr uint32_t kMaxBlock = 128 * 1024;

vrt_status fail(vrt_status st, const std::string& msg) {
    vrt::set_error(msg);
    return st;
}

void put32(std::vector<uint8_t>& b, uint32_t v) {
    for (int i = 0; i < 4; i++) b.push_back((uint8_t)(v >> (8 * i)));
}
void put64(std::vector<uint8_t>& b, uint64_t v) {
    for (int i = 0; i < 8; i++) b.push_back((uint8_t)(v >> (8 * i)));
}
uint32_t get32(const uint8_t* p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }
uint64_t get64(const uint8_t* p) { return (uint64_t)get32(p) | (uint64_t)get32(p + 4) << 32; }

// One zstd frame (RFC 8878) of raw blocks: single segment, 8-byte content size.
void zstd_raw_frame(std::vector<uint8_t>& out, const uint8_t* src, size_t n) {
    put32(out, kZstdMagic);
    out.push_back(0xE0);  // FCS field 8 bytes, single segment, no checksum, no dictionary
    put64(out, n);
    size_t off = 0;
    do {
        const size_t len = n - off < kMaxBlock ? n - off : kMaxBlock;
        const uint32_t last = off + len == n ? 1u : 0u;
        const uint32_t hdr = last | 0u << 1 | (uint32_t)len << 3;  // block type 0 = raw
        out.push_back((uint8_t)hdr);
        out.push_back((uint8_t)(hdr >> 8));
        out.push_back((uint8_t)(hdr >> 16));
        out.insert(out.end(), src + off, src + off + len);
        off += len;
    } while (off < n);
}

void write_blob(std::vector<uint8_t>& file, const uint8_t* src, size_t n) {
    std::vector<uint8_t> frame;
    zstd_raw_frame(frame, src, n);
    put32(file, (uint32_t)frame.size());
    file.insert(file.end(), frame.begin(), frame.end());
}

using zstd_decompress_fn = size_t (*)(void*, size_t, const void*, size_t);
using zstd_is_error_fn = unsigned (*)(size_t);

struct LibZstd {
    zstd_decompress_fn decompress = nullptr;
    zstd_is_error_fn is_error = nullptr;
    LibZstd() {
        void* h = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) return;
        decompress = (zstd_decompress_fn)dlsym(h, "ZSTD_decompress");
        is_error = (zstd_is_error_fn)dlsym(h, "ZSTD_isError");
        if (!decompress || !is_error) decompress = nullptr;
    }
};

const LibZstd& libzstd() {
    static LibZstd z;
    return z;
}

// Decode the zstd frames of one blob into exactly `want` bytes.
vrt_status read_frames(const uint8_t* p, size_t n, uint8_t* dst, size_t want) {
    size_t got = 0, off = 0;
    const uint8_t* const blob = p;
    bool compressed = false;
    while (off < n) {
        if (n - off < 5 || get32(p + off) != kZstdMagic) return fail(VRT_ERR_FORMAT, "cvox: bad zstd frame");
        const uint8_t fhd = p[off + 4];
        size_t q = off + 5;
        const uint32_t fcs_flag = fhd >> 6, single = (fhd >> 5) & 1, checksum = (fhd >> 2) & 1, did = fhd & 3;
        if (!single) q += 1;  // window descriptor
        const size_t did_len = did == 0 ? 0 : (did == 1 ? 1 : (did == 2 ? 2 : 4));
        if (q + did_len > n) return fail(VRT_ERR_FORMAT, "cvox: truncated zstd frame header");
        uint32_t dict = 0;
        for (size_t k = 0; k < did_len; k++) dict |= (uint32_t)p[q + k] << (8 * k);
        if (dict) return fail(VRT_ERR_FORMAT, "cvox: zstd frame needs a dictionary");
        q += did_len;
        const size_t fcs_bytes = fcs_flag == 0 ? (single ? 1 : 0) : (fcs_flag == 1 ? 2 : (fcs_flag == 2 ? 4 : 8));
        q += fcs_bytes;
        if (q > n) return fail(VRT_ERR_FORMAT, "cvox: truncated zstd frame header");
        for (;;) {
            if (q + 3 > n) return fail(VRT_ERR_FORMAT, "cvox: truncated zstd block");
            const uint32_t hdr = (uint32_t)p[q] | (uint32_t)p[q + 1] << 8 | (uint32_t)p[q + 2] << 16;
            q += 3;
            const uint32_t last = hdr & 1, type = (hdr >> 1) & 3, size = hdr >> 3;
            if (type == 0) {
                if (q + size > n || got + size > want) return fail(VRT_ERR_FORMAT, "cvox: raw block overruns");
                std::memcpy(dst + got, p + q, size);
                got += size;
                q += size;
            } else if (type == 1) {
                if (q + 1 > n || got + size > want) return fail(VRT_ERR_FORMAT, "cvox: RLE block overruns");
                std::memset(dst + got, p[q], size);
                got += size;
                q += 1;
            } else if (type == 2) {
                compressed = true;
                break;
            } else {
                return fail(VRT_ERR_FORMAT, "cvox: reserved zstd block type");
            }
            if (last) break;
        }
        if (compressed) break;
        if (checksum) q += 4;
        off = q;
    }
    if (compressed) {
        const LibZstd& z = libzstd();
        if (!z.decompress)
            return fail(VRT_ERR_FORMAT, "cvox: compressed zstd blocks need libzstd.so.1, which is not available");
        const size_t r = z.decompress(dst, want, blob, n);
        if (z.is_error(r) || r != want) return fail(VRT_ERR_FORMAT, "cvox: zstd decompression failed");
        return VRT_OK;
    }
    if (got != want) return fail(VRT_ERR_FORMAT, "cvox: blob shorter than expected");
    return VRT_OK;
}

struct Reader {
    const std::vector<uint8_t>& f;
    size_t off = 0;
    bool take(size_t n) {
        if (off + n > f.size()) return false;
        off += n;
        return true;
    }
};

}  // namespace

extern "C" {

vrt_status vrt_cvox_write(const char* path, uint32_t n, const int32_t* sector_idx, const uint64_t* alloc_mask,
                          const uint8_t* bricks) {
    if (!path || (n && (!sector_idx || !alloc_mask))) return fail(VRT_ERR_INVALID_ARG, "null argument");
    std::vector<uint8_t> file;
    put64(file, kMagic);
    put32(file, n);
    // palette of default materials: Color 0,0,0, MetalFuzziness 255, Emission 0 (VoxelMap.h:22-26)
    std::vector<uint8_t> palette(256 * 16, 0);
    for (int i = 0; i < 256; i++) palette[i * 16 + 3] = 255;
    write_blob(file, palette.data(), palette.size());
    std::vector<uint8_t> pack;
    const uint8_t* src = bricks;
    auto flush = [&](bool final) {
        if (pack.size() >= kMaxPack || final) {
            put32(file, (uint32_t)pack.size());
            write_blob(file, pack.data(), pack.size());
            pack.clear();
        }
    };
    for (uint32_t i = 0; i < n; i++) {
        const size_t nb = (size_t)__builtin_popcountll(alloc_mask[i]);
        if (nb && !src) return fail(VRT_ERR_INVALID_ARG, "null brick data");
        put32(pack, (uint32_t)sector_idx[i]);
        put64(pack, alloc_mask[i]);
        if (nb) pack.insert(pack.end(), src, src + nb * 512);
        if (src) src += nb * 512;
        flush(false);
    }
    flush(true);
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(VRT_ERR_IO, std::string("cvox: cannot open ") + path);
    const size_t w = std::fwrite(file.data(), 1, file.size(), fp);
    const int c = std::fclose(fp);
    if (w != file.size() || c != 0) return fail(VRT_ERR_IO, "cvox: write failed");
    return VRT_OK;
}

vrt_status vrt_cvox_read(const char* path, vrt_sector_stream** out) {
    if (!path || !out) return fail(VRT_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(VRT_ERR_IO, std::string("cvox: cannot open ") + path);
    std::vector<uint8_t> f;
    uint8_t buf[1 << 16];
    size_t r;
    while ((r = std::fread(buf, 1, sizeof(buf), fp)) > 0) f.insert(f.end(), buf, buf + r);
    std::fclose(fp);
    Reader rd{f};
    if (!rd.take(12) || get64(f.data()) != kMagic) return fail(VRT_ERR_FORMAT, "cvox: not a version-4 cvox file");
    const uint32_t n = get32(f.data() + 8);
    // palette blob (discarded: the library stores raw voxel ids)
    if (!rd.take(4)) return fail(VRT_ERR_FORMAT, "cvox: truncated palette");
    const uint32_t pal_len = get32(f.data() + rd.off - 4);
    std::vector<uint8_t> palette(256 * 16);
    if (!rd.take(pal_len)) return fail(VRT_ERR_FORMAT, "cvox: truncated palette");
    vrt_status st = read_frames(f.data() + rd.off - pal_len, pal_len, palette.data(), palette.size());
    if (st != VRT_OK) return st;
    std::vector<int32_t> idx;
    std::vector<uint64_t> masks;
    std::vector<uint8_t> bricks, pack;
    size_t pp = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (pp == pack.size()) {
            if (!rd.take(8)) return fail(VRT_ERR_FORMAT, "cvox: truncated pack header");
            const uint32_t raw = get32(f.data() + rd.off - 8), len = get32(f.data() + rd.off - 4);
            if (raw > 64u * 1024 * 1024 || !rd.take(len)) return fail(VRT_ERR_FORMAT, "cvox: bad pack");
            pack.assign(raw, 0);
            if ((st = read_frames(f.data() + rd.off - len, len, pack.data(), raw)) != VRT_OK) return st;
            pp = 0;
        }
        if (pp + 12 > pack.size()) return fail(VRT_ERR_FORMAT, "cvox: truncated sector record");
        const uint32_t key = get32(pack.data() + pp);
        const uint64_t mask = get64(pack.data() + pp + 4);
        pp += 12;
        const size_t nb = (size_t)__builtin_popcountll(mask);
        if (pp + nb * 512 > pack.size()) return fail(VRT_ERR_FORMAT, "cvox: truncated bricks");
        idx.push_back((int32_t)key);
        masks.push_back(mask);
        bricks.insert(bricks.end(), pack.begin() + (long)pp, pack.begin() + (long)(pp + nb * 512));
        pp += nb * 512;
    }
    auto* s = (vrt_sector_stream*)std::calloc(1, sizeof(vrt_sector_stream));
    if (!s) return fail(VRT_ERR_OUT_OF_MEMORY, "out of host memory");
    s->n_sectors = n;
    s->n_bricks = bricks.size() / 512;
    s->sector_idx = (int32_t*)std::malloc(sizeof(int32_t) * (n ? n : 1));
    s->alloc_mask = (uint64_t*)std::malloc(sizeof(uint64_t) * (n ? n : 1));
    s->bricks = (uint8_t*)std::malloc(bricks.size() ? bricks.size() : 1);
    if (!s->sector_idx || !s->alloc_mask || !s->bricks) {
        vrt_sector_stream_free(s);
        return fail(VRT_ERR_OUT_OF_MEMORY, "out of host memory");
    }
    if (n) {
        std::memcpy(s->sector_idx, idx.data(), sizeof(int32_t) * n);
        std::memcpy(s->alloc_mask, masks.data(), sizeof(uint64_t) * n);
    }
    if (!bricks.empty()) std::memcpy(s->bricks, bricks.data(), bricks.size());
    // extent: the smallest sector box from 0 holding every record with non-negative coordinates
    for (uint32_t i = 0; i < n; i++) {
        int32_t x, y, z;
        vrt::sector_index_unpack(idx[i], x, y, z);
        if (x >= 0 && (uint32_t)x + 1 > s->sectors_x) s->sectors_x = (uint32_t)x + 1;
        if (y >= 0 && (uint32_t)y + 1 > s->sectors_y) s->sectors_y = (uint32_t)y + 1;
        if (z >= 0 && (uint32_t)z + 1 > s->sectors_z) s->sectors_z = (uint32_t)z + 1;
    }
    *out = s;
    return VRT_OK;
}

}  // extern "C"
