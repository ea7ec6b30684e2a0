// icbc_containers.cu -- DDS / KTX files of BC1 blocks and the golden-file
// compare of icbc's test driver (icbc_test.cpp:155-279).  Host code; blocks
// may live in device memory, in which case they are copied out first.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/icbc_gpu.h"

namespace {

constexpr uint32_t fourcc(const char s[4]) {
    return (uint32_t)(uint8_t)s[0] | ((uint32_t)(uint8_t)s[1] << 8) | ((uint32_t)(uint8_t)s[2] << 16) |
           ((uint32_t)(uint8_t)s[3] << 24);
}

size_t block_bytes(int32_t w, int32_t h) { return 8 * (size_t)((w + 3) / 4) * (size_t)((h + 3) / 4); }

// Host view of `blocks`: the pointer itself, or a copy of device memory.
int host_blocks(const void *blocks, size_t bytes, std::vector<uint8_t> &copy, const uint8_t **out) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, blocks) == cudaSuccess && a.type == cudaMemoryTypeDevice) {
        copy.resize(bytes);
        if (cudaMemcpy(copy.data(), blocks, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return ICBC_GPU_ERR_CUDA;
        *out = copy.data();
    } else {
        cudaGetLastError();  // a host pointer unknown to CUDA is not an error here
        *out = static_cast<const uint8_t *>(blocks);
    }
    return ICBC_GPU_OK;
}

void put32(std::vector<uint8_t> &v, uint32_t x) {
    for (int i = 0; i < 4; i++) v.push_back((uint8_t)(x >> (8 * i)));
}

// The 128-byte DDS preamble: "DDS " and the 124-byte header (caps, pixel
// format, width, height, linear size of the top level) with a DXT1 FourCC
// pixel format; with more than one level also the mip count and the
// complex / mipmap caps.
std::vector<uint8_t> dds_header(int32_t w, int32_t h, int32_t levels = 1) {
    const uint32_t caps = 0x1, pixelformat = 0x1000, width = 0x4, height = 0x2, linearsize = 0x80000;
    const uint32_t mipcount = levels > 1 ? 0x20000 : 0;
    std::vector<uint8_t> v;
    put32(v, fourcc("DDS "));
    put32(v, 124);
    put32(v, caps | pixelformat | width | height | linearsize | mipcount);
    put32(v, (uint32_t)h);
    put32(v, (uint32_t)w);
    put32(v, (uint32_t)block_bytes(w, h));
    put32(v, 0);  // depth
    put32(v, (uint32_t)levels);  // mip levels
    for (int i = 0; i < 11; i++) put32(v, 0);
    put32(v, 32);     // pixel format size
    put32(v, 0x4);    // DDPF_FOURCC
    put32(v, fourcc("DXT1"));
    for (int i = 0; i < 5; i++) put32(v, 0);  // bit count, masks
    put32(v, 0x1000 | (levels > 1 ? 0x400008u : 0u));  // DDSCAPS_TEXTURE (| MIPMAP | COMPLEX)
    for (int i = 0; i < 3; i++) put32(v, 0);
    put32(v, 0);
    return v;
}

int write_file(const char *path, const std::vector<uint8_t> &head, const uint8_t *data, size_t bytes) {
    FILE *f = std::fopen(path, "wb");
    if (!f) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    const bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size() &&
                    std::fwrite(data, 1, bytes, f) == bytes;
    return (std::fclose(f) == 0 && ok) ? ICBC_GPU_OK : ICBC_GPU_ERR_INVALID_ARGUMENT;
}

}  // namespace

extern "C" {

int icbc_gpu_write_dds(const char *path, int32_t width, int32_t height, const void *blocks) {
    if (!path || !blocks || width < 1 || height < 1) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    const size_t bytes = block_bytes(width, height);
    std::vector<uint8_t> copy;
    const uint8_t *data = nullptr;
    const int st = host_blocks(blocks, bytes, copy, &data);
    if (st) return st;
    return write_file(path, dds_header(width, height), data, bytes);
}

int icbc_gpu_write_dds_mips(const char *path, int32_t width, int32_t height, int32_t levels, const void *blocks) {
    if (!path || !blocks || width < 1 || height < 1 || levels < 1 || levels > icbc_gpu_mip_levels(width, height))
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    size_t bytes = 0;
    for (int32_t k = 0, w = width, h = height; k < levels; k++, w = w > 1 ? w >> 1 : 1, h = h > 1 ? h >> 1 : 1)
        bytes += block_bytes(w, h);
    std::vector<uint8_t> copy;
    const uint8_t *data = nullptr;
    const int st = host_blocks(blocks, bytes, copy, &data);
    if (st) return st;
    return write_file(path, dds_header(width, height, levels), data, bytes);
}

int icbc_gpu_write_ktx(const char *path, int32_t width, int32_t height, const void *blocks) {
    if (!path || !blocks || width < 1 || height < 1) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    const size_t bytes = block_bytes(width, height);
    std::vector<uint8_t> copy;
    const uint8_t *data = nullptr;
    const int st = host_blocks(blocks, bytes, copy, &data);
    if (st) return st;
    static const uint8_t ident[12] = {0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<uint8_t> head(ident, ident + 12);
    put32(head, 0x04030201);  // endianness
    put32(head, 0);           // glType (compressed)
    put32(head, 1);           // glTypeSize
    put32(head, 0);           // glFormat (compressed)
    put32(head, 0x83F0);      // GL_COMPRESSED_RGB_S3TC_DXT1_EXT
    put32(head, 0x1908);      // GL_RGBA base internal format, as the reference writes it
    put32(head, (uint32_t)width);
    put32(head, (uint32_t)height);
    put32(head, 0);  // depth
    put32(head, 0);  // array elements
    put32(head, 1);  // faces
    put32(head, 1);  // mip levels
    put32(head, 0);  // key/value bytes
    put32(head, (uint32_t)bytes);  // imageSize of level 0
    return write_file(path, head, data, bytes);
}

int icbc_gpu_compare_dds(const char *path, int32_t width, int32_t height, const void *blocks) {
    if (!path || !blocks || width < 1 || height < 1) return -ICBC_GPU_ERR_INVALID_ARGUMENT;
    const size_t bytes = block_bytes(width, height);
    std::vector<uint8_t> copy;
    const uint8_t *data = nullptr;
    const int st = host_blocks(blocks, bytes, copy, &data);
    if (st) return -st;
    FILE *f = std::fopen(path, "rb");
    if (!f) return -ICBC_GPU_ERR_NOT_FOUND;
    std::vector<uint8_t> file(bytes);
    const bool ok = std::fseek(f, 128, SEEK_SET) == 0 && std::fread(file.data(), 1, bytes, f) == bytes;
    std::fclose(f);
    if (!ok) return -ICBC_GPU_ERR_NOT_FOUND;
    return std::memcmp(file.data(), data, bytes) == 0 ? 1 : 0;
}

}  // extern "C"
