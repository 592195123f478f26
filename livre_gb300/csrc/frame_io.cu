/*
 * Frame output: RGBA8 frames as PNG files, the step after the framebuffer
 * copy (livre/eq/render/shaders/fragTexCopy.glsl:11-15) where the reference
 * grabs the channel's image (livre/eq/FrameGrabber.cpp:55-111, JPEG through
 * libjpeg-turbo). PNG keeps the frame lossless and needs no codec library:
 * the zlib stream is made of stored deflate blocks (RFC 1950/1951), with the
 * CRC-32 of each chunk (ISO 3309) and the Adler-32 of the pixel data.
 * The frame's row 0 is the bottom row (GL convention); the file is written
 * top row first.
 */
#include <cstdio>
#include <cstring>
#include <vector>

#include "lv_runtime.h"

namespace
{
uint32_t crc_table_entry(uint32_t n)
{
    uint32_t c = n;
    for (int k = 0; k < 8; ++k)
        c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    return c;
}

struct Crc32
{
    uint32_t table[256];
    Crc32()
    {
        for (uint32_t n = 0; n < 256; ++n)
            table[n] = crc_table_entry(n);
    }
    uint32_t update(uint32_t crc, const uint8_t* p, size_t n) const
    {
        uint32_t c = crc ^ 0xFFFFFFFFu;
        for (size_t i = 0; i < n; ++i)
            c = table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
        return c ^ 0xFFFFFFFFu;
    }
};

void put32(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back(uint8_t(x >> 24));
    v.push_back(uint8_t(x >> 16));
    v.push_back(uint8_t(x >> 8));
    v.push_back(uint8_t(x));
}

void chunk(std::vector<uint8_t>& png, const Crc32& crc, const char type[4],
           const std::vector<uint8_t>& data)
{
    put32(png, uint32_t(data.size()));
    const size_t start = png.size();
    png.insert(png.end(), type, type + 4);
    png.insert(png.end(), data.begin(), data.end());
    put32(png, crc.update(0, png.data() + start, png.size() - start));
}
} // namespace

extern "C" lv_status lv_frame_encode_png(const uint8_t* rgba8, uint32_t width, uint32_t height,
                                         uint8_t* out, size_t capacity, size_t* size)
{
    if (!rgba8 || !size || width == 0 || height == 0 || width > (1u << 24) ||
        height > (1u << 24))
        return LV_EINVAL;
    static const Crc32 crc;
    /* filtered scanlines: filter byte 0, then the row, top row first */
    const size_t row = size_t(width) * 4;
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * height);
    for (uint32_t y = 0; y < height; ++y)
    {
        raw.push_back(0);
        const uint8_t* src = rgba8 + size_t(height - 1 - y) * row;
        raw.insert(raw.end(), src, src + row);
    }
    /* zlib: header (deflate, 32 KiB window, no dictionary), stored blocks,
     * Adler-32 */
    std::vector<uint8_t> z;
    z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do
    {
        const size_t n = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(uint8_t(n));
        z.push_back(uint8_t(n >> 8));
        z.push_back(uint8_t(~n));
        z.push_back(uint8_t(~n >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < raw.size(); ++i)
    {
        a = (a + raw[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(z, (b << 16) | a);

    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put32(ihdr, width);
    put32(ihdr, height);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0}); /* 8-bit RGBA, deflate, no interlace */
    chunk(png, crc, "IHDR", ihdr);
    chunk(png, crc, "IDAT", z);
    chunk(png, crc, "IEND", {});
    *size = png.size();
    if (!out)
        return LV_OK; /* size query */
    if (capacity < png.size())
        return LV_ENOMEM;
    std::memcpy(out, png.data(), png.size());
    return LV_OK;
}

extern "C" lv_status lv_frame_write_png(lv_ctx* ctx, const float* d_rgba, uint32_t width,
                                        uint32_t height, const char* path)
{
    if (!ctx || !d_rgba || !path || width == 0 || height == 0)
        return lv::fail(ctx, LV_EINVAL, "invalid frame");
    const size_t n = size_t(width) * height;
    lv::DeviceBuffer d8;
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    /* the frame may still be rendering on any stream (lv_render returns with
     * its ray cast queued; batches render on their own streams) */
    LV_CUDA(ctx, cudaDeviceSynchronize());
    LV_CUDA(ctx, d8.reserve(n * 4));
    lv_status st = lv_frame_to_rgba8(ctx, d_rgba, width, height, d8.as<uint8_t>(), nullptr);
    if (st != LV_OK)
        return st;
    std::vector<uint8_t> host(n * 4);
    LV_CUDA(ctx, cudaMemcpy(host.data(), d8.ptr, n * 4, cudaMemcpyDeviceToHost));
    size_t bytes = 0;
    lv_frame_encode_png(host.data(), width, height, nullptr, 0, &bytes);
    std::vector<uint8_t> png(bytes);
    st = lv_frame_encode_png(host.data(), width, height, png.data(), png.size(), &bytes);
    if (st != LV_OK)
        return lv::fail(ctx, st, "PNG encoding");
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return lv::fail(ctx, LV_EINVAL, std::string("cannot open ") + path);
    const size_t w = std::fwrite(png.data(), 1, png.size(), f);
    const int closed = std::fclose(f);
    if (w != png.size() || closed != 0)
        return lv::fail(ctx, LV_EDEVICE, std::string("short write to ") + path);
    return LV_OK;
}
