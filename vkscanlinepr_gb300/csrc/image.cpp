// image.cpp — writes an RGBA8 frame to an image file (host code only).
//
// The reference presents its frame through a Vulkan swapchain
// (core/scanline/scanline_rasterizer.cpp:610-695) and never writes a file.
// Headless, the frame is a host buffer; this writes it as PNG (truecolour
// with alpha, the image data in stored deflate blocks, so no compression
// library is needed), as binary PPM (RGB, alpha dropped) or as PAM (RGBA).
// Row 0 of the buffer is the first row of the file: framebuffer row y is
// scene row y, with no vertical flip.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sr.h"

namespace sr {
sr_status report_error(sr_status s, const char* msg);   // api.cu
}

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
    // CRC-32 with the reflected polynomial 0xEDB88320 (PNG specification, annex D)
    for (uint32_t n = 0; n < 256; ++n) {
        uint32_t c = n;
        for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = true;
}

uint32_t crc_update(uint32_t c, const uint8_t* p, size_t n) {
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return c;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

// One PNG chunk: length, type, data, CRC of type and data.
void chunk(std::vector<uint8_t>& out, const char type[4], const std::vector<uint8_t>& data) {
    put_be32(out, (uint32_t)data.size());
    const size_t t0 = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    const uint32_t c = crc_update(0xFFFFFFFFu, out.data() + t0, out.size() - t0) ^ 0xFFFFFFFFu;
    put_be32(out, c);
}

std::vector<uint8_t> encode_png(const uint8_t* rgba, uint32_t w, uint32_t h) {
    if (!crc_ready) crc_init();
    // filtered scanlines: filter type 0 (none), then the row
    const size_t row = (size_t)w * 4;
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * h);
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba + y * row, rgba + (y + 1) * row);
    }
    // zlib stream (RFC 1950) of stored deflate blocks (RFC 1951, BTYPE 00)
    std::vector<uint8_t> z;
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(raw.size() - pos, 65535);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + (long)pos, raw.begin() + (long)(pos + len));
        pos += len;
    } while (pos < raw.size());
    // Adler-32 of the uncompressed data
    uint32_t s1 = 1, s2 = 0;
    for (size_t i = 0; i < raw.size(); ++i) {
        s1 = (s1 + raw[i]) % 65521u;
        s2 = (s2 + s1) % 65521u;
    }
    put_be32(z, (s2 << 16) | s1);

    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.push_back(8);   // bit depth
    ihdr.push_back(6);   // colour type: truecolour with alpha
    ihdr.push_back(0);   // compression: deflate
    ihdr.push_back(0);   // filter method 0
    ihdr.push_back(0);   // no interlace
    chunk(out, "IHDR", ihdr);
    chunk(out, "IDAT", z);
    chunk(out, "IEND", {});
    return out;
}

}  // namespace

extern "C" sr_status sr_write_image(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height,
                                    int format) {
    if (!path || !rgba) return sr::report_error(SR_ERR_INVALID_ARG, "NULL argument");
    if (width == 0 || height == 0 || width > 65535 || height > 65535)
        return sr::report_error(SR_ERR_INVALID_ARG, "image size outside 1..65535");
    if (format != SR_IMAGE_PNG && format != SR_IMAGE_PPM && format != SR_IMAGE_PAM)
        return sr::report_error(SR_ERR_INVALID_ARG, "unknown image format");
    std::vector<uint8_t> bytes;
    if (format == SR_IMAGE_PNG) {
        bytes = encode_png(rgba, width, height);
    } else {
        char head[128];
        int n = format == SR_IMAGE_PPM
                    ? snprintf(head, sizeof head, "P6\n%u %u\n255\n", width, height)
                    : snprintf(head, sizeof head, "P7\nWIDTH %u\nHEIGHT %u\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n",
                               width, height);
        bytes.assign(head, head + n);
        const size_t px = (size_t)width * height;
        if (format == SR_IMAGE_PPM) {
            bytes.reserve(bytes.size() + px * 3);
            for (size_t i = 0; i < px; ++i) bytes.insert(bytes.end(), rgba + 4 * i, rgba + 4 * i + 3);
        } else {
            bytes.insert(bytes.end(), rgba, rgba + px * 4);
        }
    }
    FILE* f = fopen(path, "wb");
    if (!f) return sr::report_error(SR_ERR_INVALID_ARG, (std::string("cannot open ") + path).c_str());
    const size_t wrote = fwrite(bytes.data(), 1, bytes.size(), f);
    const int closed = fclose(f);
    if (wrote != bytes.size() || closed != 0)
        return sr::report_error(SR_ERR_INVALID_ARG, (std::string("cannot write ") + path).c_str());
    return SR_OK;
}
