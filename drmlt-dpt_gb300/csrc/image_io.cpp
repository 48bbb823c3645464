// Host-side image output: OpenEXR writer (scanline, half-float RGB, no
// compression), replacing WriteImage (src/image.cpp:45-58), which writes the
// film through OpenImageIO as a 3-channel HALF image.
//
// File layout (OpenEXR 2.x single-part scanline file):
//   magic 20000630, version 2 (no flags);
//   header attributes (name, type, byte size, value), each NUL-terminated
//   name/type: channels (chlist B, G, R: HALF, linear 0, sampling 1 1),
//   compression (NONE), dataWindow = displayWindow = (0, 0)-(W-1, H-1),
//   lineOrder (INCREASING_Y), pixelAspectRatio 1, screenWindowCenter (0, 0),
//   screenWindowWidth 1; a NUL ends the header;
//   offset table: one uint64 file offset per scanline;
//   per scanline: int32 y, int32 byte count, then the B, G and R rows.
// All integers little-endian. Channels are stored in name order (B, G, R).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "drmlt_capi.h"
#include "errors.h"

namespace {

// IEEE 754 binary32 -> binary16, round to nearest even; overflow goes to
// infinity, NaN stays NaN (quiet), values below half the smallest subnormal
// go to signed zero.
uint16_t float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t exp = (x >> 23) & 0xffu;
    uint32_t man = x & 0x7fffffu;
    if (exp == 0xffu) return uint16_t(sign | 0x7c00u | (man ? (0x200u | (man >> 13)) : 0u));
    const int e = int(exp) - 112;  // rebiased exponent (127 -> 15)
    if (e >= 31) return uint16_t(sign | 0x7c00u);
    if (e <= 0) {  // half subnormal: value / 2^-24, from the 24-bit significand
        if (exp == 0) return uint16_t(sign);  // float zero or subnormal (< 2^-126)
        const int shift = 14 - e;
        if (shift > 24) return uint16_t(sign);
        man |= 0x800000u;
        uint32_t h = man >> shift;
        const uint32_t rem = man & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (h & 1u))) h++;
        return uint16_t(sign | h);
    }
    uint32_t h = (uint32_t(e) << 10) | (man >> 13);
    const uint32_t rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;  // a carry may reach infinity: correct
    return uint16_t(sign | h);
}

struct Out {
    std::vector<unsigned char> b;
    void u8(unsigned v) { b.push_back(static_cast<unsigned char>(v)); }
    void i32(int32_t v) {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        for (int k = 0; k < 4; k++) u8((u >> (8 * k)) & 0xffu);
    }
    void u64(uint64_t v) {
        for (int k = 0; k < 8; k++) u8(unsigned((v >> (8 * k)) & 0xffu));
    }
    void f32(float v) {
        int32_t i;
        std::memcpy(&i, &v, 4);
        i32(i);
    }
    void str(const char *s) {
        for (; *s; s++) u8(static_cast<unsigned char>(*s));
        u8(0);
    }
    void attr(const char *name, const char *type, int size) {
        str(name);
        str(type);
        i32(size);
    }
};

}  // namespace

extern "C" int drmlt_write_exr(const char *filename, int width, int height, const float *rgb) {
    if (!filename || !rgb || width <= 0 || height <= 0)
        return drmlt::set_error(DRMLT_E_ARG, "drmlt_write_exr: null argument or empty image");
    Out o;
    o.i32(20000630);
    o.i32(2);
    o.attr("channels", "chlist", 3 * (2 + 16) + 1);
    for (const char *c : {"B", "G", "R"}) {
        o.str(c);
        o.i32(1);  // HALF
        o.u8(0);   // pLinear
        o.u8(0);
        o.u8(0);
        o.u8(0);
        o.i32(1);
        o.i32(1);
    }
    o.u8(0);
    o.attr("compression", "compression", 1);
    o.u8(0);  // NO_COMPRESSION
    for (const char *w : {"dataWindow", "displayWindow"}) {
        o.attr(w, "box2i", 16);
        o.i32(0);
        o.i32(0);
        o.i32(width - 1);
        o.i32(height - 1);
    }
    o.attr("lineOrder", "lineOrder", 1);
    o.u8(0);  // INCREASING_Y
    o.attr("pixelAspectRatio", "float", 4);
    o.f32(1.0f);
    o.attr("screenWindowCenter", "v2f", 8);
    o.f32(0.0f);
    o.f32(0.0f);
    o.attr("screenWindowWidth", "float", 4);
    o.f32(1.0f);
    o.u8(0);  // end of header
    const size_t table = o.b.size();
    const int32_t rowBytes = int32_t(3 * 2 * size_t(width));
    const uint64_t first = table + 8 * uint64_t(height);
    for (int y = 0; y < height; y++) o.u64(first + uint64_t(y) * (8 + uint64_t(rowBytes)));
    for (int y = 0; y < height; y++) {
        o.i32(y);
        o.i32(rowBytes);
        for (int c = 2; c >= 0; c--)  // B, G, R
            for (int x = 0; x < width; x++) {
                const uint16_t h = float_to_half(rgb[(size_t(y) * width + x) * 3 + c]);
                o.u8(h & 0xffu);
                o.u8(h >> 8);
            }
    }
    FILE *f = std::fopen(filename, "wb");
    if (!f) return drmlt::set_error(DRMLT_E_IO, (std::string("cannot open ") + filename).c_str());
    const size_t n = std::fwrite(o.b.data(), 1, o.b.size(), f);
    const int closed = std::fclose(f);
    if (n != o.b.size() || closed != 0)
        return drmlt::set_error(DRMLT_E_IO, (std::string("cannot write ") + filename).c_str());
    return DRMLT_OK;
}
