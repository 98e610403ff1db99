// Image files on the host: the HDR mean image as OpenEXR and the display
// bytes as PNG.  The reference only shows its result in the window (the
// blit into the B8G8R8A8_SRGB swapchain, RenderTechniquePT.cpp:143-167);
// a headless renderer writes files instead.  Both writers are plain C++
// with no library behind them: EXR without compression, PNG with stored
// (uncompressed) deflate blocks.  Every multi-byte field is written byte by
// byte in the byte order its format fixes, so the files are the same on
// every host.
#include <cmath>
#include <cstring>
#include <fstream>

#include "vcr_internal.h"

namespace vcr {
namespace {

void put_u32le(std::vector<uint8_t>& b, uint32_t v) {
  for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
void put_u64le(std::vector<uint8_t>& b, uint64_t v) {
  for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}
void put_f32le(std::vector<uint8_t>& b, float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  put_u32le(b, u);
}
void put_u32be(std::vector<uint8_t>& b, uint32_t v) {
  for (int i = 3; i >= 0; --i) b.push_back((uint8_t)(v >> (8 * i)));
}
void put_str(std::vector<uint8_t>& b, const char* s) { b.insert(b.end(), s, s + std::strlen(s) + 1); }

// One header attribute: name, type name, value size, value bytes.
void put_attr(std::vector<uint8_t>& b, const char* name, const char* type, const std::vector<uint8_t>& value) {
  put_str(b, name);
  put_str(b, type);
  put_u32le(b, (uint32_t)value.size());
  b.insert(b.end(), value.begin(), value.end());
}

}  // namespace

// IEEE 754 binary32 -> binary16, rounded to nearest, ties to even; values
// beyond the largest half (65504) after rounding become infinity, NaNs stay
// NaNs (quiet, sign kept), results below the normal range are subnormal or
// zero.  Integer arithmetic on the bit fields only.
uint16_t float_to_half_rne(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t exp = (x >> 23) & 0xFFu;
  uint32_t man = x & 0x7FFFFFu;
  if (exp == 0xFFu) return (uint16_t)(sign | 0x7C00u | (man ? 0x200u | (man >> 13) : 0u));
  // the value is man' * 2^(exp - 150) with man' = man | 2^23 for normal floats
  const int e = (int)exp - 127;  // unbiased exponent
  if (e > 15) return (uint16_t)(sign | 0x7C00u);
  if (e >= -14) {  // normal half: keep 10 of the 23 mantissa bits
    uint32_t h = ((uint32_t)(e + 15) << 10) | (man >> 13);
    const uint32_t rest = man & 0x1FFFu;
    if (rest > 0x1000u || (rest == 0x1000u && (h & 1u))) ++h;  // a carry into the exponent is correct
    return (uint16_t)(sign | h);                                 // (and gives 0x7C00 = inf past 65504)
  }
  if (exp == 0) return (uint16_t)sign;  // float zero or subnormal: far below half's smallest subnormal
  // subnormal half: value / 2^-24, rounded; man' * 2^(e - 23) / 2^-24 = man' >> (-e - 1)
  man |= 0x800000u;
  const int shift = -e - 1;  // >= 14
  if (shift > 24) return (uint16_t)sign;  // below half of the smallest subnormal
  uint32_t h = man >> shift;
  const uint32_t rest = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
  if (rest > half || (rest == half && (h & 1u))) ++h;  // may round up into the smallest normal
  return (uint16_t)(sign | h);
}

}  // namespace vcr

using namespace vcr;

// OpenEXR 2.0, single part, scan lines, NO_COMPRESSION: magic and version,
// the required header attributes (channels B, G, R in name order,
// compression, dataWindow, displayWindow, lineOrder, pixelAspectRatio,
// screenWindowCenter, screenWindowWidth), the table of line offsets, then
// one chunk a line (y, byte count, the line's B values, G values, R values).
extern "C" VCR_API vcr_status vcr_write_exr(const char* path, uint32_t width, uint32_t height, const float* rgb,
                                            uint32_t type) {
  if (!path || !rgb) return fail(nullptr, VCR_ERR_INVALID, "null argument");
  if (!width || !height || width > (1u << 30) || height > (1u << 30))
    return fail(nullptr, VCR_ERR_INVALID, "image size %u x %u", width, height);
  if (type != VCR_EXR_HALF && type != VCR_EXR_FLOAT) return fail(nullptr, VCR_ERR_INVALID, "exr type %u", type);
  const uint32_t bytes = type == VCR_EXR_HALF ? 2u : 4u;
  const uint64_t line_bytes = 3ull * width * bytes;
  if (line_bytes > 0x7FFFFFFFull) return fail(nullptr, VCR_ERR_INVALID, "image line of %u pixels", width);

  std::vector<uint8_t> h;
  put_u32le(h, 20000630u);  // magic 0x762f3101 in file byte order
  put_u32le(h, 2u);         // version 2, no flags: single-part scan-line file
  std::vector<uint8_t> v;
  for (const char* name : {"B", "G", "R"}) {
    put_str(v, name);
    put_u32le(v, type);                   // pixel type: 1 HALF, 2 FLOAT
    v.insert(v.end(), {0, 0, 0, 0});      // pLinear, 3 reserved
    put_u32le(v, 1u);                     // x sampling
    put_u32le(v, 1u);                     // y sampling
  }
  v.push_back(0);
  put_attr(h, "channels", "chlist", v);
  put_attr(h, "compression", "compression", {0});  // NO_COMPRESSION
  v.clear();
  for (uint32_t c : {0u, 0u, width - 1u, height - 1u}) put_u32le(v, c);
  put_attr(h, "dataWindow", "box2i", v);
  put_attr(h, "displayWindow", "box2i", v);
  put_attr(h, "lineOrder", "lineOrder", {0});  // INCREASING_Y
  v.clear();
  put_f32le(v, 1.0f);
  put_attr(h, "pixelAspectRatio", "float", v);
  v.clear();
  put_f32le(v, 0.0f);
  put_f32le(v, 0.0f);
  put_attr(h, "screenWindowCenter", "v2f", v);
  v.clear();
  put_f32le(v, 1.0f);
  put_attr(h, "screenWindowWidth", "float", v);
  h.push_back(0);  // end of header

  const uint64_t chunk = 8ull + line_bytes;
  const uint64_t first = h.size() + 8ull * height;
  for (uint32_t y = 0; y < height; ++y) put_u64le(h, first + chunk * y);

  std::ofstream out(path, std::ios::binary);
  if (!out.good()) return fail(nullptr, VCR_ERR_IO, "cannot create %s", path);
  out.write(reinterpret_cast<const char*>(h.data()), (std::streamsize)h.size());
  std::vector<uint8_t> line;
  line.reserve((size_t)chunk);
  for (uint32_t y = 0; y < height; ++y) {
    line.clear();
    put_u32le(line, y);
    put_u32le(line, (uint32_t)line_bytes);
    const float* row = rgb + 3ull * width * y;
    for (int c = 2; c >= 0; --c)  // B, G, R
      for (uint32_t x = 0; x < width; ++x) {
        const float f = row[3ull * x + (uint32_t)c];
        if (type == VCR_EXR_HALF) {
          const uint16_t s = float_to_half_rne(f);
          line.push_back((uint8_t)s);
          line.push_back((uint8_t)(s >> 8));
        } else {
          put_f32le(line, f);
        }
      }
    out.write(reinterpret_cast<const char*>(line.data()), (std::streamsize)line.size());
  }
  if (!out.good()) return fail(nullptr, VCR_ERR_IO, "write failed: %s", path);
  return VCR_OK;
}

namespace vcr {
namespace {

// CRC-32 of PNG chunks (ISO 3309 polynomial, reflected: 0xEDB88320).
uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
  static uint32_t table[256];
  static bool ready = false;
  if (!ready) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    ready = true;
  }
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
  return crc;
}

void put_chunk(std::ofstream& out, const char* kind, const std::vector<uint8_t>& data) {
  std::vector<uint8_t> b;
  put_u32be(b, (uint32_t)data.size());
  b.insert(b.end(), kind, kind + 4);
  b.insert(b.end(), data.begin(), data.end());
  uint32_t crc = crc32_update(0xFFFFFFFFu, b.data() + 4, b.size() - 4) ^ 0xFFFFFFFFu;
  put_u32be(b, crc);
  out.write(reinterpret_cast<const char*>(b.data()), (std::streamsize)b.size());
}

}  // namespace
}  // namespace vcr

// PNG, 8-bit RGBA, filter 0 on every row; the zlib stream (RFC 1950) holds
// stored deflate blocks (RFC 1951 BTYPE 00) of at most 65,535 bytes and the
// Adler-32 of the filtered rows.
extern "C" VCR_API vcr_status vcr_write_png(const char* path, uint32_t width, uint32_t height, const uint8_t* rgba) {
  if (!path || !rgba) return fail(nullptr, VCR_ERR_INVALID, "null argument");
  if (!width || !height || width > (1u << 24) || height > (1u << 24))
    return fail(nullptr, VCR_ERR_INVALID, "image size %u x %u", width, height);
  const uint64_t row = 1ull + 4ull * width;
  const uint64_t raw = row * height;
  const uint64_t blocks = (raw + 65534) / 65535;
  if (2 + raw + 5 * blocks + 4 > 0x7FFFFFFFull) return fail(nullptr, VCR_ERR_INVALID, "image too large for one IDAT");
  std::vector<uint8_t> z;
  z.reserve((size_t)(2 + raw + 5 * blocks + 4));
  z.push_back(0x78);  // deflate, 32 KB window
  z.push_back(0x01);  // (0x78 << 8 | 0x01) % 31 == 0, no dictionary
  uint32_t a = 1, b = 0;  // Adler-32 sums
  uint64_t left = raw, block_left = 0;
  for (uint32_t y = 0; y < height; ++y)
    for (uint64_t i = 0; i < row; ++i) {
      if (block_left == 0) {
        const uint32_t len = (uint32_t)(left < 65535 ? left : 65535);
        z.push_back(left <= 65535 ? 1 : 0);  // BFINAL on the last block, BTYPE 00
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        block_left = len;
      }
      const uint8_t byte = i == 0 ? 0 : rgba[(4ull * width) * y + (i - 1)];
      z.push_back(byte);
      a = (a + byte) % 65521u;
      b = (b + a) % 65521u;
      --block_left;
      --left;
    }
  put_u32be(z, (b << 16) | a);

  std::ofstream out(path, std::ios::binary);
  if (!out.good()) return fail(nullptr, VCR_ERR_IO, "cannot create %s", path);
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  out.write(reinterpret_cast<const char*>(sig), 8);
  std::vector<uint8_t> ihdr;
  put_u32be(ihdr, width);
  put_u32be(ihdr, height);
  ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8 bits, RGBA, deflate, filter set 0, no interlace
  put_chunk(out, "IHDR", ihdr);
  put_chunk(out, "IDAT", z);
  put_chunk(out, "IEND", {});
  if (!out.good()) return fail(nullptr, VCR_ERR_IO, "write failed: %s", path);
  return VCR_OK;
}
