// hdr_io.cpp -- Radiance .hdr parsing on the host (or3_read_hdr).
//
// Replaces the file-reading half of HDRImage::ReadFromRadianceFile
// (src/tools/HDRImage.cpp:12-186) for the GPU path: the header ("#?" program
// line, key=value lines up to a blank line, then "-Y <height> +X <width>"),
// and the scanlines, either flat RGBE quadruples or the run-length form (a
// scanline starts 2, 2, width >> 8, width & 255; then each of the four
// channels in turn as runs: a count byte above 128 repeats the next byte
// count - 128 times, a count byte of 1..128 is followed by that many literal
// bytes).  As in the reference, widths below 8 or above 0x7fff are flat, and
// a scanline that does not start with the run-length marker switches the rest
// of the image to flat pixels.  The output is the RGBE bytes; the conversion
// to floats (RGBE2Color) runs on the device.
#include <cstdio>
#include <cstring>
#include <string>

#include "or3.h"

namespace {

struct Reader {
  const uint8_t *p, *end;
  bool line(std::string &out) {
    out.clear();
    if (p >= end) return false;
    while (p < end && *p != '\n') out.push_back((char)*p++);
    if (p < end) p++;  // the newline
    return true;
  }
  bool bytes(uint8_t *dst, size_t n) {
    if ((size_t)(end - p) < n) return false;
    std::memcpy(dst, p, n);
    p += n;
    return true;
  }
};

bool parse_dims(const std::string &s, uint32_t *w, uint32_t *h) {
  char ya[3] = {0}, xa[3] = {0};
  long hh = 0, ww = 0;
  if (std::sscanf(s.c_str(), "%2s %ld %2s %ld", ya, &hh, xa, &ww) != 4) return false;
  if (std::strcmp(ya, "-Y") != 0 || std::strcmp(xa, "+X") != 0) return false;  // the only orientation read
  if (hh <= 0 || ww <= 0 || hh > (1 << 20) || ww > (1 << 20)) return false;
  *w = (uint32_t)ww;
  *h = (uint32_t)hh;
  return true;
}

// scanlines from the reader into out (w * h * 4 bytes)
bool pixels(Reader &r, uint32_t w, uint32_t h, uint8_t *out) {
  const size_t total = (size_t)w * h;
  if (w < 8 || w > 0x7fff) return r.bytes(out, 4 * total);
  std::string scan(4 * (size_t)w, '\0');
  for (uint32_t y = 0; y < h; y++) {
    uint8_t q[4];
    if (!r.bytes(q, 4)) return false;
    if (q[0] != 2 || q[1] != 2 || (q[2] & 0x80)) {
      // not run-length encoded: this quadruple is a pixel, the rest is flat
      uint8_t *dst = out + 4 * (size_t)y * w;
      std::memcpy(dst, q, 4);
      return r.bytes(dst + 4, 4 * (total - (size_t)y * w - 1));
    }
    if ((((uint32_t)q[2] << 8) | q[3]) != w) return false;
    for (int c = 0; c < 4; c++) {
      uint8_t *ch = reinterpret_cast<uint8_t *>(&scan[(size_t)c * w]);
      uint32_t x = 0;
      while (x < w) {
        uint8_t b[2];
        if (!r.bytes(b, 2)) return false;
        if (b[0] > 128) {
          const uint32_t n = b[0] - 128u;
          if (n == 0 || n > w - x) return false;
          std::memset(ch + x, b[1], n);
          x += n;
        } else {
          const uint32_t n = b[0];
          if (n == 0 || n > w - x) return false;
          ch[x++] = b[1];
          if (n > 1) {
            if (!r.bytes(ch + x, n - 1)) return false;
            x += n - 1;
          }
        }
      }
    }
    uint8_t *dst = out + 4 * (size_t)y * w;
    for (uint32_t x = 0; x < w; x++)
      for (int c = 0; c < 4; c++) dst[4 * x + c] = (uint8_t)scan[(size_t)c * w + x];
  }
  return true;
}

}  // namespace

extern "C" int or3_read_hdr(const uint8_t *file, size_t length, uint32_t *width_out, uint32_t *height_out,
                            uint8_t *rgbe, size_t capacity) {
  if (!file || !width_out || !height_out) return OR3_ERR_INVALID_ARGUMENT;
  Reader r{file, file + length};
  std::string s;
  if (!r.line(s) || s.compare(0, 2, "#?") != 0) return OR3_ERR_INVALID_ARGUMENT;
  for (;;) {  // header lines up to the blank line
    if (!r.line(s)) return OR3_ERR_INVALID_ARGUMENT;
    if (s.empty()) break;
    if (s.compare(0, 7, "FORMAT=") == 0 && s != "FORMAT=32-bit_rle_rgbe") return OR3_ERR_INVALID_ARGUMENT;
  }
  uint32_t w = 0, h = 0;
  if (!r.line(s) || !parse_dims(s, &w, &h)) return OR3_ERR_INVALID_ARGUMENT;
  *width_out = w;
  *height_out = h;
  if (!rgbe) return OR3_OK;
  if (capacity < 4 * (size_t)w * h) return OR3_ERR_INVALID_ARGUMENT;
  return pixels(r, w, h, rgbe) ? OR3_OK : OR3_ERR_INVALID_ARGUMENT;
}
