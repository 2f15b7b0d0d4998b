#include "tiff.hpp"

#include <filesystem>
#include <fstream>
#include <iterator>

#include "ini.hpp"

namespace dcgpu {

namespace {

// TIFF 6.0 tags read here
enum : uint16_t {
  kImageWidth = 256, kImageLength = 257, kBitsPerSample = 258, kCompression = 259, kPhotometric = 262,
  kStripOffsets = 273, kSamplesPerPixel = 277, kRowsPerStrip = 278, kStripByteCounts = 279,
  kXResolution = 282, kYResolution = 283, kPlanarConfig = 284, kXPosition = 286, kYPosition = 287,
  kPredictor = 317, kTileWidth = 322
};

class Bytes {
 public:
  Bytes(std::vector<uint8_t> d, std::string name) : d_(std::move(d)), name_(std::move(name)) {}
  void set_big_endian(bool b) { be_ = b; }
  bool big_endian() const { return be_; }
  size_t size() const { return d_.size(); }
  const uint8_t* at(uint64_t off, uint64_t len) const {
    if (off > d_.size() || len > d_.size() - off) fail("truncated file");
    return d_.data() + off;
  }
  uint64_t uint(uint64_t off, int len) const {
    const uint8_t* p = at(off, len);
    uint64_t v = 0;
    for (int i = 0; i < len; ++i) v |= static_cast<uint64_t>(p[be_ ? len - 1 - i : i]) << (8 * i);
    return v;
  }
  [[noreturn]] void fail(const std::string& why) const {
    throw ConfigError("TIFF file '" + name_ + "': " + why);
  }

 private:
  std::vector<uint8_t> d_;
  std::string name_;
  bool be_ = false;
};

struct Entry {
  uint16_t type = 0;
  uint32_t count = 0;
  uint64_t value_off = 0;  // file offset of the value(s)
};

int type_size(uint16_t type) {
  switch (type) {
    case 1: case 2: case 6: case 7: return 1;   // BYTE ASCII SBYTE UNDEFINED
    case 3: case 8: return 2;                   // SHORT SSHORT
    case 4: case 9: case 11: return 4;          // LONG SLONG FLOAT
    case 5: case 10: case 12: return 8;         // RATIONAL SRATIONAL DOUBLE
    default: return 0;
  }
}

// i-th value of an integer-typed entry
uint64_t entry_uint(const Bytes& b, const Entry& e, uint32_t i) {
  if (i >= e.count) b.fail("tag value index out of range");
  const int sz = type_size(e.type);
  if (e.type != 1 && e.type != 3 && e.type != 4) b.fail("unexpected tag type");
  return b.uint(e.value_off + static_cast<uint64_t>(i) * sz, sz);
}

// RATIONAL as libtiff stores it: the quotient in double precision, kept as float
float entry_rational(const Bytes& b, const Entry& e) {
  if (e.type != 5 || e.count < 1) b.fail("resolution / position tags must be RATIONAL");
  const double num = static_cast<double>(b.uint(e.value_off, 4));
  const double den = static_cast<double>(b.uint(e.value_off + 4, 4));
  return den == 0.0 ? 0.0f : static_cast<float>(num / den);
}

void unpack_bits(const Bytes& b, const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
  size_t i = 0;
  while (i < n) {
    const int c = static_cast<int8_t>(p[i++]);
    if (c >= 0) {
      if (i + c + 1 > n) b.fail("PackBits literal run past the end of the strip");
      out.insert(out.end(), p + i, p + i + c + 1);
      i += c + 1;
    } else if (c != -128) {
      if (i >= n) b.fail("PackBits repeat run past the end of the strip");
      out.insert(out.end(), static_cast<size_t>(1 - c), p[i++]);
    }
  }
}

// LZW of TIFF 6.0 section 13: MSB-first codes of 9 to 12 bits, 256 = clear, 257 = end of
// information, the code width growing one code early (at 511, 1023, 2047 entries)
void lzw_decode(const Bytes& b, const uint8_t* p, size_t n, std::vector<uint8_t>& out) {
  constexpr int kClear = 256, kEoi = 257, kMaxCodes = 4096;
  std::vector<int> prefix(kMaxCodes, -1), length(kMaxCodes, 1);
  std::vector<uint8_t> last(kMaxCodes), first(kMaxCodes);
  for (int c = 0; c < 256; ++c) last[c] = first[c] = static_cast<uint8_t>(c);
  int next = 258, width = 9, prev = -1;
  uint64_t bitpos = 0;
  const uint64_t nbits = static_cast<uint64_t>(n) * 8;
  std::vector<uint8_t> tmp;
  auto read = [&]() -> int {
    if (bitpos + width > nbits) return kEoi;  // a strip may end without an explicit EOI
    int v = 0;
    for (int k = 0; k < width; ++k, ++bitpos) v = (v << 1) | ((p[bitpos >> 3] >> (7 - (bitpos & 7))) & 1);
    return v;
  };
  auto emit = [&](int code) {
    tmp.resize(length[code]);
    for (int c = code, k = length[code] - 1; k >= 0; c = prefix[c], --k) tmp[k] = last[c];
    out.insert(out.end(), tmp.begin(), tmp.end());
  };
  for (;;) {
    int code = read();
    if (code == kEoi) break;
    if (code == kClear) {
      next = 258;
      width = 9;
      code = read();
      if (code == kEoi) break;
      if (code >= 256) b.fail("LZW code after a clear code is not a literal");
      emit(code);
      prev = code;
      continue;
    }
    if (prev < 0) b.fail("LZW data does not start with a clear code");
    if (code > next || next >= kMaxCodes) b.fail("LZW code out of sequence");
    // new entry: the previous string + the first byte of the current one (KwKwK when the
    // current code is the entry being defined)
    const uint8_t f = code < next ? first[code] : first[prev];
    prefix[next] = prev;
    last[next] = f;
    first[next] = first[prev];
    length[next] = length[prev] + 1;
    ++next;
    emit(code);
    prev = code;
    if (next >= (1 << width) - 1 && width < 12) ++width;
  }
}

}  // namespace

TiffGray read_tiff_gray(const std::string& path) {
  namespace fs = std::filesystem;
  if (!fs::exists(path)) throw ConfigError("File '" + fs::absolute(path).string() + "' does not exists.");
  std::ifstream f(path, std::ios::binary);
  if (!f) throw ConfigError("Error opening TIFF file '" + path + "'");
  Bytes b(std::vector<uint8_t>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>()), path);
  if (b.size() < 8) throw ConfigError("Error opening TIFF file '" + path + "'");
  const uint8_t* h = b.at(0, 4);
  if (h[0] == 'I' && h[1] == 'I') b.set_big_endian(false);
  else if (h[0] == 'M' && h[1] == 'M') b.set_big_endian(true);
  else throw ConfigError("Error opening TIFF file '" + path + "'");
  if (b.uint(2, 2) != 42) throw ConfigError("Error opening TIFF file '" + path + "'");
  const uint64_t ifd = b.uint(4, 4);
  const uint64_t nent = b.uint(ifd, 2);
  std::vector<std::pair<uint16_t, Entry>> entries;
  for (uint64_t i = 0; i < nent; ++i) {
    const uint64_t o = ifd + 2 + 12 * i;
    Entry e;
    const uint16_t tag = static_cast<uint16_t>(b.uint(o, 2));
    e.type = static_cast<uint16_t>(b.uint(o + 2, 2));
    e.count = static_cast<uint32_t>(b.uint(o + 4, 4));
    const uint64_t bytes = static_cast<uint64_t>(type_size(e.type)) * e.count;
    e.value_off = bytes <= 4 ? o + 8 : b.uint(o + 8, 4);
    entries.emplace_back(tag, e);
  }
  auto find = [&](uint16_t tag) -> const Entry* {
    for (const auto& te : entries)
      if (te.first == tag) return &te.second;
    return nullptr;
  };
  auto get = [&](uint16_t tag, uint64_t dflt) -> uint64_t {
    const Entry* e = find(tag);
    return e ? entry_uint(b, *e, 0) : dflt;
  };

  TiffGray t;
  const Entry* ph = find(kPhotometric);
  if (!ph) b.fail("no PhotometricInterpretation tag");
  const uint64_t photometric = entry_uint(b, *ph, 0);
  // tiff_file.cc:25-29: WhiteIsZero (0) or BlackIsZero (1)
  if (photometric != 0 && photometric != 1)
    throw ConfigError("TIFF file '" + path + "' must be in grayscale");
  t.black_is_zero = photometric == 1;
  t.bits = static_cast<uint16_t>(get(kBitsPerSample, 1));
  t.rows = static_cast<uint32_t>(get(kImageLength, 0));
  t.cols = static_cast<uint32_t>(get(kImageWidth, 0));
  const Entry* xr = find(kXResolution);
  const Entry* yr = find(kYResolution);
  t.x_res = xr ? entry_rational(b, *xr) : 0.0f;
  t.y_res = yr ? entry_rational(b, *yr) : 0.0f;
  // tiff_file.cc:36-38 (FloatCmp::le with a relative tolerance: a non-positive value)
  if (!(t.x_res > 0.0f) || !(t.y_res > 0.0f))
    throw ConfigError("TIFF file '" + path + "' has negative resolution");
  const Entry* xp = find(kXPosition);
  const Entry* yp = find(kYPosition);
  t.x_off = xp ? entry_rational(b, *xp) : 0.0f;
  t.y_off = yp ? entry_rational(b, *yp) : 0.0f;
  // tiff_grayscale.cc:68-79: 1, 2, 4 or 8 bytes per sample
  if (t.bits != 8 && t.bits != 16 && t.bits != 32 && t.bits != 64)
    throw ConfigError("Encoding with " + std::to_string(t.bits) + " bits not implemented");
  if (t.rows == 0 || t.cols == 0) b.fail("empty image");
  if (find(kTileWidth)) b.fail("tiled images are not supported (strips only)");
  if (get(kSamplesPerPixel, 1) != 1) b.fail("only one sample per pixel is supported");
  if (get(kPlanarConfig, 1) != 1) b.fail("only contiguous planar configuration is supported");
  const uint64_t compression = get(kCompression, 1);
  const uint64_t predictor = get(kPredictor, 1);
  if (compression != 1 && compression != 5 && compression != 32773)
    b.fail("compression " + std::to_string(compression) + " is not supported (none, LZW, PackBits)");
  if (predictor != 1 && !(predictor == 2 && compression == 5)) b.fail("unsupported predictor");

  const int bps = t.bits / 8;
  const uint64_t row_bytes = static_cast<uint64_t>(t.cols) * bps;
  const uint64_t total = row_bytes * t.rows;
  const Entry* so = find(kStripOffsets);
  const Entry* sc = find(kStripByteCounts);
  if (!so || !sc || so->count != sc->count || so->count == 0) b.fail("missing or inconsistent strip tags");
  std::vector<uint8_t> raw;
  raw.reserve(total);
  for (uint32_t s = 0; s < so->count && raw.size() < total; ++s) {
    const uint64_t off = entry_uint(b, *so, s), len = entry_uint(b, *sc, s);
    const uint8_t* p = b.at(off, len);
    if (compression == 1) raw.insert(raw.end(), p, p + len);
    else if (compression == 32773) unpack_bits(b, p, len, raw);
    else lzw_decode(b, p, len, raw);
  }
  if (raw.size() < total) b.fail("image data shorter than ImageLength x ImageWidth");

  // samples in native order, then the predictor's running sums along each scanline
  std::vector<uint64_t> v(static_cast<size_t>(t.rows) * t.cols);
  for (size_t k = 0; k < v.size(); ++k) {
    uint64_t x = 0;
    for (int i = 0; i < bps; ++i) x |= static_cast<uint64_t>(raw[k * bps + i]) << (8 * (b.big_endian() ? bps - 1 - i : i));
    v[k] = x;
  }
  const uint64_t mask = t.bits == 64 ? ~uint64_t{0} : ((uint64_t{1} << t.bits) - 1);
  if (predictor == 2)
    for (uint32_t r = 0; r < t.rows; ++r)
      for (uint32_t c = 1; c < t.cols; ++c) {
        const size_t k = static_cast<size_t>(r) * t.cols + c;
        v[k] = (v[k] + v[k - 1]) & mask;
      }
  // tiff_grayscale.cc:25,46-52: divided by 2^bits (1 << bits in a 64-bit size_t; for 64-bit
  // samples that shift count wraps to 0 in the reference's x86-64 build, a divisor of 1)
  const uint64_t max = t.bits == 64 ? 1 : (uint64_t{1} << t.bits);
  t.px.resize(v.size());
  for (size_t k = 0; k < v.size(); ++k) {
    const uint64_t val = t.black_is_zero ? v[k] : max - v[k];
    t.px[k] = static_cast<double>(val) / static_cast<double>(max);
  }
  return t;
}

}  // namespace dcgpu
