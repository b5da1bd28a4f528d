// NCC model files.  The byte format is the reference's, so files written by
// either side load in the other byte for byte (src/ncc_matching/persist.cpp,
// text conventions of src/core/model_text.hpp):
//
//   "MVKIT_NCC 1\n" <FNV-1a 64 of the body, decimal> "\n" <body>
//   body: levels polarity angle_start angle_extent angle_step \n
//         origin_row origin_col width height \n
//         level0_origin_row level0_origin_col \n
//         width*height lines "mask gray" (level-0 raster minus the template mean)
//
// Numbers are written in the classic "C" form: integers (and doubles that
// are integers within 2^53) in plain decimal, other doubles with 17
// significant digits in the %g style, negative zero as "-0".
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstring>
#include <fstream>
#include <locale>
#include <sstream>
#include <string>
#include <string_view>
#include <system_error>

#include "ncc_model.h"

namespace mvg {
namespace {

constexpr size_t kMaxModelFile = 64u * 1024u * 1024u;  // persist.cpp:14
constexpr size_t kMaxModelPixels = 1048576;           // persist.cpp:14
constexpr std::string_view kMagic = "MVKIT_NCC 1";

uint64_t fnv1a64(std::string_view bytes) {
  uint64_t h = 14695981039346656037ULL;
  for (const unsigned char b : bytes) {
    h ^= b;
    h *= 1099511628211ULL;
  }
  return h;
}

// Appends numbers in the file's decimal conventions.
struct Writer {
  std::string out;
  void put(char c) { out.push_back(c); }
  void put_int(int64_t v) {
    char b[24];
    const auto r = std::to_chars(b, b + sizeof(b), v);
    out.append(b, r.ptr);
  }
  void put_size(size_t v) {
    char b[24];
    const auto r = std::to_chars(b, b + sizeof(b), v);
    out.append(b, r.ptr);
  }
  void put_real(double v) {
    if (v == 0.) {
      if (std::signbit(v)) out.push_back('-');
      out.push_back('0');
      return;
    }
    if (v >= -9007199254740992. && v <= 9007199254740992.) {
      const int64_t i = static_cast<int64_t>(v);
      if (static_cast<double>(i) == v) return put_int(i);
    }
    char b[40];
    const auto r = std::to_chars(b, b + sizeof(b), v, std::chars_format::general, 17);
    out.append(b, r.ptr);
  }
};

[[noreturn]] void decode_error(const char* what) { raise(kDecodeError, what); }

// Whitespace-separated fields of a model body (the six classic-locale ASCII
// blanks).  Numbers parse like the C++ stream extractors in the classic
// locale: a leading '+' is accepted, and anything std::from_chars does not
// finish (an exponent it rejects, inf/nan words, hex) goes to a classic
// istringstream.
class Fields {
 public:
  explicit Fields(std::string_view s) : s_(s) {}
  static bool blank(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t' || c == '\v' || c == '\f'; }
  void skip() {
    while (!s_.empty() && blank(s_.front())) s_.remove_prefix(1);
  }
  bool at_end() {
    skip();
    return s_.empty();
  }
  template <class T> T next() {
    skip();
    const std::string_view whole = s_;
    if (s_.empty()) decode_error("invalid or truncated model field");
    if (s_.front() == '+') {
      s_.remove_prefix(1);
      if (s_.empty() || s_.front() == '+' || s_.front() == '-') decode_error("invalid or truncated model field");
    }
    T v{};
    const auto r = std::from_chars(s_.data(), s_.data() + s_.size(), v);
    bool slow = r.ec != std::errc{};
    if constexpr (std::is_floating_point_v<T>) {
      const char* e = r.ptr;
      slow = slow || (e != s_.data() + s_.size() && (*e == 'e' || *e == 'E' || *e == 'x' || *e == 'X'));
      const char f = s_.front();
      slow = slow || f == 'i' || f == 'I' || f == 'n' || f == 'N';
    }
    if (!slow) {
      s_.remove_prefix(size_t(r.ptr - s_.data()));
      return v;
    }
    std::istringstream in{std::string(whole)};
    in.imbue(std::locale::classic());
    if (!(in >> v)) decode_error("invalid or truncated model field");
    const auto at = in.tellg();
    s_ = at < 0 ? std::string_view{} : whole.substr(size_t(at));
    return v;
  }
  double real() {
    const double v = next<double>();
    if (!std::isfinite(v)) decode_error("non-finite model field");
    return v;
  }
  size_t count(size_t limit) {
    const int64_t v = next<int64_t>();
    if (v < 0 || uint64_t(v) > limit) raise(kLimitExceeded, "model count exceeds budget");
    return size_t(v);
  }

 private:
  std::string_view s_;
};

}  // namespace

// serialize(), src/ncc_matching/persist.cpp:33-43
std::string serialize_model(const HostModel& m) {
  if (m.levels.empty()) raise(kInvalidState, "cannot save empty model");
  const ModelLevel& L = m.levels.front();
  const CreateParams& o = m.params;
  Writer w;
  w.out.reserve(64 + L.gray.size() * 8);
  w.put_int(o.levels);
  w.put(' ');
  w.put_int(o.ignore_polarity ? 1 : 0);
  w.put(' ');
  w.put_real(o.angle_start);
  w.put(' ');
  w.put_real(o.angle_extent);
  w.put(' ');
  w.put_real(o.angle_step);
  w.put('\n');
  w.put_real(m.origin_row);
  w.put(' ');
  w.put_real(m.origin_col);
  w.put(' ');
  w.put_size(L.width);
  w.put(' ');
  w.put_size(L.height);
  w.put('\n');
  w.put_real(L.orow);
  w.put(' ');
  w.put_real(L.ocol);
  w.put('\n');
  for (size_t i = 0; i < L.gray.size(); ++i) {
    w.put_int(L.mask[i]);
    w.put(' ');
    w.put_real(L.gray[i]);
    w.put('\n');
  }
  if (w.out.size() > kMaxModelFile) raise(kLimitExceeded, "serialized model exceeds file budget");
  char b[24];
  const auto r = std::to_chars(b, b + sizeof(b), fnv1a64(w.out));
  std::string file;
  file.reserve(kMagic.size() + 22 + w.out.size());
  file.append(kMagic);
  file.push_back('\n');
  file.append(b, r.ptr);
  file.push_back('\n');
  file.append(w.out);
  return file;
}

// deserialize(), src/ncc_matching/persist.cpp:44-77
HostModel deserialize_model(std::string_view bytes, bool rasters) {
  if (bytes.size() > kMaxModelFile + 128) raise(kLimitExceeded, "model file exceeds budget");
  // signature line (std::getline: up to the first '\n', which is consumed)
  const size_t nl = bytes.find('\n');
  const std::string_view magic = bytes.substr(0, nl);
  std::string_view rest = nl == std::string_view::npos ? std::string_view{} : bytes.substr(nl + 1);
  if (magic != kMagic)
    raise(magic.substr(0, 10) == "MVKIT_NCC " ? kUnsupported : kDecodeError, "invalid model signature or version");
  // checksum: an unsigned decimal (stream rules: leading blanks skipped),
  // then exactly one '\n'
  uint64_t expected = 0;
  {
    size_t p = 0;
    while (p < rest.size() && Fields::blank(rest[p])) ++p;
    size_t q = p;
    while (q < rest.size() && !Fields::blank(rest[q])) ++q;
    std::istringstream in{std::string(rest.substr(p, q - p))};
    in.imbue(std::locale::classic());
    if (!(in >> expected)) decode_error("invalid or truncated model field");
    const auto at = in.tellg();  // -1 once the whole token was consumed
    const size_t used = p + (at < 0 ? q - p : size_t(at));
    if (used >= rest.size() || rest[used] != '\n') decode_error("invalid checksum header");
    rest.remove_prefix(used + 1);
  }
  if (fnv1a64(rest) != expected) decode_error("NCC model checksum mismatch");

  Fields f(rest);
  CreateParams o;
  o.levels = int(f.count(16));
  o.ignore_polarity = f.count(1) != 0;
  o.angle_start = f.real();
  o.angle_extent = f.real();
  o.angle_step = f.real();
  if (o.angle_extent < 0 || o.angle_extent > 6.283185307179586 || o.angle_step <= 0 ||
      !std::isfinite(o.angle_start + o.angle_extent))
    decode_error("invalid trained angle interval");
  const double origin_row = f.real(), origin_col = f.real();
  ModelLevel first;
  first.width = f.count(kMaxModelPixels);
  first.height = f.count(kMaxModelPixels);
  if (!first.width || !first.height || first.height > kMaxModelPixels / first.width)
    raise(kLimitExceeded, "invalid model dimensions");
  first.orow = f.real();
  first.ocol = f.real();
  const size_t px = first.width * first.height;
  first.gray.resize(px);
  first.mask.resize(px);
  long double rsum = 0, csum = 0;
  size_t n = 0;
  for (size_t i = 0; i < px; ++i) {
    first.mask[i] = uint8_t(f.count(1));
    first.gray[i] = f.real();
    if (first.mask[i]) {
      rsum += i / first.width;
      csum += i % first.width;
      ++n;
    }
  }
  // the stored centroids must be the raster's and differ from the absolute
  // origin by whole pixels
  const double dr = origin_row - first.orow, dc = origin_col - first.ocol;
  if (n < 4 || std::abs(first.orow - double(rsum / n)) > 1e-10 || std::abs(first.ocol - double(csum / n)) > 1e-10 ||
      origin_row < first.orow || origin_col < first.ocol || std::abs(dr - std::round(dr)) > 1e-8 ||
      std::abs(dc - std::round(dc)) > 1e-8)
    decode_error("invalid template domain centroid");
  if (!f.at_end()) decode_error("trailing model data");
  try {
    return rebuild_model(std::move(first), o, origin_row, origin_col, rasters);
  } catch (const Error& e) {
    raise(e.status == kLimitExceeded ? kLimitExceeded : kDecodeError, "invalid prepared NCC model");
  }
}

// write() / read() with the file-level checks of src/core/model_io.hpp:13-19
// and src/core/model_io.cpp:39-50.
void write_model_file(const HostModel& m, const std::string& path) {
  const std::string bytes = serialize_model(m);
  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) raise(kIoError, "cannot open model for writing");
  out.write(bytes.data(), std::streamsize(bytes.size()));
  out.flush();
  if (!out) raise(kIoError, "cannot write model file");
}

HostModel read_model_file(const std::string& path, bool rasters) {
  std::ifstream in(path, std::ios::binary | std::ios::ate);
  if (!in) raise(kIoError, "cannot open model for reading");
  const auto size = in.tellg();
  if (size < 0 || size > std::streamoff(kMaxModelFile + 128)) raise(kLimitExceeded, "model file exceeds size limit");
  std::string bytes(size_t(size), '\0');
  in.seekg(0);
  if (!bytes.empty()) in.read(bytes.data(), std::streamsize(bytes.size()));
  if (!in) raise(kIoError, "cannot read model file");
  return deserialize_model(bytes, rasters);
}

}  // namespace mvg
