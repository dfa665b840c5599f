// netcdf3.cpp -- NetCDF-3 (CDF-1 / CDF-2) reader; see netcdf3.h.
//
// Layout (NetCDF classic format specification):
//   header  = 'C' 'D' 'F' version numrecs dim_list gatt_list var_list
//   list    = ABSENT (two zero words) | tag nelems [item ...]
//   dim     = name dim_length            (length 0 marks the record dim)
//   attr    = name nc_type nelems values (padded to 4 bytes)
//   var     = name nelems [dimid ...] vatt_list nc_type vsize begin
//   name    = nelems chars (padded to 4 bytes)
// Integers are big-endian; `begin` is 4 bytes in CDF-1 and 8 in CDF-2.
// Fixed-size variable data is contiguous at `begin`; record variables hold
// one slab per record at begin + r * record_size, where record_size is the
// sum of the record variables' vsize (or the unpadded slab size when there
// is a single record variable).

#include "netcdf3.h"

#include <errno.h>
#include <stdio.h>
#include <string.h>

#include <memory>

namespace mr {
namespace nc3 {

namespace {

constexpr uint32_t kTagDimension = 0x0A;
constexpr uint32_t kTagVariable = 0x0B;
constexpr uint32_t kTagAttribute = 0x0C;
constexpr int kIoError = -3;
constexpr int kReadError = -4;

int type_size(int t) {
  switch (t) {
    case NC_BYTE: case NC_CHAR: return 1;
    case NC_SHORT: return 2;
    case NC_INT: case NC_FLOAT: return 4;
    case NC_DOUBLE: return 8;
    default: return 0;
  }
}

struct FileCloser {
  void operator()(FILE *f) const { if (f) fclose(f); }
};

class Cursor {
 public:
  explicit Cursor(FILE *f) : f_(f) {}
  bool ok() const { return ok_; }
  uint32_t u32() {
    unsigned char b[4];
    if (!read(b, 4)) return 0;
    return (uint32_t(b[0]) << 24) | (uint32_t(b[1]) << 16) | (uint32_t(b[2]) << 8) | uint32_t(b[3]);
  }
  uint64_t u64() {
    const uint64_t hi = u32();
    const uint64_t lo = u32();
    return (hi << 32) | lo;
  }
  std::string name() {
    const uint32_t n = u32();
    if (!ok_ || n > (1u << 20)) { ok_ = false; return std::string(); }
    std::string s(n, '\0');
    if (n && !read(&s[0], n)) return std::string();
    skip((4 - n % 4) % 4);
    return s;
  }
  void skip(uint64_t n) {
    if (!ok_ || n == 0) return;
    if (fseeko(f_, static_cast<off_t>(n), SEEK_CUR) != 0) ok_ = false;
  }
  bool read(void *dst, size_t n) {
    if (!ok_) return false;
    if (fread(dst, 1, n, f_) != n) ok_ = false;
    return ok_;
  }

 private:
  FILE *f_;
  bool ok_ = true;
};

bool skip_attributes(Cursor &c) {
  const uint32_t tag = c.u32();
  const uint32_t n = c.u32();
  if (!c.ok()) return false;
  if (tag == 0 && n == 0) return true;
  if (tag != kTagAttribute) return false;
  for (uint32_t i = 0; i < n && c.ok(); ++i) {
    c.name();
    const int t = static_cast<int>(c.u32());
    const uint64_t count = c.u32();
    const int sz = type_size(t);
    if (!sz) return false;
    const uint64_t bytes = count * sz;
    c.skip(bytes + (4 - bytes % 4) % 4);
  }
  return c.ok();
}

Result parse_header(FILE *f, Header *h) {
  Cursor c(f);
  unsigned char magic[4];
  if (!c.read(magic, 4) || memcmp(magic, "CDF", 3) != 0)
    return {kReadError, "not a NetCDF-3 file (bad magic)"};
  if (magic[3] != 1 && magic[3] != 2)
    return {kReadError, "unsupported NetCDF format version " + std::to_string(magic[3]) +
                            " (only classic and 64-bit offset are read)"};
  h->version = magic[3];
  const uint32_t numrecs = c.u32();
  h->numrecs = numrecs == 0xFFFFFFFFu ? 0 : numrecs;
  // dimensions
  uint32_t tag = c.u32();
  uint32_t n = c.u32();
  if (!c.ok()) return {kReadError, "truncated header"};
  if (!(tag == 0 && n == 0)) {
    if (tag != kTagDimension) return {kReadError, "malformed dimension list"};
    for (uint32_t i = 0; i < n && c.ok(); ++i) {
      h->dim_names.push_back(c.name());
      h->dim_lengths.push_back(c.u32());
    }
  }
  if (!skip_attributes(c)) return {kReadError, "malformed global attributes"};
  tag = c.u32();
  n = c.u32();
  if (!c.ok()) return {kReadError, "truncated header"};
  if (!(tag == 0 && n == 0)) {
    if (tag != kTagVariable) return {kReadError, "malformed variable list"};
    for (uint32_t i = 0; i < n && c.ok(); ++i) {
      Variable v;
      v.name = c.name();
      const uint32_t nd = c.u32();
      if (nd > 1024) return {kReadError, "malformed variable"};
      for (uint32_t d = 0; d < nd; ++d) v.dimids.push_back(c.u32());
      if (!skip_attributes(c)) return {kReadError, "malformed variable attributes"};
      v.type = static_cast<int>(c.u32());
      v.vsize = c.u32();
      v.begin = h->version == 1 ? c.u32() : c.u64();
      for (uint32_t d : v.dimids)
        if (d >= h->dim_lengths.size()) return {kReadError, "variable uses an unknown dimension"};
      v.is_record = !v.dimids.empty() && h->dim_lengths[v.dimids[0]] == 0;
      h->vars.push_back(v);
    }
  }
  if (!c.ok()) return {kReadError, "truncated header"};
  int nrec_vars = 0;
  uint64_t single_slab = 0;
  for (const Variable &v : h->vars) {
    if (!v.is_record) continue;
    ++nrec_vars;
    h->record_size += v.vsize;
    uint64_t slab = type_size(v.type);
    for (size_t d = 1; d < v.dimids.size(); ++d) slab *= h->dim_lengths[v.dimids[d]];
    single_slab = slab;
  }
  if (nrec_vars == 1) h->record_size = single_slab;
  return {};
}

template <typename T>
T load_be(const unsigned char *p);

template <>
int8_t load_be<int8_t>(const unsigned char *p) { return static_cast<int8_t>(p[0]); }
template <>
uint8_t load_be<uint8_t>(const unsigned char *p) { return p[0]; }
template <>
int16_t load_be<int16_t>(const unsigned char *p) {
  return static_cast<int16_t>((uint16_t(p[0]) << 8) | uint16_t(p[1]));
}
template <>
int32_t load_be<int32_t>(const unsigned char *p) {
  return static_cast<int32_t>((uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) |
                              (uint32_t(p[2]) << 8) | uint32_t(p[3]));
}
template <>
float load_be<float>(const unsigned char *p) {
  const uint32_t u = static_cast<uint32_t>(load_be<int32_t>(p));
  float f;
  memcpy(&f, &u, 4);
  return f;
}
template <>
double load_be<double>(const unsigned char *p) {
  const uint64_t hi = static_cast<uint32_t>(load_be<int32_t>(p));
  const uint64_t lo = static_cast<uint32_t>(load_be<int32_t>(p + 4));
  const uint64_t u = (hi << 32) | lo;
  double d;
  memcpy(&d, &u, 8);
  return d;
}

// Converts `count` big-endian values of type `t` to double and (optionally)
// to the f32 the reference's bathymetry axes use.
void convert(const unsigned char *src, uint64_t count, int t, double *dst, float *dst32) {
  for (uint64_t i = 0; i < count; ++i) {
    double d;
    float f;
    switch (t) {
      case NC_BYTE: { const int8_t v = load_be<int8_t>(src + i); d = v; f = static_cast<float>(v); break; }
      case NC_CHAR: { const uint8_t v = load_be<uint8_t>(src + i); d = v; f = static_cast<float>(v); break; }
      case NC_SHORT: { const int16_t v = load_be<int16_t>(src + 2 * i); d = v; f = static_cast<float>(v); break; }
      case NC_INT: { const int32_t v = load_be<int32_t>(src + 4 * i); d = v; f = static_cast<float>(v); break; }
      case NC_FLOAT: { const float v = load_be<float>(src + 4 * i); d = v; f = v; break; }
      default: { const double v = load_be<double>(src + 8 * i); d = v; f = static_cast<float>(v); break; }
    }
    dst[i] = d;
    if (dst32) dst32[i] = f;
  }
}

}  // namespace

Result read_variable(const std::string &path, const std::string &name, std::vector<double> *values,
                     int *type, std::vector<float> *raw_f32) {
  std::unique_ptr<FILE, FileCloser> f(fopen(path.c_str(), "rb"));
  if (!f) return {kIoError, "cannot open '" + path + "': " + strerror(errno)};
  Header h;
  Result r = parse_header(f.get(), &h);
  if (r.code) {
    r.message = path + ": " + r.message;
    return r;
  }
  const Variable *var = nullptr;
  for (const Variable &v : h.vars)
    if (v.name == name) var = &v;
  if (!var) return {kReadError, path + ": no variable named '" + name + "'"};
  const int sz = type_size(var->type);
  if (!sz) return {kReadError, path + ": variable '" + name + "' has unsupported type " +
                                   std::to_string(var->type)};
  uint64_t per_slab = 1;
  for (size_t d = var->is_record ? 1 : 0; d < var->dimids.size(); ++d)
    per_slab *= h.dim_lengths[var->dimids[d]];
  const uint64_t slabs = var->is_record ? h.numrecs : 1;
  const uint64_t count = per_slab * slabs;
  if (fseeko(f.get(), 0, SEEK_END) != 0) return {kIoError, path + ": seek failed"};
  const uint64_t file_size = static_cast<uint64_t>(ftello(f.get()));
  const uint64_t slab_bytes = per_slab * sz;
  const uint64_t last_end =
      var->begin + (slabs ? (slabs - 1) * (var->is_record ? h.record_size : 0) : 0) + slab_bytes;
  if (slabs && last_end > file_size)
    return {kReadError, path + ": variable '" + name + "' extends past the end of the file"};
  values->assign(count, 0.0);
  if (raw_f32) raw_f32->assign(count, 0.0f);
  std::vector<unsigned char> buf(slab_bytes);
  for (uint64_t s = 0; s < slabs; ++s) {
    const uint64_t off = var->begin + s * (var->is_record ? h.record_size : 0);
    if (fseeko(f.get(), static_cast<off_t>(off), SEEK_SET) != 0 ||
        (slab_bytes && fread(buf.data(), 1, slab_bytes, f.get()) != slab_bytes))
      return {kIoError, path + ": read of '" + name + "' failed"};
    convert(buf.data(), per_slab, var->type, values->data() + s * per_slab,
            raw_f32 ? raw_f32->data() + s * per_slab : nullptr);
  }
  *type = var->type;
  return {};
}

}  // namespace nc3
}  // namespace mr
