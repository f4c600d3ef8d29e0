// netCDF classic file formats (CDF-1, CDF-2 = 64-bit offset, CDF-5 = 64-bit
// data): the header grammar and data layout of the published "NetCDF Classic
// and 64-bit Offset Format" specification and its CDF-5 extension, restated
// for reading and writing MPAS mesh and history files without HDF5.
//
// Layout recap.  All values big-endian.  Header: magic "CDF" + version byte,
// record count, then dimension, global attribute and variable lists, each a
// 4-byte tag + element count (or 8 zero bytes / 12 for CDF-5 when absent).
// Counts, lengths, dimension ids and vsize are 4 bytes (8 in CDF-5); variable
// offsets 4 bytes in CDF-1, 8 otherwise; names and attribute values are padded
// to 4 bytes.  Fixed-size variables are stored whole, one after another;
// record variables (first dimension unlimited) interleave: record r of a
// variable sits at begin + r * recsize, recsize being the sum of the record
// variables' padded sizes.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "common.hh"
#include "mpaso_io.h"

namespace mpaso {
namespace {

constexpr uint32_t kDimTag = 0x0A, kVarTag = 0x0B, kAttTag = 0x0C;
constexpr uint32_t kStreaming = 0xFFFFFFFFu;

int type_size(int32_t t) {
  switch (t) {
    case MPASO_NC_BYTE:
    case MPASO_NC_CHAR: return 1;
    case MPASO_NC_SHORT: return 2;
    case MPASO_NC_INT:
    case MPASO_NC_FLOAT: return 4;
    case MPASO_NC_DOUBLE:
    case MPASO_NC_INT64: return 8;
    default: return 0;
  }
}

int64_t pad4(int64_t n) { return (n + 3) & ~int64_t(3); }

struct Att {
  std::string name;
  int32_t type = 0;
  int64_t n = 0;
  std::vector<uint8_t> be;  // values, big-endian, unpadded
};

struct Dim {
  std::string name;
  int64_t len = 0;  // 0: the record dimension
};

struct Var {
  std::string name;
  std::vector<int32_t> dims;
  std::vector<Att> atts;
  int32_t type = 0;
  int64_t vsize = 0;  // padded bytes of the variable (of one record for record variables)
  int64_t begin = 0;
  bool rec = false;
  int64_t count = 0;  // elements (per record for record variables)
};

struct NcFile {
  FILE *fp = nullptr;
  std::string path;
  int version = 1;
  bool define = false, writable = false;
  int64_t numrecs = 0, recsize = 0;
  std::vector<Dim> dims;
  std::vector<Att> gatts;
  std::vector<Var> vars;
  ~NcFile() {
    if (fp) fclose(fp);
  }
};

[[noreturn]] void io_fail(const NcFile &f, const std::string &msg) { fail(MPASO_ERR_IO, f.path + ": " + msg); }

// ---------------------------------------------------------------- bytes
void put_be(std::vector<uint8_t> &b, uint64_t v, int n) {
  for (int i = n - 1; i >= 0; --i) b.push_back((uint8_t)(v >> (8 * i)));
}
uint64_t get_be(const uint8_t *p, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; ++i) v = (v << 8) | p[i];
  return v;
}

// Sequential header reader over the open file.
struct Reader {
  NcFile &f;
  int64_t pos = 0;
  int64_t size = 0;  // bytes in the file
  explicit Reader(NcFile &file) : f(file) {
    const long at = ftell(f.fp);
    if (at < 0 || fseek(f.fp, 0, SEEK_END) != 0) io_fail(f, "cannot size the file");
    size = (int64_t)ftell(f.fp);
    if (size < 0 || fseek(f.fp, at, SEEK_SET) != 0) io_fail(f, "cannot size the file");
    pos = at;
  }
  // Bytes of a count or size field (NON_NEG: 4, 8 in CDF-5).
  int nn() const { return f.version == 5 ? 8 : 4; }
  // Refuses a count read from the header whose entries, at `each` bytes at
  // least, could not fit in what is left of the file -- before any vector is
  // sized by it, so a corrupt or truncated header costs no large allocation.
  int64_t fits(int64_t n, int64_t each, const char *what) {
    const int64_t left = size - pos;
    if (n < 0 || (each > 0 && n > left / each)) io_fail(f, std::string("truncated or corrupt header (") + what + ")");
    return n;
  }
  void bytes(void *dst, int64_t n) {
    if (n > 0 && fread(dst, 1, (size_t)n, f.fp) != (size_t)n) io_fail(f, "truncated header");
    pos += n;
  }
  uint64_t be(int n) {
    uint8_t b[8];
    bytes(b, n);
    return get_be(b, n);
  }
  int64_t nonneg() {  // NON_NEG: 4 bytes, 8 in CDF-5
    const uint64_t v = be(f.version == 5 ? 8 : 4);
    if (v > (uint64_t)INT64_MAX) io_fail(f, "count out of range");
    return (int64_t)v;
  }
  std::string name() {
    const int64_t n = nonneg();
    if (n <= 0 || n > 4096) io_fail(f, "bad name length");
    std::string s((size_t)n, '\0');
    bytes(&s[0], n);
    skip(pad4(n) - n);
    return s;
  }
  void skip(int64_t n) {
    uint8_t b[8];
    while (n > 0) {
      const int64_t k = n < 8 ? n : 8;
      bytes(b, k);
      n -= k;
    }
  }
  // tag + count; ABSENT is a zero tag with a zero count
  int64_t list(uint32_t tag) {
    const uint32_t t = (uint32_t)be(4);
    const int64_t n = nonneg();
    if (t == 0 && n == 0) return 0;
    if (t != tag) io_fail(f, "malformed header (unexpected list tag)");
    return n;
  }
  std::vector<Att> atts() {
    // an attribute takes at least a name (count + 4), a type and a count
    std::vector<Att> out((size_t)fits(list(kAttTag), 2 * nn() + 8, "attribute count"));
    for (Att &a : out) {
      a.name = name();
      a.type = (int32_t)be(4);
      const int ts = type_size(a.type);
      if (!ts || (a.type == MPASO_NC_INT64 && f.version != 5)) io_fail(f, "bad attribute type");
      a.n = nonneg();
      if (a.n < 0 || a.n > (int64_t)1 << 30) io_fail(f, "attribute too large");
      fits(a.n, ts, "attribute length");
      a.be.resize((size_t)(a.n * ts));
      bytes(a.be.data(), (int64_t)a.be.size());
      skip(pad4((int64_t)a.be.size()) - (int64_t)a.be.size());
    }
    return out;
  }
};

int64_t var_count(const NcFile &f, const Var &v) {
  int64_t n = 1;
  for (size_t i = v.rec ? 1 : 0; i < v.dims.size(); ++i) {
    const int64_t d = f.dims[v.dims[i]].len;
    if (d < 0 || (d > 0 && n > INT64_MAX / d)) io_fail(f, "variable size overflows");
    n *= d;
  }
  return n;
}

// Record size: padded sizes summed, except a lone byte/char/short record variable
// whose records are not padded.
int64_t record_size(const NcFile &f) {
  int64_t total = 0, nrec = 0;
  const Var *only = nullptr;
  for (const Var &v : f.vars)
    if (v.rec) total += v.vsize, ++nrec, only = &v;
  if (nrec == 1 && type_size(only->type) < 4) return only->count * type_size(only->type);
  return total;
}

void read_header(NcFile &f) {
  Reader r(f);
  char magic[4];
  r.bytes(magic, 4);
  if (memcmp(magic, "CDF", 3) != 0) io_fail(f, "not a netCDF classic file (HDF5-based netCDF-4 needs libhdf5)");
  f.version = magic[3];
  if (f.version != 1 && f.version != 2 && f.version != 5) io_fail(f, "unknown netCDF classic version");
  const uint64_t nr = r.be(f.version == 5 ? 8 : 4);
  const bool streaming = f.version == 5 ? nr == ~0ULL : nr == kStreaming;
  f.numrecs = streaming ? -1 : (int64_t)nr;
  // a dimension takes at least a name (count + 4) and a length
  f.dims.resize((size_t)r.fits(r.list(kDimTag), 2 * r.nn() + 4, "dimension count"));
  int nrecdims = 0;
  for (Dim &d : f.dims) {
    d.name = r.name();
    d.len = r.nonneg();
    if (d.len == 0) ++nrecdims;
  }
  if (nrecdims > 1) io_fail(f, "more than one record dimension");
  f.gatts = r.atts();
  // a variable takes at least a name (count + 4), a dimension count, an empty
  // attribute list (tag + count), a type, a size and a 4-byte offset
  f.vars.resize((size_t)r.fits(r.list(kVarTag), 4 * r.nn() + 16, "variable count"));
  for (Var &v : f.vars) {
    v.name = r.name();
    const int64_t nd = r.nonneg();
    if (nd > 64) io_fail(f, "too many dimensions");
    r.fits(nd, r.nn(), "dimension ids");
    v.dims.resize((size_t)nd);
    for (int32_t &d : v.dims) {
      const int64_t id = r.nonneg();
      if (id >= (int64_t)f.dims.size()) io_fail(f, "bad dimension id");
      d = (int32_t)id;
    }
    v.atts = r.atts();
    v.type = (int32_t)r.be(4);
    if (!type_size(v.type) || (v.type == MPASO_NC_INT64 && f.version != 5)) io_fail(f, "bad variable type");
    v.vsize = r.nonneg();
    v.begin = (int64_t)r.be(f.version == 1 ? 4 : 8);
    for (size_t i = 1; i < v.dims.size(); ++i)
      if (f.dims[v.dims[i]].len == 0) io_fail(f, "record dimension not first");
    v.rec = !v.dims.empty() && f.dims[v.dims[0]].len == 0;
    v.count = var_count(f, v);
    // vsize can be clamped for huge variables in CDF-1/2: recompute it
    v.vsize = pad4(v.count * type_size(v.type));
  }
  f.recsize = record_size(f);
  if (f.numrecs < 0) {  // streaming: the records present in the file
    int64_t start = -1;
    for (const Var &v : f.vars)
      if (v.rec && (start < 0 || v.begin < start)) start = v.begin;
    fseeko(f.fp, 0, SEEK_END);
    const int64_t size = ftello(f.fp);
    f.numrecs = (start < 0 || f.recsize == 0) ? 0 : (size - start) / f.recsize;
  }
}

std::vector<uint8_t> encode_header(const NcFile &f) {
  std::vector<uint8_t> b = {'C', 'D', 'F', (uint8_t)f.version};
  const int nn = f.version == 5 ? 8 : 4;
  auto nonneg = [&](int64_t v) { put_be(b, (uint64_t)v, nn); };
  auto name = [&](const std::string &s) {
    nonneg((int64_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
    b.resize(b.size() + (size_t)(pad4((int64_t)s.size()) - (int64_t)s.size()), 0);
  };
  auto list = [&](uint32_t tag, size_t n) {
    put_be(b, n ? tag : 0, 4);
    nonneg((int64_t)n);
  };
  auto atts = [&](const std::vector<Att> &as) {
    list(kAttTag, as.size());
    for (const Att &a : as) {
      name(a.name);
      put_be(b, (uint32_t)a.type, 4);
      nonneg(a.n);
      b.insert(b.end(), a.be.begin(), a.be.end());
      b.resize(b.size() + (size_t)(pad4((int64_t)a.be.size()) - (int64_t)a.be.size()), 0);
    }
  };
  nonneg(f.numrecs);
  list(kDimTag, f.dims.size());
  for (const Dim &d : f.dims) {
    name(d.name);
    nonneg(d.len);
  }
  atts(f.gatts);
  list(kVarTag, f.vars.size());
  for (const Var &v : f.vars) {
    name(v.name);
    nonneg((int64_t)v.dims.size());
    for (int32_t d : v.dims) nonneg(d);
    atts(v.atts);
    put_be(b, (uint32_t)v.type, 4);
    // CDF-1/2 clamp vsize of a variable past 4 GiB (only the last may be that large)
    nonneg(f.version != 5 && v.vsize > 0xFFFFFFFCLL ? 0xFFFFFFFFLL : v.vsize);
    put_be(b, (uint64_t)v.begin, f.version == 1 ? 4 : 8);
  }
  return b;
}

// ---------------------------------------------------------------- conversion
// External (big-endian, file type) <-> memory (native, mem type).
struct Val {
  bool is_int;
  int64_t i;
  double d;
};

Val load_ext(const uint8_t *p, int32_t t) {
  switch (t) {
    case MPASO_NC_BYTE: return {true, (int8_t)p[0], 0.0};
    case MPASO_NC_CHAR: return {true, (int64_t)p[0], 0.0};
    case MPASO_NC_SHORT: return {true, (int16_t)(uint16_t)get_be(p, 2), 0.0};
    case MPASO_NC_INT: return {true, (int32_t)(uint32_t)get_be(p, 4), 0.0};
    case MPASO_NC_INT64: return {true, (int64_t)get_be(p, 8), 0.0};
    case MPASO_NC_FLOAT: {
      const uint32_t u = (uint32_t)get_be(p, 4);
      float x;
      memcpy(&x, &u, 4);
      return {false, 0, (double)x};
    }
    default: {
      const uint64_t u = get_be(p, 8);
      double x;
      memcpy(&x, &u, 8);
      return {false, 0, x};
    }
  }
}

Val load_mem(const uint8_t *p, int32_t t) {
  switch (t) {
    case MPASO_NC_BYTE: return {true, *(const int8_t *)p, 0.0};
    case MPASO_NC_CHAR: return {true, (int64_t)*p, 0.0};
    case MPASO_NC_SHORT: {
      int16_t x;
      memcpy(&x, p, 2);
      return {true, x, 0.0};
    }
    case MPASO_NC_INT: {
      int32_t x;
      memcpy(&x, p, 4);
      return {true, x, 0.0};
    }
    case MPASO_NC_INT64: {
      int64_t x;
      memcpy(&x, p, 8);
      return {true, x, 0.0};
    }
    case MPASO_NC_FLOAT: {
      float x;
      memcpy(&x, p, 4);
      return {false, 0, (double)x};
    }
    default: {
      double x;
      memcpy(&x, p, 8);
      return {false, 0, x};
    }
  }
}

// Integer range of a type (CHAR: bytes).
void int_range(int32_t t, int64_t &lo, int64_t &hi) {
  switch (t) {
    case MPASO_NC_BYTE: lo = -128, hi = 127; break;
    case MPASO_NC_CHAR: lo = 0, hi = 255; break;
    case MPASO_NC_SHORT: lo = -32768, hi = 32767; break;
    case MPASO_NC_INT: lo = INT32_MIN, hi = INT32_MAX; break;
    default: lo = INT64_MIN, hi = INT64_MAX;
  }
}

bool is_float(int32_t t) { return t == MPASO_NC_FLOAT || t == MPASO_NC_DOUBLE; }

// Value converted to type t; false when it does not fit (integer targets).
bool fits(const Val &v, int32_t t) {
  if (is_float(t)) return true;
  int64_t lo, hi;
  int_range(t, lo, hi);
  if (v.is_int) return v.i >= lo && v.i <= hi;
  return v.d == v.d && v.d >= (double)lo && v.d <= (double)hi;
}

void store(uint8_t *p, const Val &v, int32_t t, bool big_endian) {
  const int n = type_size(t);
  uint64_t u = 0;
  if (t == MPASO_NC_FLOAT) {
    const float x = (float)(v.is_int ? (double)v.i : v.d);
    uint32_t w;
    memcpy(&w, &x, 4);
    u = w;
  } else if (t == MPASO_NC_DOUBLE) {
    const double x = v.is_int ? (double)v.i : v.d;
    memcpy(&u, &x, 8);
  } else {
    const int64_t x = v.is_int ? v.i : (int64_t)v.d;
    u = (uint64_t)x;
  }
  if (big_endian) {
    for (int i = 0; i < n; ++i) p[i] = (uint8_t)(u >> (8 * (n - 1 - i)));
  } else {
    // native order: write through the integer of the type's width
    switch (n) {
      case 1: *p = (uint8_t)u; break;
      case 2: {
        const uint16_t w = (uint16_t)u;
        memcpy(p, &w, 2);
        break;
      }
      case 4: {
        const uint32_t w = (uint32_t)u;
        memcpy(p, &w, 4);
        break;
      }
      default: memcpy(p, &u, 8);
    }
  }
}

void check_types(const NcFile &f, int32_t ext, int32_t mem) {
  if (!type_size(mem)) fail(MPASO_ERR_ARG, "unknown memory type");
  if ((ext == MPASO_NC_CHAR) != (mem == MPASO_NC_CHAR))
    fail(MPASO_ERR_ARG, f.path + ": CHAR data converts only to and from CHAR");
}

// File bytes [count elements of ext] -> memory [mem].
void from_file(const NcFile &f, int64_t off, int64_t count, int32_t ext, int32_t mem, void *out) {
  check_types(f, ext, mem);
  const int es = type_size(ext), ms = type_size(mem);
  const int64_t chunk = 1 << 16;
  std::vector<uint8_t> buf((size_t)(chunk * es));
  if (fseeko(f.fp, off, SEEK_SET) != 0) io_fail(f, "seek failed");
  uint8_t *dst = (uint8_t *)out;
  for (int64_t done = 0; done < count;) {
    const int64_t k = count - done < chunk ? count - done : chunk;
    if (fread(buf.data(), 1, (size_t)(k * es), f.fp) != (size_t)(k * es)) io_fail(f, "truncated data");
    for (int64_t i = 0; i < k; ++i) {
      const Val v = load_ext(buf.data() + i * es, ext);
      if (!fits(v, mem)) fail(MPASO_ERR_ARG, f.path + ": value out of range of the memory type");
      store(dst + (done + i) * ms, v, mem, false);
    }
    done += k;
  }
}

// Memory [count elements of mem] -> file bytes [ext], zero padding to `padded` bytes.
void to_file(const NcFile &f, int64_t off, int64_t count, int32_t ext, int32_t mem, const void *in,
             int64_t padded) {
  check_types(f, ext, mem);
  const int es = type_size(ext), ms = type_size(mem);
  const int64_t chunk = 1 << 16;
  std::vector<uint8_t> buf((size_t)(chunk * es));
  if (fseeko(f.fp, off, SEEK_SET) != 0) io_fail(f, "seek failed");
  const uint8_t *src = (const uint8_t *)in;
  for (int64_t done = 0; done < count;) {
    const int64_t k = count - done < chunk ? count - done : chunk;
    for (int64_t i = 0; i < k; ++i) {
      const Val v = load_mem(src + (done + i) * ms, mem);
      if (!fits(v, ext)) fail(MPASO_ERR_ARG, f.path + ": value out of range of the file type");
      store(buf.data() + i * es, v, ext, true);
    }
    if (fwrite(buf.data(), 1, (size_t)(k * es), f.fp) != (size_t)(k * es)) io_fail(f, "write failed");
    done += k;
  }
  static const uint8_t zeros[4] = {0, 0, 0, 0};
  const int64_t pad = padded - count * es;
  if (pad > 0 && fwrite(zeros, 1, (size_t)pad, f.fp) != (size_t)pad) io_fail(f, "write failed");
}

void write_numrecs(NcFile &f) {
  std::vector<uint8_t> b;
  put_be(b, (uint64_t)f.numrecs, f.version == 5 ? 8 : 4);
  if (fseeko(f.fp, 4, SEEK_SET) != 0 || fwrite(b.data(), 1, b.size(), f.fp) != b.size())
    io_fail(f, "write failed");
}

// ---------------------------------------------------------------- lookup
NcFile &handle(mpaso_nc h);
Var &find_var(NcFile &f, const char *name) {
  require(name != nullptr, MPASO_ERR_ARG, "null name");
  for (Var &v : f.vars)
    if (v.name == name) return v;
  fail(MPASO_ERR_NOTFOUND, f.path + ": no variable " + name);
}
std::vector<Att> &att_list(NcFile &f, const char *var) { return var ? find_var(f, var).atts : f.gatts; }

void copy_name(const std::string &s, char *buf, int32_t buflen) {
  require(buf != nullptr && buflen > (int32_t)s.size(), MPASO_ERR_ARG, "name buffer too small");
  memcpy(buf, s.c_str(), s.size() + 1);
}

void check_name(const char *name) {
  require(name && *name && !strchr(name, '/') && strlen(name) < 4096, MPASO_ERR_ARG, "bad name");
}

}  // namespace
}  // namespace mpaso

struct mpaso_nc_s {
  mpaso::NcFile f;
};

namespace mpaso {
namespace {
NcFile &handle(mpaso_nc h) {
  require(h != nullptr, MPASO_ERR_ARG, "null file handle");
  return h->f;
}
void data_mode(NcFile &f) { require(!f.define, MPASO_ERR_ARG, f.path + ": still in define mode"); }
}  // namespace
}  // namespace mpaso

using namespace mpaso;

extern "C" {

int mpaso_nc_open(const char *path, int32_t writable, mpaso_nc *out) {
  return guarded("mpaso_nc_open", [&] {
    require(path && out, MPASO_ERR_ARG, "null argument");
    auto h = std::make_unique<mpaso_nc_s>();
    NcFile &f = h->f;
    f.path = path;
    f.writable = writable != 0;
    f.fp = fopen(path, f.writable ? "r+b" : "rb");
    if (!f.fp) fail(MPASO_ERR_IO, std::string(path) + ": cannot open");
    read_header(f);
    *out = h.release();
  });
}

int mpaso_nc_create(const char *path, int32_t version, mpaso_nc *out) {
  return guarded("mpaso_nc_create", [&] {
    require(path && out, MPASO_ERR_ARG, "null argument");
    require(version == 1 || version == 2 || version == 5, MPASO_ERR_ARG, "version must be 1, 2 or 5");
    auto h = std::make_unique<mpaso_nc_s>();
    NcFile &f = h->f;
    f.path = path;
    f.version = version;
    f.define = f.writable = true;
    f.fp = fopen(path, "w+b");
    if (!f.fp) fail(MPASO_ERR_IO, std::string(path) + ": cannot create");
    *out = h.release();
  });
}

int mpaso_nc_close(mpaso_nc h) {
  return guarded("mpaso_nc_close", [&] {
    std::unique_ptr<mpaso_nc_s> own(h);
    NcFile &f = handle(h);
    if (f.define) {
      const int rc = mpaso_nc_enddef(h);
      if (rc != MPASO_OK) fail(rc, "enddef at close failed");
    }
    if (f.writable) {
      write_numrecs(f);
      if (fflush(f.fp) != 0) io_fail(f, "flush failed");
    }
  });
}

int mpaso_nc_def_dim(mpaso_nc h, const char *name, int64_t len) {
  return guarded("mpaso_nc_def_dim", [&] {
    NcFile &f = handle(h);
    require(f.define, MPASO_ERR_ARG, "not in define mode");
    check_name(name);
    require(len >= 0, MPASO_ERR_ARG, "negative dimension length");
    require(len <= (f.version == 5 ? INT64_MAX : (int64_t)INT32_MAX), MPASO_ERR_ARG,
            "dimension too long for this version");
    for (const Dim &d : f.dims) {
      require(d.name != name, MPASO_ERR_ARG, std::string("dimension exists: ") + name);
      require(!(len == 0 && d.len == 0), MPASO_ERR_ARG, "only one record dimension");
    }
    f.dims.push_back({name, len});
  });
}

int mpaso_nc_def_var(mpaso_nc h, const char *name, int32_t type, int32_t ndims, const char *const *dims) {
  return guarded("mpaso_nc_def_var", [&] {
    NcFile &f = handle(h);
    require(f.define, MPASO_ERR_ARG, "not in define mode");
    check_name(name);
    require(type_size(type) && (type != MPASO_NC_INT64 || f.version == 5), MPASO_ERR_ARG,
            "type not available in this version");
    require(ndims >= 0 && ndims <= 64 && (ndims == 0 || dims), MPASO_ERR_ARG, "bad dimensions");
    for (const Var &v : f.vars) require(v.name != name, MPASO_ERR_ARG, std::string("variable exists: ") + name);
    Var v;
    v.name = name, v.type = type;
    for (int32_t i = 0; i < ndims; ++i) {
      int32_t id = -1;
      for (size_t j = 0; j < f.dims.size(); ++j)
        if (dims[i] && f.dims[j].name == dims[i]) id = (int32_t)j;
      require(id >= 0, MPASO_ERR_NOTFOUND, std::string("no dimension ") + (dims[i] ? dims[i] : "(null)"));
      require(i == 0 || f.dims[id].len != 0, MPASO_ERR_ARG, "the record dimension must come first");
      v.dims.push_back(id);
    }
    v.rec = ndims > 0 && f.dims[v.dims[0]].len == 0;
    v.count = var_count(f, v);
    v.vsize = pad4(v.count * type_size(type));
    f.vars.push_back(v);
  });
}

int mpaso_nc_put_att(mpaso_nc h, const char *var, const char *name, int32_t type, int64_t n, const void *values) {
  return guarded("mpaso_nc_put_att", [&] {
    NcFile &f = handle(h);
    require(f.define, MPASO_ERR_ARG, "not in define mode");
    check_name(name);
    require(type_size(type) && (type != MPASO_NC_INT64 || f.version == 5), MPASO_ERR_ARG, "bad attribute type");
    require(n >= 0 && (n == 0 || values), MPASO_ERR_ARG, "bad attribute values");
    Att a;
    a.name = name, a.type = type, a.n = n;
    a.be.resize((size_t)(n * type_size(type)));
    for (int64_t i = 0; i < n; ++i)
      store(a.be.data() + i * type_size(type), load_mem((const uint8_t *)values + i * type_size(type), type), type,
            true);
    auto &list = att_list(f, var);
    for (Att &x : list)
      if (x.name == name) {
        x = a;
        return;
      }
    list.push_back(a);
  });
}

int mpaso_nc_enddef(mpaso_nc h) {
  return guarded("mpaso_nc_enddef", [&] {
    NcFile &f = handle(h);
    require(f.define, MPASO_ERR_ARG, "not in define mode");
    // offsets depend on the header size, which does not depend on their values
    const int64_t hsize = (int64_t)encode_header(f).size();
    int64_t off = hsize;
    for (Var &v : f.vars)
      if (!v.rec) v.begin = off, off += v.vsize;
    for (Var &v : f.vars)
      if (v.rec) v.begin = off, off += v.vsize;
    f.recsize = record_size(f);
    const int64_t limit = f.version == 1 ? (int64_t)INT32_MAX : INT64_MAX;
    for (const Var &v : f.vars)
      require(v.begin <= limit, MPASO_ERR_ARG, f.path + ": data past 2 GiB need version 2 or 5");
    if (f.version != 5) {  // CDF-1/2: only the last fixed variable / last record variable may pass 4 GiB
      for (size_t i = 0; i + 1 < f.vars.size(); ++i)
        require(f.vars[i].vsize <= 0xFFFFFFFCLL, MPASO_ERR_ARG, f.path + ": variable past 4 GiB needs version 5");
    }
    const std::vector<uint8_t> b = encode_header(f);
    if (fseeko(f.fp, 0, SEEK_SET) != 0 || fwrite(b.data(), 1, b.size(), f.fp) != b.size()) io_fail(f, "write failed");
    f.define = false;
  });
}

int mpaso_nc_put_var(mpaso_nc h, const char *name, int32_t mem_type, const void *data) {
  return guarded("mpaso_nc_put_var", [&] {
    NcFile &f = handle(h);
    data_mode(f);
    require(f.writable, MPASO_ERR_ARG, "file opened read-only");
    Var &v = find_var(f, name);
    require(!v.rec, MPASO_ERR_ARG, v.name + " is a record variable: use mpaso_nc_put_rec");
    require(data || v.count == 0, MPASO_ERR_ARG, "null data");
    to_file(f, v.begin, v.count, v.type, mem_type, data, v.vsize);
  });
}

int mpaso_nc_put_rec(mpaso_nc h, const char *name, int64_t rec, int32_t mem_type, const void *data) {
  return guarded("mpaso_nc_put_rec", [&] {
    NcFile &f = handle(h);
    data_mode(f);
    require(f.writable, MPASO_ERR_ARG, "file opened read-only");
    Var &v = find_var(f, name);
    require(v.rec, MPASO_ERR_ARG, v.name + " is not a record variable");
    require(rec >= 0 && rec <= f.numrecs, MPASO_ERR_ARG, "record index past the end + 1");
    require(data || v.count == 0, MPASO_ERR_ARG, "null data");
    const bool lone_short = f.recsize < v.vsize;  // unpadded lone small-type record variable
    to_file(f, v.begin + rec * f.recsize, v.count, v.type, mem_type, data,
            lone_short ? v.count * type_size(v.type) : v.vsize);
    if (rec == f.numrecs) {
      f.numrecs = rec + 1;
      write_numrecs(f);
    }
  });
}

int mpaso_nc_get_var(mpaso_nc h, const char *name, int32_t mem_type, void *out) {
  return guarded("mpaso_nc_get_var", [&] {
    NcFile &f = handle(h);
    data_mode(f);
    Var &v = find_var(f, name);
    require(out || v.count == 0, MPASO_ERR_ARG, "null output");
    if (!v.rec) {
      from_file(f, v.begin, v.count, v.type, mem_type, out);
      return;
    }
    for (int64_t r = 0; r < f.numrecs; ++r)
      from_file(f, v.begin + r * f.recsize, v.count, v.type, mem_type,
                (uint8_t *)out + r * v.count * type_size(mem_type));
  });
}

int mpaso_nc_get_rec(mpaso_nc h, const char *name, int64_t rec, int32_t mem_type, void *out) {
  return guarded("mpaso_nc_get_rec", [&] {
    NcFile &f = handle(h);
    data_mode(f);
    Var &v = find_var(f, name);
    require(v.rec, MPASO_ERR_ARG, v.name + " is not a record variable");
    require(rec >= 0 && rec < f.numrecs, MPASO_ERR_ARG, "record index out of range");
    require(out || v.count == 0, MPASO_ERR_ARG, "null output");
    from_file(f, v.begin + rec * f.recsize, v.count, v.type, mem_type, out);
  });
}

int mpaso_nc_inq(mpaso_nc h, int32_t *version, int64_t *numrecs, int32_t *ndims, int32_t *nvars, int32_t *ngatts) {
  return guarded("mpaso_nc_inq", [&] {
    NcFile &f = handle(h);
    if (version) *version = f.version;
    if (numrecs) *numrecs = f.numrecs;
    if (ndims) *ndims = (int32_t)f.dims.size();
    if (nvars) *nvars = (int32_t)f.vars.size();
    if (ngatts) *ngatts = (int32_t)f.gatts.size();
  });
}

int mpaso_nc_inq_dim(mpaso_nc h, const char *name, int64_t *len) {
  return guarded("mpaso_nc_inq_dim", [&] {
    NcFile &f = handle(h);
    require(name && len, MPASO_ERR_ARG, "null argument");
    for (const Dim &d : f.dims)
      if (d.name == name) {
        *len = d.len == 0 ? f.numrecs : d.len;
        return;
      }
    fail(MPASO_ERR_NOTFOUND, f.path + ": no dimension " + name);
  });
}

int mpaso_nc_dim_name(mpaso_nc h, int32_t id, char *buf, int32_t buflen, int64_t *len) {
  return guarded("mpaso_nc_dim_name", [&] {
    NcFile &f = handle(h);
    require(id >= 0 && id < (int32_t)f.dims.size(), MPASO_ERR_ARG, "dimension id out of range");
    copy_name(f.dims[id].name, buf, buflen);
    if (len) *len = f.dims[id].len == 0 ? f.numrecs : f.dims[id].len;
  });
}

int mpaso_nc_var_name(mpaso_nc h, int32_t id, char *buf, int32_t buflen) {
  return guarded("mpaso_nc_var_name", [&] {
    NcFile &f = handle(h);
    require(id >= 0 && id < (int32_t)f.vars.size(), MPASO_ERR_ARG, "variable id out of range");
    copy_name(f.vars[id].name, buf, buflen);
  });
}

int mpaso_nc_inq_var(mpaso_nc h, const char *name, int32_t *type, int32_t *ndims, int64_t *shape, int32_t *is_record) {
  return guarded("mpaso_nc_inq_var", [&] {
    NcFile &f = handle(h);
    const Var &v = find_var(f, name);
    require(v.dims.size() <= 8 || !shape, MPASO_ERR_ARG, "more than 8 dimensions");
    if (type) *type = v.type;
    if (ndims) *ndims = (int32_t)v.dims.size();
    if (shape)
      for (size_t i = 0; i < v.dims.size(); ++i) shape[i] = f.dims[v.dims[i]].len == 0 ? f.numrecs : f.dims[v.dims[i]].len;
    if (is_record) *is_record = v.rec ? 1 : 0;
  });
}

int mpaso_nc_var_dim_name(mpaso_nc h, const char *var, int32_t i, char *buf, int32_t buflen) {
  return guarded("mpaso_nc_var_dim_name", [&] {
    NcFile &f = handle(h);
    const Var &v = find_var(f, var);
    require(i >= 0 && i < (int32_t)v.dims.size(), MPASO_ERR_ARG, "dimension index out of range");
    copy_name(f.dims[v.dims[i]].name, buf, buflen);
  });
}

int mpaso_nc_get_att(mpaso_nc h, const char *var, const char *name, int32_t *type, int64_t *n, void *out,
                     int64_t cap_bytes) {
  return guarded("mpaso_nc_get_att", [&] {
    NcFile &f = handle(h);
    require(name != nullptr, MPASO_ERR_ARG, "null name");
    for (const Att &a : att_list(f, var))
      if (a.name == name) {
        if (type) *type = a.type;
        if (n) *n = a.n;
        if (out) {
          const int ts = type_size(a.type);
          require(cap_bytes >= a.n * ts, MPASO_ERR_ARG, "attribute buffer too small");
          for (int64_t i = 0; i < a.n; ++i)
            store((uint8_t *)out + i * ts, load_ext(a.be.data() + i * ts, a.type), a.type, false);
        }
        return;
      }
    fail(MPASO_ERR_NOTFOUND, f.path + ": no attribute " + name);
  });
}

int mpaso_nc_att_name(mpaso_nc h, const char *var, int32_t id, char *buf, int32_t buflen) {
  return guarded("mpaso_nc_att_name", [&] {
    NcFile &f = handle(h);
    const auto &list = att_list(f, var);
    require(id >= 0 && id < (int32_t)list.size(), MPASO_ERR_ARG, "attribute id out of range");
    copy_name(list[id].name, buf, buflen);
  });
}

}  // extern "C"
