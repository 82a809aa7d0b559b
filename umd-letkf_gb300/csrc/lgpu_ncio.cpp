// lgpu_ncio.cpp -- the file formats on either side of the analysis path, host
// code: NetCDF classic files read and written without the netCDF library.
//
// The reference reads observations (src/subclass.letkf_obsio/letkf_obsio_nc.F90
// :150-330), reads and writes ensemble state (src/subclass.letkf_stateio/
// letkf_stateio_nc.F90:196-370) and writes the solver's and the ocean
// localizer's diagnostics (src/letkf_solver.F90:397-527,
// src/subclass.letkf_localizer/letkf_loc_ocean.F90:249-322) through
// netCDF-Fortran.  Here the published classic format is read and written
// directly:
//
//   file    = 'C' 'D' 'F' version, numrecs, dimensions, global attributes,
//             variables (name, dimension ids, attributes, type, vsize,
//             begin), then the data; everything big-endian
//   version 1 = classic (32-bit offsets), 2 = 64-bit offset, 5 = 64-bit
//             data (64-bit counts and sizes, extra integer types)
//   data    = every fixed-size variable contiguous at its `begin`, padded
//             to 4 bytes; record variables interleaved record by record
//             (one record = each record variable's slab in turn, each
//             padded to 4 bytes unless it is the only record variable).
//
// Reading takes versions 1, 2 and 5 and converts any numeric type to float
// or int.  Writing produces version 1 (as nf90_create(..., NF90_CLOBBER)
// does for the diagnostics) and switches to version 2 when the file passes
// 2 GiB.  NetCDF-4 files (HDF5 containers, which stateio_nc writes with
// nf90_hdf5 and deflate) are refused with LGPU_ERR_UNSUPPORTED: convert them
// to a classic format first (e.g. nccopy -k classic).
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "letkf_gpu.h"

namespace {

thread_local std::string g_io_err;

int io_fail(int code, const std::string &msg) {
  g_io_err = msg;
  return code;
}

enum NcType { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6, NC_UBYTE = 7,
              NC_USHORT = 8, NC_UINT = 9, NC_INT64 = 10, NC_UINT64 = 11 };

int type_size(int t) {
  switch (t) {
  case NC_BYTE: case NC_CHAR: case NC_UBYTE: return 1;
  case NC_SHORT: case NC_USHORT: return 2;
  case NC_INT: case NC_FLOAT: case NC_UINT: return 4;
  case NC_DOUBLE: case NC_INT64: case NC_UINT64: return 8;
  default: return 0;
  }
}

const uint32_t TAG_DIM = 0x0A, TAG_VAR = 0x0B, TAG_ATT = 0x0C;

// ------------------------------------------------------------------ reader
struct Dim { std::string name; uint64_t len; };
struct Var {
  std::string name;
  std::vector<int> dimids;
  int type = 0;
  uint64_t vsize = 0, begin = 0;
  bool record = false;
};

struct NcFile {
  std::vector<unsigned char> hdr;   // header bytes (read in full)
  FILE *f = nullptr;
  int version = 0;
  uint64_t numrecs = 0, recsize = 0;
  int recdim = -1;
  std::vector<Dim> dims;
  std::vector<Var> vars;
  std::string path;
  ~NcFile() { if (f) fclose(f); }
};

struct Cursor {
  const std::vector<unsigned char> &b;
  size_t p = 0;
  bool ok = true;
  explicit Cursor(const std::vector<unsigned char> &buf) : b(buf) {}
  uint64_t be(int n) {
    if (p + n > b.size()) { ok = false; return 0; }
    uint64_t v = 0;
    for (int i = 0; i < n; i++) v = (v << 8) | b[p + i];
    p += n;
    return v;
  }
  void skip(uint64_t n) {
    if (p + n > b.size()) { ok = false; return; }
    p += n;
  }
};

uint64_t pad4(uint64_t n) { return (n + 3) & ~(uint64_t)3; }

int nc_open(NcFile &nc, const char *path) {
  if (!path) return io_fail(LGPU_ERR_ARG, "null path");
  nc.path = path;
  nc.f = fopen(path, "rb");
  if (!nc.f) return io_fail(LGPU_ERR_ARG, std::string("cannot open ") + path + ": " + strerror(errno));
  unsigned char magic[8] = {0};
  if (fread(magic, 1, 8, nc.f) < 4) return io_fail(LGPU_ERR_ARG, std::string(path) + ": not a netCDF file");
  if (magic[0] == 0x89 && magic[1] == 'H' && magic[2] == 'D' && magic[3] == 'F')
    return io_fail(LGPU_ERR_UNSUPPORTED, std::string(path) + ": a NetCDF-4 (HDF5) file; only the classic formats "
                                         "(CDF-1, CDF-2, CDF-5) are read: convert it, e.g. nccopy -k classic");
  if (magic[0] != 'C' || magic[1] != 'D' || magic[2] != 'F' || (magic[3] != 1 && magic[3] != 2 && magic[3] != 5))
    return io_fail(LGPU_ERR_ARG, std::string(path) + ": not a netCDF classic file");
  nc.version = magic[3];
  // read the header: grow until it parses
  size_t want = 1 << 16;
  for (;;) {
    nc.hdr.assign(want, 0);
    fseek(nc.f, 0, SEEK_SET);
    const size_t got = fread(nc.hdr.data(), 1, want, nc.f);
    nc.hdr.resize(got);
    Cursor c(nc.hdr);
    c.skip(4);
    const int ns = nc.version == 5 ? 8 : 4;   // size of counts
    const int os = nc.version == 1 ? 4 : 8;   // size of offsets
    nc.numrecs = c.be(ns);
    nc.dims.clear();
    nc.vars.clear();
    auto name = [&](std::string &out) {
      const uint64_t n = c.be(ns);
      if (!c.ok || c.p + n > nc.hdr.size()) { c.ok = false; return; }
      out.assign(reinterpret_cast<const char *>(&nc.hdr[c.p]), n);
      c.skip(pad4(n));
    };
    auto atts = [&]() {
      const uint64_t tag = c.be(4), n = c.be(ns);
      if (tag != 0 && tag != TAG_ATT) { c.ok = false; return; }
      for (uint64_t i = 0; i < n && c.ok; i++) {
        std::string an;
        name(an);
        const int t = (int)c.be(4);
        const uint64_t ne = c.be(ns);
        c.skip(pad4(ne * type_size(t)));
      }
    };
    uint64_t tag = c.be(4), n = c.be(ns);
    if (tag != 0 && tag != TAG_DIM) c.ok = false;
    for (uint64_t i = 0; i < n && c.ok; i++) {
      Dim d;
      name(d.name);
      d.len = c.be(ns);
      nc.dims.push_back(d);
    }
    atts();
    tag = c.be(4);
    n = c.be(ns);
    if (tag != 0 && tag != TAG_VAR) c.ok = false;
    for (uint64_t i = 0; i < n && c.ok; i++) {
      Var v;
      name(v.name);
      const uint64_t nd = c.be(ns);
      for (uint64_t q = 0; q < nd && c.ok; q++) v.dimids.push_back((int)c.be(ns));
      atts();
      v.type = (int)c.be(4);
      v.vsize = c.be(ns);
      v.begin = c.be(os);
      nc.vars.push_back(v);
    }
    if (c.ok) break;
    if (got < want) return io_fail(LGPU_ERR_ARG, std::string(path) + ": malformed netCDF header");
    want *= 4;
    if (want > ((size_t)1 << 30)) return io_fail(LGPU_ERR_ARG, std::string(path) + ": netCDF header too large");
  }
  for (size_t i = 0; i < nc.dims.size(); i++)
    if (nc.dims[i].len == 0) nc.recdim = (int)i;
  int nrecvars = 0;
  for (auto &v : nc.vars) {
    for (int d : v.dimids)
      if (d < 0 || d >= (int)nc.dims.size()) return io_fail(LGPU_ERR_ARG, nc.path + ": bad dimension id");
    if (type_size(v.type) == 0) return io_fail(LGPU_ERR_ARG, nc.path + ": unknown type of variable " + v.name);
    v.record = !v.dimids.empty() && v.dimids[0] == nc.recdim;
    nrecvars += v.record;
  }
  nc.recsize = 0;
  for (auto &v : nc.vars)
    if (v.record) {
      uint64_t slab = type_size(v.type);
      for (size_t q = 1; q < v.dimids.size(); q++) slab *= nc.dims[v.dimids[q]].len;
      nc.recsize += nrecvars == 1 ? slab : pad4(slab);
    }
  return LGPU_OK;
}

const Var *find_var(const NcFile &nc, const char *name) {
  for (auto &v : nc.vars)
    if (v.name == name) return &v;
  return nullptr;
}

// shape in file order (slowest first); the record dimension counts numrecs
std::vector<uint64_t> var_shape(const NcFile &nc, const Var &v) {
  std::vector<uint64_t> s;
  for (size_t q = 0; q < v.dimids.size(); q++)
    s.push_back(v.record && q == 0 ? nc.numrecs : nc.dims[v.dimids[q]].len);
  return s;
}

double decode(const unsigned char *p, int t) {
  uint64_t u = 0;
  const int n = type_size(t);
  for (int i = 0; i < n; i++) u = (u << 8) | p[i];
  switch (t) {
  case NC_BYTE: return (double)(int8_t)u;
  case NC_CHAR: case NC_UBYTE: return (double)(uint8_t)u;
  case NC_SHORT: return (double)(int16_t)u;
  case NC_USHORT: return (double)(uint16_t)u;
  case NC_INT: return (double)(int32_t)u;
  case NC_UINT: return (double)(uint32_t)u;
  case NC_INT64: return (double)(int64_t)u;
  case NC_UINT64: return (double)u;
  case NC_FLOAT: { uint32_t w = (uint32_t)u; float x; std::memcpy(&x, &w, 4); return x; }
  case NC_DOUBLE: { double x; std::memcpy(&x, &u, 8); return x; }
  default: return 0.0;
  }
}

// every value of variable `name` in file order, converted by `put`
template <class Put>
int read_values(const char *path, const char *name, uint64_t n, Put put) {
  NcFile nc;
  int rc = nc_open(nc, path);
  if (rc != LGPU_OK) return rc;
  const Var *v = name ? find_var(nc, name) : nullptr;
  if (!v) return io_fail(LGPU_ERR_ARG, std::string("variable \"") + (name ? name : "") + "\" not in " + nc.path);
  const std::vector<uint64_t> shape = var_shape(nc, *v);
  uint64_t total = 1;
  for (uint64_t s : shape) total *= s;
  if (total != n)
    return io_fail(LGPU_ERR_ARG, nc.path + ": variable \"" + name + "\" holds " + std::to_string(total) +
                                     " values, " + std::to_string(n) + " expected");
  const int ts = type_size(v->type);
  uint64_t per_rec = 1;   // values in one record's slab (or the whole fixed variable)
  for (size_t q = v->record ? 1 : 0; q < shape.size(); q++) per_rec *= shape[q];
  const uint64_t nrec = v->record ? nc.numrecs : 1;
  std::vector<unsigned char> buf(per_rec * ts);
  uint64_t k = 0;
  for (uint64_t r = 0; r < nrec; r++) {
    const uint64_t off = v->begin + (v->record ? r * nc.recsize : 0);
    if (fseek(nc.f, (long)off, SEEK_SET) != 0 || fread(buf.data(), 1, buf.size(), nc.f) != buf.size())
      return io_fail(LGPU_ERR_ARG, nc.path + ": truncated data of \"" + name + "\"");
    for (uint64_t i = 0; i < per_rec; i++) put(k++, decode(&buf[i * ts], v->type));
  }
  return LGPU_OK;
}

// ------------------------------------------------------------------ writer
struct WAtt { std::string name; std::string text; };
struct WVar {
  std::string name;
  std::vector<int> dimids;
  std::vector<WAtt> atts;
  const float *data = nullptr;   // NC_FLOAT values in file order (null: fill value)
  uint64_t n = 0;                // values (per record for record variables)
  bool record = false;
};

struct Writer {
  std::vector<Dim> dims;   // len 0 = the record dimension
  std::vector<WVar> vars;
  uint64_t numrecs = 0;

  int dim(const std::string &name, uint64_t len) {
    dims.push_back({name, len});
    return (int)dims.size() - 1;
  }
  WVar &var(const std::string &name, std::vector<int> dimids, const float *data) {
    WVar v;
    v.name = name;
    v.dimids = dimids;
    v.data = data;
    v.n = 1;
    for (size_t q = 0; q < dimids.size(); q++) {
      if (dims[dimids[q]].len == 0) v.record = true;
      else v.n *= dims[dimids[q]].len;
    }
    vars.push_back(v);
    return vars.back();
  }

  int write(const char *path) {
    if (!path) return io_fail(LGPU_ERR_ARG, "null path");
    // sizes: version 1 unless an offset passes 2^31 - 1
    int nrec = 0;
    for (auto &v : vars) nrec += v.record;
    uint64_t fixed = 0, recsize = 0;
    for (auto &v : vars) {
      if (v.record) recsize += nrec == 1 ? 4 * v.n : pad4(4 * v.n);
      else fixed += pad4(4 * v.n);
    }
    int version = 1;
    std::vector<unsigned char> h;
    uint64_t hdr_len = 0;
    for (int pass = 0; pass < 2; pass++) {
      h = header(version, hdr_len);
      hdr_len = h.size();
      if (version == 1 && hdr_len + fixed + recsize * numrecs > 0x7fffffffULL) {
        version = 2;
        pass = -1;
        hdr_len = 0;
        continue;
      }
    }
    FILE *f = fopen(path, "wb");
    if (!f) return io_fail(LGPU_ERR_ARG, std::string("cannot create ") + path + ": " + strerror(errno));
    bool ok = fwrite(h.data(), 1, h.size(), f) == h.size();
    std::vector<unsigned char> buf;
    auto put_vals = [&](const WVar &v, uint64_t first, bool pad) {
      buf.assign(pad ? pad4(4 * v.n) : 4 * v.n, 0);
      for (uint64_t i = 0; i < v.n; i++) {
        uint32_t w;
        if (v.data) std::memcpy(&w, &v.data[first + i], 4);
        else { const float fill = 9.9692099683868690e+36f; std::memcpy(&w, &fill, 4); }
        buf[4 * i] = w >> 24; buf[4 * i + 1] = (w >> 16) & 0xff; buf[4 * i + 2] = (w >> 8) & 0xff;
        buf[4 * i + 3] = w & 0xff;
      }
      ok = ok && fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    };
    for (auto &v : vars)
      if (!v.record) put_vals(v, 0, true);
    for (uint64_t r = 0; r < numrecs; r++)
      for (auto &v : vars)
        if (v.record) put_vals(v, r * v.n, nrec > 1);
    ok = (fclose(f) == 0) && ok;
    if (!ok) return io_fail(LGPU_ERR_ARG, std::string("write failed: ") + path);
    return LGPU_OK;
  }

 private:
  static void be(std::vector<unsigned char> &h, uint64_t v, int n) {
    for (int i = n - 1; i >= 0; i--) h.push_back((unsigned char)(v >> (8 * i)));
  }
  static void name(std::vector<unsigned char> &h, const std::string &s) {
    be(h, s.size(), 4);
    h.insert(h.end(), s.begin(), s.end());
    while (h.size() % 4) h.push_back(0);
  }
  std::vector<unsigned char> header(int version, uint64_t hdr_len) const {
    const int os = version == 1 ? 4 : 8;
    std::vector<unsigned char> h = {'C', 'D', 'F', (unsigned char)version};
    be(h, numrecs, 4);
    if (dims.empty()) { be(h, 0, 4); be(h, 0, 4); }
    else {
      be(h, TAG_DIM, 4);
      be(h, dims.size(), 4);
      for (auto &d : dims) { name(h, d.name); be(h, d.len, 4); }
    }
    be(h, 0, 4); be(h, 0, 4);   // no global attributes
    if (vars.empty()) { be(h, 0, 4); be(h, 0, 4); return h; }
    be(h, TAG_VAR, 4);
    be(h, vars.size(), 4);
    int nrec = 0;
    for (auto &v : vars) nrec += v.record;
    uint64_t off_fixed = hdr_len, off_rec = 0;
    for (auto &v : vars) if (!v.record) off_rec += pad4(4 * v.n);
    off_rec += hdr_len;
    for (auto &v : vars) {
      name(h, v.name);
      be(h, v.dimids.size(), 4);
      for (int d : v.dimids) be(h, d, 4);
      if (v.atts.empty()) { be(h, 0, 4); be(h, 0, 4); }
      else {
        be(h, TAG_ATT, 4);
        be(h, v.atts.size(), 4);
        for (auto &a : v.atts) {
          name(h, a.name);
          be(h, NC_CHAR, 4);
          be(h, a.text.size(), 4);
          h.insert(h.end(), a.text.begin(), a.text.end());
          while (h.size() % 4) h.push_back(0);
        }
      }
      be(h, NC_FLOAT, 4);
      const uint64_t vsize = pad4(4 * v.n);
      be(h, vsize > 0xffffffffULL ? 0xffffffffULL : vsize, 4);
      if (v.record) {
        be(h, off_rec, os);
        off_rec += nrec == 1 ? 4 * v.n : pad4(4 * v.n);
      } else {
        be(h, off_fixed, os);
        off_fixed += pad4(4 * v.n);
      }
    }
    return h;
  }
};

bool grid_ok(int nx, int ny, const float *lat_nom, const float *lon_nom) {
  return nx > 0 && ny > 0 && lat_nom && lon_nom;
}

}  // namespace

extern "C" {

const char *lgpu_io_last_error(void) { return g_io_err.c_str(); }

// parse_ens_filename (src/letkf_state_helper.F90:445-510)
int lgpu_ens_filename(const char *pattern, int ensmem, char *out, int cap) {
  if (!pattern || !out || cap <= 0) return io_fail(LGPU_ERR_ARG, "ens_filename: bad arguments");
  std::string s = pattern;
  for (int n = 1; n <= 9; n++) {
    const std::string key = "#ENS" + std::to_string(n) + "#";
    const size_t i = s.find(key);
    if (i == std::string::npos) continue;
    std::string val;
    if (ensmem >= 0) {
      char b[32];
      snprintf(b, sizeof b, "%0*d", n, ensmem);
      val = b;
    } else if (ensmem == -1 || ensmem == -2) val = "mean";      // ENS_BKG_MEAN, ENS_ANA_MEAN
    else if (ensmem == -3 || ensmem == -4) val = "sprd";        // ENS_BKG_SPRD, ENS_ANA_SPRD
    else return io_fail(LGPU_ERR_ARG, "Illegal 'ensmem' given to str_ens_pattern");
    for (size_t p = s.find(key); p != std::string::npos; p = s.find(key)) s.replace(p, key.size(), val);
    break;
  }
  std::string type;
  if (ensmem >= 0 || ensmem == -2 || ensmem == -4) type = "ana";
  else if (ensmem == -1 || ensmem == -3) type = "bkg";
  else return io_fail(LGPU_ERR_ARG, "illegal ensmem given to write_state");
  for (size_t p = s.find("#TYPE#"); p != std::string::npos; p = s.find("#TYPE#")) s.replace(p, 6, type);
  if ((int)s.size() + 1 > cap) return io_fail(LGPU_ERR_CAPACITY, "ens_filename: output buffer too small");
  std::memcpy(out, s.c_str(), s.size() + 1);
  return LGPU_OK;
}

int lgpu_nc_dim_len(const char *path, const char *dim, long long *len) {
  if (!dim || !len) return io_fail(LGPU_ERR_ARG, "nc_dim_len: bad arguments");
  NcFile nc;
  int rc = nc_open(nc, path);
  if (rc != LGPU_OK) return rc;
  for (size_t i = 0; i < nc.dims.size(); i++)
    if (nc.dims[i].name == dim) {
      *len = (long long)((int)i == nc.recdim ? nc.numrecs : nc.dims[i].len);
      return LGPU_OK;
    }
  return io_fail(LGPU_ERR_ARG, std::string("dimension \"") + dim + "\" not in " + nc.path);
}

int lgpu_nc_var_info(const char *path, const char *var, int *ndims, long long *dims, int maxdims) {
  if (!var || !ndims) return io_fail(LGPU_ERR_ARG, "nc_var_info: bad arguments");
  NcFile nc;
  int rc = nc_open(nc, path);
  if (rc != LGPU_OK) return rc;
  const Var *v = find_var(nc, var);
  if (!v) return io_fail(LGPU_ERR_ARG, std::string("variable \"") + var + "\" not in " + nc.path);
  const std::vector<uint64_t> s = var_shape(nc, *v);
  *ndims = (int)s.size();
  for (int i = 0; i < (int)s.size() && i < maxdims && dims; i++) dims[i] = (long long)s[i];
  return LGPU_OK;
}

int lgpu_nc_read_float(const char *path, const char *var, float *out, long long n) {
  if (!out || n < 0) return io_fail(LGPU_ERR_ARG, "nc_read_float: bad arguments");
  return read_values(path, var, (uint64_t)n, [&](uint64_t i, double x) { out[i] = (float)x; });
}

int lgpu_nc_read_int(const char *path, const char *var, int *out, long long n) {
  if (!out || n < 0) return io_fail(LGPU_ERR_ARG, "nc_read_int: bad arguments");
  // values beyond the int range saturate
  return read_values(path, var, (uint64_t)n, [&](uint64_t i, double x) {
    out[i] = x >= 2147483647.0 ? 2147483647 : (x <= -2147483648.0 ? (-2147483647 - 1) : (int)x);
  });
}

// obsio_nc_read_obs (src/subclass.letkf_obsio/letkf_obsio_nc.F90:150-237):
// dimension "obs", variables obid, plat, lat, lon, depth, hr, val, err, qc.
// With lat == NULL only *nobs is set.
int lgpu_read_obs_nc(const char *path, int cap, int *nobs, float *lat, float *lon, float *zdim, float *time,
                     float *val, float *err, int *obsid, int *platid, int *qc) {
  if (!nobs) return io_fail(LGPU_ERR_ARG, "read_obs_nc: bad arguments");
  long long n = 0;
  int rc = lgpu_nc_dim_len(path, "obs", &n);
  if (rc != LGPU_OK) return io_fail(rc, std::string("Reading dimension \"obs\": ") + g_io_err);
  *nobs = (int)n;
  if (!lat) return LGPU_OK;
  if (!lon || !zdim || !time || !val || !err || !obsid || !platid || !qc)
    return io_fail(LGPU_ERR_ARG, "read_obs_nc: bad arguments");
  if (n > cap) return io_fail(LGPU_ERR_CAPACITY, "read_obs_nc: " + std::to_string(n) + " observations, room for " +
                                                    std::to_string(cap));
  struct { const char *name; int *i; float *f; } items[] = {
      {"obid", obsid, nullptr}, {"plat", platid, nullptr}, {"lat", nullptr, lat}, {"lon", nullptr, lon},
      {"depth", nullptr, zdim}, {"hr", nullptr, time}, {"val", nullptr, val}, {"err", nullptr, err},
      {"qc", qc, nullptr}};
  for (auto &it : items) {
    rc = it.i ? lgpu_nc_read_int(path, it.name, it.i, n) : lgpu_nc_read_float(path, it.name, it.f, n);
    if (rc != LGPU_OK) return io_fail(rc, std::string("\"") + it.name + "\" in " + path + ": " + g_io_err);
  }
  return LGPU_OK;
}

// obsio_nc_read_hx (letkf_obsio_nc.F90:244-306): one member's H(x) from "hx",
// or val + inc with read_inc
int lgpu_read_hx_nc(const char *path, int nobs, int read_inc, float *hx) {
  if (!hx || nobs < 0) return io_fail(LGPU_ERR_ARG, "read_hx_nc: bad arguments");
  long long n = 0;
  int rc = lgpu_nc_dim_len(path, "obs", &n);
  if (rc != LGPU_OK) return rc;
  if (n != nobs) return io_fail(LGPU_ERR_ARG, "error in obsio_nc_read_hx(), obs in file does not match expected.");
  if (!read_inc) return lgpu_nc_read_float(path, "hx", hx, n);
  std::vector<float> v((size_t)n);
  if ((rc = lgpu_nc_read_float(path, "val", v.data(), n)) != LGPU_OK) return rc;
  if ((rc = lgpu_nc_read_float(path, "inc", hx, n)) != LGPU_OK) return rc;
  for (long long i = 0; i < n; i++) hx[i] = hx[i] + v[(size_t)i];
  return LGPU_OK;
}

// stateio_nc_read_state (letkf_stateio_nc.F90:196-245): variable `var` of
// shape (nx, ny, nz) in Fortran order, i.e. [nz][ny][nx] in file order after
// any leading record dimension of length 1; out receives nx * ny * nz floats
int lgpu_read_state_nc(const char *path, const char *var, int nx, int ny, int nz, float *out) {
  if (!var || !out || nx <= 0 || ny <= 0 || nz <= 0) return io_fail(LGPU_ERR_ARG, "read_state_nc: bad arguments");
  int nd = 0;
  long long d[8] = {0};
  int rc = lgpu_nc_var_info(path, var, &nd, d, 8);
  if (rc != LGPU_OK) return rc;
  long long total = 1;
  for (int i = 0; i < nd; i++) total *= d[i];
  if (total != (long long)nx * ny * nz)
    return io_fail(LGPU_ERR_ARG, std::string(path) + " " + var + ": " + std::to_string(total) + " values, grid holds " +
                                     std::to_string((long long)nx * ny * nz));
  return lgpu_nc_read_float(path, var, out, total);
}

// stateio_nc_write_state (letkf_stateio_nc.F90:252-370) in a classic file:
// dimensions time (record), lon, lat and the vertical grid; coordinate
// variables with their attributes; each state variable [time][vt][lat][lon],
// one record.  vals[v] holds nz_v * ny * nx floats of variable v (2-D
// variables: nz_v = 1 on a vertical grid of its own, given by vtgrid index).
int lgpu_write_state_nc(const char *path, int nx, int ny, const float *lon_nom, const float *lat_nom, int nvt,
                        const char *const *vt_names, const int *vt_len, const float *const *vt_nom, int nvar,
                        const char *const *names, const int *var_vt, const float *const *vals) {
  if (!grid_ok(nx, ny, lat_nom, lon_nom) || nvt < 0 || nvar < 0 || (nvt && (!vt_names || !vt_len || !vt_nom)) ||
      (nvar && (!names || !var_vt || !vals)))
    return io_fail(LGPU_ERR_ARG, "write_state_nc: bad arguments");
  Writer w;
  const int dt = w.dim("time", 0);
  w.var("time", {dt}, nullptr).atts = {{"axis", "T"}};
  const int dx = w.dim("lon", nx);
  w.var("lon", {dx}, lon_nom).atts = {{"long_name", "longitude"}, {"units", "degrees_east"}, {"axis", "X"}};
  const int dy = w.dim("lat", ny);
  w.var("lat", {dy}, lat_nom).atts = {{"long_name", "latitude"}, {"units", "degrees_north"}, {"axis", "Y"}};
  std::vector<int> dz(nvt);
  for (int i = 0; i < nvt; i++) {
    if (!vt_names[i] || vt_len[i] <= 0 || !vt_nom[i]) return io_fail(LGPU_ERR_ARG, "write_state_nc: bad vertical grid");
    dz[i] = w.dim(vt_names[i], vt_len[i]);
    w.var(vt_names[i], {dz[i]}, vt_nom[i]).atts = {{"axis", "Z"}};
  }
  for (int v = 0; v < nvar; v++) {
    if (!names[v] || !vals[v] || var_vt[v] < 0 || var_vt[v] >= nvt)
      return io_fail(LGPU_ERR_ARG, "cannot find vertical grid in stateio_nc_write_init");
    w.var(names[v], {dt, dz[var_vt[v]], dy, dx}, vals[v]);
  }
  w.numrecs = 1;
  return w.write(path);
}

// letkf_solver_final's diag.solver.nc (src/letkf_solver.F90:397-527)
int lgpu_write_diag_nc(const char *path, int nx, int ny, int groups, const float *lat_nom, const float *lon_nom,
                       const float *maxhz, const float *obscount, const float *lg_obscount, const float *lg_obsloc) {
  if (!grid_ok(nx, ny, lat_nom, lon_nom) || groups <= 0 || !maxhz || !obscount || !lg_obscount || !lg_obsloc)
    return io_fail(LGPU_ERR_ARG, "write_diag_nc: bad arguments");
  Writer w;
  const int dt = w.dim("time", 1), dy = w.dim("lat", ny), dx = w.dim("lon", nx), dg = w.dim("loc_group", groups);
  w.var("lat", {dy}, lat_nom).atts = {{"axis", "Y"}, {"units", "degrees_north"}};
  w.var("lon", {dx}, lon_nom).atts = {{"axis", "X"}, {"units", "degrees_east"}};
  w.var("col_maxhz", {dt, dy, dx}, maxhz).atts = {{"long_name", "max observation search radius for the column"},
                                                  {"units", "m"}};
  w.var("col_obscount", {dt, dy, dx}, obscount).atts = {{"long_name", "observations per horizontal gridpoint"}};
  w.var("lg_obscount", {dt, dg, dy, dx}, lg_obscount).atts = {{"long_name", "observations per localization group"}};
  w.var("lg_obsloc", {dt, dg, dy, dx}, lg_obsloc).atts = {
      {"long_name", "sum of localization values for observations used"}};
  return w.write(path);
}

// loc_ocean_final's diag.loc_ocean.nc (letkf_loc_ocean.F90:249-322)
int lgpu_write_loc_diag_nc(const char *path, int nx, int ny, const float *lat_nom, const float *lon_nom,
                           const float *surf_lvl, const float *surf_depth) {
  if (!grid_ok(nx, ny, lat_nom, lon_nom) || !surf_lvl || !surf_depth)
    return io_fail(LGPU_ERR_ARG, "write_loc_diag_nc: bad arguments");
  Writer w;
  const int dt = w.dim("time", 1), dy = w.dim("lat", ny), dx = w.dim("lon", nx);
  w.var("lat", {dy}, lat_nom).atts = {{"axis", "Y"}, {"units", "degrees_north"}};
  w.var("lon", {dx}, lon_nom).atts = {{"axis", "X"}, {"units", "degrees_east"}};
  w.var("vtloc_surf_lvl", {dt, dy, dx}, surf_lvl).atts = {
      {"long_name", "depth, in levels, of the surface localization group"}};
  w.var("vtloc_surf_depth", {dt, dy, dx}, surf_depth).atts = {
      {"long_name", "depth, in meters, of the surface localization group"}, {"units", "meters"}};
  return w.write(path);
}

}  // extern "C"
