// Field output and input in the netCDF classic format, 64-bit offset
// variant (CDF-2): the single-rank path of pnet_out_chunk
// (common/mpi_parallel.f90:7481-8176) in every mode it documents, and the
// read back of one frame for restarts.
//
// pnet_out_chunk(var_name, file_name, imode, ia1, ia2, ia3, ifrmd, imem, var,
// np, mp, lp, ih): at ifrmd == 0 it creates the file (NF_64BIT_OFFSET) if it
// does not exist, defines the dimensions the mode uses and the unlimited t if
// absent, and defines var_name if absent (:7596-7715); then it writes the
// mode's part of var as frame ifrmd+1 (:7746-8170; make_plan below lists the
// modes).  Fortran dimension order (x,y,z,t) is netCDF's (t,z,y,x), so x
// varies fastest in the file, as in the caller's array.
//
// The file format follows the published netCDF classic format
// specification: a big-endian header (magic "CDF\2", record count,
// dimension, global attribute and variable lists), then the fixed-size
// variables, then the records, each holding one slab of every record
// variable.  Adding a variable to a file rewrites it (as netCDF's redef
// does); writing a frame of an existing variable writes in place and extends
// the record count, filling the frames in between with the default fill
// value of the type.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mpdata.h"
#include "mpdata_common.cuh"
#include "mpdata_stages.cuh"

namespace {

enum : unsigned { NC_DIMENSION = 10, NC_VARIABLE = 11, NC_ATTRIBUTE = 12 };
enum : unsigned { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };
constexpr double kFill = 9.9692099683868690e+36;  // NC_FILL_DOUBLE; NC_FILL_FLOAT is its float

size_t type_size(unsigned t) {
  switch (t) {
    case NC_BYTE: case NC_CHAR: return 1;
    case NC_SHORT: return 2;
    case NC_INT: case NC_FLOAT: return 4;
    case NC_DOUBLE: return 8;
    default: return 0;
  }
}
size_t pad4(size_t n) { return (n + 3) & ~size_t(3); }

struct Dim {
  std::string name;
  unsigned long long len;  // 0 = the record dimension
};
struct Att {
  std::string name;
  unsigned type;
  unsigned n;
  std::vector<unsigned char> raw;  // big-endian values, unpadded
};
struct Var {
  std::string name;
  std::vector<unsigned> dims;
  std::vector<Att> atts;
  unsigned type;
  unsigned long long vsize;  // bytes of one record slab (or of the whole variable), padded
  unsigned long long begin;
};
struct Model {
  int version = 2;
  unsigned long long numrecs = 0;
  std::vector<Dim> dims;
  std::vector<Att> gatts;
  std::vector<Var> vars;
};

// ---- big-endian encoding -------------------------------------------------
struct Out {
  std::vector<unsigned char> b;
  void u32(unsigned long long v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
  }
  void u64(unsigned long long v) {
    for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
  }
  void name(const std::string& s) {
    u32(s.size());
    b.insert(b.end(), s.begin(), s.end());
    while (b.size() % 4) b.push_back(0);
  }
  void atts(const std::vector<Att>& a) {
    if (a.empty()) {
      u32(0);
      u32(0);
      return;
    }
    u32(NC_ATTRIBUTE);
    u32(a.size());
    for (const Att& t : a) {
      name(t.name);
      u32(t.type);
      u32(t.n);
      b.insert(b.end(), t.raw.begin(), t.raw.end());
      while (b.size() % 4) b.push_back(0);
    }
  }
};

struct In {
  const unsigned char* p;
  size_t n, i = 0;
  bool ok = true;
  unsigned long long u32() {
    if (i + 4 > n) { ok = false; return 0; }
    unsigned long long v = ((unsigned long long)p[i] << 24) | ((unsigned long long)p[i + 1] << 16) |
                           ((unsigned long long)p[i + 2] << 8) | p[i + 3];
    i += 4;
    return v;
  }
  unsigned long long u64() {
    const unsigned long long hi = u32();
    return (hi << 32) | u32();
  }
  std::string name() {
    const size_t len = (size_t)u32();
    if (!ok || i + len > n) { ok = false; return std::string(); }
    std::string s((const char*)p + i, len);
    i = pad4(i + len);
    return s;
  }
  std::vector<Att> atts() {
    std::vector<Att> a;
    const unsigned tag = (unsigned)u32();
    const unsigned cnt = (unsigned)u32();
    if (tag == 0 && cnt == 0) return a;
    if (tag != NC_ATTRIBUTE) { ok = false; return a; }
    for (unsigned k = 0; k < cnt && ok; k++) {
      Att t;
      t.name = name();
      t.type = (unsigned)u32();
      t.n = (unsigned)u32();
      const size_t bytes = type_size(t.type) * t.n;
      if (!type_size(t.type) || i + bytes > n) { ok = false; break; }
      t.raw.assign(p + i, p + i + bytes);
      i = pad4(i + bytes);
      a.push_back(t);
    }
    return a;
  }
};

bool is_rec(const Model& m, const Var& v) { return !v.dims.empty() && m.dims[v.dims[0]].len == 0; }

unsigned long long slab_bytes(const Model& m, const Var& v) {
  unsigned long long n = type_size(v.type);
  for (size_t d = 0; d < v.dims.size(); d++)
    if (!(d == 0 && m.dims[v.dims[d]].len == 0)) n *= m.dims[v.dims[d]].len;
  return pad4(n);
}

// bytes of one record; with exactly one record variable its slab is not padded
unsigned long long rec_bytes(const Model& m) {
  unsigned long long r = 0;
  int nrec = 0;
  const Var* only = nullptr;
  for (const Var& v : m.vars)
    if (is_rec(m, v)) { r += v.vsize; nrec++; only = &v; }
  if (nrec == 1) {
    unsigned long long n = type_size(only->type);
    for (size_t d = 1; d < only->dims.size(); d++) n *= m.dims[only->dims[d]].len;
    return n;
  }
  return r;
}

std::vector<unsigned char> encode(const Model& m) {
  Out o;
  o.b = {'C', 'D', 'F', (unsigned char)m.version};
  o.u32(m.numrecs);
  if (m.dims.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(NC_DIMENSION);
    o.u32(m.dims.size());
    for (const Dim& d : m.dims) {
      o.name(d.name);
      o.u32(d.len);
    }
  }
  o.atts(m.gatts);
  if (m.vars.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(NC_VARIABLE);
    o.u32(m.vars.size());
    for (const Var& v : m.vars) {
      o.name(v.name);
      o.u32(v.dims.size());
      for (unsigned d : v.dims) o.u32(d);
      o.atts(v.atts);
      o.u32(v.type);
      o.u32(v.vsize > 0xfffffffcULL ? 0xffffffffULL : v.vsize);
      if (m.version == 1) o.u32(v.begin); else o.u64(v.begin);
    }
  }
  return o.b;
}

bool decode(const std::vector<unsigned char>& f, Model& m) {
  if (f.size() < 8 || f[0] != 'C' || f[1] != 'D' || f[2] != 'F' || (f[3] != 1 && f[3] != 2)) return false;
  In in{f.data(), f.size()};
  in.i = 4;
  m = Model();
  m.version = f[3];
  m.numrecs = in.u32();
  unsigned tag = (unsigned)in.u32(), cnt = (unsigned)in.u32();
  if (tag == NC_DIMENSION) {
    for (unsigned k = 0; k < cnt && in.ok; k++) {
      Dim d;
      d.name = in.name();
      d.len = in.u32();
      m.dims.push_back(d);
    }
  } else if (tag != 0 || cnt != 0) {
    return false;
  }
  m.gatts = in.atts();
  tag = (unsigned)in.u32();
  cnt = (unsigned)in.u32();
  if (tag == NC_VARIABLE) {
    for (unsigned k = 0; k < cnt && in.ok; k++) {
      Var v;
      v.name = in.name();
      const unsigned nd = (unsigned)in.u32();
      for (unsigned d = 0; d < nd && in.ok; d++) {
        const unsigned id = (unsigned)in.u32();
        if (id >= m.dims.size()) return false;
        v.dims.push_back(id);
      }
      v.atts = in.atts();
      v.type = (unsigned)in.u32();
      in.u32();  // vsize: recomputed from the dimensions
      v.begin = m.version == 1 ? in.u32() : in.u64();
      if (!type_size(v.type)) return false;
      m.vars.push_back(v);
    }
  } else if (tag != 0 || cnt != 0) {
    return false;
  }
  if (!in.ok) return false;
  for (Var& v : m.vars) v.vsize = slab_bytes(m, v);
  return true;
}

// begin offsets for a header of the model's size: fixed variables first, then records
void layout(Model& m) {
  unsigned long long off = encode(m).size();
  for (Var& v : m.vars)
    if (!is_rec(m, v)) { v.begin = off; off += v.vsize; }
  for (Var& v : m.vars)
    if (is_rec(m, v)) { v.begin = off; off += v.vsize; }
}

unsigned long long rec_offset(const Model& m, const Var& v, unsigned long long r) {
  return v.begin + r * rec_bytes(m);
}

std::vector<unsigned char> fill_slab(const Var& v) {
  std::vector<unsigned char> s(v.vsize, 0);
  const size_t ts = type_size(v.type);
  unsigned char be[8];
  if (v.type == NC_DOUBLE) {
    unsigned long long b;
    std::memcpy(&b, &kFill, 8);
    for (int k = 0; k < 8; k++) be[k] = (unsigned char)(b >> (56 - 8 * k));
  } else {
    const float f = (float)kFill;
    unsigned b;
    std::memcpy(&b, &f, 4);
    for (int k = 0; k < 4; k++) be[k] = (unsigned char)(b >> (24 - 8 * k));
  }
  if (v.type == NC_DOUBLE || v.type == NC_FLOAT)
    for (size_t t = 0; t + ts <= s.size(); t += ts) std::memcpy(&s[t], be, ts);
  return s;
}

bool read_file(const std::string& path, std::vector<unsigned char>& out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out.resize(n > 0 ? (size_t)n : 0);
  const bool ok = n >= 0 && std::fread(out.data(), 1, out.size(), f) == out.size();
  std::fclose(f);
  return ok;
}

bool pwrite_at(FILE* f, unsigned long long off, const void* p, size_t n) {
  return fseeko(f, (off_t)off, SEEK_SET) == 0 && std::fwrite(p, 1, n, f) == n;
}

// Rebuild the whole file for a changed model (same record count): the data
// of every variable the old file holds are copied to their new places, new
// variables get fill values.
int rewrite(const std::string& path, const Model& old, const std::vector<unsigned char>& oldbytes, Model& m) {
  layout(m);
  std::vector<unsigned char> out = encode(m);
  unsigned long long end = out.size(), rec0 = 0;
  bool any_rec = false;
  for (const Var& v : m.vars) {
    if (is_rec(m, v)) {
      rec0 = any_rec ? (v.begin < rec0 ? v.begin : rec0) : v.begin;
      any_rec = true;
    } else if (v.begin + v.vsize > end) {
      end = v.begin + v.vsize;
    }
  }
  if (any_rec) end = rec0 + rec_bytes(m) * m.numrecs;
  out.resize(end, 0);
  for (const Var& v : m.vars) {
    const Var* o = nullptr;
    for (const Var& w : old.vars)
      if (w.name == v.name) o = &w;
    const bool rec = is_rec(m, v);
    const unsigned long long nslab = rec ? m.numrecs : 1;
    const std::vector<unsigned char> fill = fill_slab(v);
    const size_t len = (size_t)(rec ? (rec_bytes(m) < v.vsize ? rec_bytes(m) : v.vsize) : v.vsize);
    for (unsigned long long r = 0; r < nslab; r++) {
      const unsigned long long dst = rec ? rec_offset(m, v, r) : v.begin;
      if (o && (!rec || r < old.numrecs)) {
        const unsigned long long src = rec ? rec_offset(old, *o, r) : o->begin;
        if (src + len > oldbytes.size()) return MPDATA_E_IO;
        std::memcpy(&out[dst], &oldbytes[src], len);
      } else {
        std::memcpy(&out[dst], fill.data(), len);
      }
    }
  }
  const std::string tmp = path + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return MPDATA_E_IO;
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  if (std::fclose(f) != 0 || !ok) return MPDATA_E_IO;
  return std::rename(tmp.c_str(), path.c_str()) == 0 ? MPDATA_OK : MPDATA_E_IO;
}

int find_dim(const Model& m, const char* name) {
  for (size_t d = 0; d < m.dims.size(); d++)
    if (m.dims[d].name == name) return (int)d;
  return -1;
}
int find_var(const Model& m, const char* name) {
  for (size_t v = 0; v < m.vars.size(); v++)
    if (m.vars[v].name == name) return (int)v;
  return -1;
}

// ---- what one call defines and writes --------------------------------------
// pnet_out_chunk on a single rank: every edge flag is set, the rank sits at
// position 1 along each axis and at no sub-domain offset.  Per imode
// (:7548-7573 lengths, :7606-7640 dimensions, :7671-7712 the variable,
// :7746-7846 starts and counts, :7847-8170 the data):
//  0, 1   the interior, float / double (x,y,z,t)
//  2-4    the staggered block var(1:np+ia1, 1:mp+ia2, 1:lp+ia3), double, with
//         dimensions of those lengths (var declared with the ia*imem extents)
//  6-8    the right, top and sky halo strips var(np+1:np+ih, ...) at offset
//         ih of a 2*ih-long dimension (on one rank the left, bottom and
//         ground strips are overwritten before the single write)
//  9      var(np-ih+1:np, mp-ih+1:mp, lp-ih+1:lp) at offset ih of 2*ih-long
//         dimensions (the corner indices the reference forms on one rank)
//  10, 13 the xy plane at k = ia3 (written when (ia3-1)/lp == 0) or k = 1,
//         double (x,y,t), no z dimension defined
//  11, 12 the xz plane at j = ia2, the yz plane at i = ia1, through single
//         precision into a double (x,z,t) / (y,z,t) variable
//  20-22  the z line at (ia1,ia2), the y line at (ia1,ia3), the x line at
//         (ia2,ia3), float (z,t) / (y,t) / (x,t)
//  30     a float (t) variable, defined and never written
//  34     the interior, float (x,y,z), no time
//  35     the plane k = 1-ih (the ground halo), double (x,y), no time
// Planes and lines are written only when (ia-1)/n == 0 for each fixed index
// (the rank-position tests); otherwise nothing is written.  Modes 3 and 4
// fill their temporaries over a block smaller than the one they write for
// some offset combinations (unset or out-of-range elements in the
// reference); here the block the counts describe is written from var.
struct Plan {
  bool def[3];                // define x, y, z when absent
  unsigned long long len[3];  // with these lengths
  unsigned type;              // the variable's type when it is defined
  unsigned axes;              // its spatial dimensions: bit 0 x, 1 y, 2 z
  bool rec;                   // it has the record dimension t
  bool sp;                    // the values pass through single precision
  bool write;                 // anything is written
  int b0[3], cnt[3];          // the box of var: first index (1-based), count
  int st[3];                  // its start in the variable (0-based)
};

bool make_plan(int imode, int ia1, int ia2, int ia3, int np, int mp, int lp, int ih, Plan& p) {
  p = Plan{};
  for (int a = 0; a < 3; a++) {
    p.def[a] = true;
    p.b0[a] = 1;
  }
  p.len[0] = np;
  p.len[1] = mp;
  p.len[2] = lp;
  p.cnt[0] = np;
  p.cnt[1] = mp;
  p.cnt[2] = lp;
  p.axes = 7u;
  p.rec = true;
  p.write = true;
  p.type = NC_DOUBLE;
  // the rank-position tests of the planes and lines (:7847-7854)
  const bool in1 = (ia1 - 1) / np == 0, in2 = (ia2 - 1) / mp == 0, in3 = (ia3 - 1) / lp == 0;
  switch (imode) {
    case 0:
      p.type = NC_FLOAT;
      p.sp = true;
      break;
    case 1:
      break;
    case 2: case 3: case 4:
      p.len[0] = (unsigned long long)(np + ia1);
      p.len[1] = (unsigned long long)(mp + ia2);
      p.len[2] = (unsigned long long)(lp + ia3);
      p.cnt[0] = np + ia1;
      p.cnt[1] = mp + ia2;
      p.cnt[2] = lp + ia3;
      break;
    case 6: case 7: case 8: {
      const int a = imode - 6;
      p.len[a] = 2ULL * ih;
      p.b0[a] = (a == 0 ? np : a == 1 ? mp : lp) + 1;
      p.cnt[a] = ih;
      p.st[a] = ih;
      break;
    }
    case 9: {
      const int n[3] = {np, mp, lp};
      for (int a = 0; a < 3; a++) {
        p.len[a] = 2ULL * ih;
        p.b0[a] = n[a] - ih + 1;
        p.cnt[a] = ih;
        p.st[a] = ih;
      }
      break;
    }
    case 10: case 13:
      p.def[2] = false;
      p.axes = 3u;
      p.b0[2] = imode == 10 ? ia3 : 1;
      p.cnt[2] = 1;
      p.write = imode == 13 || in3;
      break;
    case 11:
      p.def[1] = false;
      p.axes = 5u;
      p.sp = true;
      p.b0[1] = ia2;
      p.cnt[1] = 1;
      p.write = in2;
      break;
    case 12:
      p.def[0] = false;
      p.axes = 6u;
      p.sp = true;
      p.b0[0] = ia1;
      p.cnt[0] = 1;
      p.write = in1;
      break;
    case 20: case 21: case 22: {
      const int keep = imode == 20 ? 2 : imode == 21 ? 1 : 0;  // the line's axis
      const int fix[3] = {ia1, ia2, ia3};
      const bool in[3] = {in1, in2, in3};
      p.type = NC_FLOAT;
      p.sp = true;
      p.axes = 1u << keep;
      p.write = true;
      for (int a = 0; a < 3; a++)
        if (a != keep) {
          p.def[a] = false;
          p.b0[a] = fix[a];
          p.cnt[a] = 1;
          p.write = p.write && in[a];
        }
      break;
    }
    case 30:
      for (int a = 0; a < 3; a++) p.def[a] = false;
      p.axes = 0u;
      p.type = NC_FLOAT;
      p.write = false;
      break;
    case 34:
      p.type = NC_FLOAT;
      p.sp = true;
      p.rec = false;
      break;
    case 35:
      p.rec = false;
      p.axes = 3u;
      p.b0[2] = 1 - ih;
      p.cnt[2] = 1;
      break;
    default:
      return false;
  }
  return true;
}

// ---- box gather to big-endian bytes ----------------------------------------
// Element e of the box (x fastest) of a caller array whose allocation starts
// at base (index 1-ih on each axis, row strides sx, sx*sy), as the value of
// buffer type B converted to the file type T.
struct Box {
  long o0;  // offset of the box's first element from base
  int cx, cy, cz;
  long sy, sz;  // element strides of y and z
};
template <class R, class B, class T>
__device__ __host__ inline void put_be(const R* base, const Box& b, long e, unsigned char* out) {
  const int i = (int)(e % b.cx);
  const long r = e / b.cx;
  const int j = (int)(r % b.cy), k = (int)(r / b.cy);
  const T v = (T)(B)base[b.o0 + i + j * b.sy + k * b.sz];
  unsigned long long bits = 0;
#if defined(__CUDA_ARCH__)
  bits = sizeof(T) == 8 ? (unsigned long long)__double_as_longlong((double)v) : (unsigned long long)__float_as_uint((float)v);
#else
  std::memcpy(&bits, &v, sizeof(T));
#endif
  unsigned char* o = out + e * (long)sizeof(T);
  for (int q = 0; q < (int)sizeof(T); q++) o[q] = (unsigned char)(bits >> (8 * ((int)sizeof(T) - 1 - q)));
}
template <class R, class B, class T>
__global__ void k_pack_be(const R* base, Box b, unsigned char* out) {
  const long n = (long)b.cx * b.cy * b.cz;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    put_be<R, B, T>(base, b, e, out);
}

template <class R, class B, class T>
int gather(const R* var, const Box& b, int on_device, void* stream, std::vector<unsigned char>& out) {
  const long n = (long)b.cx * b.cy * b.cz;
  out.resize((size_t)n * sizeof(T));
  if (!on_device) {
    for (long e = 0; e < n; e++) put_be<R, B, T>(var, b, e, out.data());
    return MPDATA_OK;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* d = nullptr;
  if (cudaMallocAsync(&d, out.size(), s) != cudaSuccess) return MPDATA_E_CUDA;
  const long blocks = (n + 255) / 256;
  k_pack_be<R, B, T><<<(unsigned)(blocks < 1216 ? (blocks < 1 ? 1 : blocks) : 1216), 256, 0, s>>>(var, b, d);
  mpdata::add_launches(1);
  int rc = cudaGetLastError() == cudaSuccess ? MPDATA_OK : MPDATA_E_CUDA;
  if (rc == MPDATA_OK && cudaMemcpyAsync(out.data(), d, out.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    rc = MPDATA_E_CUDA;
  cudaFreeAsync(d, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) rc = MPDATA_E_CUDA;
  return rc;
}

template <class R>
int out_chunk(const char* var_name, const char* file_name, int imode, int ia1, int ia2, int ia3, int ifrmd,
              int imem, const R* var, int np, int mp, int lp, int ih, int on_device, void* stream) {
  if (!var_name || !file_name || !var) return MPDATA_E_NULL;
  if (np < 1 || mp < 1 || lp < 1 || ih < 0 || ifrmd < 0 || !*var_name) return MPDATA_E_DIMS;
  Plan pl;
  if (!make_plan(imode, ia1, ia2, ia3, np, mp, lp, ih, pl)) return MPDATA_E_UNSUPPORTED;
  // the caller's array: var(1-ih:n+ia*imem+ih) on each axis (:7510-7512)
  const long ext[3] = {(long)np + (long)ia1 * imem, (long)mp + (long)ia2 * imem, (long)lp + (long)ia3 * imem};
  for (int a = 0; a < 3; a++) {
    if (ext[a] < 1 || pl.len[a] < 1) return MPDATA_E_DIMS;
    if (pl.write && (pl.cnt[a] < 1 || pl.b0[a] < 1 - ih || (long)pl.b0[a] + pl.cnt[a] - 1 > ext[a] + ih))
      return MPDATA_E_DIMS;
  }
  const std::string path(file_name);
  std::vector<unsigned char> bytes;
  Model m;
  const bool exists = read_file(path, bytes);
  if (exists && !decode(bytes, m)) return MPDATA_E_IO;
  Model old = m;
  bool changed = !exists;
  int vi = find_var(m, var_name);
  if (ifrmd == 0) {  // :7596-7715: dimensions and the variable are defined only at frame 0
    const char* dn[3] = {"x", "y", "z"};
    int did[4];
    for (int a = 0; a < 3; a++) {
      did[a] = find_dim(m, dn[a]);
      if (did[a] < 0 && pl.def[a]) {
        if (pl.len[a] > 0xffffffffULL) return MPDATA_E_TOO_LARGE;
        m.dims.push_back(Dim{dn[a], pl.len[a]});
        did[a] = (int)m.dims.size() - 1;
        changed = true;
      }
    }
    did[3] = find_dim(m, "t");
    if (did[3] < 0) {
      m.dims.push_back(Dim{"t", 0});
      did[3] = (int)m.dims.size() - 1;
      changed = true;
    }
    if (vi < 0) {
      Var v;
      v.name = var_name;
      if (pl.rec) v.dims.push_back((unsigned)did[3]);
      for (int a = 2; a >= 0; a--)
        if (pl.axes >> a & 1u) {
          if (did[a] < 0) return MPDATA_E_DIMS;  // the mode uses a dimension it does not define
          v.dims.push_back((unsigned)did[a]);
        }
      v.type = pl.type;
      v.begin = 0;
      m.vars.push_back(v);
      m.vars.back().vsize = slab_bytes(m, m.vars.back());
      if (m.vars.back().vsize > 0xfffffffcULL) return MPDATA_E_TOO_LARGE;  // a CDF-2 slab size is 32-bit
      vi = (int)m.vars.size() - 1;
      changed = true;
    }
  }
  if (vi < 0) return MPDATA_E_IO;  // the reference's write to an undefined variable fails
  Var& v = m.vars[vi];
  const bool rec = is_rec(m, v);
  // the variable's spatial lengths along x, y, z (1 where it has no such
  // dimension); its dimensions must run t, z, y, x and hold the box
  unsigned long long L[3] = {1, 1, 1};
  {
    int last = 3;
    for (size_t d = rec ? 1 : 0; d < v.dims.size(); d++) {
      const std::string& nm = m.dims[v.dims[d]].name;
      const int a = nm == "x" ? 0 : nm == "y" ? 1 : nm == "z" ? 2 : -1;
      if (a < 0 || a >= last || m.dims[v.dims[d]].len == 0) return MPDATA_E_DIMS;
      L[a] = m.dims[v.dims[d]].len;
      last = a;
    }
    if (rec != pl.rec || (v.type != NC_FLOAT && v.type != NC_DOUBLE)) return MPDATA_E_DIMS;
    if (pl.write)
      for (int a = 0; a < 3; a++)
        if ((unsigned long long)pl.st[a] + (unsigned long long)pl.cnt[a] > L[a]) return MPDATA_E_DIMS;
  }
  std::vector<unsigned char> data;
  if (pl.write) {
    const long sx = ext[0] + 2L * ih, sy = ext[1] + 2L * ih;
    const Box b{(long)(pl.b0[0] - 1 + ih) + (long)(pl.b0[1] - 1 + ih) * sx + (long)(pl.b0[2] - 1 + ih) * sx * sy,
                pl.cnt[0], pl.cnt[1], pl.cnt[2], sx, sx * sy};
    int rc;
    if (v.type == NC_DOUBLE)
      rc = pl.sp ? gather<R, float, double>(var, b, on_device, stream, data)
                 : gather<R, double, double>(var, b, on_device, stream, data);
    else
      rc = pl.sp ? gather<R, float, float>(var, b, on_device, stream, data)
                 : gather<R, double, float>(var, b, on_device, stream, data);
    if (rc) return rc;
  }
  if (changed) {
    const int rc = rewrite(path, old, bytes, m);
    if (rc) return rc;
  }
  if (!pl.write) return MPDATA_OK;
  const bool whole = pl.st[0] == 0 && pl.st[1] == 0 && pl.st[2] == 0 && (unsigned long long)pl.cnt[0] == L[0] &&
                     (unsigned long long)pl.cnt[1] == L[1] && (unsigned long long)pl.cnt[2] == L[2];
  const unsigned long long r = rec ? (unsigned long long)ifrmd : 0;
  FILE* f = std::fopen(path.c_str(), "r+b");
  if (!f) return MPDATA_E_IO;
  bool ok = true;
  const size_t len = rec ? (size_t)(rec_bytes(m) < v.vsize ? rec_bytes(m) : v.vsize) : (size_t)v.vsize;
  const unsigned long long off = rec ? rec_offset(m, v, r) : v.begin;
  const bool fresh = rec && r + 1 > m.numrecs;
  std::vector<unsigned char> slab;
  if (whole) {
    slab.swap(data);
    slab.resize(len, 0);
  } else {  // a box inside the slab: start from what the slab holds (fill values if new)
    if (fresh) {
      slab = fill_slab(v);
    } else {
      slab.resize(len);
      ok = std::fseek(f, (long)off, SEEK_SET) == 0 && std::fread(slab.data(), 1, len, f) == len;
    }
    slab.resize(len, 0);
    const size_t ts = type_size(v.type);
    size_t e = 0;
    for (int k = 0; k < pl.cnt[2]; k++)
      for (int j = 0; j < pl.cnt[1]; j++) {
        const unsigned long long row = ((unsigned long long)(pl.st[2] + k) * L[1] + (unsigned long long)(pl.st[1] + j)) * L[0] +
                                       (unsigned long long)pl.st[0];
        std::memcpy(&slab[row * ts], &data[e * ts], (size_t)pl.cnt[0] * ts);
        e += (size_t)pl.cnt[0];
      }
  }
  // extend the records with fill values if needed, then write the slab
  if (ok && fresh) {
    for (unsigned long long q = m.numrecs; q <= r && ok; q++)
      for (const Var& w : m.vars)
        if (is_rec(m, w) && !(&w == &v && q == r)) {
          const std::vector<unsigned char> fill = fill_slab(w);
          const size_t wl = rec_bytes(m) < w.vsize ? (size_t)rec_bytes(m) : (size_t)w.vsize;
          ok = ok && pwrite_at(f, rec_offset(m, w, q), fill.data(), wl);
        }
    m.numrecs = r + 1;
    const unsigned char nr[4] = {(unsigned char)(m.numrecs >> 24), (unsigned char)(m.numrecs >> 16),
                                 (unsigned char)(m.numrecs >> 8), (unsigned char)m.numrecs};
    ok = ok && pwrite_at(f, 4, nr, 4);
  }
  ok = ok && pwrite_at(f, off, slab.data(), len);
  if (std::fclose(f) != 0) ok = false;
  return ok ? MPDATA_OK : MPDATA_E_IO;
}

// one frame of a float or double (x,y,z[,t]) variable into the interior of a
// psi-shaped caller array (halo untouched)
template <class R>
int in_chunk(const char* var_name, const char* file_name, int ifrmd, R* var, int np, int mp, int lp, int ih,
             int on_device, void* stream) {
  if (!var_name || !file_name || !var) return MPDATA_E_NULL;
  if (np < 1 || mp < 1 || lp < 1 || ih < 0 || ifrmd < 0) return MPDATA_E_DIMS;
  std::vector<unsigned char> bytes;
  Model m;
  if (!read_file(file_name, bytes) || !decode(bytes, m)) return MPDATA_E_IO;
  const int vi = find_var(m, var_name);
  if (vi < 0) return MPDATA_E_IO;
  const Var& v = m.vars[vi];
  const bool rec = is_rec(m, v);
  const size_t nd = v.dims.size();
  if (nd != (rec ? 4u : 3u) || m.dims[v.dims[nd - 1]].len != (unsigned long long)np ||
      m.dims[v.dims[nd - 2]].len != (unsigned long long)mp || m.dims[v.dims[nd - 3]].len != (unsigned long long)lp ||
      (v.type != NC_FLOAT && v.type != NC_DOUBLE))
    return MPDATA_E_DIMS;
  if (rec && (unsigned long long)ifrmd >= m.numrecs) return MPDATA_E_IO;
  const unsigned long long off = rec ? rec_offset(m, v, ifrmd) : v.begin;
  const size_t ts = type_size(v.type), n = (size_t)np * mp * lp;
  if (off + n * ts > bytes.size()) return MPDATA_E_IO;
  const int sx = np + 2 * ih, sy = mp + 2 * ih, sz = lp + 2 * ih;
  const size_t total = (size_t)sx * sy * sz;
  std::vector<R> host(on_device ? total : 0);
  R* dst = on_device ? host.data() : var;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (on_device) {  // keep the halo: start from the device array
    if (cudaMemcpyAsync(host.data(), var, total * sizeof(R), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return MPDATA_E_CUDA;
  }
  size_t t = 0;
  for (int k = 0; k < lp; k++)
    for (int j = 0; j < mp; j++)
      for (int i = 0; i < np; i++, t++) {
        const unsigned char* p = &bytes[off + t * ts];
        unsigned long long b = 0;
        for (size_t q = 0; q < ts; q++) b = (b << 8) | p[q];
        double val;
        if (ts == 8) {
          std::memcpy(&val, &b, 8);
        } else {
          unsigned b4 = (unsigned)b;
          float f;
          std::memcpy(&f, &b4, 4);
          val = f;
        }
        dst[(size_t)(i + ih) + (size_t)(j + ih) * sx + (size_t)(k + ih) * sx * sy] = (R)val;
      }
  if (on_device) {
    if (cudaMemcpyAsync(var, host.data(), total * sizeof(R), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return MPDATA_E_CUDA;
  }
  return MPDATA_OK;
}

}  // namespace

extern "C" {

int mpdata_pnet_out_chunk_f64(const char* var_name, const char* file_name, int imode, int ia1, int ia2, int ia3,
                              int ifrmd, int imem, const double* var, int np, int mp, int lp, int ih,
                              int on_device, void* stream) {
  return out_chunk<double>(var_name, file_name, imode, ia1, ia2, ia3, ifrmd, imem, var, np, mp, lp, ih, on_device,
                           stream);
}
int mpdata_pnet_out_chunk_f32(const char* var_name, const char* file_name, int imode, int ia1, int ia2, int ia3,
                              int ifrmd, int imem, const float* var, int np, int mp, int lp, int ih, int on_device,
                              void* stream) {
  return out_chunk<float>(var_name, file_name, imode, ia1, ia2, ia3, ifrmd, imem, var, np, mp, lp, ih, on_device,
                          stream);
}
int mpdata_pnet_in_chunk_f64(const char* var_name, const char* file_name, int ifrmd, double* var, int np, int mp,
                             int lp, int ih, int on_device, void* stream) {
  return in_chunk<double>(var_name, file_name, ifrmd, var, np, mp, lp, ih, on_device, stream);
}
int mpdata_pnet_in_chunk_f32(const char* var_name, const char* file_name, int ifrmd, float* var, int np, int mp,
                             int lp, int ih, int on_device, void* stream) {
  return in_chunk<float>(var_name, file_name, ifrmd, var, np, mp, lp, ih, on_device, stream);
}

}  // extern "C"
