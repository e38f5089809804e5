// The reference's shearing-filter bank file ("SHFM0002"), read and written on
// the host.  Layout (little-endian), as save_shearing_filters.m:46-84 writes
// it and ShearConfig::readFromFile (demoImageDenoise/shearconfig.cpp:26-78)
// reads it:
//   8 bytes  "SHFM0002"
//   uint16   number of scales
//   uint16   data type: 0 = single, 2 = double
//   per scale: uint16 filter size n, uint16 number of directions d, then d
//              filters of n x n values, each in MATLAB (column-major) order
//   4 times:   uint16 size F, then F x F values, column-major: the pyramid
//              filters h0, h1, g0, g1
// The library keeps filters row-major; reading and writing transpose.
#include <cstdio>
#include <cstring>
#include <memory>

#include "internal.h"

namespace nsst {

namespace {

struct FileCloser {
  void operator()(FILE* f) const {
    if (f) std::fclose(f);
  }
};
using FilePtr = std::unique_ptr<FILE, FileCloser>;

bool get_u16(FILE* f, int* v) {
  unsigned char b[2];
  if (std::fread(b, 1, 2, f) != 2) return false;
  *v = (int)b[0] | ((int)b[1] << 8);
  return true;
}
bool put_u16(FILE* f, int v) {
  const unsigned char b[2] = {(unsigned char)(v & 0xff), (unsigned char)((v >> 8) & 0xff)};
  return std::fwrite(b, 1, 2, f) == 2;
}

// n x n values, column-major in the file, row-major in `out`
bool get_matrix(FILE* f, int n, int dtype, double* out) {
  const size_t cnt = (size_t)n * n, es = dtype == kShfmDouble ? 8 : 4;
  std::vector<unsigned char> raw(cnt * es);
  if (std::fread(raw.data(), 1, raw.size(), f) != raw.size()) return false;
  for (size_t k = 0; k < cnt; k++) {
    const unsigned char* b = raw.data() + k * es;
    double v;
    if (es == 8) {
      uint64_t u = 0;
      for (int i = 7; i >= 0; i--) u = (u << 8) | b[i];
      std::memcpy(&v, &u, 8);
    } else {
      uint32_t u = 0;
      for (int i = 3; i >= 0; i--) u = (u << 8) | b[i];
      float x;
      std::memcpy(&x, &u, 4);
      v = x;
    }
    const size_t r = k % n, c = k / n;  // column-major position k
    out[r * n + c] = v;
  }
  return true;
}

bool put_matrix(FILE* f, int n, int dtype, const double* in) {
  const size_t cnt = (size_t)n * n, es = dtype == kShfmDouble ? 8 : 4;
  std::vector<unsigned char> raw(cnt * es);
  for (size_t k = 0; k < cnt; k++) {
    const size_t r = k % n, c = k / n;
    const double v = in[r * n + c];
    unsigned char* b = raw.data() + k * es;
    if (es == 8) {
      uint64_t u;
      std::memcpy(&u, &v, 8);
      for (int i = 0; i < 8; i++) b[i] = (unsigned char)((u >> (8 * i)) & 0xff);
    } else {
      const float x = (float)v;
      uint32_t u;
      std::memcpy(&u, &x, 4);
      for (int i = 0; i < 4; i++) b[i] = (unsigned char)((u >> (8 * i)) & 0xff);
    }
  }
  return std::fwrite(raw.data(), 1, raw.size(), f) == raw.size();
}

}  // namespace

bool read_filter_file(const char* path, FilterSet* fs, std::string* err) {
  FilePtr f(std::fopen(path, "rb"));
  if (!f) {
    *err = std::string("cannot open ") + path;
    return false;
  }
  char magic[8];
  if (std::fread(magic, 1, 8, f.get()) != 8 || std::memcmp(magic, "SHFM0002", 8) != 0) {
    *err = "not an SHFM0002 shearing-filter file";
    return false;
  }
  int nscales = 0, dtype = 0;
  if (!get_u16(f.get(), &nscales) || !get_u16(f.get(), &dtype)) {
    *err = "truncated header";
    return false;
  }
  if (dtype != kShfmSingle && dtype != kShfmDouble) {
    *err = "unknown data type code " + std::to_string(dtype) + " (0 single, 2 double)";
    return false;
  }
  if (nscales < 1 || nscales > NSST_MAX_LEVELS) {
    *err = "number of scales must be in [1, 8]";
    return false;
  }
  fs->nlev = nscales;
  fs->dtype = dtype;
  for (int j = 0; j < nscales; j++) {
    int n = 0, d = 0;
    if (!get_u16(f.get(), &n) || !get_u16(f.get(), &d) || n < 1 || d < 1) {
      *err = "truncated or empty scale header";
      return false;
    }
    fs->dsize[j] = n;
    fs->ndir[j] = d;
    fs->shear[j].assign((size_t)d * n * n, 0.0);
    for (int k = 0; k < d; k++)
      if (!get_matrix(f.get(), n, dtype, fs->shear[j].data() + (size_t)k * n * n)) {
        *err = "truncated shearing filters";
        return false;
      }
  }
  fs->pf.name = "file";
  for (int k = 0; k < 4; k++) {
    int F = 0;
    if (!get_u16(f.get(), &F) || F < 1) {
      *err = "truncated pyramid filter header";
      return false;
    }
    fs->pf.F[k] = F;
    fs->pf.h[k].assign((size_t)F * F, 0.0);
    if (!get_matrix(f.get(), F, dtype, fs->pf.h[k].data())) {
      *err = "truncated pyramid filters";
      return false;
    }
  }
  return true;
}

bool write_filter_file(const char* path, const FilterSet& fs, std::string* err) {
  FilePtr f(std::fopen(path, "wb"));
  if (!f) {
    *err = std::string("cannot create ") + path;
    return false;
  }
  bool ok = std::fwrite("SHFM0002", 1, 8, f.get()) == 8 && put_u16(f.get(), fs.nlev) && put_u16(f.get(), fs.dtype);
  for (int j = 0; ok && j < fs.nlev; j++) {
    const int n = fs.dsize[j], d = fs.ndir[j];
    ok = put_u16(f.get(), n) && put_u16(f.get(), d);
    for (int k = 0; ok && k < d; k++) ok = put_matrix(f.get(), n, fs.dtype, fs.shear[j].data() + (size_t)k * n * n);
  }
  for (int k = 0; ok && k < 4; k++)
    ok = put_u16(f.get(), fs.pf.F[k]) && put_matrix(f.get(), fs.pf.F[k], fs.dtype, fs.pf.h[k].data());
  if (ok) ok = std::fflush(f.get()) == 0;
  if (!ok) *err = std::string("write failed: ") + path;
  return ok;
}

}  // namespace nsst
