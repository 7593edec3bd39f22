// NIfTI-1 single-file images (.nii, and .nii.gz where zlib is available) for
// the command-line reconstruction (the reference reads and writes them with
// nifti/nifti1_io.c from apps/command_line_tools/rec_spect.cpp:447-606).
// Written from the NIfTI-1 format definition: a 348-byte header (sizeof_hdr,
// dim[8] at byte 40, datatype at 70, bitpix at 72, pixdim[8] at 76,
// vox_offset at 108, scl_slope / scl_inter at 112 / 116, magic "n+1" at
// 344), a 4-byte extension flag, then the voxels at vox_offset; either byte
// order (detected from sizeof_hdr).  Readers convert every integer and real
// datatype to float32 and apply a non-zero scl_slope; writers store float32.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#ifdef NRGB_ZLIB
#include <zlib.h>
#endif

#include "et_array_interface.h"
#include "et_common.h"

namespace nrgb {
namespace {

constexpr int kHeaderBytes = 348;
constexpr int kDataOffset = 352;  // header + extension flag

bool ends_with(const std::string& s, const char* suffix) {
  const size_t n = std::strlen(suffix);
  return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

// Whole-file read / write through stdio or zlib (by the .gz suffix).
bool read_file(const std::string& path, std::vector<unsigned char>* out) {
  out->clear();
  if (ends_with(path, ".gz")) {
#ifdef NRGB_ZLIB
    gzFile f = gzopen(path.c_str(), "rb");
    if (!f) return false;
    unsigned char buf[1 << 16];
    int n;
    while ((n = gzread(f, buf, sizeof(buf))) > 0) out->insert(out->end(), buf, buf + n);
    const bool ok = n == 0;
    gzclose(f);
    return ok;
#else
    return false;
#endif
  }
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  unsigned char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out->insert(out->end(), buf, buf + n);
  const bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

bool write_file(const std::string& path, const std::vector<unsigned char>& data) {
  if (ends_with(path, ".gz")) {
#ifdef NRGB_ZLIB
    gzFile f = gzopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = gzwrite(f, data.data(), static_cast<unsigned>(data.size())) == static_cast<int>(data.size());
    return gzclose(f) == Z_OK && ok;
#else
    return false;
#endif
  }
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
  return std::fclose(f) == 0 && ok;
}

template <class T>
T get(const unsigned char* p, bool swap) {
  unsigned char b[sizeof(T)];
  std::memcpy(b, p, sizeof(T));
  if (swap)
    for (size_t i = 0; i < sizeof(T) / 2; ++i) std::swap(b[i], b[sizeof(T) - 1 - i]);
  T v;
  std::memcpy(&v, b, sizeof(T));
  return v;
}

template <class T>
void put(unsigned char* p, T v) {
  std::memcpy(p, &v, sizeof(T));
}

struct Header {
  bool swap = false;
  int dims[7] = {1, 1, 1, 1, 1, 1, 1};  // dim[1..7]
  int ndim = 0;
  int datatype = 0;
  size_t offset = 0;
  float slope = 0.0f, inter = 0.0f;
  size_t voxels() const {
    size_t n = 1;
    for (int i = 0; i < ndim; ++i) n *= static_cast<size_t>(dims[i]);
    return n;
  }
};

int parse_header(const std::vector<unsigned char>& f, Header* h) {
  if (f.size() < static_cast<size_t>(kHeaderBytes)) return kErrParameters;
  const unsigned char* p = f.data();
  const int32_t sz = get<int32_t>(p, false);
  if (sz == kHeaderBytes) {
    h->swap = false;
  } else if (get<int32_t>(p, true) == kHeaderBytes) {
    h->swap = true;
  } else {
    return kErrParameters;
  }
  if (std::memcmp(p + 344, "n+1", 4) != 0) return kErrParameters;  // single-file NIfTI-1 only
  h->ndim = get<int16_t>(p + 40, h->swap);
  if (h->ndim < 1 || h->ndim > 7) return kErrParameters;
  for (int i = 0; i < h->ndim; ++i) {
    h->dims[i] = get<int16_t>(p + 42 + 2 * i, h->swap);
    if (h->dims[i] < 1) return kErrParameters;
  }
  h->datatype = get<int16_t>(p + 70, h->swap);
  const float off = get<float>(p + 108, h->swap);
  h->offset = off >= kDataOffset ? static_cast<size_t>(off) : kDataOffset;
  h->slope = get<float>(p + 112, h->swap);
  h->inter = get<float>(p + 116, h->swap);
  return kOk;
}

int bytes_of(int datatype) {
  switch (datatype) {
    case 2: case 256: return 1;     // uint8, int8
    case 4: case 512: return 2;     // int16, uint16
    case 8: case 768: case 16: return 4;  // int32, uint32, float32
    case 64: return 8;              // float64
    default: return 0;
  }
}

}  // namespace
}  // namespace nrgb

using namespace nrgb;

extern "C" {

int nrgb_nifti_info(const char* path, int* dims) {
  if (!path || !dims) return kErrParameters;
  std::vector<unsigned char> f;
  if (!read_file(path, &f)) return kErrParameters;
  Header h;
  int s = parse_header(f, &h);
  if (s != kOk) return s;
  dims[0] = h.ndim;
  for (int i = 0; i < 7; ++i) dims[1 + i] = i < h.ndim ? h.dims[i] : 1;
  return kOk;
}

int nrgb_nifti_read(const char* path, float* data, long long n_voxels) {
  if (!path || !data) return kErrParameters;
  std::vector<unsigned char> f;
  if (!read_file(path, &f)) return kErrParameters;
  Header h;
  int s = parse_header(f, &h);
  if (s != kOk) return s;
  const int b = bytes_of(h.datatype);
  const size_t n = h.voxels();
  if (b == 0 || static_cast<long long>(n) != n_voxels || h.offset + n * b > f.size()) return kErrParameters;
  const unsigned char* p = f.data() + h.offset;
  const bool scale = h.slope != 0.0f && !(h.slope == 1.0f && h.inter == 0.0f);
  for (size_t i = 0; i < n; ++i, p += b) {
    double v;
    switch (h.datatype) {
      case 2: v = *p; break;
      case 256: v = static_cast<int8_t>(*p); break;
      case 4: v = get<int16_t>(p, h.swap); break;
      case 512: v = get<uint16_t>(p, h.swap); break;
      case 8: v = get<int32_t>(p, h.swap); break;
      case 768: v = get<uint32_t>(p, h.swap); break;
      case 16: v = get<float>(p, h.swap); break;
      default: v = get<double>(p, h.swap); break;
    }
    data[i] = scale ? static_cast<float>(v * h.slope + h.inter) : static_cast<float>(v);
  }
  return kOk;
}

int nrgb_nifti_write(const char* path, const float* data, const int* dims) {
  if (!path || !data || !dims || dims[0] < 1 || dims[0] > 7) return kErrParameters;
  size_t n = 1;
  for (int i = 1; i <= dims[0]; ++i) {
    if (dims[i] < 1 || dims[i] > 32767) return kErrParameters;
    n *= static_cast<size_t>(dims[i]);
  }
  std::vector<unsigned char> f(kDataOffset + n * sizeof(float), 0);
  unsigned char* p = f.data();
  put<int32_t>(p, kHeaderBytes);
  put<int16_t>(p + 40, static_cast<int16_t>(dims[0]));
  for (int i = 1; i <= 7; ++i) put<int16_t>(p + 40 + 2 * i, static_cast<int16_t>(i <= dims[0] ? dims[i] : 1));
  put<int16_t>(p + 70, 16);  // float32
  put<int16_t>(p + 72, 32);  // bitpix
  for (int i = 0; i < 8; ++i) put<float>(p + 76 + 4 * i, 1.0f);  // qfac and unit voxels
  put<float>(p + 108, static_cast<float>(kDataOffset));
  put<float>(p + 112, 1.0f);  // scl_slope
  std::memcpy(p + 344, "n+1", 4);
  std::memcpy(p + kDataOffset, data, n * sizeof(float));
  return write_file(path, f) ? kOk : kErrParameters;
}

int nrgb_nifti_gzip_supported(void) {
#ifdef NRGB_ZLIB
  return 1;
#else
  return 0;
#endif
}

}  // extern "C"
