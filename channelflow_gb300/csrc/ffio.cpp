// channelflow's binary FlowField format (.ff), read and written on the host.
//
// Format (channelflow/flowfield.cpp:2642-2723 writes it, :216-356 reads it;
// primitive encodings cfbasics/cfbasics.h:368-470):
//   int32 major, minor, update (2, 0, 9 from channelflowVersion,
//   utilfuncs.cpp:810-814), int32 Nx, Ny, Nz, Nd, char xzstate, char ystate
//   ('S' or 'P'), float64 Lx, Lz, a, b, char padded ('1' or '0'); all
//   integers and doubles big-endian.  Then the data:
//   * spectral in x,z and padded: for each component i and y index ny, the
//     modes nx = 0..Nxd then nx = Nx-Nxd..Nx-1, each with nz = 0..Nzd/2,
//     as (re, im) pairs, where Nxd = 2(Nx/6) and Nzd = 2(Nz/3)+1;
//   * spectral in x,z, not padded: every (nx, nz < Nz/2+1) as (re, im);
//   * physical: every real value [i][ny][nx][nz < 2(Nz/2+1)].
// Buffers passed in and out are the FlowField's spectral storage, complex
// [i][ny][nx][Nz/2+1] (channelflow/flowfield.h:383-402).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cfgpu.h"

int cfgpu_record_error(int code, const std::string& msg);

namespace {

void put_be32(std::vector<unsigned char>& o, uint32_t v) {
  for (int s = 24; s >= 0; s -= 8) o.push_back((unsigned char)(v >> s));
}
void put_be64(std::vector<unsigned char>& o, double d) {
  uint64_t v;
  memcpy(&v, &d, 8);
  for (int s = 56; s >= 0; s -= 8) o.push_back((unsigned char)(v >> s));
}
uint32_t get_be32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}
double get_be64(const unsigned char* p) {
  uint64_t v = 0;
  for (int k = 0; k < 8; ++k) v = (v << 8) | p[k];
  double d;
  memcpy(&d, &v, 8);
  return d;
}

constexpr size_t kHeaderBytes = 3 * 4 + 4 * 4 + 2 + 4 * 8 + 1;  // 63

struct Header {
  int major, minor, update, Nx, Ny, Nz, Nd;
  char xz, y;
  double Lx, Lz, a, b;
  bool padded;
};

int read_file(const char* path, std::vector<unsigned char>& buf) {
  FILE* f = fopen(path, "rb");
  if (!f) return cfgpu_record_error(CFGPU_EINVAL, std::string("can't open file ") + path);
  unsigned char chunk[1 << 16];
  size_t n;
  while ((n = fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
  fclose(f);
  return CFGPU_OK;
}

int parse_header(const std::vector<unsigned char>& b, Header& h) {
  if (b.size() < kHeaderBytes) return cfgpu_record_error(CFGPU_EINVAL, "file too short for a .ff header");
  const unsigned char* p = b.data();
  int* ints[7] = {&h.major, &h.minor, &h.update, &h.Nx, &h.Ny, &h.Nz, &h.Nd};
  for (int k = 0; k < 7; ++k) *ints[k] = (int)get_be32(p + 4 * k);
  p += 28;
  h.xz = (char)p[0];
  h.y = (char)p[1];
  p += 2;
  h.Lx = get_be64(p);
  h.Lz = get_be64(p + 8);
  h.a = get_be64(p + 16);
  h.b = get_be64(p + 24);
  p += 32;
  h.padded = p[0] != '0';
  if (h.Nx <= 0 || h.Ny <= 0 || h.Nz <= 0 || h.Nd <= 0 || h.Nx > (1 << 16) || h.Ny > (1 << 16) ||
      h.Nz > (1 << 16) || h.Nd > 64)
    return cfgpu_record_error(CFGPU_EINVAL, "implausible .ff header dimensions");
  return CFGPU_OK;
}

// Number of doubles in the data section for this header.
size_t data_doubles(const Header& h) {
  const size_t Mz = h.Nz / 2 + 1;
  if (h.xz == 'S' && h.padded) {
    const size_t Nxd = 2 * (h.Nx / 6), Nzd = 2 * (h.Nz / 3) + 1;
    return (size_t)h.Nd * h.Ny * (2 * Nxd + 1) * (Nzd / 2 + 1) * 2;
  }
  if (h.xz == 'S') return (size_t)h.Nd * h.Ny * h.Nx * Mz * 2;
  return (size_t)h.Nd * h.Ny * h.Nx * 2 * Mz;
}

}  // namespace

extern "C" {

cfgpu_status cfgpu_ff_write(const char* path, int Nx, int Ny, int Nz, int Nd, double Lx, double Lz, double a,
                            double b, int padded, const double* data) {
  if (!path || !data || Nx <= 0 || Ny <= 0 || Nz <= 0 || Nd <= 0)
    return cfgpu_record_error(CFGPU_EINVAL, "bad argument");
  const size_t Mz = Nz / 2 + 1;
  std::vector<unsigned char> o;
  o.reserve(kHeaderBytes + (size_t)Nd * Ny * Nx * Mz * 16);
  for (int v : {2, 0, 9, Nx, Ny, Nz, Nd}) put_be32(o, (uint32_t)v);
  o.push_back('S');
  o.push_back('S');
  for (double v : {Lx, Lz, a, b}) put_be64(o, v);
  o.push_back(padded ? '1' : '0');
  auto put_mode = [&](int i, int ny, int nx, int nz) {
    const size_t k = 2 * ((((size_t)i * Ny + ny) * Nx + nx) * Mz + nz);
    put_be64(o, data[k]);
    put_be64(o, data[k + 1]);
  };
  for (int i = 0; i < Nd; ++i)
    for (int ny = 0; ny < Ny; ++ny) {
      if (padded) {
        const int Nxd = 2 * (Nx / 6), Nzd = 2 * (Nz / 3) + 1;
        for (int nx = 0; nx <= Nxd; ++nx)
          for (int nz = 0; nz <= Nzd / 2; ++nz) put_mode(i, ny, nx, nz);
        for (int nx = Nx - Nxd; nx < Nx; ++nx)
          for (int nz = 0; nz <= Nzd / 2; ++nz) put_mode(i, ny, nx, nz);
      } else {
        for (int nx = 0; nx < Nx; ++nx)
          for (int nz = 0; nz < (int)Mz; ++nz) put_mode(i, ny, nx, nz);
      }
    }
  FILE* f = fopen(path, "wb");
  if (!f) return cfgpu_record_error(CFGPU_EINVAL, std::string("can't open file ") + path);
  const size_t w = fwrite(o.data(), 1, o.size(), f);
  const int cl = fclose(f);
  if (w != o.size() || cl != 0) return cfgpu_record_error(CFGPU_EINVAL, std::string("short write to ") + path);
  return CFGPU_OK;
}

cfgpu_status cfgpu_ff_read_header(const char* path, int* dims, double* geom, int* padded, char* state) {
  if (!path || !dims || !geom) return cfgpu_record_error(CFGPU_EINVAL, "bad argument");
  std::vector<unsigned char> b;
  int s = read_file(path, b);
  if (s != CFGPU_OK) return s;
  Header h;
  if ((s = parse_header(b, h)) != CFGPU_OK) return s;
  dims[0] = h.Nx; dims[1] = h.Ny; dims[2] = h.Nz; dims[3] = h.Nd;
  geom[0] = h.Lx; geom[1] = h.Lz; geom[2] = h.a; geom[3] = h.b;
  if (padded) *padded = h.padded ? 1 : 0;
  if (state) { state[0] = h.xz; state[1] = h.y; }
  return CFGPU_OK;
}

cfgpu_status cfgpu_ff_read(const char* path, double* data, size_t ndoubles) {
  if (!path || !data) return cfgpu_record_error(CFGPU_EINVAL, "bad argument");
  std::vector<unsigned char> b;
  int s = read_file(path, b);
  if (s != CFGPU_OK) return s;
  Header h;
  if ((s = parse_header(b, h)) != CFGPU_OK) return s;
  if (h.xz != 'S' || h.y != 'S')
    return cfgpu_record_error(CFGPU_ENOTSUP, "only fields saved in spectral state (xz and y) are read");
  const size_t Mz = h.Nz / 2 + 1;
  const size_t need = (size_t)h.Nd * h.Ny * h.Nx * Mz * 2;
  if (ndoubles < need) return cfgpu_record_error(CFGPU_EINVAL, "output buffer too small for the field");
  if (b.size() < kHeaderBytes + 8 * data_doubles(h)) return cfgpu_record_error(CFGPU_EINVAL, "truncated .ff file");
  memset(data, 0, need * sizeof(double));
  const unsigned char* p = b.data() + kHeaderBytes;
  auto get_mode = [&](int i, int ny, int nx, int nz) {
    const size_t k = 2 * ((((size_t)i * h.Ny + ny) * h.Nx + nx) * Mz + nz);
    data[k] = get_be64(p);
    data[k + 1] = get_be64(p + 8);
    p += 16;
  };
  for (int i = 0; i < h.Nd; ++i)
    for (int ny = 0; ny < h.Ny; ++ny) {
      if (h.padded) {
        const int Nxd = 2 * (h.Nx / 6), Nzd = 2 * (h.Nz / 3) + 1;
        for (int nx = 0; nx <= Nxd; ++nx)
          for (int nz = 0; nz <= Nzd / 2; ++nz) get_mode(i, ny, nx, nz);
        for (int nx = h.Nx - Nxd; nx < h.Nx; ++nx)
          for (int nz = 0; nz <= Nzd / 2; ++nz) get_mode(i, ny, nx, nz);
      } else {
        for (int nx = 0; nx < h.Nx; ++nx)
          for (int nz = 0; nz < (int)Mz; ++nz) get_mode(i, ny, nx, nz);
      }
    }
  return CFGPU_OK;
}

}  // extern "C"
