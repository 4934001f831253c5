// io.cu — particle-field state files: vpm_save (the role of FLOWVPM's
// vpm.save, src/FLOWUnsteady_simulation.jl:436-440) and vpm_load (vpm.read!,
// :264).  No HDF5 library is available to this build, so the field is written
// as one raw little-endian FP64 file plus an XDMF description of it, which
// ParaView reads the way it reads FLOWVPM's .xmf/.h5 pairs.
//
// <path>.pfield[.<num>].bin: a 64-byte header
//   char magic[8] = "VPMFIELD", uint32 version = 2, uint32 header bytes = 64,
//   int64 n, int64 n_static, double t, int64 nt, int64 reserved[2],
// then, particle-major: X (n×3), Γ (n×3), σ (n), C (n×3: C_d and its two
// Lagrangian averages), static flag (n: 0 or 1), vol (n), circulation (n).
// Version 1 files end after the static flag (their static particles are the
// last n_static) and load with vol 0 and circulation 1.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"

namespace {

constexpr char kMagic[8] = {'V', 'P', 'M', 'F', 'I', 'E', 'L', 'D'};
constexpr uint32_t kVersion = 2;
constexpr uint32_t kHeaderBytes = 64;

struct Header {
  char magic[8];
  uint32_t version;
  uint32_t header_bytes;
  int64_t n;
  int64_t n_static;
  double t;
  int64_t nt;
  int64_t reserved[2];
};
static_assert(sizeof(Header) == kHeaderBytes, "header layout");

std::string base_name(const std::string& p) {
  const size_t k = p.find_last_of('/');
  return k == std::string::npos ? p : p.substr(k + 1);
}

// Device SoA rows [0, n) of `rows` rows (leading dimension ld) into host
// particle-major storage out[i*rows + r].
cudaError_t rows_to_host(const double* dev, int rows, int64_t ld, int64_t n, double* out,
                         cudaStream_t st) {
  std::vector<double> row(static_cast<size_t>(n));
  for (int r = 0; r < rows; ++r) {
    cudaError_t e = cudaMemcpyAsync(row.data(), dev + r * ld, n * sizeof(double),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    for (int64_t i = 0; i < n; ++i) out[i * rows + r] = row[size_t(i)];
  }
  return cudaSuccess;
}

void xdmf_item(FILE* f, const char* indent, const std::string& bin, int64_t n, int comps,
               int64_t seek) {
  if (comps == 1)
    std::fprintf(f, "%s<DataItem DataType=\"Float\" Precision=\"8\" Dimensions=\"%lld\" ", indent,
                 (long long)n);
  else
    std::fprintf(f, "%s<DataItem DataType=\"Float\" Precision=\"8\" Dimensions=\"%lld %d\" ",
                 indent, (long long)n, comps);
  std::fprintf(f, "Format=\"Binary\" Endian=\"Little\" Seek=\"%lld\">%s</DataItem>\n",
               (long long)seek, bin.c_str());
}

}  // namespace

extern "C" int vpm_save(vpm_ctx* c, const char* path, int64_t num) {
  if (!c) return vpm::set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!path || !path[0]) return vpm::set_error(&c->err, VPM_ERR_INVALID, "empty path");
  int dev_prev = 0;
  cudaGetDevice(&dev_prev);
  if (dev_prev != c->device) cudaSetDevice(c->device);
  const int64_t n = c->n;
  const size_t n1 = static_cast<size_t>(n), n3 = 3 * n1;
  std::vector<double> X(n3), G(n3), S(n1), C(n3), st(n1), vol(n1), circ(n1);
  cudaError_t e = rows_to_host(c->X, 3, c->ld, n, X.data(), c->st);
  if (e == cudaSuccess) e = rows_to_host(c->G, 3, c->ld, n, G.data(), c->st);
  if (e == cudaSuccess) e = rows_to_host(c->S, 1, c->ld, n, S.data(), c->st);
  if (e == cudaSuccess) e = rows_to_host(c->C, 3, c->ld, n, C.data(), c->st);
  if (e == cudaSuccess) e = rows_to_host(c->vol, 1, c->ld, n, vol.data(), c->st);
  if (e == cudaSuccess) e = rows_to_host(c->circ, 1, c->ld, n, circ.data(), c->st);
  if (dev_prev != c->device) cudaSetDevice(dev_prev);
  if (e != cudaSuccess)
    return vpm::set_error(&c->err, VPM_ERR_CUDA, std::string("save: ") + cudaGetErrorString(e));
  for (int64_t i = 0; i < n; ++i) st[size_t(i)] = c->hstat[size_t(i)] ? 1.0 : 0.0;

  std::string stem = std::string(path) + ".pfield";
  if (num >= 0) stem += "." + std::to_string(num);
  const std::string bin = stem + ".bin", xmf = stem + ".xmf";
  Header h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.header_bytes = kHeaderBytes;
  h.n = n;
  h.n_static = c->n_static;
  h.t = c->t;
  h.nt = c->nt;
  FILE* f = std::fopen(bin.c_str(), "wb");
  if (!f) return vpm::set_error(&c->err, VPM_ERR_INVALID, "cannot open " + bin);
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
  for (const std::vector<double>* a : {&X, &G, &S, &C, &st, &vol, &circ})
    ok = ok && (a->empty() || std::fwrite(a->data(), sizeof(double), a->size(), f) == a->size());
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return vpm::set_error(&c->err, VPM_ERR_INVALID, "cannot write " + bin);

  f = std::fopen(xmf.c_str(), "w");
  if (!f) return vpm::set_error(&c->err, VPM_ERR_INVALID, "cannot open " + xmf);
  const std::string b = base_name(bin);
  const int64_t oX = kHeaderBytes, oG = oX + 24 * n, oS = oG + 24 * n, oC = oS + 8 * n,
                oT = oC + 24 * n, oV = oT + 8 * n, oR = oV + 8 * n;
  std::fprintf(f, "<?xml version=\"1.0\" ?>\n<Xdmf Version=\"3.0\">\n <Domain>\n");
  std::fprintf(f, "  <Grid Name=\"particles\" GridType=\"Uniform\">\n");
  std::fprintf(f, "   <Time Value=\"%.17g\"/>\n", c->t);
  std::fprintf(f, "   <Topology TopologyType=\"Polyvertex\" NumberOfElements=\"%lld\" "
                  "NodesPerElement=\"1\"/>\n", (long long)n);
  std::fprintf(f, "   <Geometry GeometryType=\"XYZ\">\n");
  xdmf_item(f, "    ", b, n, 3, oX);
  std::fprintf(f, "   </Geometry>\n");
  const struct { const char* name; const char* type; int comps; int64_t seek; } attrs[] = {
      {"Gamma", "Vector", 3, oG}, {"sigma", "Scalar", 1, oS}, {"C", "Vector", 3, oC},
      {"static", "Scalar", 1, oT}, {"vol", "Scalar", 1, oV}, {"circulation", "Scalar", 1, oR}};
  for (const auto& a : attrs) {
    std::fprintf(f, "   <Attribute Name=\"%s\" AttributeType=\"%s\" Center=\"Node\">\n", a.name,
                 a.type);
    xdmf_item(f, "    ", b, n, a.comps, a.seek);
    std::fprintf(f, "   </Attribute>\n");
  }
  std::fprintf(f, "  </Grid>\n </Domain>\n</Xdmf>\n");
  if (std::fclose(f) != 0) return vpm::set_error(&c->err, VPM_ERR_INVALID, "cannot write " + xmf);
  return VPM_OK;
}

extern "C" int vpm_load(vpm_ctx* c, const char* file, int load_time) {
  if (!c) return vpm::set_error(nullptr, VPM_ERR_INVALID, "null context");
  if (!file || !file[0]) return vpm::set_error(&c->err, VPM_ERR_INVALID, "empty path");
  FILE* f = std::fopen(file, "rb");
  if (!f) return vpm::set_error(&c->err, VPM_ERR_INVALID, std::string("cannot open ") + file);
  Header h;
  const bool head_ok = std::fread(&h, sizeof(h), 1, f) == 1;
  if (!head_ok || std::memcmp(h.magic, kMagic, 8) != 0 || (h.version != 1 && h.version != 2) ||
      h.header_bytes != kHeaderBytes || h.n < 0 || h.n_static < 0 || h.n_static > h.n) {
    std::fclose(f);
    return vpm::set_error(&c->err, VPM_ERR_INVALID, std::string("not a particle-field file: ") + file);
  }
  if (h.n > c->cap) {
    std::fclose(f);
    return vpm::set_error(&c->err, VPM_ERR_CAPACITY, "saved field exceeds the context capacity");
  }
  const int64_t n = h.n;
  const size_t n1 = static_cast<size_t>(n), n3 = 3 * n1;
  std::vector<double> X(n3), G(n3), S(n1), C(n3), st(n1), vol(n1, 0.0), circ(n1, 1.0);
  bool ok = true;
  for (std::vector<double>* a : {&X, &G, &S, &C, &st})
    ok = ok && (a->empty() || std::fread(a->data(), sizeof(double), a->size(), f) == a->size());
  if (h.version >= 2)
    for (std::vector<double>* a : {&vol, &circ})
      ok = ok && (a->empty() || std::fread(a->data(), sizeof(double), a->size(), f) == a->size());
  std::fclose(f);
  if (!ok) return vpm::set_error(&c->err, VPM_ERR_INVALID, std::string("truncated file: ") + file);
  // Static flags: 0 or 1 each, as many ones as the header's static count
  // (version 1: the last n_static particles).
  std::vector<uint8_t> flags(n1);
  int64_t nstat = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double v = st[size_t(i)];
    if (v != 0.0 && v != 1.0)
      return vpm::set_error(&c->err, VPM_ERR_INVALID, std::string("bad static flag in ") + file);
    flags[size_t(i)] = v != 0.0 ? 1 : 0;
    nstat += flags[size_t(i)];
    if (h.version == 1 && (flags[size_t(i)] != 0) != (i >= n - h.n_static))
      return vpm::set_error(&c->err, VPM_ERR_INVALID,
                            std::string("static flags disagree with the static count in ") + file);
  }
  if (nstat != h.n_static)
    return vpm::set_error(&c->err, VPM_ERR_INVALID,
                          std::string("static flags disagree with the static count in ") + file);
  int rc = vpm_set_particles(c, n, X.data(), 3, G.data(), 3, S.data(), 1);
  if (rc == VPM_OK) rc = ctx_set_static_flags(c, flags.data(), n);
  if (rc == VPM_OK)
    rc = vpm_set_attributes(c, 0, n, vol.data(), 1, circ.data(), 1, C.data(), 3);
  if (rc != VPM_OK) return rc;
  if (load_time) {
    c->t = h.t;
    c->nt = h.nt;
  }
  return VPM_OK;
}
