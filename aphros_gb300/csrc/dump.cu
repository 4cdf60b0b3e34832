// Field dumps of resident simulations in aphros's raw + XMF format: the
// binary array of dump::Raw (cells x-fastest, one element type, written from
// byte `seek` = 0; dump/raw.ipp:73-158) and the XDMF description beside it
// that dump::Raw::WriteWithXmf writes (dump/raw.ipp:204-226, text of
// dump/xmf.ipp:9-60 and :170-212).  Values are converted to the element type
// on the device and move to and from the host in chunks through the pinned
// staging buffer, so a 512^3 field needs no second full-size host copy.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace aphgpu {
namespace {

constexpr size_t kDumpChunk = size_t(1) << 23;  // elements per transfer

int Precision(int type) {
  return type == APHGPU_DUMP_UINT16 ? 2 : type == APHGPU_DUMP_FLOAT32 ? 4 : 8;
}

const char* TypeName(int type) {
  return type == APHGPU_DUMP_UINT16 ? "UShort" : type == APHGPU_DUMP_FLOAT32 ? "Float" : "Double";
}

bool ValidType(int type) {
  return type == APHGPU_DUMP_UINT16 || type == APHGPU_DUMP_FLOAT32 || type == APHGPU_DUMP_FLOAT64;
}

// A number as the reference's XMF writer prints it (a stream with
// precision 16 in the default float format, i.e. "%.16g").
std::string Num(double v) {
  char b[64];
  std::snprintf(b, sizeof(b), "%.16g", v);
  return b;
}

std::string Ints3(long long z, long long y, long long x) {
  return std::to_string(z) + " " + std::to_string(y) + " " + std::to_string(x);
}

// XMF of one cell-centred scalar field of an nx*ny*nz mesh with cubic cells
// of edge h and origin 0, stored whole (start 0, stride 1) from byte 0 of
// `binpath`.  Vector components are listed z, y, x as in the reference.
std::string XmfText(int nx, int ny, int nz, double h, const char* name, const char* binpath,
                    int type) {
  const std::string dims = Ints3(nz, ny, nx);
  std::string s;
  s += "<?xml version=\"1.0\" ?>\n";
  s += "<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n";
  s += "<Xdmf Version=\"2.0\">\n";
  s += "  <Domain>\n";
  s += "    <Grid Name=\"mesh\" GridType=\"Uniform\">\n";
  s += "      <Topology TopologyType=\"3DCORECTMesh\" Dimensions=\"" +
       Ints3(nz + 1, ny + 1, nx + 1) + "\"/>\n";
  s += "      <Geometry GeometryType=\"ORIGIN_DXDYDZ\">\n";
  s += "        <DataItem Name=\"Origin\" Dimensions=\"3\" NumberType=\"Float\" Precision=\"8\" "
       "Format=\"XML\">\n";
  s += "          " + Num(0.0) + " " + Num(0.0) + " " + Num(0.0) + "\n";
  s += "        </DataItem>\n";
  s += "        <DataItem Name=\"Spacing\" Dimensions=\"3\" NumberType=\"Float\" Precision=\"8\" "
       "Format=\"XML\">\n";
  s += "          " + Num(h) + " " + Num(h) + " " + Num(h) + "\n";
  s += "        </DataItem>\n";
  s += "      </Geometry>\n";
  s += std::string("      <Attribute Name=\"") + name + "\" AttributeType=\"Scalar\" Center=\"Cell\">\n";
  s += "        <DataItem ItemType=\"HyperSlab\" Dimensions=\"" + dims + "\" Type=\"HyperSlab\">\n";
  s += "          <DataItem Dimensions=\"3 3\" Format=\"XML\">\n";
  s += "            0 0 0\n";
  s += "            1 1 1\n";
  s += "            " + dims + "\n";
  s += "          </DataItem>\n";
  s += "          <DataItem Dimensions=\"" + dims + "\" Seek=\"0\" Precision=\"" +
       std::to_string(Precision(type)) + "\" NumberType=\"" + TypeName(type) +
       "\" Format=\"Binary\">\n";
  s += std::string("            ") + binpath + "\n";
  s += "          </DataItem>\n";
  s += "        </DataItem>\n";
  s += "      </Attribute>\n";
  s += "    </Grid>\n";
  s += "  </Domain>\n";
  s += "</Xdmf>\n";
  return s;
}

// value converted as C++ converts a double to the element type (round to
// nearest for float; truncation toward zero for uint16, where values outside
// [0, 65535], undefined in C++, are clamped)
__global__ void KToElem(int64_t n, const double* __restrict__ src, void* dst, int type) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = src[i];
    if (type == APHGPU_DUMP_FLOAT64) {
      static_cast<double*>(dst)[i] = v;
    } else if (type == APHGPU_DUMP_FLOAT32) {
      static_cast<float*>(dst)[i] = __double2float_rn(v);
    } else {
      const double t = v != v ? 0.0 : fmin(fmax(trunc(v), 0.0), 65535.0);
      static_cast<uint16_t*>(dst)[i] = (uint16_t)t;
    }
  }
}

__global__ void KFromElem(int64_t n, const void* __restrict__ src, double* dst, int type) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (type == APHGPU_DUMP_FLOAT64) {
      dst[i] = static_cast<const double*>(src)[i];
    } else if (type == APHGPU_DUMP_FLOAT32) {
      dst[i] = (double)static_cast<const float*>(src)[i];
    } else {
      dst[i] = (double)static_cast<const uint16_t*>(src)[i];
    }
  }
}

// Device array of a field id, or null with the error set.
double* FieldPtr(aphgpu_ctx* ctx, int field) {
  switch (field) {
    case APHGPU_FIELD_PRESSURE: return ctx->x;
    case APHGPU_FIELD_RHS: return ctx->has_system ? ctx->b : nullptr;
    case APHGPU_FIELD_VF: return ctx->vof_ready ? ctx->u : nullptr;
    case APHGPU_FIELD_CURVATURE: return ctx->vof_ready ? ctx->kappa : nullptr;
    default: return nullptr;
  }
}

// Scratch of the conversion kernels (one chunk of the widest element).
int DumpScratch(aphgpu_ctx* ctx, void** out) {
  if (!ctx->dump_scratch) {
    char* p = nullptr;
    APH_TRY(Alloc(ctx, &p, (int64_t)(8 * kDumpChunk)));
    ctx->dump_scratch = p;
  }
  *out = ctx->dump_scratch;
  return APHGPU_OK;
}

std::string WithoutExt(const std::string& path) {
  const size_t slash = path.find_last_of('/');
  const size_t dot = path.find_last_of('.');
  if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return path;
  return path.substr(0, dot);
}

// Text between the first `key` after `from` and the next quote.
bool Attr(const std::string& s, size_t from, const std::string& key, std::string* out) {
  const size_t a = s.find(key + "=\"", from);
  if (a == std::string::npos) return false;
  const size_t b = a + key.size() + 2;
  const size_t e = s.find('"', b);
  if (e == std::string::npos) return false;
  *out = s.substr(b, e - b);
  return true;
}

std::string Trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  const size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

}  // namespace
}  // namespace aphgpu

using namespace aphgpu;

extern "C" {

int aphgpu_xmf_text(int nx, int ny, int nz, double h, const char* name, const char* binpath,
                    int type, char* out, int cap, int* len) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !name || !binpath || !ValidType(type) || cap < 0)
    return APHGPU_ERR_ARG;
  const std::string s = XmfText(nx, ny, nz, h, name, binpath, type);
  if (len) *len = (int)s.size();
  if (out && cap > 0) {
    const size_t n = std::min(s.size(), (size_t)cap - 1);
    std::memcpy(out, s.data(), n);
    out[n] = 0;
  }
  return APHGPU_OK;
}

int aphgpu_dump_raw(aphgpu_ctx* ctx, int field, int type, const char* rawpath, const char* name) {
  if (!ctx || !ctx->stream || !rawpath || !name || !ValidType(type)) return APHGPU_ERR_ARG;
  double* src = FieldPtr(ctx, field);
  if (!src) return SetError(ctx, APHGPU_ERR_STATE, "field %d is not available", field);
  APH_CUDA(ctx, cudaSetDevice(ctx->device));
  const int64_t N = ctx->N;
  const size_t es = (size_t)Precision(type);
  void* scratch = nullptr;
  APH_TRY(DumpScratch(ctx, &scratch));
  void* stage = nullptr;
  APH_TRY(Staging(ctx, es * kDumpChunk, &stage));
  FILE* f = std::fopen(rawpath, "wb");
  if (!f) return SetError(ctx, APHGPU_ERR_ARG, "cannot open '%s' for writing", rawpath);
  int rc = APHGPU_OK;
  for (int64_t off = 0; off < N && rc == APHGPU_OK; off += (int64_t)kDumpChunk) {
    const int64_t n = std::min<int64_t>((int64_t)kDumpChunk, N - off);
    KToElem<<<FlatBlocks(n), kFlatThreads, 0, ctx->stream>>>(n, src + off, scratch, type);
    ctx->launches += 1;
    rc = CheckCuda(ctx, cudaGetLastError(), "dump conversion");
    if (rc == APHGPU_OK)
      rc = CheckCuda(ctx, cudaMemcpyAsync(stage, scratch, es * (size_t)n, cudaMemcpyDeviceToHost,
                                          ctx->stream), "dump copy");
    if (rc == APHGPU_OK) rc = CheckCuda(ctx, cudaStreamSynchronize(ctx->stream), "dump sync");
    if (rc == APHGPU_OK && std::fwrite(stage, es, (size_t)n, f) != (size_t)n)
      rc = SetError(ctx, APHGPU_ERR_ARG, "short write to '%s'", rawpath);
  }
  if (std::fclose(f) != 0 && rc == APHGPU_OK)
    rc = SetError(ctx, APHGPU_ERR_ARG, "cannot close '%s'", rawpath);
  if (rc != APHGPU_OK) return rc;
  const std::string xmfpath = WithoutExt(rawpath) + ".xmf";
  const std::string x = XmfText(ctx->d.nx, ctx->d.ny, ctx->d.nz, ctx->h, name, rawpath, type);
  FILE* g = std::fopen(xmfpath.c_str(), "wb");
  if (!g) return SetError(ctx, APHGPU_ERR_ARG, "cannot open '%s' for writing", xmfpath.c_str());
  const bool ok = std::fwrite(x.data(), 1, x.size(), g) == x.size();
  if (std::fclose(g) != 0 || !ok)
    return SetError(ctx, APHGPU_ERR_ARG, "cannot write '%s'", xmfpath.c_str());
  return APHGPU_OK;
}

int aphgpu_read_raw(aphgpu_ctx* ctx, int field, const char* xmfpath, const char* rawpath) {
  if (!ctx || !ctx->stream || !xmfpath) return APHGPU_ERR_ARG;
  double* dst = FieldPtr(ctx, field);
  if (!dst) return SetError(ctx, APHGPU_ERR_STATE, "field %d is not available", field);
  APH_CUDA(ctx, cudaSetDevice(ctx->device));
  // metadata (the subset of dump::Xmf::ReadXmf this reader supports: the
  // whole array from byte `seek`, start 0 and stride 1, as the reference's
  // sequential reader)
  std::string text;
  {
    FILE* f = std::fopen(xmfpath, "rb");
    if (!f) return SetError(ctx, APHGPU_ERR_ARG, "cannot open '%s'", xmfpath);
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    std::fclose(f);
  }
  const size_t attr = text.find("<Attribute");
  const size_t bin = text.find("Format=\"Binary\"", attr == std::string::npos ? 0 : attr);
  std::string dims, seek, prec, ntype;
  if (attr == std::string::npos || bin == std::string::npos)
    return SetError(ctx, APHGPU_ERR_ARG, "'%s': no binary attribute", xmfpath);
  const size_t item = text.rfind("<DataItem", bin);
  if (!Attr(text, item, "Dimensions", &dims) || !Attr(text, item, "Seek", &seek) ||
      !Attr(text, item, "Precision", &prec) || !Attr(text, item, "NumberType", &ntype))
    return SetError(ctx, APHGPU_ERR_ARG, "'%s': incomplete binary data item", xmfpath);
  const size_t body = text.find('>', bin) + 1;
  const std::string binpath = Trim(text.substr(body, text.find("</DataItem>", body) - body));
  const size_t slab = text.find("<DataItem Dimensions=\"3 3\"", attr);
  if (slab != std::string::npos) {
    const size_t b = text.find('>', slab) + 1;
    const std::string rows = text.substr(b, text.find("</DataItem>", b) - b);
    int v[9];
    if (std::sscanf(rows.c_str(), "%d %d %d %d %d %d %d %d %d", &v[0], &v[1], &v[2], &v[3],
                    &v[4], &v[5], &v[6], &v[7], &v[8]) != 9 ||
        v[0] || v[1] || v[2] || v[3] != 1 || v[4] != 1 || v[5] != 1)
      return SetError(ctx, APHGPU_ERR_UNSUPPORTED, "'%s': only start 0, stride 1", xmfpath);
  }
  int type = -1;
  if (ntype == "Double" && prec == "8") type = APHGPU_DUMP_FLOAT64;
  if (ntype == "Float" && prec == "4") type = APHGPU_DUMP_FLOAT32;
  if (ntype == "UShort" && prec == "2") type = APHGPU_DUMP_UINT16;
  if (type < 0) return SetError(ctx, APHGPU_ERR_ARG, "'%s': type %s/%s", xmfpath, ntype.c_str(),
                                prec.c_str());
  long long dz = 0, dy = 0, dx = 0;
  if (std::sscanf(dims.c_str(), "%lld %lld %lld", &dz, &dy, &dx) != 3 || dx != ctx->d.nx ||
      dy != ctx->d.ny || dz != ctx->d.nz)
    return SetError(ctx, APHGPU_ERR_ARG, "'%s': dimensions '%s' differ from the mesh", xmfpath,
                    dims.c_str());
  const long long off0 = std::atoll(seek.c_str());
  const std::string path = rawpath ? std::string(rawpath) : binpath;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return SetError(ctx, APHGPU_ERR_ARG, "cannot open '%s'", path.c_str());
  if (off0 < 0 || std::fseek(f, (long)off0, SEEK_SET) != 0) {
    std::fclose(f);
    return SetError(ctx, APHGPU_ERR_ARG, "'%s': cannot seek to %lld", path.c_str(), off0);
  }
  const int64_t N = ctx->N;
  const size_t es = (size_t)Precision(type);
  void* scratch = nullptr;
  void* stage = nullptr;
  int rc = DumpScratch(ctx, &scratch);
  if (rc == APHGPU_OK) rc = Staging(ctx, es * kDumpChunk, &stage);
  for (int64_t off = 0; off < N && rc == APHGPU_OK; off += (int64_t)kDumpChunk) {
    const int64_t n = std::min<int64_t>((int64_t)kDumpChunk, N - off);
    if (std::fread(stage, es, (size_t)n, f) != (size_t)n) {
      rc = SetError(ctx, APHGPU_ERR_ARG, "'%s': file shorter than the mesh", path.c_str());
      break;
    }
    rc = CheckCuda(ctx, cudaMemcpyAsync(scratch, stage, es * (size_t)n, cudaMemcpyHostToDevice,
                                        ctx->stream), "read copy");
    if (rc != APHGPU_OK) break;
    KFromElem<<<FlatBlocks(n), kFlatThreads, 0, ctx->stream>>>(n, scratch, dst + off, type);
    ctx->launches += 1;
    rc = CheckCuda(ctx, cudaGetLastError(), "read conversion");
    // the staging buffer is reused by the next chunk only after this copy
    if (rc == APHGPU_OK) rc = CheckCuda(ctx, cudaStreamSynchronize(ctx->stream), "read sync");
  }
  std::fclose(f);
  // a volume fraction read back gets its interface reconstructed (normals,
  // plane constants), as at aphgpu_vof_init; the step count is kept
  if (rc == APHGPU_OK && field == APHGPU_FIELD_VF) rc = VofReconstruct(ctx);
  return rc;
}

}  // extern "C"
