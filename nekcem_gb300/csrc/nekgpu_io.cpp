// Output of the GPU state: the reference's VTK legacy binary file
// (param(81) = 3, src/io.F:562-640 with src/io_vtkbin.c and the cell
// numbering of vtk_dump_header_nonswap, src/io_dumpvtk.F:718-810), and
// checkpoints of the device state for an exact resume.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "nekgpu_internal.h"

using namespace nekgpu;

struct nekgpu_ctx : public Context {};

namespace {

// big-endian 32-bit words (the reference swaps on little-endian hosts:
// swap_float_byte / swap_int_byte, src/io_util.c)
void put_be(std::vector<unsigned char>& b, uint32_t v) {
  b.push_back((unsigned char)(v >> 24));
  b.push_back((unsigned char)(v >> 16));
  b.push_back((unsigned char)(v >> 8));
  b.push_back((unsigned char)v);
}
void put_be_float(std::vector<unsigned char>& b, double d) {
  const float f = (float)d;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  put_be(b, u);
}
void put_text(std::vector<unsigned char>& b, const char* s) {
  b.insert(b.end(), s, s + std::strlen(s));
}

// VECTORS block: writefield (src/io_vtkbin.c:171-200), components of a node
// interleaved as vtk_nonswap_field packs them (src/io_dumpvtk.F:858-880)
void put_vectors(std::vector<unsigned char>& b, const char* name, const double* c0,
                 const double* c1, const double* c2, long n) {
  char line[128];
  std::snprintf(line, sizeof(line), "VECTORS %s ", name);
  put_text(b, line);
  put_text(b, " float \n");
  for (long i = 0; i < n; ++i) {
    put_be_float(b, c0[i]);
    put_be_float(b, c1[i]);
    put_be_float(b, c2[i]);
  }
  put_text(b, " \n");
}

int write_file(const char* path, const std::vector<unsigned char>& b) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return NEKGPU_ERR_ARG;
  const size_t w = std::fwrite(b.data(), 1, b.size(), f);
  const int cl = std::fclose(f);
  return (w == b.size() && cl == 0) ? NEKGPU_OK : NEKGPU_ERR_ARG;
}

struct CkHeader {
  char magic[8];
  int32_t version, form, nx1, npml;
  int64_t nelt, npts, aux_len, istep;
  double time;
  int64_t disp_len;  // 6 * nodes of the elements holding dispersive currents
};

}  // namespace

extern "C" int nekgpu_write_vtk(nekgpu_ctx* c, const char* path, const double* solhn,
                                const double* solen, long ld) {
  if (!c || !path || (solhn == nullptr) != (solen == nullptr) || (solhn && ld < c->npts))
    return NEKGPU_ERR_ARG;
  if (c->ndim == 2) return NEKGPU_ERR_UNSUPPORTED;  // hexahedral cells only
  if ((long)c->host_x.size() != c->npts || !c->have_state) return NEKGPU_ERR_STATE;
  const long P = c->npts;
  const int n = c->nx;
  std::vector<double> hn(3 * P), en(3 * P);
  int st = nekgpu_get_state(c, hn.data(), en.data(), P);
  if (st) return st;
  const long ncell = (long)(n - 1) * (n - 1) * (n - 1) * c->nelt;
  std::vector<unsigned char> b;
  b.reserve((size_t)(P * 12 * (solhn ? 5 : 3) + ncell * 40 + 512));
  // writeheader (src/io_vtkbin.c:54-71)
  put_text(b, "# vtk DataFile Version 2.0 \n");
  put_text(b, "Electromagnetic Field  \n");
  put_text(b, "BINARY \n");
  put_text(b, "DATASET UNSTRUCTURED_GRID \n");
  // writenodes (:73-95)
  char line[128];
  std::snprintf(line, sizeof(line), "POINTS  %ld ", P);
  put_text(b, line);
  put_text(b, " float  \n");
  for (long i = 0; i < P; ++i) {
    put_be_float(b, c->host_x[i]);
    put_be_float(b, c->host_y[i]);
    put_be_float(b, c->host_z[i]);
  }
  put_text(b, " \n");
  // write3dcells (:132-169) with the sub-hexahedra of vtk_dump_header_nonswap
  std::snprintf(line, sizeof(line), "CELLS %ld  %ld \n", ncell, 9 * ncell);
  put_text(b, line);
  const long n2 = (long)n * n, n3 = n2 * n;
  for (long e = 0; e < c->nelt; ++e)
    for (int j = 1; j < n; ++j) {
      long cnt = (j - 1) * n2 + e * n3;
      for (long i = 0; i < (long)(n - 1) * (n - 1); ++i) {
        const long v[4] = {cnt, cnt + 1, cnt + n + 1, cnt + n};
        put_be(b, 8);
        for (int q = 0; q < 4; ++q) put_be(b, (uint32_t)v[q]);
        for (int q = 0; q < 4; ++q) put_be(b, (uint32_t)(v[q] + n2));
        cnt = cnt + 1;
        if ((cnt + 1) % n == 0) cnt = cnt + 1;
      }
    }
  put_text(b, "\n");
  std::snprintf(line, sizeof(line), "CELL_TYPES %ld \n", ncell);
  put_text(b, line);
  for (long i = 0; i < ncell; ++i) put_be(b, 12);
  put_text(b, "\n");
  std::snprintf(line, sizeof(line), "POINT_DATA %ld \n", P);
  put_text(b, line);
  // cem_out_fields3: fields 1 "E ", 2 "H ", 3 "solE", 4 "solH" (getfieldname_)
  put_vectors(b, "E ", en.data(), en.data() + P, en.data() + 2 * P, P);
  put_vectors(b, "H ", hn.data(), hn.data() + P, hn.data() + 2 * P, P);
  if (solhn) {
    put_vectors(b, "solE", solen, solen + ld, solen + 2 * ld, P);
    put_vectors(b, "solH", solhn, solhn + ld, solhn + 2 * ld, P);
  }
  return write_file(path, b);
}

// ---- checkpoints -----------------------------------------------------------
// Raw device state: the fields, the RK register, (with PML) the auxiliary
// fields and (with dispersive media) the currents, each with its registers,
// as the context holds them; reloaded into a context of the same form, mesh
// and dispersive lists the run continues bit for bit.
namespace {

const double* state_ptr(Context* c) { return c->form == NEKGPU_PLAIN ? c->d_u[0] : c->d_u[c->cur]; }
long aux_len(const Context* c) {
  if (!c->npml) return 0;
  return (c->form == NEKGPU_PLAIN || c->ndim == 2) ? 6 * c->npts
                                                    : 6L * c->npml * c->nx * c->nx * c->nx;
}

}  // namespace

extern "C" int nekgpu_checkpoint_save(nekgpu_ctx* c, const char* path, double time, long istep) {
  if (!c || !path) return NEKGPU_ERR_ARG;
  if (!c->have_state) return NEKGPU_ERR_STATE;
  CkHeader h{};
  std::memcpy(h.magic, "NEKGPUCK", 8);
  h.version = 2;
  h.form = c->form;
  h.nx1 = c->nx;
  h.npml = c->npml;
  h.nelt = c->nelt;
  h.npts = c->npts;
  h.aux_len = aux_len(c);
  h.istep = istep;
  h.time = time;
  h.disp_len = 6 * c->disp_n;
  const long ns = 6 * c->npts;
  std::vector<double> buf(2 * ns + 2 * h.aux_len + 2 * h.disp_len);
  if (check_cuda(cudaStreamSynchronize(c->stream)) ||
      check_cuda(cudaMemcpy(buf.data(), state_ptr(c), ns * 8, cudaMemcpyDeviceToHost)) ||
      check_cuda(cudaMemcpy(buf.data() + ns, c->d_k, ns * 8, cudaMemcpyDeviceToHost)))
    return NEKGPU_ERR_CUDA;
  if (h.aux_len &&
      (check_cuda(cudaMemcpy(buf.data() + 2 * ns, c->d_pml_aux, h.aux_len * 8, cudaMemcpyDeviceToHost)) ||
       check_cuda(cudaMemcpy(buf.data() + 2 * ns + h.aux_len, c->d_pml_k, h.aux_len * 8,
                             cudaMemcpyDeviceToHost))))
    return NEKGPU_ERR_CUDA;
  double* dd = buf.data() + 2 * ns + 2 * h.aux_len;
  if (h.disp_len &&
      (check_cuda(cudaMemcpy(dd, c->d_disp_aux, h.disp_len * 8, cudaMemcpyDeviceToHost)) ||
       check_cuda(cudaMemcpy(dd + h.disp_len, c->d_disp_k, h.disp_len * 8, cudaMemcpyDeviceToHost))))
    return NEKGPU_ERR_CUDA;
  FILE* f = std::fopen(path, "wb");
  if (!f) return NEKGPU_ERR_ARG;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
            std::fwrite(buf.data(), 8, buf.size(), f) == buf.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? NEKGPU_OK : NEKGPU_ERR_ARG;
}

extern "C" int nekgpu_checkpoint_load(nekgpu_ctx* c, const char* path, double* time, long* istep) {
  if (!c || !path) return NEKGPU_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return NEKGPU_ERR_ARG;
  CkHeader h{};
  bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, "NEKGPUCK", 8) == 0 &&
            h.version == 2;
  if (ok && (h.form != c->form || h.nx1 != c->nx || h.nelt != c->nelt || h.npts != c->npts ||
             h.npml != c->npml || h.aux_len != aux_len(c) || h.disp_len != 6 * c->disp_n)) {
    std::fclose(f);
    return NEKGPU_ERR_MESH;  // a checkpoint of another mesh or form
  }
  const long ns = 6 * c->npts;
  std::vector<double> buf(ok ? 2 * ns + 2 * h.aux_len + 2 * h.disp_len : 0);
  ok = ok && std::fread(buf.data(), 8, buf.size(), f) == buf.size();
  std::fclose(f);
  if (!ok) return NEKGPU_ERR_ARG;
  if (check_cuda(cudaStreamSynchronize(c->stream)) ||
      check_cuda(cudaMemcpy(const_cast<double*>(state_ptr(c)), buf.data(), ns * 8,
                            cudaMemcpyHostToDevice)) ||
      check_cuda(cudaMemcpy(c->d_k, buf.data() + ns, ns * 8, cudaMemcpyHostToDevice)))
    return NEKGPU_ERR_CUDA;
  if (h.aux_len &&
      (check_cuda(cudaMemcpy(c->d_pml_aux, buf.data() + 2 * ns, h.aux_len * 8, cudaMemcpyHostToDevice)) ||
       check_cuda(cudaMemcpy(c->d_pml_k, buf.data() + 2 * ns + h.aux_len, h.aux_len * 8,
                             cudaMemcpyHostToDevice))))
    return NEKGPU_ERR_CUDA;
  const double* dd = buf.data() + 2 * ns + 2 * h.aux_len;
  if (h.disp_len &&
      (check_cuda(cudaMemcpy(c->d_disp_aux, dd, h.disp_len * 8, cudaMemcpyHostToDevice)) ||
       check_cuda(cudaMemcpy(c->d_disp_k, dd + h.disp_len, h.disp_len * 8, cudaMemcpyHostToDevice))))
    return NEKGPU_ERR_CUDA;
  c->have_state = true;
  if (time) *time = h.time;
  if (istep) *istep = h.istep;
  return NEKGPU_OK;
}
