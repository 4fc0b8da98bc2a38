// RRTMG_SW host side: the shortwave tables (rrtmg_sw_init.f90) reduced to
// 112 g-points, uploaded in fp64 and fp32, and the launch of the column kernel
// (sw_kernel.cuh) in either precision.  This unit holds the fp64 kernels and is
// compiled without fp contraction, so that they round as the fp64 restatement
// does; the fp32 kernels are in sw_solver_f32.cu.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/gb_rrtmg_lw.h"
#include "lw_context.h"
#include "lw_tables.h"
#include "sw_kernel.cuh"
#include "sw_solver.h"

// ------------------------------------------------------------------ host side
namespace {

bool build_sw_tables(const char* path, double cpdair, gbsw::SwTab& S, std::vector<double>& blob, std::string& err) {
  std::map<std::string, GbTableEntry> tab;
  if (!gb_read_container(path, tab, err)) return false;
  auto need = [&](const std::string& n) -> const GbTableEntry* {
    auto it = tab.find(n);
    if (it == tab.end()) {
      err = "SW table file lacks " + n;
      return nullptr;
    }
    return &it->second;
  };
  auto put = [&](const std::string& n) -> int {  // append a float64 array, return its offset (-1 if absent)
    auto it = tab.find(n);
    if (it == tab.end() || it->second.is_int) return -1;
    const int off = (int)blob.size();
    blob.insert(blob.end(), it->second.d.begin(), it->second.d.end());
    return off;
  };
  std::memset(&S, 0, sizeof(S));
  const char* ints[] = {"ngc", "ngs", "ngb", "nspa", "nspb"};
  for (const char* n : ints)
    if (!need(n) || !need(n)->is_int) return false;
  const char* dbl[] = {"preflog", "tref", "wavenum2", "abari", "bbari", "cbari", "dbari", "ebari", "fbari", "grav",
                       "secdy", "avogad"};
  for (const char* n : dbl)
    if (!need(n)) return false;
  for (int k = 0; k < 59; ++k) {
    S.preflog[k] = tab["preflog"].d[k];
    S.tref[k] = tab["tref"].d[k];
  }
  for (int k = 0; k < gbsw::NB; ++k) {
    S.wavenum2[k] = tab["wavenum2"].d[k];
    S.nspa[k] = tab["nspa"].i[k];
    S.nspb[k] = tab["nspb"].i[k];
  }
  for (int g = 0; g < gbsw::NG; ++g) S.ngb[g] = tab["ngb"].i[g];
  for (int k = 0; k < 5; ++k) {
    S.abari[k] = tab["abari"].d[k];
    S.bbari[k] = tab["bbari"].d[k];
    S.cbari[k] = tab["cbari"].d[k];
    S.dbari[k] = tab["dbari"].d[k];
    S.ebari[k] = tab["ebari"].d[k];
    S.fbari[k] = tab["fbari"].d[k];
  }
  S.grav = tab["grav"].d[0];
  S.avogad = tab["avogad"].d[0];
  S.heatfac = S.grav * tab["secdy"].d[0] / (cpdair * 1.e2);  // rrtmg_sw_init.f90:259
  // exp_tbl (rrtmg_sw_init.f90:109-118), in double precision
  const int ntbl = 10000;
  const double expeps = 1.e-20, pade = 0.278;
  S.bpade = 1.0 / pade;
  S.exp_tbl = (int)blob.size();
  blob.resize(blob.size() + ntbl + 1);
  double* et = blob.data() + S.exp_tbl;
  et[0] = 1.0;
  et[ntbl] = expeps;
  for (int itr = 1; itr <= ntbl - 1; ++itr) {
    const double tfn = (double)itr / (double)ntbl;
    const double tau_tbl = S.bpade * tfn / (1.0 - tfn);
    et[itr] = std::exp(-tau_tbl);
    if (et[itr] <= expeps) et[itr] = expeps;
  }
  S.extliq1 = put("extliq1");
  S.ssaliq1 = put("ssaliq1");
  S.asyliq1 = put("asyliq1");
  S.extice2 = put("extice2");
  S.ssaice2 = put("ssaice2");
  S.asyice2 = put("asyice2");
  S.extice3 = put("extice3");
  S.ssaice3 = put("ssaice3");
  S.asyice3 = put("asyice3");
  S.fdlice3 = put("fdlice3");
  // co-albedo tables for the fp32 kernels: 1 - ssa formed in fp64, so that
  // near-conservative scattering keeps its absorption in fp32
  auto coalbedo = [&](const char* n) -> int {
    auto it = tab.find(n);
    if (it == tab.end() || it->second.is_int) return -1;
    const int off = (int)blob.size();
    for (double v : it->second.d) blob.push_back(1.0 - v);
    return off;
  };
  S.coaliq1 = coalbedo("ssaliq1");
  S.coaice2 = coalbedo("ssaice2");
  S.coaice3 = coalbedo("ssaice3");
  int g0 = 0;
  for (int k = 0; k < gbsw::NB; ++k) {
    const int b = k + 16;
    char pre[16];
    std::snprintf(pre, sizeof pre, "b%02d.", b);
    auto nm = [&](const char* s) { return std::string(pre) + s; };
    gbsw::SwBand& B = S.b[k];
    B.ng = tab["ngc"].i[k];
    B.g0 = g0;
    g0 += B.ng;
    B.absa = put(nm("absa"));
    B.absb = put(nm("absb"));
    B.absa_rows = B.absa >= 0 ? tab[nm("absa")].dims[0] : 0;
    B.absb_rows = B.absb >= 0 ? tab[nm("absb")].dims[0] : 0;
    B.selfref = put(nm("selfref"));
    B.forref = put(nm("forref"));
    B.nfor = B.forref >= 0 ? tab[nm("forref")].dims[0] : 0;
    B.sfluxref = put(nm("sfluxref"));
    B.rayl = put(nm("rayl"));
    B.rayl_per_g = B.rayl >= 0 && tab[nm("rayl")].ndim > 0;
    B.absch4 = put(nm("absch4"));
    B.abso3a = put(nm("abso3a"));
    B.abso3b = put(nm("abso3b"));
    B.rayla = put(nm("rayla"));
    B.raylb = put(nm("raylb"));
    B.absh2o = put(nm("absh2o"));
    B.absco2 = put(nm("absco2"));
    if (B.sfluxref < 0) {
      err = "SW table file lacks " + nm("sfluxref");
      return false;
    }
  }
  if (g0 != gbsw::NG) {
    err = "SW table file: g-point counts do not add up to 112";
    return false;
  }
  S.total = (int)blob.size();
  return true;
}

}  // namespace

int gb_sw_load(gb_lw_context* ctx, double cpdair, const char* table_dir) {
  std::string dir = table_dir ? table_dir : ctx->table_dir;
  const std::string path = dir + "/sw_tables.gbsw";
  std::vector<double> blob;
  gbsw::SwTab S;
  std::string err;
  if (!build_sw_tables(path.c_str(), cpdair, S, blob, err)) {
    ctx->last_error = err;
    return GB_LW_E_TABLES;
  }
  S.bpadef = (float)S.bpade;
  std::vector<float> blobf(blob.begin(), blob.end());  // the fp32 kernels' copy (every entry is within float range)
  cudaSetDevice(ctx->device);
  // the table directory is a constant block of the device: this context's
  // earlier hold (a repeated call) ends, and a new one must agree with the
  // other live contexts of the device
  ctx->sw_ready = false;
  if (ctx->sw_const_held) gb_const_release(GB_CONST_SW, ctx->device);
  ctx->sw_const_held = false;
  bool upload = false;
  if (!gb_const_acquire(GB_CONST_SW, ctx->device, &S, sizeof(S), &upload)) {
    ctx->last_error = "another context on this device holds different shortwave tables (cpdair or table files); "
                      "the contexts of a device must agree on them";
    return GB_LW_E_TABLES;
  }
  ctx->sw_const_held = true;
  cudaFree(ctx->d_sw_tables);
  cudaFree(ctx->d_sw_tables_f);
  ctx->d_sw_tables = nullptr;
  ctx->d_sw_tables_f = nullptr;
  auto drop_hold = [&]() {  // a failed load holds nothing (a later context uploads its own bytes)
    gb_const_release(GB_CONST_SW, ctx->device);
    ctx->sw_const_held = false;
  };
  if (cudaMalloc(&ctx->d_sw_tables, blob.size() * 8) != cudaSuccess ||
      cudaMalloc(&ctx->d_sw_tables_f, blobf.size() * 4) != cudaSuccess) {
    cudaGetLastError();
    drop_hold();
    ctx->last_error = "device allocation of the SW tables failed";
    return GB_LW_E_NOMEM;
  }
  cudaError_t e = cudaMemcpy(ctx->d_sw_tables, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ctx->d_sw_tables_f, blobf.data(), blobf.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && upload) e = gbsw::sw_set_tab(S);
  if (e == cudaSuccess && upload) e = gb_sw_set_tab_f32(&S);
  if (e != cudaSuccess) {
    drop_hold();
    return gb_ctx_fail(ctx, e, "SW tables");
  }
  std::map<std::string, GbTableEntry> tab;
  if (!gb_read_container(path.c_str(), tab, err) || !tab.count("rrsw_scon")) {
    ctx->last_error = "SW table file lacks rrsw_scon";
    return GB_LW_E_TABLES;
  }
  ctx->sw_scon = tab["rrsw_scon"].d[0];
  ctx->sw_ready = true;
  return GB_LW_OK;
}

size_t gb_sw_scratch_bytes(int nlay, int bits, long long slots) {
  return (size_t)slots * (size_t)gbsw::sw_slot_elems(nlay) * (bits == 32 ? sizeof(float) : sizeof(double));
}
long long gb_sw_slots(int num_sms, int bits) { return (long long)num_sms * (bits == 32 ? SW_MINB_F32 : SW_MINB_F64); }

cudaError_t gb_sw_launch(const SwArgs& a, int bits, const void* d_tables, void* scratch, long long slots,
                         cudaStream_t stream) {
  if (bits == 32) return gb_sw_launch_f32(a, (const float*)d_tables, (float*)scratch, slots, stream);
  return gbsw::sw_launch_t<double, SW_MINB_F64>(a, (const double*)d_tables, (double*)scratch, slots, stream);
}
