// RRTMG_SW host side: the shortwave tables (rrtmg_sw_init.f90) reduced to
// 112 g-points, uploaded in fp64 and fp32, and the launch of the column kernel
// (sw_kernel.cuh) in either precision; and the band cloud optics cldprop_sw
// on the device.  This unit holds the fp64 kernels and is compiled without fp
// contraction, so that they round as the fp64 restatement does; the fp32
// kernels are in sw_solver_f32.cu.
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

// ------------------------------------------------------------------ cldprop_sw
// The band cloud optics of rrtmg_sw_cldprop.f90:53-365, which BRAMS computes
// per column and hands to mcica_subcol_sw (rtm_driver.f90:1356-1368).  One
// thread per (column, layer), fp64 with the reference's operations in its
// order; outputs (14, ld, nlay), band fastest.  A layer the reference would
// STOP on keeps the clear values (taucloud 0, ssacloud 1, asmcloud 0,
// taucldorig the input tauc) and gives its column the code of that STOP.
namespace gbsw {

struct CloudLay {  // one layer's ice or liquid optics option and table position
  int mode = 0;    // 0: none (zero path); ice 1, 2, 3: the ice option; liquid 1: liquid option 1
  double rad = 0.0, fint = 0.0;
  int index = 1;
};

// ice optics of band ib (16..29) for the layer's option; the STOP code of the
// band's checks in the reference's order (fdelta first for option 3), or 0
__device__ int ice_band(const double* __restrict__ T, const CloudLay& L, int ib, double& ext, double& ssa,
                        double& g, double& forw) {
  const double eps = 1.e-06;
  ext = ssa = g = forw = 0.0;
  if (L.mode == 0) return 0;
  auto c2 = [&](int off, int rows, int i) { return tb(T, off + (i - 1) + rows * (ib - 16)); };
  if (L.mode == 1) {
    const double w2 = c_S.wavenum2[ib - 16];
    const int icx = w2 > 1.43e04 ? 1 : w2 > 7.7e03 ? 2 : w2 > 5.3e03 ? 3 : w2 > 4.0e03 ? 4 : 5;
    ext = c_S.abari[icx - 1] + c_S.bbari[icx - 1] / L.rad;
    ssa = 1.0 - c_S.cbari[icx - 1] - c_S.dbari[icx - 1] * L.rad;
    g = c_S.ebari[icx - 1] + c_S.fbari[icx - 1] * L.rad;
    if (g >= 1.0) g = 1.0 - eps;
    forw = g * g;
  } else {
    const bool f3 = L.mode == 3;
    const int rows = f3 ? 46 : 43, i = L.index;
    const int oe = f3 ? c_S.extice3 : c_S.extice2, os = f3 ? c_S.ssaice3 : c_S.ssaice2,
              og = f3 ? c_S.asyice3 : c_S.asyice2;
    ext = c2(oe, rows, i) + L.fint * (c2(oe, rows, i + 1) - c2(oe, rows, i));
    ssa = c2(os, rows, i) + L.fint * (c2(os, rows, i + 1) - c2(os, rows, i));
    g = c2(og, rows, i) + L.fint * (c2(og, rows, i + 1) - c2(og, rows, i));
    if (f3) {
      const double fdelta = c2(c_S.fdlice3, 46, i) + L.fint * (c2(c_S.fdlice3, 46, i + 1) - c2(c_S.fdlice3, 46, i));
      if (fdelta < 0.0 || fdelta > 1.0) return GB_COL_SW_OPTICS;
      forw = fdelta + 0.5 / ssa;
      if (forw > g) forw = g;
    } else {
      forw = g * g;
    }
  }
  if (ext < 0.0 || ssa > 1.0 || ssa < 0.0 || g > 1.0 || g < 0.0) return GB_COL_SW_OPTICS;
  return 0;
}

// liquid optics (option 1) of band ib; the STOP code of its checks, or 0
__device__ int liq_band(const double* __restrict__ T, const CloudLay& L, int ib, double& ext, double& ssa,
                        double& g, double& forw) {
  ext = ssa = g = forw = 0.0;
  if (L.mode == 0) return 0;
  auto c2 = [&](int off, int i) { return tb(T, off + (i - 1) + 58 * (ib - 16)); };
  const int i = L.index;
  ext = c2(c_S.extliq1, i) + L.fint * (c2(c_S.extliq1, i + 1) - c2(c_S.extliq1, i));
  ssa = c2(c_S.ssaliq1, i) + L.fint * (c2(c_S.ssaliq1, i + 1) - c2(c_S.ssaliq1, i));
  if (L.fint < 0.0 && ssa > 1.0) ssa = c2(c_S.ssaliq1, i);
  g = c2(c_S.asyliq1, i) + L.fint * (c2(c_S.asyliq1, i + 1) - c2(c_S.asyliq1, i));
  forw = g * g;
  if (ext < 0.0 || ssa > 1.0 || ssa < 0.0 || g > 1.0 || g < 0.0) return GB_COL_SW_OPTICS;
  return 0;
}

__global__ void __launch_bounds__(128) cldprop_sw_kernel(CldpropSwArgs p, const double* __restrict__ T) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)p.ncol * p.nlay) return;
  const int lay = (int)(idx / p.ncol);
  const long long icol = idx - (long long)lay * p.ncol;
  const long long o = icol + p.ld * lay;
  const double cldmin = 1.e-20;
  auto in = [&](const double* v, int ib) { return v ? v[(ib - 16) + 14 * o] : 0.0; };
  double tauctot = 0.0;
  for (int ib = 16; ib <= 29; ++ib) tauctot = tauctot + in(p.tauc, ib);
  const double ci = p.ciwp[o], cl = p.clwp[o];
  const double cwp = ci + cl;
  const bool cloudy = p.cldfrac[o] >= cldmin && (cwp >= cldmin || tauctot >= cldmin);
  int lerr = 0;
  CloudLay ice, liq;
  if (cloudy && p.inflag == 2) {
    // the layer's options and the first STOP in the reference's order: the
    // ice radius, the ice bands, the liquid radius, the liquid bands
    if (ci != 0.0) {
      ice.rad = p.rei[o];
      if (p.iceflag == 1) {
        if (ice.rad < 13.0 || ice.rad > 130.0) lerr = GB_COL_ICE_BOUNDS;
        ice.mode = 1;
      } else if (p.iceflag == 2 || p.iceflag == 3) {
        const bool f3 = p.iceflag == 3;
        if (f3 ? (ice.rad < 5.0 || ice.rad > 140.0) : (ice.rad < 5.0 || ice.rad > 131.0))
          lerr = f3 ? GB_COL_DGE_BOUNDS : GB_COL_ICE_BOUNDS;
        const double factor = (ice.rad - 2.0) / 3.0;
        int index = (int)factor;
        if (index == (f3 ? 46 : 43)) index = f3 ? 45 : 42;
        ice.fint = factor - (double)index;
        const int top = f3 ? 45 : 42;
        ice.index = index < 1 ? 1 : (index > top ? top : index);  // in the table for any input
        ice.mode = p.iceflag;
      } else {
        lerr = GB_COL_SW_UNSUPPORTED;
      }
      double e, s, g, f;
      for (int ib = 16; ib <= 29 && !lerr; ++ib) lerr = ice_band(T, ice, ib, e, s, g, f);
    }
    if (!lerr && cl != 0.0) {
      if (p.liqflag == 1) {
        liq.rad = p.rel[o];
        if (liq.rad < 2.5 || liq.rad > 60.0) lerr = GB_COL_LIQ_BOUNDS;
        int index = (int)(liq.rad - 1.5);
        if (index == 0) index = 1;
        if (index == 58) index = 57;
        liq.fint = liq.rad - 1.5 - (double)index;
        liq.index = index < 1 ? 1 : (index > 57 ? 57 : index);  // in the table for any input
        liq.mode = 1;
        double e, s, g, f;
        for (int ib = 16; ib <= 29 && !lerr; ++ib) lerr = liq_band(T, liq, ib, e, s, g, f);
      } else {
        lerr = GB_COL_SW_UNSUPPORTED;
      }
    }
  }
  const bool work = cloudy && !lerr && (p.inflag == 0 || p.inflag == 2);
  for (int ib = 16; ib <= 29; ++ib) {
    double tco = in(p.tauc, ib), tcl = 0.0, ssa = 1.0, asy = 0.0;
    if (work && p.inflag == 0) {
      const double ffp = in(p.fsfc, ib);
      const double ffp1 = 1.0 - ffp;
      const double ffpssa = 1.0 - ffp * in(p.ssac, ib);
      ssa = ffp1 * in(p.ssac, ib) / ffpssa;
      tcl = ffpssa * tco;
      asy = (in(p.asmc, ib) - ffp) / (ffp1);
    } else if (work) {
      double extcoice, ssacoice, gice, forwice, extcoliq, ssacoliq, gliq, forwliq;
      ice_band(T, ice, ib, extcoice, ssacoice, gice, forwice);
      liq_band(T, liq, ib, extcoliq, ssacoliq, gliq, forwliq);
      const double tauliqorig = cl * extcoliq;
      const double tauiceorig = ci * extcoice;
      tco = tauliqorig + tauiceorig;
      const double ssaliq = ssacoliq * (1.0 - forwliq) / (1.0 - forwliq * ssacoliq);
      const double tauliq = (1.0 - forwliq * ssacoliq) * tauliqorig;
      const double ssaice = ssacoice * (1.0 - forwice) / (1.0 - forwice * ssacoice);
      const double tauice = (1.0 - forwice * ssacoice) * tauiceorig;
      const double scatliq = ssaliq * tauliq;
      double scatice = ssaice * tauice;
      tcl = tauliq + tauice;
      if (tcl == 0.0) tcl = cldmin;
      if (scatice == 0.0) scatice = cldmin;
      ssa = (scatliq + scatice) / tcl;
      if (p.iceflag == 3) {
        asy = (1.0 / (scatliq + scatice)) *
              (scatliq * (gliq - forwliq) / (1.0 - forwliq) + scatice * ((gice - forwice) / (1.0 - forwice)));
      } else {
        asy = (scatliq * (gliq - forwliq) / (1.0 - forwliq) + scatice * (gice - forwice) / (1.0 - forwice)) /
              (scatliq + scatice);
      }
    }
    const long long q = (ib - 16) + 14 * o;
    if (p.taucldorig) p.taucldorig[q] = tco;
    p.taucloud[q] = tcl;
    p.ssacloud[q] = ssa;
    p.asmcloud[q] = asy;
  }
  if (lerr) {
    if (p.col_err) atomicMax(p.col_err + icol, lerr);
    atomicMax(p.err_flag, lerr);
  }
}

}  // namespace gbsw

cudaError_t gb_cldprop_sw_launch(const CldpropSwArgs& a, const double* d_tables, cudaStream_t stream) {
  const long long n = (long long)a.ncol * a.nlay;
  if (n == 0) return cudaSuccess;
  const int threads = 128;
  gbsw::cldprop_sw_kernel<<<(int)((n + threads - 1) / threads), threads, 0, stream>>>(a, d_tables);
  return cudaGetLastError();
}
