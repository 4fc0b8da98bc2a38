// C ABI of the RRTMG_SW path (include/gb_rrtmg_lw.h): rrtmg_sw_ini and
// rrtmg_sw (rrtmg_sw_init.f90:47, rrtmg_sw_rad.f90:243) on device or host arrays.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "../../include/gb_rrtmg_lw.h"
#include "lw_context.h"
#include "lw_mcica.h"
#include "sw_solver.h"

namespace {

#define CKS(call)                                                    \
  do {                                                               \
    cudaError_t _e = (call);                                         \
    if (_e != cudaSuccess) return gb_ctx_fail(ctx, _e, #call);       \
  } while (0)

// earth_sun (rrtmg_sw_rad.f90:590-608)
double earth_sun(int idn) {
  const double pi = 2.0 * std::asin(1.0);
  const double gamma = 2.0 * pi * (idn - 1) / 365.0;
  return 1.000110 + .034221 * std::cos(gamma) + .001289 * std::sin(gamma) + .000719 * std::cos(2.0 * gamma) +
         .000077 * std::sin(2.0 * gamma);
}

// the driver's argument checks and clamps (rrtmg_sw_rad.f90:448-456) and the
// flux adjustment of inatm_sw for isolvar < 0 (:893-939)
int prepare(gb_lw_context* ctx, int ncol, int nlay, int* icld, int* iaer, double adjes, int dyofyr, double scon,
            int isolvar, int inflgsw, int iceflgsw, int liqflgsw, int64_t ld_in, int64_t ld_out, SwArgs& a) {
  if (!ctx || !icld || !iaer) return GB_LW_E_ARGS;
  if (!ctx->sw_ready) {
    ctx->last_error = "gb_rrtmg_sw_ini has not been called on this context";
    return GB_LW_E_ARGS;
  }
  if (*icld < 0 || *icld > 3) *icld = 2;
  if (*iaer != 0 && *iaer != 6 && *iaer != 10) *iaer = 0;
  if (ncol < 0 || nlay < 1 || nlay > GB_MAXLAY || ld_in < ncol || ld_out < ncol) return GB_LW_E_ARGS;
  if (inflgsw < 0 || inflgsw > 2 || iceflgsw < 0 || iceflgsw > 3 || liqflgsw < 0 || liqflgsw > 1) return GB_LW_E_ARGS;
  if (isolvar >= 0 || *iaer == 6) {
    ctx->last_error = "solar variability options isolvar >= 0 and aerosol option iaer = 6 are not implemented";
    return GB_LW_E_SW_UNSUPPORTED;
  }
  std::memset(&a, 0, sizeof(a));
  a.ncol = ncol;
  a.nlay = nlay;
  a.ld = ld_in;
  a.ldo = ld_out;
  a.icld = *icld;
  a.iaer = *iaer;
  a.inflag = inflgsw;
  a.iceflag = iceflgsw;
  a.liqflag = liqflgsw;
  double adjflx = adjes;
  if (dyofyr > 0) adjflx = earth_sun(dyofyr);
  const double solvar = scon > 0.0 ? scon / ctx->sw_scon : 1.0;
  for (int b = 0; b < 14; ++b) a.adjflux[b] = adjflx * solvar;
  return 0;
}

int launch(gb_lw_context* ctx, const SwArgs& a, cudaStream_t stream) {
  const int bits = ctx->sw_bits;
  const long long slots = gb_sw_slots(ctx->num_sms, bits);
  const size_t need = gb_sw_scratch_bytes(a.nlay, bits, slots);
  if (need > ctx->sw_scratch_bytes) {
    cudaFree(ctx->d_sw_scratch);
    ctx->d_sw_scratch = nullptr;
    ctx->sw_scratch_bytes = 0;
    if (cudaMalloc(&ctx->d_sw_scratch, need) != cudaSuccess) {
      cudaGetLastError();
      ctx->last_error = "device allocation of the SW scratch slots failed";
      return GB_LW_E_NOMEM;
    }
    ctx->sw_scratch_bytes = need;
  }
  const void* tables = bits == 32 ? (const void*)ctx->d_sw_tables_f : (const void*)ctx->d_sw_tables;
  cudaError_t e = gb_sw_launch(a, bits, tables, ctx->d_sw_scratch, slots, stream);
  return e == cudaSuccess ? GB_LW_OK : gb_ctx_fail(ctx, e, "SW column kernel");
}

}  // namespace

int gb_rrtmg_sw_ini(gb_lw_context* ctx, double cpdair, const char* table_dir) {
  if (!ctx) return GB_LW_E_ARGS;
  return gb_sw_load(ctx, cpdair, table_dir);
}

int gb_rrtmg_sw_set_precision(gb_lw_context* ctx, int bits) {
  if (!ctx || (bits != 32 && bits != 64)) return GB_LW_E_ARGS;
  ctx->sw_bits = bits;
  return GB_LW_OK;
}

int gb_rrtmg_sw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int* icld, int* iaer,
                       const double* play, const double* plev, const double* tlay, const double* tlev,
                       const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                       const double* ch4vmr, const double* n2ovmr, const double* o2vmr, const double* asdir,
                       const double* asdif, const double* aldir, const double* aldif, const double* coszen,
                       double adjes, int dyofyr, double scon, int isolvar, int inflgsw, int iceflgsw, int liqflgsw,
                       const double* cldfmcl, const double* taucmcl, const double* ssacmcl, const double* asmcmcl,
                       const double* fsfcmcl, const double* ciwpmcl, const double* clwpmcl, const double* reicmcl,
                       const double* relqmcl, const double* tauaer, const double* ssaaer, const double* asmaer,
                       const double* ecaer, double* swuflx, double* swdflx, double* swhr, double* swuflxc,
                       double* swdflxc, double* swhrc, int64_t ld_in, int64_t ld_out, int* d_col_status) {
  (void)tlev;
  (void)tsfc;
  (void)n2ovmr;
  (void)ecaer;
  SwArgs a;
  int rc = prepare(ctx, ncol, nlay, icld, iaer, adjes, dyofyr, scon, isolvar, inflgsw, iceflgsw, liqflgsw, ld_in,
                   ld_out, a);
  if (rc || ncol == 0) return rc;
  const double* req[] = {play, plev, tlay, h2ovmr, o3vmr, co2vmr, ch4vmr, o2vmr, asdir, asdif, aldir, aldif,
                         coszen, swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc};
  for (const double* p : req)
    if (!p) return GB_LW_E_ARGS;
  if (*icld >= 1 && (!cldfmcl || !taucmcl || !ssacmcl || !asmcmcl || !fsfcmcl || !ciwpmcl || !clwpmcl || !reicmcl ||
                     !relqmcl))
    return GB_LW_E_ARGS;
  if (*iaer == 10 && (!tauaer || !ssaaer || !asmaer)) return GB_LW_E_ARGS;
  a.play = play; a.plev = plev; a.tlay = tlay; a.h2ovmr = h2ovmr; a.o3vmr = o3vmr; a.co2vmr = co2vmr;
  a.ch4vmr = ch4vmr; a.o2vmr = o2vmr; a.asdir = asdir; a.asdif = asdif; a.aldir = aldir; a.aldif = aldif;
  a.coszen = coszen;
  a.cldfmcl = cldfmcl; a.taucmcl = taucmcl; a.ssacmcl = ssacmcl; a.asmcmcl = asmcmcl; a.fsfcmcl = fsfcmcl;
  a.ciwpmcl = ciwpmcl; a.clwpmcl = clwpmcl; a.reicmcl = reicmcl; a.relqmcl = relqmcl;
  a.tauaer = tauaer; a.ssaaer = ssaaer; a.asmaer = asmaer;
  a.swuflx = swuflx; a.swdflx = swdflx; a.swhr = swhr; a.swuflxc = swuflxc; a.swdflxc = swdflxc; a.swhrc = swhrc;
  a.col_err = d_col_status;
  a.err_flag = ctx->d_err;
  cudaSetDevice(ctx->device);
  return launch(ctx, a, (cudaStream_t)stream);
}

int gb_rrtmg_sw(gb_lw_context* ctx, int ncol, int nlay, int* icld, int* iaer, const double* play,
                const double* plev, const double* tlay, const double* tlev, const double* tsfc,
                const double* h2ovmr, const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                const double* n2ovmr, const double* o2vmr, const double* asdir, const double* asdif,
                const double* aldir, const double* aldif, const double* coszen, double adjes, int dyofyr,
                double scon, int isolvar, int inflgsw, int iceflgsw, int liqflgsw, const double* cldfmcl,
                const double* taucmcl, const double* ssacmcl, const double* asmcmcl, const double* fsfcmcl,
                const double* ciwpmcl, const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                const double* tauaer, const double* ssaaer, const double* asmaer, const double* ecaer,
                double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc, double* swhrc,
                int64_t ld_in, int64_t ld_out) {
  (void)ecaer;
  SwArgs a;
  int rc = prepare(ctx, ncol, nlay, icld, iaer, adjes, dyofyr, scon, isolvar, inflgsw, iceflgsw, liqflgsw, ld_in,
                   ld_out, a);
  if (rc || ncol == 0) return rc;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->streams[0];
  const size_t C = (size_t)ncol, L = (size_t)nlay, G = 112;
  const bool clouds = *icld >= 1, aer = *iaer == 10;
  // one device buffer for the call: inputs at leading dimension ncol, then outputs
  // (play, tlay and five gases by layer, plev by level, five surface arrays,
  // the clouds and aerosols when read, four level and two layer outputs)
  const size_t n = C * L * 7 + C * (L + 1) + C * 5 + (clouds ? G * C * L * 7 + 2 * C * L : 0) +
                   (aer ? 3 * C * L * 14 : 0) + 4 * C * (L + 1) + 2 * C * L;
  double* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    ctx->last_error = "device allocation for gb_rrtmg_sw failed";
    return GB_LW_E_NOMEM;
  }
  double* p = d;
  auto take = [&](size_t k) {
    double* r = p;
    p += k;
    if ((size_t)(p - d) > n) rc = GB_LW_E_ARGS;  // never copied to or launched on: checked before each use
    return r;
  };
  auto up = [&](const double* src, size_t width, size_t rows, size_t spitch) -> const double* {
    double* dst = take(width * rows);
    if (!rc && cudaMemcpy2DAsync(dst, width * 8, src, spitch * 8, width * 8, rows, cudaMemcpyHostToDevice, s) !=
                   cudaSuccess)
      rc = GB_LW_E_CUDA;
    return dst;
  };
  a.ld = (long long)C;
  a.ldo = (long long)C;
  a.play = up(play, C, L, ld_in);
  a.plev = up(plev, C, L + 1, ld_in);
  a.tlay = up(tlay, C, L, ld_in);
  a.h2ovmr = up(h2ovmr, C, L, ld_in);
  a.o3vmr = up(o3vmr, C, L, ld_in);
  a.co2vmr = up(co2vmr, C, L, ld_in);
  a.ch4vmr = up(ch4vmr, C, L, ld_in);
  a.o2vmr = up(o2vmr, C, L, ld_in);
  a.asdir = up(asdir, C, 1, C);
  a.asdif = up(asdif, C, 1, C);
  a.aldir = up(aldir, C, 1, C);
  a.aldif = up(aldif, C, 1, C);
  a.coszen = up(coszen, C, 1, C);
  if (clouds) {
    a.cldfmcl = up(cldfmcl, G * C, L, G * ld_in);
    a.taucmcl = up(taucmcl, G * C, L, G * ld_in);
    a.ssacmcl = up(ssacmcl, G * C, L, G * ld_in);
    a.asmcmcl = up(asmcmcl, G * C, L, G * ld_in);
    a.fsfcmcl = up(fsfcmcl, G * C, L, G * ld_in);
    a.ciwpmcl = up(ciwpmcl, G * C, L, G * ld_in);
    a.clwpmcl = up(clwpmcl, G * C, L, G * ld_in);
    a.reicmcl = up(reicmcl, C, L, ld_in);
    a.relqmcl = up(relqmcl, C, L, ld_in);
  }
  if (aer) {
    a.tauaer = up(tauaer, C, L * 14, ld_in);
    a.ssaaer = up(ssaaer, C, L * 14, ld_in);
    a.asmaer = up(asmaer, C, L * 14, ld_in);
  }
  a.swuflx = take(C * (L + 1));
  a.swdflx = take(C * (L + 1));
  a.swuflxc = take(C * (L + 1));
  a.swdflxc = take(C * (L + 1));
  a.swhr = take(C * L);
  a.swhrc = take(C * L);
  a.col_err = nullptr;
  a.err_flag = ctx->d_err_host;
  if (!rc) rc = cudaMemsetAsync(ctx->d_err_host, 0, 4, s) == cudaSuccess ? 0 : GB_LW_E_CUDA;
  if (!rc) rc = launch(ctx, a, s);
  auto down = [&](double* dst, const double* src, size_t rows) {
    if (cudaMemcpy2DAsync(dst, ld_out * 8, src, C * 8, C * 8, rows, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      rc = GB_LW_E_CUDA;
  };
  if (!rc) {
    down(swuflx, a.swuflx, L + 1);
    down(swdflx, a.swdflx, L + 1);
    down(swuflxc, a.swuflxc, L + 1);
    down(swdflxc, a.swdflxc, L + 1);
    down(swhr, a.swhr, L);
    down(swhrc, a.swhrc, L);
  }
  int h = 0;
  if (!rc && cudaMemcpyAsync(&h, ctx->d_err_host, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = GB_LW_E_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) rc = GB_LW_E_CUDA;
  cudaFree(d);
  if (rc) {
    if (ctx->last_error.empty()) ctx->last_error = cudaGetErrorString(cudaGetLastError());
    return rc;
  }
  return h;
}

// ---------------------------------------------------------------- mcica_subcol_sw
namespace {

// the shortwave g-point bands (rrtmg_sw_init.f90 swcmbdat ngb: 6, 12, 8, 8, 10,
// 10, 2, 10, 8, 6, 6, 8, 6, 12 g-points in bands 16..29)
void sw_ngb(int* ngb) {
  static const int ng[14] = {6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12};
  int k = 0;
  for (int b = 0; b < 14; ++b)
    for (int g = 0; g < ng[b]; ++g) ngb[k++] = 16 + b;
}

}  // namespace

int gb_mcica_subcol_sw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int icld, int permuteseed,
                              int* irng, const double* play, const double* cldfrac, const double* ciwp,
                              const double* clwp, const double* rei, const double* rel, const double* tauc,
                              const double* ssac, const double* asmc, const double* fsfc, const double* alpha,
                              double* cldfmcl, double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl,
                              double* taucmcl, double* ssacmcl, double* asmcmcl, double* fsfcmcl, int64_t ld,
                              int seed_per_column) {
  if (!ctx || !irng) return GB_LW_E_ARGS;
  if (icld == 0) return GB_LW_OK;  // mcica_subcol_gen_sw.f90:264
  if (icld < 0 || icld > 5) return GB_LW_E_ICLD;
  if (ncol < 0 || nlay < 1 || ld < ncol) return GB_LW_E_ARGS;
  if (*irng != 0) *irng = 1;
  if (icld >= 4 && !alpha) return GB_LW_E_ARGS;
  if (*irng == 0 && nlay < 4) return GB_LW_E_ARGS;
  const double* req[] = {play, cldfrac, ciwp, clwp, rei, rel, tauc, ssac, asmc, fsfc};
  for (const double* p : req)
    if (!p) return GB_LW_E_ARGS;
  double* outs[] = {cldfmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl};
  for (double* p : outs)
    if (!p) return GB_LW_E_ARGS;
  if (ncol == 0) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  const size_t need = gb_mcica_draw_count(ncol, nlay, icld, SW_NGPT);
  if (need > ctx->draws_elems) {
    cudaFree(ctx->d_draws);
    ctx->d_draws = nullptr;
    ctx->draws_elems = 0;
    if (cudaMalloc(&ctx->d_draws, need * 8) != cudaSuccess) {
      cudaGetLastError();
      return GB_LW_E_NOMEM;
    }
    ctx->draws_elems = need;
  }
  McicaArgs a{};
  a.mode = *irng == 0 ? MCICA_PERCOL_KISS : (seed_per_column ? MCICA_PERCOL_MT : MCICA_STREAM_MT);
  a.ncol = ncol;
  a.nlay = nlay;
  a.icld = icld;
  a.seed = permuteseed;
  a.ncol_call = seed_per_column ? 1 : ncol;
  a.ld = ld;
  a.play = play; a.cldfrac = cldfrac; a.ciwp = ciwp; a.clwp = clwp; a.rei = rei; a.rel = rel;
  a.tauc = tauc; a.alpha = alpha;
  a.cldfmcl = cldfmcl; a.ciwpmcl = ciwpmcl; a.clwpmcl = clwpmcl; a.taucmcl = taucmcl;
  a.reicmcl = reicmcl; a.relqmcl = relqmcl;
  a.nsub = SW_NGPT;
  a.nbnd = 14;
  a.band0 = 15;
  a.ssac = ssac; a.asmc = asmc; a.fsfc = fsfc;
  a.ssacmcl = ssacmcl; a.asmcmcl = asmcmcl; a.fsfcmcl = fsfcmcl;
  sw_ngb(a.ngb);
  CKS(gb_mcica_launch(a, ctx->d_draws, ctx->d_err, (cudaStream_t)stream, seed_per_column != 0));
  return GB_LW_OK;
}

int gb_mcica_subcol_sw(gb_lw_context* ctx, int ncol, int nlay, int icld, int permuteseed, int* irng,
                       const double* play, const double* cldfrac, const double* ciwp, const double* clwp,
                       const double* rei, const double* rel, const double* tauc, const double* ssac,
                       const double* asmc, const double* fsfc, const double* alpha, double* cldfmcl,
                       double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl, double* taucmcl,
                       double* ssacmcl, double* asmcmcl, double* fsfcmcl, int64_t ld, int seed_per_column) {
  if (!ctx || !irng) return GB_LW_E_ARGS;
  if (icld == 0) return GB_LW_OK;
  if (icld < 0 || icld > 5) return GB_LW_E_ICLD;
  if (ncol < 0 || nlay < 1 || ld < ncol) return GB_LW_E_ARGS;
  if (ncol == 0) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->streams[0];
  const size_t C = (size_t)ncol, L = (size_t)nlay, n2 = C * L, nm = (size_t)SW_NGPT * n2, nb = 14 * n2;
  // inputs: 7 layer arrays (play, cldfrac, ciwp, clwp, rei, rel, alpha), 4 band
  // arrays (tauc, ssac, asmc, fsfc); outputs: 7 sub-column arrays and 2 radii
  const size_t total = 7 * n2 + 4 * nb + 7 * nm + 2 * n2;
  double* d = nullptr;
  if (cudaMalloc(&d, total * 8) != cudaSuccess) {
    cudaGetLastError();
    return GB_LW_E_NOMEM;
  }
  double* lay[7];
  for (int k = 0; k < 7; ++k) lay[k] = d + k * n2;
  double* band[4];
  for (int k = 0; k < 4; ++k) band[k] = d + 7 * n2 + k * nb;
  double* sub[7];
  for (int k = 0; k < 7; ++k) sub[k] = d + 7 * n2 + 4 * nb + k * nm;
  double* rad[2] = {d + 7 * n2 + 4 * nb + 7 * nm, d + 7 * n2 + 4 * nb + 7 * nm + n2};
  int rc = GB_LW_OK;
  auto h2d = [&](double* dst, const double* src, size_t w, size_t spitch) {
    if (!rc && cudaMemcpy2DAsync(dst, w * 8, src, spitch * 8, w * 8, L, cudaMemcpyHostToDevice, s) != cudaSuccess)
      rc = gb_ctx_fail(ctx, cudaGetLastError(), "mcica_sw H2D");
  };
  const double* lin[6] = {play, cldfrac, ciwp, clwp, rei, rel};
  for (int k = 0; k < 6; ++k) h2d(lay[k], lin[k], C, (size_t)ld);
  if (alpha) h2d(lay[6], alpha, C, (size_t)ld);
  const double* bin[4] = {tauc, ssac, asmc, fsfc};
  for (int k = 0; k < 4; ++k) h2d(band[k], bin[k], 14 * C, 14 * (size_t)ld);
  if (!rc)
    rc = gb_mcica_subcol_sw_device(ctx, s, ncol, nlay, icld, permuteseed, irng, lay[0], lay[1], lay[2], lay[3],
                                   lay[4], lay[5], band[0], band[1], band[2], band[3], alpha ? lay[6] : nullptr,
                                   sub[0], sub[1], sub[2], rad[0], rad[1], sub[3], sub[4], sub[5], sub[6], ncol,
                                   seed_per_column);
  auto d2h = [&](double* dst, const double* src, size_t w, size_t dpitch) {
    if (!rc && cudaMemcpy2DAsync(dst, dpitch * 8, src, w * 8, w * 8, L, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      rc = gb_ctx_fail(ctx, cudaGetLastError(), "mcica_sw D2H");
  };
  double* hout[7] = {cldfmcl, ciwpmcl, clwpmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl};
  for (int k = 0; k < 7; ++k) d2h(hout[k], sub[k], (size_t)SW_NGPT * C, (size_t)SW_NGPT * ld);
  d2h(reicmcl, rad[0], C, (size_t)ld);
  d2h(relqmcl, rad[1], C, (size_t)ld);
  cudaError_t e = cudaStreamSynchronize(s);
  if (!rc && e != cudaSuccess) rc = gb_ctx_fail(ctx, e, "mcica_sw sync");
  if (!rc) {
    int h = 0;
    cudaMemcpy(&h, ctx->d_err, 4, cudaMemcpyDeviceToHost);
    cudaMemset(ctx->d_err, 0, 4);
    rc = h;
  }
  cudaFree(d);
  return rc;
}

int gb_cldprop_sw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int inflag, int iceflag, int liqflag,
                         const double* cldfrac, const double* tauc, const double* ssac, const double* asmc,
                         const double* fsfc, const double* ciwp, const double* clwp, const double* rei,
                         const double* rel, double* taucloud, double* ssacloud, double* asmcloud, double* taucldorig,
                         int64_t ld, int* d_col_status) {
  if (!ctx || ncol < 0 || nlay < 1 || nlay > GB_MAXLAY || ld < ncol || inflag < 0 || inflag > 2 || iceflag < 0 ||
      iceflag > 3 || liqflag < 0 || liqflag > 1 || !cldfrac || !ciwp || !clwp || !rei || !rel || !taucloud ||
      !ssacloud || !asmcloud || (inflag == 0 && (!tauc || !ssac || !asmc || !fsfc)))
    return GB_LW_E_ARGS;
  if (!ctx->sw_ready) {
    ctx->last_error = "gb_rrtmg_sw_ini has not been called on this context";
    return GB_LW_E_ARGS;
  }
  if (ncol == 0) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = d_col_status ? cudaMemsetAsync(d_col_status, 0, sizeof(int) * (size_t)ncol, st) : cudaSuccess;
  if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "cldprop_sw status");
  CldpropSwArgs a;
  a.ncol = ncol;
  a.nlay = nlay;
  a.ld = ld;
  a.inflag = inflag;
  a.iceflag = iceflag;
  a.liqflag = liqflag;
  a.cldfrac = cldfrac;
  a.tauc = tauc;
  a.ssac = ssac;
  a.asmc = asmc;
  a.fsfc = fsfc;
  a.ciwp = ciwp;
  a.clwp = clwp;
  a.rei = rei;
  a.rel = rel;
  a.taucldorig = taucldorig;
  a.taucloud = taucloud;
  a.ssacloud = ssacloud;
  a.asmcloud = asmcloud;
  a.col_err = d_col_status;
  a.err_flag = ctx->d_err;
  e = gb_cldprop_sw_launch(a, ctx->d_sw_tables, st);
  if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "cldprop_sw launch");
  return GB_LW_OK;
}
