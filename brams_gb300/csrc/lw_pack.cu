// BRAMS model state -> rrtmg_lw column inputs, and the heating rates back
// into the model's theta tendency, on the device: the column packing and
// write-back of radrrtmdrv (src/brams/radiate/rtm_driver.f90:978-1231 and
// :1443-1456), so that a model whose fields live on the GPU feeds the
// solver and takes its tendency without a host round trip.
//
// One thread per column (j outer, i inner, the driver's order), walking the
// column's levels.  BRAMS fields and constants are default real (float32);
// each statement mixes them with real(8) as the driver does: float32
// operations round to float32 before they meet a double.  The unit is
// compiled without multiply-add contraction, so every operation rounds as
// the driver's.  Ozone, aerosols and the chemistry-coupled gas paths stay
// with the caller (they come from the ozone climatology and CARMA).
#include <cuda_runtime.h>
#include <stdint.h>

#include "lw_context.h"

namespace gbpk {

// rconstants.f90:15-46 (default real); mem_rrtm.f90:13-23 (real(8))
constexpr float kCp = 1004.0f, kRgas = 287.0f, kP00 = 1.0e5f, kStefan = 5.6696e-8f;
constexpr double kAdjust = 0.01;  // Pa -> hPa
constexpr double kPmAr = 28.96;

struct PackArgs {
  int mzp, mxp, myp, ia, ja, ni, ncol, iceflg, firsttime;
  long long ld;
  float cpor, cpi;
  const float *pi0, *pp, *theta, *rv, *rlongup, *albedt, *cldf, *lwl, *iwl, *rel, *rei;
  double *play, *plev, *tlay, *tlev, *tsfc, *h2ovmr, *co2, *ch4, *n2o, *o2, *cfc11, *cfc12, *cfc22, *ccl4, *emis,
      *cldfrac, *ciwp, *clwp, *reic, *relq;
};

__global__ void __launch_bounds__(128) pack_kernel(PackArgs a) {
  const int noc = blockIdx.x * blockDim.x + threadIdx.x;
  if (noc >= a.ncol) return;
  const int i = a.ia - 1 + noc % a.ni, j = a.ja - 1 + noc / a.ni;  // zero-based grid point
  const long long c3 = (long long)a.mzp * ((long long)i + (long long)a.mxp * j);
  const long long c2 = (long long)i + (long long)a.mxp * j;
  const int nlay = a.mzp - 1;
  const long long ld = a.ld;
  auto at = [&](double* p, int l) -> double& { return p[noc + ld * l]; };
  // :990 surface temperature from the upward longwave flux; :997 emissivity
  // (left at 0 on the driver's first call); :1001-1003 surface pressure
  at(a.tsfc, 0) = pow((double)(a.rlongup[c2] / kStefan), 0.25);
  const double em = a.firsttime ? 0.0 : (double)(1.0f - a.albedt[c2]);
  for (int b = 0; b < 16; ++b) at(a.emis, b) = em;
  const float e0 = a.pi0[c3] + a.pp[c3], e1 = a.pi0[c3 + 1] + a.pp[c3 + 1];
  const float ps = (((a.pi0[c3] + a.pp[c3]) + a.pi0[c3 + 1]) + a.pp[c3 + 1]) * a.cpi * 0.5f;
  const double psurf = ((double)kP00 * pow((double)ps, (double)a.cpor)) * kAdjust;
  // :1018-1043 layer k-1 from model level k (zero-based: layer L from level
  // L+1), then :1052-1061 layer and interior interface values
  double p_prev = 0.0, t_prev = 0.0, plev_n1 = 0.0, plev_n2 = 0.0, tlev_n1 = 0.0, tlev_n2 = 0.0, play_top = 0.0;
  for (int L = 0; L < nlay; ++L) {
    const long long o = c3 + L + 1;
    const double picpi = (double)((a.pi0[o] + a.pp[o]) * a.cpi);
    const double p = ((double)kP00 * pow(picpi, (double)a.cpor)) * kAdjust;
    const double t = (double)a.theta[o] * picpi;
    at(a.play, L) = p;
    at(a.tlay, L) = t;
    if (L >= 1) {
      const double pl = (p + p_prev) * 0.5, tl = (t + t_prev) * 0.5;
      at(a.plev, L) = pl;
      at(a.tlev, L) = tl;
      plev_n2 = plev_n1, plev_n1 = pl;
      tlev_n2 = tlev_n1, tlev_n1 = tl;
    }
    p_prev = p, t_prev = t, play_top = p;
    // :1224 vapour of layer L is q of layer L+1 (the top layer repeats the
    // last model level, :1045)
    const int lq = L + 2 < a.mzp ? L + 2 : a.mzp - 1;
    at(a.h2ovmr, L) = (double)a.rv[c3 + lq] * (1.0 / (18.01528 / kPmAr));
    at(a.cldfrac, L) = (double)a.cldf[o];
    at(a.clwp, L) = (double)a.lwl[o];
    at(a.ciwp, L) = (double)a.iwl[o];
    at(a.relq, L) = (double)a.rel[o];
    const float r = a.rei[o];
    float ri = 0.0f;  // the driver leaves reic at 0 for other ice options
    if (a.iceflg == 1) ri = fminf(130.0f, fmaxf(13.0f, r));
    else if (a.iceflg == 2) ri = fminf(131.0f, fmaxf(5.0f, r));
    else if (a.iceflg == 3) ri = fminf(140.0f, fmaxf(5.0f, 0.9021f * r - 7.0365f));
    at(a.reic, L) = (double)ri;
    // :1176-1231 fixed gases (single-precision literals times real(8) ratios)
    at(a.co2, L) = (double)379.0e-6f * (1.0 / (44.01 / kPmAr));
    at(a.ch4, L) = (double)1774.0e-9f * (1.0 / (16.04 / kPmAr));
    at(a.n2o, L) = (double)319.0e-9f * (1.0 / (46.0055 / kPmAr));
    at(a.o2, L) = (double)0.209488f * (1.0 / (64.0 / kPmAr));
    at(a.cfc11, L) = (double)0.251e-9f;
    at(a.cfc12, L) = (double)0.538e-9f;
    at(a.cfc22, L) = (double)0.169e-9f;
    at(a.ccl4, L) = (double)0.093e-9f;
  }
  // :1063-1069 surface interface; :1072-1076 top interface extrapolated
  at(a.plev, 0) = psurf;
  const float th0 = a.theta[c3], th1 = a.theta[c3 + 1];
  const float tl0 = 0.5f * ((th0 * e0) * a.cpi + (th1 * e1) * a.cpi);
  at(a.tlev, 0) = (double)tl0;
  if (nlay == 2) {  // the interface below the top one is the surface
    plev_n2 = psurf;
    tlev_n2 = (double)tl0;
  }
  const double ptop = plev_n1 - 2.0 * (plev_n1 - play_top);
  at(a.plev, nlay) = ptop;
  at(a.tlev, nlay) = tlev_n1 + (tlev_n1 - tlev_n2) / (plev_n1 - plev_n2) * (ptop - plev_n1);
}

struct UnpackArgs {
  int mzp, mxp, ia, ja, ni, ncol;
  long long ld_hr, ld_flx;
  const double *hr, *swhr, *dflx;
  float *fthrd, *rlong;
};

// :1446-1456: rlong from the surface downward flux; fthrd(k) = (swhr + hr)
// of layer k-1 / 86400 for k = 2..mzp-1, copied to the bottom and top levels
__global__ void __launch_bounds__(128) unpack_kernel(UnpackArgs a) {
  const int noc = blockIdx.x * blockDim.x + threadIdx.x;
  if (noc >= a.ncol) return;
  const int i = a.ia - 1 + noc % a.ni, j = a.ja - 1 + noc / a.ni;
  const long long c3 = (long long)a.mzp * ((long long)i + (long long)a.mxp * j);
  a.rlong[(long long)i + (long long)a.mxp * j] = (float)a.dflx[noc];
  float f = 0.0f;
  for (int k = 1; k <= a.mzp - 2; ++k) {
    const long long o = noc + a.ld_hr * (k - 1);
    f = (float)(((a.swhr ? a.swhr[o] : 0.0) + a.hr[o]) / (double)86400.0f);
    a.fthrd[c3 + k] = f;
    if (k == 1) a.fthrd[c3] = f;
  }
  a.fthrd[c3 + a.mzp - 1] = f;
}

// the shortwave-only inputs and output of the same loops: coszen and the
// four albedos per packed column (:989, :992-996; the albedos stay 0 on the
// first call, as allocated at :933-936), and rshort from the surface
// downward shortwave flux, 0 below 0.5 W m-2 (:1448-1449)
struct PackSwArgs {
  int mxp, ia, ja, ni, ncol, firsttime;
  const float *cosz, *albedt;
  double *coszen, *asdir, *asdif, *aldir, *aldif;
};
__global__ void __launch_bounds__(128) pack_sw_kernel(PackSwArgs a) {
  const int noc = blockIdx.x * blockDim.x + threadIdx.x;
  if (noc >= a.ncol) return;
  const long long c2 = (long long)(a.ia - 1 + noc % a.ni) + (long long)a.mxp * (a.ja - 1 + noc / a.ni);
  a.coszen[noc] = (double)a.cosz[c2];
  const double al = a.firsttime ? 0.0 : (double)a.albedt[c2];
  a.asdir[noc] = al;
  a.aldir[noc] = al;
  a.asdif[noc] = al;
  a.aldif[noc] = al;
}

struct UnpackSwArgs {
  int mxp, ia, ja, ni, ncol;
  const double* swdflx;
  float* rshort;
};
__global__ void __launch_bounds__(128) unpack_sw_kernel(UnpackSwArgs a) {
  const int noc = blockIdx.x * blockDim.x + threadIdx.x;
  if (noc >= a.ncol) return;
  const long long c2 = (long long)(a.ia - 1 + noc % a.ni) + (long long)a.mxp * (a.ja - 1 + noc / a.ni);
  const double f = a.swdflx[noc];
  a.rshort[c2] = f < 0.5 ? 0.0f : (float)f;
}

bool box_ok(int mzp, int mxp, int myp, int ia, int iz, int ja, int jz) {
  return mzp >= 3 && mxp >= 1 && myp >= 1 && ia >= 1 && iz >= ia && iz <= mxp && ja >= 1 && jz >= ja && jz <= myp &&
         (long long)(iz - ia + 1) * (jz - ja + 1) <= 0x7FFFFFFFLL;
}

}  // namespace gbpk

int gb_rtm_pack_lw_device(gb_lw_context* ctx, void* stream, int mzp, int mxp, int myp, int ia, int iz, int ja, int jz,
                          int iceflgsw, int firsttime, const float* pi0, const float* pp, const float* theta,
                          const float* rv, const float* rlongup, const float* albedt, const float* cldf,
                          const float* lwl, const float* iwl, const float* rel, const float* rei, double* play,
                          double* plev, double* tlay, double* tlev, double* tsfc, double* h2ovmr, double* co2vmr,
                          double* ch4vmr, double* n2ovmr, double* o2vmr, double* cfc11vmr, double* cfc12vmr,
                          double* cfc22vmr, double* ccl4vmr, double* emis, double* cldfrac, double* ciwp,
                          double* clwp, double* reic, double* relq, int64_t ld) {
  if (!ctx || !gbpk::box_ok(mzp, mxp, myp, ia, iz, ja, jz)) return GB_LW_E_ARGS;
  const int ni = iz - ia + 1, ncol = ni * (jz - ja + 1);
  if (mzp - 1 > GB_MAXLAY || ld < ncol) return GB_LW_E_ARGS;
  const void* in[] = {pi0, pp, theta, rv, rlongup, albedt, cldf, lwl, iwl, rel, rei};
  const void* out[] = {play, plev, tlay, tlev, tsfc, h2ovmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr,
                       cfc12vmr, cfc22vmr, ccl4vmr, emis, cldfrac, ciwp, clwp, reic, relq};
  for (const void* p : in)
    if (!p) return GB_LW_E_ARGS;
  for (const void* p : out)
    if (!p) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  gbpk::PackArgs a{};
  a.mzp = mzp, a.mxp = mxp, a.myp = myp, a.ia = ia, a.ja = ja, a.ni = ni, a.ncol = ncol;
  a.iceflg = iceflgsw, a.firsttime = firsttime != 0, a.ld = ld;
  a.cpor = gbpk::kCp / gbpk::kRgas;  // default-real cp/rgas and 1/cp, as rconstants.f90:43-45
  a.cpi = 1.0f / gbpk::kCp;
  a.pi0 = pi0, a.pp = pp, a.theta = theta, a.rv = rv, a.rlongup = rlongup, a.albedt = albedt;
  a.cldf = cldf, a.lwl = lwl, a.iwl = iwl, a.rel = rel, a.rei = rei;
  a.play = play, a.plev = plev, a.tlay = tlay, a.tlev = tlev, a.tsfc = tsfc, a.h2ovmr = h2ovmr;
  a.co2 = co2vmr, a.ch4 = ch4vmr, a.n2o = n2ovmr, a.o2 = o2vmr, a.cfc11 = cfc11vmr, a.cfc12 = cfc12vmr;
  a.cfc22 = cfc22vmr, a.ccl4 = ccl4vmr, a.emis = emis, a.cldfrac = cldfrac, a.ciwp = ciwp, a.clwp = clwp;
  a.reic = reic, a.relq = relq;
  gbpk::pack_kernel<<<(ncol + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GB_LW_OK : gb_ctx_fail(ctx, e, "column packing launch");
}

int gb_rtm_unpack_lw_device(gb_lw_context* ctx, void* stream, int mzp, int mxp, int myp, int ia, int iz, int ja,
                            int jz, const double* hr, const double* swhr, const double* dflx, int64_t ld_hr,
                            int64_t ld_flx, float* fthrd, float* rlong) {
  if (!ctx || !gbpk::box_ok(mzp, mxp, myp, ia, iz, ja, jz) || !hr || !dflx || !fthrd || !rlong) return GB_LW_E_ARGS;
  const int ni = iz - ia + 1, ncol = ni * (jz - ja + 1);
  if (ld_hr < ncol || ld_flx < ncol) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  gbpk::UnpackArgs a{};
  a.mzp = mzp, a.mxp = mxp, a.ia = ia, a.ja = ja, a.ni = ni, a.ncol = ncol;
  a.ld_hr = ld_hr, a.ld_flx = ld_flx, a.hr = hr, a.swhr = swhr, a.dflx = dflx, a.fthrd = fthrd, a.rlong = rlong;
  gbpk::unpack_kernel<<<(ncol + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GB_LW_OK : gb_ctx_fail(ctx, e, "tendency write-back launch");
}

int gb_rtm_pack_sw_device(gb_lw_context* ctx, void* stream, int mxp, int myp, int ia, int iz, int ja, int jz,
                          int firsttime, const float* cosz, const float* albedt, double* coszen, double* asdir,
                          double* asdif, double* aldir, double* aldif) {
  if (!ctx || !gbpk::box_ok(3, mxp, myp, ia, iz, ja, jz) || !cosz || !albedt || !coszen || !asdir || !asdif ||
      !aldir || !aldif)
    return GB_LW_E_ARGS;
  const int ni = iz - ia + 1, ncol = ni * (jz - ja + 1);
  cudaSetDevice(ctx->device);
  gbpk::PackSwArgs a{};
  a.mxp = mxp, a.ia = ia, a.ja = ja, a.ni = ni, a.ncol = ncol, a.firsttime = firsttime != 0;
  a.cosz = cosz, a.albedt = albedt, a.coszen = coszen, a.asdir = asdir, a.asdif = asdif, a.aldir = aldir;
  a.aldif = aldif;
  gbpk::pack_sw_kernel<<<(ncol + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GB_LW_OK : gb_ctx_fail(ctx, e, "shortwave packing launch");
}

int gb_rtm_unpack_sw_device(gb_lw_context* ctx, void* stream, int mxp, int myp, int ia, int iz, int ja, int jz,
                            const double* swdflx, float* rshort) {
  if (!ctx || !gbpk::box_ok(3, mxp, myp, ia, iz, ja, jz) || !swdflx || !rshort) return GB_LW_E_ARGS;
  const int ni = iz - ia + 1, ncol = ni * (jz - ja + 1);
  cudaSetDevice(ctx->device);
  gbpk::UnpackSwArgs a{};
  a.mxp = mxp, a.ia = ia, a.ja = ja, a.ni = ni, a.ncol = ncol, a.swdflx = swdflx, a.rshort = rshort;
  gbpk::unpack_sw_kernel<<<(ncol + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GB_LW_OK : gb_ctx_fail(ctx, e, "shortwave write-back launch");
}
