// RRTMG_SW column solver for GB300 (sm_103a): the shortwave McICA path that
// BRAMS calls right after the longwave one (rtm_driver.f90:1386).
//
// The reference solves one column at a time (rrtmg_sw_rad.f90:460-586):
// inatm_sw, cldprmc_sw, setcoef_sw and spcvmc_sw, which runs taumol_sw and
// then, per g-point, the delta-scaled two-stream layer properties (reftra_sw)
// and the adding method (vrtqdr_sw).  Here a block of 128 threads solves a
// column and persistent blocks walk the columns:
//
//   1. one thread per layer: inatm_sw's column amounts and setcoef_sw's
//      interpolation indices and factors, into shared memory;
//   2. per band, one thread per (layer, g) cell: taumol_sw's gas and
//      Rayleigh optical depths into the block's scratch slot; per band the
//      solar-source layer and each g-point's source (sfluxzen);
//   3. one thread per g-point (112 live): from the model top down, each
//      layer's cloud optics (cldprmc_sw), its clear and total delta-scaled
//      optics, two reftra_sw evaluations and the direct beam, and the
//      downward adding recurrence; the layer and level values go to the slot;
//      then from the surface up the upward adding recurrence and the level
//      fluxes;
//   4. the g-point sums of the four fluxes per level (weighted by the
//      incoming flux of each g-point), net fluxes and heating rates.
//
// Everything is fp64, as the reference computes it: the two-stream solution
// subtracts nearly equal terms for thick layers and the SW fluxes are large
// (~1000 W m-2), so parity is kept at rounding level rather than at a
// tolerance.  The reference's exp_tbl lookups are kept (same quantised index).
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
#include "sw_solver.h"

namespace gbsw {

constexpr int NG = SW_NGPT;  // 112
constexpr int NB = 14;
constexpr int NT = 128;      // threads per column block
constexpr int NVL = 16;      // scratch values per (level, g): 10 layer values and 6 level values

// offsets (in doubles) of a band's reduced tables in the table blob (-1: absent)
struct SwBand {
  int ng, g0;
  int absa, absb, absa_rows, absb_rows, selfref, forref, nfor, sfluxref, rayl, rayl_per_g;
  int absch4, abso3a, abso3b, rayla, raylb, absh2o, absco2;
};
struct SwTab {
  SwBand b[NB];
  int ngb[NG];  // band 16..29 of each g-point
  int nspa[NB], nspb[NB];
  double preflog[59], tref[59], wavenum2[NB];
  int exp_tbl;  // [10001]
  int extliq1, ssaliq1, asyliq1, extice2, ssaice2, asyice2, extice3, ssaice3, asyice3, fdlice3;
  double abari[5], bbari[5], cbari[5], dbari[5], ebari[5], fbari[5];
  double bpade, heatfac, avogad, grav;
  int total;
};
__constant__ SwTab c_S;

__device__ __forceinline__ double tb(const double* __restrict__ T, int off) { return __ldg(T + off); }

// exp(-ze) as the reference forms it: Taylor below od_lo, else exp_tbl at
// the quantised index (reftra.f90:150-159, spcvmc.f90:445-456)
__device__ __forceinline__ double expo(const double* __restrict__ T, double ze) {
  if (ze <= 0.06) return 1.0 - ze + 0.5 * ze * ze;
  const double tblind = ze / (c_S.bpade + ze);
  const int itind = (int)(10000.0 * tblind + 0.5);
  return tb(T, c_S.exp_tbl + itind);
}

// reftra_sw for one layer (rrtmg_sw_reftra.f90:107-326, kmodts = 2)
__device__ void reftra(const double* __restrict__ T, bool chk, double zg, double prmuz, double zto1, double zw,
                       double& pref, double& prefd, double& ptra, double& ptrad) {
  if (!chk) {
    pref = 0.0;
    ptra = 1.0;
    prefd = 0.0;
    ptrad = 1.0;
    return;
  }
  const double eps = 1.e-08, zwcrit = 0.9999995;
  const double zg3 = 3.0 * zg;
  const double zgamma1 = (8.0 - zw * (5.0 + zg3)) * 0.25;
  const double zgamma2 = 3.0 * (zw * (1.0 - zg)) * 0.25;
  const double zgamma3 = (2.0 - zg3 * prmuz) * 0.25;
  const double zgamma4 = 1.0 - zgamma3;
  double zwo = 0.0, denom = 1.0;
  if (zg != 1.0) {
    const double q = zg / (1.0 - zg);
    denom = (1.0 - (1.0 - zw) * (q * q));
  }
  if (zw > 0.0 && denom != 0.0) zwo = zw / denom;
  if (zwo >= zwcrit) {
    const double za = zgamma1 * prmuz;
    const double za1 = za - zgamma3;
    const double zgt = zgamma1 * zto1;
    const double ze1 = fmin(zto1 / prmuz, 500.0);
    const double ze2 = expo(T, ze1);
    pref = (zgt - za1 * (1.0 - ze2)) / (1.0 + zgt);
    ptra = 1.0 - pref;
    prefd = zgt / (1.0 + zgt);
    ptrad = 1.0 - prefd;
    if (ze2 == 1.0) {
      pref = 0.0;
      ptra = 1.0;
      prefd = 0.0;
      ptrad = 1.0;
    }
    return;
  }
  const double za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
  const double za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
  const double zrk = sqrt(zgamma1 * zgamma1 - zgamma2 * zgamma2);
  const double zrp = zrk * prmuz;
  const double zrp1 = 1.0 + zrp;
  const double zrm1 = 1.0 - zrp;
  const double zrk2 = 2.0 * zrk;
  const double zrpp = 1.0 - zrp * zrp;
  const double zrkg = zrk + zgamma1;
  const double zr1 = zrm1 * (za2 + zrk * zgamma3);
  const double zr2 = zrp1 * (za2 - zrk * zgamma3);
  const double zr3 = zrk2 * (zgamma3 - za2 * prmuz);
  const double zr4 = zrpp * zrkg;
  const double zr5 = zrpp * (zrk - zgamma1);
  const double zt1 = zrp1 * (za1 + zrk * zgamma4);
  const double zt2 = zrm1 * (za1 - zrk * zgamma4);
  const double zt3 = zrk2 * (zgamma4 + za1 * prmuz);
  const double zbeta = (zgamma1 - zrk) / zrkg;
  const double ze1 = fmin(zrk * zto1, 500.0);
  const double ze2 = fmin(zto1 / prmuz, 500.0);
  const double zem1 = expo(T, ze1);
  const double zep1 = 1.0 / zem1;
  const double zem2 = expo(T, ze2);
  const double zep2 = 1.0 / zem2;
  const double zdenr = zr4 * zep1 + zr5 * zem1;
  const double zdent = zr4 * zep1 + zr5 * zem1;  // zt4 = zr4, zt5 = zr5
  if (zdenr >= -eps && zdenr <= eps) {
    pref = eps;
    ptra = zem2;
  } else {
    pref = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
    ptra = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdent;
  }
  const double zemm = zem1 * zem1;
  const double zdend = 1.0 / ((1.0 - zbeta * zemm) * zrkg);
  prefd = zgamma2 * (1.0 - zemm) * zdend;
  ptrad = zrk2 * zem1 * zdend;
}

// per-layer setcoef values in shared memory
struct Lay {
  double fac00, fac01, fac10, fac11, selffac, selffrac, forfac, forfrac;
  double colh2o, colco2, colo3, colch4, colo2, colmol, pdp;
  int jp, jt, jt1, indself, indfor, lower;
};
struct Smem {
  Lay* L;          // [nl]
  double* sfz;     // [NG] sfluxzen
  int* iscal;      // [0] laytrop, [1] status, [4 + k] solar-source layer of band k
};
__host__ __device__ inline size_t sw_smem_bytes(int nl) { return (size_t)nl * sizeof(Lay) + NG * 8 + 32 * 4; }
__device__ inline Smem carve(char* p, int nl) {
  Smem s;
  s.L = reinterpret_cast<Lay*>(p);
  p += (size_t)nl * sizeof(Lay);
  s.sfz = reinterpret_cast<double*>(p);
  p += NG * 8;
  s.iscal = reinterpret_cast<int*>(p);
  return s;
}

__device__ __forceinline__ double in2(const double* __restrict__ a, long long ld, long long icol, int k) {
  return __ldg(a + icol + ld * k);
}

// the binary-species parameter (taumol.f90:306-312): speccomb, js, fs
__device__ __forceinline__ void binary(double a, double b, double strrat, double mult, double& speccomb, int& js,
                                       double& fs) {
  const double oneminus = 1.0 - 1.e-06;
  speccomb = a + strrat * b;
  double specparm = a / speccomb;
  if (specparm >= oneminus) specparm = oneminus;
  const double specmult = mult * (specparm);
  js = 1 + (int)specmult;
  fs = fmod(specmult, 1.0);
}

// one taumol_sw cell: band index k (0..13), layer lay (0-based), g-point ig
// (1-based within the band); taug and taur (rrtmg_sw_taumol.f90:275-1785)
__device__ void taumol_cell(const double* __restrict__ T, const Smem& S, int k, int lay, int ig, double& taug,
                            double& taur) {
  const SwBand& B = c_S.b[k];
  const Lay& l = S.L[lay];
  const int band = k + 16;
  auto A = [&](int i) { return tb(T, B.absa + (i - 1) + B.absa_rows * (ig - 1)); };
  auto Bt = [&](int i) { return tb(T, B.absb + (i - 1) + B.absb_rows * (ig - 1)); };
  auto self = [&]() {
    const double s0 = tb(T, B.selfref + (l.indself - 1) + 10 * (ig - 1));
    const double s1 = tb(T, B.selfref + l.indself + 10 * (ig - 1));
    return l.selffac * (s0 + l.selffrac * (s1 - s0));
  };
  auto forx = [&]() {
    const double f0 = tb(T, B.forref + (l.indfor - 1) + B.nfor * (ig - 1));
    const double f1 = tb(T, B.forref + l.indfor + B.nfor * (ig - 1));
    return f0 + l.forfrac * (f1 - f0);
  };
  auto four = [&](bool upper) {
    auto t = [&](int i) { return upper ? Bt(i) : A(i); };
    int i0, i1;
    if (upper) {
      i0 = ((l.jp - 13) * 5 + (l.jt - 1)) * c_S.nspb[k] + 1;
      i1 = ((l.jp - 12) * 5 + (l.jt1 - 1)) * c_S.nspb[k] + 1;
    } else {
      i0 = ((l.jp - 1) * 5 + (l.jt - 1)) * c_S.nspa[k] + 1;
      i1 = (l.jp * 5 + (l.jt1 - 1)) * c_S.nspa[k] + 1;
    }
    return l.fac00 * t(i0) + l.fac10 * t(i0 + 1) + l.fac01 * t(i1) + l.fac11 * t(i1 + 1);
  };
  // eight-point sum of the binary-species bands (stride s1 = 9 below, 5 above)
  auto eight = [&](bool upper, int js, double fs) {
    const double f000 = (1.0 - fs) * l.fac00, f010 = (1.0 - fs) * l.fac10, f100 = fs * l.fac00,
                 f110 = fs * l.fac10, f001 = (1.0 - fs) * l.fac01, f011 = (1.0 - fs) * l.fac11,
                 f101 = fs * l.fac01, f111 = fs * l.fac11;
    int i0, i1, s1;
    if (upper) {
      i0 = ((l.jp - 13) * 5 + (l.jt - 1)) * c_S.nspb[k] + js;
      i1 = ((l.jp - 12) * 5 + (l.jt1 - 1)) * c_S.nspb[k] + js;
      s1 = 5;
    } else {
      i0 = ((l.jp - 1) * 5 + (l.jt - 1)) * c_S.nspa[k] + js;
      i1 = (l.jp * 5 + (l.jt1 - 1)) * c_S.nspa[k] + js;
      s1 = 9;
    }
    auto t = [&](int i) { return upper ? Bt(i) : A(i); };
    return f000 * t(i0) + f100 * t(i0 + 1) + f010 * t(i0 + s1) + f110 * t(i0 + s1 + 1) + f001 * t(i1) +
           f101 * t(i1 + 1) + f011 * t(i1 + s1) + f111 * t(i1 + s1 + 1);
  };
  const bool lower = l.lower;
  const double rayl0 = B.rayl >= 0 ? tb(T, B.rayl + (B.rayl_per_g ? ig - 1 : 0)) : 0.0;
  double speccomb, fs;
  int js;
  taur = l.colmol * rayl0;
  switch (band) {
    case 16:
      if (lower) {
        binary(l.colh2o, l.colch4, 252.131, 8.0, speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx());
      } else {
        taug = l.colch4 * four(true);
      }
      break;
    case 17:
    case 21:
      if (lower) {
        binary(l.colh2o, l.colco2, band == 17 ? 0.364641 : 0.0045321, 8.0, speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx());
      } else {
        binary(l.colh2o, l.colco2, band == 17 ? 0.364641 : 0.0045321, 4.0, speccomb, js, fs);
        taug = speccomb * eight(true, js, fs) + l.colh2o * l.forfac * forx();
      }
      break;
    case 18:
    case 19:
      if (lower) {
        if (band == 18)
          binary(l.colh2o, l.colch4, 38.9589, 8.0, speccomb, js, fs);
        else
          binary(l.colh2o, l.colco2, 5.49281, 8.0, speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx());
      } else {
        taug = (band == 18 ? l.colch4 : l.colco2) * four(true);
      }
      break;
    case 20: {
      const double ch4 = l.colch4 * tb(T, B.absch4 + ig - 1);
      if (lower)
        taug = l.colh2o * (four(false) + self() + l.forfac * forx()) + ch4;
      else
        taug = l.colh2o * (four(true) + l.forfac * forx()) + ch4;
      break;
    }
    case 22: {
      const double o2adj = 1.6;
      const double o2cont = 4.35e-4 * l.colo2 / (350.0 * 2.0);
      if (lower) {
        binary(l.colh2o, l.colo2, o2adj * 0.022708, 8.0, speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx()) + o2cont;
      } else {
        taug = l.colo2 * o2adj * four(true) + o2cont;
      }
      break;
    }
    case 23:
      taug = lower ? l.colh2o * (1.029 * four(false) + self() + l.forfac * forx()) : 0.0;
      break;
    case 24:
      if (lower) {
        binary(l.colh2o, l.colo2, 0.124692, 8.0, speccomb, js, fs);
        const double ra0 = tb(T, B.rayla + (ig - 1) + B.ng * (js - 1)), ra1 = tb(T, B.rayla + (ig - 1) + B.ng * js);
        taur = l.colmol * (ra0 + fs * (ra1 - ra0));
        taug = speccomb * eight(false, js, fs) + l.colo3 * tb(T, B.abso3a + ig - 1) +
               l.colh2o * (self() + l.forfac * forx());
      } else {
        taur = l.colmol * tb(T, B.raylb + ig - 1);
        taug = l.colo2 * four(true) + l.colo3 * tb(T, B.abso3b + ig - 1);
      }
      break;
    case 25:
      taug = lower ? l.colh2o * four(false) + l.colo3 * tb(T, B.abso3a + ig - 1) : l.colo3 * tb(T, B.abso3b + ig - 1);
      break;
    case 26:
      taug = 0.0;
      break;
    case 27:
      taug = l.colo3 * four(!lower);
      break;
    case 28:
      binary(l.colo3, l.colo2, 6.67029e-07, lower ? 8.0 : 4.0, speccomb, js, fs);
      taug = speccomb * eight(!lower, js, fs);
      break;
    default:  // 29
      if (lower)
        taug = l.colh2o * (four(false) + self() + l.forfac * forx()) + l.colco2 * tb(T, B.absco2 + ig - 1);
      else
        taug = l.colco2 * four(true) + l.colh2o * tb(T, B.absh2o + ig - 1);
      break;
  }
}

// the solar-source layer of band k (taumol.f90: layreffr per band, searched in
// the lower atmosphere for bands 18-26 and the upper one for 16, 17, 27-29)
__device__ int solar_layer(const Smem& S, int k, int nl, int lt) {
  const int band = k + 16;
  int ref = 0;
  bool upper = false;
  switch (band) {
    case 16: ref = 18; upper = true; break;
    case 17: ref = 30; upper = true; break;
    case 18: ref = 6; break;
    case 19: ref = 3; break;
    case 20: ref = 3; break;
    case 21: ref = 8; break;
    case 22: ref = 2; break;
    case 23: ref = 6; break;
    case 24: ref = 1; break;
    case 25: ref = 2; break;
    case 26: return lt;  // no search
    case 27: ref = 32; upper = true; break;
    case 28: ref = 42; upper = true; break;
    default: ref = 49; upper = true; break;
  }
  auto jpx = [&](int lev) { return lev >= 1 && lev <= nl ? S.L[lev - 1].jp : 0; };  // 1-based
  if (upper) {
    int ls = nl;
    for (int lay = lt + 1; lay <= nl; ++lay)
      if (jpx(lay - 1) < ref && jpx(lay) >= ref) ls = lay;
    return ls;
  }
  int ls = lt;
  for (int lay = 1; lay <= lt; ++lay)
    if (jpx(lay) < ref && jpx(lay + 1) >= ref) ls = min(lay + 1, lt);
  return ls;
}

// the incoming flux fraction of g-point ig of band k at its solar layer
// (1-based; 0 when the band's solar layer is outside the region searched)
__device__ double solar_source(const double* __restrict__ T, const Smem& S, int k, int ig, int ls, int lt, int nl) {
  const int band = k + 16;
  const SwBand& B = c_S.b[k];
  const bool in_lower = ls >= 1 && ls <= lt;
  const bool in_upper = ls > lt && ls <= nl;
  const bool lower_band = !(band == 16 || band == 17 || band >= 27);
  if (lower_band ? !in_lower : !in_upper) return 0.0;
  const Lay& l = S.L[ls - 1];
  auto sf = [&](int j) { return tb(T, B.sfluxref + (ig - 1) + B.ng * (j - 1)); };
  double speccomb, fs;
  int js;
  switch (band) {
    case 17: binary(l.colh2o, l.colco2, 0.364641, 4.0, speccomb, js, fs); break;
    case 18: binary(l.colh2o, l.colch4, 38.9589, 8.0, speccomb, js, fs); break;
    case 19: binary(l.colh2o, l.colco2, 5.49281, 8.0, speccomb, js, fs); break;
    case 21: binary(l.colh2o, l.colco2, 0.0045321, 8.0, speccomb, js, fs); break;
    case 22: binary(l.colh2o, l.colo2, 1.6 * 0.022708, 8.0, speccomb, js, fs); break;
    case 24: binary(l.colh2o, l.colo2, 0.124692, 8.0, speccomb, js, fs); break;
    case 28: binary(l.colo3, l.colo2, 6.67029e-07, 4.0, speccomb, js, fs); break;
    case 27: return (50.15 / 48.37) * sf(1);
    default: return sf(1);
  }
  return sf(js) + fs * (sf(js + 1) - sf(js));
}

// cldprmc_sw for one cell (rrtmg_sw_cldprmc.f90:103-334): on return tauc,
// ssac, asmc hold the cell's delta-scaled optics; returns a stop code
__device__ int cloud_cell(const double* __restrict__ T, const SwArgs& a, int band, double cf, double ciwp,
                          double clwp, double radice, double radliq, double fsfc, double& tauc, double& ssac,
                          double& asmc) {
  const double eps = 1.e-06, cldmin = 1.e-20;
  const double cwp = ciwp + clwp;
  if (!(cf >= cldmin && (cwp >= cldmin || tauc >= cldmin))) return 0;
  if (a.inflag == 0) {
    const double ffp = fsfc, ffp1 = 1.0 - ffp, ffpssa = 1.0 - ffp * ssac;
    const double ssacloud_a = ffp1 * ssac / ffpssa;
    const double taucloud_a = ffpssa * tauc;
    ssac = ssacloud_a;
    tauc = taucloud_a;
    asmc = (asmc - ffp) / (ffp1);
    return 0;
  }
  if (a.inflag != 2) return GB_COL_INFLAG1;
  const int ib = band;
  auto c2 = [&](int off, int rows, int i) { return tb(T, off + (i - 1) + rows * (ib - 16)); };
  double extcoice = 0, ssacoice = 0, gice = 0, forwice = 0;
  double extcoliq = 0, ssacoliq = 0, gliq = 0, forwliq = 0;
  if (ciwp != 0.0) {
    if (a.iceflag == 1) {
      if (radice < 13.0 || radice > 130.0) return GB_COL_ICE_BOUNDS;
      const double w2 = c_S.wavenum2[ib - 16];
      const int icx = w2 > 1.43e04 ? 1 : w2 > 7.7e03 ? 2 : w2 > 5.3e03 ? 3 : w2 > 4.0e03 ? 4 : 5;
      extcoice = (c_S.abari[icx - 1] + c_S.bbari[icx - 1] / radice);
      ssacoice = 1.0 - c_S.cbari[icx - 1] - c_S.dbari[icx - 1] * radice;
      gice = c_S.ebari[icx - 1] + c_S.fbari[icx - 1] * radice;
      if (gice >= 1.0) gice = 1.0 - eps;
      forwice = gice * gice;
    } else if (a.iceflag == 2 || a.iceflag == 3) {
      const bool f3 = a.iceflag == 3;
      if (f3 ? (radice < 5.0 || radice > 140.0) : (radice < 5.0 || radice > 131.0))
        return f3 ? GB_COL_DGE_BOUNDS : GB_COL_ICE_BOUNDS;
      const double factor = (radice - 2.0) / 3.0;
      int index = (int)factor;
      if (index == (f3 ? 46 : 43)) index = f3 ? 45 : 42;
      const double fint = factor - (double)index;
      const int rows = f3 ? 46 : 43;
      const int oe = f3 ? c_S.extice3 : c_S.extice2, os = f3 ? c_S.ssaice3 : c_S.ssaice2,
                og = f3 ? c_S.asyice3 : c_S.asyice2;
      extcoice = c2(oe, rows, index) + fint * (c2(oe, rows, index + 1) - c2(oe, rows, index));
      ssacoice = c2(os, rows, index) + fint * (c2(os, rows, index + 1) - c2(os, rows, index));
      gice = c2(og, rows, index) + fint * (c2(og, rows, index + 1) - c2(og, rows, index));
      if (f3) {
        const double fdelta = c2(c_S.fdlice3, 46, index) + fint * (c2(c_S.fdlice3, 46, index + 1) -
                                                                   c2(c_S.fdlice3, 46, index));
        if (fdelta < 0.0 || fdelta > 1.0) return GB_COL_SW_OPTICS;
        forwice = fdelta + 0.5 / ssacoice;
        if (forwice > gice) forwice = gice;
      } else {
        forwice = gice * gice;
      }
    } else {
      return GB_COL_SW_UNSUPPORTED;
    }
    if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0) return GB_COL_SW_OPTICS;
  }
  if (clwp != 0.0) {
    if (a.liqflag != 1) return GB_COL_SW_UNSUPPORTED;
    if (radliq < 2.5 || radliq > 60.0) return GB_COL_LIQ_BOUNDS;
    int index = (int)(radliq - 1.5);
    if (index == 0) index = 1;
    if (index == 58) index = 57;
    const double fint = radliq - 1.5 - (double)index;
    extcoliq = c2(c_S.extliq1, 58, index) + fint * (c2(c_S.extliq1, 58, index + 1) - c2(c_S.extliq1, 58, index));
    ssacoliq = c2(c_S.ssaliq1, 58, index) + fint * (c2(c_S.ssaliq1, 58, index + 1) - c2(c_S.ssaliq1, 58, index));
    if (fint < 0.0 && ssacoliq > 1.0) ssacoliq = c2(c_S.ssaliq1, 58, index);
    gliq = c2(c_S.asyliq1, 58, index) + fint * (c2(c_S.asyliq1, 58, index + 1) - c2(c_S.asyliq1, 58, index));
    forwliq = gliq * gliq;
    if (extcoliq < 0.0 || ssacoliq > 1.0 || ssacoliq < 0.0 || gliq > 1.0 || gliq < 0.0) return GB_COL_SW_OPTICS;
  }
  const double tauliqorig = clwp * extcoliq;
  const double tauiceorig = ciwp * extcoice;
  const double ssaliq = ssacoliq * (1.0 - forwliq) / (1.0 - forwliq * ssacoliq);
  const double tauliq = (1.0 - forwliq * ssacoliq) * tauliqorig;
  const double ssaice = ssacoice * (1.0 - forwice) / (1.0 - forwice * ssacoice);
  const double tauice = (1.0 - forwice * ssacoice) * tauiceorig;
  const double scatliq = ssaliq * tauliq;
  double scatice = ssaice * tauice;
  tauc = tauliq + tauice;
  if (tauc == 0.) tauc = cldmin;
  if (scatice == 0.) scatice = cldmin;
  ssac = (scatliq + scatice) / tauc;
  if (a.iceflag == 3)
    asmc = (1.0 / (scatliq + scatice)) *
           (scatliq * (gliq - forwliq) / (1.0 - forwliq) + scatice * ((gice - forwice) / (1.0 - forwice)));
  else
    asmc = (scatliq * (gliq - forwliq) / (1.0 - forwliq) + scatice * (gice - forwice) / (1.0 - forwice)) /
           (scatliq + scatice);
  return 0;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// one column by the block
__device__ void sw_column(const SwArgs& a, long long icol, const Smem& S, double* __restrict__ scr,
                          const double* __restrict__ T) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nl = a.nlay;
  const long long ld = a.ld;
  if (tid < 32) S.iscal[tid] = 0;
  __syncthreads();
  // ---- 1. inatm_sw and setcoef_sw per layer (rrtmg_sw_rad.f90:957-976, setcoef.f90:95-225)
  const double amd = 28.9660, amw = 18.0160, stpfac = 296.0 / 1013.0;
  int bad = 0;
  for (int lay = tid; lay < nl; lay += NT) {
    Lay& L = S.L[lay];
    const double pavel = in2(a.play, ld, icol, lay), tavel = in2(a.tlay, ld, icol, lay);
    const double pdp = in2(a.plev, ld, icol, lay) - in2(a.plev, ld, icol, lay + 1);
    const double h2o = in2(a.h2ovmr, ld, icol, lay);
    const double amm = (1.0 - h2o) * amd + h2o * amw;
    const double coldry = pdp * 1.e3 * c_S.avogad / (1.e2 * c_S.grav * amm * (1.0 + h2o));
    const double w1 = coldry * h2o, w2 = coldry * in2(a.co2vmr, ld, icol, lay),
                 w3 = coldry * in2(a.o3vmr, ld, icol, lay), w6 = coldry * in2(a.ch4vmr, ld, icol, lay),
                 w7 = coldry * in2(a.o2vmr, ld, icol, lay);
    if (!(pavel > 0.0) || !(tavel > 0.0) || !isfinite(pavel) || !isfinite(tavel)) bad = 1;
    L.pdp = pdp;
    const double plog = log(pavel);
    int jp = (int)(36.0 - 5 * (plog + 0.04));
    jp = jp < 1 ? 1 : (jp > 58 ? 58 : jp);
    const double fp = 5.0 * (c_S.preflog[jp - 1] - plog);
    int jt = (int)(3.0 + (tavel - c_S.tref[jp - 1]) / 15.0);
    jt = jt < 1 ? 1 : (jt > 4 ? 4 : jt);
    const double ft = ((tavel - c_S.tref[jp - 1]) / 15.0) - (double)(jt - 3);
    int jt1 = (int)(3.0 + (tavel - c_S.tref[jp]) / 15.0);
    jt1 = jt1 < 1 ? 1 : (jt1 > 4 ? 4 : jt1);
    const double ft1 = ((tavel - c_S.tref[jp]) / 15.0) - (double)(jt1 - 3);
    const double water = w1 / coldry;
    const double scalefac = pavel * stpfac / tavel;
    L.jp = jp;
    L.jt = jt;
    L.jt1 = jt1;
    const bool low = plog > 4.56;
    if (low) atomicAdd(&S.iscal[0], 1);
    L.forfac = scalefac / (1. + water);
    if (low) {
      double factor = (332.0 - tavel) / 36.0;
      L.indfor = min(2, max(1, (int)factor));
      L.forfrac = factor - (double)L.indfor;
      L.selffac = water * L.forfac;
      factor = (tavel - 188.0) / 7.2;
      L.indself = min(9, max(1, (int)factor - 7));
      L.selffrac = factor - (double)(L.indself + 7);
    } else {
      const double factor = (tavel - 188.0) / 36.0;
      L.indfor = 3;
      L.forfrac = factor - 1.0;
      L.selffac = 0.0;
      L.selffrac = 0.0;
      L.indself = 0;
    }
    L.colh2o = 1.e-20 * w1;
    L.colco2 = 1.e-20 * w2;
    L.colo3 = 1.e-20 * w3;
    L.colch4 = 1.e-20 * w6;
    L.colo2 = 1.e-20 * w7;
    L.colmol = 1.e-20 * coldry + L.colh2o;
    if (L.colco2 == 0.0) L.colco2 = 1.e-32 * coldry;
    if (L.colch4 == 0.0) L.colch4 = 1.e-32 * coldry;
    if (L.colo2 == 0.0) L.colo2 = 1.e-32 * coldry;
    const double compfp = 1.0 - fp;
    L.fac10 = compfp * ft;
    L.fac00 = compfp * (1.0 - ft);
    L.fac11 = fp * ft1;
    L.fac01 = fp * (1.0 - ft1);
  }
  bad = __syncthreads_or(bad);
  const int lt = S.iscal[0];
  // taumol treats layers 1..laytrop as the lower atmosphere (by index)
  for (int lay = tid; lay < nl; lay += NT) S.L[lay].lower = lay < lt;
  if (tid < NB) S.iscal[4 + tid] = solar_layer(S, tid, nl, lt);
  __syncthreads();
  // ---- 2. taumol_sw per band and cell into the slot; the solar source per g-point
  double* sg = scr;                       // taug [nl][NG]
  double* sr = scr + (size_t)nl * NG;     // taur [nl][NG]
  for (int k = 0; k < NB; ++k) {
    const SwBand& B = c_S.b[k];
    for (int i = tid; i < nl * B.ng; i += NT) {
      const int lay = i / B.ng, ig = i - lay * B.ng + 1;
      double tg, tr;
      taumol_cell(T, S, k, lay, ig, tg, tr);
      sg[(size_t)lay * NG + B.g0 + ig - 1] = tg;
      sr[(size_t)lay * NG + B.g0 + ig - 1] = tr;
    }
  }
  if (tid < NG) {
    const int k = c_S.ngb[tid] - 16;
    S.sfz[tid] = solar_source(T, S, k, tid - c_S.b[k].g0 + 1, S.iscal[4 + k], lt, nl);
  }
  __syncthreads();
  // ---- 3. per g-point: optics, reftra, adding (spcvmc_sw :150-440, vrtqdr_sw)
  const bool live = tid < NG;
  const int g = live ? tid : NG - 1;
  const int band = c_S.ngb[g];
  const int ibm = band - 15;
  double prmu0 = __ldg(a.coszen + icol);
  if (prmu0 < 1.e-10) prmu0 = 1.e-10;
  const double albp = ibm >= 10 && ibm <= 13 ? __ldg(a.asdir + icol) : __ldg(a.aldir + icol);
  const double albd = ibm >= 10 && ibm <= 13 ? __ldg(a.asdif + icol) : __ldg(a.aldif + icol);
  const double zincflx = live ? a.adjflux[band - 16] * S.sfz[g] * prmu0 : 0.0;
  // slot layout after taug/taur: per (level k = 1..nl+1, value v) at ((2*nl) + (k-1)*NVL + v) * NG + g
  double* V = scr + (size_t)2 * nl * NG;
  auto at = [&](int k, int v) -> double& { return V[((size_t)(k - 1) * NVL + v) * NG + g]; };
  enum { RC, RDC, TC, TDC, DBC, RT, RDT, TT, TDT, DBT, ZTDC, RDNDC, TDBC, ZTDT, RDNDT, TDBT };
  int err = 0;
  // top-down: layer jk (1 = top) is model layer ikl = nl + 1 - jk
  double tdbc = 1.0, tdbt = 1.0, ztdc = 1.0, ztdt = 1.0, rdndc = 0.0, rdndt = 0.0;
  for (int jk = 1; jk <= nl; ++jk) {
    const int lay = nl - jk;  // 0-based model layer
    const double taug = sg[(size_t)lay * NG + g], taur = sr[(size_t)lay * NG + g];
    double taua = 0.0, ssaa = 1.0, asma = 0.0;
    if (a.iaer == 10) {
      const long long o = icol + ld * (lay + (long long)nl * (ibm - 1));
      taua = __ldg(a.tauaer + o);
      ssaa = __ldg(a.ssaaer + o);
      asma = __ldg(a.asmaer + o);
    }
    double cf = 0.0, tcm = 0.0, wcm = 1.0, gcm = 0.0;
    if (a.icld >= 1) {
      const long long o = g + (long long)NG * (icol + ld * lay);
      cf = __ldg(a.cldfmcl + o);
      tcm = __ldg(a.taucmcl + o);
      wcm = __ldg(a.ssacmcl + o);
      gcm = __ldg(a.asmcmcl + o);
      const int e = cloud_cell(T, a, band, cf, __ldg(a.ciwpmcl + o), __ldg(a.clwpmcl + o),
                               in2(a.reicmcl, ld, icol, lay), in2(a.relqmcl, ld, icol, lay), __ldg(a.fsfcmcl + o),
                               tcm, wcm, gcm);
      if (e && live) err = e;
    }
    // clear-sky optics with delta scaling, then the cloud's added (spcvmc.f90:180-227)
    double ztauc = taur + taug + taua;
    double zomcc = taur * 1.0 + taua * ssaa;
    double zgcc = asma * ssaa * taua / zomcc;
    zomcc = zomcc / ztauc;
    const double zf = zgcc * zgcc, zwf = zomcc * zf;
    ztauc = (1.0 - zwf) * ztauc;
    zomcc = (zomcc - zwf) / (1.0 - zwf);
    zgcc = (zgcc - zf) / (1.0 - zf);
    const double ztauo = ztauc + tcm;
    double zomco = ztauc * zomcc + tcm * wcm;
    const double zgco = (tcm * wcm * gcm + ztauc * zomcc * zgcc) / zomco;
    zomco = zomco / ztauo;
    double rc, rdc, trc, tdc, ro, rdo, tro, tdo;
    reftra(T, true, zgcc, prmu0, ztauc, zomcc, rc, rdc, trc, tdc);
    reftra(T, cf > 1.e-12, zgco, prmu0, ztauo, zomco, ro, rdo, tro, tdo);
    const double zclear = 1.0 - cf, zcloud = cf;
    const double rt = zclear * rc + zcloud * ro, rdt = zclear * rdc + zcloud * rdo;
    const double tt = zclear * trc + zcloud * tro, tdt = zclear * tdc + zcloud * tdo;
    const double dbc = expo(T, ztauc / prmu0);
    const double dbt = zclear * dbc + zcloud * expo(T, ztauo / prmu0);
    // level jk values, then the downward recurrence to level jk+1 (vrtqdr.f90:63-80)
    if (live) {
      at(jk, ZTDC) = ztdc;
      at(jk, RDNDC) = rdndc;
      at(jk, TDBC) = tdbc;
      at(jk, ZTDT) = ztdt;
      at(jk, RDNDT) = rdndt;
      at(jk, TDBT) = tdbt;
      at(jk, RC) = rc;
      at(jk, RDC) = rdc;
      at(jk, TC) = trc;
      at(jk, TDC) = tdc;
      at(jk, DBC) = dbc;
      at(jk, RT) = rt;
      at(jk, RDT) = rdt;
      at(jk, TT) = tt;
      at(jk, TDT) = tdt;
      at(jk, DBT) = dbt;
    }
    if (jk == 1) {
      ztdc = trc;
      rdndc = rdc;
      ztdt = tt;
      rdndt = rdt;
    } else {
      double zr = 1.0 / (1.0 - rdc * rdndc);
      const double nztdc = tdbc * trc + (tdc * ((ztdc - tdbc) + tdbc * rc * rdndc)) * zr;
      rdndc = rdc + tdc * tdc * rdndc * zr;
      ztdc = nztdc;
      zr = 1.0 / (1.0 - rdt * rdndt);
      const double nztdt = tdbt * tt + (tdt * ((ztdt - tdbt) + tdbt * rt * rdndt)) * zr;
      rdndt = rdt + tdt * tdt * rdndt * zr;
      ztdt = nztdt;
    }
    tdbc = dbc * tdbc;
    tdbt = dbt * tdbt;
  }
  if (live) {
    at(nl + 1, ZTDC) = ztdc;
    at(nl + 1, RDNDC) = rdndc;
    at(nl + 1, TDBC) = tdbc;
    at(nl + 1, ZTDT) = ztdt;
    at(nl + 1, RDNDT) = rdndt;
    at(nl + 1, TDBT) = tdbt;
  }
  __syncthreads();  // every warp is done with taug/taur: their area takes the level sums
  // bottom-up (vrtqdr.f90:44-60) and the level fluxes (:82-88); level jk is
  // output level nl + 2 - jk (1 = surface)
  double rupc = albp, rupdc = albd, rupt = albp, rupdt = albd;
  for (int jk = nl + 1; jk >= 1; --jk) {
    if (jk <= nl) {
      double zr = 1.0 / (1.0 - rupdc * at(jk, RDC));
      const double nrupc = at(jk, RC) + (at(jk, TDC) * ((at(jk, TC) - at(jk, DBC)) * rupdc + at(jk, DBC) * rupc)) * zr;
      rupdc = at(jk, RDC) + at(jk, TDC) * at(jk, TDC) * rupdc * zr;
      rupc = nrupc;
      zr = 1.0 / (1.0 - rupdt * at(jk, RDT));
      const double nrupt = at(jk, RT) + (at(jk, TDT) * ((at(jk, TT) - at(jk, DBT)) * rupdt + at(jk, DBT) * rupt)) * zr;
      rupdt = at(jk, RDT) + at(jk, TDT) * at(jk, TDT) * rupdt * zr;
      rupt = nrupt;
    }
    double zr = 1.0 / (1.0 - at(jk, RDNDC) * rupdc);
    const double tdc = at(jk, TDBC), ztc = at(jk, ZTDC);
    const double cu = (tdc * rupc + (ztc - tdc) * rupdc) * zr;
    const double cd = tdc + (ztc - tdc + tdc * rupc * at(jk, RDNDC)) * zr;
    zr = 1.0 / (1.0 - at(jk, RDNDT) * rupdt);
    const double tdt = at(jk, TDBT), ztt = at(jk, ZTDT);
    const double fu = (tdt * rupt + (ztt - tdt) * rupdt) * zr;
    const double fd = tdt + (ztt - tdt + tdt * rupt * at(jk, RDNDT)) * zr;
    // g-point sums: warp butterflies, then the four warps' partials in order
    const double s0 = warp_sum(zincflx * fu), s1 = warp_sum(zincflx * fd), s2 = warp_sum(zincflx * cu),
                 s3 = warp_sum(zincflx * cd);
    // the level's four sums go to the slot's free taug area (no longer read)
    if (lane == 0) {
      double* p = sg + ((size_t)(jk - 1) * 4) * 4 + warp * 4;
      p[0] = s0;
      p[1] = s1;
      p[2] = s2;
      p[3] = s3;
    }
  }
  if (err) atomicMax(&S.iscal[1], err);
  __syncthreads();
  // ---- 4. outputs: fluxes per level, net fluxes, heating rates (rrtmg_sw_rad.f90:552-584)
  int st = S.iscal[1];
  if (bad) st = GB_COL_BADVAL;
  if (tid == 0) {
    if (a.col_err) a.col_err[icol] = st;
    if (st) atomicMax(a.err_flag, st);
  }
  const long long ldo = a.ldo;
  for (int k = tid; k <= nl; k += NT) {  // output level k+1 (1-based) = level jk = nl + 1 - k from the top
    const int jk = nl + 1 - k;
    const double* p = sg + ((size_t)(jk - 1) * 4) * 4;
    double v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = ((p[q] + p[4 + q]) + p[8 + q]) + p[12 + q];
    const long long o = icol + ldo * k;
    a.swuflx[o] = v[0];
    a.swdflx[o] = v[1];
    a.swuflxc[o] = v[2];
    a.swdflxc[o] = v[3];
  }
  __syncthreads();
  for (int k = tid; k < nl; k += NT) {
    const int jk0 = nl + 1 - k, jk1 = nl - k;  // output levels k+1 and k+2
    const double* p0 = sg + ((size_t)(jk0 - 1) * 4) * 4;
    const double* p1 = sg + ((size_t)(jk1 - 1) * 4) * 4;
    double f[2][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      f[0][q] = ((p0[q] + p0[4 + q]) + p0[8 + q]) + p0[12 + q];
      f[1][q] = ((p1[q] + p1[4 + q]) + p1[8 + q]) + p1[12 + q];
    }
    const double zdpgcp = c_S.heatfac / S.L[k].pdp;
    const long long o = icol + ldo * k;
    const double n0 = f[0][1] - f[0][0], n1 = f[1][1] - f[1][0];
    const double c0 = f[0][3] - f[0][2], c1 = f[1][3] - f[1][2];
    a.swhr[o] = k == nl - 1 ? 0.0 : (n1 - n0) * zdpgcp;
    a.swhrc[o] = k == nl - 1 ? 0.0 : (c1 - c0) * zdpgcp;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(NT, 4) sw_kernel(const __grid_constant__ SwArgs a, const double* __restrict__ T,
                                                   double* __restrict__ scratch, long long slot_doubles) {
  extern __shared__ __align__(16) char smem_raw[];
  const Smem S = carve(smem_raw, a.nlay);
  double* scr = scratch + (long long)blockIdx.x * slot_doubles;
  for (long long icol = blockIdx.x; icol < a.ncol; icol += gridDim.x) sw_column(a, icol, S, scr, T);
}

}  // namespace gbsw

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
  cudaSetDevice(ctx->device);
  cudaFree(ctx->d_sw_tables);
  ctx->d_sw_tables = nullptr;
  if (cudaMalloc(&ctx->d_sw_tables, blob.size() * 8) != cudaSuccess) {
    cudaGetLastError();
    ctx->last_error = "device allocation of the SW tables failed";
    return GB_LW_E_NOMEM;
  }
  cudaError_t e = cudaMemcpy(ctx->d_sw_tables, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(gbsw::c_S, &S, sizeof(S));
  if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "SW tables");
  std::map<std::string, GbTableEntry> tab;
  if (!gb_read_container(path.c_str(), tab, err) || !tab.count("rrsw_scon")) {
    ctx->last_error = "SW table file lacks rrsw_scon";
    return GB_LW_E_TABLES;
  }
  ctx->sw_scon = tab["rrsw_scon"].d[0];
  ctx->sw_ready = true;
  return GB_LW_OK;
}

size_t gb_sw_smem_bytes(int nlay) { return gbsw::sw_smem_bytes(nlay); }
size_t gb_sw_slot_doubles(int nlay) { return (size_t)(2 * nlay + (nlay + 1) * gbsw::NVL) * gbsw::NG; }

cudaError_t gb_sw_launch(const SwArgs& a, const double* d_tables, double* scratch, long long slots,
                         cudaStream_t stream) {
  if (a.ncol <= 0) return cudaSuccess;
  const size_t smem = gbsw::sw_smem_bytes(a.nlay);
  const void* fn = (const void*)gbsw::sw_kernel;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  long long nb = slots < a.ncol ? slots : a.ncol;
  gbsw::sw_kernel<<<(int)nb, gbsw::NT, smem, stream>>>(a, d_tables, scratch, (long long)gb_sw_slot_doubles(a.nlay));
  return cudaGetLastError();
}
