// CPU oracle for RRTMG_LW -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Double-precision restatement of the reference Fortran, statement for
// statement, with Fortran semantics kept explicitly:
//   * 1-based subscripts (macros below take Fortran indices);
//   * int() truncation toward zero, real-to-integer assignment truncation;
//   * default-real (single precision) literals rounded through float
//     (e.g. 1.e20 in taumol.f90:747, the band-4 g-point factors :1044-1050);
//   * evaluation order of sums kept left to right as written.
// Each function cites the reference file:line range it follows; paths are
// relative to src/rrtmg/RRTMG_LW/src/ of luflarois/brams.
#include "oracle.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- tables
struct Arr {
  std::vector<double> d;
  std::vector<int> i;
  int dims[4] = {1, 1, 1, 1};
  int ndim = 0;
  bool is_int = false;
};

std::map<std::string, Arr> g_tab;

bool load_container(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char magic[8];
  uint32_t count = 0;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "GBLWTBL1", 8) == 0 &&
            std::fread(&count, 4, 1, f) == 1;
  for (uint32_t e = 0; ok && e < count; ++e) {
    char name[49] = {0};
    uint32_t hdr[6];
    uint64_t nbytes = 0;
    ok = std::fread(name, 1, 48, f) == 48 && std::fread(hdr, 4, 6, f) == 6 &&
         std::fread(&nbytes, 8, 1, f) == 1;
    if (!ok) break;
    Arr a;
    a.is_int = hdr[0] == 1;
    a.ndim = (int)hdr[1];
    for (int k = 0; k < 4; ++k) a.dims[k] = (int)hdr[2 + k];
    if (a.is_int) {
      a.i.resize(nbytes / 4);
      ok = std::fread(a.i.data(), 1, nbytes, f) == nbytes;
    } else {
      a.d.resize(nbytes / 8);
      ok = std::fread(a.d.data(), 1, nbytes, f) == nbytes;
    }
    g_tab[name] = std::move(a);
  }
  std::fclose(f);
  return ok;
}

const double* T(const std::string& n) {
  auto it = g_tab.find(n);
  if (it == g_tab.end()) {
    std::fprintf(stderr, "oracle: missing table %s\n", n.c_str());
    std::abort();
  }
  return it->second.d.data();
}
const int* TI(const std::string& n) { return g_tab.at(n).i.data(); }
std::string bn(int b, const char* n) {
  char s[64];
  std::snprintf(s, sizeof s, "b%02d.%s", b, n);
  return s;
}

// rrlw_* module state after rrtmg_lw_ini
constexpr int NGPT = 140, NBND = 16, NTBL = 10000;
const double TBLINT = 10000.0;
double tau_tbl[NTBL + 1], exp_tbl[NTBL + 1], tfn_tbl[NTBL + 1];
double bpade, heatfac, fluxfac, oneminus, grav, avogad;
int ngb[NGPT], ngs[NBND], nspa[NBND], nspb[NBND];
double delwave[NBND];
const double *pref, *preflog, *tref, *chi_mls, *totplnk, *totplk16, *totplnkderiv, *totplk16deriv;
const double *absice0, *absice1, *absice2, *absice3, *absliq1;
double abscld1, absliq0;
int ixindx[4] = {1, 2, 3, 4};
bool g_ready = false;

inline double chi(int m, int jp) { return chi_mls[(m - 1) + 7 * (jp - 1)]; }  // chi_mls(7,59)
inline double fr(float x) { return (double)x; }  // default-real literal

// ---------------------------------------------------------------- per-column work
struct Col {
  int nlayers = 0;
  std::vector<double> pavel, tavel, pz, tz, coldry, wbrodl, wkl /*(7,l)*/, wx /*(4,l)*/;
  double tbound = 0, pwvcm = 0;
  double semiss[NBND];
  std::vector<double> cldfmc, taucmc, ciwpmc, clwpmc, relqmc, reicmc, taua /*(l,16)*/;
  int inflag = 0, iceflag = 0, liqflag = 0;
  // non-McICA random overlap (rtrn): layer cloud fraction and cldprop's
  // band cloud optical depths taucloud(l, ib), ib < ncbands
  int rtrn = 0, ncbands = 0;
  std::vector<double> cldfr_lay, taucloud;
  // setcoef
  int laytrop = 0;
  std::vector<int> jp, jt, jt1, indself, indfor, indminor;
  std::vector<double> planklay, planklev, colh2o, colco2, colo3, coln2o, colco, colch4, colo2,
      colbrd, fac00, fac01, fac10, fac11, rat_h2oco2, rat_h2oco2_1, rat_h2oo3, rat_h2oo3_1,
      rat_h2on2o, rat_h2on2o_1, rat_h2och4, rat_h2och4_1, rat_n2oco2, rat_n2oco2_1, rat_o3co2,
      rat_o3co2_1, selffac, selffrac, forfac, forfrac, minorfrac, scaleminor, scaleminorn2;
  double plankbnd[NBND], dplankbnd_dt[NBND];
  std::vector<double> taug, fracs, taut;  // (l, 140): index l + (ig-1)*n
  // outputs
  std::vector<double> totuflux, totdflux, fnet, htr, totuclfl, totdclfl, fnetc, htrc, dtotuflux_dt,
      dtotuclfl_dt;

  void alloc(int nlay) {
    nlayers = nlay;
    int n = nlay + 1;
    for (auto* v : {&pavel, &tavel, &coldry, &wbrodl, &relqmc, &reicmc})
      v->assign(n + 1, 0.0);
    pz.assign(n + 1, 0.0);
    tz.assign(n + 1, 0.0);
    wkl.assign(7 * (n + 1), 0.0);
    wx.assign(4 * (n + 1), 0.0);
    for (auto* v : {&cldfmc, &taucmc, &ciwpmc, &clwpmc}) v->assign(NGPT * (n + 1), 0.0);
    taua.assign((n + 1) * NBND, 0.0);
    for (auto* v : {&jp, &jt, &jt1, &indself, &indfor, &indminor}) v->assign(n + 1, 0);
    for (auto* v : {&colh2o, &colco2, &colo3, &coln2o, &colco, &colch4, &colo2, &colbrd, &fac00,
                    &fac01, &fac10, &fac11, &rat_h2oco2, &rat_h2oco2_1, &rat_h2oo3, &rat_h2oo3_1,
                    &rat_h2on2o, &rat_h2on2o_1, &rat_h2och4, &rat_h2och4_1, &rat_n2oco2,
                    &rat_n2oco2_1, &rat_o3co2, &rat_o3co2_1, &selffac, &selffrac, &forfac,
                    &forfrac, &minorfrac, &scaleminor, &scaleminorn2})
      v->assign(n + 1, 0.0);
    planklay.assign((n + 1) * NBND, 0.0);
    planklev.assign((n + 1) * NBND, 0.0);
    taug.assign((n + 1) * NGPT, 0.0);
    fracs.assign((n + 1) * NGPT, 0.0);
    taut.assign((n + 1) * NGPT, 0.0);
    for (auto* v : {&totuflux, &totdflux, &fnet, &htr, &totuclfl, &totdclfl, &fnetc, &htrc,
                    &dtotuflux_dt, &dtotuclfl_dt})
      v->assign(n + 1, 0.0);
  }
  // 2-D helpers with Fortran subscripts
  double& WKL(int m, int l) { return wkl[(m - 1) + 7 * l]; }
  double& WX(int m, int l) { return wx[(m - 1) + 4 * l]; }
  double& CF(std::vector<double>& a, int ig, int l) { return a[(ig - 1) + NGPT * l]; }
  double& PLAY(int l, int b) { return planklay[l + (nlayers + 1) * (b - 1)]; }
  double& PLEV(int l, int b) { return planklev[l + (nlayers + 1) * (b - 1)]; }
  double& TAUG(int l, int ig) { return taug[l + (nlayers + 1) * (ig - 1)]; }
  double& FRACS(int l, int ig) { return fracs[l + (nlayers + 1) * (ig - 1)]; }
  double& TAUT(int l, int ig) { return taut[l + (nlayers + 1) * (ig - 1)]; }
  double& TAUA(int l, int b) { return taua[l + (nlayers + 1) * (b - 1)]; }
  double& TAUCL(int l, int b) { return taucloud[(l - 1) + nlayers * (b - 1)]; }  // (nlayers, 16)
};

enum { ERR_OK = 0, ERR_NOT_INIT = 1, ERR_INFLAG1 = 2, ERR_ICE_SMALL = 3, ERR_ICE_BOUNDS = 4,
       ERR_DGE_BOUNDS = 5, ERR_LIQ_BOUNDS = 6, ERR_ICLD = 7, ERR_KISS_PMID = 8,
       ERR_LAYTROP = 9, ERR_ARGS = 10 };

// ---------------------------------------------------------------- inatm
// rrtmg_lw_rad.f90:598-924
void inatm(int iplon, int ncol, int nlay, int icld, int iaer, const double* play,
           const double* plev, const double* tlay, const double* tlev, const double* tsfc,
           const double* h2ovmr, const double* o3vmr, const double* co2vmr, const double* ch4vmr,
           const double* n2ovmr, const double* o2vmr, const double* cfc11vmr,
           const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
           const double* emis, int inflglw, int iceflglw, int liqflglw, const double* cldfmcl,
           const double* taucmcl, const double* ciwpmcl, const double* clwpmcl,
           const double* reicmcl, const double* relqmcl, const double* tauaer, Col& c) {
  const double amd = 28.9660, amw = 18.0160;
  auto A2 = [&](const double* a, int i, int k) { return a[(i - 1) + (size_t)ncol * (k - 1)]; };
  c.alloc(nlay);
  int nlayers = nlay;
  double amttl = 0.0, wvttl = 0.0;
  c.tbound = tsfc[iplon - 1];
  c.pz[0] = A2(plev, iplon, 1);
  c.tz[0] = A2(tlev, iplon, 1);
  for (int l = 1; l <= nlayers; ++l) {
    c.pavel[l] = A2(play, iplon, l);
    c.tavel[l] = A2(tlay, iplon, l);
    c.pz[l] = A2(plev, iplon, l + 1);
    c.tz[l] = A2(tlev, iplon, l + 1);
    c.WKL(1, l) = A2(h2ovmr, iplon, l);
    c.WKL(2, l) = A2(co2vmr, iplon, l);
    c.WKL(3, l) = A2(o3vmr, iplon, l);
    c.WKL(4, l) = A2(n2ovmr, iplon, l);
    c.WKL(6, l) = A2(ch4vmr, iplon, l);
    c.WKL(7, l) = A2(o2vmr, iplon, l);
    double amm = (1.0 - c.WKL(1, l)) * amd + c.WKL(1, l) * amw;
    c.coldry[l] = (c.pz[l - 1] - c.pz[l]) * 1.e3 * avogad / (1.e2 * grav * amm * (1.0 + c.WKL(1, l)));
  }
  for (int l = 1; l <= nlayers; ++l) {
    c.WX(1, l) = A2(ccl4vmr, iplon, l);
    c.WX(2, l) = A2(cfc11vmr, iplon, l);
    c.WX(3, l) = A2(cfc12vmr, iplon, l);
    c.WX(4, l) = A2(cfc22vmr, iplon, l);
  }
  for (int l = 1; l <= nlayers; ++l) {
    double summol = 0.0;
    for (int imol = 2; imol <= 7; ++imol) summol = summol + c.WKL(imol, l);
    c.wbrodl[l] = c.coldry[l] * (1.0 - summol);
    for (int imol = 1; imol <= 7; ++imol) c.WKL(imol, l) = c.coldry[l] * c.WKL(imol, l);
    amttl = amttl + c.coldry[l] + c.WKL(1, l);
    wvttl = wvttl + c.WKL(1, l);
    for (int ix = 1; ix <= 4; ++ix)
      if (ixindx[ix - 1] != 0) c.WX(ixindx[ix - 1], l) = c.coldry[l] * c.WX(ix, l) * 1.e-20;
  }
  double wvsh = (amw * wvttl) / (amd * amttl);
  c.pwvcm = wvsh * (1.e3 * c.pz[0]) / (1.e2 * grav);
  for (int n = 1; n <= NBND; ++n) c.semiss[n - 1] = emis[(iplon - 1) + (size_t)ncol * (n - 1)];
  if (iaer >= 1) {
    for (int l = 1; l <= nlayers; ++l)
      for (int ib = 1; ib <= NBND; ++ib)
        c.TAUA(l, ib) = tauaer[(iplon - 1) + (size_t)ncol * ((l - 1) + (size_t)nlay * (ib - 1))];
  }
  if (icld >= 1) {
    c.inflag = inflglw;
    c.iceflag = iceflglw;
    c.liqflag = liqflglw;
    for (int l = 1; l <= nlayers; ++l) {
      for (int ig = 1; ig <= NGPT; ++ig) {
        size_t o = (ig - 1) + (size_t)NGPT * ((iplon - 1) + (size_t)ncol * (l - 1));
        c.CF(c.cldfmc, ig, l) = cldfmcl[o];
        c.CF(c.taucmc, ig, l) = taucmcl[o];
        c.CF(c.ciwpmc, ig, l) = ciwpmcl[o];
        c.CF(c.clwpmc, ig, l) = clwpmcl[o];
      }
      c.reicmc[l] = A2(reicmcl, iplon, l);
      c.relqmc[l] = A2(relqmcl, iplon, l);
    }
  }
}

// ---------------------------------------------------------------- cldprmc
// rrtmg_lw_cldprmc.f90:51-273 (McICA cloud optical depth per g-point)
int cldprmc(Col& c) {
  const double cldmin = 1.e-20;
  static const int icb[16] = {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5};
  double abscoice, abscoliq;
  for (int lay = 1; lay <= c.nlayers; ++lay) {
    for (int ig = 1; ig <= NGPT; ++ig) {
      double cwp = c.CF(c.ciwpmc, ig, lay) + c.CF(c.clwpmc, ig, lay);
      if (c.CF(c.cldfmc, ig, lay) >= cldmin &&
          (cwp >= cldmin || c.CF(c.taucmc, ig, lay) >= cldmin)) {
        if (c.inflag == 0) {
          return ERR_OK;  // the reference returns from the whole routine here
        } else if (c.inflag == 1) {
          return ERR_INFLAG1;
        } else if (c.inflag == 2) {
          double radice = c.reicmc[lay];
          if (c.CF(c.ciwpmc, ig, lay) == 0.0) {
            abscoice = 0.0;
          } else if (c.iceflag == 0) {
            if (radice < 10.0) return ERR_ICE_SMALL;
            abscoice = absice0[0] + absice0[1] / radice;
          } else if (c.iceflag == 1) {
            if (radice < 13.0 || radice > 130.0) return ERR_ICE_BOUNDS;
            int ib = icb[ngb[ig - 1] - 1];
            abscoice = absice1[0 + 2 * (ib - 1)] + absice1[1 + 2 * (ib - 1)] / radice;
          } else if (c.iceflag == 2) {
            if (radice < 5.0 || radice > 131.0) return ERR_ICE_BOUNDS;
            double factor = (radice - 2.0) / 3.0;
            int index = (int)factor;
            if (index == 43) index = 42;
            double fint = factor - (double)(float)index;
            int ib = ngb[ig - 1];
            const double* a = absice2 + 43 * (ib - 1);
            abscoice = a[index - 1] + fint * (a[index] - (a[index - 1]));
          } else if (c.iceflag == 3) {
            if (radice < 5.0 || radice > 140.0) return ERR_DGE_BOUNDS;
            double factor = (radice - 2.0) / 3.0;
            int index = (int)factor;
            if (index == 46) index = 45;
            double fint = factor - (double)(float)index;
            int ib = ngb[ig - 1];
            const double* a = absice3 + 46 * (ib - 1);
            abscoice = a[index - 1] + fint * (a[index] - (a[index - 1]));
          } else {
            abscoice = 0.0;  // unset in the reference for other iceflag values
          }
          if (c.CF(c.clwpmc, ig, lay) == 0.0) {
            abscoliq = 0.0;
          } else if (c.liqflag == 0) {
            abscoliq = absliq0;
          } else if (c.liqflag == 1) {
            double radliq = c.relqmc[lay];
            if (radliq < 2.5 || radliq > 60.0) return ERR_LIQ_BOUNDS;
            int index = (int)(radliq - 1.5);
            if (index == 0) index = 1;
            if (index == 58) index = 57;
            double fint = radliq - 1.5 - (double)(float)index;
            int ib = ngb[ig - 1];
            const double* a = absliq1 + 58 * (ib - 1);
            abscoliq = a[index - 1] + fint * (a[index] - (a[index - 1]));
          } else {
            abscoliq = 0.0;
          }
          c.CF(c.taucmc, ig, lay) = c.CF(c.ciwpmc, ig, lay) * abscoice + c.CF(c.clwpmc, ig, lay) * abscoliq;
        }
      }
    }
  }
  return ERR_OK;
}

// ---------------------------------------------------------------- setcoef
// rrtmg_lw_setcoef.f90:50-434
int setcoef(Col& c, int idrv) {
  const int nlayers = c.nlayers;
  auto TP = [&](int i, int b) { return totplnk[(i - 1) + 181 * (b - 1)]; };
  auto TPD = [&](int i, int b) { return totplnkderiv[(i - 1) + 181 * (b - 1)]; };
  auto clampi = [](int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); };
  double stpfac = 296.0 / 1013.0;
  int indbound = clampi((int)(c.tbound - 159.0), 1, 180);
  double tbndfrac = c.tbound - 159.0 - (double)(float)indbound;
  int indlev0 = clampi((int)(c.tz[0] - 159.0), 1, 180);
  double t0frac = c.tz[0] - 159.0 - (double)(float)indlev0;
  c.laytrop = 0;
  int nlower_by_p = 0;
  bool prefix = true;
  for (int lay = 1; lay <= nlayers; ++lay) {
    int indlay = clampi((int)(c.tavel[lay] - 159.0), 1, 180);
    double tlayfrac = c.tavel[lay] - 159.0 - (double)(float)indlay;
    int indlev = clampi((int)(c.tz[lay] - 159.0), 1, 180);
    double tlevfrac = c.tz[lay] - 159.0 - (double)(float)indlev;
    // bands 1-15 (:204-226) and band 16 via the istart /= 16 branch (:252-269)
    for (int iband = 1; iband <= 16; ++iband) {
      if (lay == 1) {
        double dbdtlev = TP(indbound + 1, iband) - TP(indbound, iband);
        c.plankbnd[iband - 1] = c.semiss[iband - 1] * (TP(indbound, iband) + tbndfrac * dbdtlev);
        dbdtlev = TP(indlev0 + 1, iband) - TP(indlev0, iband);
        c.PLEV(0, iband) = TP(indlev0, iband) + t0frac * dbdtlev;
        if (idrv == 1) {
          dbdtlev = TPD(indbound + 1, iband) - TPD(indbound, iband);
          c.dplankbnd_dt[iband - 1] = c.semiss[iband - 1] * (TPD(indbound, iband) + tbndfrac * dbdtlev);
        }
      }
      double dbdtlev = TP(indlev + 1, iband) - TP(indlev, iband);
      double dbdtlay = TP(indlay + 1, iband) - TP(indlay, iband);
      c.PLAY(lay, iband) = TP(indlay, iband) + tlayfrac * dbdtlay;
      c.PLEV(lay, iband) = TP(indlev, iband) + tlevfrac * dbdtlev;
    }
    double plog = std::log(c.pavel[lay]);
    int jp = clampi((int)(36.0 - 5 * (plog + 0.04)), 1, 58);
    c.jp[lay] = jp;
    int jp1 = jp + 1;
    double fp = 5.0 * (preflog[jp - 1] - plog);
    int jt = clampi((int)(3.0 + (c.tavel[lay] - tref[jp - 1]) / 15.0), 1, 4);
    c.jt[lay] = jt;
    double ft = ((c.tavel[lay] - tref[jp - 1]) / 15.0) - (double)(float)(jt - 3);
    int jt1 = clampi((int)(3.0 + (c.tavel[lay] - tref[jp1 - 1]) / 15.0), 1, 4);
    c.jt1[lay] = jt1;
    double ft1 = ((c.tavel[lay] - tref[jp1 - 1]) / 15.0) - (double)(float)(jt1 - 3);
    double water = c.WKL(1, lay) / c.coldry[lay];
    double scalefac = c.pavel[lay] * stpfac / c.tavel[lay];
    if (plog > 4.56) {
      c.laytrop = c.laytrop + 1;
      if (nlower_by_p != lay - 1) prefix = false;
      nlower_by_p++;
      c.forfac[lay] = scalefac / (1. + water);
      double factor = (332.0 - c.tavel[lay]) / 36.0;
      c.indfor[lay] = std::min(2, std::max(1, (int)factor));
      c.forfrac[lay] = factor - (double)(float)c.indfor[lay];
      c.selffac[lay] = water * c.forfac[lay];
      factor = (c.tavel[lay] - 188.0) / 7.2;
      c.indself[lay] = std::min(9, std::max(1, (int)factor - 7));
      c.selffrac[lay] = factor - (double)(float)(c.indself[lay] + 7);
      c.scaleminor[lay] = c.pavel[lay] / c.tavel[lay];
      c.scaleminorn2[lay] = (c.pavel[lay] / c.tavel[lay]) * (c.wbrodl[lay] / (c.coldry[lay] + c.WKL(1, lay)));
      factor = (c.tavel[lay] - 180.8) / 7.2;
      c.indminor[lay] = std::min(18, std::max(1, (int)factor));
      c.minorfrac[lay] = factor - (double)(float)c.indminor[lay];
      c.rat_h2oco2[lay] = chi(1, jp) / chi(2, jp);
      c.rat_h2oco2_1[lay] = chi(1, jp + 1) / chi(2, jp + 1);
      c.rat_h2oo3[lay] = chi(1, jp) / chi(3, jp);
      c.rat_h2oo3_1[lay] = chi(1, jp + 1) / chi(3, jp + 1);
      c.rat_h2on2o[lay] = chi(1, jp) / chi(4, jp);
      c.rat_h2on2o_1[lay] = chi(1, jp + 1) / chi(4, jp + 1);
      c.rat_h2och4[lay] = chi(1, jp) / chi(6, jp);
      c.rat_h2och4_1[lay] = chi(1, jp + 1) / chi(6, jp + 1);
      c.rat_n2oco2[lay] = chi(4, jp) / chi(2, jp);
      c.rat_n2oco2_1[lay] = chi(4, jp + 1) / chi(2, jp + 1);
    } else {
      c.forfac[lay] = scalefac / (1. + water);
      double factor = (c.tavel[lay] - 188.0) / 36.0;
      c.indfor[lay] = 3;
      c.forfrac[lay] = factor - 1.0;
      c.selffac[lay] = water * c.forfac[lay];
      c.scaleminor[lay] = c.pavel[lay] / c.tavel[lay];
      c.scaleminorn2[lay] = (c.pavel[lay] / c.tavel[lay]) * (c.wbrodl[lay] / (c.coldry[lay] + c.WKL(1, lay)));
      factor = (c.tavel[lay] - 180.8) / 7.2;
      c.indminor[lay] = std::min(18, std::max(1, (int)factor));
      c.minorfrac[lay] = factor - (double)(float)c.indminor[lay];
      c.rat_h2oco2[lay] = chi(1, jp) / chi(2, jp);
      c.rat_h2oco2_1[lay] = chi(1, jp + 1) / chi(2, jp + 1);
      c.rat_o3co2[lay] = chi(3, jp) / chi(2, jp);
      c.rat_o3co2_1[lay] = chi(3, jp + 1) / chi(2, jp + 1);
    }
    c.colh2o[lay] = 1.e-20 * c.WKL(1, lay);
    c.colco2[lay] = 1.e-20 * c.WKL(2, lay);
    c.colo3[lay] = 1.e-20 * c.WKL(3, lay);
    c.coln2o[lay] = 1.e-20 * c.WKL(4, lay);
    c.colco[lay] = 1.e-20 * c.WKL(5, lay);
    c.colch4[lay] = 1.e-20 * c.WKL(6, lay);
    c.colo2[lay] = 1.e-20 * c.WKL(7, lay);
    if (c.colco2[lay] == 0.0) c.colco2[lay] = 1.e-32 * c.coldry[lay];
    if (c.colo3[lay] == 0.0) c.colo3[lay] = 1.e-32 * c.coldry[lay];
    if (c.coln2o[lay] == 0.0) c.coln2o[lay] = 1.e-32 * c.coldry[lay];
    if (c.colco[lay] == 0.0) c.colco[lay] = 1.e-32 * c.coldry[lay];
    if (c.colch4[lay] == 0.0) c.colch4[lay] = 1.e-32 * c.coldry[lay];
    c.colbrd[lay] = 1.e-20 * c.wbrodl[lay];
    double compfp = 1. - fp;
    c.fac10[lay] = compfp * ft;
    c.fac00[lay] = compfp * (1.0 - ft);
    c.fac11[lay] = fp * ft1;
    c.fac01[lay] = fp * (1.0 - ft1);
    c.selffac[lay] = c.colh2o[lay] * c.selffac[lay];
    c.forfac[lay] = c.colh2o[lay] * c.forfac[lay];
  }
  // The reference's taumol treats layers 1..laytrop as the lower atmosphere;
  // that only matches setcoef's per-layer branch when the lower layers form a
  // prefix (pressure decreasing with index).  Otherwise the reference reads
  // uninitialised coefficients; both this oracle and the CUDA library reject it.
  if (!prefix) return ERR_LAYTROP;
  for (int lay = 1; lay <= c.laytrop; ++lay)
    if (c.jp[lay] > 12) return ERR_LAYTROP;
  for (int lay = c.laytrop + 1; lay <= nlayers; ++lay)
    if (c.jp[lay] < 13) return ERR_LAYTROP;
  return ERR_OK;
}

// ---------------------------------------------------------------- taumol helpers
// The binary-species three-point stencil used by every lower-atmosphere
// binary band (e.g. rrtmg_lw_taumol.f90:582-650 for band 3).
struct Fk {
  int mode;  // 0 interior (2-point), 1 specparm < 0.125, 2 specparm > 0.875
  double f00, f10, f20, f01, f11, f21;  // fac000,fac100,fac200 / fac010,fac110,fac210
};
Fk stencil(double specparm, double fs, double fac00, double fac10) {
  Fk k;
  if (specparm < 0.125) {
    double p = fs - 1;
    double p4 = (p * p) * (p * p);
    double fk0 = p4, fk1 = 1 - p - 2.0 * p4, fk2 = p + p4;
    k.mode = 1;
    k.f00 = fk0 * fac00; k.f10 = fk1 * fac00; k.f20 = fk2 * fac00;
    k.f01 = fk0 * fac10; k.f11 = fk1 * fac10; k.f21 = fk2 * fac10;
  } else if (specparm > 0.875) {
    double p = -fs;
    double p4 = (p * p) * (p * p);
    double fk0 = p4, fk1 = 1 - p - 2.0 * p4, fk2 = p + p4;
    k.mode = 2;
    k.f00 = fk0 * fac00; k.f10 = fk1 * fac00; k.f20 = fk2 * fac00;
    k.f01 = fk0 * fac10; k.f11 = fk1 * fac10; k.f21 = fk2 * fac10;
  } else {
    k.mode = 0;
    k.f00 = (1.0 - fs) * fac00; k.f01 = (1.0 - fs) * fac10;
    k.f10 = fs * fac00; k.f11 = fs * fac10;
    k.f20 = k.f21 = 0.0;
  }
  return k;
}
// tau_major of the lower atmosphere; A(i) = absa(i, ig)
template <class F>
double major9(double speccomb, const Fk& k, int ind0, F A) {
  if (k.mode == 1)
    return speccomb * (k.f00 * A(ind0) + k.f10 * A(ind0 + 1) + k.f20 * A(ind0 + 2) +
                       k.f01 * A(ind0 + 9) + k.f11 * A(ind0 + 10) + k.f21 * A(ind0 + 11));
  if (k.mode == 2)
    return speccomb * (k.f20 * A(ind0 - 1) + k.f10 * A(ind0) + k.f00 * A(ind0 + 1) +
                       k.f21 * A(ind0 + 8) + k.f11 * A(ind0 + 9) + k.f01 * A(ind0 + 10));
  return speccomb * (k.f00 * A(ind0) + k.f10 * A(ind0 + 1) + k.f01 * A(ind0 + 9) + k.f11 * A(ind0 + 10));
}

struct Spec {
  double comb, parm, mult, f;
  int j;
};
// speccomb / specparm / specmult / js / fs block (e.g. taumol.f90:517-522)
Spec spec(double a, double rat, double b, double scale) {
  Spec s;
  s.comb = a + rat * b;
  s.parm = a / s.comb;
  if (s.parm >= oneminus) s.parm = oneminus;
  s.mult = scale * (s.parm);
  s.j = 1 + (int)s.mult;
  s.f = std::fmod(s.mult, 1.0);
  return s;
}

// ---------------------------------------------------------------- taumol
// rrtmg_lw_taumol.f90:50-3218
void taumol(Col& c) {
  const int nlayers = c.nlayers, laytrop = c.laytrop;
  // ---- band 1 (:299-399)
  {
    const int b = 1, ng = 10, g0 = 0;
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref")),
                 *kam = T(bn(b, "ka_mn2")), *kbm = T(bn(b, "kb_mn2"));
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    for (int lay = 1; lay <= laytrop; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[0] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[0] + 1;
      int inds = c.indself[lay];
      if (inds > 10) inds = 1;
      int indf = c.indfor[lay], indm = c.indminor[lay];
      double pp = c.pavel[lay];
      double corradj = 1.;
      if (pp < 250.0) corradj = 1.0 - 0.15 * (250.0 - pp) / 154.4;
      double scalen2 = c.colbrd[lay] * c.scaleminorn2[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = c.selffac[lay] * (sr[(inds - 1) + 10 * (ig - 1)] + c.selffrac[lay] *
                         (sr[inds + 10 * (ig - 1)] - sr[(inds - 1) + 10 * (ig - 1)]));
        double taufor = c.forfac[lay] * (fo[(indf - 1) + 4 * (ig - 1)] + c.forfrac[lay] *
                        (fo[indf + 4 * (ig - 1)] - fo[(indf - 1) + 4 * (ig - 1)]));
        double taun2 = scalen2 * (kam[(indm - 1) + 19 * (ig - 1)] + c.minorfrac[lay] *
                       (kam[indm + 19 * (ig - 1)] - kam[(indm - 1) + 19 * (ig - 1)]));
        c.TAUG(lay, g0 + ig) = corradj * (c.colh2o[lay] * (c.fac00[lay] * A(ind0) + c.fac10[lay] * A(ind0 + 1) +
                                c.fac01[lay] * A(ind1) + c.fac11[lay] * A(ind1 + 1)) + tauself + taufor + taun2);
        c.FRACS(lay, g0 + ig) = fa[ig - 1];
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[0] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[0] + 1;
      int indf = c.indfor[lay], indm = c.indminor[lay];
      double pp = c.pavel[lay];
      double corradj = 1.0 - 0.15 * (pp / 95.6);
      double scalen2 = c.colbrd[lay] * c.scaleminorn2[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        double taufor = c.forfac[lay] * (fo[(indf - 1) + 4 * (ig - 1)] + c.forfrac[lay] *
                        (fo[indf + 4 * (ig - 1)] - fo[(indf - 1) + 4 * (ig - 1)]));
        double taun2 = scalen2 * (kbm[(indm - 1) + 19 * (ig - 1)] + c.minorfrac[lay] *
                       (kbm[indm + 19 * (ig - 1)] - kbm[(indm - 1) + 19 * (ig - 1)]));
        c.TAUG(lay, g0 + ig) = corradj * (c.colh2o[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                                c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1)) + taufor + taun2);
        c.FRACS(lay, g0 + ig) = fb[ig - 1];
      }
    }
  }
  // common helpers for continuum terms
  auto tself = [&](const double* sr, int inds, int ig, int lay) {
    return c.selffac[lay] * (sr[(inds - 1) + 10 * (ig - 1)] + c.selffrac[lay] *
           (sr[inds + 10 * (ig - 1)] - sr[(inds - 1) + 10 * (ig - 1)]));
  };
  auto tfor = [&](const double* fo, int indf, int ig, int lay) {
    return c.forfac[lay] * (fo[(indf - 1) + 4 * (ig - 1)] + c.forfrac[lay] *
           (fo[indf + 4 * (ig - 1)] - fo[(indf - 1) + 4 * (ig - 1)]));
  };
  // minor with temperature interpolation only: k(indm,ig), shape (19,ng)
  auto mint = [&](const double* k, int indm, int ig, int lay) {
    return (k[(indm - 1) + 19 * (ig - 1)] + c.minorfrac[lay] *
           (k[indm + 19 * (ig - 1)] - k[(indm - 1) + 19 * (ig - 1)]));
  };
  // minor with eta and temperature interpolation: k(jm,indm,ig), shape (n,19,ng)
  auto mint2 = [&](const double* k, int n, int jm, double fm, int indm, int ig, int lay) {
    auto K = [&](int a, int t) { return k[(a - 1) + n * ((t - 1) + 19 * (ig - 1))]; };
    double m1 = K(jm, indm) + fm * (K(jm + 1, indm) - K(jm, indm));
    double m2 = K(jm, indm + 1) + fm * (K(jm + 1, indm + 1) - K(jm, indm + 1));
    return m1 + c.minorfrac[lay] * (m2 - m1);
  };
  auto inds_of = [&](int lay) { int i = c.indself[lay]; return i > 10 ? 1 : i; };
  // ---- band 2 (:402-474)
  {
    const int b = 2, ng = 12, g0 = 10;
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref"));
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    for (int lay = 1; lay <= laytrop; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[1] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[1] + 1;
      int inds = inds_of(lay), indf = c.indfor[lay];
      double pp = c.pavel[lay];
      double corradj = 1.0 - .05 * (pp - 100.0) / 900.0;
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        c.TAUG(lay, g0 + ig) = corradj * (c.colh2o[lay] * (c.fac00[lay] * A(ind0) + c.fac10[lay] * A(ind0 + 1) +
                                c.fac01[lay] * A(ind1) + c.fac11[lay] * A(ind1 + 1)) + tauself + taufor);
        c.FRACS(lay, g0 + ig) = fa[ig - 1];
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[1] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[1] + 1;
      int indf = c.indfor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        double taufor = tfor(fo, indf, ig, lay);
        c.TAUG(lay, g0 + ig) = c.colh2o[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                               c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1)) + taufor;
        c.FRACS(lay, g0 + ig) = fb[ig - 1];
      }
    }
  }
  // ---- bands 3, 4, 5: binary lower (H2O/CO2) and binary upper (nspb = 5)
  for (int b = 3; b <= 5; ++b) {
    const int ngv[3] = {16, 14, 16}, g0v[3] = {22, 38, 52};
    const int ng = ngv[b - 3], g0 = g0v[b - 3];
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref"));
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    double refrat_planck_a, refrat_planck_b, refrat_m_a = 0, refrat_m_b = 0;
    const double *kam = nullptr, *kbm = nullptr, *ccl4 = nullptr;
    if (b == 3) {  // :477-792
      refrat_planck_a = chi(1, 9) / chi(2, 9);
      refrat_planck_b = chi(1, 13) / chi(2, 13);
      refrat_m_a = chi(1, 3) / chi(2, 3);
      refrat_m_b = chi(1, 13) / chi(2, 13);
      kam = T(bn(b, "ka_mn2o"));
      kbm = T(bn(b, "kb_mn2o"));
    } else if (b == 4) {  // :795-1054
      refrat_planck_a = chi(1, 11) / chi(2, 11);
      refrat_planck_b = chi(3, 13) / chi(2, 13);
    } else {  // band 5 :1057-1332
      refrat_planck_a = chi(1, 5) / chi(2, 5);
      refrat_planck_b = chi(3, 43) / chi(2, 43);
      refrat_m_a = chi(1, 7) / chi(2, 7);
      kam = T(bn(b, "ka_mo3"));
      ccl4 = T(bn(b, "ccl4"));
    }
    for (int lay = 1; lay <= laytrop; ++lay) {
      Spec s = spec(c.colh2o[lay], c.rat_h2oco2[lay], c.colco2[lay], 8.0);
      Spec s1 = spec(c.colh2o[lay], c.rat_h2oco2_1[lay], c.colco2[lay], 8.0);
      Spec sm{};
      double adjcoln2o = 0.0;
      if (b == 3) {
        sm = spec(c.colh2o[lay], refrat_m_a, c.colco2[lay], 8.0);
        double chi_n2o = c.coln2o[lay] / c.coldry[lay];
        double ratn2o = 1.e20 * chi_n2o / chi(4, c.jp[lay] + 1);
        if (ratn2o > 1.5) {
          double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
          adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
        } else {
          adjcoln2o = c.coln2o[lay];
        }
      } else if (b == 5) {
        sm = spec(c.colh2o[lay], refrat_m_a, c.colco2[lay], 8.0);
      }
      Spec sp = spec(c.colh2o[lay], refrat_planck_a, c.colco2[lay], 8.0);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[b - 1] + s.j;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[b - 1] + s1.j;
      int inds = inds_of(lay), indf = c.indfor[lay], indm = c.indminor[lay];
      Fk k0 = stencil(s.parm, s.f, c.fac00[lay], c.fac10[lay]);
      Fk k1 = stencil(s1.parm, s1.f, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        double tau_major = major9(s.comb, k0, ind0, A);
        double tau_major1 = major9(s1.comb, k1, ind1, A);
        double t;
        if (b == 3) {
          double absn2o = mint2(kam, 9, sm.j, sm.f, indm, ig, lay);
          t = tau_major + tau_major1 + tauself + taufor + adjcoln2o * absn2o;
        } else if (b == 4) {
          t = tau_major + tau_major1 + tauself + taufor;
        } else {
          double abso3 = mint2(kam, 9, sm.j, sm.f, indm, ig, lay);
          t = tau_major + tau_major1 + tauself + taufor + abso3 * c.colo3[lay] +
              c.WX(1, lay) * ccl4[ig - 1];
        }
        c.TAUG(lay, g0 + ig) = t;
        c.FRACS(lay, g0 + ig) = fa[(ig - 1) + ng * (sp.j - 1)] + sp.f *
                                (fa[(ig - 1) + ng * sp.j] - fa[(ig - 1) + ng * (sp.j - 1)]);
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      // band 3 keys on H2O/CO2 above laytrop; bands 4 and 5 on O3/CO2
      double ka_ = (b == 3) ? c.colh2o[lay] : c.colo3[lay];
      double r0 = (b == 3) ? c.rat_h2oco2[lay] : c.rat_o3co2[lay];
      double r1 = (b == 3) ? c.rat_h2oco2_1[lay] : c.rat_o3co2_1[lay];
      Spec s = spec(ka_, r0, c.colco2[lay], 4.0);
      Spec s1 = spec(ka_, r1, c.colco2[lay], 4.0);
      double fac000 = (1.0 - s.f) * c.fac00[lay], fac010 = (1.0 - s.f) * c.fac10[lay];
      double fac100 = s.f * c.fac00[lay], fac110 = s.f * c.fac10[lay];
      double fac001 = (1.0 - s1.f) * c.fac01[lay], fac011 = (1.0 - s1.f) * c.fac11[lay];
      double fac101 = s1.f * c.fac01[lay], fac111 = s1.f * c.fac11[lay];
      Spec sm{};
      double adjcoln2o = 0.0;
      if (b == 3) {
        sm = spec(c.colh2o[lay], refrat_m_b, c.colco2[lay], 4.0);
        double chi_n2o = c.coln2o[lay] / c.coldry[lay];
        double ratn2o = fr(1.e20f) * chi_n2o / chi(4, c.jp[lay] + 1);  // default real 1.e20 (:751)
        if (ratn2o > 1.5) {
          double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
          adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
        } else {
          adjcoln2o = c.coln2o[lay];
        }
      }
      Spec sp = spec(ka_, refrat_planck_b, c.colco2[lay], 4.0);
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[b - 1] + s.j;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[b - 1] + s1.j;
      int indm = c.indminor[lay];
      int indf = c.indfor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        double tmaj = s.comb * (fac000 * B(ind0) + fac100 * B(ind0 + 1) + fac010 * B(ind0 + 5) +
                                fac110 * B(ind0 + 6)) +
                      s1.comb * (fac001 * B(ind1) + fac101 * B(ind1 + 1) + fac011 * B(ind1 + 5) +
                                 fac111 * B(ind1 + 6));
        double t;
        if (b == 3) {
          double taufor = tfor(fo, indf, ig, lay);
          double absn2o = mint2(kbm, 5, sm.j, sm.f, indm, ig, lay);
          t = tmaj + taufor + adjcoln2o * absn2o;
        } else if (b == 4) {
          t = tmaj;
        } else {
          t = tmaj + c.WX(1, lay) * ccl4[ig - 1];
        }
        c.TAUG(lay, g0 + ig) = t;
        c.FRACS(lay, g0 + ig) = fb[(ig - 1) + ng * (sp.j - 1)] + sp.f *
                                (fb[(ig - 1) + ng * sp.j] - fb[(ig - 1) + ng * (sp.j - 1)]);
      }
      if (b == 4) {  // :1044-1050, default-real factors
        c.TAUG(lay, g0 + 8) = c.TAUG(lay, g0 + 8) * fr(0.92f);
        c.TAUG(lay, g0 + 9) = c.TAUG(lay, g0 + 9) * fr(0.88f);
        c.TAUG(lay, g0 + 10) = c.TAUG(lay, g0 + 10) * fr(1.07f);
        c.TAUG(lay, g0 + 11) = c.TAUG(lay, g0 + 11) * fr(1.1f);
        c.TAUG(lay, g0 + 12) = c.TAUG(lay, g0 + 12) * fr(0.99f);
        c.TAUG(lay, g0 + 13) = c.TAUG(lay, g0 + 13) * fr(0.88f);
        c.TAUG(lay, g0 + 14) = c.TAUG(lay, g0 + 14) * fr(0.943f);
      }
    }
  }
  // ---- band 6 (:1335-1421)
  {
    const int b = 6, ng = 8, g0 = 68;
    const double *ka = T(bn(b, "ka")), *fa = T(bn(b, "fracrefa")), *sr = T(bn(b, "selfref")),
                 *fo = T(bn(b, "forref")), *kam = T(bn(b, "ka_mco2")), *c11 = T(bn(b, "cfc11adj")),
                 *c12 = T(bn(b, "cfc12"));
    const int ra = 65 * nspa[b - 1];
    for (int lay = 1; lay <= laytrop; ++lay) {
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.77);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[5] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[5] + 1;
      int inds = inds_of(lay), indf = c.indfor[lay], indm = c.indminor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        double absco2 = mint(kam, indm, ig, lay);
        c.TAUG(lay, g0 + ig) = c.colh2o[lay] * (c.fac00[lay] * A(ind0) + c.fac10[lay] * A(ind0 + 1) +
                               c.fac01[lay] * A(ind1) + c.fac11[lay] * A(ind1 + 1)) +
                               tauself + taufor + adjcolco2 * absco2 + c.WX(2, lay) * c11[ig - 1] +
                               c.WX(3, lay) * c12[ig - 1];
        c.FRACS(lay, g0 + ig) = fa[ig - 1];
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      for (int ig = 1; ig <= ng; ++ig) {
        c.TAUG(lay, g0 + ig) = 0.0 + c.WX(2, lay) * c11[ig - 1] + c.WX(3, lay) * c12[ig - 1];
        c.FRACS(lay, g0 + ig) = fa[ig - 1];
      }
    }
  }
  // ---- band 7 (:1424-1698)
  {
    const int b = 7, ng = 12, g0 = 76;
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref")),
                 *kam = T(bn(b, "ka_mco2")), *kbm = T(bn(b, "kb_mco2"));
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    double refrat_planck_a = chi(1, 3) / chi(3, 3);
    double refrat_m_a = chi(1, 3) / chi(3, 3);
    for (int lay = 1; lay <= laytrop; ++lay) {
      Spec s = spec(c.colh2o[lay], c.rat_h2oo3[lay], c.colo3[lay], 8.0);
      Spec s1 = spec(c.colh2o[lay], c.rat_h2oo3_1[lay], c.colo3[lay], 8.0);
      Spec sm = spec(c.colh2o[lay], refrat_m_a, c.colo3[lay], 8.0);
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = fr(1.e20f) * chi_co2 / chi(2, c.jp[lay] + 1);  // default real (:1503)
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 3.0 + std::pow(ratco2 - 3.0, 0.79);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      Spec sp = spec(c.colh2o[lay], refrat_planck_a, c.colo3[lay], 8.0);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[6] + s.j;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[6] + s1.j;
      int inds = inds_of(lay), indf = c.indfor[lay], indm = c.indminor[lay];
      Fk k0 = stencil(s.parm, s.f, c.fac00[lay], c.fac10[lay]);
      Fk k1 = stencil(s1.parm, s1.f, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        double absco2 = mint2(kam, 9, sm.j, sm.f, indm, ig, lay);
        double tau_major = major9(s.comb, k0, ind0, A);
        double tau_major1 = major9(s1.comb, k1, ind1, A);
        c.TAUG(lay, g0 + ig) = tau_major + tau_major1 + tauself + taufor + adjcolco2 * absco2;
        c.FRACS(lay, g0 + ig) = fa[(ig - 1) + ng * (sp.j - 1)] + sp.f *
                                (fa[(ig - 1) + ng * sp.j] - fa[(ig - 1) + ng * (sp.j - 1)]);
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = fr(1.e20f) * chi_co2 / chi(2, c.jp[lay] + 1);  // default real (:1662)
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.79);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[6] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[6] + 1;
      int indm = c.indminor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        double absco2 = mint(kbm, indm, ig, lay);
        c.TAUG(lay, g0 + ig) = c.colo3[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                               c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1)) + adjcolco2 * absco2;
        c.FRACS(lay, g0 + ig) = fb[ig - 1];
      }
      c.TAUG(lay, g0 + 6) = c.TAUG(lay, g0 + 6) * 0.92;
      c.TAUG(lay, g0 + 7) = c.TAUG(lay, g0 + 7) * 0.88;
      c.TAUG(lay, g0 + 8) = c.TAUG(lay, g0 + 8) * 1.07;
      c.TAUG(lay, g0 + 9) = c.TAUG(lay, g0 + 9) * 1.1;
      c.TAUG(lay, g0 + 10) = c.TAUG(lay, g0 + 10) * 0.99;
      c.TAUG(lay, g0 + 11) = c.TAUG(lay, g0 + 11) * 0.855;
    }
  }
  // ---- band 8 (:1701-1824)
  {
    const int b = 8, ng = 8, g0 = 88;
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref")),
                 *kaco2 = T(bn(b, "ka_mco2")), *kan2o = T(bn(b, "ka_mn2o")), *kao3 = T(bn(b, "ka_mo3")),
                 *kbco2 = T(bn(b, "kb_mco2")), *kbn2o = T(bn(b, "kb_mn2o")), *c12 = T(bn(b, "cfc12")),
                 *c22 = T(bn(b, "cfc22adj"));
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    for (int lay = 1; lay <= laytrop; ++lay) {
      double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.65);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[7] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[7] + 1;
      int inds = inds_of(lay), indf = c.indfor[lay], indm = c.indminor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        double absco2 = mint(kaco2, indm, ig, lay);
        double abso3 = mint(kao3, indm, ig, lay);
        double absn2o = mint(kan2o, indm, ig, lay);
        c.TAUG(lay, g0 + ig) = c.colh2o[lay] * (c.fac00[lay] * A(ind0) + c.fac10[lay] * A(ind0 + 1) +
                               c.fac01[lay] * A(ind1) + c.fac11[lay] * A(ind1 + 1)) +
                               tauself + taufor + adjcolco2 * absco2 + c.colo3[lay] * abso3 +
                               c.coln2o[lay] * absn2o + c.WX(3, lay) * c12[ig - 1] +
                               c.WX(4, lay) * c22[ig - 1];
        c.FRACS(lay, g0 + ig) = fa[ig - 1];
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      double chi_co2 = c.colco2[lay] / c.coldry[lay];
      double ratco2 = 1.e20 * chi_co2 / chi(2, c.jp[lay] + 1);
      double adjcolco2;
      if (ratco2 > 3.0) {
        double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.65);
        adjcolco2 = adjfac * chi(2, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcolco2 = c.colco2[lay];
      }
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[7] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[7] + 1;
      int indm = c.indminor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        double absco2 = mint(kbco2, indm, ig, lay);
        double absn2o = mint(kbn2o, indm, ig, lay);
        c.TAUG(lay, g0 + ig) = c.colo3[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                               c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1)) +
                               adjcolco2 * absco2 + c.coln2o[lay] * absn2o +
                               c.WX(3, lay) * c12[ig - 1] + c.WX(4, lay) * c22[ig - 1];
        c.FRACS(lay, g0 + ig) = fb[ig - 1];
      }
    }
  }
  // ---- band 9 (:1827-2090)
  {
    const int b = 9, ng = 12, g0 = 96;
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref")),
                 *kam = T(bn(b, "ka_mn2o")), *kbm = T(bn(b, "kb_mn2o"));
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    double refrat_planck_a = chi(1, 9) / chi(6, 9);
    double refrat_m_a = chi(1, 3) / chi(6, 3);
    for (int lay = 1; lay <= laytrop; ++lay) {
      Spec s = spec(c.colh2o[lay], c.rat_h2och4[lay], c.colch4[lay], 8.0);
      Spec s1 = spec(c.colh2o[lay], c.rat_h2och4_1[lay], c.colch4[lay], 8.0);
      Spec sm = spec(c.colh2o[lay], refrat_m_a, c.colch4[lay], 8.0);
      double chi_n2o = c.coln2o[lay] / (c.coldry[lay]);
      double ratn2o = 1.e20 * chi_n2o / chi(4, c.jp[lay] + 1);
      double adjcoln2o;
      if (ratn2o > 1.5) {
        double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
        adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcoln2o = c.coln2o[lay];
      }
      Spec sp = spec(c.colh2o[lay], refrat_planck_a, c.colch4[lay], 8.0);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[8] + s.j;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[8] + s1.j;
      int inds = inds_of(lay), indf = c.indfor[lay], indm = c.indminor[lay];
      Fk k0 = stencil(s.parm, s.f, c.fac00[lay], c.fac10[lay]);
      Fk k1 = stencil(s1.parm, s1.f, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        double absn2o = mint2(kam, 9, sm.j, sm.f, indm, ig, lay);
        double tau_major = major9(s.comb, k0, ind0, A);
        double tau_major1 = major9(s1.comb, k1, ind1, A);
        c.TAUG(lay, g0 + ig) = tau_major + tau_major1 + tauself + taufor + adjcoln2o * absn2o;
        c.FRACS(lay, g0 + ig) = fa[(ig - 1) + ng * (sp.j - 1)] + sp.f *
                                (fa[(ig - 1) + ng * sp.j] - fa[(ig - 1) + ng * (sp.j - 1)]);
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      double chi_n2o = c.coln2o[lay] / (c.coldry[lay]);
      double ratn2o = 1.e20 * chi_n2o / chi(4, c.jp[lay] + 1);
      double adjcoln2o;
      if (ratn2o > 1.5) {
        double adjfac = 0.5 + std::pow(ratn2o - 0.5, 0.65);
        adjcoln2o = adjfac * chi(4, c.jp[lay] + 1) * c.coldry[lay] * 1.e-20;
      } else {
        adjcoln2o = c.coln2o[lay];
      }
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[8] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[8] + 1;
      int indm = c.indminor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        double absn2o = mint(kbm, indm, ig, lay);
        c.TAUG(lay, g0 + ig) = c.colch4[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                               c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1)) + adjcoln2o * absn2o;
        c.FRACS(lay, g0 + ig) = fb[ig - 1];
      }
    }
  }
  // ---- bands 10 (:2093-2160) and 11 (:2163-2243): H2O only, band 11 adds O2 minor
  for (int b = 10; b <= 11; ++b) {
    const int ng = (b == 10) ? 6 : 8, g0 = (b == 10) ? 108 : 114;
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref"));
    const double* kam = (b == 11) ? T(bn(b, "ka_mo2")) : nullptr;
    const double* kbm = (b == 11) ? T(bn(b, "kb_mo2")) : nullptr;
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    for (int lay = 1; lay <= laytrop; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[b - 1] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[b - 1] + 1;
      int inds = inds_of(lay), indf = c.indfor[lay], indm = c.indminor[lay];
      double scaleo2 = c.colo2[lay] * c.scaleminor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        double t = c.colh2o[lay] * (c.fac00[lay] * A(ind0) + c.fac10[lay] * A(ind0 + 1) +
                   c.fac01[lay] * A(ind1) + c.fac11[lay] * A(ind1 + 1)) + tauself + taufor;
        if (b == 11) t = t + scaleo2 * mint(kam, indm, ig, lay);
        c.TAUG(lay, g0 + ig) = t;
        c.FRACS(lay, g0 + ig) = fa[ig - 1];
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[b - 1] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[b - 1] + 1;
      int indf = c.indfor[lay], indm = c.indminor[lay];
      double scaleo2 = c.colo2[lay] * c.scaleminor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        double taufor = tfor(fo, indf, ig, lay);
        double t = c.colh2o[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                   c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1)) + taufor;
        if (b == 11) t = t + scaleo2 * mint(kbm, indm, ig, lay);
        c.TAUG(lay, g0 + ig) = t;
        c.FRACS(lay, g0 + ig) = fb[ig - 1];
      }
    }
  }
  // ---- bands 12 (:2246-2449), 13 (:2452-2712), 15 (:2779-3004), 16 (:3007-3216):
  //      binary lower atmosphere with band-specific minors and upper formulation
  for (int b : {12, 13, 15, 16}) {
    const int ng = (b == 12) ? 8 : (b == 13) ? 4 : 2;
    const int g0 = (b == 12) ? 122 : (b == 13) ? 130 : (b == 15) ? 136 : 138;
    const double *ka = T(bn(b, "ka")), *fa = T(bn(b, "fracrefa")), *sr = T(bn(b, "selfref")),
                 *fo = T(bn(b, "forref"));
    const int ra = 65 * nspa[b - 1];
    double refrat_planck_a, refrat_m_a = 0, refrat_m_a3 = 0;
    if (b == 12) refrat_planck_a = chi(1, 10) / chi(2, 10);
    else if (b == 13) {
      refrat_planck_a = chi(1, 5) / chi(4, 5);
      refrat_m_a = chi(1, 1) / chi(4, 1);
      refrat_m_a3 = chi(1, 3) / chi(4, 3);
    } else if (b == 15) {
      refrat_planck_a = chi(4, 1) / chi(2, 1);
      refrat_m_a = chi(4, 1) / chi(2, 1);
    } else refrat_planck_a = chi(1, 6) / chi(6, 6);
    for (int lay = 1; lay <= laytrop; ++lay) {
      double a, r0, r1, bcol;  // key species pair
      if (b == 12) { a = c.colh2o[lay]; bcol = c.colco2[lay]; r0 = c.rat_h2oco2[lay]; r1 = c.rat_h2oco2_1[lay]; }
      else if (b == 13) { a = c.colh2o[lay]; bcol = c.coln2o[lay]; r0 = c.rat_h2on2o[lay]; r1 = c.rat_h2on2o_1[lay]; }
      else if (b == 15) { a = c.coln2o[lay]; bcol = c.colco2[lay]; r0 = c.rat_n2oco2[lay]; r1 = c.rat_n2oco2_1[lay]; }
      else { a = c.colh2o[lay]; bcol = c.colch4[lay]; r0 = c.rat_h2och4[lay]; r1 = c.rat_h2och4_1[lay]; }
      Spec s = spec(a, r0, bcol, 8.0);
      Spec s1 = spec(a, r1, bcol, 8.0);
      Spec sm{}, sm3{};
      double adjcolco2 = 0.0, scalen2 = 0.0;
      if (b == 13) {
        sm = spec(c.colh2o[lay], refrat_m_a, c.coln2o[lay], 8.0);
        double chi_co2 = c.colco2[lay] / (c.coldry[lay]);
        double ratco2 = 1.e20 * chi_co2 / 3.55e-4;
        if (ratco2 > 3.0) {
          double adjfac = 2.0 + std::pow(ratco2 - 2.0, 0.68);
          adjcolco2 = adjfac * fr(3.55e-4f) * c.coldry[lay] * 1.e-20;  // default real (:2538)
        } else {
          adjcolco2 = c.colco2[lay];
        }
        sm3 = spec(c.colh2o[lay], refrat_m_a3, c.coln2o[lay], 8.0);
      } else if (b == 15) {
        sm = spec(c.coln2o[lay], refrat_m_a, c.colco2[lay], 8.0);
      }
      Spec sp = spec(a, refrat_planck_a, bcol, 8.0);
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[b - 1] + s.j;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[b - 1] + s1.j;
      int inds = inds_of(lay), indf = c.indfor[lay], indm = c.indminor[lay];
      if (b == 15) scalen2 = c.colbrd[lay] * c.scaleminor[lay];
      Fk k0 = stencil(s.parm, s.f, c.fac00[lay], c.fac10[lay]);
      Fk k1 = stencil(s1.parm, s1.f, c.fac01[lay], c.fac11[lay]);
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        double tau_major = major9(s.comb, k0, ind0, A);
        double tau_major1 = major9(s1.comb, k1, ind1, A);
        double t = tau_major + tau_major1 + tauself + taufor;
        if (b == 13) {
          double absco2 = mint2(T(bn(b, "ka_mco2")), 9, sm.j, sm.f, indm, ig, lay);
          double absco = mint2(T(bn(b, "ka_mco")), 9, sm3.j, sm3.f, indm, ig, lay);
          t = t + adjcolco2 * absco2 + c.colco[lay] * absco;
        } else if (b == 15) {
          // taun2 = scalen2*(n2m1 + minorfrac*(n2m2-n2m1)) (:2908-2912)
          const double* k = T(bn(b, "ka_mn2"));
          auto K = [&](int aa, int tt) { return k[(aa - 1) + 9 * ((tt - 1) + 19 * (ig - 1))]; };
          double n2m1 = K(sm.j, indm) + sm.f * (K(sm.j + 1, indm) - K(sm.j, indm));
          double n2m2 = K(sm.j, indm + 1) + sm.f * (K(sm.j + 1, indm + 1) - K(sm.j, indm + 1));
          double taun2 = scalen2 * (n2m1 + c.minorfrac[lay] * (n2m2 - n2m1));
          t = t + taun2;
        }
        c.TAUG(lay, g0 + ig) = t;
        c.FRACS(lay, g0 + ig) = fa[(ig - 1) + ng * (sp.j - 1)] + sp.f *
                                (fa[(ig - 1) + ng * sp.j] - fa[(ig - 1) + ng * (sp.j - 1)]);
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      if (b == 12 || b == 15) {
        for (int ig = 1; ig <= ng; ++ig) {
          c.TAUG(lay, g0 + ig) = 0.0;
          c.FRACS(lay, g0 + ig) = 0.0;
        }
      } else if (b == 13) {
        const double *kbm = T(bn(b, "kb_mo3")), *fb = T(bn(b, "fracrefb"));
        int indm = c.indminor[lay];
        for (int ig = 1; ig <= ng; ++ig) {
          double abso3 = mint(kbm, indm, ig, lay);
          c.TAUG(lay, g0 + ig) = c.colo3[lay] * abso3;
          c.FRACS(lay, g0 + ig) = fb[ig - 1];
        }
      } else {  // band 16: nspb(16) = 0 pins ind0 = ind1 = 1 (:3190-3191)
        const double *kb = T(bn(b, "kb")), *fb = T(bn(b, "fracrefb"));
        const int rb = 235;
        int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[15] + 1;
        int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[15] + 1;
        for (int ig = 1; ig <= ng; ++ig) {
          auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
          c.TAUG(lay, g0 + ig) = c.colch4[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                                 c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1));
          c.FRACS(lay, g0 + ig) = fb[ig - 1];
        }
      }
    }
  }
  // ---- band 14 (:2715-2776): CO2 only
  {
    const int b = 14, ng = 2, g0 = 134;
    const double *ka = T(bn(b, "ka")), *kb = T(bn(b, "kb")), *fa = T(bn(b, "fracrefa")),
                 *fb = T(bn(b, "fracrefb")), *sr = T(bn(b, "selfref")), *fo = T(bn(b, "forref"));
    const int ra = 65 * nspa[b - 1], rb = 235 * nspb[b - 1];
    for (int lay = 1; lay <= laytrop; ++lay) {
      int ind0 = ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[13] + 1;
      int ind1 = (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[13] + 1;
      int inds = inds_of(lay), indf = c.indfor[lay];
      for (int ig = 1; ig <= ng; ++ig) {
        auto A = [&](int i) { return ka[(i - 1) + ra * (ig - 1)]; };
        double tauself = tself(sr, inds, ig, lay), taufor = tfor(fo, indf, ig, lay);
        c.TAUG(lay, g0 + ig) = c.colco2[lay] * (c.fac00[lay] * A(ind0) + c.fac10[lay] * A(ind0 + 1) +
                               c.fac01[lay] * A(ind1) + c.fac11[lay] * A(ind1 + 1)) + tauself + taufor;
        c.FRACS(lay, g0 + ig) = fa[ig - 1];
      }
    }
    for (int lay = laytrop + 1; lay <= nlayers; ++lay) {
      int ind0 = ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[13] + 1;
      int ind1 = ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[13] + 1;
      for (int ig = 1; ig <= ng; ++ig) {
        auto B = [&](int i) { return kb[(i - 1) + rb * (ig - 1)]; };
        c.TAUG(lay, g0 + ig) = c.colco2[lay] * (c.fac00[lay] * B(ind0) + c.fac10[lay] * B(ind0 + 1) +
                               c.fac01[lay] * B(ind1) + c.fac11[lay] * B(ind1 + 1));
        c.FRACS(lay, g0 + ig) = fb[ig - 1];
      }
    }
  }
}

// ---------------------------------------------------------------- rtrnmc
// rrtmg_lw_rtrnmc.f90:51-595
void rtrnmc(Col& c, int idrv) {
  const int nlayers = c.nlayers;
  const double wtdiff = 0.5, rec_6 = 0.166667;
  static const double a0[16] = {1.66, 1.55, 1.58, 1.66, 1.54, 1.454, 1.89, 1.33,
                                1.668, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66};
  static const double a1[16] = {0.00, 0.25, 0.22, 0.00, 0.13, 0.446, -0.10, 0.40,
                                -0.006, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  static const double a2[16] = {0.00, -12.0, -11.7, 0.00, -0.72, -0.243, 0.19, -0.062,
                                0.414, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  double secdiff[16];
  for (int ibnd = 1; ibnd <= 16; ++ibnd) {
    if (ibnd == 1 || ibnd == 4 || ibnd >= 10) {
      secdiff[ibnd - 1] = 1.66;
    } else {
      secdiff[ibnd - 1] = a0[ibnd - 1] + a1[ibnd - 1] * std::exp(a2[ibnd - 1] * c.pwvcm);
      if (secdiff[ibnd - 1] > 1.80) secdiff[ibnd - 1] = 1.80;
      if (secdiff[ibnd - 1] < 1.50) secdiff[ibnd - 1] = 1.50;
    }
  }
  const int n = nlayers + 1;
  std::vector<double> urad(n, 0), drad(n, 0), clrurad(n, 0), clrdrad(n, 0), d_urad_dt(n, 0),
      d_clrurad_dt(n, 0);
  std::vector<double> atrans(n), atot(n), bbugas(n), bbutot(n);
  std::vector<double> odcld(n * NGPT, 0), abscld(n * NGPT, 0), efclfrac(n * NGPT, 0);
  std::vector<int> icldlyr(n, 0);
  auto L = [&](std::vector<double>& a, int lay, int ig) -> double& { return a[lay + n * (ig - 1)]; };
  for (int lev = 0; lev <= nlayers; ++lev) {
    c.totuflux[lev] = c.totdflux[lev] = c.totuclfl[lev] = c.totdclfl[lev] = 0.0;
    if (idrv == 1) c.dtotuflux_dt[lev] = c.dtotuclfl_dt[lev] = 0.0;
  }
  if (c.rtrn) {
    // rrtmg_lw_rtrn.f90:319-336: cloud prep per layer and cloud band; the
    // sweeps below are rtrn's (:361-603 match rtrnmc's statement for
    // statement with the cloud band ib of :343-349 for the g-point index of
    // odcld/efclfrac and cldfrac(lev) for cldfmc(igc, lev)), so the band
    // values are spread over the g-points of the spectral bands that read them
    static const int ipat[3][16] = {{1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
                                    {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5},
                                    {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16}};
    const int row = c.ncbands == 1 ? 0 : (c.ncbands == 5 ? 1 : 2);
    std::vector<double> bod(16), bab(16), bef(16);
    for (int lay = 1; lay <= nlayers; ++lay) {
      icldlyr[lay] = 0;
      const double cf = c.cldfr_lay[lay];
      for (int ib = 1; ib <= c.ncbands; ++ib) {
        if (cf >= 1.e-6) {
          bod[ib - 1] = secdiff[ib - 1] * c.TAUCL(lay, ib);
          const double transcld = std::exp(-bod[ib - 1]);
          bab[ib - 1] = 1.0 - transcld;
          bef[ib - 1] = bab[ib - 1] * cf;
          icldlyr[lay] = 1;
        } else {
          bod[ib - 1] = bab[ib - 1] = bef[ib - 1] = 0.0;
          icldlyr[lay] = 0;
        }
      }
      for (int ig = 1; ig <= NGPT; ++ig) {
        const int ib = ipat[row][ngb[ig - 1] - 1];
        L(odcld, lay, ig) = bod[ib - 1];
        L(abscld, lay, ig) = bab[ib - 1];
        L(efclfrac, lay, ig) = bef[ib - 1];
        c.CF(c.cldfmc, ig, lay) = cf;
      }
    }
  } else {
    for (int lay = 1; lay <= nlayers; ++lay) {
      icldlyr[lay] = 0;
      for (int ig = 1; ig <= NGPT; ++ig) {
        if (c.CF(c.cldfmc, ig, lay) == 1.0) {
          int ib = ngb[ig - 1];
          L(odcld, lay, ig) = secdiff[ib - 1] * c.CF(c.taucmc, ig, lay);
          double transcld = std::exp(-L(odcld, lay, ig));
          L(abscld, lay, ig) = 1.0 - transcld;
          L(efclfrac, lay, ig) = L(abscld, lay, ig) * c.CF(c.cldfmc, ig, lay);
          icldlyr[lay] = 1;
        } else {
          L(odcld, lay, ig) = 0.0;
          L(abscld, lay, ig) = 0.0;
          L(efclfrac, lay, ig) = 0.0;
        }
      }
    }
  }
  int igc = 1;
  for (int iband = 1; iband <= 16; ++iband) {
    for (; igc <= ngs[iband - 1]; ++igc) {
      double radld = 0.0, radclrd = 0.0, bbd = 0.0;
      int iclddn = 0;
      for (int lev = nlayers; lev >= 1; --lev) {
        double plfrac = c.FRACS(lev, igc);
        double blay = c.PLAY(lev, iband);
        double dplankup = c.PLEV(lev, iband) - blay;
        double dplankdn = c.PLEV(lev - 1, iband) - blay;
        double odepth = secdiff[iband - 1] * c.TAUT(lev, igc);
        if (odepth < 0.0) odepth = 0.0;
        double efcl = L(efclfrac, lev, igc), cldf = c.CF(c.cldfmc, igc, lev);
        if (icldlyr[lev] == 1) {
          iclddn = 1;
          double odtot = odepth + L(odcld, lev, igc);
          if (odtot < 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            double odepth_rec = rec_6 * odepth;
            double gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            atot[lev] = odtot - 0.5 * odtot * odtot;
            double odtot_rec = rec_6 * odtot;
            double bbdtot = plfrac * (blay + dplankdn * odtot_rec);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            radld = radld - radld * (atrans[lev] + efcl * (1. - atrans[lev])) + gassrc +
                    cldf * (bbdtot * atot[lev] - gassrc);
            drad[lev - 1] = drad[lev - 1] + radld;
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + dplankup * odtot_rec);
          } else if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            double odepth_rec = rec_6 * odepth;
            double gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            odtot = odepth + L(odcld, lev, igc);
            double tblind = odtot / (bpade + odtot);
            int ittot = (int)(TBLINT * tblind + 0.5);
            double tfactot = tfn_tbl[ittot];
            double bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            atot[lev] = 1. - exp_tbl[ittot];
            radld = radld - radld * (atrans[lev] + efcl * (1.0 - atrans[lev])) + gassrc +
                    cldf * (bbdtot * atot[lev] - gassrc);
            drad[lev - 1] = drad[lev - 1] + radld;
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          } else {
            double tblind = odepth / (bpade + odepth);
            int itgas = (int)(TBLINT * tblind + 0.5);
            odepth = tau_tbl[itgas];
            atrans[lev] = 1.0 - exp_tbl[itgas];
            double tfacgas = tfn_tbl[itgas];
            double gassrc = atrans[lev] * plfrac * (blay + tfacgas * dplankdn);
            odtot = odepth + L(odcld, lev, igc);
            tblind = odtot / (bpade + odtot);
            int ittot = (int)(TBLINT * tblind + 0.5);
            double tfactot = tfn_tbl[ittot];
            double bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + tfacgas * dplankdn);
            atot[lev] = 1.0 - exp_tbl[ittot];
            radld = radld - radld * (atrans[lev] + efcl * (1.0 - atrans[lev])) + gassrc +
                    cldf * (bbdtot * atot[lev] - gassrc);
            drad[lev - 1] = drad[lev - 1] + radld;
            bbugas[lev] = plfrac * (blay + tfacgas * dplankup);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          }
        } else {
          if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            odepth = rec_6 * odepth;
            bbd = plfrac * (blay + dplankdn * odepth);
            bbugas[lev] = plfrac * (blay + dplankup * odepth);
          } else {
            double tblind = odepth / (bpade + odepth);
            int itr = (int)(TBLINT * tblind + 0.5);
            double transc = exp_tbl[itr];
            atrans[lev] = 1.0 - transc;
            double tausfac = tfn_tbl[itr];
            bbd = plfrac * (blay + tausfac * dplankdn);
            bbugas[lev] = plfrac * (blay + tausfac * dplankup);
          }
          radld = radld + (bbd - radld) * atrans[lev];
          drad[lev - 1] = drad[lev - 1] + radld;
        }
        if (iclddn == 1) {
          radclrd = radclrd + (bbd - radclrd) * atrans[lev];
          clrdrad[lev - 1] = clrdrad[lev - 1] + radclrd;
        } else {
          radclrd = radld;
          clrdrad[lev - 1] = drad[lev - 1];
        }
      }
      double rad0 = c.FRACS(1, igc) * c.plankbnd[iband - 1];
      double d_rad0_dt = 0.0;
      if (idrv == 1) d_rad0_dt = c.FRACS(1, igc) * c.dplankbnd_dt[iband - 1];
      double reflect = 1.0 - c.semiss[iband - 1];
      double radlu = rad0 + reflect * radld;
      double radclru = rad0 + reflect * radclrd;
      urad[0] = urad[0] + radlu;
      clrurad[0] = clrurad[0] + radclru;
      double d_radlu_dt = 0.0, d_radclru_dt = 0.0;
      if (idrv == 1) {
        d_radlu_dt = d_rad0_dt;
        d_urad_dt[0] = d_urad_dt[0] + d_radlu_dt;
        d_radclru_dt = d_rad0_dt;
        d_clrurad_dt[0] = d_clrurad_dt[0] + d_radclru_dt;
      }
      for (int lev = 1; lev <= nlayers; ++lev) {
        double efcl = L(efclfrac, lev, igc), cldf = c.CF(c.cldfmc, igc, lev);
        if (icldlyr[lev] == 1) {
          double gassrc = bbugas[lev] * atrans[lev];
          radlu = radlu - radlu * (atrans[lev] + efcl * (1.0 - atrans[lev])) + gassrc +
                  cldf * (bbutot[lev] * atot[lev] - gassrc);
          urad[lev] = urad[lev] + radlu;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * cldf * (1.0 - atot[lev]) + d_radlu_dt * (1.0 - cldf) * (1.0 - atrans[lev]);
            d_urad_dt[lev] = d_urad_dt[lev] + d_radlu_dt;
          }
        } else {
          radlu = radlu + (bbugas[lev] - radlu) * atrans[lev];
          urad[lev] = urad[lev] + radlu;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * (1.0 - atrans[lev]);
            d_urad_dt[lev] = d_urad_dt[lev] + d_radlu_dt;
          }
        }
        if (iclddn == 1) {
          radclru = radclru + (bbugas[lev] - radclru) * atrans[lev];
          clrurad[lev] = clrurad[lev] + radclru;
        } else {
          radclru = radlu;
          clrurad[lev] = urad[lev];
        }
        if (idrv == 1) {
          if (iclddn == 1) {
            d_radclru_dt = d_radclru_dt * (1.0 - atrans[lev]);
            d_clrurad_dt[lev] = d_clrurad_dt[lev] + d_radclru_dt;
          } else {
            d_radclru_dt = d_radlu_dt;
            d_clrurad_dt[lev] = d_urad_dt[lev];
          }
        }
      }
    }
    // band output (:538-563)
    for (int lev = nlayers; lev >= 0; --lev) {
      double uflux = urad[lev] * wtdiff, dflux = drad[lev] * wtdiff;
      urad[lev] = 0.0;
      drad[lev] = 0.0;
      c.totuflux[lev] = c.totuflux[lev] + uflux * delwave[iband - 1];
      c.totdflux[lev] = c.totdflux[lev] + dflux * delwave[iband - 1];
      double uclfl = clrurad[lev] * wtdiff, dclfl = clrdrad[lev] * wtdiff;
      clrurad[lev] = 0.0;
      clrdrad[lev] = 0.0;
      c.totuclfl[lev] = c.totuclfl[lev] + uclfl * delwave[iband - 1];
      c.totdclfl[lev] = c.totdclfl[lev] + dclfl * delwave[iband - 1];
    }
    if (idrv == 1) {
      for (int lev = nlayers; lev >= 0; --lev) {
        double duflux_dt = d_urad_dt[lev] * wtdiff;
        d_urad_dt[lev] = 0.0;
        c.dtotuflux_dt[lev] = c.dtotuflux_dt[lev] + duflux_dt * delwave[iband - 1] * fluxfac;
        double duclfl_dt = d_clrurad_dt[lev] * wtdiff;
        d_clrurad_dt[lev] = 0.0;
        c.dtotuclfl_dt[lev] = c.dtotuclfl_dt[lev] + duclfl_dt * delwave[iband - 1] * fluxfac;
      }
    }
  }
  c.totuflux[0] = c.totuflux[0] * fluxfac;
  c.totdflux[0] = c.totdflux[0] * fluxfac;
  c.fnet[0] = c.totuflux[0] - c.totdflux[0];
  c.totuclfl[0] = c.totuclfl[0] * fluxfac;
  c.totdclfl[0] = c.totdclfl[0] * fluxfac;
  c.fnetc[0] = c.totuclfl[0] - c.totdclfl[0];
  for (int lev = 1; lev <= nlayers; ++lev) {
    c.totuflux[lev] = c.totuflux[lev] * fluxfac;
    c.totdflux[lev] = c.totdflux[lev] * fluxfac;
    c.fnet[lev] = c.totuflux[lev] - c.totdflux[lev];
    c.totuclfl[lev] = c.totuclfl[lev] * fluxfac;
    c.totdclfl[lev] = c.totdclfl[lev] * fluxfac;
    c.fnetc[lev] = c.totuclfl[lev] - c.totdclfl[lev];
    int l = lev - 1;
    c.htr[l] = heatfac * (c.fnet[l] - c.fnet[lev]) / (c.pz[l] - c.pz[lev]);
    c.htrc[l] = heatfac * (c.fnetc[l] - c.fnetc[lev]) / (c.pz[l] - c.pz[lev]);
  }
  c.htr[nlayers] = 0.0;
  c.htrc[nlayers] = 0.0;
}

// ---------------------------------------------------------------- rtrnmr
// rrtmg_lw_rtrnmr.f90:51-806: the non-McICA transfer with maximum/random
// cloud overlap on layer cloud fractions and cldprop's band optical depths.
// The overlap factors faccmb1/faccmb2 (and their downward copies) are read
// at a cloudy layer whose neighbour is clear (istcld = 1) although the
// reference writes them only where istcld /= 1 (:434-438, :507-512); its
// automatic arrays leave those entries undefined.  They are taken as 0 here
// (zeroed arrays), the value the rest of the algorithm expects at the first
// cloudy layer of a block (rad is 0 there, so only faccmb enters radmod).
// faccmb1/2 at the top (:434-438 with lev = nlayers) read cldfrac(nlayers+1),
// which the driver zeroes (nomcica.f90 inatm); faccmb1d/2d at the bottom
// (:507-512 with lev = 1) read cldfrac(0), outside the array: 0 is taken
// there too (no cloud below the surface).
void rtrnmr(Col& c, int idrv) {
  const int nlayers = c.nlayers;
  const double wtdiff = 0.5, rec_6 = 0.166667;
  static const int ipat[3][16] = {{1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
                                  {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5},
                                  {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16}};
  static const double a0[16] = {1.66, 1.55, 1.58, 1.66, 1.54, 1.454, 1.89, 1.33,
                                1.668, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66, 1.66};
  static const double a1[16] = {0.00, 0.25, 0.22, 0.00, 0.13, 0.446, -0.10, 0.40,
                                -0.006, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  static const double a2[16] = {0.00, -12.0, -11.7, 0.00, -0.72, -0.243, 0.19, -0.062,
                                0.414, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00};
  double secdiff[16];
  for (int ibnd = 1; ibnd <= 16; ++ibnd) {  // :287-295
    if (ibnd == 1 || ibnd == 4 || ibnd >= 10) {
      secdiff[ibnd - 1] = 1.66;
    } else {
      secdiff[ibnd - 1] = a0[ibnd - 1] + a1[ibnd - 1] * std::exp(a2[ibnd - 1] * c.pwvcm);
      if (secdiff[ibnd - 1] > 1.80) secdiff[ibnd - 1] = 1.80;
      if (secdiff[ibnd - 1] < 1.50) secdiff[ibnd - 1] = 1.50;
    }
  }
  const int n = nlayers + 2;
  std::vector<double> urad(n, 0), drad(n, 0), clrurad(n, 0), clrdrad(n, 0), d_urad_dt(n, 0),
      d_clrurad_dt(n, 0), atrans(n, 0), atot(n, 0), bbugas(n, 0), bbutot(n, 0);
  std::vector<double> odcld(n * 16, 0.0);
  std::vector<int> icldlyr(n, 0), istcld(n, 0), istcldd(n, 0);
  // faccld1..faccmb2 (1 .. nlayers+1) and faccld1d..faccmb2d (0 .. nlayers)
  std::vector<double> faccld1(n, 0), faccld2(n, 0), facclr1(n, 0), facclr2(n, 0), faccmb1(n, 0), faccmb2(n, 0);
  std::vector<double> faccld1d(n, 0), faccld2d(n, 0), facclr1d(n, 0), facclr2d(n, 0), faccmb1d(n, 0),
      faccmb2d(n, 0);
  auto OD = [&](int lay, int ib) -> double& { return odcld[lay + n * (ib - 1)]; };
  const std::vector<double>& cf = c.cldfr_lay;  // cldfrac(1 .. nlayers)
  auto CF = [&](int l) -> double {
    if (l >= 1 && l <= nlayers) return cf[l];
    return 0.0;
  };
  for (int lev = 0; lev <= nlayers; ++lev) {
    c.totuflux[lev] = c.totdflux[lev] = c.totuclfl[lev] = c.totdclfl[lev] = 0.0;
    if (idrv == 1) c.dtotuflux_dt[lev] = c.dtotuclfl_dt[lev] = 0.0;
  }
  for (int lay = 1; lay <= nlayers; ++lay) {  // :334-343
    for (int ib = 1; ib <= c.ncbands; ++ib) {
      if (cf[lay] >= 1.e-6) {
        OD(lay, ib) = secdiff[ib - 1] * c.TAUCL(lay, ib);
        icldlyr[lay] = 1;
      } else {
        OD(lay, ib) = 0.0;
        icldlyr[lay] = 0;
      }
    }
  }
  // maximum/random overlap parameters, upward (:347-440)
  double rat1 = 0.0, rat2 = 0.0, fmax, fmin;
  istcld[1] = 1;
  istcldd[nlayers] = 1;
  for (int lev = 1; lev <= nlayers; ++lev) {
    if (icldlyr[lev] == 1) {
      istcld[lev + 1] = 0;
      if (lev == nlayers) {
        faccld1[lev + 1] = faccld2[lev + 1] = facclr1[lev + 1] = facclr2[lev + 1] = 0.0;
        faccmb1[lev + 1] = faccmb2[lev + 1] = 0.0;
      } else if (CF(lev + 1) >= CF(lev)) {
        faccld1[lev + 1] = 0.0;
        faccld2[lev + 1] = 0.0;
        if (istcld[lev] == 1) {
          facclr1[lev + 1] = 0.0;
          facclr2[lev + 1] = 0.0;
          if (CF(lev) < 1.0) facclr2[lev + 1] = (CF(lev + 1) - CF(lev)) / (1.0 - CF(lev));
          facclr2[lev] = 0.0;
          faccld2[lev] = 0.0;
        } else {
          fmax = std::max(CF(lev), CF(lev - 1));
          if (CF(lev + 1) > fmax) {
            facclr1[lev + 1] = rat2;
            facclr2[lev + 1] = (CF(lev + 1) - fmax) / (1.0 - fmax);
          } else if (CF(lev + 1) < fmax) {
            facclr1[lev + 1] = (CF(lev + 1) - CF(lev)) / (CF(lev - 1) - CF(lev));
            facclr2[lev + 1] = 0.0;
          } else {
            facclr1[lev + 1] = rat2;
            facclr2[lev + 1] = 0.0;
          }
        }
        if (facclr1[lev + 1] > 0.0 || facclr2[lev + 1] > 0.0) {
          rat1 = 1.0;
          rat2 = 0.0;
        } else {
          rat1 = 0.0;
          rat2 = 0.0;
        }
      } else {
        facclr1[lev + 1] = 0.0;
        facclr2[lev + 1] = 0.0;
        if (istcld[lev] == 1) {
          faccld1[lev + 1] = 0.0;
          faccld2[lev + 1] = (CF(lev) - CF(lev + 1)) / CF(lev);
          facclr2[lev] = 0.0;
          faccld2[lev] = 0.0;
        } else {
          fmin = std::min(CF(lev), CF(lev - 1));
          if (CF(lev + 1) <= fmin) {
            faccld1[lev + 1] = rat1;
            faccld2[lev + 1] = (fmin - CF(lev + 1)) / fmin;
          } else {
            faccld1[lev + 1] = (CF(lev) - CF(lev + 1)) / (CF(lev) - fmin);
            faccld2[lev + 1] = 0.0;
          }
        }
        if (faccld1[lev + 1] > 0.0 || faccld2[lev + 1] > 0.0) {
          rat1 = 0.0;
          rat2 = 1.0;
        } else {
          rat1 = 0.0;
          rat2 = 0.0;
        }
      }
      if (istcld[lev] != 1) {  // max(0., ...): a default-real 0
        faccmb1[lev + 1] = std::max<double>(0.0, std::min<double>(CF(lev + 1) - CF(lev), CF(lev - 1) - CF(lev)));
        faccmb2[lev + 1] = std::max<double>(0.0, std::min<double>(CF(lev) - CF(lev + 1), CF(lev) - CF(lev - 1)));
      }
    } else {
      istcld[lev + 1] = 1;
    }
  }
  // downward (:442-514); rat1/rat2 carry over from the loop above
  for (int lev = nlayers; lev >= 1; --lev) {
    if (icldlyr[lev] == 1) {
      istcldd[lev - 1] = 0;
      if (lev == 1) {
        faccld1d[lev - 1] = faccld2d[lev - 1] = facclr1d[lev - 1] = facclr2d[lev - 1] = 0.0;
        faccmb1d[lev - 1] = faccmb2d[lev - 1] = 0.0;
      } else if (CF(lev - 1) >= CF(lev)) {
        faccld1d[lev - 1] = 0.0;
        faccld2d[lev - 1] = 0.0;
        if (istcldd[lev] == 1) {
          facclr1d[lev - 1] = 0.0;
          facclr2d[lev - 1] = 0.0;
          if (CF(lev) < 1.0) facclr2d[lev - 1] = (CF(lev - 1) - CF(lev)) / (1.0 - CF(lev));
          facclr2d[lev] = 0.0;
          faccld2d[lev] = 0.0;
        } else {
          fmax = std::max(CF(lev), CF(lev + 1));
          if (CF(lev - 1) > fmax) {
            facclr1d[lev - 1] = rat2;
            facclr2d[lev - 1] = (CF(lev - 1) - fmax) / (1.0 - fmax);
          } else if (CF(lev - 1) < fmax) {
            facclr1d[lev - 1] = (CF(lev - 1) - CF(lev)) / (CF(lev + 1) - CF(lev));
            facclr2d[lev - 1] = 0.0;
          } else {
            facclr1d[lev - 1] = rat2;
            facclr2d[lev - 1] = 0.0;
          }
        }
        if (facclr1d[lev - 1] > 0.0 || facclr2d[lev - 1] > 0.0) {
          rat1 = 1.0;
          rat2 = 0.0;
        } else {
          rat1 = 0.0;
          rat2 = 0.0;
        }
      } else {
        facclr1d[lev - 1] = 0.0;
        facclr2d[lev - 1] = 0.0;
        if (istcldd[lev] == 1) {
          faccld1d[lev - 1] = 0.0;
          faccld2d[lev - 1] = (CF(lev) - CF(lev - 1)) / CF(lev);
          facclr2d[lev] = 0.0;
          faccld2d[lev] = 0.0;
        } else {
          fmin = std::min(CF(lev), CF(lev + 1));
          if (CF(lev - 1) <= fmin) {
            faccld1d[lev - 1] = rat1;
            faccld2d[lev - 1] = (fmin - CF(lev - 1)) / fmin;
          } else {
            faccld1d[lev - 1] = (CF(lev) - CF(lev - 1)) / (CF(lev) - fmin);
            faccld2d[lev - 1] = 0.0;
          }
        }
        if (faccld1d[lev - 1] > 0.0 || faccld2d[lev - 1] > 0.0) {
          rat1 = 0.0;
          rat2 = 1.0;
        } else {
          rat1 = 0.0;
          rat2 = 0.0;
        }
      }
      if (istcldd[lev] != 1) {
        faccmb1d[lev - 1] = std::max<double>(0.0, std::min<double>(CF(lev + 1) - CF(lev), CF(lev - 1) - CF(lev)));
        faccmb2d[lev - 1] = std::max<double>(0.0, std::min<double>(CF(lev) - CF(lev + 1), CF(lev) - CF(lev - 1)));
      }
    } else {
      istcldd[lev - 1] = 1;
    }
  }
  const int row = c.ncbands == 1 ? 0 : (c.ncbands == 5 ? 1 : 2);
  int igc = 1;
  for (int iband = 1; iband <= 16; ++iband) {  // :516-806
    const int ib = ipat[row][iband - 1];
    for (; igc <= ngs[iband - 1]; ++igc) {
      double radld = 0.0, radclrd = 0.0, bbd = 0.0;
      double cldradd = 0.0, clrradd = 0.0, rad = 0.0, oldcld, oldclr, radmod;
      int iclddn = 0;
      for (int lev = nlayers; lev >= 1; --lev) {
        const double plfrac = c.FRACS(lev, igc);
        const double blay = c.PLAY(lev, iband);
        const double dplankup = c.PLEV(lev, iband) - blay;
        const double dplankdn = c.PLEV(lev - 1, iband) - blay;
        double odepth = secdiff[iband - 1] * c.TAUT(lev, igc);
        if (odepth < 0.0) odepth = 0.0;
        if (icldlyr[lev] == 1) {
          iclddn = 1;
          double odtot = odepth + OD(lev, ib), gassrc, bbdtot;
          if (odtot < 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            const double odepth_rec = rec_6 * odepth;
            gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            atot[lev] = odtot - 0.5 * odtot * odtot;
            const double odtot_rec = rec_6 * odtot;
            bbdtot = plfrac * (blay + dplankdn * odtot_rec);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + dplankup * odtot_rec);
          } else if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            const double odepth_rec = rec_6 * odepth;
            gassrc = plfrac * (blay + dplankdn * odepth_rec) * atrans[lev];
            odtot = odepth + OD(lev, ib);
            const double tblind = odtot / (bpade + odtot);
            const int ittot = (int)(TBLINT * tblind + 0.5);
            const double tfactot = tfn_tbl[ittot];
            bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + dplankdn * odepth_rec);
            atot[lev] = 1.0 - exp_tbl[ittot];
            bbugas[lev] = plfrac * (blay + dplankup * odepth_rec);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          } else {
            double tblind = odepth / (bpade + odepth);
            const int itgas = (int)(TBLINT * tblind + 0.5);
            odepth = tau_tbl[itgas];
            atrans[lev] = 1.0 - exp_tbl[itgas];
            const double tfacgas = tfn_tbl[itgas];
            gassrc = atrans[lev] * plfrac * (blay + tfacgas * dplankdn);
            odtot = odepth + OD(lev, ib);
            tblind = odtot / (bpade + odtot);
            const int ittot = (int)(TBLINT * tblind + 0.5);
            const double tfactot = tfn_tbl[ittot];
            bbdtot = plfrac * (blay + tfactot * dplankdn);
            bbd = plfrac * (blay + tfacgas * dplankdn);
            atot[lev] = 1.0 - exp_tbl[ittot];
            bbugas[lev] = plfrac * (blay + tfacgas * dplankup);
            bbutot[lev] = plfrac * (blay + tfactot * dplankup);
          }
          if (istcldd[lev] == 1) {
            cldradd = cf[lev] * radld;
            clrradd = radld - cldradd;
            oldcld = cldradd;
            oldclr = clrradd;
            rad = 0.0;
          }
          const double ttot = 1.0 - atot[lev];
          const double cldsrc = bbdtot * atot[lev];
          cldradd = cldradd * ttot + cf[lev] * cldsrc;
          clrradd = clrradd * (1.0 - atrans[lev]) + (1.0 - cf[lev]) * gassrc;
          radld = cldradd + clrradd;
          drad[lev - 1] = drad[lev - 1] + radld;
          radmod = rad * (facclr1d[lev - 1] * (1. - atrans[lev]) + faccld1d[lev - 1] * ttot) -
                   faccmb1d[lev - 1] * gassrc + faccmb2d[lev - 1] * cldsrc;
          oldcld = cldradd - radmod;
          oldclr = clrradd + radmod;
          rad = -radmod + facclr2d[lev - 1] * oldclr - faccld2d[lev - 1] * oldcld;
          cldradd = cldradd + rad;
          clrradd = clrradd - rad;
        } else {
          if (odepth <= 0.06) {
            atrans[lev] = odepth - 0.5 * odepth * odepth;
            odepth = rec_6 * odepth;
            bbd = plfrac * (blay + dplankdn * odepth);
            bbugas[lev] = plfrac * (blay + dplankup * odepth);
          } else {
            const double tblind = odepth / (bpade + odepth);
            const int itr = (int)(TBLINT * tblind + 0.5);
            const double transc = exp_tbl[itr];
            atrans[lev] = 1.0 - transc;
            const double tausfac = tfn_tbl[itr];
            bbd = plfrac * (blay + tausfac * dplankdn);
            bbugas[lev] = plfrac * (blay + tausfac * dplankup);
          }
          radld = radld + (bbd - radld) * atrans[lev];
          drad[lev - 1] = drad[lev - 1] + radld;
        }
        if (iclddn == 1) {
          radclrd = radclrd + (bbd - radclrd) * atrans[lev];
          clrdrad[lev - 1] = clrdrad[lev - 1] + radclrd;
        } else {
          radclrd = radld;
          clrdrad[lev - 1] = drad[lev - 1];
        }
      }
      const double rad0 = c.FRACS(1, igc) * c.plankbnd[iband - 1];
      double d_rad0_dt = 0.0;
      if (idrv == 1) d_rad0_dt = c.FRACS(1, igc) * c.dplankbnd_dt[iband - 1];
      const double reflect = 1.0 - c.semiss[iband - 1];
      double radlu = rad0 + reflect * radld;
      double radclru = rad0 + reflect * radclrd;
      urad[0] = urad[0] + radlu;
      clrurad[0] = clrurad[0] + radclru;
      double d_radlu_dt = 0.0, d_radclru_dt = 0.0;
      if (idrv == 1) {
        d_radlu_dt = d_rad0_dt;
        d_urad_dt[0] = d_urad_dt[0] + d_radlu_dt;
        d_radclru_dt = d_rad0_dt;
        d_clrurad_dt[0] = d_clrurad_dt[0] + d_radclru_dt;
      }
      double cldradu = 0.0, clrradu = 0.0;
      for (int lev = 1; lev <= nlayers; ++lev) {
        if (icldlyr[lev] == 1) {
          const double gassrc = bbugas[lev] * atrans[lev];
          if (istcld[lev] == 1) {
            cldradu = cf[lev] * radlu;
            clrradu = radlu - cldradu;
            oldcld = cldradu;
            oldclr = clrradu;
            rad = 0.0;
          }
          const double ttot = 1.0 - atot[lev];
          const double cldsrc = bbutot[lev] * atot[lev];
          cldradu = cldradu * ttot + cf[lev] * cldsrc;
          clrradu = clrradu * (1.0 - atrans[lev]) + (1.0 - cf[lev]) * gassrc;
          radlu = cldradu + clrradu;
          urad[lev] = urad[lev] + radlu;
          radmod = rad * (facclr1[lev + 1] * (1.0 - atrans[lev]) + faccld1[lev + 1] * ttot) -
                   faccmb1[lev + 1] * gassrc + faccmb2[lev + 1] * cldsrc;
          oldcld = cldradu - radmod;
          oldclr = clrradu + radmod;
          rad = -radmod + facclr2[lev + 1] * oldclr - faccld2[lev + 1] * oldcld;
          cldradu = cldradu + rad;
          clrradu = clrradu - rad;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * cf[lev] * (1.0 - atot[lev]) + d_radlu_dt * (1.0 - cf[lev]) * (1.0 - atrans[lev]);
            d_urad_dt[lev] = d_urad_dt[lev] + d_radlu_dt;
          }
        } else {
          radlu = radlu + (bbugas[lev] - radlu) * atrans[lev];
          urad[lev] = urad[lev] + radlu;
          if (idrv == 1) {
            d_radlu_dt = d_radlu_dt * (1.0 - atrans[lev]);
            d_urad_dt[lev] = d_urad_dt[lev] + d_radlu_dt;
          }
        }
        if (iclddn == 1) {
          radclru = radclru + (bbugas[lev] - radclru) * atrans[lev];
          clrurad[lev] = clrurad[lev] + radclru;
        } else {
          radclru = radlu;
          clrurad[lev] = urad[lev];
        }
        if (idrv == 1) {
          if (iclddn == 1) {
            d_radclru_dt = d_radclru_dt * (1.0 - atrans[lev]);
            d_clrurad_dt[lev] = d_clrurad_dt[lev] + d_radclru_dt;
          } else {
            d_radclru_dt = d_radlu_dt;
            d_clrurad_dt[lev] = d_urad_dt[lev];
          }
        }
      }
    }
    for (int lev = nlayers; lev >= 0; --lev) {  // band output (:762-775)
      const double uflux = urad[lev] * wtdiff, dflux = drad[lev] * wtdiff;
      urad[lev] = 0.0;
      drad[lev] = 0.0;
      c.totuflux[lev] = c.totuflux[lev] + uflux * delwave[iband - 1];
      c.totdflux[lev] = c.totdflux[lev] + dflux * delwave[iband - 1];
      const double uclfl = clrurad[lev] * wtdiff, dclfl = clrdrad[lev] * wtdiff;
      clrurad[lev] = 0.0;
      clrdrad[lev] = 0.0;
      c.totuclfl[lev] = c.totuclfl[lev] + uclfl * delwave[iband - 1];
      c.totdclfl[lev] = c.totdclfl[lev] + dclfl * delwave[iband - 1];
    }
    if (idrv == 1) {
      for (int lev = nlayers; lev >= 0; --lev) {
        const double duflux_dt = d_urad_dt[lev] * wtdiff;
        d_urad_dt[lev] = 0.0;
        c.dtotuflux_dt[lev] = c.dtotuflux_dt[lev] + duflux_dt * delwave[iband - 1] * fluxfac;
        const double duclfl_dt = d_clrurad_dt[lev] * wtdiff;
        d_clrurad_dt[lev] = 0.0;
        c.dtotuclfl_dt[lev] = c.dtotuclfl_dt[lev] + duclfl_dt * delwave[iband - 1] * fluxfac;
      }
    }
  }
  c.totuflux[0] = c.totuflux[0] * fluxfac;  // :779-806
  c.totdflux[0] = c.totdflux[0] * fluxfac;
  c.fnet[0] = c.totuflux[0] - c.totdflux[0];
  c.totuclfl[0] = c.totuclfl[0] * fluxfac;
  c.totdclfl[0] = c.totdclfl[0] * fluxfac;
  c.fnetc[0] = c.totuclfl[0] - c.totdclfl[0];
  for (int lev = 1; lev <= nlayers; ++lev) {
    c.totuflux[lev] = c.totuflux[lev] * fluxfac;
    c.totdflux[lev] = c.totdflux[lev] * fluxfac;
    c.fnet[lev] = c.totuflux[lev] - c.totdflux[lev];
    c.totuclfl[lev] = c.totuclfl[lev] * fluxfac;
    c.totdclfl[lev] = c.totdclfl[lev] * fluxfac;
    c.fnetc[lev] = c.totuclfl[lev] - c.totdclfl[lev];
    const int l = lev - 1;
    c.htr[l] = heatfac * (c.fnet[l] - c.fnet[lev]) / (c.pz[l] - c.pz[lev]);
    c.htrc[l] = heatfac * (c.fnetc[l] - c.fnetc[lev]) / (c.pz[l] - c.pz[lev]);
  }
  c.htr[nlayers] = 0.0;
  c.htrc[nlayers] = 0.0;
}

}  // namespace
extern "C" int ora_cldprop(int nlayers, int inflag, int iceflag, int liqflag, const double* cldfrac,
                           const double* tauc, const double* ciwp, const double* clwp, const double* rei,
                           const double* rel, int* ncbands_out, double* taucloud);
namespace {

// one column through inatm..rtrnmc (rrtmg_lw_rad.f90:486-570)
struct Args {
  int ncol, nlay, icld, idrv;
  const double *play, *plev, *tlay, *tlev, *tsfc, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr,
      *o2vmr, *cfc11vmr, *cfc12vmr, *cfc22vmr, *ccl4vmr, *emis;
  int inflglw, iceflglw, liqflglw;
  const double *cldfmcl, *taucmcl, *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl, *tauaer;
};

// The operation-counting build (flop_count.h) defines ORA_PHASE to attribute
// the operations counted so far to a phase; in the oracle itself it is empty.
#ifndef ORA_PHASE
#define ORA_PHASE(k)
#endif

int run_column(const Args& a, int iplon, Col& c) {
  const int iaer = 10;
  ORA_PHASE(-1);
  inatm(iplon, a.ncol, a.nlay, a.icld, iaer, a.play, a.plev, a.tlay, a.tlev, a.tsfc, a.h2ovmr,
        a.o3vmr, a.co2vmr, a.ch4vmr, a.n2ovmr, a.o2vmr, a.cfc11vmr, a.cfc12vmr, a.cfc22vmr,
        a.ccl4vmr, a.emis, a.inflglw, a.iceflglw, a.liqflglw, a.cldfmcl, a.taucmcl, a.ciwpmcl,
        a.clwpmcl, a.reicmcl, a.relqmcl, a.tauaer, c);
  ORA_PHASE(0);
  int err = cldprmc(c);
  if (err) return err;
  ORA_PHASE(1);
  err = setcoef(c, a.idrv);
  if (err) return err;
  ORA_PHASE(2);
  taumol(c);
  for (int k = 1; k <= c.nlayers; ++k)
    for (int ig = 1; ig <= NGPT; ++ig) c.TAUT(k, ig) = c.TAUG(k, ig) + c.TAUA(k, ngb[ig - 1]);
  ORA_PHASE(3);
  rtrnmc(c, a.idrv);
  ORA_PHASE(4);
  return 0;
}

// Band-level clouds of the non-McICA driver (rrtmg_lw_rad.nomcica.f90):
// cldfr (ncol, nlay), taucld (16, ncol, nlay), cicewp, cliqwp, reice, reliq
// (ncol, nlay).
struct CloudsR {
  const double *cldfr, *taucld, *cicewp, *cliqwp, *reice, *reliq;
};

// one column of the non-McICA driver (rrtmg_lw_rad.nomcica.f90:470-553:
// inatm, cldprop, setcoef, taumol, then rtrn for icld = 1 and rtrnmr
// otherwise; the state part of inatm is the McICA driver's, its cloud part
// :886-920 copies the band-level clouds below for icld >= 1 and leaves them
// zero for icld = 0)
int run_column_rtrn(const Args& a, const CloudsR& cl, int iplon, Col& c) {
  const int iaer = 10;
  inatm(iplon, a.ncol, a.nlay, 0, iaer, a.play, a.plev, a.tlay, a.tlev, a.tsfc, a.h2ovmr, a.o3vmr,
        a.co2vmr, a.ch4vmr, a.n2ovmr, a.o2vmr, a.cfc11vmr, a.cfc12vmr, a.cfc22vmr, a.ccl4vmr, a.emis,
        a.inflglw, a.iceflglw, a.liqflglw, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
        a.tauaer, c);
  const int nl = c.nlayers;
  std::vector<double> cf(nl), ci(nl), cw(nl), ri(nl), rl(nl), tc(16 * nl);
  for (int l = 1; l <= nl && a.icld >= 1; ++l) {
    const size_t o = (iplon - 1) + (size_t)a.ncol * (l - 1);
    cf[l - 1] = cl.cldfr[o];
    ci[l - 1] = cl.cicewp[o];
    cw[l - 1] = cl.cliqwp[o];
    ri[l - 1] = cl.reice[o];
    rl[l - 1] = cl.reliq[o];
    for (int n = 1; n <= 16; ++n) tc[(n - 1) + 16 * (l - 1)] = cl.taucld[(n - 1) + 16 * o];
  }
  c.rtrn = 1;
  c.cldfr_lay.assign(nl + 1, 0.0);
  for (int l = 1; l <= nl; ++l) c.cldfr_lay[l] = cf[l - 1];
  c.taucloud.assign((size_t)nl * 16, 0.0);
  int err = ora_cldprop(nl, a.inflglw, a.iceflglw, a.liqflglw, cf.data(), tc.data(), ci.data(), cw.data(),
                        ri.data(), rl.data(), &c.ncbands, c.taucloud.data());
  if (err) return err;
  err = setcoef(c, a.idrv);
  if (err) return err;
  taumol(c);
  for (int k = 1; k <= c.nlayers; ++k)
    for (int ig = 1; ig <= NGPT; ++ig) c.TAUT(k, ig) = c.TAUG(k, ig) + c.TAUA(k, ngb[ig - 1]);
  if (a.icld == 1)
    rtrnmc(c, a.idrv);
  else
    rtrnmr(c, a.idrv);
  c.rtrn = 0;
  return 0;
}

}  // namespace

// ================================================================ C API
extern "C" {

int ora_init(double cpdair, const char* ref_path, const char* k_path) {
  g_tab.clear();
  if (!load_container(ref_path) || !load_container(k_path)) return ERR_ARGS;
  pref = T("pref"); preflog = T("preflog"); tref = T("tref"); chi_mls = T("chi_mls");
  totplnk = T("totplnk"); totplk16 = T("totplk16");
  totplnkderiv = T("totplnkderiv"); totplk16deriv = T("totplk16deriv");
  absice0 = T("absice0"); absice1 = T("absice1"); absice2 = T("absice2");
  absice3 = T("absice3"); absliq1 = T("absliq1");
  abscld1 = T("abscld1")[0]; absliq0 = T("absliq0")[0];
  grav = T("grav")[0]; avogad = T("avogad")[0];
  double secdy = T("secdy")[0];
  for (int i = 0; i < NGPT; ++i) ngb[i] = TI("ngb")[i];
  for (int i = 0; i < NBND; ++i) {
    ngs[i] = TI("ngs")[i]; nspa[i] = TI("nspa")[i]; nspb[i] = TI("nspb")[i];
    delwave[i] = T("delwave")[i];
  }
  // rrtmg_lw_init.f90:120-142 lookup tables; lwdatinit :298 heatfac
  const double expeps = 1.e-20, pade = 0.278;
  tau_tbl[0] = 0.0; tau_tbl[NTBL] = 1.e10;
  exp_tbl[0] = 1.0; exp_tbl[NTBL] = expeps;
  tfn_tbl[0] = 0.0; tfn_tbl[NTBL] = 1.0;
  bpade = 1.0 / pade;
  for (int itr = 1; itr <= NTBL - 1; ++itr) {
    // tfn = real(itr)/real(ntbl): a single-precision division, then promoted
    double tfn = (double)((float)itr / (float)NTBL);
    tau_tbl[itr] = bpade * tfn / (1.0 - tfn);
    exp_tbl[itr] = std::exp(-tau_tbl[itr]);
    if (exp_tbl[itr] <= expeps) exp_tbl[itr] = expeps;
    if (tau_tbl[itr] < 0.06)
      tfn_tbl[itr] = tau_tbl[itr] / 6.0;
    else
      tfn_tbl[itr] = 1.0 - 2.0 * ((1.0 / tau_tbl[itr]) - (exp_tbl[itr] / (1. - exp_tbl[itr])));
  }
  heatfac = grav * secdy / (cpdair * 1.e2);
  oneminus = 1.0 - 1.e-6;
  double pi = 2.0 * std::asin(1.0);
  fluxfac = pi * 2.e4;
  g_ready = true;
  return 0;
}

int ora_rrtmg_lw(int ncol, int nlay, int* icld, int idrv, const double* play, const double* plev,
                 const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                 const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                 const double* n2ovmr, const double* o2vmr, const double* cfc11vmr,
                 const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
                 const double* emis, int inflglw, int iceflglw, int liqflglw,
                 const double* cldfmcl, const double* taucmcl, const double* ciwpmcl,
                 const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                 const double* tauaer, double* uflx, double* dflx, double* hr, double* uflxc,
                 double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt, int nthreads) {
  if (!g_ready) return ERR_NOT_INIT;
  if (ncol < 0 || nlay < 1) return ERR_ARGS;
  if (*icld < 0 || *icld > 3) *icld = 2;  // rrtmg_lw_rad.f90:465
  Args a{ncol, nlay, *icld, idrv, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr,
         n2ovmr, o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, inflglw, iceflglw,
         liqflglw, cldfmcl, taucmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, tauaer};
  auto work = [&](int c0, int c1, int* err) {
    Col c;
    for (int iplon = c0 + 1; iplon <= c1; ++iplon) {
      int e = run_column(a, iplon, c);
      if (e) { *err = e; return; }
      // rrtmg_lw_rad.f90:572-590
      for (int k = 0; k <= nlay; ++k) {
        size_t o = (iplon - 1) + (size_t)ncol * k;
        uflx[o] = c.totuflux[k]; dflx[o] = c.totdflux[k];
        uflxc[o] = c.totuclfl[k]; dflxc[o] = c.totdclfl[k];
      }
      for (int k = 0; k <= nlay - 1; ++k) {
        size_t o = (iplon - 1) + (size_t)ncol * k;
        hr[o] = c.htr[k]; hrc[o] = c.htrc[k];
      }
      if (idrv == 1) {
        for (int k = 0; k <= nlay; ++k) {
          size_t o = (iplon - 1) + (size_t)ncol * k;
          duflx_dt[o] = c.dtotuflux_dt[k]; duflxc_dt[o] = c.dtotuclfl_dt[k];
        }
      }
    }
  };
  if (nthreads <= 1 || ncol < 2) {
    int err = 0;
    work(0, ncol, &err);
    return err;
  }
  std::vector<std::thread> th;
  std::vector<int> errs(nthreads, 0);
  for (int t = 0; t < nthreads; ++t) {
    int c0 = (int)((long long)ncol * t / nthreads), c1 = (int)((long long)ncol * (t + 1) / nthreads);
    th.emplace_back(work, c0, c1, &errs[t]);
  }
  for (auto& t : th) t.join();
  for (int e : errs)
    if (e) return e;
  return 0;
}

// rrtmg_lw of the non-McICA driver (rrtmg_lw_rad.nomcica.f90:99-560): icld
// outside 0..3 becomes 2 (:456); icld 1 takes random cloud overlap (rtrn),
// the others maximum/random overlap (rtrnmr; icld 0 with no clouds).
int ora_rrtmg_lw_nomcica(int ncol, int nlay, int* icld_io, int idrv, const double* play, const double* plev,
                      const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                      const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                      const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr,
                      const double* cfc22vmr, const double* ccl4vmr, const double* emis, int inflglw,
                      int iceflglw, int liqflglw, const double* cldfr, const double* taucld,
                      const double* cicewp, const double* cliqwp, const double* reice, const double* reliq,
                      const double* tauaer, double* uflx, double* dflx, double* hr, double* uflxc,
                      double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt) {
  if (!g_ready) return ERR_NOT_INIT;
  if (ncol < 0 || nlay < 1 || !icld_io) return ERR_ARGS;
  if (*icld_io < 0 || *icld_io > 3) *icld_io = 2;
  const int icld = *icld_io;
  Args a{ncol, nlay, icld, idrv, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr,
         n2ovmr, o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, inflglw, iceflglw,
         liqflglw, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, tauaer};
  CloudsR cl{cldfr, taucld, cicewp, cliqwp, reice, reliq};
  Col c;
  for (int iplon = 1; iplon <= ncol; ++iplon) {
    const int e = run_column_rtrn(a, cl, iplon, c);
    if (e) return e;
    for (int k = 0; k <= nlay; ++k) {
      const size_t o = (iplon - 1) + (size_t)ncol * k;
      uflx[o] = c.totuflux[k]; dflx[o] = c.totdflux[k];
      uflxc[o] = c.totuclfl[k]; dflxc[o] = c.totdclfl[k];
      if (idrv == 1) { duflx_dt[o] = c.dtotuflux_dt[k]; duflxc_dt[o] = c.dtotuclfl_dt[k]; }
    }
    for (int k = 0; k <= nlay - 1; ++k) {
      const size_t o = (iplon - 1) + (size_t)ncol * k;
      hr[o] = c.htr[k]; hrc[o] = c.htrc[k];
    }
  }
  return 0;
}

int ora_column_intermediates(int ncol, int nlay, int icol, int icld, const double* play,
                             const double* plev, const double* tlay, const double* tlev,
                             const double* tsfc, const double* h2ovmr, const double* o3vmr,
                             const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                             const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr,
                             const double* cfc22vmr, const double* ccl4vmr, const double* emis,
                             int inflglw, int iceflglw, int liqflglw, const double* cldfmcl,
                             const double* taucmcl, const double* ciwpmcl, const double* clwpmcl,
                             const double* reicmcl, const double* relqmcl, const double* tauaer,
                             double* taug, double* fracs, double* taut, double* planklay,
                             double* planklev, double* plankbnd, double* taucmc, int* laytrop) {
  if (!g_ready) return ERR_NOT_INIT;
  Args a{ncol, nlay, icld, 1, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr,
         n2ovmr, o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, inflglw, iceflglw,
         liqflglw, cldfmcl, taucmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, tauaer};
  Col c;
  int e = run_column(a, icol, c);
  if (e) return e;
  for (int l = 1; l <= nlay; ++l)
    for (int ig = 1; ig <= NGPT; ++ig) {
      size_t o = (l - 1) + (size_t)nlay * (ig - 1);
      if (taug) taug[o] = c.TAUG(l, ig);
      if (fracs) fracs[o] = c.FRACS(l, ig);
      if (taut) taut[o] = c.TAUT(l, ig);
      if (taucmc) taucmc[(ig - 1) + NGPT * (l - 1)] = c.CF(c.taucmc, ig, l);
    }
  for (int b = 1; b <= 16; ++b) {
    for (int l = 1; l <= nlay; ++l)
      if (planklay) planklay[(l - 1) + nlay * (b - 1)] = c.PLAY(l, b);
    for (int l = 0; l <= nlay; ++l)
      if (planklev) planklev[l + (nlay + 1) * (b - 1)] = c.PLEV(l, b);
    if (plankbnd) plankbnd[b - 1] = c.plankbnd[b - 1];
  }
  if (laytrop) *laytrop = c.laytrop;
  return 0;
}

// rrtmg_lw_cldprop.f90:50-295
int ora_cldprop(int nlayers, int inflag, int iceflag, int liqflag, const double* cldfrac,
                const double* tauc, const double* ciwp, const double* clwp, const double* rei,
                const double* rel, int* ncbands_out, double* taucloud) {
  if (!g_ready) return ERR_NOT_INIT;
  const double cldmin = 1.e-20;
  static const int icb[3][16] = {{1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
                                 {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5},
                                 {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16}};
  double abscoice[16] = {0}, abscoliq[16] = {0};
  int ncbands = 1, iceind = 0, liqind = 0;
  std::vector<double> tauctot(nlayers + 1, 0.0);
  for (int lay = 1; lay <= nlayers; ++lay)
    for (int ib = 1; ib <= 16; ++ib) {
      taucloud[(lay - 1) + nlayers * (ib - 1)] = 0.0;
      tauctot[lay] = tauctot[lay] + tauc[(ib - 1) + 16 * (lay - 1)];
    }
  for (int lay = 1; lay <= nlayers; ++lay) {
    double cwp = ciwp[lay - 1] + clwp[lay - 1];
    if (cldfrac[lay - 1] >= cldmin && (cwp >= cldmin || tauctot[lay] >= cldmin)) {
      if (inflag == 0) {
        ncbands = 16;
        for (int ib = 1; ib <= ncbands; ++ib)
          taucloud[(lay - 1) + nlayers * (ib - 1)] = tauc[(ib - 1) + 16 * (lay - 1)];
      } else if (inflag == 1) {
        ncbands = 16;
        for (int ib = 1; ib <= ncbands; ++ib) taucloud[(lay - 1) + nlayers * (ib - 1)] = abscld1 * cwp;
      } else if (inflag == 2) {
        double radice = rei[lay - 1];
        if (ciwp[lay - 1] == 0.0) {
          abscoice[0] = 0.0;
          iceind = 0;
        } else if (iceflag == 0) {
          if (radice < 10.0) return ERR_ICE_SMALL;
          abscoice[0] = absice0[0] + absice0[1] / radice;
          iceind = 0;
        } else if (iceflag == 1) {
          if (radice < 13.0 || radice > 130.0) return ERR_ICE_BOUNDS;
          ncbands = 5;
          for (int ib = 1; ib <= ncbands; ++ib)
            abscoice[ib - 1] = absice1[0 + 2 * (ib - 1)] + absice1[1 + 2 * (ib - 1)] / radice;
          iceind = 1;
        } else if (iceflag == 2) {
          if (radice < 5.0 || radice > 131.0) return ERR_ICE_BOUNDS;
          ncbands = 16;
          double factor = (radice - 2.0) / 3.0;
          int index = (int)factor;
          if (index == 43) index = 42;
          double fint = factor - (double)(float)index;
          for (int ib = 1; ib <= ncbands; ++ib) {
            const double* a = absice2 + 43 * (ib - 1);
            abscoice[ib - 1] = a[index - 1] + fint * (a[index] - (a[index - 1]));
          }
          iceind = 2;
        } else if (iceflag == 3) {
          if (radice < 5.0 || radice > 140.0) return ERR_DGE_BOUNDS;
          ncbands = 16;
          double factor = (radice - 2.0) / 3.0;
          int index = (int)factor;
          if (index == 46) index = 45;
          double fint = factor - (double)(float)index;
          for (int ib = 1; ib <= ncbands; ++ib) {
            const double* a = absice3 + 46 * (ib - 1);
            abscoice[ib - 1] = a[index - 1] + fint * (a[index] - (a[index - 1]));
          }
          iceind = 2;
        }
        if (clwp[lay - 1] == 0.0) {
          abscoliq[0] = 0.0;
          liqind = 0;
          if (iceind == 1) iceind = 2;
        } else if (liqflag == 0) {
          abscoliq[0] = absliq0;
          liqind = 0;
          if (iceind == 1) iceind = 2;
        } else if (liqflag == 1) {
          double radliq = rel[lay - 1];
          if (radliq < 2.5 || radliq > 60.0) return ERR_LIQ_BOUNDS;
          int index = (int)(radliq - 1.5);
          if (index == 0) index = 1;
          if (index == 58) index = 57;
          double fint = radliq - 1.5 - (double)(float)index;
          ncbands = 16;
          for (int ib = 1; ib <= ncbands; ++ib) {
            const double* a = absliq1 + 58 * (ib - 1);
            abscoliq[ib - 1] = a[index - 1] + fint * (a[index] - (a[index - 1]));
          }
          liqind = 2;
        }
        for (int ib = 1; ib <= ncbands; ++ib)
          taucloud[(lay - 1) + nlayers * (ib - 1)] =
              ciwp[lay - 1] * abscoice[icb[iceind][ib - 1] - 1] + clwp[lay - 1] * abscoliq[icb[liqind][ib - 1] - 1];
      }
    }
  }
  *ncbands_out = ncbands;
  return 0;
}

// ---------------------------------------------------------------- random numbers
namespace {
// MersenneTwister module, mcica_random_numbers.f90:77-306 (uint32 arithmetic =
// the Fortran int32 wraparound with logical ishft)
struct MT {
  uint32_t s[624];
  int cur;
  explicit MT(int32_t seed) {
    s[0] = (uint32_t)seed;
    for (int i = 1; i < 624; ++i) s[i] = 1812433253u * (s[i - 1] ^ (s[i - 1] >> 30)) + (uint32_t)i;
    cur = 624;
  }
  static uint32_t twist(uint32_t u, uint32_t v) {
    uint32_t mix = (u & 0x80000000u) | (v & 0x7fffffffu);
    return (mix >> 1) ^ ((v & 1u) ? 0x9908b0dfu : 0u);
  }
  void next_state() {
    for (int k = 0; k <= 624 - 397 - 1; ++k) s[k] = s[k + 397] ^ twist(s[k], s[k + 1]);
    for (int k = 624 - 397; k <= 624 - 2; ++k) s[k] = s[k + 397 - 624] ^ twist(s[k], s[k + 1]);
    s[623] = s[396] ^ twist(s[623], s[0]);
    cur = 0;
  }
  static uint32_t temper(uint32_t y) {
    uint32_t x = y ^ (y >> 11);
    x = x ^ ((x << 7) & 0x9d2c5680u);
    x = x ^ ((x << 15) & 0xefc60000u);
    return x ^ (x >> 18);
  }
  uint32_t get_int() {
    if (cur >= 624) next_state();
    return temper(s[cur++]);
  }
  // getRandomReal (:276-295): both branches equal u32 / (2^32 - 1)
  double get_real() {
    int32_t li = (int32_t)get_int();
    if (li < 0) return ((double)li + 4294967296.0) / (4294967296.0 - 1.0);
    return ((double)li) / (4294967296.0 - 1.0);
  }
};

// kissvec (mcica_subcol_gen_lw.f90:711-743) for one column
struct Kiss {
  uint32_t s1, s2, s3, s4;
  double next() {
    s1 = 69069u * s1 + 1327217885u;
    auto m = [](uint32_t k, int n) { return n >= 0 ? (k ^ (k << n)) : (k ^ (k >> (-n))); };
    s2 = m(m(m(s2, 13), -17), 5);
    s3 = 18000u * (s3 & 65535u) + (s3 >> 16);
    s4 = 30903u * (s4 & 65535u) + (s4 >> 16);
    int32_t kiss = (int32_t)(s1 + s2 + (s3 << 16) + s4);
    return kiss * 2.328306e-10 + 0.5;
  }
};
}  // namespace

void ora_mt_draws(int32_t seed, int n, uint32_t* ints, double* reals) {
  MT a(seed), b(seed);
  for (int i = 0; i < n; ++i) {
    if (ints) ints[i] = a.get_int();
    if (reals) reals[i] = b.get_real();
  }
}

void ora_kiss_draws(int32_t s1, int32_t s2, int32_t s3, int32_t s4, int n, double* reals) {
  Kiss k{(uint32_t)s1, (uint32_t)s2, (uint32_t)s3, (uint32_t)s4};
  for (int i = 0; i < n; ++i) reals[i] = k.next();
}

}  // extern "C"

namespace {

// generate_stochastic_clouds (mcica_subcol_gen_lw.f90:403-703) and its
// shortwave twin generate_stochastic_clouds_sw (mcica_subcol_gen_sw.f90:
// 298-757): nsub sub-columns, sub-column isub takes the band optical
// properties of band ngb_of[isub] - band0 (tauc is (nbnd, ncol, nlay)); the
// shortwave one also copies ssac, asmc, fsfc (1, 0, 0 in clear cells).
int mcica_generate(int nsub, const int* ngb_of, int band0, int nbnd, int ncol, int nlay, int icld, int permuteseed,
                   int* irng, const double* play, const double* cld, const double* ciwp, const double* clwp,
                   const double* rei, const double* rel, const double* tauc, const double* ssac, const double* asmc,
                   const double* fsfc, const double* alpha, double* cld_stoch, double* ciwp_stoch,
                   double* clwp_stoch, double* reicmcl, double* relqmcl, double* tauc_stoch, double* ssac_stoch,
                   double* asmc_stoch, double* fsfc_stoch) {
  if (icld == 0) return 0;
  if (icld < 0 || icld > 5) return ERR_ICLD;
  size_t nc = (size_t)ncol * nlay;
  for (size_t i = 0; i < nc; ++i) { reicmcl[i] = rei[i]; relqmcl[i] = rel[i]; }
  std::vector<double> pmid(nc);
  for (size_t i = 0; i < nc; ++i) pmid[i] = play[i] * 1.e2;
  if (*irng != 0) *irng = 1;
  const double cldmin = 1.0e-20;
  std::vector<double> cldf(nc);
  for (size_t i = 0; i < nc; ++i) {
    cldf[i] = cld[i];
    if (cldf[i] < cldmin) cldf[i] = 0.0;
  }
  auto IX = [&](int isub, int i, int ilev) {  // (nsub, ncol, nlay), 1-based
    return (size_t)(isub - 1) + (size_t)nsub * ((size_t)(i - 1) + (size_t)ncol * (ilev - 1));
  };
  auto CI = [&](int i, int ilev) { return (size_t)(i - 1) + (size_t)ncol * (ilev - 1); };
  std::vector<double> CDF(nc * nsub), CDF2;
  std::vector<Kiss> kiss;
  MT* mt = nullptr;
  if (*irng == 0) {
    kiss.resize(ncol);
    for (int i = 1; i <= ncol; ++i) {
      if (nlay < 4 || pmid[CI(i, 1)] < pmid[CI(i, 2)]) return ERR_KISS_PMID;
      auto sd = [&](int l) { double p = pmid[CI(i, l)]; return (int32_t)((p - (double)(int)p) * 1000000000); };
      kiss[i - 1] = Kiss{(uint32_t)sd(1), (uint32_t)sd(2), (uint32_t)sd(3), (uint32_t)sd(4)};
    }
    for (int k = 1; k <= permuteseed; ++k)
      for (int i = 0; i < ncol; ++i) kiss[i].next();
  } else {
    mt = new MT(permuteseed);
  }
  auto kiss_all = [&](std::vector<double>& r) {
    r.resize(ncol);
    for (int i = 0; i < ncol; ++i) r[i] = kiss[i].next();
  };
  std::vector<double> rn;
  if (icld == 1 || icld == 2) {
    if (*irng == 0) {
      for (int isub = 1; isub <= nsub; ++isub)
        for (int ilev = 1; ilev <= nlay; ++ilev) {
          kiss_all(rn);
          for (int i = 1; i <= ncol; ++i) CDF[IX(isub, i, ilev)] = rn[i - 1];
        }
    } else {
      for (int isub = 1; isub <= nsub; ++isub)
        for (int i = 1; i <= ncol; ++i)
          for (int ilev = 1; ilev <= nlay; ++ilev) CDF[IX(isub, i, ilev)] = mt->get_real();
    }
    if (icld == 2) {
      for (int ilev = 2; ilev <= nlay; ++ilev)
        for (int i = 1; i <= ncol; ++i)
          for (int isub = 1; isub <= nsub; ++isub) {
            if (CDF[IX(isub, i, ilev - 1)] > 1.0 - cldf[CI(i, ilev - 1)])
              CDF[IX(isub, i, ilev)] = CDF[IX(isub, i, ilev - 1)];
            else
              CDF[IX(isub, i, ilev)] = CDF[IX(isub, i, ilev)] * (1.0 - cldf[CI(i, ilev - 1)]);
          }
    }
  } else if (icld == 3) {
    if (*irng == 0) {
      for (int isub = 1; isub <= nsub; ++isub) {
        kiss_all(rn);
        for (int ilev = 1; ilev <= nlay; ++ilev)
          for (int i = 1; i <= ncol; ++i) CDF[IX(isub, i, ilev)] = rn[i - 1];
      }
    } else {
      for (int isub = 1; isub <= nsub; ++isub)
        for (int i = 1; i <= ncol; ++i) {
          double r = mt->get_real();
          for (int ilev = 1; ilev <= nlay; ++ilev) CDF[IX(isub, i, ilev)] = r;
        }
    }
  } else {  // icld 4, 5: exponential (random) overlap with alpha
    CDF2.resize(nc * nsub);
    for (int isub = 1; isub <= nsub; ++isub)
      for (int i = 1; i <= ncol; ++i)
        for (int ilev = 1; ilev <= nlay; ++ilev) {
          if (*irng == 0) {
            // kissvec over all columns, keeping column i's value (:581-586)
            kiss_all(rn); CDF[IX(isub, i, ilev)] = rn[i - 1];
            kiss_all(rn); CDF2[IX(isub, i, ilev)] = rn[i - 1];
          } else {
            CDF[IX(isub, i, ilev)] = mt->get_real();
            CDF2[IX(isub, i, ilev)] = mt->get_real();
          }
        }
    for (int ilev = 2; ilev <= nlay; ++ilev)
      for (int i = 1; i <= ncol; ++i)
        for (int isub = 1; isub <= nsub; ++isub)
          if (CDF2[IX(isub, i, ilev)] < alpha[CI(i, ilev)]) CDF[IX(isub, i, ilev)] = CDF[IX(isub, i, ilev - 1)];
  }
  delete mt;
  for (int ilev = 1; ilev <= nlay; ++ilev)
    for (int i = 1; i <= ncol; ++i)
      for (int isub = 1; isub <= nsub; ++isub) {
        size_t o = IX(isub, i, ilev);
        bool cloudy = CDF[o] >= 1.0 - cldf[CI(i, ilev)];
        const int n = ngb_of[isub - 1] - band0;  // 1-based band of the optical properties
        const size_t ob = (size_t)(n - 1) + (size_t)nbnd * CI(i, ilev);
        if (cloudy) {
          cld_stoch[o] = 1.0;
          clwp_stoch[o] = clwp[CI(i, ilev)];
          ciwp_stoch[o] = ciwp[CI(i, ilev)];
          tauc_stoch[o] = tauc[ob];
          if (ssac_stoch) {
            ssac_stoch[o] = ssac[ob];
            asmc_stoch[o] = asmc[ob];
            fsfc_stoch[o] = fsfc[ob];
          }
        } else {
          cld_stoch[o] = 0.0;
          clwp_stoch[o] = 0.0;
          ciwp_stoch[o] = 0.0;
          tauc_stoch[o] = 0.0;
          if (ssac_stoch) {
            ssac_stoch[o] = 1.0;
            asmc_stoch[o] = 0.0;
            fsfc_stoch[o] = 0.0;
          }
        }
      }
  return 0;
}

}  // namespace

extern "C" {

// mcica_subcol_lw (mcica_subcol_gen_lw.f90:183-265)
int ora_mcica_subcol_lw(int ncol, int nlay, int icld, int permuteseed, int* irng,
                        const double* play, const double* cld, const double* ciwp,
                        const double* clwp, const double* rei, const double* rel,
                        const double* tauc, const double* alpha, double* cld_stoch,
                        double* ciwp_stoch, double* clwp_stoch, double* reicmcl, double* relqmcl,
                        double* tauc_stoch) {
  if (!g_ready) return ERR_NOT_INIT;
  return mcica_generate(NGPT, ngb, 0, 16, ncol, nlay, icld, permuteseed, irng, play, cld, ciwp, clwp, rei, rel, tauc,
                        nullptr, nullptr, nullptr, alpha, cld_stoch, ciwp_stoch, clwp_stoch, reicmcl, relqmcl,
                        tauc_stoch, nullptr, nullptr, nullptr);
}

// mcica_subcol_sw (mcica_subcol_gen_sw.f90:181-296): 112 sub-columns; the
// g-point bands are the shortwave ones (rrtmg_sw_init.f90 swcmbdat ngb:
// 6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12 g-points in bands 16..29);
// tauc, ssac, asmc, fsfc are (14, ncol, nlay).  Needs no oracle tables.
int ora_mcica_subcol_sw(int ncol, int nlay, int icld, int permuteseed, int* irng, const double* play,
                        const double* cld, const double* ciwp, const double* clwp, const double* rei,
                        const double* rel, const double* tauc, const double* ssac, const double* asmc,
                        const double* fsfc, const double* alpha, double* cld_stoch, double* ciwp_stoch,
                        double* clwp_stoch, double* reicmcl, double* relqmcl, double* tauc_stoch,
                        double* ssac_stoch, double* asmc_stoch, double* fsfc_stoch) {
  static const int ng[14] = {6, 12, 8, 8, 10, 10, 2, 10, 8, 6, 6, 8, 6, 12};
  int ngb_sw[112], k = 0;
  for (int b = 0; b < 14; ++b)
    for (int g = 0; g < ng[b]; ++g) ngb_sw[k++] = 16 + b;
  return mcica_generate(112, ngb_sw, 15, 14, ncol, nlay, icld, permuteseed, irng, play, cld, ciwp, clwp, rei, rel,
                        tauc, ssac, asmc, fsfc, alpha, cld_stoch, ciwp_stoch, clwp_stoch, reicmcl, relqmcl,
                        tauc_stoch, ssac_stoch, asmc_stoch, fsfc_stoch);
}

void ora_get_tables(double* tau, double* ex, double* tfn, double* hf, double* ff) {
  for (int i = 0; i <= NTBL; ++i) {
    if (tau) tau[i] = tau_tbl[i];
    if (ex) ex[i] = exp_tbl[i];
    if (tfn) tfn[i] = tfn_tbl[i];
  }
  if (hf) *hf = heatfac;
  if (ff) *ff = fluxfac;
}

const char* ora_error_string(int code) {
  switch (code) {
    case ERR_OK: return "ok";
    case ERR_NOT_INIT: return "oracle not initialised";
    case ERR_INFLAG1: return "INFLAG = 1 OPTION NOT AVAILABLE WITH MCICA";
    case ERR_ICE_SMALL: return "ICE RADIUS TOO SMALL";
    case ERR_ICE_BOUNDS: return "ICE RADIUS OUT OF BOUNDS";
    case ERR_DGE_BOUNDS: return "ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS";
    case ERR_LIQ_BOUNDS: return "LIQUID EFFECTIVE RADIUS OUT OF BOUNDS";
    case ERR_ICLD: return "MCICA_SUBCOL_LW: INVALID ICLD";
    case ERR_KISS_PMID: return "MCICA_SUBCOL: KISSVEC SEED GENERATOR REQUIRES PMID FROM BOTTOM FOUR LAYERS.";
    case ERR_LAYTROP: return "lower-atmosphere layers are not a contiguous prefix (pressure must decrease with layer index)";
    case ERR_ARGS: return "invalid arguments or unreadable tables";
  }
  return "unknown error";
}

}  // extern "C"
