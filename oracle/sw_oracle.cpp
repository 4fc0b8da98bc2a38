// CPU oracle for RRTMG_SW -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Double-precision restatement of the reference's shortwave McICA path
// (src/rrtmg/RRTMG_SW/src of luflarois/brams), statement for statement:
// rrtmg_sw_rad.f90 (rrtmg_sw :243-586, inatm_sw :612-1040), cldprmc_sw
// (rrtmg_sw_cldprmc.f90:43-338), setcoef_sw (rrtmg_sw_setcoef.f90:27-240),
// taumol_sw (rrtmg_sw_taumol.f90:50-1787), spcvmc_sw (rrtmg_sw_spcvmc.f90:
// 30-664), reftra_sw (rrtmg_sw_reftra.f90:27-330), vrtqdr_sw
// (rrtmg_sw_vrtqdr.f90:24-171), the lookup table of rrtmg_sw_ini
// (rrtmg_sw_init.f90:99-118) and the band cloud optics cldprop_sw
// (rrtmg_sw_cldprop.f90:53-365) the driver feeds to the McICA generator.  Tables come from sw_tables.gbsw, which
// brams_gb300/data/extract_sw_tables.py extracts from the reference source
// and reduces with the reference's cmbgb routines.
//
// Fortran semantics kept: 1-based subscripts (the accessors take Fortran
// indices), truncating int(), mod(x, 1) for x >= 0, default-real literals
// rounded through float (none on this path's arithmetic but the parameter
// rrsw_scon, read from the table file), left-to-right evaluation.
//
// Scope: solar variability option isolvar < 0 (BRAMS's -1), aerosol options
// iaer 0 and 10, cloud options inflag 0 and 2 with iceflag 1-3 and liqflag
// 1; the other options return ERR_UNSUPPORTED (iceflag 0 and liqflag 0
// with a nonzero water path read coefficients the reference never sets).
// Where the reference reads storage it never wrote -- jp(nlayers+1) in the
// lower-atmosphere solar-layer search of bands 18-26 (taumol.f90:549 etc.),
// jp(0) in the upper-atmosphere search of bands 16, 17, 27-29 when laytrop
// is 0 -- the value is taken as 0 (the condition then fails), and a band
// whose solar-source layer is never reached keeps sfluxzen 0.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include <stdint.h>

namespace {

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
    ok = std::fread(name, 1, 48, f) == 48 && std::fread(hdr, 4, 6, f) == 6 && std::fread(&nbytes, 8, 1, f) == 1;
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
  return it == g_tab.end() ? nullptr : it->second.d.data();
}
const int* TI(const std::string& n) {
  auto it = g_tab.find(n);
  return it == g_tab.end() ? nullptr : it->second.i.data();
}
std::string bn(int b, const char* n) {
  char s[64];
  std::snprintf(s, sizeof s, "b%02d.%s", b, n);
  return s;
}

enum { ERR_OK = 0, ERR_NOT_INIT = 1, ERR_INFLAG1 = 2, ERR_ICE_BOUNDS = 4, ERR_DGE_BOUNDS = 5,
       ERR_LIQ_BOUNDS = 6, ERR_ARGS = 10, ERR_OPTICS = 13, ERR_UNSUPPORTED = 14 };

constexpr int NGPT = 112, NBND = 14, NTBL = 10000;
const double TBLINT = 10000.0, OD_LO = 0.06;
double exp_tbl[NTBL + 1], bpade, heatfac, rrsw_scon;
const double *pref, *preflog, *tref, *wavenum2;
const double *extliq1, *ssaliq1, *asyliq1, *extice2, *ssaice2, *asyice2, *extice3, *ssaice3, *asyice3, *fdlice3;
const double *abari, *bbari, *cbari, *dbari, *ebari, *fbari;
int ngc[NBND], ngs[NBND], ngb[NGPT], nspa[NBND], nspb[NBND];
bool g_ready = false;

// a band's reduced tables (absa/absb are the equivalenced flat views taumol indexes)
struct Band {
  int ng = 0;
  const double *absa = nullptr, *absb = nullptr, *selfref = nullptr, *forref = nullptr, *sfluxref = nullptr;
  const double *rayl = nullptr, *absch4 = nullptr, *abso3a = nullptr, *abso3b = nullptr, *rayla = nullptr,
               *raylb = nullptr, *absh2o = nullptr, *absco2 = nullptr;
  int nsf = 1;  // second extent of sfluxref (1, 5 or 9)
  double A(int i, int ig) const { return absa[(i - 1) + (size_t)absa_rows * (ig - 1)]; }
  double B(int i, int ig) const { return absb[(i - 1) + (size_t)absb_rows * (ig - 1)]; }
  double SELF(int i, int ig) const { return selfref[(i - 1) + 10 * (ig - 1)]; }
  double FOR(int i, int ig) const { return forref[(i - 1) + nfor * (ig - 1)]; }
  double SF(int ig, int j) const { return sfluxref[(ig - 1) + ng * (j - 1)]; }
  double RAYLA(int ig, int j) const { return rayla[(ig - 1) + ng * (j - 1)]; }
  int absa_rows = 0, absb_rows = 0, nfor = 3;
} band[30];

// cloud tables are (rows, 16:29) in Fortran; ib is the band number 16..29
inline double C2(const double* t, int rows, int i, int ib) { return t[(i - 1) + (size_t)rows * (ib - 16)]; }

struct Col {
  int nlayers = 0;
  std::vector<double> pavel, tavel, pz, tz, pdp, coldry, wkl;  // wkl(7, l)
  double tbound = 0;
  double adjflux[30];
  // McICA cloud (ig, l), aerosol (l, ib)
  std::vector<double> cldfmc, taucmc, ssacmc, asmcmc, fsfcmc, ciwpmc, clwpmc, taormc, reicmc, relqmc;
  std::vector<double> taua, ssaa, asma;
  // setcoef
  int laytrop = 0, layswtch = 0, laylow = 0;
  std::vector<int> jp, jt, jt1, indself, indfor;
  std::vector<double> colh2o, colco2, colo3, coln2o, colch4, colo2, colmol, co2mult, fac00, fac01, fac10, fac11,
      selffac, selffrac, forfac, forfrac;
  // taumol: (l, ig)
  std::vector<double> taug, taur, sfluxzen;
  void alloc(int nlay) {
    nlayers = nlay;
    const int n = nlay + 2;
    for (auto* v : {&pavel, &tavel, &pz, &tz, &pdp, &coldry, &reicmc, &relqmc}) v->assign(n, 0.0);
    wkl.assign(7 * n, 0.0);
    for (auto* v : {&cldfmc, &taucmc, &ssacmc, &asmcmc, &fsfcmc, &ciwpmc, &clwpmc, &taormc}) v->assign(NGPT * n, 0.0);
    for (auto* v : {&taua, &ssaa, &asma}) v->assign(n * NBND, 0.0);
    for (auto* v : {&jp, &jt, &jt1, &indself, &indfor}) v->assign(n, 0);
    for (auto* v : {&colh2o, &colco2, &colo3, &coln2o, &colch4, &colo2, &colmol, &co2mult, &fac00, &fac01, &fac10,
                    &fac11, &selffac, &selffrac, &forfac, &forfrac})
      v->assign(n, 0.0);
    taug.assign(n * NGPT, 0.0);
    taur.assign(n * NGPT, 0.0);
    sfluxzen.assign(NGPT + 1, 0.0);
  }
  double& W(int m, int l) { return wkl[(m - 1) + 7 * l]; }
  double& CM(std::vector<double>& v, int ig, int l) { return v[(ig - 1) + NGPT * l]; }
  double& AER(std::vector<double>& v, int l, int ib) { return v[l + (nlayers + 2) * (ib - 1)]; }  // ib 1..14
  double& TG(int l, int ig) { return taug[l + (nlayers + 2) * (ig - 1)]; }
  double& TR(int l, int ig) { return taur[l + (nlayers + 2) * (ig - 1)]; }
};

struct Args {
  int ncol, nlay, icld, iaer;
  const double *play, *plev, *tlay, *tlev, *tsfc, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr, *o2vmr;
  const double *asdir, *asdif, *aldir, *aldif, *coszen;
  double adjes;
  int dyofyr;
  double scon;
  int isolvar, inflgsw, iceflgsw, liqflgsw;
  const double *cldfmcl, *taucmcl, *ssacmcl, *asmcmcl, *fsfcmcl, *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl;
  const double *tauaer, *ssaaer, *asmaer;
};

// earth_sun (rrtmg_sw_rad.f90:590-608)
double earth_sun(int idn) {
  const double pi = 2.0 * std::asin(1.0);
  const double gamma = 2.0 * pi * (idn - 1) / 365.0;
  return 1.000110 + .034221 * std::cos(gamma) + .001289 * std::sin(gamma) + .000719 * std::cos(2.0 * gamma) +
         .000077 * std::sin(2.0 * gamma);
}

// ---------------------------------------------------------------- inatm_sw (rrtmg_sw_rad.f90:612-1040)
void inatm_sw(const Args& a, int iplon, Col& c) {
  const int nl = a.nlay;
  auto in2 = [&](const double* p, int l) { return p[(iplon - 1) + (size_t)a.ncol * (l - 1)]; };  // (ncol, .)
  const double amd = 28.9660, amw = 18.0160;
  const double avogad = T("avogad")[0], grav = T("grav")[0];
  std::fill(c.wkl.begin(), c.wkl.end(), 0.0);
  std::fill(c.cldfmc.begin(), c.cldfmc.end(), 0.0);
  std::fill(c.taucmc.begin(), c.taucmc.end(), 0.0);
  std::fill(c.ssacmc.begin(), c.ssacmc.end(), 1.0);
  std::fill(c.asmcmc.begin(), c.asmcmc.end(), 0.0);
  std::fill(c.fsfcmc.begin(), c.fsfcmc.end(), 0.0);
  std::fill(c.ciwpmc.begin(), c.ciwpmc.end(), 0.0);
  std::fill(c.clwpmc.begin(), c.clwpmc.end(), 0.0);
  std::fill(c.reicmc.begin(), c.reicmc.end(), 0.0);
  std::fill(c.relqmc.begin(), c.relqmc.end(), 0.0);
  std::fill(c.taua.begin(), c.taua.end(), 0.0);
  std::fill(c.ssaa.begin(), c.ssaa.end(), 1.0);
  std::fill(c.asma.begin(), c.asma.end(), 0.0);
  // solar variability option -1 (BRAMS): solvar = scon / rrsw_scon if scon > 0 else 1 (:905-939)
  double adjflx = a.adjes;
  if (a.dyofyr > 0) adjflx = earth_sun(a.dyofyr);
  const double solvar = a.scon > 0.0 ? a.scon / rrsw_scon : double(1.0);
  for (int ib = 16; ib <= 29; ++ib) c.adjflux[ib] = adjflx * solvar;
  c.tbound = a.tsfc[iplon - 1];
  c.pz[0] = a.plev[(iplon - 1)];
  c.tz[0] = a.tlev[(iplon - 1)];
  for (int l = 1; l <= nl; ++l) {
    c.pavel[l] = in2(a.play, l);
    c.tavel[l] = in2(a.tlay, l);
    c.pz[l] = in2(a.plev, l + 1);
    c.tz[l] = in2(a.tlev, l + 1);
    c.pdp[l] = c.pz[l - 1] - c.pz[l];
    c.W(1, l) = in2(a.h2ovmr, l);
    c.W(2, l) = in2(a.co2vmr, l);
    c.W(3, l) = in2(a.o3vmr, l);
    c.W(4, l) = in2(a.n2ovmr, l);
    c.W(6, l) = in2(a.ch4vmr, l);
    c.W(7, l) = in2(a.o2vmr, l);
    const double amm = (1.0 - c.W(1, l)) * amd + c.W(1, l) * amw;
    c.coldry[l] = (c.pz[l - 1] - c.pz[l]) * 1.e3 * avogad / (1.e2 * grav * amm * (1.0 + c.W(1, l)));
  }
  for (int l = 1; l <= nl; ++l)
    for (int imol = 1; imol <= 7; ++imol) c.W(imol, l) = c.coldry[l] * c.W(imol, l);
  if (a.iaer >= 1) {
    for (int l = 1; l <= nl; ++l)
      for (int ib = 1; ib <= NBND; ++ib) {
        const size_t o = (iplon - 1) + (size_t)a.ncol * ((l - 1) + (size_t)nl * (ib - 1));  // (ncol, nlay, 14)
        c.AER(c.taua, l, ib) = a.tauaer[o];
        c.AER(c.ssaa, l, ib) = a.ssaaer[o];
        c.AER(c.asma, l, ib) = a.asmaer[o];
      }
  }
  if (a.icld >= 1) {
    for (int l = 1; l <= nl; ++l) {
      for (int ig = 1; ig <= NGPT; ++ig) {
        const size_t o = (ig - 1) + (size_t)NGPT * ((iplon - 1) + (size_t)a.ncol * (l - 1));  // (112, ncol, nlay)
        c.CM(c.cldfmc, ig, l) = a.cldfmcl[o];
        c.CM(c.taucmc, ig, l) = a.taucmcl[o];
        c.CM(c.ssacmc, ig, l) = a.ssacmcl[o];
        c.CM(c.asmcmc, ig, l) = a.asmcmcl[o];
        c.CM(c.fsfcmc, ig, l) = a.fsfcmcl[o];
        c.CM(c.ciwpmc, ig, l) = a.ciwpmcl[o];
        c.CM(c.clwpmc, ig, l) = a.clwpmcl[o];
      }
      c.reicmc[l] = in2(a.reicmcl, l);
      c.relqmc[l] = in2(a.relqmcl, l);
    }
  }
}

// ---------------------------------------------------------------- cldprmc_sw (rrtmg_sw_cldprmc.f90:43-338)
int cldprmc_sw(Col& c, int inflag, int iceflag, int liqflag) {
  const double eps = 1.e-06, cldmin = 1.e-20;
  const int nl = c.nlayers;
  for (int lay = 1; lay <= nl; ++lay)
    for (int ig = 1; ig <= NGPT; ++ig) c.CM(c.taormc, ig, lay) = c.CM(c.taucmc, ig, lay);
  for (int lay = 1; lay <= nl; ++lay) {
    for (int ig = 1; ig <= NGPT; ++ig) {
      const double cwp = c.CM(c.ciwpmc, ig, lay) + c.CM(c.clwpmc, ig, lay);
      if (!(c.CM(c.cldfmc, ig, lay) >= cldmin && (cwp >= cldmin || c.CM(c.taucmc, ig, lay) >= cldmin))) continue;
      if (inflag == 0) {
        const double taucldorig_a = c.CM(c.taucmc, ig, lay);
        const double ffp = c.CM(c.fsfcmc, ig, lay);
        const double ffp1 = 1.0 - ffp;
        const double ffpssa = 1.0 - ffp * c.CM(c.ssacmc, ig, lay);
        const double ssacloud_a = ffp1 * c.CM(c.ssacmc, ig, lay) / ffpssa;
        const double taucloud_a = ffpssa * taucldorig_a;
        c.CM(c.taormc, ig, lay) = taucldorig_a;
        c.CM(c.ssacmc, ig, lay) = ssacloud_a;
        c.CM(c.taucmc, ig, lay) = taucloud_a;
        c.CM(c.asmcmc, ig, lay) = (c.CM(c.asmcmc, ig, lay) - ffp) / (ffp1);
      } else if (inflag == 1) {
        return ERR_INFLAG1;
      } else if (inflag == 2) {
        const double radice = c.reicmc[lay];
        const int ib = ngb[ig - 1];
        double extcoice = 0, ssacoice = 0, gice = 0, forwice = 0, fdelta = 0;
        double extcoliq = 0, ssacoliq = 0, gliq = 0, forwliq = 0;
        const double ciwp = c.CM(c.ciwpmc, ig, lay), clwp = c.CM(c.clwpmc, ig, lay);
        if (ciwp == 0.0) {
          extcoice = ssacoice = gice = forwice = 0.0;
        } else if (iceflag == 1) {
          if (radice < 13.0 || radice > 130.0) return ERR_ICE_BOUNDS;
          const double w2 = wavenum2[ib - 16];
          int icx = 0;
          if (w2 > 1.43e04) icx = 1;
          else if (w2 > 7.7e03) icx = 2;
          else if (w2 > 5.3e03) icx = 3;
          else if (w2 > 4.0e03) icx = 4;
          else if (w2 >= 2.5e03) icx = 5;
          extcoice = (abari[icx - 1] + bbari[icx - 1] / radice);
          ssacoice = 1.0 - cbari[icx - 1] - dbari[icx - 1] * radice;
          gice = ebari[icx - 1] + fbari[icx - 1] * radice;
          if (gice >= 1.0) gice = 1.0 - eps;
          forwice = gice * gice;
          if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0) return ERR_OPTICS;
        } else if (iceflag == 2) {
          if (radice < 5.0 || radice > 131.0) return ERR_ICE_BOUNDS;
          const double factor = (radice - 2.0) / 3.0;
          int index = (int)factor;
          if (index == 43) index = 42;
          const double fint = factor - (double)index;
          extcoice = C2(extice2, 43, index, ib) + fint * (C2(extice2, 43, index + 1, ib) - C2(extice2, 43, index, ib));
          ssacoice = C2(ssaice2, 43, index, ib) + fint * (C2(ssaice2, 43, index + 1, ib) - C2(ssaice2, 43, index, ib));
          gice = C2(asyice2, 43, index, ib) + fint * (C2(asyice2, 43, index + 1, ib) - C2(asyice2, 43, index, ib));
          forwice = gice * gice;
          if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0) return ERR_OPTICS;
        } else if (iceflag == 3) {
          if (radice < 5.0 || radice > 140.0) return ERR_DGE_BOUNDS;
          const double factor = (radice - 2.0) / 3.0;
          int index = (int)factor;
          if (index == 46) index = 45;
          const double fint = factor - (double)index;
          extcoice = C2(extice3, 46, index, ib) + fint * (C2(extice3, 46, index + 1, ib) - C2(extice3, 46, index, ib));
          ssacoice = C2(ssaice3, 46, index, ib) + fint * (C2(ssaice3, 46, index + 1, ib) - C2(ssaice3, 46, index, ib));
          gice = C2(asyice3, 46, index, ib) + fint * (C2(asyice3, 46, index + 1, ib) - C2(asyice3, 46, index, ib));
          fdelta = C2(fdlice3, 46, index, ib) + fint * (C2(fdlice3, 46, index + 1, ib) - C2(fdlice3, 46, index, ib));
          if (fdelta < 0.0 || fdelta > 1.0) return ERR_OPTICS;
          forwice = fdelta + 0.5 / ssacoice;
          if (forwice > gice) forwice = gice;
          if (extcoice < 0.0 || ssacoice > 1.0 || ssacoice < 0.0 || gice > 1.0 || gice < 0.0) return ERR_OPTICS;
        } else {
          return ERR_UNSUPPORTED;
        }
        if (clwp == 0.0) {
          extcoliq = ssacoliq = gliq = forwliq = 0.0;
        } else if (liqflag == 1) {
          const double radliq = c.relqmc[lay];
          if (radliq < 2.5 || radliq > 60.0) return ERR_LIQ_BOUNDS;
          int index = (int)(radliq - 1.5);
          if (index == 0) index = 1;
          if (index == 58) index = 57;
          const double fint = radliq - 1.5 - (double)index;
          extcoliq = C2(extliq1, 58, index, ib) + fint * (C2(extliq1, 58, index + 1, ib) - C2(extliq1, 58, index, ib));
          ssacoliq = C2(ssaliq1, 58, index, ib) + fint * (C2(ssaliq1, 58, index + 1, ib) - C2(ssaliq1, 58, index, ib));
          if (fint < 0.0 && ssacoliq > 1.0) ssacoliq = C2(ssaliq1, 58, index, ib);
          gliq = C2(asyliq1, 58, index, ib) + fint * (C2(asyliq1, 58, index + 1, ib) - C2(asyliq1, 58, index, ib));
          forwliq = gliq * gliq;
          if (extcoliq < 0.0 || ssacoliq > 1.0 || ssacoliq < 0.0 || gliq > 1.0 || gliq < 0.0) return ERR_OPTICS;
        } else {
          return ERR_UNSUPPORTED;
        }
        const double tauliqorig = clwp * extcoliq;
        const double tauiceorig = ciwp * extcoice;
        c.CM(c.taormc, ig, lay) = tauliqorig + tauiceorig;
        const double ssaliq = ssacoliq * (1.0 - forwliq) / (1.0 - forwliq * ssacoliq);
        const double tauliq = (1.0 - forwliq * ssacoliq) * tauliqorig;
        const double ssaice = ssacoice * (1.0 - forwice) / (1.0 - forwice * ssacoice);
        const double tauice = (1.0 - forwice * ssacoice) * tauiceorig;
        const double scatliq = ssaliq * tauliq;
        double scatice = ssaice * tauice;
        c.CM(c.taucmc, ig, lay) = tauliq + tauice;
        if (c.CM(c.taucmc, ig, lay) == 0.) c.CM(c.taucmc, ig, lay) = cldmin;
        if (scatice == 0.) scatice = cldmin;
        c.CM(c.ssacmc, ig, lay) = (scatliq + scatice) / c.CM(c.taucmc, ig, lay);
        if (iceflag == 3) {
          c.CM(c.asmcmc, ig, lay) = (1.0 / (scatliq + scatice)) *
                                    (scatliq * (gliq - forwliq) / (1.0 - forwliq) +
                                     scatice * ((gice - forwice) / (1.0 - forwice)));
        } else {
          c.CM(c.asmcmc, ig, lay) = (scatliq * (gliq - forwliq) / (1.0 - forwliq) +
                                     scatice * (gice - forwice) / (1.0 - forwice)) /
                                    (scatliq + scatice);
        }
      }
    }
  }
  return 0;
}

// ---------------------------------------------------------------- setcoef_sw (rrtmg_sw_setcoef.f90:27-240)
void setcoef_sw(Col& c) {
  const double stpfac = 296.0 / 1013.0;
  c.laytrop = c.layswtch = c.laylow = 0;
  for (int lay = 1; lay <= c.nlayers; ++lay) {
    const double plog = std::log(c.pavel[lay]);
    int jp = (int)(36.0 - 5 * (plog + 0.04));
    if (jp < 1) jp = 1;
    else if (jp > 58) jp = 58;
    c.jp[lay] = jp;
    const int jp1 = jp + 1;
    const double fp = 5.0 * (preflog[jp - 1] - plog);
    int jt = (int)(3.0 + (c.tavel[lay] - tref[jp - 1]) / 15.0);
    if (jt < 1) jt = 1;
    else if (jt > 4) jt = 4;
    c.jt[lay] = jt;
    const double ft = ((c.tavel[lay] - tref[jp - 1]) / 15.0) - (double)(jt - 3);
    int jt1 = (int)(3.0 + (c.tavel[lay] - tref[jp1 - 1]) / 15.0);
    if (jt1 < 1) jt1 = 1;
    else if (jt1 > 4) jt1 = 4;
    c.jt1[lay] = jt1;
    const double ft1 = ((c.tavel[lay] - tref[jp1 - 1]) / 15.0) - (double)(jt1 - 3);
    const double water = c.W(1, lay) / c.coldry[lay];
    const double scalefac = c.pavel[lay] * stpfac / c.tavel[lay];
    auto cols = [&]() {
      c.colh2o[lay] = 1.e-20 * c.W(1, lay);
      c.colco2[lay] = 1.e-20 * c.W(2, lay);
      c.colo3[lay] = 1.e-20 * c.W(3, lay);
      c.coln2o[lay] = 1.e-20 * c.W(4, lay);
      c.colch4[lay] = 1.e-20 * c.W(6, lay);
      c.colo2[lay] = 1.e-20 * c.W(7, lay);
      c.colmol[lay] = 1.e-20 * c.coldry[lay] + c.colh2o[lay];
      if (c.colco2[lay] == 0.0) c.colco2[lay] = 1.e-32 * c.coldry[lay];
      if (c.coln2o[lay] == 0.0) c.coln2o[lay] = 1.e-32 * c.coldry[lay];
      if (c.colch4[lay] == 0.0) c.colch4[lay] = 1.e-32 * c.coldry[lay];
      if (c.colo2[lay] == 0.0) c.colo2[lay] = 1.e-32 * c.coldry[lay];
      const double co2reg = 3.55e-24 * c.coldry[lay];
      c.co2mult[lay] = (c.colco2[lay] - co2reg) * 272.63 * std::exp(-1919.4 / c.tavel[lay]) / (8.7604e-4 * c.tavel[lay]);
    };
    if (plog > 4.56) {
      c.laytrop = c.laytrop + 1;
      if (plog >= 6.62) c.laylow = c.laylow + 1;
      c.forfac[lay] = scalefac / (1. + water);
      double factor = (332.0 - c.tavel[lay]) / 36.0;
      c.indfor[lay] = std::min(2, std::max(1, (int)factor));
      c.forfrac[lay] = factor - (double)c.indfor[lay];
      c.selffac[lay] = water * c.forfac[lay];
      factor = (c.tavel[lay] - 188.0) / 7.2;
      c.indself[lay] = std::min(9, std::max(1, (int)factor - 7));
      c.selffrac[lay] = factor - (double)(c.indself[lay] + 7);
      cols();
    } else {
      c.forfac[lay] = scalefac / (1. + water);
      const double factor = (c.tavel[lay] - 188.0) / 36.0;
      c.indfor[lay] = 3;
      c.forfrac[lay] = factor - 1.0;
      cols();
      c.selffac[lay] = 0.0;
      c.selffrac[lay] = 0.0;
      c.indself[lay] = 0;
    }
    const double compfp = 1.0 - fp;
    c.fac10[lay] = compfp * ft;
    c.fac00[lay] = compfp * (1.0 - ft);
    c.fac11[lay] = fp * ft1;
    c.fac01[lay] = fp * (1.0 - ft1);
  }
}

// ---------------------------------------------------------------- taumol_sw (rrtmg_sw_taumol.f90:50-1787)
struct Interp8 {
  double f000, f100, f010, f110, f001, f101, f011, f111;
};
// the binary-species parameter of a layer: specparm, js and fs (taumol.f90:306-312 etc.)
void binary(double a, double b, double strrat, double mult, double oneminus, double& speccomb, int& js, double& fs) {
  speccomb = a + strrat * b;
  double specparm = a / speccomb;
  if (specparm >= oneminus) specparm = oneminus;
  const double specmult = mult * (specparm);
  js = 1 + (int)specmult;
  fs = std::fmod(specmult, 1.0);
}
Interp8 interp8(const Col& c, int lay, double fs) {
  Interp8 f;
  f.f000 = (1.0 - fs) * c.fac00[lay];
  f.f010 = (1.0 - fs) * c.fac10[lay];
  f.f100 = fs * c.fac00[lay];
  f.f110 = fs * c.fac10[lay];
  f.f001 = (1.0 - fs) * c.fac01[lay];
  f.f011 = (1.0 - fs) * c.fac11[lay];
  f.f101 = fs * c.fac01[lay];
  f.f111 = fs * c.fac11[lay];
  return f;
}
// the eight-point lower/upper-atmosphere sum with row strides (9 or 5)
template <class Get>
double sum8(const Interp8& f, int ind0, int ind1, int s1, Get get) {
  return f.f000 * get(ind0) + f.f100 * get(ind0 + 1) + f.f010 * get(ind0 + s1) + f.f110 * get(ind0 + s1 + 1) +
         f.f001 * get(ind1) + f.f101 * get(ind1 + 1) + f.f011 * get(ind1 + s1) + f.f111 * get(ind1 + s1 + 1);
}
int jpx(const Col& c, int l) { return (l >= 1 && l <= c.nlayers) ? c.jp[l] : 0; }

void taumol_sw(Col& c, double oneminus) {
  const int nl = c.nlayers, lt = c.laytrop;
  std::fill(c.sfluxzen.begin(), c.sfluxzen.end(), 0.0);
  auto self = [&](const Band& B, int lay, int ig) {
    const int inds = c.indself[lay];
    return c.selffac[lay] * (B.SELF(inds, ig) + c.selffrac[lay] * (B.SELF(inds + 1, ig) - B.SELF(inds, ig)));
  };
  auto forx = [&](const Band& B, int lay, int ig) {
    const int indf = c.indfor[lay];
    return B.FOR(indf, ig) + c.forfrac[lay] * (B.FOR(indf + 1, ig) - B.FOR(indf, ig));
  };
  auto forf = [&](const Band& B, int lay, int ig) { return c.forfac[lay] * forx(B, lay, ig); };
  auto four = [&](const double* tab, int rows, int lay, int ind0, int ind1, int ig) {
    auto t = [&](int i) { return tab[(i - 1) + (size_t)rows * (ig - 1)]; };
    return c.fac00[lay] * t(ind0) + c.fac10[lay] * t(ind0 + 1) + c.fac01[lay] * t(ind1) + c.fac11[lay] * t(ind1 + 1);
  };
  auto ia0 = [&](int lay, int b, int js) { return ((c.jp[lay] - 1) * 5 + (c.jt[lay] - 1)) * nspa[b - 16] + js; };
  auto ia1 = [&](int lay, int b, int js) { return (c.jp[lay] * 5 + (c.jt1[lay] - 1)) * nspa[b - 16] + js; };
  auto ib0 = [&](int lay, int b, int js) { return ((c.jp[lay] - 13) * 5 + (c.jt[lay] - 1)) * nspb[b - 16] + js; };
  auto ib1 = [&](int lay, int b, int js) { return ((c.jp[lay] - 12) * 5 + (c.jt1[lay] - 1)) * nspb[b - 16] + js; };
  // laysolfr searches: lower atmosphere (bands 18-26), upper atmosphere (16, 17, 27-29)
  auto lower_solar = [&](int layreffr) {
    int laysolfr = lt;
    for (int lay = 1; lay <= lt; ++lay)
      if (c.jp[lay] < layreffr && jpx(c, lay + 1) >= layreffr) laysolfr = std::min(lay + 1, lt);
    return laysolfr;
  };
  auto upper_solar = [&](int layreffr) {
    int laysolfr = nl;
    for (int lay = lt + 1; lay <= nl; ++lay)
      if (jpx(c, lay - 1) < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
    return laysolfr;
  };
  // ---- band 16 (:275-383)
  {
    const Band& B = band[16];
    const int g0 = 0;
    for (int lay = 1; lay <= lt; ++lay) {
      double speccomb, fs;
      int js;
      binary(c.colh2o[lay], c.colch4[lay], 252.131, 8.0, oneminus, speccomb, js, fs);
      const Interp8 f = interp8(c, lay, fs);
      const int ind0 = ia0(lay, 16, js), ind1 = ia1(lay, 16, js);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        c.TG(lay, g0 + ig) = speccomb * sum8(f, ind0, ind1, 9, [&](int i) { return B.A(i, ig); }) +
                             c.colh2o[lay] * (self(B, lay, ig) + forf(B, lay, ig));
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    const int laysolfr = upper_solar(18);
    for (int lay = lt + 1; lay <= nl; ++lay) {
      const int ind0 = ib0(lay, 16, 1), ind1 = ib1(lay, 16, 1);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        c.TG(lay, g0 + ig) = c.colch4[lay] * four(B.absb, B.absb_rows, lay, ind0, ind1, ig);
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, 1);
        c.TR(lay, g0 + ig) = tauray;
      }
    }
  }
  // bands 17, 21 and 28: binary species in both regions; the solar source in
  // the upper region (17, 28) or the lower one (21)
  auto binary_both = [&](int b, int g0, double strrat, int layreffr, bool h2o_major, bool solar_lower) {
    const Band& B = band[b];
    const int laysolfr_lo = solar_lower ? lower_solar(layreffr) : -1;
    for (int lay = 1; lay <= lt; ++lay) {
      double speccomb, fs;
      int js;
      if (h2o_major)
        binary(c.colh2o[lay], c.colco2[lay], strrat, 8.0, oneminus, speccomb, js, fs);
      else
        binary(c.colo3[lay], c.colo2[lay], strrat, 8.0, oneminus, speccomb, js, fs);
      const Interp8 f = interp8(c, lay, fs);
      const int ind0 = ia0(lay, b, js), ind1 = ia1(lay, b, js);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        double t = speccomb * sum8(f, ind0, ind1, 9, [&](int i) { return B.A(i, ig); });
        if (h2o_major) t = t + c.colh2o[lay] * (self(B, lay, ig) + forf(B, lay, ig));
        c.TG(lay, g0 + ig) = t;
        if (lay == laysolfr_lo) c.sfluxzen[g0 + ig] = B.SF(ig, js) + fs * (B.SF(ig, js + 1) - B.SF(ig, js));
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    int laysolfr = solar_lower ? -1 : nl;
    for (int lay = lt + 1; lay <= nl; ++lay) {
      if (!solar_lower && jpx(c, lay - 1) < layreffr && c.jp[lay] >= layreffr) laysolfr = lay;
      double speccomb, fs;
      int js;
      if (h2o_major)
        binary(c.colh2o[lay], c.colco2[lay], strrat, 4.0, oneminus, speccomb, js, fs);
      else
        binary(c.colo3[lay], c.colo2[lay], strrat, 4.0, oneminus, speccomb, js, fs);
      const Interp8 f = interp8(c, lay, fs);
      const int ind0 = ib0(lay, b, js), ind1 = ib1(lay, b, js);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        double t = speccomb * sum8(f, ind0, ind1, 5, [&](int i) { return B.B(i, ig); });
        if (h2o_major) t = t + c.colh2o[lay] * c.forfac[lay] * forx(B, lay, ig);
        c.TG(lay, g0 + ig) = t;
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, js) + fs * (B.SF(ig, js + 1) - B.SF(ig, js));
        c.TR(lay, g0 + ig) = tauray;
      }
    }
  };
  binary_both(17, ngs[0], 0.364641, 30, true, false);
  // bands 18, 19, 22, 24: binary species and solar source in the lower region, one absorber above
  auto lower_binary = [&](int b, int g0, double strrat, int layreffr) {
    const Band& B = band[b];
    const int laysolfr = lower_solar(layreffr);
    const double o2adj = 1.6;
    for (int lay = 1; lay <= lt; ++lay) {
      double speccomb, fs;
      int js;
      if (b == 18)
        binary(c.colh2o[lay], c.colch4[lay], strrat, 8.0, oneminus, speccomb, js, fs);
      else if (b == 19)
        binary(c.colh2o[lay], c.colco2[lay], strrat, 8.0, oneminus, speccomb, js, fs);
      else if (b == 22)
        binary(c.colh2o[lay], c.colo2[lay], o2adj * strrat, 8.0, oneminus, speccomb, js, fs);
      else
        binary(c.colh2o[lay], c.colo2[lay], strrat, 8.0, oneminus, speccomb, js, fs);
      const Interp8 f = interp8(c, lay, fs);
      const int ind0 = ia0(lay, b, js), ind1 = ia1(lay, b, js);
      const double o2cont = 4.35e-4 * c.colo2[lay] / (350.0 * 2.0);
      for (int ig = 1; ig <= B.ng; ++ig) {
        double tauray;
        const double k8 = sum8(f, ind0, ind1, 9, [&](int i) { return B.A(i, ig); });
        double t;
        if (b == 24) {
          tauray = c.colmol[lay] * (B.RAYLA(ig, js) + fs * (B.RAYLA(ig, js + 1) - B.RAYLA(ig, js)));
          t = speccomb * k8 + c.colo3[lay] * B.abso3a[ig - 1] + c.colh2o[lay] * (self(B, lay, ig) + forf(B, lay, ig));
        } else {
          tauray = c.colmol[lay] * B.rayl[0];
          t = speccomb * k8 + c.colh2o[lay] * (self(B, lay, ig) + forf(B, lay, ig));
          if (b == 22) t = t + o2cont;
        }
        c.TG(lay, g0 + ig) = t;
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, js) + fs * (B.SF(ig, js + 1) - B.SF(ig, js));
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      const int ind0 = ib0(lay, b, 1), ind1 = ib1(lay, b, 1);
      const double o2cont = 4.35e-4 * c.colo2[lay] / (350.0 * 2.0);
      for (int ig = 1; ig <= B.ng; ++ig) {
        const double k4 = four(B.absb, B.absb_rows, lay, ind0, ind1, ig);
        double t, tauray;
        if (b == 18) {
          t = c.colch4[lay] * k4;
          tauray = c.colmol[lay] * B.rayl[0];
        } else if (b == 19) {
          t = c.colco2[lay] * k4;
          tauray = c.colmol[lay] * B.rayl[0];
        } else if (b == 22) {
          t = c.colo2[lay] * o2adj * k4 + o2cont;
          tauray = c.colmol[lay] * B.rayl[0];
        } else {
          t = c.colo2[lay] * k4 + c.colo3[lay] * B.abso3b[ig - 1];
          tauray = c.colmol[lay] * B.raylb[ig - 1];
        }
        c.TG(lay, g0 + ig) = t;
        c.TR(lay, g0 + ig) = tauray;
      }
    }
  };
  lower_binary(18, ngs[1], 38.9589, 6);
  lower_binary(19, ngs[2], 5.49281, 3);
  // ---- band 20 (:764-859)
  {
    const Band& B = band[20];
    const int g0 = ngs[3];
    const int laysolfr = lower_solar(3);
    for (int lay = 1; lay <= lt; ++lay) {
      const int ind0 = ia0(lay, 20, 1), ind1 = ia1(lay, 20, 1);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        c.TG(lay, g0 + ig) = c.colh2o[lay] * (four(B.absa, B.absa_rows, lay, ind0, ind1, ig) + self(B, lay, ig) +
                                              forf(B, lay, ig)) +
                             c.colch4[lay] * B.absch4[ig - 1];
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, 1);
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay) {
      const int ind0 = ib0(lay, 20, 1), ind1 = ib1(lay, 20, 1);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        c.TG(lay, g0 + ig) = c.colh2o[lay] * (four(B.absb, B.absb_rows, lay, ind0, ind1, ig) + forf(B, lay, ig)) +
                             c.colch4[lay] * B.absch4[ig - 1];
        c.TR(lay, g0 + ig) = tauray;
      }
    }
  }
  binary_both(21, ngs[4], 0.0045321, 8, true, true);
  lower_binary(22, ngs[5], 0.022708, 2);
  // ---- band 23 (:1131-1214)
  {
    const Band& B = band[23];
    const int g0 = ngs[6];
    const int laysolfr = lower_solar(6);
    const double givfac = 1.029;
    for (int lay = 1; lay <= lt; ++lay) {
      const int ind0 = ia0(lay, 23, 1), ind1 = ia1(lay, 23, 1);
      for (int ig = 1; ig <= B.ng; ++ig) {
        const double tauray = c.colmol[lay] * B.rayl[ig - 1];
        c.TG(lay, g0 + ig) = c.colh2o[lay] * (givfac * four(B.absa, B.absa_rows, lay, ind0, ind1, ig) +
                                              self(B, lay, ig) + forf(B, lay, ig));
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, 1);
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay)
      for (int ig = 1; ig <= B.ng; ++ig) {
        c.TG(lay, g0 + ig) = 0.0;
        c.TR(lay, g0 + ig) = c.colmol[lay] * B.rayl[ig - 1];
      }
  }
  lower_binary(24, ngs[7], 0.124692, 1);
  // ---- band 25 (:1338-1411)
  {
    const Band& B = band[25];
    const int g0 = ngs[8];
    const int laysolfr = lower_solar(2);
    for (int lay = 1; lay <= lt; ++lay) {
      const int ind0 = ia0(lay, 25, 1), ind1 = ia1(lay, 25, 1);
      for (int ig = 1; ig <= B.ng; ++ig) {
        const double tauray = c.colmol[lay] * B.rayl[ig - 1];
        c.TG(lay, g0 + ig) = c.colh2o[lay] * four(B.absa, B.absa_rows, lay, ind0, ind1, ig) +
                             c.colo3[lay] * B.abso3a[ig - 1];
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, 1);
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    for (int lay = lt + 1; lay <= nl; ++lay)
      for (int ig = 1; ig <= B.ng; ++ig) {
        const double tauray = c.colmol[lay] * B.rayl[ig - 1];
        c.TG(lay, g0 + ig) = c.colo3[lay] * B.abso3b[ig - 1];
        c.TR(lay, g0 + ig) = tauray;
      }
  }
  // ---- band 26 (:1414-1474)
  {
    const Band& B = band[26];
    const int g0 = ngs[9];
    const int laysolfr = lt;
    for (int lay = 1; lay <= nl; ++lay)
      for (int ig = 1; ig <= B.ng; ++ig) {
        if (lay <= lt && lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, 1);
        c.TG(lay, g0 + ig) = 0.0;
        c.TR(lay, g0 + ig) = c.colmol[lay] * B.rayl[ig - 1];
      }
  }
  // ---- band 27 (:1477-1565)
  {
    const Band& B = band[27];
    const int g0 = ngs[10];
    const double scalekur = 50.15 / 48.37;
    for (int lay = 1; lay <= lt; ++lay) {
      const int ind0 = ia0(lay, 27, 1), ind1 = ia1(lay, 27, 1);
      for (int ig = 1; ig <= B.ng; ++ig) {
        const double tauray = c.colmol[lay] * B.rayl[ig - 1];
        c.TG(lay, g0 + ig) = c.colo3[lay] * four(B.absa, B.absa_rows, lay, ind0, ind1, ig);
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    const int laysolfr = upper_solar(32);
    for (int lay = lt + 1; lay <= nl; ++lay) {
      const int ind0 = ib0(lay, 27, 1), ind1 = ib1(lay, 27, 1);
      for (int ig = 1; ig <= B.ng; ++ig) {
        const double tauray = c.colmol[lay] * B.rayl[ig - 1];
        c.TG(lay, g0 + ig) = c.colo3[lay] * four(B.absb, B.absb_rows, lay, ind0, ind1, ig);
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = scalekur * B.SF(ig, 1);
        c.TR(lay, g0 + ig) = tauray;
      }
    }
  }
  binary_both(28, ngs[11], 6.67029e-07, 42, false, false);
  // ---- band 29 (:1695-1785)
  {
    const Band& B = band[29];
    const int g0 = ngs[12];
    for (int lay = 1; lay <= lt; ++lay) {
      const int ind0 = ia0(lay, 29, 1), ind1 = ia1(lay, 29, 1);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        c.TG(lay, g0 + ig) = c.colh2o[lay] * (four(B.absa, B.absa_rows, lay, ind0, ind1, ig) + self(B, lay, ig) +
                                              forf(B, lay, ig)) +
                             c.colco2[lay] * B.absco2[ig - 1];
        c.TR(lay, g0 + ig) = tauray;
      }
    }
    const int laysolfr = upper_solar(49);
    for (int lay = lt + 1; lay <= nl; ++lay) {
      const int ind0 = ib0(lay, 29, 1), ind1 = ib1(lay, 29, 1);
      const double tauray = c.colmol[lay] * B.rayl[0];
      for (int ig = 1; ig <= B.ng; ++ig) {
        c.TG(lay, g0 + ig) = c.colco2[lay] * four(B.absb, B.absb_rows, lay, ind0, ind1, ig) +
                             c.colh2o[lay] * B.absh2o[ig - 1];
        if (lay == laysolfr) c.sfluxzen[g0 + ig] = B.SF(ig, 1);
        c.TR(lay, g0 + ig) = tauray;
      }
    }
  }
}

// ---------------------------------------------------------------- reftra_sw (rrtmg_sw_reftra.f90:27-330)
// Reflectance and transmittance of each layer (two-stream, kmodts = 2).
void reftra_sw(int nlayers, const std::vector<char>& lrtchk, const double* pgg, double prmuz, const double* ptau,
               const double* pw, double* pref, double* prefd, double* ptra, double* ptrad) {
  const double eps = 1.e-08;
  const double zwcrit = 0.9999995;
  for (int jk = 1; jk <= nlayers; ++jk) {
    if (!lrtchk[jk]) {
      pref[jk] = 0.0;
      ptra[jk] = 1.0;
      prefd[jk] = 0.0;
      ptrad[jk] = 1.0;
      continue;
    }
    const double zto1 = ptau[jk], zw = pw[jk], zg = pgg[jk];
    const double zg3 = 3.0 * zg;
    const double zgamma1 = (8.0 - zw * (5.0 + zg3)) * 0.25;
    const double zgamma2 = 3.0 * (zw * (1.0 - zg)) * 0.25;
    const double zgamma3 = (2.0 - zg3 * prmuz) * 0.25;
    const double zgamma4 = 1.0 - zgamma3;
    double zwo = 0.0, denom = 1.0;
    if (zg != 1.0) denom = (1.0 - (1.0 - zw) * std::pow(zg / (1.0 - zg), 2));
    if (zw > 0.0 && denom != 0.0) zwo = zw / denom;
    auto expo = [&](double ze) {
      if (ze <= OD_LO) return 1.0 - ze + 0.5 * ze * ze;
      const double tblind = ze / (bpade + ze);
      const int itind = (int)(TBLINT * tblind + 0.5);
      return exp_tbl[itind];
    };
    if (zwo >= zwcrit) {
      // conservative scattering
      const double za = zgamma1 * prmuz;
      const double za1 = za - zgamma3;
      const double zgt = zgamma1 * zto1;
      const double ze1 = std::min<double>(zto1 / prmuz, 500.0);
      const double ze2 = expo(ze1);
      pref[jk] = (zgt - za1 * (1.0 - ze2)) / (1.0 + zgt);
      ptra[jk] = 1.0 - pref[jk];
      prefd[jk] = zgt / (1.0 + zgt);
      ptrad[jk] = 1.0 - prefd[jk];
      if (ze2 == 1.0) {
        pref[jk] = 0.0;
        ptra[jk] = 1.0;
        prefd[jk] = 0.0;
        ptrad[jk] = 1.0;
      }
    } else {
      // non-conservative scattering
      const double za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
      const double za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
      const double zrk = std::sqrt(std::pow(zgamma1, 2) - std::pow(zgamma2, 2));
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
      const double zt4 = zr4;
      const double zt5 = zr5;
      const double zbeta = (zgamma1 - zrk) / zrkg;
      const double ze1 = std::min<double>(zrk * zto1, 500.0);
      const double ze2 = std::min<double>(zto1 / prmuz, 500.0);
      const double zem1 = expo(ze1);
      const double zep1 = 1.0 / zem1;
      const double zem2 = expo(ze2);
      const double zep2 = 1.0 / zem2;
      const double zdenr = zr4 * zep1 + zr5 * zem1;
      const double zdent = zt4 * zep1 + zt5 * zem1;
      if (zdenr >= -eps && zdenr <= eps) {
        pref[jk] = eps;
        ptra[jk] = zem2;
      } else {
        pref[jk] = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
        ptra[jk] = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdent;
      }
      const double zemm = zem1 * zem1;
      const double zdend = 1.0 / ((1.0 - zbeta * zemm) * zrkg);
      prefd[jk] = zgamma2 * (1.0 - zemm) * zdend;
      ptrad[jk] = zrk2 * zem1 * zdend;
    }
  }
}

// ---------------------------------------------------------------- vrtqdr_sw (rrtmg_sw_vrtqdr.f90:24-171)
// Adding of the layers from the surface up (albedo of the underlying medium)
// and from the top down, then the upward and downward fluxes at each level.
void vrtqdr_sw(int klev, const double* pref, const double* prefd, const double* ptra, const double* ptrad,
               const double* pdbt, double* prdnd, double* prup, double* prupd, const double* ptdbt, double* pfd,
               double* pfu) {
  std::vector<double> ztdn(klev + 2);
  double zreflect = 1.0 / (1.0 - prefd[klev + 1] * prefd[klev]);
  prup[klev] = pref[klev] + (ptrad[klev] * ((ptra[klev] - pdbt[klev]) * prefd[klev + 1] + pdbt[klev] * pref[klev + 1])) *
                                zreflect;
  prupd[klev] = prefd[klev] + ptrad[klev] * ptrad[klev] * prefd[klev + 1] * zreflect;
  for (int jk = 1; jk <= klev - 1; ++jk) {
    const int ikp = klev + 1 - jk;
    const int ikx = ikp - 1;
    zreflect = 1.0 / (1.0 - prupd[ikp] * prefd[ikx]);
    prup[ikx] = pref[ikx] + (ptrad[ikx] * ((ptra[ikx] - pdbt[ikx]) * prupd[ikp] + pdbt[ikx] * prup[ikp])) * zreflect;
    prupd[ikx] = prefd[ikx] + ptrad[ikx] * ptrad[ikx] * prupd[ikp] * zreflect;
  }
  ztdn[1] = 1.0;
  prdnd[1] = 0.0;
  ztdn[2] = ptra[1];
  prdnd[2] = prefd[1];
  for (int jk = 2; jk <= klev; ++jk) {
    const int ikp = jk + 1;
    zreflect = 1.0 / (1.0 - prefd[jk] * prdnd[jk]);
    ztdn[ikp] = ptdbt[jk] * ptra[jk] + (ptrad[jk] * ((ztdn[jk] - ptdbt[jk]) + ptdbt[jk] * pref[jk] * prdnd[jk])) * zreflect;
    prdnd[ikp] = prefd[jk] + ptrad[jk] * ptrad[jk] * prdnd[jk] * zreflect;
  }
  for (int jk = 1; jk <= klev + 1; ++jk) {
    zreflect = 1.0 / (1.0 - prdnd[jk] * prupd[jk]);
    pfu[jk] = (ptdbt[jk] * prup[jk] + (ztdn[jk] - ptdbt[jk]) * prupd[jk]) * zreflect;
    pfd[jk] = ptdbt[jk] + (ztdn[jk] - ptdbt[jk] + ptdbt[jk] * prup[jk] * prdnd[jk]) * zreflect;
  }
}

// ---------------------------------------------------------------- spcvmc_sw (rrtmg_sw_spcvmc.f90:30-664)
// icpr = 1 (cldprmc ran), idelm = 1 (delta-scaled direct beam) as the driver
// sets them; outputs the broadband total and clear fluxes (levels 1..klev+1
// from the surface).
void spcvmc_sw(Col& c, const double* palbd, const double* palbp, double prmu0, double oneminus, double* pbbfd,
               double* pbbfu, double* pbbcd, double* pbbcu) {
  const int klev = c.nlayers;
  const double repclc = 1.e-12;
  for (int jk = 1; jk <= klev + 1; ++jk) pbbcd[jk] = pbbcu[jk] = pbbfd[jk] = pbbfu[jk] = 0.0;
  taumol_sw(c, oneminus);
  const int n = klev + 2;
  std::vector<char> lrtchkclr(n), lrtchkcld(n);
  std::vector<double> ztauc(n), zomcc(n), zgcc(n), ztauo(n), zomco(n), zgco(n);
  std::vector<double> zrefc(n), zrefdc(n), ztrac(n), ztradc(n), zrefo(n), zrefdo(n), ztrao(n), ztrado(n);
  std::vector<double> zref(n), zrefd(n), ztra(n), ztrad(n), zdbtc(n), zdbt(n), ztdbtc(n), ztdbt(n);
  std::vector<double> zrdndc(n), zrupc(n), zrupdc(n), zrdnd(n), zrup(n), zrupd(n), zcd(n), zcu(n), zfd(n), zfu(n);
  auto expo = [&](double ze) {
    if (ze <= OD_LO) return 1.0 - ze + 0.5 * ze * ze;
    const double tblind = ze / (bpade + ze);
    const int itind = (int)(TBLINT * tblind + 0.5);
    return exp_tbl[itind];
  };
  int iw = 0;
  for (int jb = 16; jb <= 29; ++jb) {
    const int ibm = jb - 15;
    const int igt = ngc[ibm - 1];
    for (int jg = 1; jg <= igt; ++jg) {
      iw = iw + 1;
      const double zincflx = c.adjflux[jb] * c.sfluxzen[iw] * prmu0;
      ztdbtc[1] = 1.0;
      zdbtc[klev + 1] = 0.0;
      ztrac[klev + 1] = 0.0;
      ztradc[klev + 1] = 0.0;
      zrefc[klev + 1] = palbp[ibm - 1];
      zrefdc[klev + 1] = palbd[ibm - 1];
      zrupc[klev + 1] = palbp[ibm - 1];
      zrupdc[klev + 1] = palbd[ibm - 1];
      ztrao[klev + 1] = 0.0;
      ztrado[klev + 1] = 0.0;
      zrefo[klev + 1] = palbp[ibm - 1];
      zrefdo[klev + 1] = palbd[ibm - 1];
      ztdbt[1] = 1.0;
      zdbt[klev + 1] = 0.0;
      ztra[klev + 1] = 0.0;
      ztrad[klev + 1] = 0.0;
      zref[klev + 1] = palbp[ibm - 1];
      zrefd[klev + 1] = palbd[ibm - 1];
      zrup[klev + 1] = palbp[ibm - 1];
      zrupd[klev + 1] = palbd[ibm - 1];
      for (int jk = 1; jk <= klev; ++jk) {
        const int ikl = klev + 1 - jk;
        lrtchkclr[jk] = 1;
        lrtchkcld[jk] = c.CM(c.cldfmc, iw, ikl) > repclc;
        ztauc[jk] = c.TR(ikl, iw) + c.TG(ikl, iw) + c.AER(c.taua, ikl, ibm);
        zomcc[jk] = c.TR(ikl, iw) * 1.0 + c.AER(c.taua, ikl, ibm) * c.AER(c.ssaa, ikl, ibm);
        zgcc[jk] = c.AER(c.asma, ikl, ibm) * c.AER(c.ssaa, ikl, ibm) * c.AER(c.taua, ikl, ibm) / zomcc[jk];
        zomcc[jk] = zomcc[jk] / ztauc[jk];
        // delta scaling of the clear sky
        const double zf = zgcc[jk] * zgcc[jk];
        const double zwf = zomcc[jk] * zf;
        ztauc[jk] = (1.0 - zwf) * ztauc[jk];
        zomcc[jk] = (zomcc[jk] - zwf) / (1.0 - zwf);
        zgcc[jk] = (zgcc[jk] - zf) / (1.0 - zf);
        // total sky: the cloud's (already delta-scaled) optics added (icpr >= 1)
        const double tcm = c.CM(c.taucmc, iw, ikl), wcm = c.CM(c.ssacmc, iw, ikl), gcm = c.CM(c.asmcmc, iw, ikl);
        ztauo[jk] = ztauc[jk] + tcm;
        zomco[jk] = ztauc[jk] * zomcc[jk] + tcm * wcm;
        zgco[jk] = (tcm * wcm * gcm + ztauc[jk] * zomcc[jk] * zgcc[jk]) / zomco[jk];
        zomco[jk] = zomco[jk] / ztauo[jk];
      }
      reftra_sw(klev, lrtchkclr, zgcc.data(), prmu0, ztauc.data(), zomcc.data(), zrefc.data(), zrefdc.data(),
                ztrac.data(), ztradc.data());
      reftra_sw(klev, lrtchkcld, zgco.data(), prmu0, ztauo.data(), zomco.data(), zrefo.data(), zrefdo.data(),
                ztrao.data(), ztrado.data());
      for (int jk = 1; jk <= klev; ++jk) {
        const int ikl = klev + 1 - jk;
        const double zclear = 1.0 - c.CM(c.cldfmc, iw, ikl);
        const double zcloud = c.CM(c.cldfmc, iw, ikl);
        zref[jk] = zclear * zrefc[jk] + zcloud * zrefo[jk];
        zrefd[jk] = zclear * zrefdc[jk] + zcloud * zrefdo[jk];
        ztra[jk] = zclear * ztrac[jk] + zcloud * ztrao[jk];
        ztrad[jk] = zclear * ztradc[jk] + zcloud * ztrado[jk];
        const double zdbtmc = expo(ztauc[jk] / prmu0);
        zdbtc[jk] = zdbtmc;
        ztdbtc[jk + 1] = zdbtc[jk] * ztdbtc[jk];
        const double zdbtmo = expo(ztauo[jk] / prmu0);
        zdbt[jk] = zclear * zdbtmc + zcloud * zdbtmo;
        ztdbt[jk + 1] = zdbt[jk] * ztdbt[jk];
      }
      vrtqdr_sw(klev, zrefc.data(), zrefdc.data(), ztrac.data(), ztradc.data(), zdbtc.data(), zrdndc.data(),
                zrupc.data(), zrupdc.data(), ztdbtc.data(), zcd.data(), zcu.data());
      vrtqdr_sw(klev, zref.data(), zrefd.data(), ztra.data(), ztrad.data(), zdbt.data(), zrdnd.data(), zrup.data(),
                zrupd.data(), ztdbt.data(), zfd.data(), zfu.data());
      for (int jk = 1; jk <= klev + 1; ++jk) {
        const int ikl = klev + 2 - jk;
        pbbfu[ikl] = pbbfu[ikl] + zincflx * zfu[jk];
        pbbfd[ikl] = pbbfd[ikl] + zincflx * zfd[jk];
        pbbcu[ikl] = pbbcu[ikl] + zincflx * zcu[jk];
        pbbcd[ikl] = pbbcd[ikl] + zincflx * zcd[jk];
      }
    }
  }
}

// one column: inatm_sw, cldprmc_sw, setcoef_sw, albedos, spcvmc_sw, outputs (rrtmg_sw_rad.f90:460-586)
int run_column(const Args& a, int iplon, Col& c, double* uf, double* df, double* hr, double* ufc, double* dfc,
               double* hrc) {
  const double zepsec = 1.e-06, zepzen = 1.e-10;
  const double oneminus = 1.0 - zepsec;
  c.alloc(a.nlay);
  inatm_sw(a, iplon, c);
  int e = cldprmc_sw(c, a.inflgsw, a.iceflgsw, a.liqflgsw);
  if (e) return e;
  setcoef_sw(c);
  double cossza = a.coszen[iplon - 1];
  if (cossza < zepzen) cossza = zepzen;
  double albdir[NBND], albdif[NBND];
  for (int ib = 1; ib <= 9; ++ib) {
    albdir[ib - 1] = a.aldir[iplon - 1];
    albdif[ib - 1] = a.aldif[iplon - 1];
  }
  albdir[NBND - 1] = a.aldir[iplon - 1];
  albdif[NBND - 1] = a.aldif[iplon - 1];
  for (int ib = 10; ib <= 13; ++ib) {
    albdir[ib - 1] = a.asdir[iplon - 1];
    albdif[ib - 1] = a.asdif[iplon - 1];
  }
  if (a.icld == 0) {
    std::fill(c.cldfmc.begin(), c.cldfmc.end(), 0.0);
    std::fill(c.taucmc.begin(), c.taucmc.end(), 0.0);
    std::fill(c.taormc.begin(), c.taormc.end(), 0.0);
    std::fill(c.asmcmc.begin(), c.asmcmc.end(), 0.0);
    std::fill(c.ssacmc.begin(), c.ssacmc.end(), 1.0);
  }
  if (a.iaer == 0) {
    std::fill(c.taua.begin(), c.taua.end(), 0.0);
    std::fill(c.asma.begin(), c.asma.end(), 0.0);
    std::fill(c.ssaa.begin(), c.ssaa.end(), 1.0);
  }
  const int nl = a.nlay;
  std::vector<double> bbfd(nl + 2), bbfu(nl + 2), bbcd(nl + 2), bbcu(nl + 2), nflx(nl + 2), nflxc(nl + 2);
  spcvmc_sw(c, albdif, albdir, cossza, oneminus, bbfd.data(), bbfu.data(), bbcd.data(), bbcu.data());
  for (int i = 1; i <= nl + 1; ++i) {
    const size_t o = (iplon - 1) + (size_t)a.ncol * (i - 1);
    ufc[o] = bbcu[i];
    dfc[o] = bbcd[i];
    uf[o] = bbfu[i];
    df[o] = bbfd[i];
    nflxc[i] = bbcd[i] - bbcu[i];
    nflx[i] = bbfd[i] - bbfu[i];
  }
  for (int i = 1; i <= nl; ++i) {
    const size_t o = (iplon - 1) + (size_t)a.ncol * (i - 1);
    const double zdpgcp = heatfac / c.pdp[i];
    hrc[o] = (nflxc[i + 1] - nflxc[i]) * zdpgcp;
    hr[o] = (nflx[i + 1] - nflx[i]) * zdpgcp;
  }
  const size_t ot = (iplon - 1) + (size_t)a.ncol * (nl - 1);
  hrc[ot] = 0.0;
  hr[ot] = 0.0;
  return 0;
}

}  // namespace

extern "C" {

// rrtmg_sw_ini (rrtmg_sw_init.f90:47-172): the lookup table and heatfac; the
// reduced tables come from the container file.
int ora_sw_init(double cpdair, const char* tables_path) {
  g_tab.clear();
  if (!load_container(tables_path)) return ERR_ARGS;
  pref = T("pref");
  preflog = T("preflog");
  tref = T("tref");
  wavenum2 = T("wavenum2");
  if (!pref || !preflog || !tref || !wavenum2 || !T("grav") || !T("secdy") || !T("avogad")) return ERR_ARGS;
  for (int k = 0; k < NBND; ++k) {
    ngc[k] = TI("ngc")[k];
    ngs[k] = TI("ngs")[k];
    nspa[k] = TI("nspa")[k];
    nspb[k] = TI("nspb")[k];
  }
  for (int k = 0; k < NGPT; ++k) ngb[k] = TI("ngb")[k];
  extliq1 = T("extliq1"); ssaliq1 = T("ssaliq1"); asyliq1 = T("asyliq1");
  extice2 = T("extice2"); ssaice2 = T("ssaice2"); asyice2 = T("asyice2");
  extice3 = T("extice3"); ssaice3 = T("ssaice3"); asyice3 = T("asyice3"); fdlice3 = T("fdlice3");
  abari = T("abari"); bbari = T("bbari"); cbari = T("cbari"); dbari = T("dbari"); ebari = T("ebari"); fbari = T("fbari");
  rrsw_scon = T("rrsw_scon")[0];
  heatfac = T("grav")[0] * T("secdy")[0] / (cpdair * 1.e2);
  // exp_tbl (rrtmg_sw_init.f90:109-118)
  const double expeps = 1.e-20, pade = 0.278;
  exp_tbl[0] = 1.0;
  exp_tbl[NTBL] = expeps;
  bpade = 1.0 / pade;
  for (int itr = 1; itr <= NTBL - 1; ++itr) {
    const double tfn = (double)itr / (double)NTBL;
    const double tau_tbl = bpade * tfn / (1.0 - tfn);
    exp_tbl[itr] = std::exp(-tau_tbl);
    if (exp_tbl[itr] <= expeps) exp_tbl[itr] = expeps;
  }
  for (int b = 16; b <= 29; ++b) {
    Band& B = band[b];
    B.ng = ngc[b - 16];
    auto get = [&](const char* n) { return T(bn(b, n)); };
    B.absa = get("absa");
    B.absb = get("absb");
    B.selfref = get("selfref");
    B.forref = get("forref");
    B.sfluxref = get("sfluxref");
    B.rayl = get("rayl");
    B.absch4 = get("absch4");
    B.abso3a = get("abso3a");
    B.abso3b = get("abso3b");
    B.rayla = get("rayla");
    B.raylb = get("raylb");
    B.absh2o = get("absh2o");
    B.absco2 = get("absco2");
    if (B.absa) B.absa_rows = g_tab[bn(b, "absa")].dims[0];
    if (B.absb) B.absb_rows = g_tab[bn(b, "absb")].dims[0];
    if (B.forref) B.nfor = g_tab[bn(b, "forref")].dims[0];
  }
  g_ready = true;
  return 0;
}

// rrtmg_sw (rrtmg_sw_rad.f90:243-586) on Fortran-ordered arrays:
// play tlay h2ovmr o3vmr co2vmr ch4vmr n2ovmr o2vmr reicmcl relqmcl (ncol, nlay),
// plev tlev (ncol, nlay+1), tsfc asdir asdif aldir aldif coszen (ncol),
// McICA arrays (112, ncol, nlay), aerosols (ncol, nlay, 14), outputs
// (ncol, nlay+1) and heating rates (ncol, nlay).  icld and iaer are in/out as
// in the reference (icld outside 0..3 -> 2; iaer not 0, 6, 10 -> 0).
int ora_rrtmg_sw(int ncol, int nlay, int* icld, int* iaer, const double* play, const double* plev,
                 const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                 const double* o3vmr, const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                 const double* o2vmr, const double* asdir, const double* asdif, const double* aldir,
                 const double* aldif, const double* coszen, double adjes, int dyofyr, double scon, int isolvar,
                 int inflgsw, int iceflgsw, int liqflgsw, const double* cldfmcl, const double* taucmcl,
                 const double* ssacmcl, const double* asmcmcl, const double* fsfcmcl, const double* ciwpmcl,
                 const double* clwpmcl, const double* reicmcl, const double* relqmcl, const double* tauaer,
                 const double* ssaaer, const double* asmaer, double* swuflx, double* swdflx, double* swhr,
                 double* swuflxc, double* swdflxc, double* swhrc, int nthreads) {
  if (!g_ready) return ERR_NOT_INIT;
  if (ncol < 0 || nlay < 1 || !icld || !iaer) return ERR_ARGS;
  if (*icld < 0 || *icld > 3) *icld = 2;
  if (*iaer != 0 && *iaer != 6 && *iaer != 10) *iaer = 0;
  if (isolvar >= 0 || *iaer == 6) return ERR_UNSUPPORTED;
  Args a{ncol, nlay, *icld, *iaer, play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
         asdir, asdif, aldir, aldif, coszen, adjes, dyofyr, scon, isolvar, inflgsw, iceflgsw, liqflgsw,
         cldfmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, tauaer, ssaaer, asmaer};
  const int nt = std::max(1, std::min(nthreads, ncol));
  std::vector<int> err(nt, 0);
  auto work = [&](int t) {
    Col c;
    for (int iplon = 1 + t; iplon <= ncol; iplon += nt) {
      const int e = run_column(a, iplon, c, swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc);
      if (e && !err[t]) err[t] = e;
    }
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, t);
    for (auto& x : th) x.join();
  }
  for (int e : err)
    if (e) return e;
  return 0;
}

// cldprmc_sw alone on one column's McICA cells (for cross-checks of the two
// cloud-optics restatements): cldfmc taucmc ssacmc asmcmc fsfcmc ciwpmc
// clwpmc (112, nlayers), reicmc relqmc (nlayers); outputs taormc taucmc
// ssacmc asmcmc (112, nlayers).  Returns cldprmc_sw's status.
int ora_cldprmc_sw_column(int nlayers, int inflag, int iceflag, int liqflag, const double* cldfmc,
                          const double* taucmc, const double* ssacmc, const double* asmcmc, const double* fsfcmc,
                          const double* ciwpmc, const double* clwpmc, const double* reicmc, const double* relqmc,
                          double* taormc_out, double* taucmc_out, double* ssacmc_out, double* asmcmc_out) {
  if (!g_ready) return ERR_NOT_INIT;
  Col c;
  c.alloc(nlayers);
  for (int lay = 1; lay <= nlayers; ++lay) {
    for (int ig = 1; ig <= NGPT; ++ig) {
      const int i = (ig - 1) + NGPT * (lay - 1);
      c.CM(c.cldfmc, ig, lay) = cldfmc[i];
      c.CM(c.taucmc, ig, lay) = taucmc[i];
      c.CM(c.ssacmc, ig, lay) = ssacmc[i];
      c.CM(c.asmcmc, ig, lay) = asmcmc[i];
      c.CM(c.fsfcmc, ig, lay) = fsfcmc[i];
      c.CM(c.ciwpmc, ig, lay) = ciwpmc[i];
      c.CM(c.clwpmc, ig, lay) = clwpmc[i];
    }
    c.reicmc[lay] = reicmc[lay - 1];
    c.relqmc[lay] = relqmc[lay - 1];
  }
  const int err = cldprmc_sw(c, inflag, iceflag, liqflag);
  for (int lay = 1; lay <= nlayers; ++lay)
    for (int ig = 1; ig <= NGPT; ++ig) {
      const int i = (ig - 1) + NGPT * (lay - 1);
      taormc_out[i] = c.CM(c.taormc, ig, lay);
      taucmc_out[i] = c.CM(c.taucmc, ig, lay);
      ssacmc_out[i] = c.CM(c.ssacmc, ig, lay);
      asmcmc_out[i] = c.CM(c.asmcmc, ig, lay);
    }
  return err;
}

// cldprop_sw (rrtmg_sw_cldprop.f90:53-365): the band cloud optics of one
// column, which BRAMS computes per column and hands to mcica_subcol_sw
// (rtm_driver.f90:1356-1368).  Inputs cldfrac ciwp clwp rei rel (nlayers);
// tauc ssac asmc fsfc (14, nlayers), read for inflag 0 (tauc also for the
// cloudy test); outputs taucldorig taucloud ssacloud asmcloud (nlayers, 14),
// the reference's (nlayers, 16:29) columns.  Returns the code of the first
// STOP the reference reaches (outputs of the layers before it are written),
// ERR_UNSUPPORTED where the reference would read coefficients it never set
// (iceflag 0, liqflag 0 with a nonzero water path).
int ora_cldprop_sw(int nlayers, int inflag, int iceflag, int liqflag, const double* cldfrac, const double* tauc,
                   const double* ssac, const double* asmc, const double* fsfc, const double* ciwp, const double* clwp,
                   const double* rei, const double* rel, double* taucldorig, double* taucloud, double* ssacloud,
                   double* asmcloud) {
  if (!g_ready) return ERR_NOT_INIT;
  const double eps = 1.e-06, cldmin = 1.e-20;
  auto IN = [&](const double* v, int ib, int lay) { return v[(ib - 16) + NBND * (lay - 1)]; };  // (ib-15, lay)
  auto OUT = [&](double* v, int lay, int ib) -> double& { return v[(lay - 1) + nlayers * (ib - 16)]; };
  std::vector<double> tauctot(nlayers + 1, 0.0);
  for (int lay = 1; lay <= nlayers; ++lay)
    for (int ib = 16; ib <= 29; ++ib) {
      OUT(taucldorig, lay, ib) = IN(tauc, ib, lay);
      OUT(taucloud, lay, ib) = 0.0;
      OUT(ssacloud, lay, ib) = 1.0;
      OUT(asmcloud, lay, ib) = 0.0;
      tauctot[lay] = tauctot[lay] + IN(tauc, ib, lay);
    }
  double extcoice[30], ssacoice[30], gice[30], forwice[30], fdelta[30];
  double extcoliq[30], ssacoliq[30], gliq[30], forwliq[30];
  for (int lay = 1; lay <= nlayers; ++lay) {
    const double cwp = ciwp[lay - 1] + clwp[lay - 1];
    if (!(cldfrac[lay - 1] >= cldmin && (cwp >= cldmin || tauctot[lay] >= cldmin))) continue;
    if (inflag == 0) {
      for (int ib = 16; ib <= 29; ++ib) {
        const double taucldorig_a = IN(tauc, ib, lay);
        const double ffp = IN(fsfc, ib, lay);
        const double ffp1 = 1.0 - ffp;
        const double ffpssa = 1.0 - ffp * IN(ssac, ib, lay);
        const double ssacloud_a = ffp1 * IN(ssac, ib, lay) / ffpssa;
        const double taucloud_a = ffpssa * taucldorig_a;
        OUT(taucldorig, lay, ib) = taucldorig_a;
        OUT(ssacloud, lay, ib) = ssacloud_a;
        OUT(taucloud, lay, ib) = taucloud_a;
        OUT(asmcloud, lay, ib) = (IN(asmc, ib, lay) - ffp) / (ffp1);
      }
    } else if (inflag == 2) {
      const double radice = rei[lay - 1];
      if (ciwp[lay - 1] == 0.0) {
        for (int ib = 16; ib <= 29; ++ib) extcoice[ib] = ssacoice[ib] = gice[ib] = forwice[ib] = 0.0;
      } else if (iceflag == 1) {
        if (radice < 13.0 || radice > 130.0) return ERR_ICE_BOUNDS;
        for (int ib = 16; ib <= 29; ++ib) {
          const double w2 = wavenum2[ib - 16];
          int icx = 0;
          if (w2 > 1.43e04) icx = 1;
          else if (w2 > 7.7e03) icx = 2;
          else if (w2 > 5.3e03) icx = 3;
          else if (w2 > 4.0e03) icx = 4;
          else if (w2 >= 2.5e03) icx = 5;
          extcoice[ib] = abari[icx - 1] + bbari[icx - 1] / radice;
          ssacoice[ib] = 1.0 - cbari[icx - 1] - dbari[icx - 1] * radice;
          gice[ib] = ebari[icx - 1] + fbari[icx - 1] * radice;
          if (gice[ib] >= 1.0) gice[ib] = 1.0 - eps;
          forwice[ib] = gice[ib] * gice[ib];
          if (extcoice[ib] < 0.0 || ssacoice[ib] > 1.0 || ssacoice[ib] < 0.0 || gice[ib] > 1.0 || gice[ib] < 0.0)
            return ERR_OPTICS;
        }
      } else if (iceflag == 2) {
        if (radice < 5.0 || radice > 131.0) return ERR_ICE_BOUNDS;
        const double factor = (radice - 2.0) / 3.0;
        int index = (int)factor;
        if (index == 43) index = 42;
        const double fint = factor - (double)index;
        for (int ib = 16; ib <= 29; ++ib) {
          extcoice[ib] = C2(extice2, 43, index, ib) + fint * (C2(extice2, 43, index + 1, ib) - C2(extice2, 43, index, ib));
          ssacoice[ib] = C2(ssaice2, 43, index, ib) + fint * (C2(ssaice2, 43, index + 1, ib) - C2(ssaice2, 43, index, ib));
          gice[ib] = C2(asyice2, 43, index, ib) + fint * (C2(asyice2, 43, index + 1, ib) - C2(asyice2, 43, index, ib));
          forwice[ib] = gice[ib] * gice[ib];
          if (extcoice[ib] < 0.0 || ssacoice[ib] > 1.0 || ssacoice[ib] < 0.0 || gice[ib] > 1.0 || gice[ib] < 0.0)
            return ERR_OPTICS;
        }
      } else if (iceflag == 3) {
        if (radice < 5.0 || radice > 140.0) return ERR_DGE_BOUNDS;
        const double factor = (radice - 2.0) / 3.0;
        int index = (int)factor;
        if (index == 46) index = 45;
        const double fint = factor - (double)index;
        for (int ib = 16; ib <= 29; ++ib) {
          extcoice[ib] = C2(extice3, 46, index, ib) + fint * (C2(extice3, 46, index + 1, ib) - C2(extice3, 46, index, ib));
          ssacoice[ib] = C2(ssaice3, 46, index, ib) + fint * (C2(ssaice3, 46, index + 1, ib) - C2(ssaice3, 46, index, ib));
          gice[ib] = C2(asyice3, 46, index, ib) + fint * (C2(asyice3, 46, index + 1, ib) - C2(asyice3, 46, index, ib));
          fdelta[ib] = C2(fdlice3, 46, index, ib) + fint * (C2(fdlice3, 46, index + 1, ib) - C2(fdlice3, 46, index, ib));
          if (fdelta[ib] < 0.0 || fdelta[ib] > 1.0) return ERR_OPTICS;
          forwice[ib] = fdelta[ib] + 0.5 / ssacoice[ib];
          if (forwice[ib] > gice[ib]) forwice[ib] = gice[ib];
          if (extcoice[ib] < 0.0 || ssacoice[ib] > 1.0 || ssacoice[ib] < 0.0 || gice[ib] > 1.0 || gice[ib] < 0.0)
            return ERR_OPTICS;
        }
      } else {
        return ERR_UNSUPPORTED;
      }
      if (clwp[lay - 1] == 0.0) {
        for (int ib = 16; ib <= 29; ++ib) extcoliq[ib] = ssacoliq[ib] = gliq[ib] = forwliq[ib] = 0.0;
      } else if (liqflag == 1) {
        const double radliq = rel[lay - 1];
        if (radliq < 2.5 || radliq > 60.0) return ERR_LIQ_BOUNDS;
        int index = (int)(radliq - 1.5);
        if (index == 0) index = 1;
        if (index == 58) index = 57;
        const double fint = radliq - 1.5 - (double)index;
        for (int ib = 16; ib <= 29; ++ib) {
          extcoliq[ib] = C2(extliq1, 58, index, ib) + fint * (C2(extliq1, 58, index + 1, ib) - C2(extliq1, 58, index, ib));
          ssacoliq[ib] = C2(ssaliq1, 58, index, ib) + fint * (C2(ssaliq1, 58, index + 1, ib) - C2(ssaliq1, 58, index, ib));
          if (fint < 0.0 && ssacoliq[ib] > 1.0) ssacoliq[ib] = C2(ssaliq1, 58, index, ib);
          gliq[ib] = C2(asyliq1, 58, index, ib) + fint * (C2(asyliq1, 58, index + 1, ib) - C2(asyliq1, 58, index, ib));
          forwliq[ib] = gliq[ib] * gliq[ib];
          if (extcoliq[ib] < 0.0 || ssacoliq[ib] > 1.0 || ssacoliq[ib] < 0.0 || gliq[ib] > 1.0 || gliq[ib] < 0.0)
            return ERR_OPTICS;
        }
      } else {
        return ERR_UNSUPPORTED;
      }
      for (int ib = 16; ib <= 29; ++ib) {
        const double tauliqorig = clwp[lay - 1] * extcoliq[ib];
        const double tauiceorig = ciwp[lay - 1] * extcoice[ib];
        OUT(taucldorig, lay, ib) = tauliqorig + tauiceorig;
        const double ssaliq = ssacoliq[ib] * (1.0 - forwliq[ib]) / (1.0 - forwliq[ib] * ssacoliq[ib]);
        const double tauliq = (1.0 - forwliq[ib] * ssacoliq[ib]) * tauliqorig;
        const double ssaice = ssacoice[ib] * (1.0 - forwice[ib]) / (1.0 - forwice[ib] * ssacoice[ib]);
        const double tauice = (1.0 - forwice[ib] * ssacoice[ib]) * tauiceorig;
        const double scatliq = ssaliq * tauliq;
        double scatice = ssaice * tauice;
        OUT(taucloud, lay, ib) = tauliq + tauice;
        if (OUT(taucloud, lay, ib) == 0.0) OUT(taucloud, lay, ib) = cldmin;
        if (scatice == 0.0) scatice = cldmin;
        OUT(ssacloud, lay, ib) = (scatliq + scatice) / OUT(taucloud, lay, ib);
        if (iceflag == 3) {
          OUT(asmcloud, lay, ib) = (1.0 / (scatliq + scatice)) *
                                   (scatliq * (gliq[ib] - forwliq[ib]) / (1.0 - forwliq[ib]) +
                                    scatice * ((gice[ib] - forwice[ib]) / (1.0 - forwice[ib])));
        } else {
          OUT(asmcloud, lay, ib) = (scatliq * (gliq[ib] - forwliq[ib]) / (1.0 - forwliq[ib]) +
                                    scatice * (gice[ib] - forwice[ib]) / (1.0 - forwice[ib])) /
                                   (scatliq + scatice);
        }
      }
    }
  }
  return 0;
}

}  // extern "C"
