// BRAMS's zonal ozone climatology on the longwave columns (host code): the
// sigma levels radrrtmdrv forms from each column's interface pressures
// (src/brams/radiate/rtm_driver.f90:1120-1143), the per-column set-up of
// InitGetoz_rrtm (:2619-2634), getoz_rrtm's seasonal harmonic and latitude
// interpolation of ozone(18, 37, 4) and its linear interpolation in sigma
// (:2638-2823), and the flip into o3vmr (:1168-1173, no chemistry ozone).
// The table comes from brams_ozone.gblw (extracted from the driver's source
// by brams_gb300/data/extract_ozone.py).  The driver's integer year and
// month lengths (year_getoz = 365, mon_getoz = 30: integers assigned from
// 365.25 and 365.25 / 12) are kept.  Compiled without floating-point
// contraction, so the sums round as the driver's statements do.
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gb_rrtmg_lw.h"
#include "lw_tables.h"

struct gb_rtm_ozone {
  std::vector<double> oz;   // ozone(18, 37, 4), 1e-4 g/g, level fastest
  std::vector<double> sig;  // ozsig(18)
  double OZ(int k, int la, int s) const { return oz[(k - 1) + 18 * ((la - 1) + 37 * (s - 1))]; }
};

namespace {

constexpr int kNlev = 18;
constexpr int kYear = 365, kMon = 30;  // year_getoz, mon_getoz (integers)
constexpr double kPai = 3.1415926e0;   // getoz_rrtm's pai and mem_rrtm's pi
constexpr double kRlag = 14.8125e0;

// getoz_rrtm (:2638-2823) for one column: o3l(1..kmax) from sigmid(1..kmax)
int getoz(const gb_rtm_ozone& z, int kmax, const double* sigmid, double colrad, double date, bool inter,
          double* o3l) {
  if (date > kYear) date = date - kYear;
  int imon = (int)(date / kMon + 1);
  if (imon < 1) imon = 1;
  int isea = imon / 3 + 1;
  if (isea == 5) isea = 1;
  if (isea > 5) return GB_LW_E_ARGS;  // the driver's STOP 9954
  const double theta = 90.0 - (180.0 / kPai) * colrad;
  const double flat = 0.2 * theta;
  const int la = (int)(19.501e0 - flat);
  const int ll = (int)(19.001e0 - flat);
  const double rang = 2.0e0 * kPai * (date - kRlag) / kYear;
  const double rsin1 = std::sin(rang), rcos1 = std::cos(rang), rcos2 = std::cos(2.0e0 * rang);
  const double rate = (double)(19 - ll) - flat;
  double ozo3l[kNlev + 1];
  for (int k = 1; k <= kNlev; ++k) {
    const double o1 = z.OZ(k, la, 1), o2 = z.OZ(k, la, 2), o3 = z.OZ(k, la, 3), o4 = z.OZ(k, la, 4);
    const double p1 = z.OZ(k, ll, 1), p2 = z.OZ(k, ll, 2), p3 = z.OZ(k, ll, 3), p4 = z.OZ(k, ll, 4);
    const double a1 = 2.5e-1 * (o1 + o2 + o3 + o4), a2 = 0.5e0 * (o2 - o4), a3 = 0.5e0 * (o1 - o3);
    const double a4 = 2.5e-1 * (o1 + o3 - o2 - o4);
    const double b1 = 2.5e-1 * (p1 + p2 + p3 + p4), b2 = 0.5e0 * (p2 - p4), b3 = 0.5e0 * (p1 - p3);
    const double b4 = 2.5e-1 * (p1 + p3 - p2 - p4);
    const double do3a = a1 + rsin1 * a2 + rcos1 * a3 + rcos2 * a4;
    const double do3b = b1 + rsin1 * b2 + rcos1 * b3 + rcos2 * b4;
    ozo3l[k] = do3a + rate * (do3b - do3a);
    ozo3l[k] = 1.0e-04 * ozo3l[k];
  }
  const double* ozsig = z.sig.data() - 1;  // 1-based
  if (inter) {
    for (int l = 1; l <= kmax; ++l) {
      int kk = 2;
      if (sigmid[l - 1] > ozsig[1]) {
        kk = kNlev;
        for (int k = 2; k <= kNlev; ++k)
          if (sigmid[l - 1] > ozsig[k - 1] && sigmid[l - 1] <= ozsig[k]) {
            kk = k;
            break;
          }
      }
      const double aa = (ozo3l[kk] - ozo3l[kk - 1]) / (ozsig[kk] - ozsig[kk - 1]);
      const double bb = ozo3l[kk - 1] - aa * ozsig[kk - 1];
      o3l[kmax - l] = bb + aa * sigmid[l - 1];  // o3l(kmax+1-l)
    }
  } else {
    for (int l = 1; l <= kNlev; ++l) o3l[l - 1] = ozo3l[l];
  }
  return GB_LW_OK;
}

}  // namespace

extern "C" {

int gb_rtm_ozone_load(const char* table_dir, gb_rtm_ozone** out) {
  if (!out || !table_dir) return GB_LW_E_ARGS;
  *out = nullptr;
  const std::string path = std::string(table_dir) + "/brams_ozone.gblw";
  std::string err;
  auto* z = new gb_rtm_ozone;
  if (!gb_read_table_f64(path.c_str(), "ozone", z->oz, err) || !gb_read_table_f64(path.c_str(), "ozsig", z->sig, err) ||
      z->oz.size() != (size_t)kNlev * 37 * 4 || z->sig.size() != (size_t)kNlev) {
    delete z;
    return GB_LW_E_TABLES;
  }
  *out = z;
  return GB_LW_OK;
}

int gb_rtm_ozone_free(gb_rtm_ozone* z) {
  delete z;
  return GB_LW_OK;
}

int gb_rtm_ozone_lw(const gb_rtm_ozone* z, int ncol, int mzp, const double* plev, int64_t ld, const float* glat,
                    int doy, double* o3vmr, int64_t ld_out) {
  if (!z || ncol < 0 || mzp < 2 || !plev || !glat || !o3vmr || ld < ncol || ld_out < ncol) return GB_LW_E_ARGS;
  const double ro3ar = 1 / (47.998e0 / 28.96e0);  // mem_rrtm.f90:18
  std::vector<double> sig(mzp + 2), sigmid(mzp + 1), o3l(mzp > kNlev ? mzp : kNlev);
  for (int noc = 0; noc < ncol; ++noc) {
    // :1122-1140 sigma at the interfaces and the layer midpoints (1-based)
    for (int i = 2; i <= mzp; ++i) sig[i] = plev[noc + ld * (i - 1)] / plev[noc];
    sig[1] = 1.;
    sig[mzp + 1] = 0.;
    for (int k = 1; k <= mzp; ++k) sigmid[k] = (sig[k] + sig[k + 1]) / 2;
    // :2619-2634 (InitGetoz_rrtm with this column's sig)
    bool inter = kNlev != mzp;
    if (!inter)
      for (int l = 1; l <= kNlev; ++l)
        if (std::fabs(z->sig[l - 1] - sig[kNlev - l + 1]) > 0.0001) inter = true;
    // :1015 colatitude from the grid latitude; :1146 day of year
    const double colrad = kPai * (1.00e0 - ((double)glat[noc] + 90.00e0) / 180.00e0);
    const int rc = getoz(*z, mzp, sigmid.data() + 1, colrad, (double)doy, inter, o3l.data());
    if (rc) return rc;
    // :1168-1173 o3vmr(noc, k) = o3l(noc, flip(k)) * ro3ar, flip(k) = mzp + 1 - k
    for (int k = 1; k <= mzp - 1; ++k) o3vmr[noc + ld_out * (k - 1)] = o3l[mzp - k] * ro3ar;
  }
  return GB_LW_OK;
}

}  // extern "C"
