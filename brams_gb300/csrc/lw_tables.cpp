// Host-side table loading: reads the two table containers (reference tables
// and reduced k-distribution tables, format described in
// brams_gb300/tables_io.py) and lays every table out for the device as one
// float blob plus the offsets in GbTables.  This is the GPU counterpart of
// rrtmg_lw_ini (rrtmg_lw_init.f90:47-194): the per-band coefficient tables,
// Planck tables and cloud tables end up resident in device memory once per
// context.
#include "lw_tables.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {
using Entry = GbTableEntry;
}  // namespace

bool gb_read_container(const char* path, std::map<std::string, Entry>& out, std::string& err) {
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    err = std::string("cannot open table file ") + path;
    return false;
  }
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
    Entry a;
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
    out[name] = std::move(a);
  }
  std::fclose(f);
  if (!ok) err = std::string("malformed table file ") + path;
  return ok;
}

bool gb_read_table_f64(const char* path, const char* name, std::vector<double>& out, std::string& err) {
  std::map<std::string, Entry> tab;
  if (!gb_read_container(path, tab, err)) return false;
  auto it = tab.find(name);
  if (it == tab.end() || it->second.is_int) {
    err = std::string("table file ") + path + " has no float64 array " + name;
    return false;
  }
  out = it->second.d;
  return true;
}

bool gb_build_tables(const char* ref_path, const char* k_path, double cpdair, GbTables& T,
                     std::vector<float>& blob, std::string& err, std::vector<double>* cloud64) {
  std::map<std::string, Entry> tab;
  if (!gb_read_container(ref_path, tab, err) || !gb_read_container(k_path, tab, err)) return false;
  auto need = [&](const std::string& n) -> const Entry* {
    auto it = tab.find(n);
    if (it == tab.end()) {
      err = "missing table " + n;
      return nullptr;
    }
    return &it->second;
  };
  std::memset(&T, 0, sizeof(T));
  blob.clear();
  auto push = [&](size_t n) {
    int off = (int)blob.size();
    blob.resize(blob.size() + n, 0.0f);
    return off;
  };
  static const int NG[16] = GB_NG_LIST, NGS0[16] = GB_NGS0_LIST;
  const Entry *nspa = need("nspa"), *nspb = need("nspb"), *ngb = need("ngb");
  if (!nspa || !nspb || !ngb) return false;
  for (int b = 0; b < 16; ++b) {
    T.nspa[b] = nspa->i[b];
    T.nspb[b] = nspb->i[b];
  }
  for (int g = 0; g < GB_NGPT; ++g) T.ngb[g] = ngb->i[g];

  T.zero_row = push(16);
  for (int b = 1; b <= 16; ++b) {
    GbBandTab& B = T.band[b - 1];
    const int ng = NG[b - 1];
    B.ng = ng;
    B.g0 = NGS0[b - 1];
    B.ka = B.kb = B.fa = B.fb = B.sr = B.fo = -1;
    B.ma0 = B.ma1 = B.ma2 = B.mb0 = B.mb1 = B.x0 = B.x1 = -1;
    char key[64];
    auto name = [&](const char* n) {
      std::snprintf(key, sizeof key, "b%02d.%s", b, n);
      return std::string(key);
    };
    auto has = [&](const char* n) { return tab.count(name(n)) > 0; };
    // [rows][ng] from Fortran (rows..., ng): transpose
    auto put_rows_g = [&](const char* n) {
      const Entry* e = need(name(n));
      if (!e) return -1;
      size_t rows = e->size() / ng;
      int off = push(rows * ng);
      for (size_t r = 0; r < rows; ++r)
        for (int g = 0; g < ng; ++g) blob[off + r * ng + g] = (float)e->d[r + rows * g];
      return off;
    };
    B.ka = put_rows_g("ka");
    if (has("kb")) B.kb = put_rows_g("kb");
    B.sr = put_rows_g("selfref");
    B.fo = put_rows_g("forref");
    // Planck fractions: Fortran (ng) or (ng, neta) -> [neta + 1][ng]
    auto put_frac = [&](const char* n, int& nrows) {
      const Entry* e = need(name(n));
      if (!e) return -1;
      int neta = (int)(e->size() / ng);
      nrows = neta;
      int off = push((size_t)(neta + 1) * ng);
      for (int r = 0; r < neta; ++r)
        for (int g = 0; g < ng; ++g) blob[off + r * ng + g] = (float)e->d[g + (size_t)ng * r];
      for (int g = 0; g < ng; ++g) blob[off + neta * ng + g] = blob[off + (neta - 1) * ng + g];
      return off;
    };
    B.fa = put_frac("fracrefa", B.na_eta);
    if (has("fracrefb")) B.fb = put_frac("fracrefb", B.nb_eta);
    // minor tables: Fortran (19, ng) -> [19][ng]; (neta, 19, ng) -> [19][neta][ng]
    auto put_minor = [&](const char* n) {
      const Entry* e = need(name(n));
      if (!e) return -1;
      if (e->ndim == 2) return put_rows_g(n);
      int neta = e->dims[0];
      int off = push((size_t)19 * neta * ng);
      for (int t = 0; t < 19; ++t)
        for (int a = 0; a < neta; ++a)
          for (int g = 0; g < ng; ++g)
            blob[off + ((size_t)t * neta + a) * ng + g] = (float)e->d[a + (size_t)neta * (t + 19 * (size_t)g)];
      return off;
    };
    auto put_vec = [&](const char* n) {
      const Entry* e = need(name(n));
      if (!e) return -1;
      int off = push(ng);
      for (int g = 0; g < ng; ++g) blob[off + g] = (float)e->d[g];
      return off;
    };
    switch (b) {
      case 1: B.ma0 = put_minor("ka_mn2"); B.mb0 = put_minor("kb_mn2"); break;
      case 3: B.ma0 = put_minor("ka_mn2o"); B.mb0 = put_minor("kb_mn2o"); break;
      case 5: B.ma0 = put_minor("ka_mo3"); B.x0 = put_vec("ccl4"); break;
      case 6: B.ma0 = put_minor("ka_mco2"); B.x0 = put_vec("cfc11adj"); B.x1 = put_vec("cfc12"); break;
      case 7: B.ma0 = put_minor("ka_mco2"); B.mb0 = put_minor("kb_mco2"); break;
      case 8:
        B.ma0 = put_minor("ka_mco2"); B.ma1 = put_minor("ka_mn2o"); B.ma2 = put_minor("ka_mo3");
        B.mb0 = put_minor("kb_mco2"); B.mb1 = put_minor("kb_mn2o");
        B.x0 = put_vec("cfc12"); B.x1 = put_vec("cfc22adj");
        break;
      case 9: B.ma0 = put_minor("ka_mn2o"); B.mb0 = put_minor("kb_mn2o"); break;
      case 11: B.ma0 = put_minor("ka_mo2"); B.mb0 = put_minor("kb_mo2"); break;
      case 13: B.ma0 = put_minor("ka_mco2"); B.ma1 = put_minor("ka_mco"); B.mb0 = put_minor("kb_mo3"); break;
      case 15: B.ma0 = put_minor("ka_mn2"); break;
      default: break;
    }
    if (!err.empty()) return false;
  }
  // Planck tables, band-major [16][181]
  const Entry *tp = need("totplnk"), *tpd = need("totplnkderiv");
  if (!tp || !tpd) return false;
  T.totplnk = push(16 * 181);
  T.totplnkderiv = push(16 * 181);
  for (int b = 0; b < 16; ++b)
    for (int i = 0; i < 181; ++i) {
      blob[T.totplnk + b * 181 + i] = (float)tp->d[i + 181 * b];
      blob[T.totplnkderiv + b * 181 + i] = (float)tpd->d[i + 181 * b];
    }
  // cloud optics tables in the reference's (index, band) layout
  auto put_flat = [&](const char* n) {
    const Entry* e = need(n);
    if (!e) return -1;
    int off = push(e->size());
    for (size_t k = 0; k < e->size(); ++k) blob[off + k] = (float)e->d[k];
    return off;
  };
  T.absice0 = put_flat("absice0");
  T.absice1 = put_flat("absice1");
  T.absice2 = put_flat("absice2");
  T.absice3 = put_flat("absice3");
  T.absliq1 = put_flat("absliq1");
  const Entry *aliq0 = need("absliq0"), *acld1 = need("abscld1"), *pref = need("pref"),
              *preflog = need("preflog"), *tref = need("tref"), *chi = need("chi_mls"),
              *delw = need("delwave"), *grav = need("grav"), *avog = need("avogad"),
              *secdy = need("secdy");
  if (!aliq0 || !acld1 || !pref || !preflog || !tref || !chi || !delw || !grav || !avog || !secdy)
    return false;
  T.absliq0 = (float)aliq0->d[0];
  T.abscld1 = (float)acld1->d[0];
  if (cloud64) {
    std::vector<double>& c = *cloud64;
    c.clear();
    auto put64 = [&](const char* n) {
      const Entry* e = need(n);
      const int off = (int)c.size();
      c.insert(c.end(), e->d.begin(), e->d.end());
      return off;
    };
    T.c64_absice0 = put64("absice0");
    T.c64_absice1 = put64("absice1");
    T.c64_absice2 = put64("absice2");
    T.c64_absice3 = put64("absice3");
    T.c64_absliq1 = put64("absliq1");
    T.c64_absliq0 = put64("absliq0");
    T.c64_abscld1 = put64("abscld1");
    T.c64_total = (int)c.size();
  }
  for (int j = 0; j < 59; ++j) {
    T.pref[j] = (float)pref->d[j];
    T.preflog[j] = (float)preflog->d[j];
    T.tref[j] = (float)tref->d[j];
    for (int m = 0; m < 7; ++m) T.chi[m][j] = (float)chi->d[m + 7 * j];
    T.preflog64[j] = preflog->d[j];
    T.tref64[j] = tref->d[j];
    for (int m = 0; m < 7; ++m) T.chi64[m][j] = chi->d[m + 7 * j];
    auto c = [&](int m) { return chi->d[(m - 1) + 7 * j]; };
    T.rat[0][j] = (float)(c(1) / c(2));
    T.rat[1][j] = (float)(c(1) / c(3));
    T.rat[2][j] = (float)(c(1) / c(4));
    T.rat[3][j] = (float)(c(1) / c(6));
    T.rat[4][j] = (float)(c(4) / c(2));
    T.rat[5][j] = (float)(c(3) / c(2));
  }
  // the reference atmosphere again in the blob (read with per-thread indices)
  T.ref_preflog = push(59);
  T.ref_tref = push(59);
  T.ref_chi = push(7 * 59);
  T.ref_rat = push(6 * 59);
  for (int j = 0; j < 59; ++j) {
    blob[T.ref_preflog + j] = T.preflog[j];
    blob[T.ref_tref + j] = T.tref[j];
    for (int m = 0; m < 7; ++m) blob[T.ref_chi + m * 59 + j] = T.chi[m][j];
    for (int k = 0; k < 6; ++k) blob[T.ref_rat + k * 59 + j] = T.rat[k][j];
  }
  // rtrnmc's lookup tables, computed in double precision as rrtmg_lw_init.f90:120-142
  // does (tfn = real(itr)/real(ntbl) is a default-real division there)
  {
    const int ntbl = 10000;
    const double expeps = 1.e-20, bpade = 1.0 / 0.278;
    while (blob.size() % 2) blob.push_back(0.0f);
    T.tbl_tt = push(2 * (ntbl + 1));
    T.tbl_tau = push(ntbl + 1);
    for (int itr = 0; itr <= ntbl; ++itr) {
      double tau, ex, tf;
      if (itr == 0) {
        tau = 0.0; ex = 1.0; tf = 0.0;
      } else if (itr == ntbl) {
        tau = 1.e10; ex = expeps; tf = 1.0;
      } else {
        const double t = (double)((float)itr / (float)ntbl);
        tau = bpade * t / (1.0 - t);
        ex = std::exp(-tau);
        if (ex <= expeps) ex = expeps;
        tf = tau < 0.06 ? tau / 6.0 : 1.0 - 2.0 * ((1.0 / tau) - (ex / (1. - ex)));
      }
      blob[T.tbl_tt + 2 * itr] = (float)ex;
      blob[T.tbl_tt + 2 * itr + 1] = (float)tf;
      blob[T.tbl_tau + itr] = (float)tau;
    }
  }
  for (int b = 0; b < 16; ++b) T.delwave[b] = (float)delw->d[b];
  T.grav = grav->d[0];
  T.avogad = avog->d[0];
  T.heatfac = grav->d[0] * secdy->d[0] / (cpdair * 1.e2);  // lwdatinit :298
  T.fluxfac = 2.0 * std::asin(1.0) * 2.e4;                   // rrtmg_lw_rad.f90:453
  T.gpt_band = push(GB_NGPT);
  T.gpt_wgt = push(GB_NGPT);
  for (int g = 0; g < GB_NGPT; ++g) {
    const int b = T.ngb[g] - 1;
    std::memcpy(&blob[T.gpt_band + g], &b, 4);
    blob[T.gpt_wgt + g] = (float)(0.5 * (double)T.delwave[b] * T.fluxfac);
  }
  // pad to a multiple of 4 floats (16 bytes)
  while (blob.size() % 4) blob.push_back(0.0f);
  T.total_floats = (int)blob.size();
  return true;
}
