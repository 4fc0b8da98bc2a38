// Shared definitions of the GB300 RRTMG_LW solver (host + device).
#pragma once
#include <stdint.h>

#define GB_NGPT 140
#define GB_NBND 16
#define GB_MAXLAY 256  // largest nlay a launch accepts (shared memory is sized per launch)

// g-point ranges per band (parrrtm.f90 ngs*, rrtmg_lw_init.f90:326)
#define GB_NG_LIST {10, 12, 16, 14, 16, 8, 12, 8, 12, 6, 8, 8, 4, 2, 2, 2}
#define GB_NGS0_LIST {0, 10, 22, 38, 52, 68, 76, 88, 96, 108, 114, 122, 130, 134, 136, 138}

// Offsets (in floats) of every band table inside the device table blob.
// Layouts are g-fastest so that lanes holding consecutive g-points of one
// band read consecutive words:
//   ka  [65*nspa rows][ng]     (row = the reference's absa first index)
//   kb  [235*max(nspb,1) rows][ng]
//   sr  [10][ng]  fo [4][ng]
//   fa  [neta_a + 1][ng], fb [neta_b + 1][ng]   (one padding row)
//   m*  minor tables [19][neta][ng] (neta = 1 for temperature-only minors)
//   x*  per-g scalars [ng]
struct GbBandTab {
  int ng, g0;
  int ka, kb, fa, fb, sr, fo;
  int ma0, ma1, ma2, mb0, mb1;  // minor gas tables, lower (a) and upper (b)
  int x0, x1;              // per-g cross-section arrays (ccl4, cfc11adj, cfc12, cfc22adj)
  int na_eta, nb_eta;      // rows of fracrefa / fracrefb
};

struct GbTables {
  GbBandTab band[GB_NBND];
  int zero_row;                     // 16 zeros, used as the Planck-fraction row of empty bands
  int totplnk, totplnkderiv;        // [16][181] (band-major)
  int absice0, absice1, absice2, absice3, absliq1;  // cloud optics, reference layouts
  float absliq0, abscld1;
  // reference atmosphere (float) and the chi_mls ratios the bands need, per jp
  float pref[59], preflog[59], tref[59];
  float chi[7][59];
  // chi_mls ratios per pressure level (setcoef.f90:333-346, 387-394):
  // 0 h2o/co2, 1 h2o/o3, 2 h2o/n2o, 3 h2o/ch4, 4 n2o/co2, 5 o3/co2
  float rat[6][59];
  float delwave[GB_NBND];
  // double-precision copies for the decisions near truncation and branch
  // boundaries that are re-taken in fp64 (setcoef's jp/jt/jt1, taumol's specparm)
  double preflog64[59], tref64[59], chi64[7][59];
  // the same reference-atmosphere values in the float blob, for lookups whose
  // index differs from thread to thread: preflog[59], tref[59], chi[7][59], rat[6][59]
  int ref_preflog, ref_tref, ref_chi, ref_rat;
  // rtrnmc's lookup tables (rrtmg_lw_init.f90:120-142) in the float blob:
  // tbl_tt (exp_tbl, tfn_tbl) pairs [10001] (8-byte aligned), tbl_tau [10001]
  int tbl_tt, tbl_tau;
  // per g-point in the float blob: the band (0-based, as int bits) and the
  // flux weight 0.5 * delwave * fluxfac (rtrnmc.f90:538-583)
  int gpt_band, gpt_wgt;
  int ngb[GB_NGPT];
  int nspa[GB_NBND], nspb[GB_NBND];
  double heatfac, fluxfac, grav, avogad;
  int total_floats;
  // the cloud optics tables again in fp64 (for cldprop, which the reference
  // evaluates in double): offsets into a separate double blob
  int c64_absice0, c64_absice1, c64_absice2, c64_absice3, c64_absliq1, c64_absliq0, c64_abscld1, c64_total;
};

// Per-column error codes written by the kernels (0 = ok).  The values match
// the reference's STOP conditions.
enum GbColError {
  GB_COL_OK = 0,
  GB_COL_INFLAG1 = 2,     // cldprmc: 'INFLAG = 1 OPTION NOT AVAILABLE WITH MCICA'
  GB_COL_ICE_SMALL = 3,   // cldprmc: 'ICE RADIUS TOO SMALL'
  GB_COL_ICE_BOUNDS = 4,  // cldprmc: 'ICE RADIUS OUT OF BOUNDS'
  GB_COL_DGE_BOUNDS = 5,  // cldprmc: 'ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS'
  GB_COL_LIQ_BOUNDS = 6,  // cldprmc: 'LIQUID EFFECTIVE RADIUS OUT OF BOUNDS'
  GB_COL_LAYTROP = 9,     // lower-atmosphere layers not a prefix of the column
  GB_COL_BADVAL = 11,     // non-finite or non-positive pressure / temperature
  GB_COL_TCWAIT = 12,     // learned gas optics: a tensor-core wait ran out (kernel stopped early)
  GB_COL_SW_OPTICS = 13,  // cldprmc_sw: cloud extinction, albedo, asymmetry or fdelta out of range
  GB_COL_SW_UNSUPPORTED = 14,  // cldprmc_sw: ice option 0 or liquid option 0 with a nonzero path
};
