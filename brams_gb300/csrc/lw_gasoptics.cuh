// Gas optics (taumol, rrtmg_lw_taumol.f90:299-3216) as per-layer term lists.
//
// Every taugbN computes, for each layer and g-point of band N, a sum of table
// entries weighted by layer quantities: key-species interpolation in
// pressure, temperature and binary-species parameter (bilinear, or the
// three-point stencil in eta at taumol.f90:582-700), water-vapour self and
// foreign continua, minor absorbers and cross sections.  All weights and all
// table rows depend on the layer only; the g-point only selects the column of
// each table row.  So the GPU splits taumol in two:
//
//   prologue<b>(layer) -- band-specific code run once per (layer, band): the
//     reference's per-layer arithmetic (specparm/js/fs, p**4 stencil factors,
//     adjusted CO2/N2O columns, corradj, ...) producing at most MAXT[b]
//     (weight, row) terms, the Planck-fraction record and the aerosol optical
//     depth to add (rrtmg_lw_rad.f90:548-553);
//   cell(layer, g)     -- identical code for all bands: taug = sum_k w_k *
//     T[row_k + g], times the band-4/band-7 upper-atmosphere g-point factors
//     (taumol.f90:1044-1050, 1687-1692).
//
// Tables are g-fastest (see lw_common.h), so lanes holding consecutive g of a
// layer read one contiguous run per term.  Sums are reassociated relative to
// the reference (single precision); a term whose weight is zero still points
// at a valid row so that every band has a fixed trip count.
#pragma once
#include "lw_common.h"

namespace gb {

enum LayerField {
  F_FAC00, F_FAC01, F_FAC10, F_FAC11,
  F_COLH2O, F_COLCO2, F_COLO3, F_COLN2O, F_COLCO, F_COLCH4, F_COLO2, F_COLBRD,
  F_SELFFAC, F_SELFFRAC, F_FORFAC, F_FORFRAC, F_MINORFRAC, F_SCALEMINOR, F_SCALEMINORN2,
  F_COLDRY, F_PAVEL, F_WX1, F_WX2, F_WX3, F_WX4,
  NF
};
enum LayerIndex { I_JP, I_JT, I_JT1, I_INDSELF, I_INDFOR, I_INDMINOR, NI };

// Table offsets and reference constants; defined here because lw_solver.cu is
// the only translation unit that includes this header.
__constant__ GbTables c_T;

// most terms any band needs in one layer (band 13, lower atmosphere)
constexpr int MAXT_ALL = 24;
// per band: max over lower and upper atmosphere
__host__ __device__ constexpr int maxt(int b) {
  constexpr int m[17] = {0, 10, 8, 20, 16, 21, 12, 20, 16, 20, 8, 10, 16, 24, 8, 20, 16};
  return m[b];
}
__host__ __device__ constexpr int ngb_const(int b) {
  constexpr int m[17] = {0, 10, 12, 16, 14, 16, 8, 12, 8, 12, 6, 8, 8, 4, 2, 2, 2};
  return m[b];
}
__host__ __device__ constexpr int g0_const(int b) {
  constexpr int m[17] = {0, 0, 10, 22, 38, 52, 68, 76, 88, 96, 108, 114, 122, 130, 134, 136, 138};
  return m[b];
}

// fp64 column amounts of the binary species kept per layer (for decisions
// near a stencil switch or a truncation, re-taken in double precision)
enum LayerDouble { D_H2O, D_CO2, D_O3, D_N2O, D_CH4, ND };

// A binary-species amount: its fp32 value and the index of its fp64 copy.
struct Amt {
  float v;
  int d;
  __device__ __forceinline__ operator float() const { return v; }
};
// A chi_mls ratio chi(m1, jp) / chi(m2, jp): its fp32 value and how to form it in fp64.
struct Rat {
  float v;
  int m1, m2, jp;
};

struct Cell {
  const float* f;  // [NF][nl] shared memory
  const int* iv;   // [NI][nl] shared memory
  int nl, lay;
  const float* T;  // device table blob
  const double* d; // [ND][nl] shared memory: fp64 column amounts
  __device__ __forceinline__ float F(int k) const { return f[k * nl + lay]; }
  __device__ __forceinline__ int I(int k) const { return iv[k * nl + lay]; }
  __device__ __forceinline__ double D(int k) const { return d[k * nl + lay]; }
  __device__ __forceinline__ Amt A(int field) const {
    const int k = field == F_COLH2O ? D_H2O : field == F_COLCO2 ? D_CO2 : field == F_COLO3 ? D_O3
                : field == F_COLN2O ? D_N2O : D_CH4;
    return Amt{F(field), k};
  }
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Planck-fraction record of a (layer, band): frac(g) = T[off+g] + fpl*(T[off+ng+g]-T[off+g])
struct FracRec {
  int off;
  float fpl;
};

// A term list under construction: weights and absolute table offsets of row starts.
// Term k of the layer lives at t[k * stride] (term-major storage, so the
// threads of consecutive layers write and read consecutive words).
struct Terms {
  float2* t;
  int stride;
  int n;
  __device__ __forceinline__ void add(float w, int off) {
    t[n * stride] = make_float2(w, __int_as_float(off));
    ++n;
  }
  __device__ __forceinline__ void scale(float s) {
    for (int k = 0; k < n; ++k) t[k * stride].x *= s;
  }
  __device__ __forceinline__ void pad(int maxt, int off) {
    while (n < maxt) add(0.0f, off);
  }
};

// chi_mls and its ratios at reference level jp: a per-layer index, so they are
// read from the table blob (global memory) rather than the constant bank,
// which serialises loads whose address differs between threads
__device__ __forceinline__ float chi(const Cell& c, int m, int jp) { return __ldg(c.T + c_T.ref_chi + (m - 1) * 59 + jp - 1); }
// setcoef's per-layer ratios (setcoef.f90:333-346, 387-394): 0 h2o/co2,
// 1 h2o/o3, 2 h2o/n2o, 3 h2o/ch4, 4 n2o/co2, 5 o3/co2
__device__ __forceinline__ Rat rat(const Cell& c, int k, int jp) {
  constexpr int m1[6] = {1, 1, 1, 1, 4, 3}, m2[6] = {2, 3, 4, 6, 2, 2};
  return Rat{__ldg(c.T + c_T.ref_rat + k * 59 + jp - 1), m1[k], m2[k], jp};
}
// a ratio of chi_mls entries at a fixed reference level (the refrat_* constants)
__device__ __forceinline__ Rat ratio(const Cell& c, int m1, int m2, int jp) {
  return Rat{chi(c, m1, jp) / chi(c, m2, jp), m1, m2, jp};
}

struct Spec {
  float comb, parm, f;
  int j;
  int mode;  // 1: specparm < 0.125, 2: specparm > 0.875, 0: between (taumol.f90:582-611)
};
// speccomb/specparm/specmult/js/fs (e.g. taumol.f90:517-522); oneminus = 1 - 1e-6.
// Computed in fp32; where specparm lies within 1e-5 of 0.125 or 0.875, or
// scale * specparm within 1e-4 of an integer, the decisions (stencil mode,
// js, fs) are re-taken in fp64 from the fp64 column amounts and ratio, as the
// reference computes them.
// the fp64 decisions of spec() (rarely taken: kept out of line so that the
// band prologues stay small)
__device__ __noinline__ Spec spec_fp64(double a64, double b64, int m1, int m2, int jp, float scale, int jmax) {
  Spec s;
  const double r64 = c_T.chi64[m1 - 1][jp - 1] / c_T.chi64[m2 - 1][jp - 1];
  s.comb = (float)(a64 + r64 * b64);
  double p64 = a64 / (a64 + r64 * b64);
  if (p64 >= 1.0 - 1.e-6) p64 = 1.0 - 1.e-6;
  if (!(p64 >= 0.0)) p64 = 0.0;
  const double m64 = (double)scale * p64;
  const int ji = (int)m64;
  s.parm = (float)p64;
  s.j = clampi(1 + ji, 1, jmax);
  s.f = (float)(m64 - (double)ji);
  s.mode = p64 < 0.125 ? 1 : (p64 > 0.875 ? 2 : 0);
  return s;
}

__device__ __forceinline__ Spec spec(const Cell& c, Amt a, Rat rat, Amt b, float scale, int jmax) {
  Spec s;
  s.comb = a.v + rat.v * b.v;
  s.parm = __fdividef(a.v, s.comb);
  if (!(s.parm < 0.999999f)) s.parm = 0.999999f;
  if (!(s.parm >= 0.0f)) s.parm = 0.0f;  // negative amounts: outside the tables' domain
  float mult = scale * s.parm;
  const bool near = fabsf(s.parm - 0.125f) < 1.0e-5f || fabsf(s.parm - 0.875f) < 1.0e-5f ||
                    fabsf(mult - rintf(mult)) < 1.0e-4f;
  if (near) {
    const Spec d = spec_fp64(c.D(a.d), c.D(b.d), rat.m1, rat.m2, rat.jp, scale, jmax);
    s.parm = d.parm;
    s.j = d.j;
    s.f = d.f;
    s.mode = d.mode;
    return s;
  }
  int ji = (int)mult;
  s.j = clampi(1 + ji, 1, jmax);
  s.f = mult - (float)ji;
  s.mode = s.parm < 0.125f ? 1 : (s.parm > 0.875f ? 2 : 0);
  return s;
}

// --- term emitters -----------------------------------------------------------
// water-vapour self continuum (e.g. taumol.f90:344-345)
__device__ __forceinline__ void self_terms(Terms& t, const Cell& c, int sr, int ng) {
  int inds = clampi(c.I(I_INDSELF), 1, 9);
  float f = c.F(F_SELFFAC), fr = c.F(F_SELFFRAC);
  t.add(f * (1.0f - fr), sr + (inds - 1) * ng);
  t.add(f * fr, sr + inds * ng);
}
// foreign continuum (e.g. taumol.f90:346-347)
__device__ __forceinline__ void for_terms(Terms& t, const Cell& c, int fo, int ng) {
  int indf = clampi(c.I(I_INDFOR), 1, 3);
  float f = c.F(F_FORFAC), fr = c.F(F_FORFRAC);
  t.add(f * (1.0f - fr), fo + (indf - 1) * ng);
  t.add(f * fr, fo + indf * ng);
}
// temperature-interpolated minor absorber times `amount`, table [19][ng]
__device__ __forceinline__ void minor_t_terms(Terms& t, const Cell& c, float amount, int m, int ng) {
  int indm = clampi(c.I(I_INDMINOR), 1, 18);
  float mf = c.F(F_MINORFRAC);
  t.add(amount * (1.0f - mf), m + (indm - 1) * ng);
  t.add(amount * mf, m + indm * ng);
}
// eta- and temperature-interpolated minor absorber, table [19][neta][ng]
__device__ __forceinline__ void minor_et_terms(Terms& t, const Cell& c, float amount, int m, int neta, int ng,
                                               int jm, float fm) {
  int indm = clampi(c.I(I_INDMINOR), 1, 18);
  jm = clampi(jm, 1, neta - 1);
  float mf = c.F(F_MINORFRAC);
  auto row = [&](int a, int tt) { return m + ((tt - 1) * neta + (a - 1)) * ng; };
  t.add(amount * (1.0f - fm) * (1.0f - mf), row(jm, indm));
  t.add(amount * fm * (1.0f - mf), row(jm + 1, indm));
  t.add(amount * (1.0f - fm) * mf, row(jm, indm + 1));
  t.add(amount * fm * mf, row(jm + 1, indm + 1));
}
// single key species, lower atmosphere (e.g. taumol.f90:350-354)
__device__ __forceinline__ void single_lower_terms(Terms& t, const Cell& c, float key, int ka, int ng) {
  int jp = clampi(c.I(I_JP), 1, 12), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int ind0 = ((jp - 1) * 5 + (jt - 1)) + 1, ind1 = (jp * 5 + (jt1 - 1)) + 1;
  t.add(key * c.F(F_FAC00), ka + (ind0 - 1) * ng);
  t.add(key * c.F(F_FAC10), ka + ind0 * ng);
  t.add(key * c.F(F_FAC01), ka + (ind1 - 1) * ng);
  t.add(key * c.F(F_FAC11), ka + ind1 * ng);
}
// single key species, upper atmosphere (e.g. taumol.f90:388-392)
__device__ __forceinline__ void single_upper_terms(Terms& t, const Cell& c, float key, int kb, int nspb, int ng) {
  int jp = clampi(c.I(I_JP), 13, 58), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int ind0 = ((jp - 13) * 5 + (jt - 1)) * nspb + 1, ind1 = ((jp - 12) * 5 + (jt1 - 1)) * nspb + 1;
  t.add(key * c.F(F_FAC00), kb + (ind0 - 1) * ng);
  t.add(key * c.F(F_FAC10), kb + ind0 * ng);
  t.add(key * c.F(F_FAC01), kb + (ind1 - 1) * ng);
  t.add(key * c.F(F_FAC11), kb + ind1 * ng);
}
// one binary-species stencil of the lower atmosphere (taumol.f90:582-700):
// six terms in every mode (the interior two-point mode pads with zeros)
__device__ __forceinline__ void stencil9_terms(Terms& t, const Spec& s, int ind, float fa, float fb, int ka, int ng) {
  auto R = [&](int i) { return ka + (i - 1) * ng; };
  if (s.mode == 1) {
    float p = s.f - 1.0f, p4 = (p * p) * (p * p);
    float k0 = p4, k1 = 1.0f - p - 2.0f * p4, k2 = p + p4;
    t.add(s.comb * k0 * fa, R(ind)); t.add(s.comb * k1 * fa, R(ind + 1)); t.add(s.comb * k2 * fa, R(ind + 2));
    t.add(s.comb * k0 * fb, R(ind + 9)); t.add(s.comb * k1 * fb, R(ind + 10)); t.add(s.comb * k2 * fb, R(ind + 11));
  } else if (s.mode == 2) {
    float p = -s.f, p4 = (p * p) * (p * p);
    float k0 = p4, k1 = 1.0f - p - 2.0f * p4, k2 = p + p4;
    t.add(s.comb * k2 * fa, R(ind - 1)); t.add(s.comb * k1 * fa, R(ind)); t.add(s.comb * k0 * fa, R(ind + 1));
    t.add(s.comb * k2 * fb, R(ind + 8)); t.add(s.comb * k1 * fb, R(ind + 9)); t.add(s.comb * k0 * fb, R(ind + 10));
  } else {
    t.add(s.comb * (1.0f - s.f) * fa, R(ind)); t.add(s.comb * s.f * fa, R(ind + 1)); t.add(0.0f, R(ind));
    t.add(s.comb * (1.0f - s.f) * fb, R(ind + 9)); t.add(s.comb * s.f * fb, R(ind + 10)); t.add(0.0f, R(ind));
  }
}
__device__ __forceinline__ int js_lower(const Spec& s) {
  if (s.mode == 1) return clampi(s.j, 1, 7);
  if (s.mode == 2) return clampi(s.j, 2, 8);
  return clampi(s.j, 1, 8);
}
__device__ __forceinline__ void binary_lower_terms(Terms& t, const Cell& c, const Spec& s, const Spec& s1, int ka, int ng) {
  int jp = clampi(c.I(I_JP), 1, 12), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int ind0 = ((jp - 1) * 5 + (jt - 1)) * 9 + js_lower(s);
  int ind1 = (jp * 5 + (jt1 - 1)) * 9 + js_lower(s1);
  stencil9_terms(t, s, ind0, c.F(F_FAC00), c.F(F_FAC10), ka, ng);
  stencil9_terms(t, s1, ind1, c.F(F_FAC01), c.F(F_FAC11), ka, ng);
}
// upper-atmosphere binary species with nspb = 5 (taumol.f90:775-789)
__device__ __forceinline__ void binary_upper_terms(Terms& t, const Cell& c, const Spec& s, const Spec& s1, int kb, int ng) {
  int jp = clampi(c.I(I_JP), 13, 58), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int js = clampi(s.j, 1, 4), js1 = clampi(s1.j, 1, 4);
  int ind0 = ((jp - 13) * 5 + (jt - 1)) * 5 + js, ind1 = ((jp - 12) * 5 + (jt1 - 1)) * 5 + js1;
  auto R = [&](int i) { return kb + (i - 1) * ng; };
  float fa = c.F(F_FAC00), fb = c.F(F_FAC10), fc = c.F(F_FAC01), fd = c.F(F_FAC11);
  t.add(s.comb * (1.0f - s.f) * fa, R(ind0)); t.add(s.comb * s.f * fa, R(ind0 + 1));
  t.add(s.comb * (1.0f - s.f) * fb, R(ind0 + 5)); t.add(s.comb * s.f * fb, R(ind0 + 6));
  t.add(s1.comb * (1.0f - s1.f) * fc, R(ind1)); t.add(s1.comb * s1.f * fc, R(ind1 + 1));
  t.add(s1.comb * (1.0f - s1.f) * fd, R(ind1 + 5)); t.add(s1.comb * s1.f * fd, R(ind1 + 6));
}

// CO2 / N2O column adjustment (e.g. taumol.f90:545-552)
__device__ __forceinline__ float adj_col(float col, float coldry, float chiref, float thresh, float base,
                                          float expo) {
  float ratio = 1.e20f * __fdividef(__fdividef(col, coldry), chiref);
  if (ratio > thresh) {
    float adjfac = base + powf(ratio - base, expo);
    return adjfac * chiref * coldry * 1.e-20f;
  }
  return col;
}
__device__ __forceinline__ float adj_n2o(const Cell& c) {
  return adj_col(c.F(F_COLN2O), c.F(F_COLDRY), chi(c, 4, clampi(c.I(I_JP), 1, 58) + 1), 1.5f, 0.5f, 0.65f);
}

// -------------------------------------------------------------------------
// prologue<b>: terms of band b at one layer; returns the Planck-fraction record.
#define BT c_T.band[b - 1]
#define NGB ngb_const(b)

template <int b>
__device__ FracRec prologue(const Cell& c, bool lower, Terms& t);

// band 1 (taumol.f90:299-399)
template <>
__device__ FracRec prologue<1>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 1;
  float scalen2 = c.F(F_COLBRD) * c.F(F_SCALEMINORN2);
  float pp = c.F(F_PAVEL);
  if (lower) {
    float corradj = pp < 250.0f ? 1.0f - 0.15f * (250.0f - pp) / 154.4f : 1.0f;
    single_lower_terms(t, c, c.F(F_COLH2O), BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_t_terms(t, c, scalen2, BT.ma0, NGB);
    t.scale(corradj);
    return {BT.fa, 0.0f};
  }
  float corradj = 1.0f - 0.15f * (pp / 95.6f);
  single_upper_terms(t, c, c.F(F_COLH2O), BT.kb, 1, NGB);
  for_terms(t, c, BT.fo, NGB);
  minor_t_terms(t, c, scalen2, BT.mb0, NGB);
  t.scale(corradj);
  return {BT.fb, 0.0f};
}

// band 2 (taumol.f90:402-474)
template <>
__device__ FracRec prologue<2>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 2;
  if (lower) {
    float corradj = 1.0f - 0.05f * (c.F(F_PAVEL) - 100.0f) / 900.0f;
    single_lower_terms(t, c, c.F(F_COLH2O), BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    t.scale(corradj);
    return {BT.fa, 0.0f};
  }
  single_upper_terms(t, c, c.F(F_COLH2O), BT.kb, 1, NGB);
  for_terms(t, c, BT.fo, NGB);
  return {BT.fb, 0.0f};
}

// band 3 (taumol.f90:477-792)
template <>
__device__ FracRec prologue<3>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 3;
  int jp = clampi(c.I(I_JP), 1, 58);
  const Amt h2o = c.A(F_COLH2O), co2 = c.A(F_COLCO2);
  float adjcoln2o = adj_n2o(c);
  if (lower) {
    Spec s = spec(c, h2o, rat(c, 0, jp), co2, 8.0f, 9), s1 = spec(c, h2o, rat(c, 0, jp + 1), co2, 8.0f, 9);
    Spec sm = spec(c, h2o, ratio(c, 1, 2, 3), co2, 8.0f, 9);
    Spec sp = spec(c, h2o, ratio(c, 1, 2, 9), co2, 8.0f, 9);
    binary_lower_terms(t, c, s, s1, BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_et_terms(t, c, adjcoln2o, BT.ma0, 9, NGB, sm.j, sm.f);
    return {BT.fa + (sp.j - 1) * NGB, sp.f};
  }
  Spec s = spec(c, h2o, rat(c, 0, jp), co2, 4.0f, 5), s1 = spec(c, h2o, rat(c, 0, jp + 1), co2, 4.0f, 5);
  Spec sm = spec(c, h2o, ratio(c, 1, 2, 13), co2, 4.0f, 5);
  binary_upper_terms(t, c, s, s1, BT.kb, NGB);
  for_terms(t, c, BT.fo, NGB);
  minor_et_terms(t, c, adjcoln2o, BT.mb0, 5, NGB, sm.j, sm.f);
  return {BT.fb + (clampi(sm.j, 1, 4) - 1) * NGB, sm.f};  // planck ratio equals the minor one here
}

// band 4 (taumol.f90:795-1054)
template <>
__device__ FracRec prologue<4>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 4;
  int jp = clampi(c.I(I_JP), 1, 58);
  if (lower) {
    const Amt h2o = c.A(F_COLH2O), co2 = c.A(F_COLCO2);
    Spec s = spec(c, h2o, rat(c, 0, jp), co2, 8.0f, 9), s1 = spec(c, h2o, rat(c, 0, jp + 1), co2, 8.0f, 9);
    Spec sp = spec(c, h2o, ratio(c, 1, 2, 11), co2, 8.0f, 9);
    binary_lower_terms(t, c, s, s1, BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    return {BT.fa + (sp.j - 1) * NGB, sp.f};
  }
  const Amt o3 = c.A(F_COLO3), co2 = c.A(F_COLCO2);
  Spec s = spec(c, o3, rat(c, 5, jp), co2, 4.0f, 5), s1 = spec(c, o3, rat(c, 5, jp + 1), co2, 4.0f, 5);
  Spec sp = spec(c, o3, ratio(c, 3, 2, 13), co2, 4.0f, 5);
  binary_upper_terms(t, c, s, s1, BT.kb, NGB);
  return {BT.fb + (clampi(sp.j, 1, 4) - 1) * NGB, sp.f};
}

// band 5 (taumol.f90:1057-1332)
template <>
__device__ FracRec prologue<5>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 5;
  int jp = clampi(c.I(I_JP), 1, 58);
  if (lower) {
    const Amt h2o = c.A(F_COLH2O), co2 = c.A(F_COLCO2);
    Spec s = spec(c, h2o, rat(c, 0, jp), co2, 8.0f, 9), s1 = spec(c, h2o, rat(c, 0, jp + 1), co2, 8.0f, 9);
    Spec sm = spec(c, h2o, ratio(c, 1, 2, 7), co2, 8.0f, 9);
    Spec sp = spec(c, h2o, ratio(c, 1, 2, 5), co2, 8.0f, 9);
    binary_lower_terms(t, c, s, s1, BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_et_terms(t, c, c.F(F_COLO3), BT.ma0, 9, NGB, sm.j, sm.f);
    t.add(c.F(F_WX1), BT.x0);
    return {BT.fa + (sp.j - 1) * NGB, sp.f};
  }
  const Amt o3 = c.A(F_COLO3), co2 = c.A(F_COLCO2);
  Spec s = spec(c, o3, rat(c, 5, jp), co2, 4.0f, 5), s1 = spec(c, o3, rat(c, 5, jp + 1), co2, 4.0f, 5);
  Spec sp = spec(c, o3, ratio(c, 3, 2, 43), co2, 4.0f, 5);
  binary_upper_terms(t, c, s, s1, BT.kb, NGB);
  t.add(c.F(F_WX1), BT.x0);
  return {BT.fb + (clampi(sp.j, 1, 4) - 1) * NGB, sp.f};
}

// band 6 (taumol.f90:1335-1421)
template <>
__device__ FracRec prologue<6>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 6;
  if (lower) {
    int jp = clampi(c.I(I_JP), 1, 58);
    float adjcolco2 = adj_col(c.F(F_COLCO2), c.F(F_COLDRY), chi(c, 2, jp + 1), 3.0f, 2.0f, 0.77f);
    single_lower_terms(t, c, c.F(F_COLH2O), BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_t_terms(t, c, adjcolco2, BT.ma0, NGB);
  }
  t.add(c.F(F_WX2), BT.x0);
  t.add(c.F(F_WX3), BT.x1);
  return {BT.fa, 0.0f};
}

// band 7 (taumol.f90:1424-1698)
template <>
__device__ FracRec prologue<7>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 7;
  int jp = clampi(c.I(I_JP), 1, 58);
  if (lower) {
    const Amt h2o = c.A(F_COLH2O), o3 = c.A(F_COLO3);
    Spec s = spec(c, h2o, rat(c, 1, jp), o3, 8.0f, 9), s1 = spec(c, h2o, rat(c, 1, jp + 1), o3, 8.0f, 9);
    Spec sm = spec(c, h2o, ratio(c, 1, 3, 3), o3, 8.0f, 9);  // minor and planck use the same ratio
    float adjcolco2 = adj_col(c.F(F_COLCO2), c.F(F_COLDRY), chi(c, 2, jp + 1), 3.0f, 3.0f, 0.79f);
    binary_lower_terms(t, c, s, s1, BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_et_terms(t, c, adjcolco2, BT.ma0, 9, NGB, sm.j, sm.f);
    return {BT.fa + (sm.j - 1) * NGB, sm.f};
  }
  float ratio = 1.e20f * __fdividef(__fdividef(c.F(F_COLCO2), c.F(F_COLDRY)), chi(c, 2, jp + 1));
  float adjcolco2 = c.F(F_COLCO2);
  if (ratio > 3.0f) adjcolco2 = (2.0f + powf(ratio - 2.0f, 0.79f)) * chi(c, 2, jp + 1) * c.F(F_COLDRY) * 1.e-20f;
  single_upper_terms(t, c, c.F(F_COLO3), BT.kb, 1, NGB);
  minor_t_terms(t, c, adjcolco2, BT.mb0, NGB);
  return {BT.fb, 0.0f};
}

// band 8 (taumol.f90:1701-1824)
template <>
__device__ FracRec prologue<8>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 8;
  int jp = clampi(c.I(I_JP), 1, 58);
  float adjcolco2 = adj_col(c.F(F_COLCO2), c.F(F_COLDRY), chi(c, 2, jp + 1), 3.0f, 2.0f, 0.65f);
  if (lower) {
    single_lower_terms(t, c, c.F(F_COLH2O), BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_t_terms(t, c, adjcolco2, BT.ma0, NGB);
    minor_t_terms(t, c, c.F(F_COLO3), BT.ma2, NGB);
    minor_t_terms(t, c, c.F(F_COLN2O), BT.ma1, NGB);
  } else {
    single_upper_terms(t, c, c.F(F_COLO3), BT.kb, 1, NGB);
    minor_t_terms(t, c, adjcolco2, BT.mb0, NGB);
    minor_t_terms(t, c, c.F(F_COLN2O), BT.mb1, NGB);
  }
  t.add(c.F(F_WX3), BT.x0);
  t.add(c.F(F_WX4), BT.x1);
  return {lower ? BT.fa : BT.fb, 0.0f};
}

// band 9 (taumol.f90:1827-2090)
template <>
__device__ FracRec prologue<9>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 9;
  int jp = clampi(c.I(I_JP), 1, 58);
  float adjcoln2o = adj_n2o(c);
  if (lower) {
    const Amt h2o = c.A(F_COLH2O), ch4 = c.A(F_COLCH4);
    Spec s = spec(c, h2o, rat(c, 3, jp), ch4, 8.0f, 9), s1 = spec(c, h2o, rat(c, 3, jp + 1), ch4, 8.0f, 9);
    Spec sm = spec(c, h2o, ratio(c, 1, 6, 3), ch4, 8.0f, 9);
    Spec sp = spec(c, h2o, ratio(c, 1, 6, 9), ch4, 8.0f, 9);
    binary_lower_terms(t, c, s, s1, BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_et_terms(t, c, adjcoln2o, BT.ma0, 9, NGB, sm.j, sm.f);
    return {BT.fa + (sp.j - 1) * NGB, sp.f};
  }
  single_upper_terms(t, c, c.F(F_COLCH4), BT.kb, 1, NGB);
  minor_t_terms(t, c, adjcoln2o, BT.mb0, NGB);
  return {BT.fb, 0.0f};
}

// band 10 (taumol.f90:2093-2160)
template <>
__device__ FracRec prologue<10>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 10;
  if (lower) {
    single_lower_terms(t, c, c.F(F_COLH2O), BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    return {BT.fa, 0.0f};
  }
  single_upper_terms(t, c, c.F(F_COLH2O), BT.kb, 1, NGB);
  for_terms(t, c, BT.fo, NGB);
  return {BT.fb, 0.0f};
}

// band 11 (taumol.f90:2163-2243)
template <>
__device__ FracRec prologue<11>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 11;
  float scaleo2 = c.F(F_COLO2) * c.F(F_SCALEMINOR);
  if (lower) {
    single_lower_terms(t, c, c.F(F_COLH2O), BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    minor_t_terms(t, c, scaleo2, BT.ma0, NGB);
    return {BT.fa, 0.0f};
  }
  single_upper_terms(t, c, c.F(F_COLH2O), BT.kb, 1, NGB);
  for_terms(t, c, BT.fo, NGB);
  minor_t_terms(t, c, scaleo2, BT.mb0, NGB);
  return {BT.fb, 0.0f};
}

// band 12 (taumol.f90:2246-2449): zero above laytrop
template <>
__device__ FracRec prologue<12>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 12;
  if (!lower) return {c_T.zero_row, 0.0f};
  int jp = clampi(c.I(I_JP), 1, 58);
  const Amt h2o = c.A(F_COLH2O), co2 = c.A(F_COLCO2);
  Spec s = spec(c, h2o, rat(c, 0, jp), co2, 8.0f, 9), s1 = spec(c, h2o, rat(c, 0, jp + 1), co2, 8.0f, 9);
  Spec sp = spec(c, h2o, ratio(c, 1, 2, 10), co2, 8.0f, 9);
  binary_lower_terms(t, c, s, s1, BT.ka, NGB);
  self_terms(t, c, BT.sr, NGB);
  for_terms(t, c, BT.fo, NGB);
  return {BT.fa + (sp.j - 1) * NGB, sp.f};
}

// band 13 (taumol.f90:2452-2712)
template <>
__device__ FracRec prologue<13>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 13;
  if (!lower) {
    minor_t_terms(t, c, c.F(F_COLO3), BT.mb0, NGB);
    return {BT.fb, 0.0f};
  }
  int jp = clampi(c.I(I_JP), 1, 58);
  const Amt h2o = c.A(F_COLH2O), n2o = c.A(F_COLN2O);
  Spec s = spec(c, h2o, rat(c, 2, jp), n2o, 8.0f, 9), s1 = spec(c, h2o, rat(c, 2, jp + 1), n2o, 8.0f, 9);
  Spec sm = spec(c, h2o, ratio(c, 1, 4, 1), n2o, 8.0f, 9);
  Spec sm3 = spec(c, h2o, ratio(c, 1, 4, 3), n2o, 8.0f, 9);
  Spec sp = spec(c, h2o, ratio(c, 1, 4, 5), n2o, 8.0f, 9);
  // CO2 adjustment against the fixed 3.55e-4 reference (taumol.f90:2532-2540)
  float co2 = c.F(F_COLCO2), coldry = c.F(F_COLDRY);
  float ratio = 1.e20f * __fdividef(__fdividef(co2, coldry), 3.55e-4f);
  float adjcolco2 = co2;
  if (ratio > 3.0f) adjcolco2 = (2.0f + powf(ratio - 2.0f, 0.68f)) * 3.55e-4f * coldry * 1.e-20f;
  binary_lower_terms(t, c, s, s1, BT.ka, NGB);
  self_terms(t, c, BT.sr, NGB);
  for_terms(t, c, BT.fo, NGB);
  minor_et_terms(t, c, adjcolco2, BT.ma0, 9, NGB, sm.j, sm.f);
  minor_et_terms(t, c, c.F(F_COLCO), BT.ma1, 9, NGB, sm3.j, sm3.f);
  return {BT.fa + (sp.j - 1) * NGB, sp.f};
}

// band 14 (taumol.f90:2715-2776)
template <>
__device__ FracRec prologue<14>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 14;
  if (lower) {
    single_lower_terms(t, c, c.F(F_COLCO2), BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    return {BT.fa, 0.0f};
  }
  single_upper_terms(t, c, c.F(F_COLCO2), BT.kb, 1, NGB);
  return {BT.fb, 0.0f};
}

// band 15 (taumol.f90:2779-3004): zero above laytrop
template <>
__device__ FracRec prologue<15>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 15;
  if (!lower) return {c_T.zero_row, 0.0f};
  int jp = clampi(c.I(I_JP), 1, 58);
  const Amt n2o = c.A(F_COLN2O), co2 = c.A(F_COLCO2);
  Spec s = spec(c, n2o, rat(c, 4, jp), co2, 8.0f, 9), s1 = spec(c, n2o, rat(c, 4, jp + 1), co2, 8.0f, 9);
  Spec sm = spec(c, n2o, ratio(c, 4, 2, 1), co2, 8.0f, 9);  // minor and planck share the ratio
  binary_lower_terms(t, c, s, s1, BT.ka, NGB);
  self_terms(t, c, BT.sr, NGB);
  for_terms(t, c, BT.fo, NGB);
  minor_et_terms(t, c, c.F(F_COLBRD) * c.F(F_SCALEMINOR), BT.ma0, 9, NGB, sm.j, sm.f);
  return {BT.fa + (sm.j - 1) * NGB, sm.f};
}

// band 16 (taumol.f90:3007-3216); above laytrop nspb(16) = 0 pins ind0 = ind1 = 1
template <>
__device__ FracRec prologue<16>(const Cell& c, bool lower, Terms& t) {
  constexpr int b = 16;
  if (lower) {
    int jp = clampi(c.I(I_JP), 1, 58);
    const Amt h2o = c.A(F_COLH2O), ch4 = c.A(F_COLCH4);
    Spec s = spec(c, h2o, rat(c, 3, jp), ch4, 8.0f, 9), s1 = spec(c, h2o, rat(c, 3, jp + 1), ch4, 8.0f, 9);
    Spec sp = spec(c, h2o, ratio(c, 1, 6, 6), ch4, 8.0f, 9);
    binary_lower_terms(t, c, s, s1, BT.ka, NGB);
    self_terms(t, c, BT.sr, NGB);
    for_terms(t, c, BT.fo, NGB);
    return {BT.fa + (sp.j - 1) * NGB, sp.f};
  }
  float k = c.F(F_COLCH4);
  t.add(k * (c.F(F_FAC00) + c.F(F_FAC01)), BT.kb);
  t.add(k * (c.F(F_FAC10) + c.F(F_FAC11)), BT.kb + NGB);
  return {BT.fb, 0.0f};
}

#undef BT
#undef NGB

// band-4 / band-7 upper-atmosphere g-point factors (default-real literals in
// the reference, taumol.f90:1044-1050 and 1687-1692)
__constant__ float c_gscale4[14] = {1, 1, 1, 1, 1, 1, 1, 0.92f, 0.88f, 1.07f, 1.1f, 0.99f, 0.88f, 0.943f};
__constant__ float c_gscale7[12] = {1, 1, 1, 1, 1, 0.92f, 0.88f, 1.07f, 1.1f, 0.99f, 0.855f, 1};
__device__ __forceinline__ float gscale(int b, int gi) { return b == 4 ? c_gscale4[gi] : c_gscale7[gi]; }

}  // namespace gb
