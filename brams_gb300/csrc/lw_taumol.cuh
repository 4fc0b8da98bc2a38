// Gas optics of one (layer, g-point) cell for each of the 16 longwave bands.
//
// Device restatement of taugb1..taugb16 (rrtmg_lw_taumol.f90:299-3216) in
// single precision.  Where the reference loops over layers and then
// g-points, the GPU evaluates one cell per thread: lanes of a warp hold
// consecutive g-points of one band at one or a few layers, so every table
// read of a warp touches one or two contiguous runs of the g-fastest tables.
// The per-layer part of each band (binary-species parameter, stencil
// weights, minor-gas amounts) is recomputed per cell; it is cheaper than the
// shared-memory traffic of storing it.
//
// Integer table coordinates are clamped to their valid ranges.  For valid
// inputs the clamps are inactive; for invalid inputs they keep every read
// inside the tables (the reference would read out of bounds there).
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

struct Cell {
  const float* f;  // [NF][nl] shared memory
  const int* iv;   // [NI][nl] shared memory
  int nl, lay;
  __device__ __forceinline__ float F(int k) const { return f[k * nl + lay]; }
  __device__ __forceinline__ int I(int k) const { return iv[k * nl + lay]; }
};

__device__ __forceinline__ float ld(const float* __restrict__ p) { return __ldg(p); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// tauself / taufor (e.g. taumol.f90:344-347)
__device__ __forceinline__ float t_self(const Cell& c, const float* __restrict__ T, int off, int ng, int gi) {
  int inds = clampi(c.I(I_INDSELF), 1, 9);
  const float* s = T + off + gi;
  float a = ld(s + (inds - 1) * ng), b = ld(s + inds * ng);
  return c.F(F_SELFFAC) * (a + c.F(F_SELFFRAC) * (b - a));
}
__device__ __forceinline__ float t_for(const Cell& c, const float* __restrict__ T, int off, int ng, int gi) {
  int indf = clampi(c.I(I_INDFOR), 1, 3);
  const float* s = T + off + gi;
  float a = ld(s + (indf - 1) * ng), b = ld(s + indf * ng);
  return c.F(F_FORFAC) * (a + c.F(F_FORFRAC) * (b - a));
}
// temperature-interpolated minor absorber k(indm, g), table [19][ng]
__device__ __forceinline__ float m_t(const Cell& c, const float* __restrict__ T, int off, int ng, int gi) {
  int indm = clampi(c.I(I_INDMINOR), 1, 18);
  const float* s = T + off + gi;
  float a = ld(s + (indm - 1) * ng), b = ld(s + indm * ng);
  return a + c.F(F_MINORFRAC) * (b - a);
}
// eta- and temperature-interpolated minor absorber k(jm, indm, g), table [19][neta][ng]
__device__ __forceinline__ float m_et(const Cell& c, const float* __restrict__ T, int off, int neta, int ng,
                                      int gi, int jm, float fm) {
  int indm = clampi(c.I(I_INDMINOR), 1, 18);
  jm = clampi(jm, 1, neta - 1);
  const float* s = T + off + gi;
  auto K = [&](int a, int t) { return ld(s + ((t - 1) * neta + (a - 1)) * ng); };
  float m1 = K(jm, indm) + fm * (K(jm + 1, indm) - K(jm, indm));
  float m2 = K(jm, indm + 1) + fm * (K(jm + 1, indm + 1) - K(jm, indm + 1));
  return m1 + c.F(F_MINORFRAC) * (m2 - m1);
}

struct Spec {
  float comb, parm, f;
  int j;
};
// speccomb/specparm/specmult/js/fs (e.g. taumol.f90:517-522); oneminus = 1 - 1e-6
__device__ __forceinline__ Spec spec(float a, float rat, float b, float scale, int jmax) {
  Spec s;
  s.comb = a + rat * b;
  s.parm = a / s.comb;
  if (!(s.parm < 0.999999f)) s.parm = 0.999999f;
  if (!(s.parm >= 0.0f)) s.parm = 0.0f;  // negative amounts: outside the tables' domain
  float mult = scale * s.parm;
  int ji = (int)mult;
  s.j = clampi(1 + ji, 1, jmax);
  s.f = mult - (float)ji;
  return s;
}

// Lower-atmosphere binary major absorber with the three-point stencil in eta
// (taumol.f90:582-700).  A points at absa(1, g) (row stride ng), ind0 1-based.
__device__ __forceinline__ float major9(float comb, float parm, float fs, int ind0, float fa, float fb,
                                        const float* __restrict__ A, int ng) {
  auto R = [&](int i) { return ld(A + (i - 1) * ng); };
  if (parm < 0.125f) {
    float p = fs - 1.0f, p4 = (p * p) * (p * p);
    float k0 = p4, k1 = 1.0f - p - 2.0f * p4, k2 = p + p4;
    return comb * (k0 * fa * R(ind0) + k1 * fa * R(ind0 + 1) + k2 * fa * R(ind0 + 2) +
                   k0 * fb * R(ind0 + 9) + k1 * fb * R(ind0 + 10) + k2 * fb * R(ind0 + 11));
  } else if (parm > 0.875f) {
    float p = -fs, p4 = (p * p) * (p * p);
    float k0 = p4, k1 = 1.0f - p - 2.0f * p4, k2 = p + p4;
    return comb * (k2 * fa * R(ind0 - 1) + k1 * fa * R(ind0) + k0 * fa * R(ind0 + 1) +
                   k2 * fb * R(ind0 + 8) + k1 * fb * R(ind0 + 9) + k0 * fb * R(ind0 + 10));
  }
  return comb * ((1.0f - fs) * fa * R(ind0) + fs * fa * R(ind0 + 1) + (1.0f - fs) * fb * R(ind0 + 9) +
                 fs * fb * R(ind0 + 10));
}

// js clamp so that the stencil of major9 stays inside the 9-wide eta rows
__device__ __forceinline__ int js_lower(const Spec& s) {
  if (s.parm < 0.125f) return clampi(s.j, 1, 7);
  if (s.parm > 0.875f) return clampi(s.j, 2, 8);
  return clampi(s.j, 1, 8);
}

__device__ __forceinline__ float single_lower(const Cell& c, float key, const float* __restrict__ T, int ka,
                                              int ng, int gi) {
  int jp = clampi(c.I(I_JP), 1, 12), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int ind0 = ((jp - 1) * 5 + (jt - 1)) + 1, ind1 = (jp * 5 + (jt1 - 1)) + 1;
  const float* A = T + ka + gi;
  return key * (c.F(F_FAC00) * ld(A + (ind0 - 1) * ng) + c.F(F_FAC10) * ld(A + ind0 * ng) +
                c.F(F_FAC01) * ld(A + (ind1 - 1) * ng) + c.F(F_FAC11) * ld(A + ind1 * ng));
}
__device__ __forceinline__ float single_upper(const Cell& c, float key, const float* __restrict__ T, int kb,
                                              int nspb, int ng, int gi) {
  int jp = clampi(c.I(I_JP), 13, 58), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int ind0 = ((jp - 13) * 5 + (jt - 1)) * nspb + 1, ind1 = ((jp - 12) * 5 + (jt1 - 1)) * nspb + 1;
  const float* B = T + kb + gi;
  return key * (c.F(F_FAC00) * ld(B + (ind0 - 1) * ng) + c.F(F_FAC10) * ld(B + ind0 * ng) +
                c.F(F_FAC01) * ld(B + (ind1 - 1) * ng) + c.F(F_FAC11) * ld(B + ind1 * ng));
}
// lower binary: both stencils (taumol.f90:653-700 pattern)
__device__ __forceinline__ float binary_lower(const Cell& c, const Spec& s, const Spec& s1, const float* __restrict__ T,
                                              int ka, int ng, int gi) {
  int jp = clampi(c.I(I_JP), 1, 12), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int ind0 = ((jp - 1) * 5 + (jt - 1)) * 9 + js_lower(s);
  int ind1 = (jp * 5 + (jt1 - 1)) * 9 + js_lower(s1);
  const float* A = T + ka + gi;
  return major9(s.comb, s.parm, s.f, ind0, c.F(F_FAC00), c.F(F_FAC10), A, ng) +
         major9(s1.comb, s1.parm, s1.f, ind1, c.F(F_FAC01), c.F(F_FAC11), A, ng);
}
// upper binary with nspb = 5, two-point in eta (taumol.f90:775-789)
__device__ __forceinline__ float binary_upper(const Cell& c, const Spec& s, const Spec& s1, const float* __restrict__ T,
                                              int kb, int ng, int gi) {
  int jp = clampi(c.I(I_JP), 13, 58), jt = c.I(I_JT), jt1 = c.I(I_JT1);
  int js = clampi(s.j, 1, 4), js1 = clampi(s1.j, 1, 4);
  int ind0 = ((jp - 13) * 5 + (jt - 1)) * 5 + js, ind1 = ((jp - 12) * 5 + (jt1 - 1)) * 5 + js1;
  const float* B = T + kb + gi;
  auto R = [&](int i) { return ld(B + (i - 1) * ng); };
  float fa = c.F(F_FAC00), fb = c.F(F_FAC10), fc = c.F(F_FAC01), fd = c.F(F_FAC11);
  return s.comb * ((1.0f - s.f) * fa * R(ind0) + s.f * fa * R(ind0 + 1) + (1.0f - s.f) * fb * R(ind0 + 5) +
                   s.f * fb * R(ind0 + 6)) +
         s1.comb * ((1.0f - s1.f) * fc * R(ind1) + s1.f * fc * R(ind1 + 1) + (1.0f - s1.f) * fd * R(ind1 + 5) +
                    s1.f * fd * R(ind1 + 6));
}

// Planck-fraction record of a (layer, band): frac(g) = T[off+g] + fpl*(T[off+ng+g]-T[off+g])
struct FracRec {
  int off;
  float fpl;
};

__device__ __forceinline__ float chi(int m, int jp) { return c_T.chi[m - 1][jp - 1]; }
__device__ __forceinline__ float rat(int k, int jp) { return c_T.rat[k][jp - 1]; }

// CO2 / N2O column adjustment of bands 3, 6, 7, 8, 9 (e.g. taumol.f90:545-552)
__device__ __forceinline__ float adj_col(float col, float coldry, float chiref, float thresh, float base,
                                          float expo) {
  float ratio = 1.e20f * (col / coldry) / chiref;
  if (ratio > thresh) {
    float adjfac = base + powf(ratio - base, expo);
    return adjfac * chiref * coldry * 1.e-20f;
  }
  return col;
}

// -------------------------------------------------------------------------
// One cell of band b (1-based).  gi is the g-point index inside the band.
// Returns taug; writes the band's Planck-fraction record when rec != nullptr.
template <int b>
__device__ float tau_band(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec);

#define BT c_T.band[b - 1]

// band 1 (taumol.f90:299-399)
template <>
__device__ float tau_band<1>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 1;
  const int ng = BT.ng;
  float scalen2 = c.F(F_COLBRD) * c.F(F_SCALEMINORN2);
  float pp = c.F(F_PAVEL);
  if (lower) {
    if (rec) *rec = {BT.fa, 0.0f};
    float corradj = pp < 250.0f ? 1.0f - 0.15f * (250.0f - pp) / 154.4f : 1.0f;
    float taun2 = scalen2 * m_t(c, T, BT.ma0, ng, gi);
    return corradj * (single_lower(c, c.F(F_COLH2O), T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) +
                      t_for(c, T, BT.fo, ng, gi) + taun2);
  }
  if (rec) *rec = {BT.fb, 0.0f};
  float corradj = 1.0f - 0.15f * (pp / 95.6f);
  float taun2 = scalen2 * m_t(c, T, BT.mb0, ng, gi);
  return corradj * (single_upper(c, c.F(F_COLH2O), T, BT.kb, 1, ng, gi) + t_for(c, T, BT.fo, ng, gi) + taun2);
}

// band 2 (taumol.f90:402-474)
template <>
__device__ float tau_band<2>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 2;
  const int ng = BT.ng;
  if (lower) {
    if (rec) *rec = {BT.fa, 0.0f};
    float corradj = 1.0f - 0.05f * (c.F(F_PAVEL) - 100.0f) / 900.0f;
    return corradj * (single_lower(c, c.F(F_COLH2O), T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) +
                      t_for(c, T, BT.fo, ng, gi));
  }
  if (rec) *rec = {BT.fb, 0.0f};
  return single_upper(c, c.F(F_COLH2O), T, BT.kb, 1, ng, gi) + t_for(c, T, BT.fo, ng, gi);
}

// adjusted N2O column of bands 3 and 9 (taumol.f90:545-552, 1896-1903)
__device__ __forceinline__ float adj_n2o(const Cell& c) {
  return adj_col(c.F(F_COLN2O), c.F(F_COLDRY), chi(4, clampi(c.I(I_JP), 1, 58) + 1), 1.5f, 0.5f, 0.65f);
}

// band 3 (taumol.f90:477-792)
template <>
__device__ float tau_band<3>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 3;
  const int ng = BT.ng;
  int jp = clampi(c.I(I_JP), 1, 58);
  float h2o = c.F(F_COLH2O), co2 = c.F(F_COLCO2);
  float adjcoln2o = adj_n2o(c);
  if (lower) {
    Spec s = spec(h2o, rat(0, jp), co2, 8.0f, 9), s1 = spec(h2o, rat(0, jp + 1), co2, 8.0f, 9);
    Spec sm = spec(h2o, chi(1, 3) / chi(2, 3), co2, 8.0f, 9);
    if (rec) {
      Spec sp = spec(h2o, chi(1, 9) / chi(2, 9), co2, 8.0f, 9);
      *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
    }
    return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
           adjcoln2o * m_et(c, T, BT.ma0, 9, ng, gi, sm.j, sm.f);
  }
  Spec s = spec(h2o, rat(0, jp), co2, 4.0f, 5), s1 = spec(h2o, rat(0, jp + 1), co2, 4.0f, 5);
  Spec sm = spec(h2o, chi(1, 13) / chi(2, 13), co2, 4.0f, 5);
  if (rec) {
    Spec sp = spec(h2o, chi(1, 13) / chi(2, 13), co2, 4.0f, 5);
    *rec = {BT.fb + (clampi(sp.j, 1, 4) - 1) * ng, sp.f};
  }
  return binary_upper(c, s, s1, T, BT.kb, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
         adjcoln2o * m_et(c, T, BT.mb0, 5, ng, gi, sm.j, sm.f);
}

// band 4 (taumol.f90:795-1054)
template <>
__device__ float tau_band<4>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 4;
  const int ng = BT.ng;
  int jp = clampi(c.I(I_JP), 1, 58);
  if (lower) {
    float h2o = c.F(F_COLH2O), co2 = c.F(F_COLCO2);
    Spec s = spec(h2o, rat(0, jp), co2, 8.0f, 9), s1 = spec(h2o, rat(0, jp + 1), co2, 8.0f, 9);
    if (rec) {
      Spec sp = spec(h2o, chi(1, 11) / chi(2, 11), co2, 8.0f, 9);
      *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
    }
    return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi);
  }
  float o3 = c.F(F_COLO3), co2 = c.F(F_COLCO2);
  Spec s = spec(o3, rat(5, jp), co2, 4.0f, 5), s1 = spec(o3, rat(5, jp + 1), co2, 4.0f, 5);
  if (rec) {
    Spec sp = spec(o3, chi(3, 13) / chi(2, 13), co2, 4.0f, 5);
    *rec = {BT.fb + (clampi(sp.j, 1, 4) - 1) * ng, sp.f};
  }
  float t = binary_upper(c, s, s1, T, BT.kb, ng, gi);
  // g-point scale factors (taumol.f90:1044-1050); gi is 0-based
  switch (gi) {
    case 7: t *= 0.92f; break;
    case 8: t *= 0.88f; break;
    case 9: t *= 1.07f; break;
    case 10: t *= 1.1f; break;
    case 11: t *= 0.99f; break;
    case 12: t *= 0.88f; break;
    case 13: t *= 0.943f; break;
    default: break;
  }
  return t;
}

// band 5 (taumol.f90:1057-1332)
template <>
__device__ float tau_band<5>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 5;
  const int ng = BT.ng;
  int jp = clampi(c.I(I_JP), 1, 58);
  float ccl4 = c.F(F_WX1) * ld(T + BT.x0 + gi);
  if (lower) {
    float h2o = c.F(F_COLH2O), co2 = c.F(F_COLCO2);
    Spec s = spec(h2o, rat(0, jp), co2, 8.0f, 9), s1 = spec(h2o, rat(0, jp + 1), co2, 8.0f, 9);
    Spec sm = spec(h2o, chi(1, 7) / chi(2, 7), co2, 8.0f, 9);
    if (rec) {
      Spec sp = spec(h2o, chi(1, 5) / chi(2, 5), co2, 8.0f, 9);
      *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
    }
    return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
           m_et(c, T, BT.ma0, 9, ng, gi, sm.j, sm.f) * c.F(F_COLO3) + ccl4;
  }
  float o3 = c.F(F_COLO3), co2 = c.F(F_COLCO2);
  Spec s = spec(o3, rat(5, jp), co2, 4.0f, 5), s1 = spec(o3, rat(5, jp + 1), co2, 4.0f, 5);
  if (rec) {
    Spec sp = spec(o3, chi(3, 43) / chi(2, 43), co2, 4.0f, 5);
    *rec = {BT.fb + (clampi(sp.j, 1, 4) - 1) * ng, sp.f};
  }
  return binary_upper(c, s, s1, T, BT.kb, ng, gi) + ccl4;
}

// band 6 (taumol.f90:1335-1421)
template <>
__device__ float tau_band<6>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 6;
  const int ng = BT.ng;
  if (rec) *rec = {BT.fa, 0.0f};
  float cfc = c.F(F_WX2) * ld(T + BT.x0 + gi) + c.F(F_WX3) * ld(T + BT.x1 + gi);
  if (lower) {
    int jp = clampi(c.I(I_JP), 1, 58);
    float adjcolco2 = adj_col(c.F(F_COLCO2), c.F(F_COLDRY), chi(2, jp + 1), 3.0f, 2.0f, 0.77f);
    return single_lower(c, c.F(F_COLH2O), T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) +
           t_for(c, T, BT.fo, ng, gi) + adjcolco2 * m_t(c, T, BT.ma0, ng, gi) + cfc;
  }
  return cfc;
}

// band 7 (taumol.f90:1424-1698)
template <>
__device__ float tau_band<7>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 7;
  const int ng = BT.ng;
  int jp = clampi(c.I(I_JP), 1, 58);
  if (lower) {
    float h2o = c.F(F_COLH2O), o3 = c.F(F_COLO3);
    Spec s = spec(h2o, rat(1, jp), o3, 8.0f, 9), s1 = spec(h2o, rat(1, jp + 1), o3, 8.0f, 9);
    float r3 = chi(1, 3) / chi(3, 3);
    Spec sm = spec(h2o, r3, o3, 8.0f, 9);
    if (rec) {
      Spec sp = spec(h2o, r3, o3, 8.0f, 9);
      *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
    }
    // lower threshold/base 3.0 (taumol.f90:1503-1509)
    float adjcolco2 = adj_col(c.F(F_COLCO2), c.F(F_COLDRY), chi(2, jp + 1), 3.0f, 3.0f, 0.79f);
    return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
           adjcolco2 * m_et(c, T, BT.ma0, 9, ng, gi, sm.j, sm.f);
  }
  if (rec) *rec = {BT.fb, 0.0f};
  // upper: ratio threshold 3.0, base 2.0 (taumol.f90:1662-1668)
  float ratio = 1.e20f * (c.F(F_COLCO2) / c.F(F_COLDRY)) / chi(2, jp + 1);
  float adjcolco2 = c.F(F_COLCO2);
  if (ratio > 3.0f) adjcolco2 = (2.0f + powf(ratio - 2.0f, 0.79f)) * chi(2, jp + 1) * c.F(F_COLDRY) * 1.e-20f;
  float t = single_upper(c, c.F(F_COLO3), T, BT.kb, 1, ng, gi) + adjcolco2 * m_t(c, T, BT.mb0, ng, gi);
  switch (gi) {  // taumol.f90:1687-1692
    case 5: t *= 0.92f; break;
    case 6: t *= 0.88f; break;
    case 7: t *= 1.07f; break;
    case 8: t *= 1.1f; break;
    case 9: t *= 0.99f; break;
    case 10: t *= 0.855f; break;
    default: break;
  }
  return t;
}

// band 8 (taumol.f90:1701-1824)
template <>
__device__ float tau_band<8>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 8;
  const int ng = BT.ng;
  int jp = clampi(c.I(I_JP), 1, 58);
  float adjcolco2 = adj_col(c.F(F_COLCO2), c.F(F_COLDRY), chi(2, jp + 1), 3.0f, 2.0f, 0.65f);
  float cfc = c.F(F_WX3) * ld(T + BT.x0 + gi) + c.F(F_WX4) * ld(T + BT.x1 + gi);
  if (lower) {
    if (rec) *rec = {BT.fa, 0.0f};
    return single_lower(c, c.F(F_COLH2O), T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) +
           t_for(c, T, BT.fo, ng, gi) + adjcolco2 * m_t(c, T, BT.ma0, ng, gi) +
           c.F(F_COLO3) * m_t(c, T, BT.ma2, ng, gi) + c.F(F_COLN2O) * m_t(c, T, BT.ma1, ng, gi) + cfc;
  }
  if (rec) *rec = {BT.fb, 0.0f};
  return single_upper(c, c.F(F_COLO3), T, BT.kb, 1, ng, gi) + adjcolco2 * m_t(c, T, BT.mb0, ng, gi) +
         c.F(F_COLN2O) * m_t(c, T, BT.mb1, ng, gi) + cfc;
}

// band 9 (taumol.f90:1827-2090)
template <>
__device__ float tau_band<9>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 9;
  const int ng = BT.ng;
  int jp = clampi(c.I(I_JP), 1, 58);
  float adjcoln2o = adj_n2o(c);
  if (lower) {
    float h2o = c.F(F_COLH2O), ch4 = c.F(F_COLCH4);
    Spec s = spec(h2o, rat(3, jp), ch4, 8.0f, 9), s1 = spec(h2o, rat(3, jp + 1), ch4, 8.0f, 9);
    Spec sm = spec(h2o, chi(1, 3) / chi(6, 3), ch4, 8.0f, 9);
    if (rec) {
      Spec sp = spec(h2o, chi(1, 9) / chi(6, 9), ch4, 8.0f, 9);
      *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
    }
    return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
           adjcoln2o * m_et(c, T, BT.ma0, 9, ng, gi, sm.j, sm.f);
  }
  if (rec) *rec = {BT.fb, 0.0f};
  return single_upper(c, c.F(F_COLCH4), T, BT.kb, 1, ng, gi) + adjcoln2o * m_t(c, T, BT.mb0, ng, gi);
}

// band 10 (taumol.f90:2093-2160)
template <>
__device__ float tau_band<10>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 10;
  const int ng = BT.ng;
  if (lower) {
    if (rec) *rec = {BT.fa, 0.0f};
    return single_lower(c, c.F(F_COLH2O), T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) +
           t_for(c, T, BT.fo, ng, gi);
  }
  if (rec) *rec = {BT.fb, 0.0f};
  return single_upper(c, c.F(F_COLH2O), T, BT.kb, 1, ng, gi) + t_for(c, T, BT.fo, ng, gi);
}

// band 11 (taumol.f90:2163-2243)
template <>
__device__ float tau_band<11>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 11;
  const int ng = BT.ng;
  float scaleo2 = c.F(F_COLO2) * c.F(F_SCALEMINOR);
  if (lower) {
    if (rec) *rec = {BT.fa, 0.0f};
    return single_lower(c, c.F(F_COLH2O), T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) +
           t_for(c, T, BT.fo, ng, gi) + scaleo2 * m_t(c, T, BT.ma0, ng, gi);
  }
  if (rec) *rec = {BT.fb, 0.0f};
  return single_upper(c, c.F(F_COLH2O), T, BT.kb, 1, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
         scaleo2 * m_t(c, T, BT.mb0, ng, gi);
}

// band 12 (taumol.f90:2246-2449)
template <>
__device__ float tau_band<12>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 12;
  const int ng = BT.ng;
  if (!lower) {
    if (rec) *rec = {c_T.zero_row, 0.0f};
    return 0.0f;
  }
  int jp = clampi(c.I(I_JP), 1, 58);
  float h2o = c.F(F_COLH2O), co2 = c.F(F_COLCO2);
  Spec s = spec(h2o, rat(0, jp), co2, 8.0f, 9), s1 = spec(h2o, rat(0, jp + 1), co2, 8.0f, 9);
  if (rec) {
    Spec sp = spec(h2o, chi(1, 10) / chi(2, 10), co2, 8.0f, 9);
    *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
  }
  return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi);
}

// band 13 (taumol.f90:2452-2712)
template <>
__device__ float tau_band<13>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 13;
  const int ng = BT.ng;
  if (!lower) {
    if (rec) *rec = {BT.fb, 0.0f};
    return c.F(F_COLO3) * m_t(c, T, BT.mb0, ng, gi);
  }
  int jp = clampi(c.I(I_JP), 1, 58);
  float h2o = c.F(F_COLH2O), n2o = c.F(F_COLN2O);
  Spec s = spec(h2o, rat(2, jp), n2o, 8.0f, 9), s1 = spec(h2o, rat(2, jp + 1), n2o, 8.0f, 9);
  Spec sm = spec(h2o, chi(1, 1) / chi(4, 1), n2o, 8.0f, 9);
  Spec sm3 = spec(h2o, chi(1, 3) / chi(4, 3), n2o, 8.0f, 9);
  if (rec) {
    Spec sp = spec(h2o, chi(1, 5) / chi(4, 5), n2o, 8.0f, 9);
    *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
  }
  // fixed reference CO2 of 3.55e-4 (taumol.f90:2532-2540)
  float co2 = c.F(F_COLCO2), coldry = c.F(F_COLDRY);
  float ratio = 1.e20f * (co2 / coldry) / 3.55e-4f;
  float adjcolco2 = co2;
  if (ratio > 3.0f) adjcolco2 = (2.0f + powf(ratio - 2.0f, 0.68f)) * 3.55e-4f * coldry * 1.e-20f;
  return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
         adjcolco2 * m_et(c, T, BT.ma0, 9, ng, gi, sm.j, sm.f) + c.F(F_COLCO) * m_et(c, T, BT.ma1, 9, ng, gi, sm3.j, sm3.f);
}

// band 14 (taumol.f90:2715-2776)
template <>
__device__ float tau_band<14>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 14;
  const int ng = BT.ng;
  if (lower) {
    if (rec) *rec = {BT.fa, 0.0f};
    return single_lower(c, c.F(F_COLCO2), T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) +
           t_for(c, T, BT.fo, ng, gi);
  }
  if (rec) *rec = {BT.fb, 0.0f};
  return single_upper(c, c.F(F_COLCO2), T, BT.kb, 1, ng, gi);
}

// band 15 (taumol.f90:2779-3004)
template <>
__device__ float tau_band<15>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 15;
  const int ng = BT.ng;
  if (!lower) {
    if (rec) *rec = {c_T.zero_row, 0.0f};
    return 0.0f;
  }
  int jp = clampi(c.I(I_JP), 1, 58);
  float n2o = c.F(F_COLN2O), co2 = c.F(F_COLCO2);
  Spec s = spec(n2o, rat(4, jp), co2, 8.0f, 9), s1 = spec(n2o, rat(4, jp + 1), co2, 8.0f, 9);
  float r = chi(4, 1) / chi(2, 1);
  Spec sm = spec(n2o, r, co2, 8.0f, 9);
  if (rec) {
    Spec sp = spec(n2o, r, co2, 8.0f, 9);
    *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
  }
  float scalen2 = c.F(F_COLBRD) * c.F(F_SCALEMINOR);
  return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi) +
         scalen2 * m_et(c, T, BT.ma0, 9, ng, gi, sm.j, sm.f);
}

// band 16 (taumol.f90:3007-3216); above laytrop nspb(16) = 0 pins ind0 = ind1 = 1
template <>
__device__ float tau_band<16>(const Cell& c, bool lower, int gi, const float* __restrict__ T, FracRec* rec) {
  constexpr int b = 16;
  const int ng = BT.ng;
  if (lower) {
    int jp = clampi(c.I(I_JP), 1, 58);
    float h2o = c.F(F_COLH2O), ch4 = c.F(F_COLCH4);
    Spec s = spec(h2o, rat(3, jp), ch4, 8.0f, 9), s1 = spec(h2o, rat(3, jp + 1), ch4, 8.0f, 9);
    if (rec) {
      Spec sp = spec(h2o, chi(1, 6) / chi(6, 6), ch4, 8.0f, 9);
      *rec = {BT.fa + (sp.j - 1) * ng, sp.f};
    }
    return binary_lower(c, s, s1, T, BT.ka, ng, gi) + t_self(c, T, BT.sr, ng, gi) + t_for(c, T, BT.fo, ng, gi);
  }
  if (rec) *rec = {BT.fb, 0.0f};
  const float* B = T + BT.kb + gi;
  float t00 = ld(B), t10 = ld(B + ng);
  return c.F(F_COLCH4) * (c.F(F_FAC00) * t00 + c.F(F_FAC10) * t10 + c.F(F_FAC01) * t00 + c.F(F_FAC11) * t10);
}

#undef BT

}  // namespace gb
