// RRTMG_SW column kernel for GB300 (sm_103a), templated on the arithmetic
// type R of the gas optics and the two-stream solution: the shortwave McICA
// path that BRAMS calls right after the longwave one (rtm_driver.f90:1386).
//
// The reference solves one column at a time (rrtmg_sw_rad.f90:460-586):
// inatm_sw, cldprmc_sw, setcoef_sw and spcvmc_sw, which runs taumol_sw and
// then, per g-point, the delta-scaled two-stream layer properties (reftra_sw)
// and the adding method (vrtqdr_sw).  Here a block of 128 threads solves a
// column and persistent blocks walk the columns:
//
//   1. one thread per layer: inatm_sw's column amounts and setcoef_sw's
//      interpolation indices and factors (fp64), into shared memory as R;
//   2. per band, one thread per (layer, g) cell: taumol_sw's gas and
//      Rayleigh optical depths into the block's scratch slot; per band the
//      solar-source layer and each g-point's source (sfluxzen);
//   3. one thread per g-point (112 live): from the model top down, each
//      layer's cloud optics (cldprmc_sw), its clear and total delta-scaled
//      optics, two reftra_sw evaluations and the direct beam, and the
//      downward adding recurrence; the layer and level values go to the slot;
//      then from the surface up the upward adding recurrence and the level
//      flux fractions of the g-point, kept in the slot;
//   4. one thread per (level, flux): the fp64 sum over the g-points in their
//      order of the incoming flux times the flux fraction (the reference's
//      accumulation, spcvmc.f90:470-480), then net fluxes and fp64 heating
//      rates from the level sums.
//
// R = double is the reference's arithmetic: with fp contraction off the
// fluxes match the fp64 restatement at rounding level.  R = float runs the
// gas optics, cloud optics and two-stream solution in fp32 on fp32 tables
// (GB300 issues fp64 at a small fraction of the fp32 rate) and keeps fp64 for
// the layer coefficients, the incoming flux, the flux accumulation over
// g-points and the heating rates.  Decisions the reference takes on its
// double inputs (cloud presence, radius bounds) are taken on the double
// values, so the fp32 path raises the same errors on the same columns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lw_common.h"
#include "sw_solver.h"

namespace gbsw {

constexpr int NG = SW_NGPT;  // 112
constexpr int NB = 14;
constexpr int NT = 128;      // threads per column block
constexpr int NVL = 16;      // scratch values per (level, g): 10 layer values and 6 level values

// offsets (in elements) of a band's reduced tables in the table blob (-1: absent)
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
  int coaliq1, coaice2, coaice3;  // 1 - ssaliq1, 1 - ssaice2, 1 - ssaice3 (co-albedos, formed in fp64)
  double abari[5], bbari[5], cbari[5], dbari[5], ebari[5], fbari[5];
  double bpade, heatfac, avogad, grav;
  float bpadef;
  int total;
};
// one copy per translation unit (each precision's kernels live in their own unit)
static __constant__ SwTab c_S;

template <typename R>
__device__ __forceinline__ R tb(const R* __restrict__ T, int off) {
  return __ldg(T + off);
}
template <typename R>
__device__ __forceinline__ R bpade();
template <>
__device__ __forceinline__ double bpade<double>() {
  return c_S.bpade;
}
template <>
__device__ __forceinline__ float bpade<float>() {
  return c_S.bpadef;
}

// Decisions the reference takes on a double input x, with xr = (R)x.
// Rounding is monotonic, so a strict float comparison against the rounded
// constant is exact; only a tie with the rounded constant needs the double.
template <typename R>
__device__ __forceinline__ bool ge_in(double x, R xr, double c) {
  if (sizeof(R) == 8) return x >= c;
  const R cr = (R)c;
  if (xr != cr) return xr > cr;
  return x >= c;
}
template <typename R>
__device__ __forceinline__ bool gt_in(double x, R xr, double c) {
  if (sizeof(R) == 8) return x > c;
  const R cr = (R)c;
  if (xr != cr) return xr > cr;
  return x > c;
}
template <typename R>
__device__ __forceinline__ bool outside_in(double x, R xr, double lo, double hi) {
  if (sizeof(R) == 8) return x < lo || x > hi;
  const R l = (R)lo, h = (R)hi;
  if (xr != l && xr != h) return xr < l || xr > h;
  return x < lo || x > hi;
}
// x != 0 on the bits (a double too small for a float is still nonzero)
__device__ __forceinline__ bool nonzero_in(double x) {
  return (__double_as_longlong(x) << 1) != 0;
}

// Ampere-style asynchronous global -> shared copies (cp.async): each thread
// stages the next layer's (or level's) values while it computes this one;
// a thread only reads back what it copied itself, so waiting on its own
// copy groups is enough
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
template <typename R>
__device__ __forceinline__ void cp_async_r(void* smem, const R* gmem) {
  if constexpr (sizeof(R) == 4)
    cp_async4(smem, gmem);
  else
    cp_async8(smem, gmem);
}

// double -> float on the integer pipes (the fp64 pipe is GB300's narrowest):
// round to nearest (ties away from zero) for results in the normal float
// range, +-0 for double zeros and subnormals, the hardware conversion for the
// rest (float subnormals, overflow, inf, NaN)
__device__ __forceinline__ float d2f_fast(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 254u) {
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    return __uint_as_float(((hi & 0x80000000u) | ((e - 896u) << 23)) + m + ((lo >> 28) & 1u));
  }
  if (e == 0u) return __uint_as_float(hi & 0x80000000u);
  return (float)x;
}
// float -> double (exact) on the integer pipes: normal floats and zeros by
// rebiasing the exponent, subnormals, inf and NaN by the hardware conversion
__device__ __forceinline__ double f2d_fast(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u < 254u) {
    const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  if ((u << 1) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  return (double)x;
}
template <typename R>
__device__ __forceinline__ R to_r(double x) {
  if constexpr (sizeof(R) == 4)
    return d2f_fast(x);
  else
    return x;
}

// exp(-ze) as the reference forms it: Taylor below od_lo, else exp_tbl at
// the quantised index (reftra.f90:150-159, spcvmc.f90:445-456)
template <typename R>
__device__ __forceinline__ R expo(const R* __restrict__ T, R ze) {
  if (ze <= R(0.06)) return R(1.0) - ze + R(0.5) * ze * ze;
  const R tblind = ze / (bpade<R>() + ze);
  const int itind = (int)(R(10000.0) * tblind + R(0.5));
  return tb(T, c_S.exp_tbl + itind);
}

// reftra_sw for one layer (rrtmg_sw_reftra.f90:107-326, kmodts = 2)
template <typename R>
__device__ void reftra(const R* __restrict__ T, bool chk, R zg, R prmuz, R zto1, R zw, R& pref, R& prefd, R& ptra,
                       R& ptrad) {
  if (!chk) {
    pref = R(0.0);
    ptra = R(1.0);
    prefd = R(0.0);
    ptrad = R(1.0);
    return;
  }
  const R eps = R(1.e-08), zwcrit = R(0.9999995);
  const R zg3 = R(3.0) * zg;
  const R zgamma1 = (R(8.0) - zw * (R(5.0) + zg3)) * R(0.25);
  const R zgamma2 = R(3.0) * (zw * (R(1.0) - zg)) * R(0.25);
  const R zgamma3 = (R(2.0) - zg3 * prmuz) * R(0.25);
  const R zgamma4 = R(1.0) - zgamma3;
  R zwo = R(0.0), denom = R(1.0);
  if (zg != R(1.0)) {
    const R q = zg / (R(1.0) - zg);
    denom = (R(1.0) - (R(1.0) - zw) * (q * q));
  }
  if (zw > R(0.0) && denom != R(0.0)) zwo = zw / denom;
  if (zwo >= zwcrit) {
    const R za = zgamma1 * prmuz;
    const R za1 = za - zgamma3;
    const R zgt = zgamma1 * zto1;
    const R ze1 = fmin(zto1 / prmuz, R(500.0));
    const R ze2 = expo(T, ze1);
    pref = (zgt - za1 * (R(1.0) - ze2)) / (R(1.0) + zgt);
    ptra = R(1.0) - pref;
    prefd = zgt / (R(1.0) + zgt);
    ptrad = R(1.0) - prefd;
    if (ze2 == R(1.0)) {
      pref = R(0.0);
      ptra = R(1.0);
      prefd = R(0.0);
      ptrad = R(1.0);
    }
    return;
  }
  const R za1 = zgamma1 * zgamma4 + zgamma2 * zgamma3;
  const R za2 = zgamma1 * zgamma3 + zgamma2 * zgamma4;
  const R zrk = sqrt(zgamma1 * zgamma1 - zgamma2 * zgamma2);
  const R zrp = zrk * prmuz;
  const R zrp1 = R(1.0) + zrp;
  const R zrm1 = R(1.0) - zrp;
  const R zrk2 = R(2.0) * zrk;
  const R zrpp = R(1.0) - zrp * zrp;
  const R zrkg = zrk + zgamma1;
  const R zr1 = zrm1 * (za2 + zrk * zgamma3);
  const R zr2 = zrp1 * (za2 - zrk * zgamma3);
  const R zr3 = zrk2 * (zgamma3 - za2 * prmuz);
  const R zr4 = zrpp * zrkg;
  const R zr5 = zrpp * (zrk - zgamma1);
  const R zt1 = zrp1 * (za1 + zrk * zgamma4);
  const R zt2 = zrm1 * (za1 - zrk * zgamma4);
  const R zt3 = zrk2 * (zgamma4 + za1 * prmuz);
  const R zbeta = (zgamma1 - zrk) / zrkg;
  const R ze1 = fmin(zrk * zto1, R(500.0));
  const R ze2 = fmin(zto1 / prmuz, R(500.0));
  const R zem1 = expo(T, ze1);
  const R zep1 = R(1.0) / zem1;
  const R zem2 = expo(T, ze2);
  const R zep2 = R(1.0) / zem2;
  const R zdenr = zr4 * zep1 + zr5 * zem1;
  const R zdent = zr4 * zep1 + zr5 * zem1;  // zt4 = zr4, zt5 = zr5
  if (zdenr >= -eps && zdenr <= eps) {
    pref = eps;
    ptra = zem2;
  } else {
    pref = zw * (zr1 * zep1 - zr2 * zem1 - zr3 * zem2) / zdenr;
    ptra = zem2 - zem2 * zw * (zt1 * zep1 - zt2 * zem1 - zt3 * zep2) / zdent;
  }
  const R zemm = zem1 * zem1;
  const R zdend = R(1.0) / ((R(1.0) - zbeta * zemm) * zrkg);
  prefd = zgamma2 * (R(1.0) - zemm) * zdend;
  ptrad = zrk2 * zem1 * zdend;
}

// exp(-ze) with the table index taken in fp64 (the float table's entries)
__device__ __forceinline__ double expo_d(const float* __restrict__ T, double ze) {
  if (ze <= 0.06) return 1.0 - ze + 0.5 * ze * ze;
  const double tblind = ze / (c_S.bpade + ze);
  const int itind = (int)(10000.0 * tblind + 0.5);
  return (double)tb(T, c_S.exp_tbl + itind);
}

// reftra_sw in fp32 (rrtmg_sw_reftra.f90:107-326, kmodts = 2): the same
// expressions, evaluated so that fp32 keeps them accurate.
//  * zco is the co-albedo 1 - zw, carried through the optics: the
//    non-conservative k = sqrt(gamma1^2 - gamma2^2) is formed as
//    sqrt(2 zco (gamma1 + gamma2)) (gamma1 - gamma2 = 2 (1 - zw)), and the
//    conservative-scattering test zwo >= zwcrit as 1 - zwo <= 1 - zwcrit.
//  * The direct-beam reflectance and transmittance have a removable
//    singularity at k mu0 = 1 (their numerators and zdenr vanish together).
//    Dividing it out leaves q = (e1 - e2) / (1 - k mu0) with e1 = exp(-k tau),
//    e2 = exp(-tau / mu0); in the Taylor range of both (od_lo) q is formed
//    exactly as e2' (1 - (x1 + x2) / 2), elsewhere near k mu0 = 1 the table
//    entries and 1 - k mu0 are taken in fp64, as the reference selects them.
static __device__ void reftra_f(const float* __restrict__ T, bool chk, float zg, float prmuz, float zto1, float zw,
                         float zco, float& pref, float& prefd, float& ptra, float& ptrad) {
  if (!chk) {
    pref = 0.0f;
    ptra = 1.0f;
    prefd = 0.0f;
    ptrad = 1.0f;
    return;
  }
  const float zg3 = 3.0f * zg;
  const float g1 = (8.0f - zw * (5.0f + zg3)) * 0.25f;
  const float g2 = 3.0f * (zw * (1.0f - zg)) * 0.25f;
  const float g3 = (2.0f - zg3 * prmuz) * 0.25f;
  const float g4 = 1.0f - g3;
  float q2 = 0.0f, denom = 1.0f;
  if (zg != 1.0f) {
    const float qg = zg / (1.0f - zg);
    q2 = qg * qg;
    denom = 1.0f - zco * q2;
  }
  // zwo = zw / denom >= zwcrit, i.e. 1 - zwo = zco (1 - q^2) / denom <= 1 - zwcrit
  const bool cons = zw > 0.0f && denom > 0.0f && zco * (1.0f - q2) <= (float)(1.0 - 0.9999995) * denom;
  if (cons) {
    const float za = g1 * prmuz;
    const float za1 = za - g3;
    const float zgt = g1 * zto1;
    const float ze1 = fminf(zto1 / prmuz, 500.0f);
    const float ze2 = expo(T, ze1);
    if (ze2 == 1.0f) {
      pref = 0.0f;
      ptra = 1.0f;
      prefd = 0.0f;
      ptrad = 1.0f;
      return;
    }
    const float r = 1.0f / (1.0f + zgt);
    pref = (zgt - za1 * (1.0f - ze2)) * r;
    ptra = 1.0f - pref;
    prefd = zgt * r;
    ptrad = 1.0f - prefd;
    return;
  }
  const float zrk = sqrtf(2.0f * zco * (g1 + g2));
  const float zrp = zrk * prmuz;
  const float om = 1.0f - zrp, op = 1.0f + zrp;
  const float za1 = g1 * g4 + g2 * g3, za2 = g1 * g3 + g2 * g4;
  const float zrkg = zrk + g1;
  const float zbeta = (g1 - zrk) / zrkg;
  const float ze1 = fminf(zrk * zto1, 500.0f), ze2 = fminf(zto1 / prmuz, 500.0f);
  float e1 = expo(T, ze1), e2 = expo(T, ze2);
  const bool taylor = ze1 <= 0.06f && ze2 <= 0.06f;
  float q = taylor ? ze2 * (1.0f - 0.5f * (ze1 + ze2)) : (e1 - e2) / om;
  if (!taylor && fabsf(om) < 2e-2f) {
    const double zwd = zw, zgd = zg;
    const double g1d = (8.0 - zwd * (5.0 + 3.0 * zgd)) * 0.25, g2d = 3.0 * (zwd * (1.0 - zgd)) * 0.25;
    const double kd = sqrt(2.0 * (double)zco * (g1d + g2d));
    const double d1 = expo_d(T, fmin(kd * (double)zto1, 500.0)), d2 = expo_d(T, fmin((double)zto1 / (double)prmuz, 500.0));
    e1 = (float)d1;
    e2 = (float)d2;
    q = (float)((d1 - d2) / (1.0 - kd * (double)prmuz));
  }
  const float dn = zrkg + (zrk - g1) * e1 * e1;  // zdenr = (1 - k^2 mu0^2) dn / e1
  if (fabsf(om * op * dn) <= 1.e-08f * e1) {
    pref = 1.e-08f;
    ptra = e2;
  } else {
    const float rdn = 1.0f / dn;
    const float uo = (1.0f - e1 * e2) / op;
    const float a = za2, b = zrk * g3, c = za1, d = zrk * g4;
    pref = zw * ((a + b) * uo - (a - b) * e1 * q) * rdn;
    ptra = e2 - zw * ((c - d) * e1 * uo - (c + d) * q) * rdn;
  }
  const float zemm = e1 * e1;
  const float zdend = 1.0f / ((1.0f - zbeta * zemm) * zrkg);
  prefd = g2 * (1.0f - zemm) * zdend;
  ptrad = 2.0f * zrk * e1 * zdend;
}

// per-layer setcoef values in shared memory (computed in fp64, kept as R)
template <typename R>
struct Lay {
  R fac00, fac01, fac10, fac11, selffac, selffrac, forfac, forfrac;
  R colh2o, colco2, colo3, colch4, colo2, colmol;
  double pdp;
  int jp, jt, jt1, indself, indfor, lower;
};
template <typename R>
struct Smem {
  Lay<R>* L;       // [nl]
  double* sfz;     // [NG] sfluxzen, then the incoming flux of each g-point
  double* flx;     // [4 * (nl + 1)] level sums: up, down, clear up, clear down
  float* aer;      // fp32 kernels: [nl][NB][3] aerosol tau, ssa, asymmetry of the column
  char* stage;     // [2][NT][sw_stage_bytes] per-thread copy stages of the two passes
  int* iscal;      // [0] laytrop, [1] status, [4 + k] solar-source layer of band k
};
// bytes a thread stages per layer (down pass: six McICA doubles, taug, taur)
// or per level (up pass: the NVL values of its g-point), padded to 16
template <typename R>
__host__ __device__ constexpr int sw_stage_bytes() {
  return (6 * 8 + 2 * (int)sizeof(R)) > NVL * (int)sizeof(R) ? ((6 * 8 + 2 * (int)sizeof(R)) + 15) / 16 * 16
                                                               : NVL * (int)sizeof(R);
}
template <typename R>
__host__ __device__ inline size_t sw_aer_floats(int nl) {
  return sizeof(R) == 4 ? (size_t)nl * NB * 3 : 0;
}
template <typename R>
__host__ __device__ inline size_t sw_smem_bytes(int nl) {
  return (size_t)nl * sizeof(Lay<R>) + NG * 8 + (size_t)4 * (nl + 1) * 8 + sw_aer_floats<R>(nl) * 4 + 15 +
         (size_t)2 * NT * sw_stage_bytes<R>() + 32 * 4;
}
template <typename R>
__device__ inline Smem<R> carve(char* p, int nl) {
  Smem<R> s;
  s.L = reinterpret_cast<Lay<R>*>(p);
  p += (size_t)nl * sizeof(Lay<R>);
  s.sfz = reinterpret_cast<double*>(p);
  p += NG * 8;
  s.flx = reinterpret_cast<double*>(p);
  p += (size_t)4 * (nl + 1) * 8;
  s.aer = reinterpret_cast<float*>(p);
  p += sw_aer_floats<R>(nl) * 4;
  p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 15) & ~(uintptr_t)15);
  s.stage = p;
  p += (size_t)2 * NT * sw_stage_bytes<R>();
  s.iscal = reinterpret_cast<int*>(p);
  return s;
}
// elements of R in one block's scratch slot: taug, taur, and NVL values per (level, g)
__host__ __device__ inline long long sw_slot_elems(int nl) {
  return (long long)(2 * nl + (nl + 1) * NVL) * NG;
}

__device__ __forceinline__ double in2(const double* __restrict__ a, long long ld, long long icol, int k) {
  return __ldg(a + icol + ld * k);
}

// the binary-species parameter (taumol.f90:306-312): speccomb, js, fs
// (fs = fmod(specmult, 1), which for these finite arguments is specmult - trunc(specmult))
template <typename R>
__device__ __forceinline__ void binary(R a, R b, R strrat, R mult, R& speccomb, int& js, R& fs) {
  const R oneminus = R(1.0 - 1.e-06);
  speccomb = a + strrat * b;
  R specparm = a / speccomb;
  if (specparm >= oneminus) specparm = oneminus;
  const R specmult = mult * (specparm);
  js = 1 + (int)specmult;
  fs = specmult - trunc(specmult);
  // a negative or NaN column amount would index outside the table: keep js in 1..mult
  js = js < 1 ? 1 : (js > (int)mult ? (int)mult : js);
}

// one taumol_sw cell: band index k (0..13), layer lay (0-based), g-point ig
// (1-based within the band); taug and taur (rrtmg_sw_taumol.f90:275-1785)
template <typename R>
__device__ void taumol_cell(const R* __restrict__ T, const Smem<R>& S, int k, int lay, int ig, R& taug, R& taur) {
  const SwBand& B = c_S.b[k];
  const Lay<R>& l = S.L[lay];
  const int band = k + 16;
  auto A = [&](int i) { return tb(T, B.absa + (i - 1) + B.absa_rows * (ig - 1)); };
  auto Bt = [&](int i) { return tb(T, B.absb + (i - 1) + B.absb_rows * (ig - 1)); };
  auto self = [&]() {
    const R s0 = tb(T, B.selfref + (l.indself - 1) + 10 * (ig - 1));
    const R s1 = tb(T, B.selfref + l.indself + 10 * (ig - 1));
    return l.selffac * (s0 + l.selffrac * (s1 - s0));
  };
  auto forx = [&]() {
    const R f0 = tb(T, B.forref + (l.indfor - 1) + B.nfor * (ig - 1));
    const R f1 = tb(T, B.forref + l.indfor + B.nfor * (ig - 1));
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
  auto eight = [&](bool upper, int js, R fs) {
    const R f000 = (R(1.0) - fs) * l.fac00, f010 = (R(1.0) - fs) * l.fac10, f100 = fs * l.fac00,
            f110 = fs * l.fac10, f001 = (R(1.0) - fs) * l.fac01, f011 = (R(1.0) - fs) * l.fac11,
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
  const R rayl0 = B.rayl >= 0 ? tb(T, B.rayl + (B.rayl_per_g ? ig - 1 : 0)) : R(0.0);
  R speccomb, fs;
  int js;
  taur = l.colmol * rayl0;
  switch (band) {
    case 16:
      if (lower) {
        binary(l.colh2o, l.colch4, R(252.131), R(8.0), speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx());
      } else {
        taug = l.colch4 * four(true);
      }
      break;
    case 17:
    case 21:
      if (lower) {
        binary(l.colh2o, l.colco2, band == 17 ? R(0.364641) : R(0.0045321), R(8.0), speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx());
      } else {
        binary(l.colh2o, l.colco2, band == 17 ? R(0.364641) : R(0.0045321), R(4.0), speccomb, js, fs);
        taug = speccomb * eight(true, js, fs) + l.colh2o * l.forfac * forx();
      }
      break;
    case 18:
    case 19:
      if (lower) {
        if (band == 18)
          binary(l.colh2o, l.colch4, R(38.9589), R(8.0), speccomb, js, fs);
        else
          binary(l.colh2o, l.colco2, R(5.49281), R(8.0), speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx());
      } else {
        taug = (band == 18 ? l.colch4 : l.colco2) * four(true);
      }
      break;
    case 20: {
      const R ch4 = l.colch4 * tb(T, B.absch4 + ig - 1);
      if (lower)
        taug = l.colh2o * (four(false) + self() + l.forfac * forx()) + ch4;
      else
        taug = l.colh2o * (four(true) + l.forfac * forx()) + ch4;
      break;
    }
    case 22: {
      const R o2adj = R(1.6);
      const R o2cont = R(4.35e-4) * l.colo2 / R(350.0 * 2.0);
      if (lower) {
        binary(l.colh2o, l.colo2, R(1.6 * 0.022708), R(8.0), speccomb, js, fs);
        taug = speccomb * eight(false, js, fs) + l.colh2o * (self() + l.forfac * forx()) + o2cont;
      } else {
        taug = l.colo2 * o2adj * four(true) + o2cont;
      }
      break;
    }
    case 23:
      taug = lower ? l.colh2o * (R(1.029) * four(false) + self() + l.forfac * forx()) : R(0.0);
      break;
    case 24:
      if (lower) {
        binary(l.colh2o, l.colo2, R(0.124692), R(8.0), speccomb, js, fs);
        const R ra0 = tb(T, B.rayla + (ig - 1) + B.ng * (js - 1)), ra1 = tb(T, B.rayla + (ig - 1) + B.ng * js);
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
      taug = R(0.0);
      break;
    case 27:
      taug = l.colo3 * four(!lower);
      break;
    case 28:
      binary(l.colo3, l.colo2, R(6.67029e-07), lower ? R(8.0) : R(4.0), speccomb, js, fs);
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
template <typename R>
__device__ int solar_layer(const Smem<R>& S, int k, int nl, int lt) {
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
template <typename R>
__device__ double solar_source(const R* __restrict__ T, const Smem<R>& S, int k, int ig, int ls, int lt, int nl) {
  const int band = k + 16;
  const SwBand& B = c_S.b[k];
  const bool in_lower = ls >= 1 && ls <= lt;
  const bool in_upper = ls > lt && ls <= nl;
  const bool lower_band = !(band == 16 || band == 17 || band >= 27);
  if (lower_band ? !in_lower : !in_upper) return 0.0;
  const Lay<R>& l = S.L[ls - 1];
  auto sf = [&](int j) { return tb(T, B.sfluxref + (ig - 1) + B.ng * (j - 1)); };
  R speccomb, fs;
  int js;
  switch (band) {
    case 17: binary(l.colh2o, l.colco2, R(0.364641), R(4.0), speccomb, js, fs); break;
    case 18: binary(l.colh2o, l.colch4, R(38.9589), R(8.0), speccomb, js, fs); break;
    case 19: binary(l.colh2o, l.colco2, R(5.49281), R(8.0), speccomb, js, fs); break;
    case 21: binary(l.colh2o, l.colco2, R(0.0045321), R(8.0), speccomb, js, fs); break;
    case 22: binary(l.colh2o, l.colo2, R(1.6 * 0.022708), R(8.0), speccomb, js, fs); break;
    case 24: binary(l.colh2o, l.colo2, R(0.124692), R(8.0), speccomb, js, fs); break;
    case 28: binary(l.colo3, l.colo2, R(6.67029e-07), R(4.0), speccomb, js, fs); break;
    case 27: return (double)(R(50.15 / 48.37) * sf(1));
    default: return (double)sf(1);
  }
  return (double)(sf(js) + fs * (sf(js + 1) - sf(js)));
}

// cldprmc_sw for one cell (rrtmg_sw_cldprmc.f90:103-334).  cf, ciwp, clwp,
// radice, radliq are the double inputs (decisions are taken on them); tauc,
// ssac, asmc enter as the McICA values and leave as the cell's delta-scaled
// optics, coc (fp32 kernels) as its co-albedo 1 - ssac formed from the
// co-albedo tables; returns a stop code
template <typename R>
__device__ int cloud_cell(const R* __restrict__ T, const SwArgs& a, int band, double cfd, R cf, double ciwpd,
                          double clwpd, const double* prei, const double* prel, const double* pfsfc, double ssacd,
                          R& tauc, R& ssac, R& asmc, R& coc) {
  const double cldmin = 1.e-20;
  const R eps = R(1.e-06);
  if (!ge_in(cfd, cf, cldmin)) return 0;
  const R ciwp = to_r<R>(ciwpd), clwp = to_r<R>(clwpd);
  bool wp;  // cwp >= cldmin (in fp32 a tie with the threshold is not resolved)
  if constexpr (sizeof(R) == 8)
    wp = ciwpd + clwpd >= cldmin;
  else
    wp = ciwp + clwp >= (float)cldmin;
  if (!(wp || tauc >= R(cldmin))) return 0;
  if (a.inflag == 0) {
    const R ffp = to_r<R>(__ldg(pfsfc)), ffp1 = R(1.0) - ffp, ffpssa = R(1.0) - ffp * ssac;
    const R ssacloud_a = ffp1 * ssac / ffpssa;
    const R taucloud_a = ffpssa * tauc;
    if (sizeof(R) == 4) coc = (R)(1.0 - ssacd) / ffpssa;  // 1 - ssacloud_a
    ssac = ssacloud_a;
    tauc = taucloud_a;
    asmc = (asmc - ffp) / (ffp1);
    return 0;
  }
  if (a.inflag != 2) return GB_COL_INFLAG1;
  const int ib = band;
  auto c2 = [&](int off, int rows, int i) { return tb(T, off + (i - 1) + rows * (ib - 16)); };
  R extcoice = R(0), ssacoice = R(0), gice = R(0), forwice = R(0);
  R extcoliq = R(0), ssacoliq = R(0), gliq = R(0), forwliq = R(0);
  R coice = R(0), coliq = R(0);  // co-albedos of the ice and liquid optics (fp32 kernels)
  if (nonzero_in(ciwpd)) {
    const double radiced = __ldg(prei);
    const R radice = to_r<R>(radiced);
    if (a.iceflag == 1) {
      if (outside_in(radiced, radice, 13.0, 130.0)) return GB_COL_ICE_BOUNDS;
      const double w2 = c_S.wavenum2[ib - 16];
      const int icx = w2 > 1.43e04 ? 1 : w2 > 7.7e03 ? 2 : w2 > 5.3e03 ? 3 : w2 > 4.0e03 ? 4 : 5;
      extcoice = (R)(c_S.abari[icx - 1] + c_S.bbari[icx - 1] / radiced);
      ssacoice = (R)(1.0 - c_S.cbari[icx - 1] - c_S.dbari[icx - 1] * radiced);
      if (sizeof(R) == 4) coice = (R)(c_S.cbari[icx - 1] + c_S.dbari[icx - 1] * radiced);
      gice = (R)(c_S.ebari[icx - 1] + c_S.fbari[icx - 1] * radiced);
      if (gice >= R(1.0)) gice = R(1.0) - eps;
      forwice = gice * gice;
    } else if (a.iceflag == 2 || a.iceflag == 3) {
      const bool f3 = a.iceflag == 3;
      if (f3 ? outside_in(radiced, radice, 5.0, 140.0) : outside_in(radiced, radice, 5.0, 131.0))
        return f3 ? GB_COL_DGE_BOUNDS : GB_COL_ICE_BOUNDS;
      const R factor = (radice - R(2.0)) / R(3.0);
      int index = (int)factor;
      if (index == (f3 ? 46 : 43)) index = f3 ? 45 : 42;
      const R fint = factor - (R)index;
      const int rows = f3 ? 46 : 43;
      index = index < 1 ? 1 : (index > rows - 1 ? rows - 1 : index);  // in the table for any input (a NaN radius)
      const int oe = f3 ? c_S.extice3 : c_S.extice2, os = f3 ? c_S.ssaice3 : c_S.ssaice2,
                og = f3 ? c_S.asyice3 : c_S.asyice2;
      extcoice = c2(oe, rows, index) + fint * (c2(oe, rows, index + 1) - c2(oe, rows, index));
      ssacoice = c2(os, rows, index) + fint * (c2(os, rows, index + 1) - c2(os, rows, index));
      gice = c2(og, rows, index) + fint * (c2(og, rows, index + 1) - c2(og, rows, index));
      if (sizeof(R) == 4) {
        const int oc = f3 ? c_S.coaice3 : c_S.coaice2;
        coice = c2(oc, rows, index) + fint * (c2(oc, rows, index + 1) - c2(oc, rows, index));
      }
      if (f3) {
        const R fdelta = c2(c_S.fdlice3, 46, index) + fint * (c2(c_S.fdlice3, 46, index + 1) -
                                                              c2(c_S.fdlice3, 46, index));
        if (fdelta < R(0.0) || fdelta > R(1.0)) return GB_COL_SW_OPTICS;
        forwice = fdelta + R(0.5) / ssacoice;
        if (forwice > gice) forwice = gice;
      } else {
        forwice = gice * gice;
      }
    } else {
      return GB_COL_SW_UNSUPPORTED;
    }
    if (extcoice < R(0.0) || ssacoice > R(1.0) || ssacoice < R(0.0) || gice > R(1.0) || gice < R(0.0))
      return GB_COL_SW_OPTICS;
  }
  if (nonzero_in(clwpd)) {
    if (a.liqflag != 1) return GB_COL_SW_UNSUPPORTED;
    const double radliqd = __ldg(prel);
    const R radliq = to_r<R>(radliqd);
    if (outside_in(radliqd, radliq, 2.5, 60.0)) return GB_COL_LIQ_BOUNDS;
    int index = (int)(radliq - R(1.5));
    if (index == 0) index = 1;
    if (index == 58) index = 57;
    const R fint = radliq - R(1.5) - (R)index;
    extcoliq = c2(c_S.extliq1, 58, index) + fint * (c2(c_S.extliq1, 58, index + 1) - c2(c_S.extliq1, 58, index));
    ssacoliq = c2(c_S.ssaliq1, 58, index) + fint * (c2(c_S.ssaliq1, 58, index + 1) - c2(c_S.ssaliq1, 58, index));
    if (sizeof(R) == 4)
      coliq = c2(c_S.coaliq1, 58, index) + fint * (c2(c_S.coaliq1, 58, index + 1) - c2(c_S.coaliq1, 58, index));
    if (fint < R(0.0) && ssacoliq > R(1.0)) {
      ssacoliq = c2(c_S.ssaliq1, 58, index);
      if (sizeof(R) == 4) coliq = c2(c_S.coaliq1, 58, index);
    }
    gliq = c2(c_S.asyliq1, 58, index) + fint * (c2(c_S.asyliq1, 58, index + 1) - c2(c_S.asyliq1, 58, index));
    forwliq = gliq * gliq;
    if (extcoliq < R(0.0) || ssacoliq > R(1.0) || ssacoliq < R(0.0) || gliq > R(1.0) || gliq < R(0.0))
      return GB_COL_SW_OPTICS;
  }
  const R tauliqorig = clwp * extcoliq;
  const R tauiceorig = ciwp * extcoice;
  const R ssaliq = ssacoliq * (R(1.0) - forwliq) / (R(1.0) - forwliq * ssacoliq);
  const R tauliq = (R(1.0) - forwliq * ssacoliq) * tauliqorig;
  const R ssaice = ssacoice * (R(1.0) - forwice) / (R(1.0) - forwice * ssacoice);
  const R tauice = (R(1.0) - forwice * ssacoice) * tauiceorig;
  const R scatliq = ssaliq * tauliq;
  R scatice = ssaice * tauice;
  tauc = tauliq + tauice;
  // 1 - ssac: each delta-scaled part absorbs tau_orig x co-albedo
  if (sizeof(R) == 4) coc = tauc == R(0.) ? R(0.) : (tauliqorig * coliq + tauiceorig * coice) / tauc;
  if (tauc == R(0.)) tauc = R(cldmin);
  if (scatice == R(0.)) scatice = R(cldmin);
  ssac = (scatliq + scatice) / tauc;
  if (a.iceflag == 3)
    asmc = (R(1.0) / (scatliq + scatice)) *
           (scatliq * (gliq - forwliq) / (R(1.0) - forwliq) + scatice * ((gice - forwice) / (R(1.0) - forwice)));
  else
    asmc = (scatliq * (gliq - forwliq) / (R(1.0) - forwliq) + scatice * (gice - forwice) / (R(1.0) - forwice)) /
           (scatliq + scatice);
  return 0;
}

// one (level, g-point) record of the slot, written with 16-byte stores
template <typename R>
__device__ __forceinline__ void store_rec(R* dst, const R (&v)[NVL]) {
  if constexpr (sizeof(R) == 4) {
    float4* p = reinterpret_cast<float4*>(dst);
#pragma unroll
    for (int i = 0; i < NVL / 4; ++i) p[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  } else {
    double2* p = reinterpret_cast<double2*>(dst);
#pragma unroll
    for (int i = 0; i < NVL / 2; ++i) p[i] = make_double2(v[2 * i], v[2 * i + 1]);
  }
}

// one column by the block
template <typename R>
__device__ void sw_column(const SwArgs& a, long long icol, const Smem<R>& S, R* __restrict__ scr,
                          const R* __restrict__ T) {
  const int tid = threadIdx.x;
  const int nl = a.nlay;
  const long long ld = a.ld;
  if (tid < 32) S.iscal[tid] = 0;
  __syncthreads();
  // ---- 1. inatm_sw and setcoef_sw per layer in fp64 (rrtmg_sw_rad.f90:957-976, setcoef.f90:95-225)
  const double amd = 28.9660, amw = 18.0160, stpfac = 296.0 / 1013.0;
  int bad = 0;
  for (int lay = tid; lay < nl; lay += NT) {
    Lay<R>& L = S.L[lay];
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
    const double forfac = scalefac / (1. + water);
    L.forfac = (R)forfac;
    if (low) {
      double factor = (332.0 - tavel) / 36.0;
      const int indfor = min(2, max(1, (int)factor));
      L.indfor = indfor;
      L.forfrac = (R)(factor - (double)indfor);
      L.selffac = (R)(water * forfac);
      factor = (tavel - 188.0) / 7.2;
      const int indself = min(9, max(1, (int)factor - 7));
      L.indself = indself;
      L.selffrac = (R)(factor - (double)(indself + 7));
    } else {
      const double factor = (tavel - 188.0) / 36.0;
      L.indfor = 3;
      L.forfrac = (R)(factor - 1.0);
      L.selffac = R(0.0);
      L.selffrac = R(0.0);
      L.indself = 0;
    }
    const double colh2o = 1.e-20 * w1;
    double colco2 = 1.e-20 * w2, colch4 = 1.e-20 * w6, colo2 = 1.e-20 * w7;
    if (colco2 == 0.0) colco2 = 1.e-32 * coldry;
    if (colch4 == 0.0) colch4 = 1.e-32 * coldry;
    if (colo2 == 0.0) colo2 = 1.e-32 * coldry;
    L.colh2o = (R)colh2o;
    L.colco2 = (R)colco2;
    L.colo3 = (R)(1.e-20 * w3);
    L.colch4 = (R)colch4;
    L.colo2 = (R)colo2;
    L.colmol = (R)(1.e-20 * coldry + colh2o);
    const double compfp = 1.0 - fp;
    L.fac10 = (R)(compfp * ft);
    L.fac00 = (R)(compfp * (1.0 - ft));
    L.fac11 = (R)(fp * ft1);
    L.fac01 = (R)(fp * (1.0 - ft1));
  }
  bad = __syncthreads_or(bad);
  const int lt = S.iscal[0];
  // taumol treats layers 1..laytrop as the lower atmosphere (by index)
  for (int lay = tid; lay < nl; lay += NT) S.L[lay].lower = lay < lt;
  if (tid < NB) S.iscal[4 + tid] = solar_layer(S, tid, nl, lt);
  __syncthreads();
  // ---- 2. taumol_sw per band and cell into the slot; the solar source per g-point
  R* sg = scr;                       // taug [nl][NG]
  R* sr = scr + (size_t)nl * NG;     // taur [nl][NG]
  for (int k = 0; k < NB; ++k) {
    const SwBand& B = c_S.b[k];
    for (int i = tid; i < nl * B.ng; i += NT) {
      const int lay = i / B.ng, ig = i - lay * B.ng + 1;
      R tg, tr;
      taumol_cell(T, S, k, lay, ig, tg, tr);
      sg[(size_t)lay * NG + B.g0 + ig - 1] = tg;
      sr[(size_t)lay * NG + B.g0 + ig - 1] = tr;
    }
  }
  if (tid < NG) {
    const int k = c_S.ngb[tid] - 16;
    S.sfz[tid] = solar_source(T, S, k, tid - c_S.b[k].g0 + 1, S.iscal[4 + k], lt, nl);
  }
  if constexpr (sizeof(R) == 4) {
    // the column's aerosol optics once per (layer, band) instead of per g-point
    if (a.iaer == 10)
      for (int i = tid; i < nl * NB; i += NT) {
        const int lay = i / NB, b = i - lay * NB;
        const long long o = icol + ld * (lay + (long long)nl * b);
        S.aer[3 * i] = d2f_fast(__ldg(a.tauaer + o));
        S.aer[3 * i + 1] = d2f_fast(__ldg(a.ssaaer + o));
        S.aer[3 * i + 2] = d2f_fast(__ldg(a.asmaer + o));
      }
  }
  __syncthreads();
  // ---- 3. per g-point: optics, reftra, adding (spcvmc_sw :150-440, vrtqdr_sw)
  const bool live = tid < NG;
  const int g = live ? tid : NG - 1;
  const int band = c_S.ngb[g];
  const int ibm = band - 15;
  double prmu0d = __ldg(a.coszen + icol);
  if (prmu0d < 1.e-10) prmu0d = 1.e-10;
  const R prmu0 = (R)prmu0d;
  const R albp = (R)(ibm >= 10 && ibm <= 13 ? __ldg(a.asdir + icol) : __ldg(a.aldir + icol));
  const R albd = (R)(ibm >= 10 && ibm <= 13 ? __ldg(a.asdif + icol) : __ldg(a.aldif + icol));
  // the incoming flux of the g-point (fp64) replaces its source in shared memory
  if (live) S.sfz[g] = a.adjflux[band - 16] * S.sfz[g] * prmu0d;
  // slot layout after taug/taur: one record of NVL values per (level k = 1..nl+1, g-point),
  // record (k, g) at ((k - 1) * NG + g) * NVL
  R* V = scr + (size_t)2 * nl * NG;
  auto rec_of = [&](int k) { return V + ((size_t)(k - 1) * NG + g) * NVL; };
  enum { RC, RDC, TC, TDC, DBC, RT, RDT, TT, TDT, DBT, ZTDC, RDNDC, TDBC, ZTDT, RDNDT, TDBT };
  constexpr int SB = sw_stage_bytes<R>();
  auto stage = [&](int i) { return S.stage + ((size_t)(i & 1) * NT + tid) * SB; };
  // down pass: layer jk's McICA cell (six doubles) and gas optical depths, staged one layer ahead
  auto issue_down = [&](int jk) {
    char* d = stage(jk);
    const int lay = nl - jk;
    if (a.icld >= 1) {
      const long long o = g + (long long)NG * (icol + ld * lay);
      cp_async8(d, a.cldfmcl + o);
      cp_async8(d + 8, a.taucmcl + o);
      cp_async8(d + 16, a.ssacmcl + o);
      cp_async8(d + 24, a.asmcmcl + o);
      cp_async8(d + 32, a.ciwpmcl + o);
      cp_async8(d + 40, a.clwpmcl + o);
    }
    cp_async_r(d + 48, sg + (size_t)lay * NG + g);
    cp_async_r(d + 48 + sizeof(R), sr + (size_t)lay * NG + g);
    cp_commit();
  };
  int err = 0;
  // top-down: layer jk (1 = top) is model layer ikl = nl + 1 - jk
  R tdbc = R(1.0), tdbt = R(1.0), ztdc = R(1.0), ztdt = R(1.0), rdndc = R(0.0), rdndt = R(0.0);
  issue_down(1);
  for (int jk = 1; jk <= nl; ++jk) {
    const int lay = nl - jk;  // 0-based model layer
    if (jk < nl)
      issue_down(jk + 1);
    else
      cp_commit();  // an empty group keeps one group in flight
    cp_wait1();
    const char* d = stage(jk);
    const double* m = reinterpret_cast<const double*>(d);
    const R taug = *reinterpret_cast<const R*>(d + 48), taur = *reinterpret_cast<const R*>(d + 48 + sizeof(R));
    R taua = R(0.0), ssaa = R(1.0), asma = R(0.0);
    if (a.iaer == 10) {
      if constexpr (sizeof(R) == 4) {
        const float* pa = S.aer + 3 * (lay * NB + ibm - 1);
        taua = pa[0];
        ssaa = pa[1];
        asma = pa[2];
      } else {
        const long long o = icol + ld * (lay + (long long)nl * (ibm - 1));
        taua = __ldg(a.tauaer + o);
        ssaa = __ldg(a.ssaaer + o);
        asma = __ldg(a.asmaer + o);
      }
    }
    double cfd = 0.0;
    R cf = R(0.0), tcm = R(0.0), wcm = R(1.0), gcm = R(0.0), coc = R(0.0);
    if (a.icld >= 1) {
      cfd = m[0];
      cf = to_r<R>(cfd);
      tcm = to_r<R>(m[1]);
      const double wcmd = m[2];
      wcm = to_r<R>(wcmd);
      coc = R(1.0) - wcm;  // cells cldprmc_sw leaves alone keep the caller's optics
      gcm = to_r<R>(m[3]);
      const long long o = g + (long long)NG * (icol + ld * lay);
      const int e = cloud_cell(T, a, band, cfd, cf, m[4], m[5], a.reicmcl + icol + ld * lay,
                               a.relqmcl + icol + ld * lay, a.fsfcmcl + o, wcmd, tcm, wcm, gcm, coc);
      if (e && live) err = e;
    }
    // clear-sky optics with delta scaling, then the cloud's added (spcvmc.f90:180-227)
    R rc, rdc, trc, tdc, ro, rdo, tro, tdo, ztauc, ztauo;
    const bool cloud_rt = gt_in(cfd, cf, 1.e-12);
    if constexpr (sizeof(R) == 8) {
      ztauc = taur + taug + taua;
      R zomcc = taur * R(1.0) + taua * ssaa;
      R zgcc = asma * ssaa * taua / zomcc;
      zomcc = zomcc / ztauc;
      const R zf = zgcc * zgcc, zwf = zomcc * zf;
      ztauc = (R(1.0) - zwf) * ztauc;
      zomcc = (zomcc - zwf) / (R(1.0) - zwf);
      zgcc = (zgcc - zf) / (R(1.0) - zf);
      ztauo = ztauc + tcm;
      R zomco = ztauc * zomcc + tcm * wcm;
      const R zgco = (tcm * wcm * gcm + ztauc * zomcc * zgcc) / zomco;
      zomco = zomco / ztauo;
      reftra(T, true, zgcc, prmu0, ztauc, zomcc, rc, rdc, trc, tdc);
      reftra(T, cloud_rt, zgco, prmu0, ztauo, zomco, ro, rdo, tro, tdo);
    } else {
      // the same optics with the co-albedo (absorption / extinction) carried beside the albedo
      const R tau0 = taur + taug + taua;
      const R scat = taur + taua * ssaa;
      R zgcc = asma * ssaa * taua / scat;
      const R rtau = R(1.0) / tau0;
      R zomcc = scat * rtau;
      R zcoc = (taug + taua * (R(1.0) - ssaa)) * rtau;
      const R zf = zgcc * zgcc, zwf = zomcc * zf;
      const R rwf = R(1.0) / (R(1.0) - zwf);
      ztauc = (R(1.0) - zwf) * tau0;
      zomcc = (zomcc - zwf) * rwf;
      zcoc = zcoc * rwf;
      zgcc = (zgcc - zf) / (R(1.0) - zf);
      ztauo = ztauc + tcm;
      R zomco = ztauc * zomcc + tcm * wcm;
      const R zgco = (tcm * wcm * gcm + ztauc * zomcc * zgcc) / zomco;
      const R rtauo = R(1.0) / ztauo;
      const R zcoo = (ztauc * zcoc + tcm * coc) * rtauo;
      zomco = zomco * rtauo;
      reftra_f(T, true, zgcc, prmu0, ztauc, zomcc, zcoc, rc, rdc, trc, tdc);
      reftra_f(T, cloud_rt, zgco, prmu0, ztauo, zomco, zcoo, ro, rdo, tro, tdo);
    }
    const R zclear = R(1.0) - cf, zcloud = cf;
    const R rt = zclear * rc + zcloud * ro, rdt = zclear * rdc + zcloud * rdo;
    const R tt = zclear * trc + zcloud * tro, tdt = zclear * tdc + zcloud * tdo;
    const R dbc = expo(T, ztauc / prmu0);
    const R dbt = zclear * dbc + zcloud * expo(T, ztauo / prmu0);
    // level jk's record, then the downward recurrence to level jk+1 (vrtqdr.f90:63-80)
    if (live) {
      const R rec[NVL] = {rc, rdc, trc, tdc, dbc, rt, rdt, tt, tdt, dbt, ztdc, rdndc, tdbc, ztdt, rdndt, tdbt};
      store_rec(rec_of(jk), rec);
    }
    if (jk == 1) {
      ztdc = trc;
      rdndc = rdc;
      ztdt = tt;
      rdndt = rdt;
    } else {
      R zr = R(1.0) / (R(1.0) - rdc * rdndc);
      const R nztdc = tdbc * trc + (tdc * ((ztdc - tdbc) + tdbc * rc * rdndc)) * zr;
      rdndc = rdc + tdc * tdc * rdndc * zr;
      ztdc = nztdc;
      zr = R(1.0) / (R(1.0) - rdt * rdndt);
      const R nztdt = tdbt * tt + (tdt * ((ztdt - tdbt) + tdbt * rt * rdndt)) * zr;
      rdndt = rdt + tdt * tdt * rdndt * zr;
      ztdt = nztdt;
    }
    tdbc = dbc * tdbc;
    tdbt = dbt * tdbt;
  }
  if (live) {
    const R rec[NVL] = {R(0), R(0), R(0), R(0), R(0), R(0), R(0), R(0), R(0), R(0), ztdc, rdndc, tdbc, ztdt, rdndt, tdbt};
    store_rec(rec_of(nl + 1), rec);
  }
  // bottom-up (vrtqdr.f90:44-60) and the level flux fractions (:82-88); level
  // jk's record is staged one level ahead, and its first four values are
  // replaced by the level's fractions fu, fd, cu, cd
  auto issue_up = [&](int jk) {
    char* d = stage(jk);
    const char* src = reinterpret_cast<const char*>(rec_of(jk));
#pragma unroll
    for (int i = 0; i < NVL * (int)sizeof(R) / 16; ++i) cp_async16(d + 16 * i, src + 16 * i);
    cp_commit();
  };
  R rupc = albp, rupdc = albd, rupt = albp, rupdt = albd;
  issue_up(nl + 1);
  for (int jk = nl + 1; jk >= 1; --jk) {
    if (jk > 1)
      issue_up(jk - 1);
    else
      cp_commit();
    cp_wait1();
    const R* v = reinterpret_cast<const R*>(stage(jk));
    if (jk <= nl) {
      R zr = R(1.0) / (R(1.0) - rupdc * v[RDC]);
      const R nrupc = v[RC] + (v[TDC] * ((v[TC] - v[DBC]) * rupdc + v[DBC] * rupc)) * zr;
      rupdc = v[RDC] + v[TDC] * v[TDC] * rupdc * zr;
      rupc = nrupc;
      zr = R(1.0) / (R(1.0) - rupdt * v[RDT]);
      const R nrupt = v[RT] + (v[TDT] * ((v[TT] - v[DBT]) * rupdt + v[DBT] * rupt)) * zr;
      rupdt = v[RDT] + v[TDT] * v[TDT] * rupdt * zr;
      rupt = nrupt;
    }
    R zr = R(1.0) / (R(1.0) - v[RDNDC] * rupdc);
    const R tdcl = v[TDBC], ztc = v[ZTDC];
    const R cu = (tdcl * rupc + (ztc - tdcl) * rupdc) * zr;
    const R cd = tdcl + (ztc - tdcl + tdcl * rupc * v[RDNDC]) * zr;
    zr = R(1.0) / (R(1.0) - v[RDNDT] * rupdt);
    const R tdtl = v[TDBT], ztt = v[ZTDT];
    const R fu = (tdtl * rupt + (ztt - tdtl) * rupdt) * zr;
    const R fd = tdtl + (ztt - tdtl + tdtl * rupt * v[RDNDT]) * zr;
    if (live) {
      R* r = rec_of(jk);
      if constexpr (sizeof(R) == 4) {
        *reinterpret_cast<float4*>(r) = make_float4(fu, fd, cu, cd);
      } else {
        reinterpret_cast<double2*>(r)[0] = make_double2(fu, fd);
        reinterpret_cast<double2*>(r)[1] = make_double2(cu, cd);
      }
    }
  }
  if (err) atomicMax(&S.iscal[1], err);
  __syncthreads();
  // ---- 4. fp64 sums over the g-points in order: level jk, flux q
  for (int t = tid; t < 4 * (nl + 1); t += NT) {
    const int jk = t >> 2, q = t & 3;
    const R* f = V + (size_t)jk * NG * NVL + q;  // record (jk + 1, g) value q at f[g * NVL]
    double s = 0.0;
#pragma unroll 4
    for (int gg = 0; gg < NG; ++gg) {
      if constexpr (sizeof(R) == 4)
        s = fma(S.sfz[gg], f2d_fast(f[gg * NVL]), s);
      else
        s = s + S.sfz[gg] * f[gg * NVL];
    }
    S.flx[t] = s;
  }
  __syncthreads();
  // outputs: fluxes per level, net fluxes, heating rates (rrtmg_sw_rad.f90:552-584)
  int st = S.iscal[1];
  if (bad) st = GB_COL_BADVAL;
  if (tid == 0) {
    if (a.col_err) a.col_err[icol] = st;
    if (st) atomicMax(a.err_flag, st);
  }
  const long long ldo = a.ldo;
  for (int k = tid; k <= nl; k += NT) {  // output level k+1 (1-based) = level jk = nl + 1 - k from the top
    const double* p = S.flx + (size_t)(nl - k) * 4;
    const long long o = icol + ldo * k;
    a.swuflx[o] = p[0];
    a.swdflx[o] = p[1];
    a.swuflxc[o] = p[2];
    a.swdflxc[o] = p[3];
  }
  for (int k = tid; k < nl; k += NT) {
    const double* p0 = S.flx + (size_t)(nl - k) * 4;      // output level k+1
    const double* p1 = S.flx + (size_t)(nl - 1 - k) * 4;  // output level k+2
    const double zdpgcp = c_S.heatfac / S.L[k].pdp;
    const long long o = icol + ldo * k;
    const double n0 = p0[1] - p0[0], n1 = p1[1] - p1[0];
    const double c0 = p0[3] - p0[2], c1 = p1[3] - p1[2];
    a.swhr[o] = k == nl - 1 ? 0.0 : (n1 - n0) * zdpgcp;
    a.swhrc[o] = k == nl - 1 ? 0.0 : (c1 - c0) * zdpgcp;
  }
  __syncthreads();
}

template <typename R, int MINB>
__global__ void __launch_bounds__(NT, MINB) sw_kernel(const __grid_constant__ SwArgs a, const R* __restrict__ T,
                                                      R* __restrict__ scratch) {
  extern __shared__ __align__(16) char smem_raw[];
  const Smem<R> S = carve<R>(smem_raw, a.nlay);
  R* scr = scratch + (long long)blockIdx.x * sw_slot_elems(a.nlay);
  for (long long icol = blockIdx.x; icol < a.ncol; icol += gridDim.x) sw_column(a, icol, S, scr, T);
}

// uploads the table directory of this translation unit's kernels
static inline cudaError_t sw_set_tab(const SwTab& t) { return cudaMemcpyToSymbol(c_S, &t, sizeof(t)); }

// all columns of `a` with at most `slots` persistent blocks of MINB per SM
template <typename R, int MINB>
cudaError_t sw_launch_t(const SwArgs& a, const R* d_tables, R* scratch, long long slots, cudaStream_t stream) {
  if (a.ncol <= 0) return cudaSuccess;
  const size_t smem = sw_smem_bytes<R>(a.nlay);
  const void* fn = (const void*)sw_kernel<R, MINB>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long nb = slots < a.ncol ? slots : a.ncol;
  sw_kernel<R, MINB><<<(int)nb, NT, smem, stream>>>(a, d_tables, scratch);
  return cudaGetLastError();
}

}  // namespace gbsw
