// Fused RRTMG_LW column kernel for GB300 (sm_103a).
//
// A persistent grid of thread blocks; each block solves one column at a time
// (the reference's column loop, rrtmg_lw_rad.f90:486-593) and owns one slot
// of an L2-resident scratch area.  One launch covers a batch of grids (nested
// grids, ensemble members) with their own column and layer counts: the batch
// columns are numbered grid after grid and each block walks them with stride
// gridDim.x.  Phases per column, separated by barriers:
//   1. inatm + setcoef (rrtmg_lw_rad.f90:598-924, rrtmg_lw_setcoef.f90:50-434):
//      one thread per layer, coefficients into shared memory; Planck
//      interpolation with one thread per (level, band); column sums for
//      pwvcm.  All threads also scan the McICA cloud fractions to mark cloudy
//      layers and cells (rtrnmc.f90:292-331) and to check the particle sizes
//      where cldprmc would stop (cldprmc.f90:178-266).  In the fused cloud
//      mode the block instead draws the column's 140 McICA random numbers
//      (mcica_subcol_gen_lw.f90:484-512 with icld 3, Mersenne twister seeded
//      seed0 + column) and marks cell (lay, g) cloudy iff cdf(g) >= 1 -
//      cldf(lay) (:650), with the cloud optical depth of each (layer, band)
//      computed once -- the values mcica_subcol_lw would have copied into
//      every sub-column of that band.
//   2. gas optics and cell transfer coefficients, band by band: a prologue
//      per (layer, band) builds the taumol term list (lw_gasoptics.cuh), then
//      one thread per (layer, g) cell evaluates taug, adds the aerosol depth
//      (rrtmg_lw_rad.f90:548-553), takes the Planck fraction and computes the
//      cell's layer transmittance and down/up sources exactly as rtrnmc's
//      down sweep does (rtrnmc.f90:350-455): clear-sky coefficients for every
//      cell and cloudy-layer coefficients where cldfmc /= 0.  They go to the
//      block's scratch slot.  Lookup-table entries exp_tbl/tfn_tbl/tau_tbl
//      (rrtmg_lw_init.f90:125-142) are evaluated at the quantised index.
//   3. rtrnmc sweeps, one thread per g-point: each layer is then an affine
//      update radiance*A + B (rtrnmc.f90:347-529); the clear-sky stream and
//      the surface-temperature derivatives follow with their own
//      coefficients.  Per-level g-point sums are weighted by
//      0.5*delwave*fluxfac and reduced across each warp in fp32.
//   4. fp64 epilogue: per-warp partial sums added in fp64, net fluxes and
//      heating rates heatfac*dF/dp in fp64 (rtrnmc.f90:566-592).
//
// Precision: gas optics and transfer in fp32; flux accumulation across warps
// error-free (two-sum) into fp64, net fluxes and the heating-rate step in
// fp64.  Outputs follow the reference's layout:
// uflx(icol, k+1) for k = 0..nlay, hr(icol, k+1) for k = 0..nlay-1.
#include <cuda_runtime.h>
#include <math.h>
#include <cmath>
#include <stdint.h>
#include <climits>

#include "lw_common.h"
#include "lw_solver.h"
#include "lw_gasoptics.cuh"
#include "lw_mt.cuh"

namespace gb {

constexpr int NSW = 5;  // warps of the g-point sweeps (140 lanes)
constexpr float BPADE = 1.0f / 0.278f;

// ------------------------------------------------------------------ band groups
// Bands are processed in groups of consecutive bands that share one prologue
// pass and one cell pass (kGroupFirst: first band of each group, then 17).
// Term lists of a group's bands sit side by side, TGROUP term slots per layer.
constexpr int kGroupFirst[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17};
constexpr int NGROUP = (int)(sizeof(kGroupFirst) / sizeof(int)) - 1;
constexpr int group_of(int b) {
  int gr = 0;
  while (kGroupFirst[gr + 1] <= b) ++gr;
  return gr;
}
constexpr int term_offset(int b) {  // first term slot of band b in its group
  int o = 0;
  for (int k = kGroupFirst[group_of(b)]; k < b; ++k) o += maxt(k);
  return o;
}
constexpr int group_terms(int gr) { return term_offset(kGroupFirst[gr + 1] - 1) + maxt(kGroupFirst[gr + 1] - 1); }
constexpr int max_group_terms() {
  int m = 0;
  for (int gr = 0; gr < NGROUP; ++gr) m = group_terms(gr) > m ? group_terms(gr) : m;
  return m;
}
constexpr int max_group_bands() {
  int m = 0;
  for (int gr = 0; gr < NGROUP; ++gr) m = kGroupFirst[gr + 1] - kGroupFirst[gr] > m ? kGroupFirst[gr + 1] - kGroupFirst[gr] : m;
  return m;
}
constexpr int TGROUP = max_group_terms();
constexpr int GBANDS = max_group_bands();
__constant__ int c_gfirst[17] = {
#define GB_G(i) (i <= NGROUP ? kGroupFirst[i] : 0)
    GB_G(0), GB_G(1), GB_G(2), GB_G(3), GB_G(4), GB_G(5), GB_G(6), GB_G(7), GB_G(8),
    GB_G(9), GB_G(10), GB_G(11), GB_G(12), GB_G(13), GB_G(14), GB_G(15), GB_G(16)};
#undef GB_G
__constant__ int c_toff[17] = {0, term_offset(1), term_offset(2), term_offset(3), term_offset(4), term_offset(5),
                               term_offset(6), term_offset(7), term_offset(8), term_offset(9), term_offset(10),
                               term_offset(11), term_offset(12), term_offset(13), term_offset(14), term_offset(15),
                               term_offset(16)};

// ------------------------------------------------------------------ shared memory layout
struct Smem {
  float* f;        // [NF][nl]   per-layer coefficients (phases 1-2)
  int* iv;         // [NI][nl]
  float2* terms;   // [TGROUP][nl] gas-optics terms of the current band group, term-major (phase 2)
  float* part;     // [NSW][nl+1][6] warp partial fluxes (region A, phases 3-4)
  float* taua;     // [16][nl]
  float* plk_lay;  // [16][nl]
  float* plk_lev;  // [16][nl+1]
  FracRec* frec;   // [GBANDS][nl] Planck-fraction records of the current band group
  int* cldlay;     // [nl]
  int* surok;      // [nl] 1: the layer's gas optics come from the learned model
  unsigned* cbits; // [nl][5] bit g set where cldfmcl == 1
  unsigned* fbits; // [nl][5] bit g set where cldfmcl is neither 0 nor 1
  float* frac1;    // [140] Planck fractions of the bottom layer (surface source)
  double* fnet;    // [nl+1][2] net fluxes (region A after part, phase 4)
  float* misc;     // [64]: secdiff[16], plankbnd[16], dplankbnd[16], semiss[16]
  float* scal;     // [4]
  int* iscal;      // [4]: laytrop, sum of lower-layer indices, error, column error
  double* cdf;     // [140] McICA draws of the column (fused cloud mode, phase 1; in the term area)
  uint32_t* mtlo;  // [141] Mersenne-twister state words (fused cloud mode, phase 1; in the term area)
  float* tcl;      // [nl][16] cloud optical depth per (layer, band) (fused cloud mode)
  // fused cloud mode, per layer: the McICA threshold 1 - cldf as double bits
  // (cdf >= it marks a cloudy cell), the layer's cloud water paths and radii
  // as floats, and flags: bit 0 ciwp /= 0, bit 1 clwp /= 0, bit 2
  // ciwp + clwp >= 1e-20, bits 8.. the code cldprmc's radius checks stop with
  long long* cthr; // [nl]
  float4* lcw;     // [nl] (ciwp, clwp, radice, radliq)
  int* lfl;        // [nl]
  float4* prow;    // [nl+1] Planck-table row and fraction of tlev and tlay per level (phase 1)
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Region A holds, by phase: the per-layer coefficients f/iv and the term
// lists (phases 1-2; the McICA draws of the fused cloud mode borrow the term
// area during phase 1), then the warp partial sums and net fluxes (3-4).  The
// learned-only kernel (lean) runs no taumol and has no term area.
__host__ __device__ inline size_t terms_offset(int nl) { return ((size_t)(NF + NI) * nl * 4 + 15) & ~size_t(15); }
__host__ __device__ inline size_t region_a(int nl, bool lean) {
  size_t terms = lean ? 0 : (size_t)nl * TGROUP * 8;
  const size_t draws = align16(GB_NGPT * 8) + align16((GB_NGPT + 1) * 4);
  size_t coef = terms_offset(nl) + (terms > draws ? terms : draws);
  size_t part = align16((size_t)NSW * (nl + 1) * 6 * 4) + (size_t)(nl + 1) * 2 * 8;
  return align16(coef > part ? coef : part);
}

__host__ __device__ inline size_t smem_bytes(int nl, bool lean) {
  size_t a = region_a(nl, lean);
  a += align16((size_t)nl * 16 * 4);         // taua
  a += align16((size_t)nl * 16 * 4);         // plk_lay
  a += align16((size_t)(nl + 1) * 16 * 4);   // plk_lev
  a += align16((size_t)GBANDS * nl * sizeof(FracRec));
  a += 2 * align16((size_t)nl * 4);
  a += 2 * align16((size_t)nl * 5 * 4);
  a += align16(GB_NGPT * 4);
  a += align16(64 * 4) + align16(4 * 4) + align16(4 * 4);
  a += align16((size_t)nl * 16 * 4);         // tcl
  a += align16((size_t)nl * 8) + align16((size_t)nl * 16) + align16((size_t)nl * 4);  // cthr, lcw, lfl
  a += align16((size_t)(nl + 1) * 16);                                                   // prow
  return a;
}

__device__ inline Smem carve(char* base, int nl, bool lean) {
  Smem s;
  char* p = base;
  s.f = (float*)p;
  s.iv = (int*)(p + (size_t)NF * nl * 4);
  s.terms = (float2*)(p + terms_offset(nl));
  s.cdf = (double*)(p + terms_offset(nl));
  s.mtlo = (uint32_t*)(p + terms_offset(nl) + align16(GB_NGPT * 8));
  s.part = (float*)p;
  s.fnet = (double*)(p + align16((size_t)NSW * (nl + 1) * 6 * 4));
  p += region_a(nl, lean);
  s.taua = (float*)p; p += align16((size_t)nl * 16 * 4);
  s.plk_lay = (float*)p; p += align16((size_t)nl * 16 * 4);
  s.plk_lev = (float*)p; p += align16((size_t)(nl + 1) * 16 * 4);
  s.frec = (FracRec*)p; p += align16((size_t)GBANDS * nl * sizeof(FracRec));
  s.cldlay = (int*)p; p += align16((size_t)nl * 4);
  s.surok = (int*)p; p += align16((size_t)nl * 4);
  s.cbits = (unsigned*)p; p += align16((size_t)nl * 5 * 4);
  s.fbits = (unsigned*)p; p += align16((size_t)nl * 5 * 4);
  s.frac1 = (float*)p; p += align16(GB_NGPT * 4);
  s.misc = (float*)p; p += align16(64 * 4);
  s.scal = (float*)p; p += align16(4 * 4);
  s.iscal = (int*)p; p += align16(4 * 4);
  s.tcl = (float*)p; p += align16((size_t)nl * 16 * 4);
  s.cthr = (long long*)p; p += align16((size_t)nl * 8);
  s.lcw = (float4*)p; p += align16((size_t)nl * 16);
  s.lfl = (int*)p; p += align16((size_t)nl * 4);
  s.prow = (float4*)p;
  return s;
}

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ double in2(const double* __restrict__ a, long long ld, long long icol, int k) {
  return __ldg(a + icol + ld * k);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp sums of four values per lane at once (a transposed butterfly, 6
// shuffles instead of 20): lane i returns the sum over the 32 lanes of v[i & 3].
__device__ __forceinline__ float reduce4(const float (&v)[4], int lane) {
  const unsigned F = 0xffffffffu;
  const bool hi = lane & 2;
  float k0 = hi ? v[2] : v[0], k1 = hi ? v[3] : v[1];
  const float s0 = hi ? v[0] : v[2], s1 = hi ? v[1] : v[3];
  k0 += __shfl_xor_sync(F, s0, 2);
  k1 += __shfl_xor_sync(F, s1, 2);
  const bool lo = lane & 1;
  float k = lo ? k1 : k0;
  const float sx = lo ? k0 : k1;
  k += __shfl_xor_sync(F, sx, 1);
  k += __shfl_xor_sync(F, k, 4);
  k += __shfl_xor_sync(F, k, 8);
  k += __shfl_xor_sync(F, k, 16);
  return k;
}

// exp_tbl/tfn_tbl/tau_tbl at the index the reference's lookup would pick
// (rrtmg_lw_rtrnmc.f90:385-388 with rrtmg_lw_init.f90:125-142)
struct TblEntry {
  float tau, trans, tfn;
};
__device__ __forceinline__ TblEntry tbl(float od) {
  float tblind = __fdividef(od, BPADE + od);
  int itr = (int)fmaf(10000.0f, tblind, 0.5f);
  itr = itr < 0 ? 0 : (itr > 10000 ? 10000 : itr);
  TblEntry e;
  if (itr == 0) {
    e.tau = 0.0f; e.trans = 1.0f; e.tfn = 0.0f;
  } else if (itr == 10000) {
    e.tau = 1.0e10f; e.trans = 1.0e-20f; e.tfn = 1.0f;
  } else {
    float t = (float)itr * 1.0e-4f;
    float tau = BPADE * __fdividef(t, 1.0f - t);
    float ex = __expf(-tau);
    ex = ex <= 1.0e-20f ? 1.0e-20f : ex;
    e.tau = tau;
    e.trans = ex;
    e.tfn = tau < 0.06f ? tau * (1.0f / 6.0f) : fmaf(-2.0f, __fdividef(1.0f, tau) - __fdividef(ex, 1.0f - ex), 1.0f);
  }
  return e;
}

__constant__ int c_maxt[17] = {0, maxt(1), maxt(2), maxt(3), maxt(4), maxt(5), maxt(6), maxt(7), maxt(8),
                               maxt(9), maxt(10), maxt(11), maxt(12), maxt(13), maxt(14), maxt(15), maxt(16)};
__constant__ int c_icb[16] = {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5};  // cldprmc.f90:133
// diffusivity-angle coefficients (rtrnmc.f90:236-247)
__constant__ float c_a0[16] = {1.66f, 1.55f, 1.58f, 1.66f, 1.54f, 1.454f, 1.89f, 1.33f, 1.668f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f};
__constant__ float c_a1[16] = {0.f, 0.25f, 0.22f, 0.f, 0.13f, 0.446f, -0.10f, 0.40f, -0.006f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
__constant__ float c_a2[16] = {0.f, -12.0f, -11.7f, 0.f, -0.72f, -0.243f, 0.19f, -0.062f, 0.414f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};

// cldprmc's optical depth ciwp*abscoice + clwp*abscoliq of one cell
// (cldprmc.f90:194-266; the radius bounds are checked in the pre-pass), from
// w = (ciwp, clwp, radice, radliq) converted to float and flags bit 0: ciwp
// /= 0, bit 1: clwp /= 0
__device__ __forceinline__ float cloud_tau_layer(const LwArgs& a, int band, const float* __restrict__ T, float4 w,
                                                 int flags) {
  float abscoice = 0.0f, abscoliq = 0.0f;
  if (flags & 1) {
    const float radice = w.z;
    if (a.iceflag == 0) {
      abscoice = T[c_T.absice0] + T[c_T.absice0 + 1] / radice;
    } else if (a.iceflag == 1) {
      int ib = c_icb[band];
      abscoice = T[c_T.absice1 + 2 * (ib - 1)] + T[c_T.absice1 + 1 + 2 * (ib - 1)] / radice;
    } else {
      float factor = (radice - 2.0f) / 3.0f;
      int nrow = a.iceflag == 2 ? 43 : 46;
      int index = clampi((int)factor, 1, nrow - 1);
      float fint = factor - (float)index;
      const float* t = T + (a.iceflag == 2 ? c_T.absice2 : c_T.absice3) + nrow * band;
      abscoice = t[index - 1] + fint * (t[index] - t[index - 1]);
    }
  }
  if (flags & 2) {
    if (a.liqflag == 0) {
      abscoliq = c_T.absliq0;
    } else {
      const float radliq = w.w;
      int index = clampi((int)(radliq - 1.5f), 1, 57);
      float fint = radliq - 1.5f - (float)index;
      const float* t = T + c_T.absliq1 + 58 * band;
      abscoliq = t[index - 1] + fint * (t[index] - t[index - 1]);
    }
  }
  return w.x * abscoice + w.y * abscoliq;
}

// McICA cloud optics of one cell: returns cldfmc and sets odcld/efcl
// (cldprmc.f90:178-266 then rtrnmc.f90:300-312; computed only where
// cldfmc == 1, the only cells whose optical depth rtrnmc reads).
__device__ __forceinline__ float cell_cloud(const LwArgs& a, const Smem& s, long long icol, int g, int lay,
                                            float secdiff_b, int band, const float* __restrict__ T, float& odcld,
                                            float& efcl) {
  const unsigned bit = 1u << (g & 31);
  const bool one = s.cbits[lay * 5 + (g >> 5)] & bit;
  odcld = 0.0f;
  efcl = 0.0f;
  if (a.cloud_mode == LW_CLOUD_FUSED) {  // sub-column clouds are 0 or 1; optical depth per (layer, band)
    if (!one) return 0.0f;
    odcld = secdiff_b * s.tcl[lay * 16 + band];
    efcl = 1.0f - __expf(-odcld);
    return 1.0f;
  }
  if (!one) {
    if (!(s.fbits[lay * 5 + (g >> 5)] & bit)) return 0.0f;
    // fractional cldfmc: enters the cloudy-layer formulas with zero cloud optical depth
    return (float)__ldg(a.cldfmcl + (long long)g + GB_NGPT * (icol + (long long)a.ld * lay));
  }
  long long o = (long long)g + GB_NGPT * (icol + (long long)a.ld * lay);
  const double ciwp = __ldg(a.ciwpmcl + o), clwp = __ldg(a.clwpmcl + o);
  // the optical depth from this cell's water paths and the layer's radii (as
  // floats in shared memory), or the caller's taucmcl
  float tauc;
  bool from_paths = a.inflag == 2 && ciwp + clwp >= 1.e-20;
  if (!from_paths) {
    const double tin = __ldg(a.taucmcl + o);
    const long long tb = __double_as_longlong(tin);
    from_paths = a.inflag == 2 && tb >= __double_as_longlong(1.0e-20) && tb <= 0x7FF0000000000000LL;
    tauc = (float)tin;
  }
  if (from_paths) {
    const int fl = ((__double_as_longlong(ciwp) << 1) != 0LL ? 1 : 0) | ((__double_as_longlong(clwp) << 1) != 0LL ? 2 : 0);
    const float4 r = s.lcw[lay];
    tauc = cloud_tau_layer(a, band, T, make_float4((float)ciwp, (float)clwp, r.z, r.w), fl);
  }
  odcld = secdiff_b * tauc;
  efcl = 1.0f - __expf(-odcld);
  return 1.0f;
}


__device__ __forceinline__ bool cell_is_cloudy(const Smem& s, int lay, int g) {
  const unsigned bit = 1u << (g & 31);
  return ((s.cbits[lay * 5 + (g >> 5)] | s.fbits[lay * 5 + (g >> 5)]) & bit) != 0u;
}

// Transfer coefficients of one cell (rtrnmc.f90:350-455 rearranged): the
// clear-sky stream uses radiance*T + S (S = bbd*atrans down, bbugas*atrans
// up); a cloudy cell uses radiance*A + Bd (down) / + Bu (up) and scales the
// surface-temperature derivative by D.
struct CellCoef {
  float4 clr;  // T, Sd, Su, 0
  float4 cld;  // A, Bd, Bu, D
};
__device__ __forceinline__ CellCoef cell_coef(bool cloudy, float odepth, float odcld, float efcl, float cldf,
                                              float plfrac, float blay, float dplankup, float dplankdn) {
  const float rec_6 = 0.166667f;
  CellCoef r;
  float atrans, bbd, bbu, tau_q;
  if (odepth <= 0.06f) {
    atrans = fmaf(-0.5f * odepth, odepth, odepth);
    float o = rec_6 * odepth;
    bbd = plfrac * fmaf(dplankdn, o, blay);
    bbu = plfrac * fmaf(dplankup, o, blay);
    tau_q = odepth;
  } else {
    TblEntry e = tbl(odepth);
    atrans = 1.0f - e.trans;
    bbd = plfrac * fmaf(e.tfn, dplankdn, blay);
    bbu = plfrac * fmaf(e.tfn, dplankup, blay);
    tau_q = e.tau;
  }
  const float gsd = bbd * atrans, gsu = bbu * atrans;
  r.clr = make_float4(1.0f - atrans, gsd, gsu, 0.0f);
  if (cloudy) {
    float atot, bbdtot, bbutot;
    float odtot = odepth + odcld;
    if (odtot < 0.06f) {
      atot = fmaf(-0.5f * odtot, odtot, odtot);
      float o = rec_6 * odtot;
      bbdtot = plfrac * fmaf(dplankdn, o, blay);
      bbutot = plfrac * fmaf(dplankup, o, blay);
    } else {
      // odepth <= 0.06: table at odepth + odcld; otherwise at tau_tbl(itgas) + odcld
      TblEntry et = tbl((odepth <= 0.06f ? odepth : tau_q) + odcld);
      atot = 1.0f - et.trans;
      bbdtot = plfrac * fmaf(et.tfn, dplankdn, blay);
      bbutot = plfrac * fmaf(et.tfn, dplankup, blay);
    }
    float A = 1.0f - fmaf(efcl, 1.0f - atrans, atrans);
    float Bd = fmaf(cldf, fmaf(bbdtot, atot, -gsd), gsd);
    float Bu = fmaf(cldf, fmaf(bbutot, atot, -gsu), gsu);
    float D = fmaf(cldf, 1.0f - atot, (1.0f - cldf) * (1.0f - atrans));
    r.cld = make_float4(A, Bd, Bu, D);
  } else {
    r.cld = r.clr;
  }
  return r;
}

// Prologue of band b for one layer: the band-specific per-layer code
// (lw_gasoptics.cuh) writing the layer's terms and Planck-fraction record.
template <int b>
__device__ __forceinline__ void band_prologue(const Smem& s, int nl, int lay, bool lower, int slot) {
  Cell c{s.f, s.iv, nl, lay};
  Terms t{s.terms + (size_t)c_toff[b] * nl + lay, nl, 0};
  FracRec r = prologue<b>(c, lower, t);
  t.pad(maxt(b), c_T.band[b - 1].sr);
  s.frec[slot * nl + lay] = r;
}

__device__ __noinline__ void prologue_dispatch(int b, const Smem& s, int nl, int lay, bool lower, int slot) {
  switch (b) {
    case 1: band_prologue<1>(s, nl, lay, lower, slot); break;
    case 2: band_prologue<2>(s, nl, lay, lower, slot); break;
    case 3: band_prologue<3>(s, nl, lay, lower, slot); break;
    case 4: band_prologue<4>(s, nl, lay, lower, slot); break;
    case 5: band_prologue<5>(s, nl, lay, lower, slot); break;
    case 6: band_prologue<6>(s, nl, lay, lower, slot); break;
    case 7: band_prologue<7>(s, nl, lay, lower, slot); break;
    case 8: band_prologue<8>(s, nl, lay, lower, slot); break;
    case 9: band_prologue<9>(s, nl, lay, lower, slot); break;
    case 10: band_prologue<10>(s, nl, lay, lower, slot); break;
    case 11: band_prologue<11>(s, nl, lay, lower, slot); break;
    case 12: band_prologue<12>(s, nl, lay, lower, slot); break;
    case 13: band_prologue<13>(s, nl, lay, lower, slot); break;
    case 14: band_prologue<14>(s, nl, lay, lower, slot); break;
    case 15: band_prologue<15>(s, nl, lay, lower, slot); break;
    default: band_prologue<16>(s, nl, lay, lower, slot); break;
  }
}

// Scratch slot of a column (2*nl*140 float4): the clear-sky coefficients as
// three float planes [nl][140] -- T, Sd, Su -- from the start (the downward
// sweep reads T and Sd, the upward one T and Su: 8 bytes a cell each), then
// from float4 offset nl*140 the cloudy-layer coefficients float4 [nl][140]
// (A, Bd, Bu, D), written and read only for cloudy cells.
__device__ __forceinline__ void put_coef(float4* __restrict__ scr, int nl, int lay, int g, const CellCoef& cc,
                                         bool cloudy) {
  const int i = lay * GB_NGPT + g;
  float* pl = reinterpret_cast<float*>(scr);
  pl[i] = cc.clr.x;
  pl[nl * GB_NGPT + i] = cc.clr.y;
  pl[2 * nl * GB_NGPT + i] = cc.clr.z;
  if (cloudy) scr[nl * GB_NGPT + i] = cc.cld;
}

// All (band, layer) prologues of group gr, spread over the block's threads.
template <int NT>
__device__ __forceinline__ void group_prologues(int gr, const Smem& s, int nl, int laytrop) {
  const int b0 = c_gfirst[gr], nb = c_gfirst[gr + 1] - b0;
  for (int it = threadIdx.x; it < nb * nl; it += NT) {
    const int slot = it / nl, lay = it - slot * nl;
    if (!s.surok[lay]) prologue_dispatch(b0 + slot, s, nl, lay, lay < laytrop, slot);
  }
}

// One thread per (band, layer, g) cell of group gr: optical depth, Planck
// fraction and transfer coefficients into the scratch slot.
template <int NT>
__device__ __forceinline__ void group_cells(int gr, const LwArgs& a, const Smem& s, int nl, int laytrop,
                                            const float* __restrict__ T, long long icol, float4* __restrict__ scr) {
  const int b0 = c_gfirst[gr], b1 = c_gfirst[gr + 1];
  int ncell = 0;
  for (int b = b0; b < b1; ++b) ncell += nl * c_T.band[b - 1].ng;
  const bool clouds = a.icld >= 1;
  for (int cell = threadIdx.x; cell < ncell; cell += NT) {
    int b = b0, c = cell, NG = c_T.band[b0 - 1].ng;
    while (c >= nl * NG) {
      c -= nl * NG;
      ++b;
      NG = c_T.band[b - 1].ng;
    }
    const int slot = b - b0;
    const int lay = (int)(((float)c + 0.5f) * __frcp_rn((float)NG)), gi = c - lay * NG, g = c_T.band[b - 1].g0 + gi;
    float taut, plfrac;
    if (s.surok[lay]) {  // learned gas optics
      const long long o = (icol * nl + lay) * GB_NGPT + g;
      taut = __half2float(__ldg(a.sur_tau + o)) + s.taua[(b - 1) * nl + lay];
      plfrac = __half2float(__ldg(a.sur_frac + o));
    } else {
      const int M = c_maxt[b];
      const float2* tp = s.terms + (size_t)c_toff[b] * nl + lay;
      const float* Tg = T + gi;
      float acc = 0.0f;
      for (int k = 0; k < M; ++k) {
        const float2 w = tp[k * nl];
        acc = fmaf(w.x, __ldg(Tg + __float_as_int(w.y)), acc);
      }
      if ((b == 4 || b == 7) && lay >= laytrop) acc *= gscale(b, gi);
      taut = acc + s.taua[(b - 1) * nl + lay];
      const FracRec fr = s.frec[slot * nl + lay];
      const float* fp = T + fr.off + gi;
      const float f0 = __ldg(fp);
      plfrac = fmaf(fr.fpl, __ldg(fp + NG) - f0, f0);
    }
    if (lay == 0) s.frac1[g] = plfrac;
    if (a.dbg_taut) {
      a.dbg_taut[(icol * nl + lay) * GB_NGPT + g] = taut;
      a.dbg_fracs[(icol * nl + lay) * GB_NGPT + g] = plfrac;
    }
    const float secdiff = s.misc[b - 1];
    const float blay = s.plk_lay[(b - 1) * nl + lay];
    const float dplankup = s.plk_lev[(b - 1) * (nl + 1) + lay + 1] - blay;
    const float dplankdn = s.plk_lev[(b - 1) * (nl + 1) + lay] - blay;
    const float odepth = fmaxf(secdiff * taut, 0.0f);
    bool cloudy = false;
    float odcld = 0.0f, efcl = 0.0f, cldf = 0.0f;
    if (clouds && s.cldlay[lay]) {
      cldf = cell_cloud(a, s, icol, g, lay, secdiff, b - 1, T, odcld, efcl);
      cloudy = cell_is_cloudy(s, lay, g);
    }
    CellCoef cc = cell_coef(cloudy, odepth, odcld, efcl, cldf, plfrac, blay, dplankup, dplankdn);
    put_coef(scr, nl, lay, g, cc, cloudy);
  }
}

// Every layer with learned gas optics: one thread per (layer, g) cell of the
// whole column, no band passes (cells of group_cells without the gather).
template <int NT>
__device__ __forceinline__ void learned_cells(const LwArgs& a, const Smem& s, int nl, const float* __restrict__ T,
                                              long long icol, float4* __restrict__ scr) {
  const bool clouds = a.icld >= 1;
  const __half* __restrict__ st = a.sur_tau + icol * nl * GB_NGPT;
  const __half* __restrict__ sf = a.sur_frac + icol * nl * GB_NGPT;
  for (int cell = threadIdx.x; cell < nl * GB_NGPT; cell += NT) {
    const int lay = (int)(((float)cell + 0.5f) * (1.0f / GB_NGPT)), g = cell - lay * GB_NGPT;
    const int b = c_T.ngb[g] - 1;
    const float taut = __half2float(__ldg(st + cell)) + s.taua[b * nl + lay];
    const float plfrac = __half2float(__ldg(sf + cell));
    if (lay == 0) s.frac1[g] = plfrac;
    if (a.dbg_taut) {
      a.dbg_taut[(icol * nl + lay) * GB_NGPT + g] = taut;
      a.dbg_fracs[(icol * nl + lay) * GB_NGPT + g] = plfrac;
    }
    const float secdiff = s.misc[b];
    const float blay = s.plk_lay[b * nl + lay];
    const float dplankup = s.plk_lev[b * (nl + 1) + lay + 1] - blay;
    const float dplankdn = s.plk_lev[b * (nl + 1) + lay] - blay;
    const float odepth = fmaxf(secdiff * taut, 0.0f);
    bool cloudy = false;
    float odcld = 0.0f, efcl = 0.0f, cldf = 0.0f;
    if (clouds && s.cldlay[lay]) {
      cldf = cell_cloud(a, s, icol, g, lay, secdiff, b, T, odcld, efcl);
      cloudy = cell_is_cloudy(s, lay, g);
    }
    CellCoef cc = cell_coef(cloudy, odepth, odcld, efcl, cldf, plfrac, blay, dplankup, dplankdn);
    put_coef(scr, nl, lay, g, cc, cloudy);
  }
}

// ------------------------------------------------------------------ one column
// LEAN: the learned-only flavour -- a column with any layer off the network
// is not solved (returns false, the same answer in every thread) and the
// taumol code is not compiled in.
template <int NT, bool LEAN>
__device__ __forceinline__ bool solve_column(const LwArgs& a, long long icol, char* smem_raw,
                                             float4* __restrict__ scr, const float* __restrict__ T) {
  constexpr int NWARP = NT / 32;
  const int nl = a.nlay;
  const Smem s = carve(smem_raw, nl, LEAN);
  const int tid = threadIdx.x;
  const bool fused = a.cloud_mode == LW_CLOUD_FUSED;
  {
    // fused clouds: the column's 140 draws, made beforehand by a parallel
    // kernel or else here by one thread of the last warp
    if (fused && a.icld >= 1) {
      if (a.draws) {
        for (int g = tid; g < GB_NGPT; g += NT) s.cdf[g] = __ldg(a.draws + icol * GB_NGPT + g);
      } else if (tid == NT - 1) {
        gbmt::first_reals(a.seed0 + (unsigned)icol, GB_NGPT, s.mtlo, s.cdf, 1);
      }
    }
    if (tid < 4) {
      s.scal[tid] = 0.0f;
      s.iscal[tid] = 0;
    }
    int offnet = 0;
    for (int l = tid; l < nl; l += NT) {
      s.cldlay[l] = 0;
      s.surok[l] = a.sur_flag ? (int)__ldg(a.sur_flag + icol * nl + l) : 0;
      offnet |= !s.surok[l];
    }
    for (int l = tid; l < nl * 5; l += NT) s.cbits[l] = s.fbits[l] = 0u;
    if (LEAN) {
      if (__syncthreads_or(offnet)) return false;
    } else {
      __syncthreads();
    }

    // ---------------- phase 1: inatm + setcoef, one thread per layer
    const float stpfac = 296.0f / 1013.0f;
    const float amd = 28.9660f, amw = 18.0160f;
    int my_bad = 0;
    for (int lay = tid; lay < nl; lay += NT) {
      double pd = in2(a.play, a.ld, icol, lay);
      float pavel = (float)pd;
      float tavel = (float)in2(a.tlay, a.ld, icol, lay);
      double dpz = in2(a.plev, a.ld, icol, lay) - in2(a.plev, a.ld, icol, lay + 1);
      float w1 = (float)in2(a.h2ovmr, a.ld, icol, lay);
      if (LEAN || s.surok[lay]) {
        // learned gas optics: only what pwvcm and the checks need (inatm :807-870)
        const float amm = (1.0f - w1) * amd + w1 * amw;
        const float coldry = (float)dpz * 1.e3f * (float)c_T.avogad / (1.e2f * (float)c_T.grav * amm * (1.0f + w1));
        s.f[F_COLDRY * nl + lay] = coldry;
        s.f[F_COLH2O * nl + lay] = 1.e-20f * (coldry * w1);  // as colh2o = 1e-20 * wk1 below
        if (!(pavel > 0.0f) || !(tavel > 0.0f) || !isfinite(pavel) || !isfinite(tavel)) my_bad = 1;
        const float plog = __logf(pavel);
        bool lower = plog > 4.56f;
        if (fabsf(plog - 4.56f) < 1.0e-4f) lower = log(pd) > 4.56;
        if (lower) {
          atomicAdd(&s.iscal[0], 1);
          atomicAdd(&s.iscal[1], lay + 1);
        }
        continue;
      }
      float w2 = (float)in2(a.co2vmr, a.ld, icol, lay);
      float w3 = (float)in2(a.o3vmr, a.ld, icol, lay);
      float w4 = (float)in2(a.n2ovmr, a.ld, icol, lay);
      float w6 = (float)in2(a.ch4vmr, a.ld, icol, lay);
      float w7 = (float)in2(a.o2vmr, a.ld, icol, lay);
      float amm = (1.0f - w1) * amd + w1 * amw;
      float coldry = (float)dpz * 1.e3f * (float)c_T.avogad / (1.e2f * (float)c_T.grav * amm * (1.0f + w1));
      float summol = w2 + w3 + w4 + 0.0f + w6 + w7;
      float wbrodl = coldry * (1.0f - summol);
      float wk1 = coldry * w1, wk2 = coldry * w2, wk3 = coldry * w3, wk4 = coldry * w4, wk6 = coldry * w6,
            wk7 = coldry * w7;
      float* F = s.f;
      auto put = [&](int k, float v) { F[k * nl + lay] = v; };
      put(F_COLDRY, coldry);
      put(F_PAVEL, pavel);
      put(F_WX1, coldry * (float)in2(a.ccl4vmr, a.ld, icol, lay) * 1.e-20f);
      put(F_WX2, coldry * (float)in2(a.cfc11vmr, a.ld, icol, lay) * 1.e-20f);
      put(F_WX3, coldry * (float)in2(a.cfc12vmr, a.ld, icol, lay) * 1.e-20f);
      put(F_WX4, coldry * (float)in2(a.cfc22vmr, a.ld, icol, lay) * 1.e-20f);
      if (!(pavel > 0.0f) || !(tavel > 0.0f) || !isfinite(pavel) || !isfinite(tavel)) my_bad = 1;
      // setcoef (rrtmg_lw_setcoef.f90:275-430)
      float plog = __logf(pavel);
      bool lower = plog > 4.56f;
      if (fabsf(plog - 4.56f) < 1.0e-4f) lower = log(pd) > 4.56;  // decide the regime in fp64 near the switch
      int jp = clampi((int)(36.0f - 5.0f * (plog + 0.04f)), 1, 58);
      jp = lower ? (jp > 12 ? 12 : jp) : (jp < 13 ? 13 : jp);
      float fp = 5.0f * (c_T.preflog[jp - 1] - plog);
      float dt0 = (tavel - c_T.tref[jp - 1]) / 15.0f;
      int jt = clampi((int)(3.0f + dt0), 1, 4);
      float ft = dt0 - (float)(jt - 3);
      float dt1 = (tavel - c_T.tref[jp]) / 15.0f;
      int jt1 = clampi((int)(3.0f + dt1), 1, 4);
      float ft1 = dt1 - (float)(jt1 - 3);
      float water = wk1 / coldry;
      float scalefac = pavel * stpfac / tavel;
      float forfac = scalefac / (1.0f + water), forfrac, selffrac = 0.0f;
      int indfor, indself = 1;
      if (lower) {
        float factor = (332.0f - tavel) / 36.0f;
        indfor = min(2, max(1, (int)factor));
        forfrac = factor - (float)indfor;
        factor = (tavel - 188.0f) / 7.2f;
        indself = min(9, max(1, (int)factor - 7));
        selffrac = factor - (float)(indself + 7);
      } else {
        float factor = (tavel - 188.0f) / 36.0f;
        indfor = 3;
        forfrac = factor - 1.0f;
      }
      float selffac = water * forfac;
      float scaleminor = pavel / tavel;
      float scaleminorn2 = scaleminor * (wbrodl / (coldry + wk1));
      float factor = (tavel - 180.8f) / 7.2f;
      int indminor = min(18, max(1, (int)factor));
      float minorfrac = factor - (float)indminor;
      float colh2o = 1.e-20f * wk1;
      float colco2 = 1.e-20f * wk2, colo3 = 1.e-20f * wk3, coln2o = 1.e-20f * wk4, colco = 0.0f;
      float colch4 = 1.e-20f * wk6, colo2 = 1.e-20f * wk7;
      if (colco2 == 0.0f) colco2 = 1.e-32f * coldry;
      if (colo3 == 0.0f) colo3 = 1.e-32f * coldry;
      if (coln2o == 0.0f) coln2o = 1.e-32f * coldry;
      if (colco == 0.0f) colco = 1.e-32f * coldry;
      if (colch4 == 0.0f) colch4 = 1.e-32f * coldry;
      float compfp = 1.0f - fp;
      put(F_FAC10, compfp * ft);
      put(F_FAC00, compfp * (1.0f - ft));
      put(F_FAC11, fp * ft1);
      put(F_FAC01, fp * (1.0f - ft1));
      put(F_COLH2O, colh2o); put(F_COLCO2, colco2); put(F_COLO3, colo3); put(F_COLN2O, coln2o);
      put(F_COLCO, colco); put(F_COLCH4, colch4); put(F_COLO2, colo2); put(F_COLBRD, 1.e-20f * wbrodl);
      put(F_SELFFAC, colh2o * selffac); put(F_SELFFRAC, selffrac);
      put(F_FORFAC, colh2o * forfac); put(F_FORFRAC, forfrac);
      put(F_MINORFRAC, minorfrac); put(F_SCALEMINOR, scaleminor); put(F_SCALEMINORN2, scaleminorn2);
      int* IV = s.iv;
      IV[I_JP * nl + lay] = jp; IV[I_JT * nl + lay] = jt; IV[I_JT1 * nl + lay] = jt1;
      IV[I_INDSELF * nl + lay] = indself; IV[I_INDFOR * nl + lay] = indfor; IV[I_INDMINOR * nl + lay] = indminor;
      // lower layers must form the prefix 0..laytrop-1
      if (lower) {
        atomicAdd(&s.iscal[0], 1);        // laytrop
        atomicAdd(&s.iscal[1], lay + 1);  // sum of 1-based indices of lower layers
      }
    }
    // aerosol optical depths (rrtmg_lw_rad.f90:548-553), all threads
    for (int it = tid; it < 16 * nl; it += NT) {
      const int ib = it / nl, lay = it - ib * nl;
      s.taua[it] = (float)__ldg(a.tauaer + icol + (long long)a.ld * (lay + (long long)nl * ib));
    }
    // Planck interpolation per (level, band) (setcoef.f90:173-269, istart = 1):
    // table row and fraction once per level (one fp64 conversion each), then
    // one thread per (level, band)
    for (int lev = tid; lev <= nl; lev += NT) {
      const float tz = (float)in2(a.tlev, a.ld, icol, lev);
      const int ind = clampi((int)(tz - 159.0f), 1, 180);
      float4 r = make_float4(__int_as_float(ind), tz - 159.0f - (float)ind, 0.0f, 0.0f);
      if (lev < nl) {
        const float tl = (float)in2(a.tlay, a.ld, icol, lev);
        const int il = clampi((int)(tl - 159.0f), 1, 180);
        r.z = __int_as_float(il);
        r.w = tl - 159.0f - (float)il;
      }
      s.prow[lev] = r;
    }
    __syncthreads();
    for (int it = tid; it < (nl + 1) * 16; it += NT) {
      int lev = it >> 4, ib = it & 15;
      const float* tp = T + c_T.totplnk + ib * 181;
      const float4 r = s.prow[lev];
      const int ind = __float_as_int(r.x);
      s.plk_lev[ib * (nl + 1) + lev] = tp[ind - 1] + r.y * (tp[ind] - tp[ind - 1]);
      if (lev < nl) {
        const int il = __float_as_int(r.z);
        s.plk_lay[ib * nl + lev] = tp[il - 1] + r.w * (tp[il] - tp[il - 1]);
      }
    }
    if (tid < 16) {
      float tb = (float)__ldg(a.tsfc + icol);
      int ind = clampi((int)(tb - 159.0f), 1, 180);
      float fr = tb - 159.0f - (float)ind;
      float se = (float)__ldg(a.emis + icol + (long long)a.ld * tid);
      const float* tp = T + c_T.totplnk + tid * 181;
      const float* td = T + c_T.totplnkderiv + tid * 181;
      s.misc[16 + tid] = se * (tp[ind - 1] + fr * (tp[ind] - tp[ind - 1]));
      s.misc[32 + tid] = se * (td[ind - 1] + fr * (td[ind] - td[ind - 1]));
      s.misc[48 + tid] = se;
    }
    // McICA pre-pass over every (layer, g) cell: cloudy layers, the per-cell
    // "cldfmc == 1" / "cldfmc neither 0 nor 1" bits the later phases use to
    // skip loads, and cldprmc's STOP conditions.
    if (a.icld >= 1 && fused) {
      // per layer, once: the McICA threshold and the layer's cloud
      // quantities (fp64 comparisons here rather than per cell or band)
      for (int lay = tid; lay < nl; lay += NT) {
        double cf = in2(a.cldfrac, a.ld, icol, lay);
        cf = cf < 1.0e-20 ? 0.0 : cf;  // mcica_subcol_gen_lw.f90:463-470
        // cdf >= 1 - cf, compared on the bit patterns (cdf is in [0, 1], so
        // for a threshold >= 0 the integer order is the floating-point order);
        // a negative threshold takes every cell, a NaN none
        const double thr = 1.0 - cf;
        s.cthr[lay] = thr < 0.0 ? LLONG_MIN : (thr == thr ? __double_as_longlong(thr) : LLONG_MAX);
        const double ciwp = in2(a.ciwp, a.ld, icol, lay), clwp = in2(a.clwp, a.ld, icol, lay);
        const double rice = in2(a.reicmcl, a.ld, icol, lay), rliq = in2(a.relqmcl, a.ld, icol, lay);
        int fl = (ciwp != 0.0 ? 1 : 0) | (clwp != 0.0 ? 2 : 0) | (ciwp + clwp >= 1.e-20 ? 4 : 0);
        // the code cldprmc.f90:217-266 stops with for this layer's radii (inflag 2)
        int e = 0;
        if (ciwp != 0.0) {
          if (a.iceflag == 0 && rice < 10.0) e = GB_COL_ICE_SMALL;
          if (a.iceflag == 1 && (rice < 13.0 || rice > 130.0)) e = GB_COL_ICE_BOUNDS;
          if (a.iceflag == 2 && (rice < 5.0 || rice > 131.0)) e = GB_COL_ICE_BOUNDS;
          if (a.iceflag == 3 && (rice < 5.0 || rice > 140.0)) e = GB_COL_DGE_BOUNDS;
        }
        if (clwp != 0.0 && a.liqflag == 1 && (rliq < 2.5 || rliq > 60.0)) e = GB_COL_LIQ_BOUNDS;
        s.lfl[lay] = fl | (e << 8);
        s.lcw[lay] = make_float4((float)ciwp, (float)clwp, (float)rice, (float)rliq);
      }
      __syncthreads();  // draws and layer data ready
      // cloudy cells: cdf(g) >= 1 - cldf(lay) (mcica_subcol_gen_lw.f90:650), one warp per layer
      const int warp = tid >> 5, lane = tid & 31;
      const long long* cdfb = reinterpret_cast<const long long*>(s.cdf);
      for (int lay = warp; lay < nl; lay += NWARP) {
        const long long tb = s.cthr[lay];
        unsigned any = 0u;
#pragma unroll
        for (int w = 0; w < 5; ++w) {
          const int g = w * 32 + lane;
          const bool cl = g < GB_NGPT && cdfb[g] >= tb;
          const unsigned m = __ballot_sync(0xffffffffu, cl);
          if (lane == 0) s.cbits[lay * 5 + w] = m;
          any |= m;
        }
        if (lane == 0) s.cldlay[lay] = any != 0u;
      }
      __syncthreads();
      // cloud optical depth per (layer, band) where the band has a cloudy
      // sub-column (the values cldprmc computes for every such cell), and
      // cldprmc's STOP conditions
      const long long kMin = __double_as_longlong(1.0e-20), kInf = 0x7FF0000000000000LL;
      int err = 0;
      for (int it = tid; it < nl * 16; it += NT) {
        const int lay = it >> 4, band = it & 15;
        if (!s.cldlay[lay]) continue;
        const int g0 = c_T.band[band].g0, ng = c_T.band[band].ng;
        bool any = false;
        for (int g = g0; g < g0 + ng; ++g) any |= (s.cbits[lay * 5 + (g >> 5)] >> (g & 31)) & 1u;
        if (!any) continue;
        const double tin = __ldg(a.tauc + band + 16 * (icol + a.ld * lay));
        const long long tinb = __double_as_longlong(tin);
        const bool tin_ok = tinb >= kMin && tinb <= kInf;  // tin >= 1e-20
        const int fl = s.lfl[lay];
        const bool cond = (fl & 4) || tin_ok;
        s.tcl[lay * 16 + band] = a.inflag == 2 && cond ? cloud_tau_layer(a, band, T, s.lcw[lay], fl) : (float)tin;
        if (cond) {
          if (a.inflag == 1) err = GB_COL_INFLAG1;
          if (a.inflag == 2 && (fl >> 8)) err = fl >> 8;
        }
      }
      if (err) atomicMax(&s.iscal[2], err);
    } else if (a.icld >= 1) {
      // per layer, once: the particle radii as floats and the codes cldprmc's
      // radius checks stop with (cldprmc.f90:217-266): bits 0-7 ice, 8-15 liquid
      for (int lay = tid; lay < nl; lay += NT) {
        const double rice = in2(a.reicmcl, a.ld, icol, lay), rliq = in2(a.relqmcl, a.ld, icol, lay);
        int ei = 0;
        if (a.iceflag == 0 && rice < 10.0) ei = GB_COL_ICE_SMALL;
        if (a.iceflag == 1 && (rice < 13.0 || rice > 130.0)) ei = GB_COL_ICE_BOUNDS;
        if (a.iceflag == 2 && (rice < 5.0 || rice > 131.0)) ei = GB_COL_ICE_BOUNDS;
        if (a.iceflag == 3 && (rice < 5.0 || rice > 140.0)) ei = GB_COL_DGE_BOUNDS;
        const int el = a.liqflag == 1 && (rliq < 2.5 || rliq > 60.0) ? GB_COL_LIQ_BOUNDS : 0;
        s.lfl[lay] = ei | (el << 8);
        s.lcw[lay] = make_float4(0.0f, 0.0f, (float)rice, (float)rliq);
      }
      __syncthreads();
      // one warp per layer: the layer's 140 cldfmcl values tested on their bit
      // patterns (no fp64 pipe): == 1, /= 0, >= 1e-20
      const int warp = tid >> 5, lane = tid & 31;
      const long long kOne = 0x3FF0000000000000LL, kInf = 0x7FF0000000000000LL;
      const long long kMin = __double_as_longlong(1.0e-20);
      int err = 0;
      for (int lay = warp; lay < nl; lay += NWARP) {
        const long long base = GB_NGPT * (icol + (long long)a.ld * lay);
        long long cb[5];
#pragma unroll
        for (int w = 0; w < 5; ++w) {
          const int g = w * 32 + lane;
          cb[w] = g < GB_NGPT ? __double_as_longlong(__ldg(a.cldfmcl + base + g)) : 0LL;
        }
        unsigned any = 0u;
#pragma unroll
        for (int w = 0; w < 5; ++w) {
          const bool one = cb[w] == kOne;
          const bool frac = !one && (cb[w] << 1) != 0LL;  // neither +-0 nor 1 (NaN included, as /= 0 is)
          const unsigned m1 = __ballot_sync(0xffffffffu, one), mf = __ballot_sync(0xffffffffu, frac);
          if (lane == 0) {
            s.cbits[lay * 5 + w] = m1;
            s.fbits[lay * 5 + w] = mf;
          }
          any |= m1;
          if (cb[w] >= kMin && cb[w] <= kInf) {  // cldfmc >= cldmin (cldprmc.f90:178)
            const long long o = base + w * 32 + lane;
            const double ciwp = __ldg(a.ciwpmcl + o), clwp = __ldg(a.clwpmcl + o);
            const long long tb = __double_as_longlong(__ldg(a.taucmcl + o));
            if (ciwp + clwp >= 1.e-20 || (tb >= kMin && tb <= kInf)) {
              if (a.inflag == 1) err = GB_COL_INFLAG1;
              if (a.inflag == 2) {
                const int e = s.lfl[lay];
                if ((__double_as_longlong(ciwp) << 1) != 0LL && (e & 0xff)) err = e & 0xff;  // ciwp /= 0
                if ((__double_as_longlong(clwp) << 1) != 0LL && (e >> 8)) err = e >> 8;      // clwp /= 0
              }
            }
          }
        }
        if (lane == 0) s.cldlay[lay] = any != 0u;
      }
      if (err) atomicMax(&s.iscal[2], err);
    }
    // learned gas optics for every layer of this column: one pass over all cells
    const bool all_learned = LEAN || (a.sur_flag != nullptr && !__syncthreads_or(offnet));
    int anybad = __syncthreads_or(my_bad);
    const int laytrop = s.iscal[0];
    if (tid < 32) {
      if (tid == 0) {
        int err = s.iscal[2];
        // sum of 1-based indices of lower layers equals laytrop*(laytrop+1)/2 iff they form a prefix
        if (s.iscal[1] != laytrop * (laytrop + 1) / 2) err = GB_COL_LAYTROP;
        if (anybad) err = GB_COL_BADVAL;
        s.iscal[3] = err;
        if (err) {
          if (a.col_err) a.col_err[icol] = err;
          atomicMax(a.err_flag, err);
        } else if (a.col_err) {
          a.col_err[icol] = 0;
        }
      }
      // pwvcm (inatm :859-870; a fixed-order warp sum over layers) and
      // secdiff (rtrnmc.f90:258-266), one band per lane
      float amttl = 0.0f, wvttl = 0.0f;
      for (int l = tid; l < nl; l += 32) {
        const float wk1 = s.f[F_COLH2O * nl + l] * 1.e20f;
        amttl += s.f[F_COLDRY * nl + l] + wk1;
        wvttl += wk1;
      }
      amttl = __shfl_sync(0xffffffffu, warp_sum(amttl), 0);
      wvttl = __shfl_sync(0xffffffffu, warp_sum(wvttl), 0);
      if (tid < 16) {
        const int ib = tid;
        const float wvsh = (amw * wvttl) / (amd * amttl);
        const float pz0 = (float)in2(a.plev, a.ld, icol, 0);
        const float pwvcm = wvsh * (1.e3f * pz0) / (1.e2f * (float)c_T.grav);
        float sd = 1.66f;
        if (!(ib == 0 || ib == 3 || ib >= 9)) {
          sd = c_a0[ib] + c_a1[ib] * __expf(c_a2[ib] * pwvcm);
          sd = fminf(fmaxf(sd, 1.50f), 1.80f);
        }
        s.misc[ib] = sd;
      }
    }
    __syncthreads();
    // ---------------- phase 2: gas optics and cell coefficients, band by band
    if (all_learned) {
      learned_cells<NT>(a, s, nl, T, icol, scr);
      __syncthreads();
    } else {  // taumol for every layer, or for the layers outside the network's range
      for (int gr = 0; gr < NGROUP; ++gr) {
        group_prologues<NT>(gr, s, nl, laytrop);
        __syncthreads();
        group_cells<NT>(gr, a, s, nl, laytrop, T, icol, scr);
        __syncthreads();
      }
    }

    // ---------------- phase 3: sweeps, one thread per g-point
    if (tid < NSW * 32) {
      const int warp = tid >> 5, lane = tid & 31;
      const bool active = tid < GB_NGPT;
      const int g = active ? tid : GB_NGPT - 1;
      const int band = c_T.ngb[g] - 1;
      const float wgt = active ? (float)(0.5 * (double)c_T.delwave[band] * c_T.fluxfac) : 0.0f;
      const bool idrv = a.idrv == 1;
      const bool clouds = a.icld >= 1;
      float* part = s.part + warp * (nl + 1) * 6;  // this warp's [nl+1][6] partial sums
      // Levels go in blocks of four: the block's scratch loads are issued
      // together and each stream's four level sums take one reduce4.
      // downward (rtrnmc.f90:347-455): total stream and clear-sky stream
      float radld = 0.0f, radclrd = 0.0f;
      for (int L0 = nl - 1; L0 >= 0; L0 -= 4) {
        const int nb = L0 + 1 < 4 ? L0 + 1 : 4;  // levels L0, L0-1, .., L0-nb+1
        float2 c[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int L = j < nb ? L0 - j : 0;  // an address inside the slot even where nothing is loaded
          const float* pl = reinterpret_cast<const float*>(scr) + L * GB_NGPT + g;
          c[j] = j < nb ? make_float2(pl[0], pl[nl * GB_NGPT]) : make_float2(0.f, 0.f);  // T, Sd
        }
        float q0[4], q1[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          q0[j] = q1[j] = 0.0f;
          if (j < nb) {
            const int L = L0 - j;
            if (clouds && s.cldlay[L] && cell_is_cloudy(s, L, g)) {
              const float4 k = scr[(nl + L) * GB_NGPT + g];
              radld = fmaf(radld, k.x, k.y);
            } else {
              radld = fmaf(radld, c[j].x, c[j].y);
            }
            radclrd = fmaf(radclrd, c[j].x, c[j].y);
            q0[j] = radld * wgt;
            q1[j] = radclrd * wgt;
          }
        }
        const float s0 = reduce4(q0, lane), s1 = reduce4(q1, lane);
        if (lane < nb) {
          part[(L0 - lane) * 6 + 0] = s0;
          part[(L0 - lane) * 6 + 1] = s1;
        }
      }
      // surface emission and reflection (rtrnmc.f90:465-485)
      const float plfrac1 = s.frac1[g];
      const float rad0 = plfrac1 * s.misc[16 + band];
      const float reflect = 1.0f - s.misc[48 + band];
      float radlu = rad0 + reflect * radld;
      float radclru = rad0 + reflect * radclrd;
      float d_radlu = plfrac1 * s.misc[32 + band], d_radclru = d_radlu;
      // upward (rtrnmc.f90:486-529): level 0 is the surface, level L+1 follows layer L
      for (int v0 = 0; v0 <= nl; v0 += 4) {
        const int nb = nl + 1 - v0 < 4 ? nl + 1 - v0 : 4;  // levels v0 .. v0+nb-1
        float2 c[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const bool in = j < nb && v0 + j >= 1;
          const float* pl = reinterpret_cast<const float*>(scr) + (in ? v0 + j - 1 : 0) * GB_NGPT + g;
          c[j] = in ? make_float2(pl[0], pl[2 * nl * GB_NGPT]) : make_float2(0.f, 0.f);  // T, Su
        }
        float u0[4], u1[4], u2[4], u3[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          u0[j] = u1[j] = u2[j] = u3[j] = 0.0f;
          if (j < nb) {
            if (v0 + j >= 1) {
              const int L = v0 + j - 1;
              if (clouds && s.cldlay[L] && cell_is_cloudy(s, L, g)) {
                const float4 k = scr[(nl + L) * GB_NGPT + g];
                radlu = fmaf(radlu, k.x, k.z);
                d_radlu *= k.w;
              } else {
                radlu = fmaf(radlu, c[j].x, c[j].y);
                d_radlu *= c[j].x;
              }
              radclru = fmaf(radclru, c[j].x, c[j].y);
              d_radclru *= c[j].x;
            }
            u0[j] = radlu * wgt;
            u1[j] = radclru * wgt;
            u2[j] = d_radlu * wgt;
            u3[j] = d_radclru * wgt;
          }
        }
        const float s0 = reduce4(u0, lane), s1 = reduce4(u1, lane);
        float s2 = 0.0f, s3 = 0.0f;
        if (idrv) {
          s2 = reduce4(u2, lane);
          s3 = reduce4(u3, lane);
        }
        if (lane < nb) {
          float* p = part + (v0 + lane) * 6;
          p[2] = s0;
          p[3] = s1;
          p[4] = s2;
          p[5] = s3;
        }
      }
    }
    __syncthreads();

    // ---------------- phase 4: fp64 sums, net fluxes, heating rates, stores
    {
      const long long ldo = a.ldo;
      const bool idrv = a.idrv == 1;
      for (int lev = tid; lev <= nl; lev += NT) {
        // the five warps' fp32 partials summed without rounding error: Knuth's
        // two-sum keeps each addition's rounding error, and the sum and the
        // accumulated errors go to fp64 (two conversions instead of five
        // conversions and four fp64 additions; fp64 is a narrow pipe on GB300)
        double acc[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          float hi = s.part[lev * 6 + k], lo = 0.0f;
#pragma unroll
          for (int w = 1; w < NSW; ++w) {
            const float b = s.part[(w * (nl + 1) + lev) * 6 + k];
            const float sum = hi + b, bv = sum - hi;
            lo += (hi - (sum - bv)) + (b - bv);
            hi = sum;
          }
          acc[k] = (double)hi + (double)lo;
        }
        if (lev == nl) acc[0] = acc[1] = 0.0;  // no downward radiation at the model top
        long long o = icol + ldo * lev;
        a.uflx[o] = acc[2];
        a.dflx[o] = acc[0];
        a.uflxc[o] = acc[3];
        a.dflxc[o] = acc[1];
        if (idrv) {
          a.duflx_dt[o] = acc[4];
          a.duflxc_dt[o] = acc[5];
        }
        s.fnet[lev * 2 + 0] = acc[2] - acc[0];
        s.fnet[lev * 2 + 1] = acc[3] - acc[1];
      }
      __syncthreads();
      for (int l = tid; l < nl; l += NT) {
        const double dp = in2(a.plev, a.ld, icol, l) - in2(a.plev, a.ld, icol, l + 1);
        const double f = c_T.heatfac / dp;  // one division for both heating rates
        long long o = icol + ldo * l;
        a.hr[o] = f * (s.fnet[l * 2] - s.fnet[(l + 1) * 2]);
        a.hrc[o] = f * (s.fnet[l * 2 + 1] - s.fnet[(l + 1) * 2 + 1]);
      }
      __syncthreads();
    }
  }
  return true;
}

// ------------------------------------------------------------------ the kernel
// Persistent blocks walk the batch columns grid after grid; a block's columns
// increase, so its grid index only moves forward.  FLAVOR 1 is the
// learned-only kernel, which appends the columns it does not solve to
// B.fall; FLAVOR 2 is the full kernel walking that list instead of the batch.
// The unit is compiled without multiply-add contraction, so a column gives
// the same bits in every flavour and launch shape.
template <int NT, int MINB, int FLAVOR>
__global__ void __launch_bounds__(NT, MINB) lw_batch_kernel(const __grid_constant__ LwBatch B,
                                                             const float* __restrict__ T) {
  constexpr bool LEAN = FLAVOR == 1, list = FLAVOR == 2;
  extern __shared__ __align__(16) char smem_raw[];
  float4* __restrict__ scr = B.scratch + (size_t)blockIdx.x * ((size_t)2 * B.nsmax * GB_NGPT);
  const long long n = list ? (long long)*B.nfall : B.col0[B.ngrid];
  int gi = 0;
  for (long long i = blockIdx.x; i < n; i += gridDim.x) {
    const long long gc = list ? B.fall[i] : i;
    if (list) gi = 0;  // the list is in no particular order
    while (gc >= B.col0[gi + 1]) ++gi;
    const bool done = solve_column<NT, LEAN>(B.g[gi], gc - B.col0[gi], smem_raw, scr, T);
    if (LEAN && !done && threadIdx.x == 0) B.fall[atomicAdd(B.nfall, 1u)] = gc;
  }
}

// compiled shapes (threads per column block, min blocks per SM); variant 0 is the default
#define GB_LW_VARIANTS(X) X(0, 160, 5) X(1, 160, 6) X(2, 160, 4) X(3, 256, 3)
// the learned-only kernel: less shared memory and fewer registers, so more blocks fit
#define GB_LW_LEAN_VARIANTS(X) X(0, 160, 6) X(1, 160, 7) X(2, 160, 5) X(3, 256, 4)

}  // namespace gb

// ------------------------------------------------------------------ host side
namespace {

struct VariantInfo {
  int threads, min_blocks;
  const void* fn;
  cudaError_t (*launch)(const LwBatch&, const float*, int, size_t, cudaStream_t);
};

template <int NT, int MINB, int FLAVOR>
cudaError_t launch_variant(const LwBatch& b, const float* T, int nblocks, size_t smem, cudaStream_t st) {
  gb::lw_batch_kernel<NT, MINB, FLAVOR><<<nblocks, NT, smem, st>>>(b, T);
  return cudaGetLastError();
}

#define GB_LW_VARIANT_ENTRY(i, nt, mb) {nt, mb, (const void*)gb::lw_batch_kernel<nt, mb, 0>, launch_variant<nt, mb, 0>},
#define GB_LW_LEAN_ENTRY(i, nt, mb) {nt, mb, (const void*)gb::lw_batch_kernel<nt, mb, 1>, launch_variant<nt, mb, 1>},
const VariantInfo kVariants[] = {GB_LW_VARIANTS(GB_LW_VARIANT_ENTRY)};
const VariantInfo kLean[] = {GB_LW_LEAN_VARIANTS(GB_LW_LEAN_ENTRY)};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
static_assert(sizeof(kLean) / sizeof(kLean[0]) == kNumVariants, "one variant index range for both kernels");
// the full kernel over the columns the learned-only kernel hands over
const VariantInfo kList = {160, 6, (const void*)gb::lw_batch_kernel<160, 6, 2>, launch_variant<160, 6, 2>};

const VariantInfo& info(int variant, bool lean) { return lean ? kLean[variant] : kVariants[variant]; }

cudaError_t configure(int nlay, const VariantInfo& v, bool lean, int* blocks_per_sm) {
  const size_t sm = gb::smem_bytes(nlay, lean);
  cudaError_t e = cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(v.fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, v.fn, v.threads, sm);
}

// Shared-memory carve-out for `per` resident blocks: just what they need, so
// that the rest of the SM's 256 KB stays L1 for the table gathers (the
// driver otherwise sizes it for the largest block count shared memory alone
// would allow, even when registers allow fewer).
cudaError_t set_carveout(const VariantInfo& v, size_t smem, int per) {
  int dev = 0, max_sm = 0, reserved = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  if (max_sm <= 0) return cudaSuccess;
  int pct = (int)std::ceil(100.0 * (double)per * (double)(smem + reserved) / (double)max_sm);
  pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
  return cudaFuncSetAttribute(v.fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

// One launch of `variant` of the full (lean false) or learned-only kernel
// with at most `nblocks` blocks and the carve-out for those resident.
cudaError_t launch_kernel(const LwBatch& b, const float* d_tables, const VariantInfo& v, bool lean, int nblocks,
                          cudaStream_t stream) {
  int per = 0;
  cudaError_t e = configure(b.nsmax, v, lean, &per);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int resident = (nblocks + nsm - 1) / nsm;
  const size_t smem = gb::smem_bytes(b.nsmax, lean);
  e = set_carveout(v, smem, resident < per ? resident : per);
  if (e != cudaSuccess) return e;
  return v.launch(b, d_tables, nblocks, smem, stream);
}

}  // namespace

int gb_lw_num_variants() { return kNumVariants; }

LwVariant gb_lw_variant(int v, bool lean) {
  if (v < 0 || v >= kNumVariants) return LwVariant{0, 0};
  return LwVariant{info(v, lean).threads, info(v, lean).min_blocks};
}

size_t gb_lw_smem_bytes(int nlay, bool lean) { return gb::smem_bytes(nlay, lean); }

cudaError_t gb_lw_set_tables(const GbTables& T) { return cudaMemcpyToSymbol(gb::c_T, &T, sizeof(GbTables)); }

int gb_lw_slots(int nlay, int variant, bool lean) {
  if (variant < 0 || variant >= kNumVariants) variant = 0;
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (configure(nlay, info(variant, lean), lean, &per) != cudaSuccess || per < 1) per = 1;
  return nsm * per;
}

size_t gb_lw_scratch_bytes(int nlay, int slots) { return (size_t)slots * 2 * nlay * GB_NGPT * sizeof(float4); }

cudaError_t gb_lw_launch_batch(const LwBatch& b, const float* d_tables, int variant, int nblocks,
                               cudaStream_t stream) {
  if (variant < 0 || variant >= kNumVariants || b.ngrid < 1 || b.ngrid > GB_LW_MAX_GRIDS) return cudaErrorInvalidValue;
  if (b.col0[b.ngrid] <= 0 || nblocks <= 0) return cudaSuccess;
  if ((long long)nblocks > b.col0[b.ngrid]) nblocks = (int)b.col0[b.ngrid];
  if (!b.fall || !b.nfall) return launch_kernel(b, d_tables, info(variant, false), false, nblocks, stream);
  // learned gas optics: the learned-only kernel, then the full kernel over
  // the columns it handed over (its blocks find an empty list and return
  // when every column was on the network)
  cudaError_t e = cudaMemsetAsync(b.nfall, 0, sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  e = launch_kernel(b, d_tables, info(variant, true), true, nblocks, stream);
  if (e != cudaSuccess) return e;
  int per = 0;
  const VariantInfo& lv = kList;
  e = configure(b.nsmax, lv, false, &per);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nf = per * nsm < nblocks ? per * nsm : nblocks;  // scratch holds nblocks slots
  return launch_kernel(b, d_tables, lv, false, nf < 1 ? 1 : nf, stream);
}

cudaError_t gb_lw_launch(const LwArgs& a, const float* d_tables, float4* scratch, int nslots, cudaStream_t stream) {
  if (a.ncol <= 0) return cudaSuccess;
  LwBatch b;
  b.ngrid = 1;
  b.nsmax = a.nlay;
  b.col0[0] = 0;
  b.col0[1] = a.ncol;
  b.scratch = scratch;
  b.g[0] = a;
  return gb_lw_launch_batch(b, d_tables, 0, a.ncol < nslots ? a.ncol : nslots, stream);
}
