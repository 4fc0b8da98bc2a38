// Fused RRTMG_LW column kernel for GB300 (sm_103a).
//
// One thread block solves one column (the reference's column loop,
// rrtmg_lw_rad.f90:486-593).  Phases, separated by block barriers:
//   1. inatm + setcoef (rrtmg_lw_rad.f90:598-924, rrtmg_lw_setcoef.f90:50-434):
//      one thread per layer, coefficients into shared memory; Planck
//      interpolation with one thread per (level, band); column sums for pwvcm.
//      In parallel the 140 g-point threads scan the McICA cloud fractions to
//      mark cloudy layers (rtrnmc.f90:292-331) and check the cloud particle
//      sizes exactly where cldprmc would (cldprmc.f90:178-266).
//   2. taumol (rrtmg_lw_taumol.f90): one thread per (layer, g) cell, band by
//      band, writing taut = taug + aerosol (rrtmg_lw_rad.f90:548-553) to shared
//      memory, plus one Planck-fraction record per (layer, band).
//   3. rtrnmc (rrtmg_lw_rtrnmc.f90:51-595): one thread per g-point; downward
//      then upward sweep.  The upward sweep recomputes the layer
//      transmittances from taut instead of storing them, which keeps shared
//      memory per column near 40 KB.  Lookup-table entries exp_tbl/tfn_tbl/
//      tau_tbl (rrtmg_lw_init.f90:125-142) are evaluated at the quantised
//      table index instead of being loaded.  Per-level g-point sums are
//      weighted by 0.5*delwave*fluxfac and reduced across each warp in fp32.
//   4. fp64 epilogue: per-warp partial sums added in fp64, net fluxes and
//      heating rates heatfac*dF/dp in fp64 (rtrnmc.f90:566-592).
//
// Precision: gas optics and transfer in fp32; flux accumulation across warps
// and the heating-rate step in fp64.  Outputs follow the reference's layout:
// uflx(icol, k+1) for k = 0..nlay, hr(icol, k+1) for k = 0..nlay-1.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "lw_common.h"
#include "lw_solver.h"
#include "lw_gasoptics.cuh"

namespace gb {

constexpr int NT = 160;      // threads per column block (5 warps; 140 g-point lanes)
constexpr int NWARP = NT / 32;
constexpr float BPADE = 1.0f / 0.278f;

// ------------------------------------------------------------------ shared memory layout
struct Smem {
  float* f;        // [NF][nl]   per-layer coefficients (phase 1-2)
  int* iv;         // [NI][nl]
  float2* terms;   // [nl][MAXT_ALL] gas-optics terms of the current band (phase 2)
  float* part;     // [NWARP][nl+1][6] warp partial fluxes (aliases f/iv in phase 3-4)
  float* taut;     // [nl][140]
  float* taua;     // [nl][16]
  float* plk_lay;  // [nl][16]
  float* plk_lev;  // [nl+1][16]
  FracRec* frec;   // [nl][16]
  int* cldlay;     // [nl]
  double* fnet;    // [nl+1][2] net fluxes (phase 4)
  float* misc;     // [64]: secdiff[16], plankbnd[16], dplankbnd[16], semiss[16]
  float* scal;     // [4]: pwvcm pieces
  int* iscal;      // [4]: laytrop, lower-count, error
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline size_t smem_bytes(int nl) {
  size_t coef = (((size_t)(NF + NI) * nl * 4 + 7) & ~size_t(7)) + (size_t)nl * MAXT_ALL * 8;
  size_t part = (size_t)NWARP * (nl + 1) * 6 * 4;
  size_t a = align16(coef > part ? coef : part);
  a += align16((size_t)nl * GB_NGPT * 4);
  a += align16((size_t)nl * 16 * 4);
  a += align16((size_t)nl * 16 * 4);
  a += align16((size_t)(nl + 1) * 16 * 4);
  a += align16((size_t)nl * 16 * sizeof(FracRec));
  a += align16((size_t)nl * 4);
  a += align16((size_t)(nl + 1) * 2 * 8);
  a += align16(64 * 4) + align16(4 * 4) + align16(4 * 4);
  return a;
}

__device__ inline Smem carve(char* base, int nl) {
  Smem s;
  size_t coef = (((size_t)(NF + NI) * nl * 4 + 7) & ~size_t(7)) + (size_t)nl * MAXT_ALL * 8;
  size_t part = (size_t)NWARP * (nl + 1) * 6 * 4;
  char* p = base;
  s.f = (float*)p;
  s.iv = (int*)(p + (size_t)NF * nl * 4);
  s.terms = (float2*)(p + (((size_t)(NF + NI) * nl * 4 + 7) & ~size_t(7)));
  s.part = (float*)p;
  p += align16(coef > part ? coef : part);
  s.taut = (float*)p; p += align16((size_t)nl * GB_NGPT * 4);
  s.taua = (float*)p; p += align16((size_t)nl * 16 * 4);
  s.plk_lay = (float*)p; p += align16((size_t)nl * 16 * 4);
  s.plk_lev = (float*)p; p += align16((size_t)(nl + 1) * 16 * 4);
  s.frec = (FracRec*)p; p += align16((size_t)nl * 16 * sizeof(FracRec));
  s.cldlay = (int*)p; p += align16((size_t)nl * 4);
  s.fnet = (double*)p; p += align16((size_t)(nl + 1) * 2 * 8);
  s.misc = (float*)p; p += align16(64 * 4);
  s.scal = (float*)p; p += align16(4 * 4);
  s.iscal = (int*)p;
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

// exp_tbl/tfn_tbl/tau_tbl at the index the reference's lookup would pick
// (rrtmg_lw_rtrnmc.f90:385-388 with rrtmg_lw_init.f90:125-142)
struct TblEntry {
  float tau, trans, tfn;
};
__device__ __forceinline__ TblEntry tbl(float od) {
  float tblind = __fdividef(od, BPADE + od);
  int itr = (int)(10000.0f * tblind + 0.5f);
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
    e.tfn = tau < 0.06f ? tau * (1.0f / 6.0f) : 1.0f - 2.0f * (__fdividef(1.0f, tau) - __fdividef(ex, 1.0f - ex));
  }
  return e;
}

// Transfer quantities of one (layer, g) cell (rtrnmc.f90:350-455).
struct CellRT {
  float atrans, bbd, gassrc, atot, bbdtot, bbugas, bbutot;
};
__device__ __forceinline__ CellRT cell_rt(bool cloudy_layer, float odepth, float odcld, float plfrac, float blay,
                                          float dplankup, float dplankdn) {
  const float rec_6 = 0.166667f;
  CellRT r;
  if (cloudy_layer) {
    float odtot = odepth + odcld;
    if (odtot < 0.06f) {
      r.atrans = odepth - 0.5f * odepth * odepth;
      float odepth_rec = rec_6 * odepth;
      r.gassrc = plfrac * (blay + dplankdn * odepth_rec) * r.atrans;
      r.atot = odtot - 0.5f * odtot * odtot;
      float odtot_rec = rec_6 * odtot;
      r.bbdtot = plfrac * (blay + dplankdn * odtot_rec);
      r.bbd = plfrac * (blay + dplankdn * odepth_rec);
      r.bbugas = plfrac * (blay + dplankup * odepth_rec);
      r.bbutot = plfrac * (blay + dplankup * odtot_rec);
    } else if (odepth <= 0.06f) {
      r.atrans = odepth - 0.5f * odepth * odepth;
      float odepth_rec = rec_6 * odepth;
      r.gassrc = plfrac * (blay + dplankdn * odepth_rec) * r.atrans;
      TblEntry et = tbl(odtot);
      r.bbdtot = plfrac * (blay + et.tfn * dplankdn);
      r.bbd = plfrac * (blay + dplankdn * odepth_rec);
      r.atot = 1.0f - et.trans;
      r.bbugas = plfrac * (blay + dplankup * odepth_rec);
      r.bbutot = plfrac * (blay + et.tfn * dplankup);
    } else {
      TblEntry eg = tbl(odepth);
      r.atrans = 1.0f - eg.trans;
      r.gassrc = r.atrans * plfrac * (blay + eg.tfn * dplankdn);
      TblEntry et = tbl(eg.tau + odcld);
      r.bbdtot = plfrac * (blay + et.tfn * dplankdn);
      r.bbd = plfrac * (blay + eg.tfn * dplankdn);
      r.atot = 1.0f - et.trans;
      r.bbugas = plfrac * (blay + eg.tfn * dplankup);
      r.bbutot = plfrac * (blay + et.tfn * dplankup);
    }
  } else {
    if (odepth <= 0.06f) {
      r.atrans = odepth - 0.5f * odepth * odepth;
      float o = rec_6 * odepth;
      r.bbd = plfrac * (blay + dplankdn * o);
      r.bbugas = plfrac * (blay + dplankup * o);
    } else {
      TblEntry e = tbl(odepth);
      r.atrans = 1.0f - e.trans;
      r.bbd = plfrac * (blay + e.tfn * dplankdn);
      r.bbugas = plfrac * (blay + e.tfn * dplankup);
    }
    r.gassrc = 0.0f; r.atot = 0.0f; r.bbdtot = 0.0f; r.bbutot = 0.0f;
  }
  return r;
}

// McICA cloud optics of one cell: returns cldfmc and sets odcld/efcl
// (cldprmc.f90:178-266 then rtrnmc.f90:300-312; computed only where
// cldfmc == 1, the only cells whose optical depth rtrnmc reads).
__device__ __forceinline__ float cell_cloud(const LwArgs& a, long long icol, int g, int lay, float secdiff_b,
                                            int band, const float* __restrict__ T, float& odcld, float& efcl) {
  long long o = (long long)g + GB_NGPT * (icol + (long long)a.ld * lay);
  double cf = __ldg(a.cldfmcl + o);
  odcld = 0.0f;
  efcl = 0.0f;
  if (cf == 1.0) {
    double ciwp = __ldg(a.ciwpmcl + o), clwp = __ldg(a.clwpmcl + o);
    float tauc;
    double cwp = ciwp + clwp;
    double tin = __ldg(a.taucmcl + o);
    if (a.inflag == 2 && (cwp >= 1.e-20 || tin >= 1.e-20)) {
      float abscoice = 0.0f, abscoliq = 0.0f;
      if (ciwp != 0.0) {
        float radice = (float)in2(a.reicmcl, a.ld, icol, lay);
        if (a.iceflag == 0) {
          abscoice = T[c_T.absice0] + T[c_T.absice0 + 1] / radice;
        } else if (a.iceflag == 1) {
          const int icb[16] = {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5};
          int ib = icb[band];
          abscoice = T[c_T.absice1 + 2 * (ib - 1)] + T[c_T.absice1 + 1 + 2 * (ib - 1)] / radice;
        } else if (a.iceflag == 2 || a.iceflag == 3) {
          float factor = (radice - 2.0f) / 3.0f;
          int nrow = a.iceflag == 2 ? 43 : 46;
          int index = clampi((int)factor, 1, nrow - 1);
          float fint = factor - (float)index;
          const float* t = T + (a.iceflag == 2 ? c_T.absice2 : c_T.absice3) + nrow * band;
          abscoice = t[index - 1] + fint * (t[index] - t[index - 1]);
        }
      }
      if (clwp != 0.0) {
        if (a.liqflag == 0) {
          abscoliq = c_T.absliq0;
        } else {
          float radliq = (float)in2(a.relqmcl, a.ld, icol, lay);
          int index = clampi((int)(radliq - 1.5f), 1, 57);
          float fint = radliq - 1.5f - (float)index;
          const float* t = T + c_T.absliq1 + 58 * band;
          abscoliq = t[index - 1] + fint * (t[index] - t[index - 1]);
        }
      }
      tauc = (float)ciwp * abscoice + (float)clwp * abscoliq;
    } else {
      tauc = (float)tin;
    }
    odcld = secdiff_b * tauc;
    efcl = 1.0f - __expf(-odcld);
  }
  return (float)cf;
}

// ------------------------------------------------------------------ gas optics of one band
// Prologue once per layer (terms into shared memory), barrier, then one
// generic weighted gather per (layer, g) cell.
template <int b>
__device__ __forceinline__ void gas_optics_band(const Smem& s, int nl, int laytrop, const float* __restrict__ T) {
  constexpr int NG = ngb_const(b), G0 = g0_const(b), M = maxt(b);
  const int pad_off = c_T.band[b - 1].sr;
  for (int lay = threadIdx.x; lay < nl; lay += NT) {
    Cell c{s.f, s.iv, nl, lay};
    Terms t{s.terms + lay * MAXT_ALL, 0};
    FracRec r = prologue<b>(c, lay < laytrop, t);
    t.pad(M, pad_off);
    s.frec[lay * 16 + (b - 1)] = r;
  }
  __syncthreads();
  for (int cell = threadIdx.x; cell < nl * NG; cell += NT) {
    const int lay = cell / NG, gi = cell - lay * NG;
    const float2* tp = s.terms + lay * MAXT_ALL;
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < M; ++k) {
      float2 w = tp[k];
      acc = fmaf(w.x, __ldg(T + __float_as_int(w.y) + gi), acc);
    }
    if ((b == 4 || b == 7) && lay >= laytrop) acc *= gscale(b, gi);
    s.taut[lay * GB_NGPT + G0 + gi] = acc + s.taua[lay * 16 + (b - 1)];
  }
  __syncthreads();
}

// ------------------------------------------------------------------ the kernel
__global__ void __launch_bounds__(NT) lw_column_kernel(LwArgs a, const float* __restrict__ T) {
  extern __shared__ __align__(16) char smem_raw[];
  const int nl = a.nlay;
  const long long icol = blockIdx.x;
  if (icol >= a.ncol) return;
  Smem s = carve(smem_raw, nl);
  const int tid = threadIdx.x;
  if (tid < 4) {
    s.scal[tid] = 0.0f;
    s.iscal[tid] = 0;
  }
  for (int l = tid; l < nl; l += NT) s.cldlay[l] = 0;
  __syncthreads();

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
    for (int ib = 0; ib < 16; ++ib)
      s.taua[lay * 16 + ib] = (float)__ldg(a.tauaer + icol + (long long)a.ld * (lay + (long long)nl * ib));
  }
  // Planck interpolation per (level, band) (setcoef.f90:173-269, istart = 1)
  for (int it = tid; it < (nl + 1) * 16; it += NT) {
    int lev = it >> 4, ib = it & 15;
    const float* tp = T + c_T.totplnk + ib * 181;
    float tz = (float)in2(a.tlev, a.ld, icol, lev);
    int ind = clampi((int)(tz - 159.0f), 1, 180);
    float fr = tz - 159.0f - (float)ind;
    s.plk_lev[lev * 16 + ib] = tp[ind - 1] + fr * (tp[ind] - tp[ind - 1]);
    if (lev < nl) {
      float tl = (float)in2(a.tlay, a.ld, icol, lev);
      int il = clampi((int)(tl - 159.0f), 1, 180);
      float fl = tl - 159.0f - (float)il;
      s.plk_lay[lev * 16 + ib] = tp[il - 1] + fl * (tp[il] - tp[il - 1]);
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
  // McICA pre-pass: cloudy layers and cldprmc's STOP conditions
  if (tid < GB_NGPT && a.icld >= 1) {
    int err = 0;
    for (int lay = 0; lay < nl; ++lay) {
      long long o = (long long)tid + GB_NGPT * (icol + (long long)a.ld * lay);
      double cf = __ldg(a.cldfmcl + o);
      if (cf == 1.0) s.cldlay[lay] = 1;
      if (cf >= 1.e-20) {
        double ciwp = __ldg(a.ciwpmcl + o), clwp = __ldg(a.clwpmcl + o);
        if (ciwp + clwp >= 1.e-20 || __ldg(a.taucmcl + o) >= 1.e-20) {
          if (a.inflag == 1) err = GB_COL_INFLAG1;
          if (a.inflag == 2) {
            double rice = in2(a.reicmcl, a.ld, icol, lay), rliq = in2(a.relqmcl, a.ld, icol, lay);
            if (ciwp != 0.0) {
              if (a.iceflag == 0 && rice < 10.0) err = GB_COL_ICE_SMALL;
              if (a.iceflag == 1 && (rice < 13.0 || rice > 130.0)) err = GB_COL_ICE_BOUNDS;
              if (a.iceflag == 2 && (rice < 5.0 || rice > 131.0)) err = GB_COL_ICE_BOUNDS;
              if (a.iceflag == 3 && (rice < 5.0 || rice > 140.0)) err = GB_COL_DGE_BOUNDS;
            }
            if (clwp != 0.0 && a.liqflag == 1 && (rliq < 2.5 || rliq > 60.0)) err = GB_COL_LIQ_BOUNDS;
          }
        }
      }
    }
    if (err) atomicMax(&s.iscal[2], err);
  }
  int anybad = __syncthreads_or(my_bad);
  const int laytrop = s.iscal[0];
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
    // pwvcm (inatm :859-870, summed in layer order) and secdiff (rtrnmc.f90:258-266)
    float amttl = 0.0f, wvttl = 0.0f;
    for (int l = 0; l < nl; ++l) {
      float wk1 = s.f[F_COLH2O * nl + l] * 1.e20f;
      amttl = amttl + s.f[F_COLDRY * nl + l] + wk1;
      wvttl = wvttl + wk1;
    }
    float wvsh = (amw * wvttl) / (amd * amttl);
    float pz0 = (float)in2(a.plev, a.ld, icol, 0);
    float pwvcm = wvsh * (1.e3f * pz0) / (1.e2f * (float)c_T.grav);
    const float a0[16] = {1.66f, 1.55f, 1.58f, 1.66f, 1.54f, 1.454f, 1.89f, 1.33f, 1.668f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f};
    const float a1[16] = {0.f, 0.25f, 0.22f, 0.f, 0.13f, 0.446f, -0.10f, 0.40f, -0.006f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const float a2[16] = {0.f, -12.0f, -11.7f, 0.f, -0.72f, -0.243f, 0.19f, -0.062f, 0.414f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int ib = 0; ib < 16; ++ib) {
      float sd = 1.66f;
      if (!(ib == 0 || ib == 3 || ib >= 9)) {
        sd = a0[ib] + a1[ib] * __expf(a2[ib] * pwvcm);
        sd = fminf(fmaxf(sd, 1.50f), 1.80f);
      }
      s.misc[ib] = sd;
    }
  }
  __syncthreads();

  // ---------------- phase 2: taumol, band by band
  gas_optics_band<1>(s, nl, laytrop, T);
  gas_optics_band<2>(s, nl, laytrop, T);
  gas_optics_band<3>(s, nl, laytrop, T);
  gas_optics_band<4>(s, nl, laytrop, T);
  gas_optics_band<5>(s, nl, laytrop, T);
  gas_optics_band<6>(s, nl, laytrop, T);
  gas_optics_band<7>(s, nl, laytrop, T);
  gas_optics_band<8>(s, nl, laytrop, T);
  gas_optics_band<9>(s, nl, laytrop, T);
  gas_optics_band<10>(s, nl, laytrop, T);
  gas_optics_band<11>(s, nl, laytrop, T);
  gas_optics_band<12>(s, nl, laytrop, T);
  gas_optics_band<13>(s, nl, laytrop, T);
  gas_optics_band<14>(s, nl, laytrop, T);
  gas_optics_band<15>(s, nl, laytrop, T);
  gas_optics_band<16>(s, nl, laytrop, T);
  if (a.dbg_taut) {
    for (int c = tid; c < nl * GB_NGPT; c += NT) {
      int lay = c / GB_NGPT, g = c - lay * GB_NGPT;
      int b = c_T.ngb[g] - 1;
      FracRec r = s.frec[lay * 16 + b];
      const float* p = T + r.off + (g - c_T.band[b].g0);
      a.dbg_taut[(icol * nl + lay) * GB_NGPT + g] = s.taut[c];
      a.dbg_fracs[(icol * nl + lay) * GB_NGPT + g] = p[0] + r.fpl * (p[c_T.band[b].ng] - p[0]);
    }
  }

  // ---------------- phase 3: transfer, one thread per g-point
  const int warp = tid >> 5, lane = tid & 31;
  const bool active = tid < GB_NGPT;
  const int g = active ? tid : GB_NGPT - 1;
  const int band = c_T.ngb[g] - 1;
  const int ng = c_T.band[band].ng, gi = g - c_T.band[band].g0;
  const float secdiff = s.misc[band];
  const float wgt = active ? (float)(0.5 * (double)c_T.delwave[band] * c_T.fluxfac) : 0.0f;
  const bool idrv = a.idrv == 1;
  const bool clouds = a.icld >= 1;
  auto frac = [&](int lay) {
    FracRec r = s.frec[lay * 16 + band];
    const float* p = T + r.off + gi;
    float f0 = __ldg(p);
    return f0 + r.fpl * (__ldg(p + ng) - f0);
  };
  float* part = s.part;  // [NWARP][nl+1][6]
  auto emit = [&](int lev, int k, float v) {
    float sum = warp_sum(v * wgt);
    if (lane == 0) part[(warp * (nl + 1) + lev) * 6 + k] = sum;
  };
  // downward sweep (rtrnmc.f90:347-455)
  float radld = 0.0f, radclrd = 0.0f;
  bool iclddn = false;
  for (int lev = nl; lev >= 1; --lev) {
    const int L = lev - 1;  // 0-based layer
    float plfrac = frac(L);
    float blay = s.plk_lay[L * 16 + band];
    float dplankup = s.plk_lev[lev * 16 + band] - blay;
    float dplankdn = s.plk_lev[(lev - 1) * 16 + band] - blay;
    float odepth = fmaxf(secdiff * s.taut[L * GB_NGPT + g], 0.0f);
    bool cl = clouds && s.cldlay[L];
    if (cl) {
      iclddn = true;
      float odcld, efcl;
      float cldf = cell_cloud(a, icol, g, L, secdiff, band, T, odcld, efcl);
      efcl *= (cldf == 1.0f ? cldf : 0.0f);
      CellRT r = cell_rt(true, odepth, odcld, plfrac, blay, dplankup, dplankdn);
      radld = radld - radld * (r.atrans + efcl * (1.0f - r.atrans)) + r.gassrc + cldf * (r.bbdtot * r.atot - r.gassrc);
      radclrd = radclrd + (r.bbd - radclrd) * r.atrans;
    } else {
      CellRT r = cell_rt(false, odepth, 0.0f, plfrac, blay, dplankup, dplankdn);
      radld = radld + (r.bbd - radld) * r.atrans;
      if (iclddn) radclrd = radclrd + (r.bbd - radclrd) * r.atrans;
      else radclrd = radld;
    }
    emit(lev - 1, 0, radld);
    emit(lev - 1, 1, radclrd);
  }
  // surface (rtrnmc.f90:465-485)
  float plfrac1 = frac(0);
  float rad0 = plfrac1 * s.misc[16 + band];
  float d_rad0 = plfrac1 * s.misc[32 + band];
  float reflect = 1.0f - s.misc[48 + band];
  float radlu = rad0 + reflect * radld;
  float radclru = rad0 + reflect * radclrd;
  float d_radlu = d_rad0, d_radclru = d_rad0;
  emit(0, 2, radlu);
  emit(0, 3, radclru);
  if (idrv) {
    emit(0, 4, d_radlu);
    emit(0, 5, d_radclru);
  }
  // upward sweep (rtrnmc.f90:486-529)
  for (int lev = 1; lev <= nl; ++lev) {
    const int L = lev - 1;
    float plfrac = frac(L);
    float blay = s.plk_lay[L * 16 + band];
    float dplankup = s.plk_lev[lev * 16 + band] - blay;
    float dplankdn = s.plk_lev[(lev - 1) * 16 + band] - blay;
    float odepth = fmaxf(secdiff * s.taut[L * GB_NGPT + g], 0.0f);
    bool cl = clouds && s.cldlay[L];
    if (cl) {
      float odcld, efcl;
      float cldf = cell_cloud(a, icol, g, L, secdiff, band, T, odcld, efcl);
      efcl *= (cldf == 1.0f ? cldf : 0.0f);
      CellRT r = cell_rt(true, odepth, odcld, plfrac, blay, dplankup, dplankdn);
      float gassrc = r.bbugas * r.atrans;
      radlu = radlu - radlu * (r.atrans + efcl * (1.0f - r.atrans)) + gassrc + cldf * (r.bbutot * r.atot - gassrc);
      d_radlu = d_radlu * cldf * (1.0f - r.atot) + d_radlu * (1.0f - cldf) * (1.0f - r.atrans);
      radclru = radclru + (r.bbugas - radclru) * r.atrans;
      d_radclru = d_radclru * (1.0f - r.atrans);
    } else {
      CellRT r = cell_rt(false, odepth, 0.0f, plfrac, blay, dplankup, dplankdn);
      radlu = radlu + (r.bbugas - radlu) * r.atrans;
      d_radlu = d_radlu * (1.0f - r.atrans);
      if (iclddn) {
        radclru = radclru + (r.bbugas - radclru) * r.atrans;
        d_radclru = d_radclru * (1.0f - r.atrans);
      } else {
        radclru = radlu;
        d_radclru = d_radlu;
      }
    }
    emit(lev, 2, radlu);
    emit(lev, 3, radclru);
    if (idrv) {
      emit(lev, 4, d_radlu);
      emit(lev, 5, d_radclru);
    }
  }
  __syncthreads();

  // ---------------- phase 4: fp64 sums, net fluxes, heating rates, stores
  const long long ldo = a.ldo;
  for (int lev = tid; lev <= nl; lev += NT) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int w = 0; w < NWARP; ++w)
      for (int k = 0; k < 6; ++k) acc[k] += (double)part[(w * (nl + 1) + lev) * 6 + k];
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
    double dp = in2(a.plev, a.ld, icol, l) - in2(a.plev, a.ld, icol, l + 1);
    long long o = icol + ldo * l;
    a.hr[o] = c_T.heatfac * (s.fnet[l * 2] - s.fnet[(l + 1) * 2]) / dp;
    a.hrc[o] = c_T.heatfac * (s.fnet[l * 2 + 1] - s.fnet[(l + 1) * 2 + 1]) / dp;
  }
}

}  // namespace gb

// ------------------------------------------------------------------ host side
size_t gb_lw_smem_bytes(int nlay) { return gb::smem_bytes(nlay); }

cudaError_t gb_lw_set_tables(const GbTables& T) {
  return cudaMemcpyToSymbol(gb::c_T, &T, sizeof(GbTables));
}

cudaError_t gb_lw_launch(const LwArgs& a, const float* d_tables, cudaStream_t stream) {
  if (a.ncol <= 0) return cudaSuccess;
  size_t sm = gb::smem_bytes(a.nlay);
  static int configured_bytes = -1;
  if ((int)sm > configured_bytes) {
    cudaError_t e = cudaFuncSetAttribute(gb::lw_column_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    configured_bytes = (int)sm;
  }
  gb::lw_column_kernel<<<a.ncol, gb::NT, sm, stream>>>(a, d_tables);
  return cudaGetLastError();
}
