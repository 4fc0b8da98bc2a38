// RRTMG_LW column kernels for GB300 (sm_103a).
//
// The reference solves one column at a time (rrtmg_lw_rad.f90:486-593):
// inatm, cldprmc, setcoef, taumol, the aerosol add and rtrnmc.  Here one
// thread block of 160 threads solves a column, thread t standing for g-point
// t (the last warp has 12 live lanes), and persistent blocks walk the columns
// of a batch of grids.  Nothing per cell goes to global scratch:
//
//   taumol (gas_column) -- setcoef (rrtmg_lw_setcoef.f90:275-430) with one
//     thread per layer, then band by band a prologue per layer builds the
//     layer's term list (lw_gasoptics.cuh) and one thread per (layer, g) cell
//     gathers taug = sum w * table[row + g] and interpolates the Planck
//     fraction.  taug (without aerosol) and the fractions go to fp32 planes in
//     a slot owned by the block, which stays in L2 until the transfer of the
//     same column reads it.
//
//   transfer (rt_column) -- inatm's column amounts, the laytrop and value
//     checks, Planck interpolation per (layer, band) and the surface source,
//     the McICA cloud bits and cldprmc's optical depths, then rtrnmc: a
//     downward pass from the model top and an upward pass from the surface.
//     Each pass evaluates a cell's transmittance and sources in registers from
//     taug, the Planck fraction, the layer's Planck values and rtrnmc's
//     exp_tbl/tfn_tbl/tau_tbl (rrtmg_lw_init.f90:120-142, built in double
//     precision at set-up) at the reference's quantised index
//     (rtrnmc.f90:350-455 down, 486-529 up); the up pass recomputes what the
//     down pass computed instead of storing it.  The passes are software
//     pipelined: while layer l is finished, the gas optics of the layer two
//     ahead are loaded and the table entry of the next layer is looked up.
//     Per level the 32 lanes' weighted radiances are summed with a transposed
//     butterfly (two streams down, four up); the five warps' fp32 partials
//     are added error-free (two-sum) into fp64, and the net fluxes and heating
//     rates heatfac*dF/dp are fp64 (rtrnmc.f90:566-592).
//
// Kernels: lw_full_kernel (taumol then the transfer; for batches without a
// network, and for the columns a network batch hands over), lw_rt_kernel (the
// transfer on the network's fp16 taug and Planck fractions; columns with a
// layer off the network are handed over), lw_gas_kernel (taumol alone, for
// the network's training samples and the gas-optics diagnostics).
//
// Precision: gas optics and transfer in fp32, flux sums across warps
// error-free into fp64, net fluxes and the heating-rate step in fp64.
// Outputs follow the reference's layout: uflx(icol, k+1) for k = 0..nlay,
// hr(icol, k+1) for k = 0..nlay-1.  The unit is compiled without multiply-add
// contraction (every fused multiply-add is an explicit fmaf), so a column
// gives the same bits in every kernel flavour and launch shape.
#include <cuda_runtime.h>
#include <math.h>
#include <algorithm>
#include <cmath>
#include <stdint.h>
#include <climits>
#include <cstddef>

#include "lw_common.h"
#include "lw_solver.h"
#include "lw_gasoptics.cuh"

namespace gb {

constexpr float BPADE = 1.0f / 0.278f;
constexpr float REC_6 = 0.166667f;
constexpr int TGROUP = MAXT_ALL;  // term slots per layer of a band's term list
constexpr int RT_NT = 160;        // threads per column block: one per g-point
constexpr int RT_NW = RT_NT / 32;

__constant__ int c_icb[16] = {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5};  // cldprmc.f90:133
// diffusivity-angle coefficients (rtrnmc.f90:236-247)
__constant__ float c_a0[16] = {1.66f, 1.55f, 1.58f, 1.66f, 1.54f, 1.454f, 1.89f, 1.33f, 1.668f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f, 1.66f};
__constant__ float c_a1[16] = {0.f, 0.25f, 0.22f, 0.f, 0.13f, 0.446f, -0.10f, 0.40f, -0.006f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
__constant__ float c_a2[16] = {0.f, -12.0f, -11.7f, 0.f, -0.72f, -0.243f, 0.19f, -0.062f, 0.414f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ double in2(const double* __restrict__ a, long long ld, long long icol, int k) {
  return __ldg(a + icol + ld * k);
}

// setcoef's regime switch (plog <= 4.56 is the upper atmosphere,
// rrtmg_lw_setcoef.f90:312), decided in fp64 near the switch
__device__ __forceinline__ bool lower_atmosphere(double pd, float plog) {
  bool lower = plog > 4.56f;
  if (fabsf(plog - 4.56f) < 1.0e-4f) lower = log(pd) > 4.56;
  return lower;
}

// Warp sums of two values per lane at once: lane i returns the sum over the
// 32 lanes of v(i & 1) (one exchange, then four xor steps).
__device__ __forceinline__ float reduce2(float v0, float v1, int lane) {
  const unsigned F = 0xffffffffu;
  const bool lo = lane & 1;
  float k = lo ? v1 : v0;
  const float s = lo ? v0 : v1;
  k += __shfl_xor_sync(F, s, 1);
  k += __shfl_xor_sync(F, k, 2);
  k += __shfl_xor_sync(F, k, 4);
  k += __shfl_xor_sync(F, k, 8);
  k += __shfl_xor_sync(F, k, 16);
  return k;
}

// Warp sums of four values per lane at once (a transposed butterfly, 6
// shuffles instead of 20): lane i returns the sum over the 32 lanes of v[i & 3].
__device__ __forceinline__ float reduce4(float v0, float v1, float v2, float v3, int lane) {
  const unsigned F = 0xffffffffu;
  const bool hi = lane & 2;
  float k0 = hi ? v2 : v0, k1 = hi ? v3 : v1;
  const float s0 = hi ? v0 : v2, s1 = hi ? v1 : v3;
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

// Warp sums of eight values per lane at once: lane i returns the sum over the
// 32 lanes of v[i & 7] (three exchanges, then two xor steps: 9 shuffles).
__device__ __forceinline__ float reduce8(float v0, float v1, float v2, float v3, float v4, float v5, float v6,
                                         float v7, int lane) {
  const unsigned F = 0xffffffffu;
  const bool h4 = lane & 4;
  float a0 = h4 ? v4 : v0, a1 = h4 ? v5 : v1, a2 = h4 ? v6 : v2, a3 = h4 ? v7 : v3;
  const float b0 = h4 ? v0 : v4, b1 = h4 ? v1 : v5, b2 = h4 ? v2 : v6, b3 = h4 ? v3 : v7;
  a0 += __shfl_xor_sync(F, b0, 4);
  a1 += __shfl_xor_sync(F, b1, 4);
  a2 += __shfl_xor_sync(F, b2, 4);
  a3 += __shfl_xor_sync(F, b3, 4);
  const bool h2 = lane & 2;
  float c0 = h2 ? a2 : a0, c1 = h2 ? a3 : a1;
  const float d0 = h2 ? a0 : a2, d1 = h2 ? a1 : a3;
  c0 += __shfl_xor_sync(F, d0, 2);
  c1 += __shfl_xor_sync(F, d1, 2);
  const bool h1 = lane & 1;
  float k = h1 ? c1 : c0;
  const float e = h1 ? c0 : c1;
  k += __shfl_xor_sync(F, e, 1);
  k += __shfl_xor_sync(F, k, 8);
  k += __shfl_xor_sync(F, k, 16);
  return k;
}

// rtrnmc's table index of an optical depth (rrtmg_lw_rtrnmc.f90:385-388):
// itr = int(tblint * od / (bpade + od) + 0.5), within 0 .. ntbl
__device__ __forceinline__ int tbl_index(float od) {
  const float tblind = __fdividef(od, BPADE + od);
  const int itr = (int)fmaf(10000.0f, tblind, 0.5f);
  return itr < 0 ? 0 : (itr > 10000 ? 10000 : itr);
}
// (exp_tbl, tfn_tbl) and tau_tbl at an index (rrtmg_lw_init.f90:120-142,
// computed in double precision at set-up and stored as float)
__device__ __forceinline__ float2 tbl_tt(const float* __restrict__ T, int itr) {
  return __ldg(reinterpret_cast<const float2*>(T + c_T.tbl_tt) + itr);
}
// tau_tbl at an index formed in registers, bpade * t / (1 - t) at t = itr /
// 10000 (1e10 at the last entry; rrtmg_lw_init.f90:120-142), instead of a
// table load that depends on the clear cell's lookup (fp32 arithmetic: within
// a few units in the last place of the fp64-built table's float)
__device__ __forceinline__ float tbl_tau(const float* __restrict__ T, int itr) {
  (void)T;
  const float t = (float)itr * 1.0e-4f;
  return itr >= 10000 ? 1.0e10f : BPADE * t / (1.0f - t);
}

// cldprmc's optical depth ciwp*abscoice + clwp*abscoliq of one cell
// (cldprmc.f90:194-266; the radius bounds are checked beforehand), from
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

// ================================================================== taumol
struct GasSmem {
  float* f;        // [NF][nl]   per-layer setcoef quantities
  int* iv;         // [NI][nl]
  float2* terms;   // [TGROUP][nl] gas-optics terms of the current band, term-major
  FracRec* frec;   // [nl] Planck-fraction records of the current band
  double* d;       // [ND][nl] fp64 column amounts of the binary species
  int* iscal;      // [4]: laytrop
};

__host__ __device__ inline size_t gas_smem_bytes(int nl) {
  return align16((size_t)(NF + NI) * nl * 4) + align16((size_t)nl * TGROUP * 8) + align16((size_t)nl * sizeof(FracRec)) +
         align16((size_t)ND * nl * 8) + 16;
}

__device__ inline GasSmem gas_carve(char* p, int nl) {
  GasSmem s;
  s.f = (float*)p;
  s.iv = (int*)(p + (size_t)NF * nl * 4);
  p += align16((size_t)(NF + NI) * nl * 4);
  s.terms = (float2*)p;
  p += align16((size_t)nl * TGROUP * 8);
  s.frec = (FracRec*)p;
  p += align16((size_t)nl * sizeof(FracRec));
  s.d = (double*)p;
  p += align16((size_t)ND * nl * 8);
  s.iscal = (int*)p;
  return s;
}

// Prologue of band b for one layer: the band-specific per-layer code
// (lw_gasoptics.cuh) writing the layer's terms and Planck-fraction record.
template <int b>
__device__ __forceinline__ void band_prologue(const GasSmem& s, int nl, int lay, bool lower, const float* T) {
  Cell c{s.f, s.iv, nl, lay, T, s.d};
  Terms t{s.terms + lay, nl, 0};
  FracRec r = prologue<b>(c, lower, t);
  t.pad(maxt(b), c_T.band[b - 1].sr);
  s.frec[lay] = r;
}

// taumol of band b for every layer of a column: the prologue of each layer,
// then one thread per (layer, g) cell gathering taug = sum w * table[row + g]
// (the band's term count and g-points are compile-time constants, so the
// gather loop is unrolled) and interpolating the Planck fraction.  Ends with
// a barrier.
template <int b, int NT>
__device__ __forceinline__ void gas_band(const GasSmem& s, int nl, int laytrop, const float* __restrict__ T,
                                         float* gt, float* gf) {
  constexpr int NG = ngb_const(b), G0 = g0_const(b), M = maxt(b);
  for (int lay = threadIdx.x; lay < nl; lay += NT) band_prologue<b>(s, nl, lay, lay < laytrop, T);
  __syncthreads();
  for (int cell = threadIdx.x; cell < nl * NG; cell += NT) {
    const int lay = cell / NG, gi = cell - lay * NG;
    const float2* tp = s.terms + lay;
    const float* Tg = T + gi;
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const float2 w = tp[k * nl];
      acc = fmaf(w.x, __ldg(Tg + __float_as_int(w.y)), acc);
    }
    if ((b == 4 || b == 7) && lay >= laytrop) acc *= gscale(b, gi);
    const FracRec fr = s.frec[lay];
    const float* fp = T + fr.off + gi;
    const float f0 = __ldg(fp);
    gt[lay * GB_NGPT + G0 + gi] = acc;
    gf[lay * GB_NGPT + G0 + gi] = fmaf(fr.fpl, __ldg(fp + NG) - f0, f0);
  }
  __syncthreads();
}

// taumol of one column by the whole block: taug and Planck fractions of every
// (layer, g) cell into the planes gt/gf ([nl][140] each).  Ends with a barrier.
template <int NT>
__device__ void gas_column(const LwArgs& a, long long icol, const GasSmem& s, float* gt, float* gf,
                           const float* __restrict__ T) {
  const int nl = a.nlay, tid = threadIdx.x;
  if (tid == 0) s.iscal[0] = 0;
  __syncthreads();
  // setcoef (rrtmg_lw_setcoef.f90:275-430) after inatm's column amounts
  // (rrtmg_lw_rad.f90:807-867), one thread per layer
  const float stpfac = 296.0f / 1013.0f;
  const float amd = 28.9660f, amw = 18.0160f;
  for (int lay = tid; lay < nl; lay += NT) {
    const double pd = in2(a.play, a.ld, icol, lay);
    const float pavel = (float)pd;
    const float tavel = (float)in2(a.tlay, a.ld, icol, lay);
    const double dpz = in2(a.plev, a.ld, icol, lay) - in2(a.plev, a.ld, icol, lay + 1);
    const float w1 = (float)in2(a.h2ovmr, a.ld, icol, lay);
    const float w2 = (float)in2(a.co2vmr, a.ld, icol, lay);
    const float w3 = (float)in2(a.o3vmr, a.ld, icol, lay);
    const float w4 = (float)in2(a.n2ovmr, a.ld, icol, lay);
    const float w6 = (float)in2(a.ch4vmr, a.ld, icol, lay);
    const float w7 = (float)in2(a.o2vmr, a.ld, icol, lay);
    const float amm = (1.0f - w1) * amd + w1 * amw;
    const float coldry = (float)dpz * 1.e3f * (float)c_T.avogad / (1.e2f * (float)c_T.grav * amm * (1.0f + w1));
    const float summol = w2 + w3 + w4 + 0.0f + w6 + w7;
    const float wbrodl = coldry * (1.0f - summol);
    const float wk1 = coldry * w1, wk2 = coldry * w2, wk3 = coldry * w3, wk4 = coldry * w4, wk6 = coldry * w6,
                wk7 = coldry * w7;
    float* F = s.f;
    auto put = [&](int k, float v) { F[k * nl + lay] = v; };
    put(F_COLDRY, coldry);
    put(F_PAVEL, pavel);
    put(F_WX1, coldry * (float)in2(a.ccl4vmr, a.ld, icol, lay) * 1.e-20f);
    put(F_WX2, coldry * (float)in2(a.cfc11vmr, a.ld, icol, lay) * 1.e-20f);
    put(F_WX3, coldry * (float)in2(a.cfc12vmr, a.ld, icol, lay) * 1.e-20f);
    put(F_WX4, coldry * (float)in2(a.cfc22vmr, a.ld, icol, lay) * 1.e-20f);
    const float plog = __logf(pavel);
    const bool lower = lower_atmosphere(pd, plog);
    // The truncations jp, jt, jt1 (setcoef.f90:276-306) are taken in fp32 and
    // re-taken in fp64, as the reference computes them, where the fp32 value
    // lies near an integer.
    const double td = in2(a.tlay, a.ld, icol, lay);
    const float xjp = 36.0f - 5.0f * (plog + 0.04f);
    int jp = (int)xjp;
    if (fabsf(xjp - rintf(xjp)) < 2.0e-3f) jp = (int)(36.0 - 5 * (log(pd) + 0.04));
    jp = clampi(jp, 1, 58);
    jp = lower ? (jp > 12 ? 12 : jp) : (jp < 13 ? 13 : jp);
    const float fp = 5.0f * (__ldg(T + c_T.ref_preflog + jp - 1) - plog);
    const float dt0 = (tavel - __ldg(T + c_T.ref_tref + jp - 1)) / 15.0f;
    int jt = (int)(3.0f + dt0);
    if (fabsf(3.0f + dt0 - rintf(3.0f + dt0)) < 1.0e-4f) jt = (int)(3.0 + (td - c_T.tref64[jp - 1]) / 15.0);
    jt = clampi(jt, 1, 4);
    const float ft = dt0 - (float)(jt - 3);
    const float dt1 = (tavel - __ldg(T + c_T.ref_tref + jp)) / 15.0f;
    int jt1 = (int)(3.0f + dt1);
    if (fabsf(3.0f + dt1 - rintf(3.0f + dt1)) < 1.0e-4f) jt1 = (int)(3.0 + (td - c_T.tref64[jp]) / 15.0);
    jt1 = clampi(jt1, 1, 4);
    const float ft1 = dt1 - (float)(jt1 - 3);
    // fp64 column amounts of the binary species (inatm :807-867, setcoef.f90:349-362)
    {
      const double amd64 = 28.9660, amw64 = 18.0160;
      const double h = in2(a.h2ovmr, a.ld, icol, lay);
      const double amm64 = (1.0 - h) * amd64 + h * amw64;
      const double cd = dpz * 1.e3 * c_T.avogad / (1.e2 * c_T.grav * amm64 * (1.0 + h));
      auto col = [&](const double* v) {
        const double x = 1.e-20 * (cd * in2(v, a.ld, icol, lay));
        return x == 0.0 ? 1.e-32 * cd : x;
      };
      s.d[D_H2O * nl + lay] = 1.e-20 * (cd * h);
      s.d[D_CO2 * nl + lay] = col(a.co2vmr);
      s.d[D_O3 * nl + lay] = col(a.o3vmr);
      s.d[D_N2O * nl + lay] = col(a.n2ovmr);
      s.d[D_CH4 * nl + lay] = col(a.ch4vmr);
    }
    const float water = wk1 / coldry;
    const float scalefac = pavel * stpfac / tavel;
    const float forfac = scalefac / (1.0f + water);
    float forfrac, selffrac = 0.0f;
    int indfor, indself = 1;
    // truncations of temperature factors, re-taken in fp64 near an integer
    auto trunc_t = [&](float f32, double num64, double den) {
      return fabsf(f32 - rintf(f32)) < 1.0e-4f ? (int)(num64 / den) : (int)f32;
    };
    if (lower) {
      float factor = (332.0f - tavel) / 36.0f;
      indfor = min(2, max(1, trunc_t(factor, 332.0 - td, 36.0)));
      forfrac = factor - (float)indfor;
      factor = (tavel - 188.0f) / 7.2f;
      indself = min(9, max(1, trunc_t(factor, td - 188.0, 7.2) - 7));
      selffrac = factor - (float)(indself + 7);
    } else {
      const float factor = (tavel - 188.0f) / 36.0f;
      indfor = 3;
      forfrac = factor - 1.0f;
    }
    const float selffac = water * forfac;
    const float scaleminor = pavel / tavel;
    const float scaleminorn2 = scaleminor * (wbrodl / (coldry + wk1));
    const float factor = (tavel - 180.8f) / 7.2f;
    const int indminor = min(18, max(1, trunc_t(factor, td - 180.8, 7.2)));
    const float minorfrac = factor - (float)indminor;
    const float colh2o = 1.e-20f * wk1;
    float colco2 = 1.e-20f * wk2, colo3 = 1.e-20f * wk3, coln2o = 1.e-20f * wk4, colco = 0.0f;
    float colch4 = 1.e-20f * wk6;
    const float colo2 = 1.e-20f * wk7;
    if (colco2 == 0.0f) colco2 = 1.e-32f * coldry;
    if (colo3 == 0.0f) colo3 = 1.e-32f * coldry;
    if (coln2o == 0.0f) coln2o = 1.e-32f * coldry;
    if (colco == 0.0f) colco = 1.e-32f * coldry;
    if (colch4 == 0.0f) colch4 = 1.e-32f * coldry;
    const float compfp = 1.0f - fp;
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
    if (lower) atomicAdd(&s.iscal[0], 1);  // laytrop (the transfer checks that these form a prefix)
  }
  __syncthreads();
  const int laytrop = s.iscal[0];
  gas_band<1, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<2, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<3, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<4, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<5, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<6, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<7, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<8, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<9, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<10, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<11, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<12, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<13, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<14, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<15, NT>(s, nl, laytrop, T, gt, gf);
  gas_band<16, NT>(s, nl, laytrop, T, gt, gf);
}

// ================================================================== transfer
// Shared memory of one column: a fixed header, one 384-byte record per
// layer (so that every per-layer access in the loops is base + layer * 384
// + a constant), then the per-warp level sums.
struct RtHead {
  float misc[64];         // secdiff[16], plankbnd[16], dplankbnd[16], semiss[16]
  float red[2 * RT_NW];   // per-warp column sums for pwvcm
  int iscal[4];           // stop code, lower-layer count
  int pad[2];
};
struct RtLayer {
  float4 rec[16];     // per band: Planck value of the layer, level-minus-layer Planck below and
                      // above (dplankdn, dplankup), aerosol optical depth
  float tcl[16];      // fused clouds: cloud optical depth per band; caller sub-columns: the
                      // first five words are fbits (bit g: cldfmcl neither 0 nor 1); band
                      // clouds: secdiff(ib) * taucloud per cloud band ib (rtrn's odcld)
  int cldlay;         // 1: a cell of the layer has cldfmc == 1 (rtrnmc's icldlyr), or band
                      // clouds: cldfrac >= 1e-6; in the first phase: 1 where the layer is in
                      // the lower atmosphere
  int lfl;            // cloud flags of the layer (bits 0-2) and cldprmc's stop code (bits
                      // 8..); band clouds: istcld (bit 0) and istcldd (bit 1) of rtrnmr
  // McICA clouds use the words below as named; band clouds overlay them with
  // 14 floats (RtSmem::ovl): cldfrac, rtrnmr's upward overlap factors at lev+1
  // (facclr1, facclr2, faccld1, faccld2, faccmb1, faccmb2) and the downward
  // ones at lev-1, in that order
  unsigned cbits[5];  // bit g set where the cell is cloudy (cldfmc == 1)
  int pad0;
  long long cthr;     // fused clouds: McICA threshold 1 - cldf as double bits
  long long pad1;
  float4 lcw;         // (ciwp, clwp, radice, radliq) as floats
};
static_assert(sizeof(RtHead) == 320 && sizeof(RtLayer) == 384, "transfer shared-memory records");
static_assert(offsetof(RtLayer, lcw) + sizeof(float4) - offsetof(RtLayer, cbits) == 14 * sizeof(float),
              "band-cloud overlay of the McICA words");

struct RtSmem {
  RtHead* h;
  RtLayer* L;   // [nl]; in the last phase: fp64 net fluxes [nl+1][2]
  float* part;  // [RT_NW][nl+1][6] per-warp level sums: dn, dn clear, up, up clear, dup/dT,
                // dup clear/dT; in the first phase: float4 per level, the Planck-table row and
                // fraction of tlev and tlay
  __device__ __forceinline__ unsigned* fbits(int lay) const { return reinterpret_cast<unsigned*>(L[lay].tcl); }
  __device__ __forceinline__ float* ovl(int lay) const { return reinterpret_cast<float*>(L[lay].cbits); }
};

__host__ __device__ inline size_t rt_layers_bytes(int nl) {
  const size_t layers = (size_t)(nl < 1 ? 1 : nl) * sizeof(RtLayer);
  return layers > (size_t)(nl + 1) * 16 ? layers : (size_t)(nl + 1) * 16;
}
__host__ __device__ inline size_t rt_smem_bytes(int nl) {
  return sizeof(RtHead) + rt_layers_bytes(nl) + align16((size_t)RT_NW * (nl + 1) * 6 * 4);
}

__device__ inline RtSmem rt_carve(char* p, int nl) {
  RtSmem s;
  s.h = (RtHead*)p;
  p += sizeof(RtHead);
  s.L = (RtLayer*)p;
  p += rt_layers_bytes(nl);
  s.part = (float*)p;
  return s;
}

// Where taug and the Planck fractions of a column come from.
struct GasSrc {
  const float* gt;            // fp32 planes [nl][140] (taumol), or NULL
  const float* gf;
  float* gc;                  // caller sub-columns: the cells' cloud plane [nl][140], or NULL
  const __half* nt;           // fp16 rows [nl][140] (network), or NULL
  const __half* nf;
  const unsigned char* flag;  // per layer: 1 -> network, 0 -> fp32 planes
};
enum RtMode { RT_GAS = 0, RT_NET = 1, RT_MIX = 2 };

template <int MODE>
__device__ __forceinline__ bool layer_on_net(const GasSrc& src, int lay) {
  if (MODE == RT_GAS) return false;
  if (MODE == RT_NET) return true;
  return src.flag[lay] != 0;
}

template <int MODE>
__device__ __forceinline__ void gas_at(const GasSrc& src, bool net, int lay, int g, float& tg, float& pf) {
  const int o = lay * GB_NGPT + g;
  if (MODE != RT_GAS && net) {
    tg = __half2float(__ldg(src.nt + o));
    pf = __half2float(__ldg(src.nf + o));
  } else {
    tg = src.gt[o];  // plain loads: taumol wrote these planes in the same launch
    pf = src.gf[o];
  }
}

// Clear-sky layer transmittance and source factor of a cell: rtrnmc's
// odepth <= 0.06 expansion or its table lookup (rtrnmc.f90:380-413).  x is
// odepth/6 or tfn; the source from level Planck values is
// plfrac * (blay + x * dplank).  itr is the table index (used above 0.06).
struct Clr {
  float atrans, x;
  int itr;
  bool thin;
};
__device__ __forceinline__ Clr clear_cell(const float* __restrict__ T, float od) {
  Clr c;
  c.thin = od <= 0.06f;
  c.itr = tbl_index(od);
  const float2 e = tbl_tt(T, c.itr);  // looked up for every cell (branch-free), used above 0.06
  c.atrans = c.thin ? fmaf(-0.5f * od, od, od) : 1.0f - e.x;
  c.x = c.thin ? REC_6 * od : e.y;
  return c;
}

// Total (gas + cloud) absorptance and source factor of a cloudy cell
// (rtrnmc.f90:356-379): the expansion below 0.06, else the table at the
// clear cell's optical depth (odepth itself below 0.06, else tau_tbl at its
// index) plus the cloud's.
__device__ __forceinline__ void cloud_total(const float* __restrict__ T, const Clr& c, float od, float odcld,
                                            float& atot, float& x) {
  const float odtot = od + odcld;
  if (odtot < 0.06f) {
    atot = fmaf(-0.5f * odtot, odtot, odtot);
    x = REC_6 * odtot;
  } else {
    const float tauq = c.thin ? od : tbl_tau(T, c.itr);
    const float2 et = tbl_tt(T, tbl_index(tauq + odcld));
    atot = 1.0f - et.x;
    x = et.y;
  }
}

// McICA cloud of a cell flagged cloudy in the layer bits: returns cldfmc and
// sets the cloud optical depth along the diffusivity angle and its
// absorptance (cldprmc.f90:178-266, rtrnmc.f90:300-312); a fractional
// cldfmc (caller sub-columns only) enters with zero cloud optical depth.
__device__ __forceinline__ float cell_cloud(const LwArgs& a, const RtSmem& S, long long icol, int g, int lay,
                                            int band, float secdiff, bool one, const float* __restrict__ T,
                                            float& odcld, float& efcl) {
  odcld = 0.0f;
  efcl = 0.0f;
  if (a.cloud_mode == LW_CLOUD_FUSED) {
    odcld = secdiff * S.L[lay].tcl[band];
    efcl = 1.0f - __expf(-odcld);
    return 1.0f;
  }
  const long long o = (long long)g + GB_NGPT * (icol + (long long)a.ld * lay);
  if (!one) return (float)__ldg(a.cldfmcl + o);
  const double ciwp = __ldg(a.ciwpmcl + o), clwp = __ldg(a.clwpmcl + o);
  // the optical depth from this cell's water paths and the layer's radii, or the caller's taucmcl
  float tauc = 0.0f;
  bool from_paths = a.inflag == 2 && ciwp + clwp >= 1.e-20;
  if (!from_paths) {
    const double tin = __ldg(a.taucmcl + o);
    const long long tb = __double_as_longlong(tin);
    from_paths = a.inflag == 2 && tb >= __double_as_longlong(1.0e-20) && tb <= 0x7FF0000000000000LL;
    tauc = (float)tin;
  }
  if (from_paths) {
    const int fl = ((__double_as_longlong(ciwp) << 1) != 0LL ? 1 : 0) | ((__double_as_longlong(clwp) << 1) != 0LL ? 2 : 0);
    const float4 r = S.L[lay].lcw;
    tauc = cloud_tau_layer(a, band, T, make_float4((float)ciwp, (float)clwp, r.z, r.w), fl);
  }
  odcld = secdiff * tauc;
  efcl = 1.0f - __expf(-odcld);
  return 1.0f;
}

// a caller sub-column cell's cloud value for the transfer: its cloud optical
// depth (cldprmc.f90:178-266, formed as cell_cloud does) where cldfmcl = 1,
// the fraction itself where it is neither 0 nor 1
__device__ __forceinline__ float cell_value(const LwArgs& a, const RtSmem& S, int lay, int band, bool one,
                                            double cf, double ciwp, double clwp, double tin,
                                            const float* __restrict__ T) {
  if (!one) return (float)cf;
  float tauc = 0.0f;
  bool from_paths = a.inflag == 2 && ciwp + clwp >= 1.e-20;
  if (!from_paths) {
    const long long tb = __double_as_longlong(tin);
    from_paths = a.inflag == 2 && tb >= __double_as_longlong(1.0e-20) && tb <= 0x7FF0000000000000LL;
    tauc = (float)tin;
  }
  if (from_paths) {
    const int fl = ((__double_as_longlong(ciwp) << 1) != 0LL ? 1 : 0) | ((__double_as_longlong(clwp) << 1) != 0LL ? 2 : 0);
    const float4 r = S.L[lay].lcw;
    tauc = cloud_tau_layer(a, band, T, make_float4((float)ciwp, (float)clwp, r.z, r.w), fl);
  }
  return tauc;
}

// the transfer's cloud of a caller sub-column cell from its hand-over value
__device__ __forceinline__ float cell_from_value(bool one, float v, float secdiff, float& odcld, float& efcl) {
  if (!one) {
    odcld = 0.0f;
    efcl = 0.0f;
    return v;
  }
  odcld = secdiff * v;
  efcl = 1.0f - __expf(-odcld);
  return 1.0f;
}

// radius checks of cldprmc (cldprmc.f90:217-266): the code it stops with for
// ice radius `rice` (iceflag) and liquid radius `rliq` (liqflag)
__device__ __forceinline__ int ice_code(int iceflag, double rice) {
  if (iceflag == 0 && rice < 10.0) return GB_COL_ICE_SMALL;
  if (iceflag == 1 && (rice < 13.0 || rice > 130.0)) return GB_COL_ICE_BOUNDS;
  if (iceflag == 2 && (rice < 5.0 || rice > 131.0)) return GB_COL_ICE_BOUNDS;
  if (iceflag == 3 && (rice < 5.0 || rice > 140.0)) return GB_COL_DGE_BOUNDS;
  return 0;
}
__device__ __forceinline__ int liq_code(int liqflag, double rliq) {
  return liqflag == 1 && (rliq < 2.5 || rliq > 60.0) ? GB_COL_LIQ_BOUNDS : 0;
}

// rtrnmr's maximum/random overlap factors (rrtmg_lw_rtrnmr.f90:345-514), by
// one thread in fp64 from the layer fractions cf[0 .. nl-1]; lev is the
// reference's 1-based layer.  The fractions beyond the column (lev 0 and
// nl+1) are 0: the driver's cloud array is zeroed above the column
// (nomcica.f90 inatm), and below it the reference reads outside its array,
// where the surface (no cloud) is taken.  faccmb, which the reference leaves
// undefined where istcld = 1, is 0 there.  Layer lev keeps its istcld
// (istcldd) in bit 0 (1) of lfl, the upward factors at lev+1 in ovl[1..6]
// and the downward ones at lev-1 in ovl[7..12].
__device__ __noinline__ void band_overlap(const RtSmem& S, const double* __restrict__ cf, int nl) {
  auto CF = [&](int lev) -> double { return lev >= 1 && lev <= nl ? cf[lev - 1] : 0.0; };
  auto cloudy = [&](int lev) { return S.L[lev - 1].cldlay != 0; };
  enum { CLR1 = 0, CLR2, CLD1, CLD2, CMB1, CMB2 };
  double rat1 = 0.0, rat2 = 0.0;
  int st = 1;  // istcld(lev)
  for (int lev = 1; lev <= nl; ++lev) {
    if (st) S.L[lev - 1].lfl |= 1;
    float* u = S.ovl(lev - 1) + 1;  // factors at lev+1
    if (!cloudy(lev)) {
      st = 1;
      continue;
    }
    double f[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const double c0 = CF(lev), cp = CF(lev + 1), cm = CF(lev - 1);
    if (lev == nl) {
      // all six 0
    } else if (cp >= c0) {
      if (st) {
        if (c0 < 1.0) f[CLR2] = (cp - c0) / (1.0 - c0);
        if (lev >= 2) S.ovl(lev - 2)[1 + CLR2] = S.ovl(lev - 2)[1 + CLD2] = 0.0f;  // facclr2(lev), faccld2(lev)
      } else {
        const double fmax = c0 > cm ? c0 : cm;
        if (cp > fmax) {
          f[CLR1] = rat2;
          f[CLR2] = (cp - fmax) / (1.0 - fmax);
        } else if (cp < fmax) {
          f[CLR1] = (cp - c0) / (cm - c0);
        } else {
          f[CLR1] = rat2;
        }
      }
      if (f[CLR1] > 0.0 || f[CLR2] > 0.0) {
        rat1 = 1.0;
        rat2 = 0.0;
      } else {
        rat1 = rat2 = 0.0;
      }
    } else {
      if (st) {
        f[CLD2] = (c0 - cp) / c0;
        if (lev >= 2) S.ovl(lev - 2)[1 + CLR2] = S.ovl(lev - 2)[1 + CLD2] = 0.0f;
      } else {
        const double fmin = c0 < cm ? c0 : cm;
        if (cp <= fmin) {
          f[CLD1] = rat1;
          f[CLD2] = (fmin - cp) / fmin;
        } else {
          f[CLD1] = (c0 - cp) / (c0 - fmin);
        }
      }
      if (f[CLD1] > 0.0 || f[CLD2] > 0.0) {
        rat1 = 0.0;
        rat2 = 1.0;
      } else {
        rat1 = rat2 = 0.0;
      }
    }
    if (!st) {
      f[CMB1] = fmax(0.0, fmin(cp - c0, cm - c0));
      f[CMB2] = fmax(0.0, fmin(c0 - cp, c0 - cm));
    }
    for (int k = 0; k < 6; ++k) u[k] = (float)f[k];
    st = 0;
  }
  int sd = 1;  // istcldd(lev); rat1 and rat2 carry over from the loop above
  for (int lev = nl; lev >= 1; --lev) {
    if (sd) S.L[lev - 1].lfl |= 2;
    float* d = S.ovl(lev - 1) + 7;  // factors at lev-1
    if (!cloudy(lev)) {
      sd = 1;
      continue;
    }
    double f[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const double c0 = CF(lev), cp = CF(lev + 1), cm = CF(lev - 1);
    if (lev == 1) {
      // all six 0
    } else if (cm >= c0) {
      if (sd) {
        if (c0 < 1.0) f[CLR2] = (cm - c0) / (1.0 - c0);
        if (lev < nl) S.ovl(lev)[7 + CLR2] = S.ovl(lev)[7 + CLD2] = 0.0f;  // facclr2d(lev), faccld2d(lev)
      } else {
        const double fmax = c0 > cp ? c0 : cp;
        if (cm > fmax) {
          f[CLR1] = rat2;
          f[CLR2] = (cm - fmax) / (1.0 - fmax);
        } else if (cm < fmax) {
          f[CLR1] = (cm - c0) / (cp - c0);
        } else {
          f[CLR1] = rat2;
        }
      }
      if (f[CLR1] > 0.0 || f[CLR2] > 0.0) {
        rat1 = 1.0;
        rat2 = 0.0;
      } else {
        rat1 = rat2 = 0.0;
      }
    } else {
      if (sd) {
        f[CLD2] = (c0 - cm) / c0;
        if (lev < nl) S.ovl(lev)[7 + CLR2] = S.ovl(lev)[7 + CLD2] = 0.0f;
      } else {
        const double fmin = c0 < cp ? c0 : cp;
        if (cm <= fmin) {
          f[CLD1] = rat1;
          f[CLD2] = (fmin - cm) / fmin;
        } else {
          f[CLD1] = (c0 - cm) / (c0 - fmin);
        }
      }
      if (f[CLD1] > 0.0 || f[CLD2] > 0.0) {
        rat1 = 0.0;
        rat2 = 1.0;
      } else {
        rat1 = rat2 = 0.0;
      }
    }
    if (!sd) {
      f[CMB1] = fmax(0.0, fmin(cp - c0, cm - c0));
      f[CMB2] = fmax(0.0, fmin(c0 - cp, c0 - cm));
    }
    for (int k = 0; k < 6; ++k) d[k] = (float)f[k];
    sd = 0;
  }
}

// The band clouds of the non-McICA driver (nomcica.f90:886-920, rtrn.f90:319-336,
// rtrnmr.f90:334-343): per layer the fraction, icldlyr (cldfrac >= 1e-6) and
// odcld = secdiff(ib) * taucloud(ib) for the cloud bands ib < ncbands, then
// for maximum/random overlap the overlap factors.  Ends with a barrier when
// it computes them.
__device__ __forceinline__ void band_clouds(const LwArgs& a, long long icol, const RtSmem& S, int nl, bool clouds) {
  const int tid = threadIdx.x;
  if (!clouds) {
    for (int lay = tid; lay < nl; lay += RT_NT) S.L[lay].cldlay = 0;
    return;
  }
  // fp64 fractions for the overlap factors, after the Planck-table rows of the first phase
  double* cf64 = reinterpret_cast<double*>(S.part + 4 * (nl + 1));
  const int ncb = __ldg(a.ncbands + icol);
  if (tid == 0) S.h->iscal[2] = ncb;
  for (int lay = tid; lay < nl; lay += RT_NT) {
    const double cf = in2(a.cldfrac, a.ld, icol, lay);
    S.L[lay].cldlay = cf >= 1.e-6;
    S.L[lay].lfl = 0;
    float* ov = S.ovl(lay);
    ov[0] = (float)cf;
#pragma unroll
    for (int k = 1; k < 14; ++k) ov[k] = 0.0f;
    cf64[lay] = cf;
  }
  for (int it = tid; it < nl * 16; it += RT_NT) {
    const int lay = it >> 4, ib = it & 15;
    S.L[lay].tcl[ib] = ib < ncb ? S.h->misc[ib] * (float)__ldg(a.tauc + ib + 16 * (icol + a.ld * lay)) : 0.0f;
  }
  if (a.icld >= 2) {
    __syncthreads();
    if (tid == 0) band_overlap(S, cf64, nl);
  }
}

// cloud band of spectral band `band` for cldprop's band count (rtrn.f90:253-255, 345-351)
__device__ __forceinline__ int cloud_band(int ncb, int band) {
  if (ncb == 1) return 0;
  if (ncb == 5) return band < 1 ? 0 : band < 2 ? 1 : band < 5 ? 2 : band < 8 ? 3 : 4;
  return band;
}

// The transfer of one column by the block (see the file header).  RT_NET: a
// column with any layer off the network is not solved (returns false in
// every thread).  BAND: the non-McICA driver's band clouds (random overlap
// for icld 1, maximum/random otherwise).  Ends with a barrier.
template <int MODE, bool BAND = false>
__device__ bool rt_column(const LwArgs& a, long long icol, const RtSmem& S, const GasSrc& src,
                          const float* __restrict__ T) {
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nl = a.nlay;
  const bool fused = a.cloud_mode == LW_CLOUD_FUSED;
  const bool clouds = a.icld >= 1;
  if (MODE == RT_NET) {
    int off = src.flag == nullptr;
    for (int l = tid; l < nl && !off; l += RT_NT) off = src.flag[l] == 0;
    if (__syncthreads_or(off)) return false;
  }
  if (tid < 4) S.h->iscal[tid] = 0;
  // this thread's g-point, its band and flux weight (read from the table blob:
  // a constant-bank lookup indexed by the thread would be re-issued in the
  // loops wherever the compiler does not keep the value in a register)
  const bool live = tid < GB_NGPT;
  const int g = live ? tid : GB_NGPT - 1;
  const int band = __float_as_int(__ldg(T + c_T.gpt_band + g));
  const float wgt = live ? __ldg(T + c_T.gpt_wgt + g) : 0.0f;
  __syncthreads();

  // ---------------- per layer: inatm's column amounts (pwvcm), value checks, laytrop, Planck rows
  const float amd = 28.9660f, amw = 18.0160f;
  float amttl = 0.0f, wvttl = 0.0f;
  int bad = 0;
  float4* prow = reinterpret_cast<float4*>(S.part);
  for (int lay = tid; lay < nl; lay += RT_NT) {
    const double pd = in2(a.play, a.ld, icol, lay);
    const float pavel = (float)pd;
    const float tavel = (float)in2(a.tlay, a.ld, icol, lay);
    const double dpz = in2(a.plev, a.ld, icol, lay) - in2(a.plev, a.ld, icol, lay + 1);
    const float w1 = (float)in2(a.h2ovmr, a.ld, icol, lay);
    const float tz = (float)in2(a.tlev, a.ld, icol, lay);
    const float amm = (1.0f - w1) * amd + w1 * amw;
    const float coldry = (float)dpz * 1.e3f * (float)c_T.avogad / (1.e2f * (float)c_T.grav * amm * (1.0f + w1));
    const float wk1 = coldry * w1;
    amttl += coldry + wk1;
    wvttl += wk1;
    if (!(pavel > 0.0f) || !(tavel > 0.0f) || !isfinite(pavel) || !isfinite(tavel)) bad = 1;
    const bool lower = lower_atmosphere(pd, __logf(pavel));
    S.L[lay].cldlay = lower;
    if (lower) atomicAdd(&S.h->iscal[1], 1);
    // Planck-table rows of the level below and of the layer (setcoef.f90:173-269)
    const int ind = clampi((int)(tz - 159.0f), 1, 180);
    const int il = clampi((int)(tavel - 159.0f), 1, 180);
    prow[lay] = make_float4(__int_as_float(ind), tz - 159.0f - (float)ind, __int_as_float(il), tavel - 159.0f - (float)il);
    if (lay == nl - 1) {
      const float tt = (float)in2(a.tlev, a.ld, icol, nl);
      const int it = clampi((int)(tt - 159.0f), 1, 180);
      prow[nl] = make_float4(__int_as_float(it), tt - 159.0f - (float)it, 0.0f, 0.0f);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {  // fixed-order sums: within the warp, then over the warps in order
    amttl += __shfl_xor_sync(FULL, amttl, o);
    wvttl += __shfl_xor_sync(FULL, wvttl, o);
  }
  if (lane == 0) {
    S.h->red[2 * warp] = amttl;
    S.h->red[2 * warp + 1] = wvttl;
  }
  bad = __syncthreads_or(bad);
  // lower-atmosphere layers must form the prefix 0 .. laytrop-1
  const int laytrop = S.h->iscal[1];
  int notpre = 0;
  for (int lay = tid; lay < nl; lay += RT_NT) notpre |= S.L[lay].cldlay != (lay < laytrop ? 1 : 0);
  if (tid < 16) {
    // pwvcm (inatm :869-870) and secdiff (rtrnmc.f90:258-266), one band per thread
    const int ib = tid;
    float at = S.h->red[0], wt = S.h->red[1];
    for (int w = 1; w < RT_NW; ++w) {
      at += S.h->red[2 * w];
      wt += S.h->red[2 * w + 1];
    }
    const float wvsh = (amw * wt) / (amd * at);
    const float pz0 = (float)in2(a.plev, a.ld, icol, 0);
    const float pwvcm = wvsh * (1.e3f * pz0) / (1.e2f * (float)c_T.grav);
    float sd = 1.66f;
    if (!(ib == 0 || ib == 3 || ib >= 9)) {
      sd = c_a0[ib] + c_a1[ib] * __expf(c_a2[ib] * pwvcm);
      sd = fminf(fmaxf(sd, 1.50f), 1.80f);
    }
    S.h->misc[ib] = sd;
    // surface source and its temperature derivative (setcoef.f90:270-282)
    const float tb = (float)__ldg(a.tsfc + icol);
    const int ind = clampi((int)(tb - 159.0f), 1, 180);
    const float fr = tb - 159.0f - (float)ind;
    const float se = (float)__ldg(a.emis + icol + a.ld * ib);
    const float* tp = T + c_T.totplnk + ib * 181;
    const float* td = T + c_T.totplnkderiv + ib * 181;
    S.h->misc[16 + ib] = se * (tp[ind - 1] + fr * (tp[ind] - tp[ind - 1]));
    S.h->misc[32 + ib] = se * (td[ind - 1] + fr * (td[ind] - td[ind - 1]));
    S.h->misc[48 + ib] = se;
  }
  notpre = __syncthreads_or(notpre);
  // ---------------- per (layer, band): Planck values and the aerosol optical depth (rrtmg_lw_rad.f90:548-553)
#pragma unroll 2
  for (int it = tid; it < nl * 16; it += RT_NT) {
    const int lay = it >> 4, ib = it & 15;
    const float* tp = T + c_T.totplnk + ib * 181;
    const float4 r0 = prow[lay], r1 = prow[lay + 1];
    const int i0 = __float_as_int(r0.x), il = __float_as_int(r0.z), i1 = __float_as_int(r1.x);
    const float pdn = tp[i0 - 1] + r0.y * (tp[i0] - tp[i0 - 1]);
    const float pup = tp[i1 - 1] + r1.y * (tp[i1] - tp[i1 - 1]);
    const float blay = tp[il - 1] + r0.w * (tp[il] - tp[il - 1]);
    const float taua = (float)__ldg(a.tauaer + icol + a.ld * (lay + (long long)nl * ib));
    S.L[lay].rec[ib] = make_float4(blay, pdn - blay, pup - blay, taua);
  }
  // ---------------- clouds: the cells' McICA bits, cldprmc's optical depths and stop conditions
  int err = 0;
  if constexpr (BAND) {
    band_clouds(a, icol, S, nl, clouds);
  } else {
  for (int i = tid; i < nl * 5; i += RT_NT) {
    const int l = i / 5, w = i - 5 * l;
    S.L[l].cbits[w] = 0u;
    S.fbits(l)[w] = 0u;  // caller sub-columns
  }
  if (clouds && fused) {
    // per layer, once: the McICA threshold and the layer's cloud quantities
    for (int lay = tid; lay < nl; lay += RT_NT) {
      double cf = in2(a.cldfrac, a.ld, icol, lay);
      cf = cf < 1.0e-20 ? 0.0 : cf;  // mcica_subcol_gen_lw.f90:463-470
      // cdf >= 1 - cf, compared on the bit patterns (cdf is in [0, 1], so
      // for a threshold >= 0 the integer order is the floating-point order);
      // a negative threshold takes every cell, a NaN none
      const double thr = 1.0 - cf;
      S.L[lay].cthr = thr < 0.0 ? LLONG_MIN : (thr == thr ? __double_as_longlong(thr) : LLONG_MAX);
      const double ciwp = in2(a.ciwp, a.ld, icol, lay), clwp = in2(a.clwp, a.ld, icol, lay);
      const double rice = in2(a.reicmcl, a.ld, icol, lay), rliq = in2(a.relqmcl, a.ld, icol, lay);
      const int fl = (ciwp != 0.0 ? 1 : 0) | (clwp != 0.0 ? 2 : 0) | (ciwp + clwp >= 1.e-20 ? 4 : 0);
      int e = 0;
      if (ciwp != 0.0) e = ice_code(a.iceflag, rice);
      if (clwp != 0.0 && liq_code(a.liqflag, rliq)) e = GB_COL_LIQ_BOUNDS;
      S.L[lay].lfl = fl | (e << 8);
      S.L[lay].lcw = make_float4((float)ciwp, (float)clwp, (float)rice, (float)rliq);
    }
    // this g-point's draw (mcica_subcol_gen_lw.f90:484-512, icld 3) as a bit
    // pattern, and the warp's largest
    const long long cdb = __double_as_longlong(__ldg(a.draws + icol * GB_NGPT + g));
    long long mx = live ? cdb : LLONG_MIN;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long v = __shfl_xor_sync(FULL, mx, o);
      mx = v > mx ? v : mx;
    }
    __syncthreads();
    // cloudy cells: cdf(g) >= 1 - cldf(lay) (mcica_subcol_gen_lw.f90:650); a
    // layer whose threshold is above every draw of the warp has none there
    for (int lay = 0; lay < nl; ++lay) {
      const long long tb = S.L[lay].cthr;
      if (tb > mx) continue;
      const unsigned m = __ballot_sync(FULL, live && cdb >= tb);
      if (lane == 0) S.L[lay].cbits[warp] = m;
    }
    __syncthreads();
    for (int lay = tid; lay < nl; lay += RT_NT) {
      const unsigned* c = S.L[lay].cbits;
      S.L[lay].cldlay = (c[0] | c[1] | c[2] | c[3] | c[4]) != 0u;
    }
    __syncthreads();
    // cloud optical depth per (layer, band) where the band has a cloudy
    // sub-column (the values cldprmc computes for every such cell), and
    // cldprmc's stop conditions
    const long long kMin = __double_as_longlong(1.0e-20), kInf = 0x7FF0000000000000LL;
    for (int it = tid; it < nl * 16; it += RT_NT) {
      const int lay = it >> 4, ib = it & 15;
      if (!S.L[lay].cldlay) continue;
      const int g0 = c_T.band[ib].g0, ng = c_T.band[ib].ng;
      bool any = false;
      for (int k = g0; k < g0 + ng; ++k) any |= (S.L[lay].cbits[k >> 5] >> (k & 31)) & 1u;
      if (!any) continue;
      const double tin = __ldg(a.tauc + ib + 16 * (icol + a.ld * lay));
      const long long tinb = __double_as_longlong(tin);
      const bool tin_ok = tinb >= kMin && tinb <= kInf;  // tin >= 1e-20
      const int fl = S.L[lay].lfl;
      const bool cond = (fl & 4) || tin_ok;
      S.L[lay].tcl[ib] = a.inflag == 2 && cond ? cloud_tau_layer(a, ib, T, S.L[lay].lcw, fl) : (float)tin;
      if (cond) {
        if (a.inflag == 1) err = GB_COL_INFLAG1;
        if (a.inflag == 2 && (fl >> 8)) err = fl >> 8;
      }
    }
  } else if (clouds) {
    // caller sub-columns: the layer radii as floats and the codes cldprmc's
    // radius checks stop with: bits 0-7 ice, 8-15 liquid
    for (int lay = tid; lay < nl; lay += RT_NT) {
      const double rice = in2(a.reicmcl, a.ld, icol, lay), rliq = in2(a.relqmcl, a.ld, icol, lay);
      S.L[lay].lfl = ice_code(a.iceflag, rice) | (liq_code(a.liqflag, rliq) << 8);
      S.L[lay].lcw = make_float4(0.0f, 0.0f, (float)rice, (float)rliq);
    }
    __syncthreads();
    // per layer, each warp: its 32 cldfmcl values tested on their bit
    // patterns: == 1, /= 0, >= 1e-20
    const long long kOne = 0x3FF0000000000000LL, kInf = 0x7FF0000000000000LL;
    const long long kMin = __double_as_longlong(1.0e-20);
#pragma unroll 8
    for (int lay = 0; lay < nl; ++lay) {
      const long long o = g + GB_NGPT * (icol + a.ld * lay);
      const long long cb = live ? __double_as_longlong(__ldg(a.cldfmcl + o)) : 0LL;
      const bool one = cb == kOne;
      const bool frac = !one && (cb << 1) != 0LL;  // neither +-0 nor 1 (NaN included, as /= 0 is)
      const unsigned m1 = __ballot_sync(FULL, one), mf = __ballot_sync(FULL, frac);
      if (lane == 0) {
        S.L[lay].cbits[warp] = m1;
        S.fbits(lay)[warp] = mf;
      }
    }
    __syncwarp();
    // then, per cell with a cloud (independent iterations, so that several
    // cells' loads are in flight): the water paths for cldprmc's checks and,
    // where the transfer has a cloud plane, the cell's optical depth formed
    // once instead of in both passes
    const unsigned mybit = 1u << lane;
#pragma unroll 4
    for (int lay = 0; lay < nl; ++lay) {
      const bool one = S.L[lay].cbits[warp] & mybit, frac = S.fbits(lay)[warp] & mybit;
      if (!(one || frac)) continue;
      const long long o = g + GB_NGPT * (icol + a.ld * lay);
      const double cfv = one ? 1.0 : __ldg(a.cldfmcl + o);
      const long long cb = __double_as_longlong(cfv);
      if (cb >= kMin && cb <= kInf) {  // cldfmc >= cldmin (cldprmc.f90:178)
        const double ciwp = __ldg(a.ciwpmcl + o), clwp = __ldg(a.clwpmcl + o);
        const double tin = __ldg(a.taucmcl + o);
        if (src.gc) src.gc[lay * GB_NGPT + g] = cell_value(a, S, lay, band, one, cfv, ciwp, clwp, tin, T);
        const long long tb = __double_as_longlong(tin);
        if (ciwp + clwp >= 1.e-20 || (tb >= kMin && tb <= kInf)) {
          const int e = S.L[lay].lfl;
          if (a.inflag == 1) err = GB_COL_INFLAG1;
          if (a.inflag == 2) {
            if ((__double_as_longlong(ciwp) << 1) != 0LL && (e & 0xff)) err = e & 0xff;  // ciwp /= 0
            if ((__double_as_longlong(clwp) << 1) != 0LL && (e >> 8)) err = e >> 8;      // clwp /= 0
          }
        }
      } else if (src.gc) {
        src.gc[lay * GB_NGPT + g] = (float)cfv;  // a fraction below cldmin: cldfmcl itself, no cloud optics
      }
    }
    __syncthreads();
    for (int lay = tid; lay < nl; lay += RT_NT) {
      const unsigned* c = S.L[lay].cbits;
      S.L[lay].cldlay = (c[0] | c[1] | c[2] | c[3] | c[4]) != 0u;
    }
  } else {
    for (int lay = tid; lay < nl; lay += RT_NT) S.L[lay].cldlay = 0;
  }
  }
  if (err) atomicMax(&S.h->iscal[0], err);
  __syncthreads();
  if (tid == 0) {
    err = S.h->iscal[0];
    if (notpre) err = GB_COL_LAYTROP;
    if (bad) err = GB_COL_BADVAL;
    if (BAND) {  // the column status already holds cldprop's code
      if (err) {
        if (a.col_err) atomicMax(a.col_err + icol, err);
        atomicMax(a.err_flag, err);
      }
    } else if (err) {
      if (a.col_err) a.col_err[icol] = err;
      atomicMax(a.err_flag, err);
    } else if (a.col_err) {
      a.col_err[icol] = 0;
    }
  }

  const float sd = S.h->misc[band];
  const unsigned bit = 1u << lane;
  const int cband = BAND ? cloud_band(S.h->iscal[2], band) : 0;
  const bool maxrand = BAND && a.icld >= 2;
  float cr = 0.0f, kr = 0.0f, radm = 0.0f;  // rtrnmr's cloudy and clear radiances and overlap term
  float* part = S.part + warp * (nl + 1) * 6;  // this warp's level sums

  // ---------------- downward pass (rtrnmc.f90:347-455): total and clear-sky streams
  // The next layer's gas optics are loaded while this one is done; the
  // level sums of two layers share one transposed butterfly.
  float rd = 0.0f, rc = 0.0f, f1 = 0.0f, tgn, pfn, p0 = 0.0f, p1 = 0.0f;
  const float* gcp = !BAND && clouds && !fused ? src.gc : nullptr;  // the cells' cloud values, if handed over
  float cvn = 0.0f;
  bool pend = false;  // a layer's weighted radiances wait in p0, p1 (the same in every lane)
  gas_at<MODE>(src, layer_on_net<MODE>(src, nl - 1), nl - 1, g, tgn, pfn);
  if (gcp) cvn = gcp[(nl - 1) * GB_NGPT + g];
  for (int lay = nl - 1; lay >= 0; --lay) {
    const float tg = tgn, pf = pfn, cv = cvn;
    if (lay > 0) {  // in flight meanwhile
      gas_at<MODE>(src, layer_on_net<MODE>(src, lay - 1), lay - 1, g, tgn, pfn);
      if (gcp) cvn = gcp[(lay - 1) * GB_NGPT + g];
    }
    const float4 r = S.L[lay].rec[band];
    const float od = fmaxf(sd * (tg + r.w), 0.0f);
    const Clr c = clear_cell(T, od);
    const float gsd = pf * fmaf(c.x, r.y, r.x) * c.atrans;
    const float tr = 1.0f - c.atrans;
    rc = fmaf(rc, tr, gsd);
    float A = tr, B = gsd;
    if (clouds && S.L[lay].cldlay) {
      if constexpr (BAND) {
        const float* ov = S.ovl(lay);
        const float cf = ov[0], odcld = S.L[lay].tcl[cband];
        float atot, x;
        cloud_total(T, c, od, odcld, atot, x);
        const float bbdtot = pf * fmaf(x, r.y, r.x);
        if (!maxrand) {  // rtrn.f90:370-432
          const float efcl = (1.0f - __expf(-odcld)) * cf;
          A = 1.0f - fmaf(efcl, 1.0f - c.atrans, c.atrans);
          B = fmaf(cf, fmaf(bbdtot, atot, -gsd), gsd);
        } else {  // rtrnmr.f90:590-609
          if (S.L[lay].lfl & 2) {
            cr = cf * rd;
            kr = rd - cr;
            radm = 0.0f;
          }
          const float ttot = 1.0f - atot, cldsrc = bbdtot * atot;
          cr = fmaf(cr, ttot, cf * cldsrc);
          kr = fmaf(kr, tr, (1.0f - cf) * gsd);
          A = 0.0f;
          B = cr + kr;
          const float radmod = fmaf(radm, fmaf(ov[7], tr, ov[9] * ttot), fmaf(ov[12], cldsrc, -ov[11] * gsd));
          const float oc = cr - radmod, ok = kr + radmod;
          radm = fmaf(ov[8], ok, fmaf(-ov[10], oc, -radmod));
          cr += radm;
          kr -= radm;
        }
      } else {
        const bool one = S.L[lay].cbits[warp] & bit;
        if (one || (!fused && (S.fbits(lay)[warp] & bit))) {
          float odcld, efcl, atot, x;
          const float cldf = gcp ? cell_from_value(one, cv, sd, odcld, efcl)
                                 : cell_cloud(a, S, icol, g, lay, band, sd, one, T, odcld, efcl);
          cloud_total(T, c, od, odcld, atot, x);
          A = 1.0f - fmaf(efcl, 1.0f - c.atrans, c.atrans);
          B = fmaf(cldf, fmaf(pf * fmaf(x, r.y, r.x), atot, -gsd), gsd);
        }
      }
    }
    rd = fmaf(rd, A, B);
    if (lay == 0) f1 = pf;
    if (pend) {  // lanes 0, 1: layer lay+1; lanes 2, 3: layer lay
      const float s = reduce4(p0, p1, rd * wgt, rc * wgt, lane);
      if (lane < 4) part[(lay + 1 - (lane >> 1)) * 6 + (lane & 1)] = s;
    } else {
      p0 = rd * wgt;
      p1 = rc * wgt;
    }
    pend = !pend;
  }
  if (pend) {  // layer 0 on its own
    const float s = reduce2(p0, p1, lane);
    if (lane < 2) part[lane] = s;
  }

  // ---------------- surface emission and reflection (rtrnmc.f90:465-485)
  const bool idrv = a.idrv == 1;
  const float rad0 = f1 * S.h->misc[16 + band];
  const float reflect = 1.0f - S.h->misc[48 + band];
  float ru = rad0 + reflect * rd;
  float rcu = rad0 + reflect * rc;
  float du = f1 * S.h->misc[32 + band];
  float dcu = du;
  if (idrv) {
    const float s = reduce4(ru * wgt, rcu * wgt, du * wgt, dcu * wgt, lane);
    if (lane < 4) part[2 + lane] = s;
  } else {
    const float s = reduce2(ru * wgt, rcu * wgt, lane);
    if (lane < 2) part[2 + lane] = s;
  }
  // ---------------- upward pass (rtrnmc.f90:486-529): level lay+1 above layer lay
  float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f, q3 = 0.0f;
  pend = false;  // a layer's weighted values wait in q0..q3
  gas_at<MODE>(src, layer_on_net<MODE>(src, 0), 0, g, tgn, pfn);
  if (gcp) cvn = gcp[g];
  for (int lay = 0; lay < nl; ++lay) {
    const float tg = tgn, pf = pfn, cv = cvn;
    if (lay + 1 < nl) {
      gas_at<MODE>(src, layer_on_net<MODE>(src, lay + 1), lay + 1, g, tgn, pfn);
      if (gcp) cvn = gcp[(lay + 1) * GB_NGPT + g];
    }
    const float4 r = S.L[lay].rec[band];
    const float od = fmaxf(sd * (tg + r.w), 0.0f);
    const Clr c = clear_cell(T, od);
    const float gsu = pf * fmaf(c.x, r.z, r.x) * c.atrans;
    const float tr = 1.0f - c.atrans;
    rcu = fmaf(rcu, tr, gsu);
    dcu *= tr;
    float A = tr, B = gsu, D = tr;
    if (clouds && S.L[lay].cldlay) {
      if constexpr (BAND) {
        const float* ov = S.ovl(lay);
        const float cf = ov[0], odcld = S.L[lay].tcl[cband];
        float atot, x;
        cloud_total(T, c, od, odcld, atot, x);
        const float bbutot = pf * fmaf(x, r.z, r.x);
        D = fmaf(cf, 1.0f - atot, (1.0f - cf) * (1.0f - c.atrans));
        if (!maxrand) {  // rtrn.f90:495-507
          const float efcl = (1.0f - __expf(-odcld)) * cf;
          A = 1.0f - fmaf(efcl, 1.0f - c.atrans, c.atrans);
          B = fmaf(cf, fmaf(bbutot, atot, -gsu), gsu);
        } else {  // rtrnmr.f90:688-713
          if (S.L[lay].lfl & 1) {
            cr = cf * ru;
            kr = ru - cr;
            radm = 0.0f;
          }
          const float ttot = 1.0f - atot, cldsrc = bbutot * atot;
          cr = fmaf(cr, ttot, cf * cldsrc);
          kr = fmaf(kr, tr, (1.0f - cf) * gsu);
          A = 0.0f;
          B = cr + kr;
          const float radmod = fmaf(radm, fmaf(ov[1], tr, ov[3] * ttot), fmaf(ov[6], cldsrc, -ov[5] * gsu));
          const float oc = cr - radmod, ok = kr + radmod;
          radm = fmaf(ov[2], ok, fmaf(-ov[4], oc, -radmod));
          cr += radm;
          kr -= radm;
        }
      } else {
        const bool one = S.L[lay].cbits[warp] & bit;
        if (one || (!fused && (S.fbits(lay)[warp] & bit))) {
          float odcld, efcl, atot, x;
          const float cldf = gcp ? cell_from_value(one, cv, sd, odcld, efcl)
                                 : cell_cloud(a, S, icol, g, lay, band, sd, one, T, odcld, efcl);
          cloud_total(T, c, od, odcld, atot, x);
          A = 1.0f - fmaf(efcl, 1.0f - c.atrans, c.atrans);
          B = fmaf(cldf, fmaf(pf * fmaf(x, r.z, r.x), atot, -gsu), gsu);
          D = fmaf(cldf, 1.0f - atot, (1.0f - cldf) * (1.0f - c.atrans));
        }
      }
    }
    ru = fmaf(ru, A, B);
    du *= D;
    if (pend) {  // levels lay (the layer below) and lay+1
      if (idrv) {
        const float s = reduce8(q0, q1, q2, q3, ru * wgt, rcu * wgt, du * wgt, dcu * wgt, lane);
        if (lane < 8) part[(lay + (lane >> 2)) * 6 + 2 + (lane & 3)] = s;
      } else {
        const float s = reduce4(q0, q1, ru * wgt, rcu * wgt, lane);
        if (lane < 4) part[(lay + (lane >> 1)) * 6 + 2 + (lane & 1)] = s;
      }
    } else {
      q0 = ru * wgt;
      q1 = rcu * wgt;
      q2 = du * wgt;
      q3 = dcu * wgt;
    }
    pend = !pend;
  }
  if (pend) {  // level nl on its own
    float* p = part + nl * 6 + 2;
    if (idrv) {
      const float s = reduce4(q0, q1, q2, q3, lane);
      if (lane < 4) p[lane] = s;
    } else {
      const float s = reduce2(q0, q1, lane);
      if (lane < 2) p[lane] = s;
    }
  }
  __syncthreads();

  // ---------------- fp64 outputs: fluxes, net fluxes, heating rates (rtrnmc.f90:566-592)
  const long long ldo = a.ldo;
  double* fnet = reinterpret_cast<double*>(S.L);  // [nl+1][2]
  for (int lev = tid; lev <= nl; lev += RT_NT) {
    // the five warps' fp32 partials summed without rounding error: Knuth's
    // two-sum keeps each addition's rounding error, and the sum and the
    // accumulated errors go to fp64 together
    double acc[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      float hi = S.part[lev * 6 + k], lo = 0.0f;
#pragma unroll
      for (int w = 1; w < RT_NW; ++w) {
        const float b = S.part[(w * (nl + 1) + lev) * 6 + k];
        const float sum = hi + b, bv = sum - hi;
        lo += (hi - (sum - bv)) + (b - bv);
        hi = sum;
      }
      acc[k] = (double)hi + (double)lo;
    }
    if (lev == nl) acc[0] = acc[1] = 0.0;  // no downward radiation at the model top
    const long long o = icol + ldo * lev;
    a.uflx[o] = acc[2];
    a.dflx[o] = acc[0];
    a.uflxc[o] = acc[3];
    a.dflxc[o] = acc[1];
    if (idrv) {
      a.duflx_dt[o] = acc[4];
      a.duflxc_dt[o] = acc[5];
    }
    fnet[lev * 2 + 0] = acc[2] - acc[0];
    fnet[lev * 2 + 1] = acc[3] - acc[1];
  }
  __syncthreads();
  for (int l = tid; l < nl; l += RT_NT) {
    const double dp = in2(a.plev, a.ld, icol, l) - in2(a.plev, a.ld, icol, l + 1);
    const double f = c_T.heatfac / dp;  // one division for both heating rates
    const long long o = icol + ldo * l;
    a.hr[o] = f * (fnet[l * 2] - fnet[(l + 1) * 2]);
    a.hrc[o] = f * (fnet[l * 2 + 1] - fnet[(l + 1) * 2 + 1]);
  }
  __syncthreads();
  return true;
}

// ------------------------------------------------------------------ kernels
__device__ __forceinline__ int grid_of(const LwBatch& B, long long gc, int gi) {
  while (gc >= B.col0[gi + 1]) ++gi;
  return gi;
}

// The column's grid arguments are copied into shared memory (the first
// ARGS_BYTES of every kernel's dynamic shared memory): the loops then read
// them as shared-memory broadcasts instead of constant-bank loads indexed by
// the grid number, which the compiler re-issues wherever it does not keep a
// field in a register.
constexpr size_t ARGS_BYTES = (sizeof(LwArgs) + 15) & ~size_t(15);
static_assert(sizeof(LwArgs) % 4 == 0, "LwArgs copied as 32-bit words");
__device__ __forceinline__ const LwArgs& stage_args(const LwArgs& a, char* smem) {
  __syncthreads();  // every thread is done with the previous column's copy
  int* dst = reinterpret_cast<int*>(smem);
  const int* src = reinterpret_cast<const int*>(&a);
  for (int k = threadIdx.x; k < (int)(sizeof(LwArgs) / 4); k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  return *reinterpret_cast<const LwArgs*>(smem);
}

// taumol over batch columns [c0, c1): column c0 + k into slot k.
template <int NT>
__global__ void __launch_bounds__(NT) lw_gas_kernel(const __grid_constant__ LwBatch B, const float* __restrict__ T,
                                                    long long c0, long long c1) {
  extern __shared__ __align__(16) char smem_raw[];
  const GasSmem s = gas_carve(smem_raw + ARGS_BYTES, B.nsmax);
  int gi = 0;
  for (long long i = c0 + blockIdx.x; i < c1; i += gridDim.x) {
    gi = grid_of(B, i, gi);
    const LwArgs& a = stage_args(B.g[gi], smem_raw);
    const long long slot = i - c0;
    gas_column<NT>(a, i - B.col0[gi], s, B.gtau + slot * B.gstride, B.gfrac + slot * B.gstride, T);
  }
}

// The transfer on the network's gas optics over batch columns [c0, c1), one
// block per column; a column with a layer off the network is appended to
// B.fall instead.
template <int MINB>
__global__ void __launch_bounds__(RT_NT, MINB) lw_rt_kernel(const __grid_constant__ LwBatch B,
                                                             const float* __restrict__ T, long long c0, long long c1) {
  extern __shared__ __align__(16) char smem_raw[];
  const RtSmem S = rt_carve(smem_raw + ARGS_BYTES, B.nsmax);
  int gi = 0;
  for (long long i = c0 + blockIdx.x; i < c1; i += gridDim.x) {
    gi = grid_of(B, i, gi);
    const LwArgs& a = stage_args(B.g[gi], smem_raw);
    const long long icol = i - B.col0[gi];
    GasSrc src{};
    const long long row = icol * a.nlay * GB_NGPT;
    src.nt = a.sur_tau ? a.sur_tau + row : nullptr;
    src.nf = a.sur_frac ? a.sur_frac + row : nullptr;
    src.flag = a.sur_flag ? a.sur_flag + icol * a.nlay : nullptr;
    const bool done = rt_column<RT_NET>(a, icol, S, src, T);
    if (!done && threadIdx.x == 0) B.fall[atomicAdd(B.nfall, 1u)] = i;
  }
}

// taumol and the transfer of a column in one block, taumol's planes in the
// block's own slot (which stays in L2).  LIST: the columns handed over by the
// network's transfer kernel (B.fall), each layer's gas optics from the
// network or from taumol; else batch columns [c0, c1).
template <int MINB, bool LIST>
__global__ void __launch_bounds__(RT_NT, MINB) lw_full_kernel(const __grid_constant__ LwBatch B,
                                                               const float* __restrict__ T, long long c0, long long c1) {
  extern __shared__ __align__(16) char smem_raw[];
  const GasSmem gs = gas_carve(smem_raw + ARGS_BYTES, B.nsmax);
  const RtSmem S = rt_carve(smem_raw + ARGS_BYTES, B.nsmax);  // used after taumol is done with the same memory
  float* gt = B.gtau + (long long)blockIdx.x * B.gstride;
  float* gf = B.gfrac + (long long)blockIdx.x * B.gstride;
  const long long n = LIST ? (long long)*B.nfall : c1;
  int gi = 0;
  for (long long i = (LIST ? 0 : c0) + blockIdx.x; i < n; i += gridDim.x) {
    const long long gc = LIST ? B.fall[i] : i;
    gi = grid_of(B, gc, LIST ? 0 : gi);  // the list is in no particular order
    const LwArgs& a = stage_args(B.g[gi], smem_raw);
    const long long icol = gc - B.col0[gi];
    gas_column<RT_NT>(a, icol, gs, gt, gf, T);
    GasSrc src{};
    src.gt = gt;
    src.gf = gf;
    src.gc = B.gcld ? B.gcld + (long long)blockIdx.x * B.gstride : nullptr;
    if (LIST && a.sur_flag) {
      const long long row = icol * a.nlay * GB_NGPT;
      src.nt = a.sur_tau + row;
      src.nf = a.sur_frac + row;
      src.flag = a.sur_flag + icol * a.nlay;
      rt_column<RT_MIX>(a, icol, S, src, T);
    } else {
      rt_column<RT_GAS>(a, icol, S, src, T);
    }
  }
}

// The fused taumol and transfer kernel for the non-McICA driver's band
// clouds (batch columns [c0, c1), block k in slot k).
template <int MINB>
__global__ void __launch_bounds__(RT_NT, MINB) lw_band_kernel(const __grid_constant__ LwBatch B,
                                                               const float* __restrict__ T, long long c0, long long c1) {
  extern __shared__ __align__(16) char smem_raw[];
  const GasSmem gs = gas_carve(smem_raw + ARGS_BYTES, B.nsmax);
  const RtSmem S = rt_carve(smem_raw + ARGS_BYTES, B.nsmax);
  float* gt = B.gtau + (long long)blockIdx.x * B.gstride;
  float* gf = B.gfrac + (long long)blockIdx.x * B.gstride;
  int gi = 0;
  for (long long i = c0 + blockIdx.x; i < c1; i += gridDim.x) {
    gi = grid_of(B, i, gi);
    const LwArgs& a = stage_args(B.g[gi], smem_raw);
    const long long icol = i - B.col0[gi];
    gas_column<RT_NT>(a, icol, gs, gt, gf, T);
    GasSrc src{};
    src.gt = gt;
    src.gf = gf;
    rt_column<RT_GAS, true>(a, icol, S, src, T);
  }
}

constexpr int GAS_NT = 128;      // threads of the taumol kernel
constexpr int BAND_MINB = 6;
constexpr int LIST_PER_SM = 2;   // hand-over kernel blocks per SM
constexpr int LIST_MINB = 6;

// compiled shapes (min blocks per SM for the register allocation, 160
// threads each); variant 0 is the default
#define GB_LW_VARIANTS(X) X(0, 6) X(1, 7) X(2, 5) X(3, 4)

}  // namespace gb

// ------------------------------------------------------------------ host side
namespace {

struct VariantInfo {
  int min_blocks;
  const void* fn;  // the kernel this shape launches
  cudaError_t (*launch)(const LwBatch&, const float*, long long, long long, int, size_t, cudaStream_t);
};

template <int MINB>
cudaError_t launch_full(const LwBatch& b, const float* T, long long c0, long long c1, int nblocks, size_t smem,
                        cudaStream_t st) {
  gb::lw_full_kernel<MINB, false><<<nblocks, gb::RT_NT, smem, st>>>(b, T, c0, c1);
  return cudaGetLastError();
}
template <int MINB>
cudaError_t launch_net(const LwBatch& b, const float* T, long long c0, long long c1, int nblocks, size_t smem,
                       cudaStream_t st) {
  gb::lw_rt_kernel<MINB><<<nblocks, gb::RT_NT, smem, st>>>(b, T, c0, c1);
  return cudaGetLastError();
}

// batches without a network: the fused taumol + transfer kernel; with a
// network: the transfer kernel on the network's outputs
#define GB_LW_FULL_ENTRY(i, mb) {mb, (const void*)gb::lw_full_kernel<mb, false>, launch_full<mb>},
#define GB_LW_NET_ENTRY(i, mb) {mb, (const void*)gb::lw_rt_kernel<mb>, launch_net<mb>},
const VariantInfo kVariants[] = {GB_LW_VARIANTS(GB_LW_FULL_ENTRY)};
const VariantInfo kLean[] = {GB_LW_VARIANTS(GB_LW_NET_ENTRY)};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
constexpr int kMaxPerSm = 16;  // most resident column blocks per SM any shape launches

const VariantInfo& info(int variant, bool lean) { return lean ? kLean[variant] : kVariants[variant]; }

int device_sms() {
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm;
}

// shared memory of a block of the fused kernel (taumol or transfer area) or of the transfer kernel
size_t block_smem(int nlay, bool lean) {
  return gb::ARGS_BYTES +
         (lean ? gb::rt_smem_bytes(nlay) : std::max(gb::rt_smem_bytes(nlay), gb::gas_smem_bytes(nlay)));
}

// Shared-memory carve-out for `per` resident blocks of `smem` bytes: just what
// they need, so that the rest of the SM's memory stays L1 for the table
// gathers and input loads.
cudaError_t set_carveout(const void* fn, size_t smem, int per) {
  int dev = 0, max_sm = 0, reserved = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  if (max_sm <= 0) return cudaSuccess;
  int pct = (int)std::ceil(100.0 * (double)per * (double)(smem + reserved) / (double)max_sm);
  pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
  return cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

// resident blocks per SM of `fn` with `threads` and `smem` (after allowing that much shared memory)
cudaError_t occupancy(const void* fn, int threads, size_t smem, int* per) {
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, fn, threads, smem);
}

// One launch of a kernel with `nblocks` blocks and the carve-out for those resident.
template <class F>
cudaError_t launch_resident(const void* fn, int threads, size_t smem, int nblocks, F&& go) {
  int per = 0;
  cudaError_t e = occupancy(fn, threads, smem, &per);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  const int nsm = device_sms();
  const int resident = (nblocks + nsm - 1) / nsm;
  e = set_carveout(fn, smem, resident < per ? resident : per);
  if (e != cudaSuccess) return e;
  return go(nblocks);
}

cudaError_t launch_gas_range(const LwBatch& b, const float* T, long long c0, long long c1, cudaStream_t st) {
  const void* fn = (const void*)gb::lw_gas_kernel<gb::GAS_NT>;
  const size_t smem = gb::ARGS_BYTES + gb::gas_smem_bytes(b.nsmax);
  int per = 0;
  cudaError_t e = occupancy(fn, gb::GAS_NT, smem, &per);
  if (e != cudaSuccess) return e;
  long long nb = (long long)device_sms() * (per < 1 ? 1 : per);
  if (nb > c1 - c0) nb = c1 - c0;
  if (nb < 1) return cudaSuccess;
  return launch_resident(fn, gb::GAS_NT, smem, (int)nb, [&](int n) {
    gb::lw_gas_kernel<gb::GAS_NT><<<n, gb::GAS_NT, smem, st>>>(b, T, c0, c1);
    return cudaGetLastError();
  });
}

}  // namespace

int gb_lw_num_variants() { return kNumVariants; }

LwVariant gb_lw_variant(int v, bool lean) {
  if (v < 0 || v >= kNumVariants) return LwVariant{0, 0};
  return LwVariant{gb::RT_NT, info(v, lean).min_blocks};
}

size_t gb_lw_smem_bytes(int nlay) { return block_smem(nlay, false); }

cudaError_t gb_lw_set_tables(const GbTables& T) { return cudaMemcpyToSymbol(gb::c_T, &T, sizeof(GbTables)); }

int gb_lw_slots(int nlay, int variant, bool lean) {
  if (variant < 0 || variant >= kNumVariants) variant = 0;
  const VariantInfo& v = info(variant, lean);
  int per = 0;
  if (occupancy(v.fn, gb::RT_NT, block_smem(nlay, lean), &per) != cudaSuccess || per < 1) per = 1;
  return device_sms() * std::min(per, kMaxPerSm);
}

long long gb_lw_gas_slots(int nlay, long long ncols) {
  (void)nlay;
  (void)ncols;
  return (long long)device_sms() * kMaxPerSm;  // one per resident block of the fused or hand-over kernel
}

size_t gb_lw_gas_bytes(int nlay, long long slots) { return (size_t)slots * 3 * nlay * GB_NGPT * sizeof(float); }

long long gb_lw_list_slots() { return (long long)device_sms() * gb::LIST_PER_SM; }

cudaError_t gb_lw_launch_gas(const LwBatch& b, const float* d_tables, long long c0, long long c1,
                             cudaStream_t stream) {
  if (c1 <= c0) return cudaSuccess;
  if (c1 - c0 > b.gslots || !b.gtau || !b.gfrac) return cudaErrorInvalidValue;
  return launch_gas_range(b, d_tables, c0, c1, stream);
}

cudaError_t gb_lw_launch_batch(const LwBatch& b, const float* d_tables, int variant, int nblocks,
                               cudaStream_t stream) {
  if (variant < 0 || variant >= kNumVariants || b.ngrid < 1 || b.ngrid > GB_LW_MAX_GRIDS) return cudaErrorInvalidValue;
  const long long n = b.col0[b.ngrid];
  if (n <= 0 || nblocks <= 0) return cudaSuccess;
  if (!b.gtau || !b.gfrac || b.gslots < 1 || b.gstride < (long long)b.nsmax * GB_NGPT) return cudaErrorInvalidValue;
  for (int i = 0; i < b.ngrid; ++i)  // fused-cloud grids come with their McICA draws
    if (b.g[i].cloud_mode == LW_CLOUD_FUSED && b.g[i].icld >= 1 && b.g[i].ncol > 0 && !b.g[i].draws)
      return cudaErrorInvalidValue;
  int nband = 0;
  for (int i = 0; i < b.ngrid; ++i) {
    const LwArgs& g = b.g[i];
    if (g.cloud_mode != LW_CLOUD_BAND) continue;
    ++nband;
    if (g.icld >= 1 && g.ncol > 0 && (!g.ncbands || !g.cldfrac || !g.tauc)) return cudaErrorInvalidValue;
  }
  if ((long long)nblocks > n) nblocks = (int)n;
  if (nband) {
    // band clouds: every grid in that mode, taumol gas optics
    if (nband != b.ngrid || b.fall) return cudaErrorInvalidValue;
    if ((long long)nblocks > b.gslots) nblocks = (int)b.gslots;
    const void* fn = (const void*)gb::lw_band_kernel<gb::BAND_MINB>;
    const size_t smem = block_smem(b.nsmax, false);
    return launch_resident(fn, gb::RT_NT, smem, nblocks, [&](int nb) {
      gb::lw_band_kernel<gb::BAND_MINB><<<nb, gb::RT_NT, smem, stream>>>(b, d_tables, 0, n);
      return cudaGetLastError();
    });
  }
  if (!b.fall || !b.nfall) {
    // taumol and the transfer, one block per column, taumol's planes in the block's slot
    if ((long long)nblocks > b.gslots) nblocks = (int)b.gslots;
    const VariantInfo& v = info(variant, false);
    const size_t smem = block_smem(b.nsmax, false);
    return launch_resident(v.fn, gb::RT_NT, smem, nblocks,
                           [&](int nb) { return v.launch(b, d_tables, 0, n, nb, smem, stream); });
  }
  // learned gas optics: the transfer kernel on the network's outputs, then the
  // hand-over kernel over the columns it passed on (its blocks find an empty
  // list and return when every column was on the network)
  if (b.gslots < gb_lw_list_slots()) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(b.nfall, 0, sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  const VariantInfo& v = info(variant, true);
  const size_t smem = block_smem(b.nsmax, true);
  e = launch_resident(v.fn, gb::RT_NT, smem, nblocks, [&](int nb) { return v.launch(b, d_tables, 0, n, nb, smem, stream); });
  if (e != cudaSuccess) return e;
  const void* fn = (const void*)gb::lw_full_kernel<gb::LIST_MINB, true>;
  const size_t lsmem = block_smem(b.nsmax, false);
  return launch_resident(fn, gb::RT_NT, lsmem, (int)gb_lw_list_slots(), [&](int nb) {
    gb::lw_full_kernel<gb::LIST_MINB, true><<<nb, gb::RT_NT, lsmem, stream>>>(b, d_tables, 0, 0);
    return cudaGetLastError();
  });
}
