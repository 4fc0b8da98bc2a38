// cldprop on the device: the band cloud optical depths BRAMS computes on the
// host before McICA (rrtmg_lw_cldprop.f90:50-295, called per column at
// rtm_driver.f90:1250-1258), so that a caller with its cloud state on the GPU
// can feed the fused-cloud solver without a host round trip.
//
// One thread per (column, layer).  The number of bands a layer fills
// (ncbands) is the value the reference's per-call variable holds after that
// layer; when the layer's own branch does not set it (ice option 0, or a
// cloudy layer with neither ice nor liquid) it comes from the nearest cloudy
// layer below that does, which the thread finds by walking down.  All
// arithmetic is fp64 on fp64 copies of the cloud tables, like the reference.
// Output taucloud is in the McICA tauc layout (16, ld, nlay) with the band
// fastest; bands a layer does not fill stay 0.  A radius outside the bounds
// the reference STOPs on gives the column a nonzero status (the largest
// code among its failing layers) and zeros for that layer.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lw_common.h"
#include "lw_context.h"

namespace gbcp {

// a band number as a type, so that an unrolled band keeps its register values
template <int N>
struct IC {
  static constexpr int value = N;
};

struct Cloud64 {
  const double* t;
  int absice0, absice1, absice2, absice3, absliq1;
  double absliq0, abscld1;
};

// The reference's per-call ncbands after a cloudy layer: the layer's own
// setting, if its branch makes one (5 for ice option 1, 16 for options 2
// and 3 and for liquid option 1, 16 for inflag 0 and 1), else -1.
__device__ __forceinline__ int layer_sets_ncbands(int inflag, int iceflag, int liqflag, double cf, double ci,
                                                  double cl, double tauctot) {
  const double cldmin = 1.e-20;
  if (!(cf >= cldmin && (ci + cl >= cldmin || tauctot >= cldmin))) return -1;
  if (inflag != 2) return 16;
  int nb = -1;
  if (ci != 0.0) {
    if (iceflag == 1) nb = 5;
    else if (iceflag >= 2) nb = 16;
  }
  if (cl != 0.0 && liqflag == 1) nb = 16;
  return nb;
}

__device__ __forceinline__ double tau_total(const double* __restrict__ tauc_in, long long o) {
  double t = 0.0;
  if (tauc_in)
    for (int ib = 0; ib < 16; ++ib) t = t + tauc_in[ib + 16 * o];
  return t;
}

// the reference's ice band index for ice option 1 (icb(:,1) of
// rrtmg_lw_cldprop.f90:75-77: bands 1, 2, 3-5, 6-8, 9-16), zero-based, at a
// compile-time band; options 0 and 2/3 map every band to 1 and to itself
__host__ __device__ constexpr int icb1(int ib) { return ib < 1 ? 0 : ib < 2 ? 1 : ib < 5 ? 2 : ib < 8 ? 3 : 4; }

// one thread per (column, layer), columns fastest.  The 16 band values are
// formed in registers (bands unrolled; the per-band absorption coefficients
// that the reference keeps in arrays are evaluated at the band each output
// reads, with the same operations) and stored as pairs when the output is
// 16-byte aligned.
__global__ void __launch_bounds__(64) cldprop_kernel(int ncol, int nlay, long long ld, int inflag, int iceflag,
                                                     int liqflag, const double* __restrict__ cldfrac,
                                                     const double* __restrict__ tauc_in,
                                                     const double* __restrict__ ciwp, const double* __restrict__ clwp,
                                                     const double* __restrict__ rei, const double* __restrict__ rel,
                                                     double* __restrict__ taucloud, int pairs,
                                                     int* __restrict__ col_err, int* __restrict__ err_flag, Cloud64 c,
                                                     int* __restrict__ ncb_col) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)ncol * nlay) return;
  const int lay = (int)(idx / ncol);
  const long long icol = idx - (long long)lay * ncol;
  const double cldmin = 1.e-20;
  const long long o = icol + ld * lay;
  if (ncb_col && lay == nlay - 1) {
    // the column's ncbands after the whole layer loop (what the non-McICA
    // driver hands to rtrn/rtrnmr): the setting of the highest layer that
    // makes one, else the initial 1 (rrtmg_lw_cldprop.f90:173)
    int nb = -1;
    for (int l = nlay - 1; nb < 0 && l >= 0; --l) {
      const long long ol = icol + ld * l;
      nb = layer_sets_ncbands(inflag, iceflag, liqflag, cldfrac[ol], ciwp[ol], clwp[ol], tau_total(tauc_in, ol));
    }
    ncb_col[icol] = nb < 0 ? 1 : nb;
  }
  double* out = taucloud + 16 * o;
  const double tauctot = tau_total(tauc_in, o);
  const double ci = ciwp[o], cl = clwp[o], cf = cldfrac[o];
  const double cwp = ci + cl;
  int lerr = 0;
  bool cloudy = cf >= cldmin && (cwp >= cldmin || tauctot >= cldmin);
  int ncbands = 0;
  // ice: 0 none, 1 iceflag 0 (one value), 2 iceflag 1 (five values), 3 table
  // interpolation; liquid: 0 none, 1 liqflag 0 (one value), 2 interpolation
  int ice_mode = 0, liq_mode = 0, iceind = 0;
  double iv[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const double* ia = c.t;
  int irow = 1, iidx = 1, lidx = 1;
  double ifint = 0.0, lfint = 0.0;
  if (cloudy) {
    // ncbands as the reference holds it after this layer: this layer's
    // setting, else that of the nearest cloudy layer below that makes one
    ncbands = layer_sets_ncbands(inflag, iceflag, liqflag, cf, ci, cl, tauctot);
    for (int l = lay - 1; ncbands < 0 && l >= 0; --l) {
      const long long ol = icol + ld * l;
      ncbands = layer_sets_ncbands(inflag, iceflag, liqflag, cldfrac[ol], ciwp[ol], clwp[ol], tau_total(tauc_in, ol));
    }
    if (ncbands < 0) ncbands = 1;
    if (inflag == 2) {
      const double radice = rei[o];
      if (ci == 0.0) {
        iceind = 0;
      } else if (iceflag == 0) {
        if (radice < 10.0) lerr = GB_COL_ICE_SMALL;
        iv[0] = c.t[c.absice0] + c.t[c.absice0 + 1] / radice;
        ice_mode = 1;
        iceind = 0;
      } else if (iceflag == 1) {
        if (radice < 13.0 || radice > 130.0) lerr = GB_COL_ICE_BOUNDS;
#pragma unroll
        for (int ib = 0; ib < 5; ++ib) iv[ib] = c.t[c.absice1 + 2 * ib] + c.t[c.absice1 + 1 + 2 * ib] / radice;
        ice_mode = 2;
        iceind = 1;
      } else {
        irow = iceflag == 2 ? 43 : 46;
        if (iceflag == 2 ? (radice < 5.0 || radice > 131.0) : (radice < 5.0 || radice > 140.0))
          lerr = iceflag == 2 ? GB_COL_ICE_BOUNDS : GB_COL_DGE_BOUNDS;
        const double factor = (radice - 2.0) / 3.0;
        int index = (int)factor;
        if (index == irow) index = irow - 1;
        iidx = index < 1 ? 1 : (index > irow - 1 ? irow - 1 : index);  // in the table for any input
        ifint = factor - (double)(float)iidx;                          // float(index): a default-real conversion
        ia = c.t + (iceflag == 2 ? c.absice2 : c.absice3);
        ice_mode = 3;
        iceind = 2;
      }
      if (cl == 0.0) {
        if (iceind == 1) iceind = 2;
      } else if (liqflag == 0) {
        liq_mode = 1;
        if (iceind == 1) iceind = 2;
      } else {
        const double radliq = rel[o];
        if (!lerr && (radliq < 2.5 || radliq > 60.0)) lerr = GB_COL_LIQ_BOUNDS;
        int index = (int)(radliq - 1.5);
        if (index == 0) index = 1;
        if (index == 58) index = 57;
        lidx = index < 1 ? 1 : (index > 57 ? 57 : index);  // in the table for any input
        lfint = radliq - 1.5 - (double)(float)lidx;
        liq_mode = 2;
      }
    }
  }
  cloudy = cloudy && !lerr;
  // band ib of the output (rrtmg_lw_cldprop.f90:121-126, 276-287)
  auto band = [&](auto ibc) -> double {
    constexpr int ib = decltype(ibc)::value;
    if (!cloudy || ib >= ncbands) return 0.0;
    if (inflag == 0) return tauc_in[ib + 16 * o];
    if (inflag == 1) return c.abscld1 * cwp;
    double ice = 0.0, liq = 0.0;
    if (ice_mode == 1) {
      ice = iv[0];  // iceind 0: every band reads abscoice(1)
    } else if (ice_mode == 2) {
      ice = iceind == 1 ? iv[icb1(ib)] : (ib < 5 ? iv[ib < 5 ? ib : 0] : 0.0);
    } else if (ice_mode == 3) {
      const double* ab = ia + irow * ib;
      ice = ab[iidx - 1] + ifint * (ab[iidx] - ab[iidx - 1]);
    }
    if (liq_mode == 1) {
      liq = c.absliq0;  // liqind 0: every band reads abscoliq(1)
    } else if (liq_mode == 2) {
      const double* ab = c.t + c.absliq1 + 58 * ib;
      liq = ab[lidx - 1] + lfint * (ab[lidx] - ab[lidx - 1]);
    }
    return ci * ice + cl * liq;
  };
  if (pairs) {
    double2* o2 = reinterpret_cast<double2*>(out);
    o2[0] = make_double2(band(IC<0>{}), band(IC<1>{}));
    o2[1] = make_double2(band(IC<2>{}), band(IC<3>{}));
    o2[2] = make_double2(band(IC<4>{}), band(IC<5>{}));
    o2[3] = make_double2(band(IC<6>{}), band(IC<7>{}));
    o2[4] = make_double2(band(IC<8>{}), band(IC<9>{}));
    o2[5] = make_double2(band(IC<10>{}), band(IC<11>{}));
    o2[6] = make_double2(band(IC<12>{}), band(IC<13>{}));
    o2[7] = make_double2(band(IC<14>{}), band(IC<15>{}));
  } else {
    out[0] = band(IC<0>{}), out[1] = band(IC<1>{}), out[2] = band(IC<2>{}), out[3] = band(IC<3>{});
    out[4] = band(IC<4>{}), out[5] = band(IC<5>{}), out[6] = band(IC<6>{}), out[7] = band(IC<7>{});
    out[8] = band(IC<8>{}), out[9] = band(IC<9>{}), out[10] = band(IC<10>{}), out[11] = band(IC<11>{});
    out[12] = band(IC<12>{}), out[13] = band(IC<13>{}), out[14] = band(IC<14>{}), out[15] = band(IC<15>{});
  }
  if (lerr) {
    if (col_err) atomicMax(col_err + icol, lerr);
    atomicMax(err_flag, lerr);
  }
}

}  // namespace gbcp

int gb_cldprop_lw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int inflag, int iceflag, int liqflag,
                         const double* cldfrac, const double* tauc, const double* ciwp, const double* clwp,
                         const double* rei, const double* rel, double* taucloud, int64_t ld, int* d_col_status) {
  return gb_ctx_cldprop(ctx, stream, ncol, nlay, inflag, iceflag, liqflag, cldfrac, tauc, ciwp, clwp, rei, rel,
                        taucloud, ld, d_col_status, nullptr, nullptr);
}

int gb_ctx_cldprop(gb_lw_context* ctx, void* stream, int ncol, int nlay, int inflag, int iceflag, int liqflag,
                   const double* cldfrac, const double* tauc, const double* ciwp, const double* clwp, const double* rei,
                   const double* rel, double* taucloud, int64_t ld, int* d_col_status, int* d_ncbands,
                   int* d_err_flag) {
  if (!ctx || ncol < 0 || nlay < 1 || nlay > GB_MAXLAY || ld < ncol || inflag < 0 || inflag > 2 || iceflag < 0 ||
      iceflag > 3 || liqflag < 0 || liqflag > 1 || !cldfrac || !ciwp || !clwp || !rei || !rel || !taucloud ||
      (inflag == 0 && !tauc))
    return GB_LW_E_ARGS;
  if (ncol == 0) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  gbcp::Cloud64 c;
  c.t = ctx->d_cloud64;
  c.absice0 = ctx->tabs.c64_absice0;
  c.absice1 = ctx->tabs.c64_absice1;
  c.absice2 = ctx->tabs.c64_absice2;
  c.absice3 = ctx->tabs.c64_absice3;
  c.absliq1 = ctx->tabs.c64_absliq1;
  c.absliq0 = ctx->absliq0;
  c.abscld1 = ctx->abscld1;
  cudaError_t e = d_col_status ? cudaMemsetAsync(d_col_status, 0, sizeof(int) * (size_t)ncol, (cudaStream_t)stream)
                               : cudaSuccess;
  if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "cldprop status");
  const int threads = 64;
  const int pairs = ((uintptr_t)taucloud & 15) == 0;
  const long long n = (long long)ncol * nlay;
  const int blocks = (int)((n + threads - 1) / threads);
  gbcp::cldprop_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(ncol, nlay, ld, inflag, iceflag, liqflag, cldfrac,
                                                                      tauc, ciwp, clwp, rei, rel, taucloud, pairs,
                                                                      d_col_status, d_err_flag ? d_err_flag : ctx->d_err, c,
                                                                      d_ncbands);
  e = cudaGetLastError();
  if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "cldprop launch");
  return GB_LW_OK;
}
