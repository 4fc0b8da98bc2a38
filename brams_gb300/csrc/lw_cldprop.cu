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

struct Cloud64 {
  const double* t;
  int absice0, absice1, absice2, absice3, absliq1;
  double absliq0, abscld1;
};

// rrtmg_lw_cldprop.f90:75-77 (icb: ice band index per band and ice option)
__constant__ int c_icb[3][16] = {{1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
                                 {1, 2, 3, 3, 3, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5},
                                 {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16}};

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

// one thread per (column, layer), columns fastest
__global__ void cldprop_kernel(int ncol, int nlay, long long ld, int inflag, int iceflag, int liqflag,
                               const double* __restrict__ cldfrac, const double* __restrict__ tauc_in,
                               const double* __restrict__ ciwp, const double* __restrict__ clwp,
                               const double* __restrict__ rei, const double* __restrict__ rel,
                               double* __restrict__ taucloud, int* __restrict__ col_err, int* __restrict__ err_flag,
                               Cloud64 c) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)ncol * nlay) return;
  const int lay = (int)(idx / ncol);
  const long long icol = idx - (long long)lay * ncol;
  const double cldmin = 1.e-20;
  const long long o = icol + ld * lay;
  double* out = taucloud + 16 * o;
  double tc[16];
#pragma unroll
  for (int ib = 0; ib < 16; ++ib) tc[ib] = 0.0;
  const double tauctot = tau_total(tauc_in, o);
  const double ci = ciwp[o], cl = clwp[o], cf = cldfrac[o];
  const double cwp = ci + cl;
  int lerr = 0;
  if (cf >= cldmin && (cwp >= cldmin || tauctot >= cldmin)) {
    // ncbands as the reference holds it after this layer: this layer's
    // setting, else that of the nearest cloudy layer below that makes one
    int ncbands = layer_sets_ncbands(inflag, iceflag, liqflag, cf, ci, cl, tauctot);
    for (int l = lay - 1; ncbands < 0 && l >= 0; --l) {
      const long long ol = icol + ld * l;
      ncbands = layer_sets_ncbands(inflag, iceflag, liqflag, cldfrac[ol], ciwp[ol], clwp[ol], tau_total(tauc_in, ol));
    }
    if (ncbands < 0) ncbands = 1;
    if (inflag == 0) {
      for (int ib = 0; ib < 16; ++ib) tc[ib] = tauc_in[ib + 16 * o];
    } else if (inflag == 1) {
      for (int ib = 0; ib < 16; ++ib) tc[ib] = c.abscld1 * cwp;
    } else {
      double abscoice[16], abscoliq[16];
      for (int ib = 0; ib < 16; ++ib) abscoice[ib] = abscoliq[ib] = 0.0;
      int iceind = 0, liqind = 0;
      const double radice = rei[o];
      if (ci == 0.0) {
        iceind = 0;
      } else if (iceflag == 0) {
        if (radice < 10.0) lerr = GB_COL_ICE_SMALL;
        abscoice[0] = c.t[c.absice0] + c.t[c.absice0 + 1] / radice;
        iceind = 0;
      } else if (iceflag == 1) {
        if (radice < 13.0 || radice > 130.0) lerr = GB_COL_ICE_BOUNDS;
        for (int ib = 0; ib < 5; ++ib)
          abscoice[ib] = c.t[c.absice1 + 2 * ib] + c.t[c.absice1 + 1 + 2 * ib] / radice;
        iceind = 1;
      } else {
        const int nrow = iceflag == 2 ? 43 : 46;
        if (iceflag == 2 ? (radice < 5.0 || radice > 131.0) : (radice < 5.0 || radice > 140.0))
          lerr = iceflag == 2 ? GB_COL_ICE_BOUNDS : GB_COL_DGE_BOUNDS;
        const double factor = (radice - 2.0) / 3.0;
        int index = (int)factor;
        if (index == nrow) index = nrow - 1;
        index = index < 1 ? 1 : (index > nrow - 1 ? nrow - 1 : index);  // in the table for any input
        const double fint = factor - (double)(float)index;            // float(index): a default-real conversion
        const double* a = c.t + (iceflag == 2 ? c.absice2 : c.absice3);
        if (!lerr)
          for (int ib = 0; ib < 16; ++ib) {
            const double* ab = a + nrow * ib;
            abscoice[ib] = ab[index - 1] + fint * (ab[index] - ab[index - 1]);
          }
        iceind = 2;
      }
      if (cl == 0.0) {
        liqind = 0;
        if (iceind == 1) iceind = 2;
      } else if (liqflag == 0) {
        abscoliq[0] = c.absliq0;
        liqind = 0;
        if (iceind == 1) iceind = 2;
      } else {
        const double radliq = rel[o];
        if (!lerr && (radliq < 2.5 || radliq > 60.0)) lerr = GB_COL_LIQ_BOUNDS;
        int index = (int)(radliq - 1.5);
        if (index == 0) index = 1;
        if (index == 58) index = 57;
        index = index < 1 ? 1 : (index > 57 ? 57 : index);  // in the table for any input
        const double fint = radliq - 1.5 - (double)(float)index;
        if (!lerr)
          for (int ib = 0; ib < 16; ++ib) {
            const double* ab = c.t + c.absliq1 + 58 * ib;
            abscoliq[ib] = ab[index - 1] + fint * (ab[index] - ab[index - 1]);
          }
        liqind = 2;
      }
      if (!lerr)
        for (int ib = 0; ib < ncbands; ++ib)
          tc[ib] = ci * abscoice[c_icb[iceind][ib] - 1] + cl * abscoliq[c_icb[liqind][ib] - 1];
    }
  }
#pragma unroll
  for (int ib = 0; ib < 16; ++ib) out[ib] = lerr ? 0.0 : tc[ib];
  if (lerr) {
    if (col_err) atomicMax(col_err + icol, lerr);
    atomicMax(err_flag, lerr);
  }
}

}  // namespace gbcp

int gb_cldprop_lw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int inflag, int iceflag, int liqflag,
                         const double* cldfrac, const double* tauc, const double* ciwp, const double* clwp,
                         const double* rei, const double* rel, double* taucloud, int64_t ld, int* d_col_status) {
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
  const int threads = 256;
  const long long n = (long long)ncol * nlay;
  const int blocks = (int)((n + threads - 1) / threads);
  gbcp::cldprop_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(ncol, nlay, ld, inflag, iceflag, liqflag, cldfrac,
                                                                      tauc, ciwp, clwp, rei, rel, taucloud,
                                                                      d_col_status, ctx->d_err, c);
  e = cudaGetLastError();
  if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "cldprop launch");
  return GB_LW_OK;
}
