// Launch interface of the fused RRTMG_LW column kernel (lw_solver.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "lw_common.h"

// Device pointers in the reference's Fortran layout.  (ncol, .) arrays have
// leading dimension ld (>= ncol); McICA arrays are (140, ld, nlay); tauaer is
// (ld, nlay, 16); outputs (ldo, nlay+1) / (ldo, nlay).
struct LwArgs {
  int ncol, nlay;
  long long ld, ldo;
  int icld, idrv, inflag, iceflag, liqflag;
  const double *play, *plev, *tlay, *tlev, *tsfc;
  const double *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr, *o2vmr;
  const double *cfc11vmr, *cfc12vmr, *cfc22vmr, *ccl4vmr, *emis;
  const double *cldfmcl, *taucmcl, *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl, *tauaer;
  double *uflx, *dflx, *hr, *uflxc, *dflxc, *hrc, *duflx_dt, *duflxc_dt;
  int* col_err;   // optional per-column status (ncol)
  int* err_flag;  // required: max status over the launch
  float* dbg_taut;   // optional diagnostics: taut and Planck fractions per column,
  float* dbg_fracs;  // (ncol, nlay, 140) with g fastest; NULL in production calls
};

size_t gb_lw_smem_bytes(int nlay);
cudaError_t gb_lw_set_tables(const GbTables& T);
cudaError_t gb_lw_launch(const LwArgs& a, const float* d_tables, cudaStream_t stream);
