// Column shards of a batched rrtmg_lw call for a multi-GPU caller (host only).
//
// BRAMS gives each MPI rank the columns of its own subdomain
// (rtm_driver.f90:830, nofcols per subdomain; the packing loops :980-1115)
// and every rank calls rrtmg_lw on those.  Columns are independent and no
// data moves between ranks, so a caller that drives several GPUs needs only
// a plan: the batch's grids are laid end to end, and rank r takes the
// contiguous run of columns whose cumulative work (layers) falls in
// [r/N, (r+1)/N) of the total.  Each rank then solves its slices with
// gb_rrtmg_lw_batch_device on its own device; the slices keep the grids'
// leading dimensions, so outputs land in place and no gather is needed.
#include <stdint.h>

#include "../../include/gb_rrtmg_lw.h"

namespace {

// first global column index k with (work of columns 0..k-1) * nranks >= total * r
long long boundary(int ngrid, const int* ncol, const int* nlay, long long total, int nranks, int r) {
  const long long target = total * r;
  long long col = 0, before = 0;
  for (int i = 0; i < ngrid; ++i) {
    const long long need = target - before * nranks;
    const long long step = (long long)nlay[i] * nranks;
    if (need <= 0) return col;
    const long long j = (need + step - 1) / step;
    if (j <= ncol[i]) return col + j;
    col += ncol[i];
    before += (long long)ncol[i] * nlay[i];
  }
  return col;
}

}  // namespace

extern "C" int gb_rrtmg_lw_shard_plan(int ngrid, const int* ncol, const int* nlay, int nranks, int rank,
                                      int64_t* c0, int64_t* c1) {
  if (ngrid < 0 || nranks <= 0 || rank < 0 || rank >= nranks || (ngrid > 0 && (!ncol || !nlay || !c0 || !c1)))
    return GB_LW_E_ARGS;
  long long total = 0;
  for (int i = 0; i < ngrid; ++i) {
    if (ncol[i] < 0 || nlay[i] <= 0) return GB_LW_E_ARGS;
    total += (long long)ncol[i] * nlay[i];
  }
  const long long lo = boundary(ngrid, ncol, nlay, total, nranks, rank);
  const long long hi = rank + 1 == nranks ? -1 : boundary(ngrid, ncol, nlay, total, nranks, rank + 1);
  long long start = 0;
  for (int i = 0; i < ngrid; ++i) {
    const long long end = start + ncol[i];
    long long a = lo > start ? lo : start;
    if (a > end) a = end;
    long long b = (hi < 0 || hi > end) ? end : hi;
    if (b < a) b = a;
    c0[i] = a - start;
    c1[i] = b - start;
    start = end;
  }
  return 0;
}

namespace {

template <class T>
T* shift(T* p, long long elems) {
  return p ? p + elems : p;
}

}  // namespace

extern "C" int gb_rrtmg_lw_grid_slice(const gb_lw_grid* g, int64_t c0, int64_t c1, gb_lw_grid* out) {
  if (!g || !out || c0 < 0 || c1 < c0 || c1 > g->ncol) return GB_LW_E_ARGS;
  gb_lw_grid s = *g;
  const long long n = c0, ng = GB_LW_NGPT;
  s.ncol = (int)(c1 - c0);
  // McICA sub-columns are seeded per column with seed0 + column
  s.seed0 = g->seed0 + (uint32_t)c0;
  // (ld, ...) arrays: the column index is the fastest one
  for (const double** p : {&s.play, &s.plev, &s.tlay, &s.tlev, &s.tsfc, &s.h2ovmr, &s.o3vmr, &s.co2vmr, &s.ch4vmr,
                           &s.n2ovmr, &s.o2vmr, &s.cfc11vmr, &s.cfc12vmr, &s.cfc22vmr, &s.ccl4vmr, &s.emis,
                           &s.tauaer, &s.reicmcl, &s.relqmcl, &s.cldfrac, &s.ciwp, &s.clwp})
    *p = shift(*p, n);
  // (140, ld, nlay) sub-column arrays and the fused mode's (16, ld, nlay) band depths
  for (const double** p : {&s.cldfmcl, &s.taucmcl, &s.ciwpmcl, &s.clwpmcl}) *p = shift(*p, n * ng);
  s.tauc = shift(s.tauc, n * 16);
  for (double** p : {&s.uflx, &s.dflx, &s.hr, &s.uflxc, &s.dflxc, &s.hrc, &s.duflx_dt, &s.duflxc_dt})
    *p = shift(*p, n);
  s.d_col_status = shift(s.d_col_status, n);
  // learned gas optics: [(icol*nlay + lay)*140 + g] and [icol*nlay + lay]
  s.sur_tau = shift(s.sur_tau, n * g->nlay * ng);
  s.sur_frac = shift(s.sur_frac, n * g->nlay * ng);
  s.sur_flag = shift(s.sur_flag, n * g->nlay);
  *out = s;
  return 0;
}
