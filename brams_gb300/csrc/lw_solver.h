// Launch interface of the fused RRTMG_LW column kernel (lw_solver.cu).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stddef.h>

#include "lw_common.h"

// Where a grid's McICA sub-column clouds come from.
enum LwCloudMode {
  LW_CLOUD_SUBCOL = 0,  // caller-supplied (140, ld, nlay) arrays cldfmcl/ciwpmcl/clwpmcl/taucmcl
  LW_CLOUD_FUSED = 1,   // generated inside the kernel from layer clouds (icld 3, Mersenne twister,
                        // column c seeded with seed0 + c), as mcica_subcol_lw would for one column
};

// Device pointers in the reference's Fortran layout.  (ncol, .) arrays have
// leading dimension ld (>= ncol); McICA arrays are (140, ld, nlay); tauaer is
// (ld, nlay, 16); outputs (ldo, nlay+1) / (ldo, nlay).  In LW_CLOUD_FUSED mode
// cldfrac/ciwp/clwp are (ld, nlay), tauc is (16, ld, nlay) and reicmcl/relqmcl
// hold the layer radii rei/rel.
struct LwArgs {
  int ncol, nlay;
  long long ld, ldo;
  int icld, idrv, inflag, iceflag, liqflag;
  int cloud_mode;
  unsigned seed0;
  const double *play, *plev, *tlay, *tlev, *tsfc;
  const double *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr, *o2vmr;
  const double *cfc11vmr, *cfc12vmr, *cfc22vmr, *ccl4vmr, *emis;
  const double *cldfmcl, *taucmcl, *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl, *tauaer;
  const double *cldfrac, *ciwp, *clwp, *tauc;
  double *uflx, *dflx, *hr, *uflxc, *dflxc, *hrc, *duflx_dt, *duflxc_dt;
  int* col_err;   // optional per-column status (ncol)
  int* err_flag;  // required: max status over the launch
  float* dbg_taut;   // optional diagnostics: taut and Planck fractions per column,
  float* dbg_fracs;  // (ncol, nlay, 140) with g fastest; NULL in production calls
  // optional learned gas optics: taug and Planck fractions per (column, layer, g)
  // in fp16 and a per-layer flag (1: use them, 0: taumol); NULL: taumol everywhere
  const __half *sur_tau, *sur_frac;
  const unsigned char* sur_flag;
  // fused cloud mode: the columns' 140 McICA draws [ncol][140] made beforehand
  // (gb_mcica_percol_mt); NULL: the kernel draws them itself
  const double* draws;
};

// Grids of one launch: grid i owns batch columns col0[i] .. col0[i+1]-1.  The
// kernel takes this by value (kernel parameter space), so the launch carries
// no device-side descriptor and can be captured in a CUDA graph as is.
#define GB_LW_MAX_GRIDS 32
//
// Batches with learned gas optics (fall and nfall set) run in two launches:
// a learned-only kernel solves every column whose layers are all on the
// network and hands the others (batch numbering) over in fall[0 .. *nfall),
// then the full kernel solves those.  fall holds at least col0[ngrid] entries.
struct LwBatch {
  int ngrid;
  int nsmax;                              // largest nlay (scratch-slot stride)
  long long col0[GB_LW_MAX_GRIDS + 1];
  float4* scratch;                        // >= gridDim.x slots of 2*nsmax*140 float4
  long long* fall = nullptr;              // columns handed over by the learned-only kernel
  unsigned* nfall = nullptr;              // their count (device)
  LwArgs g[GB_LW_MAX_GRIDS];
};

// Compiled shapes of the column kernel: threads per column block and the
// minimum resident blocks per SM the register allocation is sized for.
struct LwVariant {
  int threads, min_blocks;
};
// The learned-only kernel (lean = true) has its own table of as many shapes.
int gb_lw_num_variants();
LwVariant gb_lw_variant(int v, bool lean = false);

size_t gb_lw_smem_bytes(int nlay, bool lean = false);
// thread blocks of `variant` that fit on the device at once for this nlay
int gb_lw_slots(int nlay, int variant = 0, bool lean = false);
// bytes of scratch for `slots` slots: per slot 2*nlay*140 float4 (clear-sky coefficient planes, cloudy cells)
size_t gb_lw_scratch_bytes(int nlay, int slots);
cudaError_t gb_lw_set_tables(const GbTables& T);
// One grid, default variant, grid = min(ncol, nslots) blocks.
cudaError_t gb_lw_launch(const LwArgs& a, const float* d_tables, float4* scratch, int nslots, cudaStream_t stream);
// All grids of `b` in one launch of `nblocks` persistent blocks of `variant`
// (with b.fall set: the learned-only kernel's `variant`, then the full kernel
// over the columns it handed over).
cudaError_t gb_lw_launch_batch(const LwBatch& b, const float* d_tables, int variant, int nblocks,
                               cudaStream_t stream);
