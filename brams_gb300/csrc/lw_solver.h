// Launch interface of the RRTMG_LW column kernels (lw_solver.cu).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stddef.h>

#include "lw_common.h"

// Where a grid's McICA sub-column clouds come from.
enum LwCloudMode {
  LW_CLOUD_SUBCOL = 0,  // caller-supplied (140, ld, nlay) arrays cldfmcl/ciwpmcl/clwpmcl/taucmcl
  LW_CLOUD_FUSED = 1,   // generated from layer clouds (icld 3, Mersenne twister,
                        // column c seeded with seed0 + c), as mcica_subcol_lw would for one column
  LW_CLOUD_BAND = 2,    // the non-McICA driver's band-level clouds (rrtmg_lw_rad.nomcica.f90):
                        // layer fractions cldfrac (ld, nlay), cldprop's optical depths tauc
                        // (16, ld, nlay) and its cloud-band count ncbands (ld); icld 1 random
                        // overlap (rtrn), 2 and 3 maximum/random overlap (rtrnmr)
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
  // optional learned gas optics: taug and Planck fractions per (column, layer, g)
  // in fp16 and a per-layer flag (1: use them, 0: taumol); NULL: taumol everywhere
  const __half *sur_tau, *sur_frac;
  const unsigned char* sur_flag;
  // fused cloud mode: the columns' 140 McICA draws [ncol][140] (gb_mcica_percol_mt);
  // required when cloud_mode is LW_CLOUD_FUSED and icld >= 1
  const double* draws;
  // band cloud mode: cldprop's cloud-band count per column (1, 5 or 16)
  const int* ncbands;
};

// Grids of one launch: grid i owns batch columns col0[i] .. col0[i+1]-1.  The
// kernels take this by value (kernel parameter space), so a launch carries
// no device-side descriptor and can be captured in a CUDA graph as is.
#define GB_LW_MAX_GRIDS 32
//
// Gas optics hand-over: taumol writes, per slot, taug (without aerosol) and
// the Planck fractions as fp32 [nlay][140] planes at gtau + slot * gstride and
// gfrac + slot * gstride; the transfer reads them.  The fused taumol and
// transfer kernel uses one slot per block (so that the planes stay in L2).
//
// Batches with learned gas optics (fall and nfall set) run in two launches:
// the transfer kernel solves every column whose layers are all on the network
// and hands the others (batch numbering) over in fall[0 .. *nfall), then the
// hand-over kernel runs taumol and the transfer for those, mixing per layer
// the network's values and taumol's.  fall holds at least col0[ngrid] entries.
struct LwBatch {
  int ngrid;
  int nsmax;                              // largest nlay (stride of the shared-memory areas)
  long long col0[GB_LW_MAX_GRIDS + 1];
  float* gtau = nullptr;                  // gas-optics hand-over (see above)
  float* gfrac = nullptr;
  float* gcld = nullptr;                  // caller sub-columns: each cloudy cell's optical depth
                                          // (or fractional cldfmcl), same slots; may be NULL
  long long gstride = 0;                  // floats per slot (>= nsmax * 140)
  long long gslots = 0;                   // slots available
  long long* fall = nullptr;              // columns handed over off the network
  unsigned* nfall = nullptr;              // their count (device)
  LwArgs g[GB_LW_MAX_GRIDS];
};

// Compiled shapes of the column kernels: threads per block (one column per
// block, one g-point per thread) and the minimum resident blocks per SM the
// register allocation is sized for.
struct LwVariant {
  int threads, min_blocks;
};
// The learned-gas-optics transfer kernel (lean = true) has its own table of as many shapes.
int gb_lw_num_variants();
LwVariant gb_lw_variant(int v, bool lean = false);

// shared memory one block needs at this nlay (one column's taumol or
// transfer area); a launch is possible iff this fits in one block
size_t gb_lw_smem_bytes(int nlay);
// column blocks of `variant` resident on the device at once for this nlay
int gb_lw_slots(int nlay, int variant = 0, bool lean = false);
// hand-over slots a batch is solved with (one per resident block)
long long gb_lw_gas_slots(int nlay, long long ncols);
// bytes of a hand-over buffer of `slots` slots (taug, fractions and cell clouds, fp32)
size_t gb_lw_gas_bytes(int nlay, long long slots);
// hand-over slots the hand-over kernel of a learned batch uses (one per block)
long long gb_lw_list_slots();
cudaError_t gb_lw_set_tables(const GbTables& T);
// All grids of `b` with `variant` at `nblocks` persistent blocks: taumol
// batches through the fused taumol + transfer kernel (block k in slot k);
// with b.fall set the learned-gas-optics transfer kernel, then the hand-over
// kernel.  Batches of LW_CLOUD_BAND grids (all grids in that mode, taumol
// only) run the band-cloud flavour of the fused kernel.
cudaError_t gb_lw_launch_batch(const LwBatch& b, const float* d_tables, int variant, int nblocks,
                               cudaStream_t stream);
// The taumol kernel alone over batch columns [c0, c1) into slots 0 .. c1-c0-1.
cudaError_t gb_lw_launch_gas(const LwBatch& b, const float* d_tables, long long c0, long long c1,
                             cudaStream_t stream);
