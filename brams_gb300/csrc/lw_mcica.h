// Launch interface of the McICA sub-column generator (lw_mcica.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

enum McicaMode {
  MCICA_PERCOL_MT = 0,    // Mersenne twister, column c seeded with seed + c (reference called per column)
  MCICA_STREAM_MT = 1,    // Mersenne twister, one sequence for the whole call (the reference's own call)
  MCICA_PERCOL_KISS = 2,  // KISS, seeds from each column's bottom pressures (irng = 0)
};

// Device pointers, Fortran layouts with column leading dimension ld:
// cldfrac/ciwp/clwp/rei/rel/play/alpha (ld, nlay); tauc (nbnd, ld, nlay);
// cldfmcl/ciwpmcl/clwpmcl/taucmcl (nsub, ld, nlay); reicmcl/relqmcl (ld, nlay).
// Longwave: 140 sub-columns, 16 bands (ngb 1..16, band0 0).  Shortwave
// (mcica_subcol_gen_sw.f90): 112 sub-columns, 14 bands (ngb 16..29, band0
// 15) and the single-scattering albedo, asymmetry and forward fraction
// (ssac, asmc, fsfc (14, ld, nlay)) copied like tauc.
struct McicaArgs {
  int mode, ncol, nlay, icld, seed, ncol_call, ndraw_per_col;
  long long ld;
  const double *play, *cldfrac, *ciwp, *clwp, *rei, *rel, *tauc, *alpha;
  double *cldfmcl, *ciwpmcl, *clwpmcl, *taucmcl, *reicmcl, *relqmcl;
  int ngb[140];
  int nsub = 140, nbnd = 16, band0 = 0;
  const double *ssac = nullptr, *asmc = nullptr, *fsfc = nullptr;
  double *ssacmcl = nullptr, *asmcmcl = nullptr, *fsfcmcl = nullptr;
};

// Fixed scratch of the allocation-free entry point: a 256-byte status area
// followed by GB_MCICA_NOALLOC_MAX_DRAWS doubles (4 Mi draws, 32 MiB in all).
#define GB_MCICA_NOALLOC_STATUS_DOUBLES 32
#define GB_MCICA_NOALLOC_MAX_DRAWS (4 * 1024 * 1024)

// Number of doubles of draw scratch the launch needs.
size_t gb_mcica_draw_count(int ncol, int nlay, int icld, int nsub = 140);
// seed_per_column: column c of the launch uses seed + c (MT) or warms KISS up
// seed + c times, reproducing one reference call per column.
cudaError_t gb_mcica_launch(const McicaArgs& a, double* d_draws, int* d_err, cudaStream_t stream,
                            bool seed_per_column);
// First ndraw Mersenne-twister reals of seeds seed0 + c for columns c = 0..ncol-1,
// draws[c * ndraw + k] (the draws of one reference call per column).
cudaError_t gb_mcica_percol_mt(int ncol, unsigned seed0, int ndraw, double* d_draws, cudaStream_t stream);
