// Launch interface of the RRTMG_SW column kernel (sw_solver.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#define SW_NGPT 112  // g-points (parrrsw.f90 ngptsw)

// Device pointers in the reference's Fortran layout (rrtmg_sw_rad.f90:243-255):
// (ld, nlay) layer arrays, (ld, nlay+1) level arrays, (ld) surface arrays,
// McICA arrays (112, ld, nlay), aerosols (ld, nlay, 14); outputs (ldo, nlay+1)
// and heating rates (ldo, nlay).
struct SwArgs {
  int ncol, nlay;
  long long ld, ldo;
  int icld, iaer, inflag, iceflag, liqflag;
  double adjflux[14];  // per band: Earth-Sun distance factor x solar-constant scaling
  const double *play, *plev, *tlay, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *o2vmr;
  const double *asdir, *asdif, *aldir, *aldif, *coszen;
  const double *cldfmcl, *taucmcl, *ssacmcl, *asmcmcl, *fsfcmcl, *ciwpmcl, *clwpmcl, *reicmcl, *relqmcl;
  const double *tauaer, *ssaaer, *asmaer;
  double *swuflx, *swdflx, *swhr, *swuflxc, *swdflxc, *swhrc;
  int* col_err;   // optional per-column status (ncol)
  int* err_flag;  // required: max status over the launch
};

struct gb_lw_context;
// loads sw_tables.gbsw of table_dir (NULL: the context's table directory) into the context
int gb_sw_load(gb_lw_context* ctx, double cpdair, const char* table_dir);
// shared memory of a column block, and doubles of one block's scratch slot
size_t gb_sw_smem_bytes(int nlay);
size_t gb_sw_slot_doubles(int nlay);
// all columns of `a` with at most `slots` persistent blocks (block k uses slot k of scratch)
cudaError_t gb_sw_launch(const SwArgs& a, const double* d_tables, double* scratch, long long slots,
                         cudaStream_t stream);
