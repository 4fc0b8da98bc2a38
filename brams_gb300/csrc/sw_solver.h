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

// cldprop_sw on device arrays: inputs (ld, nlay) and (14, ld, nlay); outputs (14, ld, nlay)
struct CldpropSwArgs {
  int ncol, nlay;
  long long ld;
  int inflag, iceflag, liqflag;
  const double *cldfrac, *tauc, *ssac, *asmc, *fsfc, *ciwp, *clwp, *rei, *rel;  // tauc..fsfc may be NULL (zeros)
  double *taucldorig, *taucloud, *ssacloud, *asmcloud;                          // taucldorig may be NULL
  int* col_err;   // optional per-column status (ncol)
  int* err_flag;  // required: max status over the launch
};
// launches it on the fp64 tables of the context's shortwave load
cudaError_t gb_cldprop_sw_launch(const CldpropSwArgs& a, const double* d_tables, cudaStream_t stream);

struct gb_lw_context;
// loads sw_tables.gbsw of table_dir (NULL: the context's table directory) into the context
int gb_sw_load(gb_lw_context* ctx, double cpdair, const char* table_dir);

// blocks per SM of the column kernel in each precision (its launch bounds)
#define SW_MINB_F64 4
#define SW_MINB_F32 6
// persistent blocks (= scratch slots) for a device of num_sms SMs, and the
// scratch bytes of `slots` slots, for a precision of 32 or 64 bits
long long gb_sw_slots(int num_sms, int bits);
size_t gb_sw_scratch_bytes(int nlay, int bits, long long slots);
// all columns of `a` with at most `slots` persistent blocks (block k uses slot
// k of scratch); d_tables is the table blob of the precision (fp32 or fp64)
cudaError_t gb_sw_launch(const SwArgs& a, int bits, const void* d_tables, void* scratch, long long slots,
                         cudaStream_t stream);
// the fp32 kernels' unit (sw_solver_f32.cu): its table directory (a gbsw::SwTab) and its launch
cudaError_t gb_sw_set_tab_f32(const void* tab);
cudaError_t gb_sw_launch_f32(const SwArgs& a, const float* d_tables, float* scratch, long long slots,
                             cudaStream_t stream);
