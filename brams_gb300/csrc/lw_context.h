// Library context shared by the C-ABI translation units (lw_capi.cu, lw_mlp_capi.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gb_rrtmg_lw.h"
#include "lw_common.h"
#include "lw_solver.h"

struct ChunkBufs {
  double* in = nullptr;   // all inputs of one chunk, packed
  double* out = nullptr;  // all outputs of one chunk, packed
  size_t in_elems = 0, out_elems = 0;
};

struct gb_lw_context {
  int device = 0;
  GbTables tabs;
  float* d_tables = nullptr;
  double* d_cloud64 = nullptr;  // cloud optics tables in fp64 (cldprop)
  double absliq0 = 0.0, abscld1 = 0.0;  // cldprop's two scalar cloud constants
  int* d_err = nullptr;      // max status of device calls
  int* d_err_host = nullptr; // status of the current host call
  cudaStream_t streams[2] = {nullptr, nullptr};
  ChunkBufs bufs[2];
  int chunk_cols = 0, chunk_nlay = 0;
  double* d_draws = nullptr;
  size_t draws_elems = 0;
  // taumol hand-over planes of the single-grid calls (one buffer per chunk stream)
  float* d_gas[2] = {nullptr, nullptr};
  size_t gas_bytes[2] = {0, 0};
  std::string last_error;
  size_t max_smem = 0;
  int num_sms = 0;
  float* d_bgas = nullptr;  // taumol hand-over planes of batched launches
  size_t bgas_bytes = 0;
  std::vector<gb_lw_tuning> tuned;  // autotuned shapes, parallel to tuned_nlay (largest nlay of the batch)
  std::vector<int> tuned_nlay;
  std::vector<gb_lw_tuning> last_tune;  // every candidate of the last autotune call
  // McICA draws of fused-cloud grids in batched calls (grown on demand)
  double* d_fdraws = nullptr;
  size_t fdraws_elems = 0;
  // columns the learned-only kernel hands over to the full kernel, and their
  // count (batches with learned gas optics; grown on demand)
  long long* d_fall = nullptr;
  unsigned* d_nfall = nullptr;
  size_t fall_elems = 0;
  // surrogate outputs of batched calls with a network (grown on demand)
  uint16_t* d_sur = nullptr;  // fp16 taug and Planck fractions
  unsigned char* d_sur_flag = nullptr;
  size_t sur_rows = 0;
  // band clouds of the non-McICA calls: cldprop's optical depths (16, ncol,
  // nlay) and cloud-band counts (ncol) (grown on demand)
  double* d_band = nullptr;
  size_t band_elems = 0;
  int* d_ncb = nullptr;
  size_t ncb_elems = 0;
  // RRTMG_SW: tables (fp64 and fp32 blobs, loaded by gb_rrtmg_sw_ini), the
  // precision of the column kernel (gb_rrtmg_sw_set_precision) and the
  // column blocks' scratch slots
  std::string table_dir;
  double* d_sw_tables = nullptr;
  float* d_sw_tables_f = nullptr;
  bool sw_ready = false;
  int sw_bits = 32;
  double sw_scon = 0.0;  // rrsw_scon of the tables (parrrsw.f90)
  void* d_sw_scratch = nullptr;
  size_t sw_scratch_bytes = 0;
  // this context's hold on its device's constant table blocks (see below)
  bool lw_const_held = false, sw_const_held = false;
};

// The kernels' constant table blocks (the longwave GbTables, the shortwave
// table directory of each precision's unit) exist once per device, while
// tables are loaded per context, so every live context on a device must hold
// the same bytes there (the same table files and cpdair).  gb_const_acquire
// takes a hold for `kind` on `device`: false, with nothing changed, when
// another live context there holds different bytes; *upload is set when no
// context held the block, so that the caller uploads its bytes.
enum GbConstKind { GB_CONST_LW = 0, GB_CONST_SW = 1 };
bool gb_const_acquire(int kind, int device, const void* bytes, size_t n, bool* upload);
void gb_const_release(int kind, int device);

// records a CUDA error on the context; returns GB_LW_E_CUDA
int gb_ctx_fail(gb_lw_context* c, cudaError_t e, const char* where);
// validates a batched call's grids and fills the launch descriptor (frac < 1: sample of each grid)
int gb_ctx_make_batch(gb_lw_context* ctx, int ngrid, const gb_lw_grid* grids, double frac, LwBatch& b);
// launches a filled descriptor with the context's shape for its largest nlay
// (first the McICA draws of its fused-cloud grids, into `draws` when given,
// else into a context buffer)
int gb_ctx_launch_batch(gb_lw_context* ctx, LwBatch& b, cudaStream_t stream);
// cldprop on device arrays (gb_cldprop_lw_device), with each column's final
// cloud-band count into d_ncbands when that is not NULL, and the status into
// d_err_flag (NULL: the context's device-call status)
int gb_ctx_cldprop(gb_lw_context* ctx, void* stream, int ncol, int nlay, int inflag, int iceflag, int liqflag,
                   const double* cldfrac, const double* tauc, const double* ciwp, const double* clwp, const double* rei,
                   const double* rel, double* taucloud, int64_t ld, int* d_col_status, int* d_ncbands,
                   int* d_err_flag);
// doubles of McICA draws a descriptor's fused-cloud grids need
size_t gb_ctx_fused_draws(const LwBatch& b);
// launches the draw kernels of a descriptor's fused-cloud grids into buf and sets their draws pointers
int gb_ctx_make_draws(gb_lw_context* ctx, LwBatch& b, double* buf, cudaStream_t stream);
