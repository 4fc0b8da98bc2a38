// Host interface of the taumol MLP kernels (lw_mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stddef.h>

#include "lw_mlp.cuh"

#define GB_NGPT_MLP 140
#define GB_MLP_TAU_FLOOR 1.0e-10f  // log(taug) is taken of max(taug, floor)

// rrtmg_lw inputs the features are made of (device, Fortran layout, leading dimension ld)
struct GbMlpGridIn {
  int ncol, nlay;
  long long ld;
  const double *play, *plev, *tlay, *tlev, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr;
};

// Device buffers of training: parameters (fp32 master, bf16 copy, Adam
// moments) and per-row activations for up to `rows` rows.
struct MlpBuffers {
  float *p32, *m, *v;
  __nv_bfloat16* p16;
  __nv_bfloat16 *z[3], *act[3], *dz[3], *dy;
  float* y;
  long long rows;
};

size_t gb_mlp_infer_smem();
cudaError_t gb_mlp_features(const GbMlpGridIn& g, double grav, double avogad, float* d_feat, cudaStream_t st);
cudaError_t gb_mlp_norm_inputs(long long rows, const float* d_feat, const GbMlpNorm& nm, __nv_bfloat16* d_x,
                               cudaStream_t st);
cudaError_t gb_mlp_norm_targets(long long rows, const float* d_tau, const float* d_frac, const GbMlpNorm& nm,
                                float* d_t, cudaStream_t st);
// forward + backward of one batch: gradients of the loss w.r.t. all parameters into d_grad (fp32, blob order)
cudaError_t gb_mlp_forward_backward(const MlpBuffers& b, long long rows, const __nv_bfloat16* d_x, const float* d_t,
                                    const float* d_w, float* d_grad, float* d_loss, cudaStream_t st);
cudaError_t gb_mlp_adam(const MlpBuffers& b, const float* d_grad, float lr, int step, cudaStream_t st);
cudaError_t gb_mlp_sync_bf16(const MlpBuffers& b, cudaStream_t st);
// surrogate taug [(icol*nlay + lay)*140 + g], Planck fractions (same layout), both fp16 (taug clamped to
// GB_MLP_HALF_MAX), and the in-range flag per layer
#define GB_MLP_HALF_MAX 65504.0f
cudaError_t gb_mlp_infer(const GbMlpGridIn& g, const GbMlpNorm& nm, const __nv_bfloat16* p16, const float* p32,
                         double grav, double avogad, __half* d_tau, __half* d_frac, unsigned char* d_flag, int nsm,
                         cudaStream_t st);

// tcgen05 inference (lw_mlp_tc.cu): weight images prepared once per parameter change
size_t gb_mlp_tc_image_bytes();
cudaError_t gb_mlp_tc_images(const __nv_bfloat16* p16, const float* p32, const GbMlpNorm& nm, void* d_img,
                             cudaStream_t st);
cudaError_t gb_mlp_infer_tc(const GbMlpGridIn& g, const GbMlpNorm& nm, const void* d_img, double grav,
                            double avogad, __half* d_tau, __half* d_frac, unsigned char* d_flag, int* d_err, int nsm,
                            cudaStream_t st);
