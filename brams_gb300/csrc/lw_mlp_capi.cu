// C ABI of the learned gas optics (declared in include/gb_rrtmg_lw.h).
//
// The network (lw_mlp.cuh) is trained on layers that the plain column kernel
// produces (gb_lw_mlp_samples), with the hand-written forward/backward
// kernels and Adam of lw_mlp.cu, and used by the column kernel through
// gb_lw_mlp_infer / gb_rrtmg_lw_batch_surrogate.  Layers whose features lie
// outside the training range keep the plain taumol.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lw_context.h"
#include "lw_mlp.h"

static_assert(GB_LW_MLP_NPARAM == GB_MLP_NPARAM, "parameter count of the ABI and the kernels differ");
static_assert(GB_LW_MLP_NNORM * sizeof(float) == sizeof(GbMlpNorm), "normalisation block of the ABI and the kernels differ");

struct gb_lw_mlp {
  gb_lw_context* ctx = nullptr;
  GbMlpNorm norm{};
  MlpBuffers b{};
  float* d_grad = nullptr;
  float* d_w = nullptr;  // loss weight per output
  int step = 0;
  int engine = GB_LW_MLP_TCGEN05;
  void* d_img = nullptr;  // tcgen05 weight images (rebuilt when the parameters change)
  bool img_dirty = true;
};

namespace {

int fail(gb_lw_context* ctx, cudaError_t e, const char* where) { return gb_ctx_fail(ctx, e, where); }

void free_rows(MlpBuffers& b) {
  for (int l = 0; l < 3; ++l) {
    cudaFree(b.z[l]);
    cudaFree(b.act[l]);
    cudaFree(b.dz[l]);
    b.z[l] = b.act[l] = b.dz[l] = nullptr;
  }
  cudaFree(b.dy);
  cudaFree(b.y);
  b.dy = nullptr;
  b.y = nullptr;
  b.rows = 0;
}

int ensure_rows(gb_lw_mlp* m, long long rows) {
  if (rows <= m->b.rows) return 0;
  free_rows(m->b);
  const size_t H = GB_MLP_H, O = GB_MLP_NOUTP;
  bool ok = true;
  for (int l = 0; l < 3; ++l) {
    ok = ok && cudaMalloc(&m->b.z[l], rows * H * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&m->b.act[l], rows * H * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&m->b.dz[l], rows * H * 2) == cudaSuccess;
  }
  ok = ok && cudaMalloc(&m->b.dy, rows * O * 2) == cudaSuccess;
  ok = ok && cudaMalloc(&m->b.y, rows * O * 4) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    free_rows(m->b);
    m->ctx->last_error = "device allocation of training activations failed";
    return GB_LW_E_NOMEM;
  }
  m->b.rows = rows;
  return 0;
}

// seeded initial weights: uniform(-s, s) with s = sqrt(3 / fan_in); biases zero
void init_params(uint64_t seed, std::vector<float>& p) {
  p.assign(GB_MLP_NPARAM, 0.0f);
  uint64_t x = seed ? seed : 0x9E3779B97F4A7C15ull;
  auto next = [&]() {  // splitmix64
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  auto fill = [&](int off, int fin, int fout, int fin_used) {
    const double s = std::sqrt(3.0 / fin_used);
    for (int i = 0; i < fin; ++i)
      for (int j = 0; j < fout; ++j) {
        const double u = (double)(next() >> 11) * (1.0 / 9007199254740992.0);
        const bool live = i < fin_used && (fout != GB_MLP_NOUTP || j < GB_MLP_NOUT);
        p[off + i * fout + j] = live ? (float)((2.0 * u - 1.0) * s) : 0.0f;
      }
  };
  fill(GB_MLP_OFF_W1, GB_MLP_KIN, GB_MLP_H, GB_MLP_NF);
  fill(GB_MLP_OFF_W2, GB_MLP_H, GB_MLP_H, GB_MLP_H);
  fill(GB_MLP_OFF_W3, GB_MLP_H, GB_MLP_H, GB_MLP_H);
  fill(GB_MLP_OFF_W4, GB_MLP_H, GB_MLP_NOUTP, GB_MLP_H);
}

void default_norm(GbMlpNorm& n) {
  for (int i = 0; i < GB_MLP_KIN; ++i) {
    n.in_mu[i] = 0.0f;
    n.in_sd[i] = 1.0f;
  }
  for (int i = 0; i < GB_MLP_NF; ++i) {
    n.in_lo[i] = -INFINITY;
    n.in_hi[i] = INFINITY;
  }
  for (int i = 0; i < GB_MLP_NOUTP; ++i) {
    n.out_mu[i] = 0.0f;
    n.out_sd[i] = 1.0f;
  }
}

GbMlpGridIn grid_in(const gb_lw_grid& g) {
  GbMlpGridIn in{};
  in.ncol = g.ncol;
  in.nlay = g.nlay;
  in.ld = g.ld_in;
  in.play = g.play; in.plev = g.plev; in.tlay = g.tlay; in.tlev = g.tlev; in.h2ovmr = g.h2ovmr;
  in.o3vmr = g.o3vmr; in.co2vmr = g.co2vmr; in.ch4vmr = g.ch4vmr; in.n2ovmr = g.n2ovmr;
  return in;
}

int upload_params(gb_lw_mlp* m, const float* host) {
  if (cudaMemcpy(m->b.p32, host, GB_MLP_NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess) return GB_LW_E_CUDA;
  cudaError_t e = gb_mlp_sync_bf16(m->b, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  m->img_dirty = true;
  return e == cudaSuccess ? 0 : fail(m->ctx, e, "parameter upload");
}

// per-column statistics over rows of a [rows][ld] array: sum, sum of squares, min, max
__global__ void colstats_kernel(long long rows, int ncols, int ld, const float* __restrict__ x, int take_log,
                                double* __restrict__ sum, double* __restrict__ sq, int* __restrict__ mn,
                                int* __restrict__ mx) {
  const int j = blockIdx.x * 32 + (threadIdx.x & 31);
  const int ry = threadIdx.x >> 5;
  if (j >= ncols) return;
  double s = 0.0, q = 0.0;
  float lo = INFINITY, hi = -INFINITY;
  for (long long r = blockIdx.y * 8LL + ry; r < rows; r += 8LL * gridDim.y) {
    float v = x[r * ld + j];
    if (take_log) v = logf(fmaxf(v, GB_MLP_TAU_FLOOR));
    s += v;
    q += (double)v * v;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  atomicAdd(sum + j, s);
  atomicAdd(sq + j, q);
  // order-preserving integer image of a float
  auto key = [](float f) { int i = __float_as_int(f); return i >= 0 ? i : i ^ 0x7FFFFFFF; };
  atomicMin(mn + j, key(lo));
  atomicMax(mx + j, key(hi));
}

float unkey(int i) { return i >= 0 ? *(float*)&i : [&] { int k = i ^ 0x7FFFFFFF; return *(float*)&k; }(); }

int colstats(gb_lw_context* ctx, cudaStream_t st, long long rows, int ncols, int ld, const float* d_x, int take_log,
             std::vector<double>& mean, std::vector<double>& sd, std::vector<float>& lo, std::vector<float>& hi) {
  double* d_acc = nullptr;
  int* d_mm = nullptr;
  if (cudaMalloc(&d_acc, 2 * ncols * sizeof(double)) != cudaSuccess || cudaMalloc(&d_mm, 2 * ncols * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d_acc);
    return GB_LW_E_NOMEM;
  }
  std::vector<int> init(2 * ncols);
  for (int j = 0; j < ncols; ++j) {
    init[j] = 0x7FFFFFFF;
    init[ncols + j] = (int)0x80000000;
  }
  cudaMemsetAsync(d_acc, 0, 2 * ncols * sizeof(double), st);
  cudaMemcpyAsync(d_mm, init.data(), 2 * ncols * sizeof(int), cudaMemcpyHostToDevice, st);
  dim3 grid((ncols + 31) / 32, 512);
  colstats_kernel<<<grid, 256, 0, st>>>(rows, ncols, ld, d_x, take_log, d_acc, d_acc + ncols, d_mm, d_mm + ncols);
  std::vector<double> acc(2 * ncols);
  std::vector<int> mm(2 * ncols);
  cudaError_t e = cudaMemcpyAsync(acc.data(), d_acc, 2 * ncols * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(mm.data(), d_mm, 2 * ncols * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_acc);
  cudaFree(d_mm);
  if (e != cudaSuccess) return fail(ctx, e, "column statistics");
  mean.resize(ncols);
  sd.resize(ncols);
  lo.resize(ncols);
  hi.resize(ncols);
  for (int j = 0; j < ncols; ++j) {
    mean[j] = acc[j] / (double)rows;
    sd[j] = std::sqrt(std::max(0.0, acc[ncols + j] / (double)rows - mean[j] * mean[j]));
    lo[j] = unkey(mm[j]);
    hi[j] = unkey(mm[ncols + j]);
  }
  return 0;
}

}  // namespace

extern "C" {

int gb_lw_mlp_create(gb_lw_context* ctx, uint64_t seed, gb_lw_mlp** out) {
  if (!ctx || !out) return GB_LW_E_ARGS;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  gb_lw_mlp* m = new gb_lw_mlp();
  m->ctx = ctx;
  default_norm(m->norm);
  bool ok = cudaMalloc(&m->b.p32, GB_MLP_NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&m->b.m, GB_MLP_NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&m->b.v, GB_MLP_NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&m->b.p16, GB_MLP_NPARAM * 2) == cudaSuccess &&
            cudaMalloc(&m->d_grad, GB_MLP_NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&m->d_w, GB_MLP_NOUTP * 4) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    gb_lw_mlp_destroy(m);
    return GB_LW_E_NOMEM;
  }
  std::vector<float> p;
  init_params(seed, p);
  std::vector<float> w(GB_MLP_NOUTP, 1.0f);
  for (int j = GB_MLP_NOUT; j < GB_MLP_NOUTP; ++j) w[j] = 0.0f;
  cudaMemset(m->b.m, 0, GB_MLP_NPARAM * 4);
  cudaMemset(m->b.v, 0, GB_MLP_NPARAM * 4);
  cudaMemcpy(m->d_w, w.data(), GB_MLP_NOUTP * 4, cudaMemcpyHostToDevice);
  int rc = upload_params(m, p.data());
  if (rc) {
    gb_lw_mlp_destroy(m);
    return rc;
  }
  *out = m;
  return GB_LW_OK;
}

int gb_lw_mlp_destroy(gb_lw_mlp* m) {
  if (!m) return GB_LW_OK;
  cudaSetDevice(m->ctx->device);
  free_rows(m->b);
  cudaFree(m->b.p32);
  cudaFree(m->b.m);
  cudaFree(m->b.v);
  cudaFree(m->b.p16);
  cudaFree(m->d_grad);
  cudaFree(m->d_w);
  cudaFree(m->d_img);
  delete m;
  return GB_LW_OK;
}

int gb_lw_mlp_get_params(gb_lw_mlp* m, float* params, float* norm) {
  if (!m) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  if (params && cudaMemcpy(params, m->b.p32, GB_MLP_NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(m->ctx, cudaGetLastError(), "parameter download");
  if (norm) std::memcpy(norm, &m->norm, sizeof(GbMlpNorm));
  return GB_LW_OK;
}

int gb_lw_mlp_set_params(gb_lw_mlp* m, const float* params, const float* norm) {
  if (!m) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  if (norm) {
    std::memcpy(&m->norm, norm, sizeof(GbMlpNorm));
    m->img_dirty = true;
  }
  if (params) {
    int rc = upload_params(m, params);
    if (rc) return rc;
    cudaMemset(m->b.m, 0, GB_MLP_NPARAM * 4);
    cudaMemset(m->b.v, 0, GB_MLP_NPARAM * 4);
    m->step = 0;
  }
  return GB_LW_OK;
}

int gb_lw_mlp_set_loss_weights(gb_lw_mlp* m, const float* w) {
  if (!m || !w) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  std::vector<float> h(w, w + GB_MLP_NOUT);
  h.resize(GB_MLP_NOUTP, 0.0f);
  if (cudaMemcpy(m->d_w, h.data(), GB_MLP_NOUTP * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(m->ctx, cudaGetLastError(), "loss weights");
  return GB_LW_OK;
}

int gb_lw_mlp_samples(gb_lw_context* ctx, void* stream, const gb_lw_grid* grid, float* d_feat, float* d_tau,
                      float* d_frac) {
  if (!ctx || !grid || !d_feat || !d_tau || !d_frac) return GB_LW_E_ARGS;
  gb_lw_grid g = *grid;
  g.icld = 0;  // gas optics do not depend on clouds
  g.sur_tau = g.sur_frac = nullptr;
  g.sur_flag = nullptr;
  LwBatch b;
  int rc = gb_ctx_make_batch(ctx, 1, &g, 1.0, b);
  if (rc) return rc;
  // the taumol kernel writes taug and the Planck fractions of column i,
  // layer l at row i * nlay + l of the caller's (rows, 140) arrays
  b.gstride = (long long)g.nlay * GB_NGPT;
  b.gslots = g.ncol;
  b.gtau = d_tau;
  b.gfrac = d_frac;
  cudaStream_t st = (cudaStream_t)stream;
  cudaSetDevice(ctx->device);
  cudaError_t e = gb_mlp_features(grid_in(g), ctx->tabs.grav, ctx->tabs.avogad, d_feat, st);
  if (e != cudaSuccess) return fail(ctx, e, "features");
  e = gb_lw_launch_gas(b, ctx->d_tables, 0, g.ncol, st);
  return e == cudaSuccess ? GB_LW_OK : fail(ctx, e, "taumol samples");
}

int gb_lw_mlp_fit_norm(gb_lw_mlp* m, void* stream, int64_t rows, const float* d_feat, const float* d_tau,
                       const float* d_frac) {
  if (!m || rows < 1 || !d_feat || !d_tau || !d_frac) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<double> mu, sd;
  std::vector<float> lo, hi;
  GbMlpNorm& n = m->norm;
  int rc = colstats(m->ctx, st, rows, GB_MLP_NF, GB_MLP_NF, d_feat, 0, mu, sd, lo, hi);
  if (rc) return rc;
  // The validity range is the training range widened by GB_MLP_RANGE_MARGIN
  // of its width on each side: layers at the edge of the training set (the
  // model-top layer, whose thickness and column amounts are the smallest of
  // every profile) must not drop out over a rounding or a slightly thinner
  // top layer.
  for (int i = 0; i < GB_MLP_NF; ++i) {
    n.in_mu[i] = (float)mu[i];
    n.in_sd[i] = (float)std::max(sd[i], 1e-6);
    const float pad = GB_MLP_RANGE_MARGIN * (hi[i] - lo[i]);
    n.in_lo[i] = lo[i] - pad;
    n.in_hi[i] = hi[i] + pad;
  }
  for (int i = GB_MLP_NF; i < GB_MLP_KIN; ++i) {
    n.in_mu[i] = 0.0f;
    n.in_sd[i] = 1.0f;
  }
  rc = colstats(m->ctx, st, rows, GB_NGPT_MLP, GB_NGPT_MLP, d_tau, 1, mu, sd, lo, hi);
  if (rc) return rc;
  for (int j = 0; j < GB_NGPT_MLP; ++j) {
    n.out_mu[j] = (float)mu[j];
    n.out_sd[j] = (float)(sd[j] > 1e-6 ? sd[j] : 1.0);
  }
  rc = colstats(m->ctx, st, rows, GB_NGPT_MLP, GB_NGPT_MLP, d_frac, 0, mu, sd, lo, hi);
  if (rc) return rc;
  for (int j = 0; j < GB_NGPT_MLP; ++j) {
    n.out_mu[GB_NGPT_MLP + j] = (float)mu[j];
    n.out_sd[GB_NGPT_MLP + j] = (float)(sd[j] > 1e-6 ? sd[j] : 1.0);
  }
  for (int j = GB_MLP_NOUT; j < GB_MLP_NOUTP; ++j) {
    n.out_mu[j] = 0.0f;
    n.out_sd[j] = 1.0f;
  }
  m->img_dirty = true;
  return GB_LW_OK;
}

int gb_lw_mlp_prepare(gb_lw_mlp* m, void* stream, int64_t rows, const float* d_feat, const float* d_tau,
                      const float* d_frac, void* d_x, float* d_t) {
  if (!m || rows < 0 || !d_feat || !d_x) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = gb_mlp_norm_inputs(rows, d_feat, m->norm, (__nv_bfloat16*)d_x, st);
  if (e == cudaSuccess && d_t) {
    if (!d_tau || !d_frac) return GB_LW_E_ARGS;
    e = gb_mlp_norm_targets(rows, d_tau, d_frac, m->norm, d_t, st);
  }
  return e == cudaSuccess ? GB_LW_OK : fail(m->ctx, e, "training inputs");
}

int gb_lw_mlp_gradients(gb_lw_mlp* m, void* stream, int64_t rows, const void* d_x, const float* d_t, float* d_grad,
                        float* d_loss) {
  if (!m || rows < 1 || (rows % 8) || !d_x || !d_t) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  int rc = ensure_rows(m, rows);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (d_loss) cudaMemsetAsync(d_loss, 0, 4, st);
  cudaError_t e = gb_mlp_forward_backward(m->b, rows, (const __nv_bfloat16*)d_x, d_t, m->d_w,
                                          d_grad ? d_grad : m->d_grad, d_loss, st);
  return e == cudaSuccess ? GB_LW_OK : fail(m->ctx, e, "forward/backward");
}

int gb_lw_mlp_train_step(gb_lw_mlp* m, void* stream, int64_t rows, const void* d_x, const float* d_t, float lr,
                         float* d_loss) {
  int rc = gb_lw_mlp_gradients(m, stream, rows, d_x, d_t, nullptr, d_loss);
  if (rc) return rc;
  m->step += 1;
  m->img_dirty = true;
  cudaError_t e = gb_mlp_adam(m->b, m->d_grad, lr, m->step, (cudaStream_t)stream);
  return e == cudaSuccess ? GB_LW_OK : fail(m->ctx, e, "adam");
}

int gb_lw_mlp_forward(gb_lw_mlp* m, void* stream, int64_t rows, const void* d_x, float* d_y) {
  if (!m || rows < 1 || (rows % 8) || !d_x || !d_y) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  int rc = ensure_rows(m, rows);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // the training forward pass writes y into the activation buffers; copy it out
  std::vector<char> none;
  float* d_t = nullptr;
  if (cudaMalloc(&d_t, (size_t)rows * GB_MLP_NOUTP * 4) != cudaSuccess) {
    cudaGetLastError();
    return GB_LW_E_NOMEM;
  }
  cudaMemsetAsync(d_t, 0, (size_t)rows * GB_MLP_NOUTP * 4, st);
  cudaError_t e = gb_mlp_forward_backward(m->b, rows, (const __nv_bfloat16*)d_x, d_t, m->d_w, m->d_grad, nullptr, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_y, m->b.y, (size_t)rows * GB_MLP_NOUTP * 4, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_t);
  return e == cudaSuccess ? GB_LW_OK : fail(m->ctx, e, "forward");
}

int gb_lw_mlp_set_engine(gb_lw_mlp* m, int engine) {
  if (!m || (engine != GB_LW_MLP_MMA_SYNC && engine != GB_LW_MLP_TCGEN05)) return GB_LW_E_ARGS;
  m->engine = engine;
  return GB_LW_OK;
}

int gb_lw_mlp_infer(gb_lw_mlp* m, void* stream, const gb_lw_grid* grid, uint16_t* d_tau16, uint16_t* d_frac16,
                    uint8_t* d_flag) {
  if (!m || !grid || !d_tau16 || !d_frac16 || !d_flag) return GB_LW_E_ARGS;
  // the tensor-core engine stores four outputs (8 bytes) at a time
  if (((uintptr_t)d_tau16 | (uintptr_t)d_frac16) & 7) return GB_LW_E_ARGS;
  __half* d_tau = reinterpret_cast<__half*>(d_tau16);
  __half* d_frac = reinterpret_cast<__half*>(d_frac16);
  if (grid->ncol < 0 || grid->nlay < 1 || grid->ld_in < grid->ncol) return GB_LW_E_ARGS;
  cudaSetDevice(m->ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (m->engine == GB_LW_MLP_TCGEN05) {
    if (!m->d_img && cudaMalloc(&m->d_img, gb_mlp_tc_image_bytes()) != cudaSuccess) {
      cudaGetLastError();
      return GB_LW_E_NOMEM;
    }
    if (m->img_dirty) {
      e = gb_mlp_tc_images(m->b.p16, m->b.p32, m->norm, m->d_img, st);
      if (e != cudaSuccess) return fail(m->ctx, e, "weight images");
      m->img_dirty = false;
    }
    e = gb_mlp_infer_tc(grid_in(*grid), m->norm, m->d_img, m->ctx->tabs.grav, m->ctx->tabs.avogad, d_tau, d_frac,
                        d_flag, m->ctx->d_err, m->ctx->num_sms, st);
  } else {
    e = gb_mlp_infer(grid_in(*grid), m->norm, m->b.p16, m->b.p32, m->ctx->tabs.grav, m->ctx->tabs.avogad, d_tau,
                     d_frac, d_flag, m->ctx->num_sms, st);
  }
  return e == cudaSuccess ? GB_LW_OK : fail(m->ctx, e, "inference");
}

int gb_rrtmg_lw_batch_surrogate(gb_lw_context* ctx, void* stream, int ngrid, const gb_lw_grid* grids, gb_lw_mlp* m) {
  if (!ctx || !m || !grids || ngrid < 1 || ngrid > GB_LW_MAX_GRIDS) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  size_t rows = 0;
  for (int i = 0; i < ngrid; ++i) rows += (size_t)std::max(grids[i].ncol, 0) * std::max(grids[i].nlay, 0);
  if (rows > ctx->sur_rows) {
    cudaFree(ctx->d_sur);
    cudaFree(ctx->d_sur_flag);
    ctx->d_sur = nullptr;
    ctx->d_sur_flag = nullptr;
    ctx->sur_rows = 0;
    if (cudaMalloc(&ctx->d_sur, rows * 2 * GB_NGPT_MLP * sizeof(uint16_t)) != cudaSuccess ||
        cudaMalloc(&ctx->d_sur_flag, rows) != cudaSuccess) {
      cudaGetLastError();
      ctx->last_error = "device allocation of the learned gas-optics buffers failed";
      return GB_LW_E_NOMEM;
    }
    ctx->sur_rows = rows;
  }
  std::vector<gb_lw_grid> g(grids, grids + ngrid);
  size_t off = 0;
  for (int i = 0; i < ngrid; ++i) {
    const size_t r = (size_t)std::max(g[i].ncol, 0) * std::max(g[i].nlay, 0);
    uint16_t* tau = ctx->d_sur + off * 2 * GB_NGPT_MLP;
    uint16_t* frac = tau + r * GB_NGPT_MLP;
    uint8_t* flag = ctx->d_sur_flag + off;
    int rc = gb_lw_mlp_infer(m, stream, &g[i], tau, frac, flag);
    if (rc) return rc;
    g[i].sur_tau = tau;
    g[i].sur_frac = frac;
    g[i].sur_flag = flag;
    off += r;
  }
  LwBatch b;
  int rc = gb_ctx_make_batch(ctx, ngrid, g.data(), 1.0, b);
  if (rc) return rc;
  return gb_ctx_launch_batch(ctx, b, (cudaStream_t)stream);
}

int gb_lw_mlp_save(gb_lw_mlp* m, const char* path) {
  if (!m || !path) return GB_LW_E_ARGS;
  std::vector<float> p(GB_MLP_NPARAM);
  int rc = gb_lw_mlp_get_params(m, p.data(), nullptr);
  if (rc) return rc;
  FILE* f = std::fopen(path, "wb");
  if (!f) return GB_LW_E_ARGS;
  const char magic[8] = {'G', 'B', 'L', 'W', 'M', 'L', 'P', '1'};
  const int32_t dims[2] = {GB_MLP_NPARAM, GB_LW_MLP_NNORM};
  bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(dims, 4, 2, f) == 2 &&
            std::fwrite(&m->norm, sizeof(GbMlpNorm), 1, f) == 1 &&
            std::fwrite(p.data(), 4, GB_MLP_NPARAM, f) == (size_t)GB_MLP_NPARAM;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GB_LW_OK : GB_LW_E_ARGS;
}

int gb_lw_mlp_load(gb_lw_context* ctx, const char* path, gb_lw_mlp** out) {
  if (!ctx || !path || !out) return GB_LW_E_ARGS;
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return GB_LW_E_TABLES;
  char magic[8];
  int32_t dims[2];
  GbMlpNorm n;
  std::vector<float> p(GB_MLP_NPARAM);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "GBLWMLP1", 8) == 0 &&
            std::fread(dims, 4, 2, f) == 2 && dims[0] == GB_MLP_NPARAM && dims[1] == GB_LW_MLP_NNORM &&
            std::fread(&n, sizeof(GbMlpNorm), 1, f) == 1 && std::fread(p.data(), 4, GB_MLP_NPARAM, f) == (size_t)GB_MLP_NPARAM;
  std::fclose(f);
  if (!ok) return GB_LW_E_TABLES;
  gb_lw_mlp* m = nullptr;
  int rc = gb_lw_mlp_create(ctx, 1, &m);
  if (rc) return rc;
  rc = gb_lw_mlp_set_params(m, p.data(), (const float*)&n);
  if (rc) {
    gb_lw_mlp_destroy(m);
    return rc;
  }
  *out = m;
  return GB_LW_OK;
}

}  // extern "C"
