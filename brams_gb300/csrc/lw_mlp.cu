// Training and inference kernels of the taumol MLP (network in lw_mlp.cuh).
//
// Training (hand-written, no library GEMM):
//   gemm_kernel      bf16 tensor-core GEMM (mma.sync m16n8k16, fp32
//                    accumulators) with transposes and fused epilogues:
//                    bias+SiLU (forward hidden layers), bias (output layer),
//                    *silu'(z) (backward), fp32 atomics (weight gradients,
//                    split over the batch);
//   loss_kernel      dL/dy of the weighted mean-square loss and the loss;
//   colsum_kernel    bias gradients;
//   adam_kernel      Adam on fp32 master weights, writing the bf16 copy.
// Inference:
//   infer_kernel     the whole network per warp on 16 layers at a time, the
//                    weights resident in shared memory, activations kept in
//                    registers between layers (an m16n8 accumulator pair is
//                    the next layer's m16k16 operand); features are computed
//                    from the rrtmg_lw inputs and outputs written per column
//                    in the layout the column kernel reads.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "lw_mlp.cuh"
#include "lw_mlp.h"

using bf16 = __nv_bfloat16;

namespace gbmlp {

// ------------------------------------------------------------------ generic GEMM
enum Epi { EPI_F32 = 0, EPI_ATOMIC = 1, EPI_BIAS_SILU = 2, EPI_BIAS_F32 = 3, EPI_DSILU = 4 };

struct GemmArgs {
  int M, N, K, ksplit;
  const bf16* A;
  long long lda;  // AT = false: A[m * lda + k]; AT = true: A[k * lda + m]
  const bf16* B;
  long long ldb;  // BT = false: B[k * ldb + n]; BT = true: B[n * ldb + k]
  float* C;
  long long ldc;  // fp32 output (EPI_F32, EPI_ATOMIC, EPI_BIAS_F32)
  bf16* Z;
  bf16* Act;
  long long ldz;  // EPI_BIAS_SILU: Z = acc + bias, Act = silu(acc + bias); EPI_DSILU: Z = acc * silu'(Zin)
  const float* bias;
  const bf16* Zin;
};

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

template <bool AT, bool BT, int EPI>
__global__ void __launch_bounds__(128) gemm_kernel(GemmArgs g) {
  constexpr int SA = AT ? BK * (BM + PAD) : BM * (BK + PAD);
  constexpr int SB = BT ? BN * (BK + PAD) : BK * (BN + PAD);
  __shared__ __align__(16) bf16 sA[SA];
  __shared__ __align__(16) bf16 sB[SB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int bm = blockIdx.y * BM, bn = blockIdx.x * BN;
  const int k0 = blockIdx.z * g.ksplit, k1 = min(g.K, k0 + g.ksplit);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;

  for (int kb = k0; kb < k1; kb += BK) {
    // ---- stage A and B tiles (8 bf16 per vector; all extents are multiples of 8)
    for (int v = tid; v < BM * BK / 8; v += 128) {
      int r, c;  // r: row of the staged tile, c: first column
      if (AT) { r = v / (BM / 8); c = (v % (BM / 8)) * 8; }  // [BK][BM]
      else { r = v / (BK / 8); c = (v % (BK / 8)) * 8; }     // [BM][BK]
      const int m = AT ? bm + c : bm + r, k = AT ? kb + r : kb + c;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (m < g.M && k < k1) val = *reinterpret_cast<const uint4*>(AT ? g.A + (long long)k * g.lda + m : g.A + (long long)m * g.lda + k);
      *reinterpret_cast<uint4*>(sA + r * ((AT ? BM : BK) + PAD) + c) = val;
    }
    for (int v = tid; v < BN * BK / 8; v += 128) {
      int r, c;
      if (BT) { r = v / (BK / 8); c = (v % (BK / 8)) * 8; }  // [BN][BK]
      else { r = v / (BN / 8); c = (v % (BN / 8)) * 8; }     // [BK][BN]
      const int n = BT ? bn + r : bn + c, k = BT ? kb + c : kb + r;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (n < g.N && k < k1) val = *reinterpret_cast<const uint4*>(BT ? g.B + (long long)n * g.ldb + k : g.B + (long long)k * g.ldb + n);
      *reinterpret_cast<uint4*>(sB + r * ((BT ? BK : BN) + PAD) + c) = val;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
        const int m0 = wm * 32 + mi * 16;
        if (AT) {
          const bf16* p = sA + (kk + (lane & 7) + ((lane >> 4) << 3)) * (BM + PAD) + m0 + ((lane >> 3) & 1) * 8;
          ldsm_x4_t(smem_u32(p), af[mi][0], af[mi][1], af[mi][2], af[mi][3]);
        } else {
          const bf16* p = sA + (m0 + (lane & 15)) * (BK + PAD) + kk + (lane >> 4) * 8;
          ldsm_x4(smem_u32(p), af[mi][0], af[mi][1], af[mi][2], af[mi][3]);
        }
      }
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int n0 = wn * 32 + np * 16;
        if (BT) {
          const bf16* p = sB + (n0 + (lane & 7) + ((lane >> 4) << 3)) * (BK + PAD) + kk + ((lane >> 3) & 1) * 8;
          ldsm_x4(smem_u32(p), bfr[2 * np][0], bfr[2 * np][1], bfr[2 * np + 1][0], bfr[2 * np + 1][1]);
        } else {
          const bf16* p = sB + (kk + (lane & 15)) * (BN + PAD) + n0 + (lane >> 4) * 8;
          ldsm_x4_t(smem_u32(p), bfr[2 * np][0], bfr[2 * np][1], bfr[2 * np + 1][0], bfr[2 * np + 1][1]);
        }
      }
#pragma unroll
      for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) mma16816(acc[mi][ni], af[mi], bfr[ni][0], bfr[ni][1]);
    }
    __syncthreads();
  }
  // ---- epilogue
  const int gq = lane >> 2, tq = lane & 3;
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int m = bm + wm * 32 + mi * 16 + gq + h * 8;
        const int n = bn + wn * 32 + ni * 8 + 2 * tq;
        if (m >= g.M || n >= g.N) continue;
        const float v0 = acc[mi][ni][2 * h], v1 = acc[mi][ni][2 * h + 1];
        if (EPI == EPI_F32) {
          *reinterpret_cast<float2*>(g.C + (long long)m * g.ldc + n) = make_float2(v0, v1);
        } else if (EPI == EPI_ATOMIC) {
          atomicAdd(g.C + (long long)m * g.ldc + n, v0);
          atomicAdd(g.C + (long long)m * g.ldc + n + 1, v1);
        } else if (EPI == EPI_BIAS_F32) {
          *reinterpret_cast<float2*>(g.C + (long long)m * g.ldc + n) = make_float2(v0 + g.bias[n], v1 + g.bias[n + 1]);
        } else if (EPI == EPI_BIAS_SILU) {
          const float z0 = v0 + g.bias[n], z1 = v1 + g.bias[n + 1];
          *reinterpret_cast<uint32_t*>(g.Z + (long long)m * g.ldz + n) = pack_bf16(z0, z1);
          *reinterpret_cast<uint32_t*>(g.Act + (long long)m * g.ldz + n) = pack_bf16(silu(z0), silu(z1));
        } else {  // EPI_DSILU
          const __nv_bfloat162 z = *reinterpret_cast<const __nv_bfloat162*>(g.Zin + (long long)m * g.ldz + n);
          const float2 zf = __bfloat1622float2(z);
          *reinterpret_cast<uint32_t*>(g.Z + (long long)m * g.ldz + n) = pack_bf16(v0 * dsilu(zf.x), v1 * dsilu(zf.y));
        }
      }
}

template <bool AT, bool BT, int EPI>
cudaError_t gemm(const GemmArgs& a0, int splits, cudaStream_t st) {
  GemmArgs a = a0;
  splits = splits < 1 ? 1 : splits;
  a.ksplit = ((a.K + splits - 1) / splits + BK - 1) / BK * BK;
  splits = (a.K + a.ksplit - 1) / a.ksplit;
  dim3 grid((a.N + BN - 1) / BN, (a.M + BM - 1) / BM, splits);
  gemm_kernel<AT, BT, EPI><<<grid, 128, 0, st>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ elementwise
// dL/dy and the loss of L = sum_j w_j (y_j - t_j)^2 / (rows * 280), j < 280
__global__ void loss_kernel(long long rows, const float* __restrict__ y, const float* __restrict__ t,
                            const float* __restrict__ w, bf16* __restrict__ dy, float* __restrict__ loss) {
  __shared__ float red[32];
  const long long n = rows * GB_MLP_NOUTP;
  const float scale = 1.0f / ((float)rows * (float)GB_MLP_NOUT);
  float part = 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(i % GB_MLP_NOUTP);
    float d = 0.0f;
    if (j < GB_MLP_NOUT) {
      const float e = y[i] - t[i];
      d = 2.0f * w[j] * e * scale;
      part += w[j] * e * e * scale;
    }
    dy[i] = __float2bfloat16_rn(d);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && loss) atomicAdd(loss, v);
  }
}

// out[n] += sum over rows of x[m][n] (bias gradients); one block per 32 columns x 256-row slab
__global__ void colsum_kernel(long long rows, int N, const bf16* __restrict__ x, float* __restrict__ out) {
  const int n = blockIdx.x * 32 + (threadIdx.x & 31);
  const int ry = threadIdx.x >> 5;  // 8 row lanes
  float s = 0.0f;
  if (n < N)
    for (long long m = blockIdx.y * 256 + ry; m < rows && m < (blockIdx.y + 1) * 256LL; m += 8) s += __bfloat162float(x[m * N + n]);
  __shared__ float red[8][33];
  red[ry][threadIdx.x & 31] = s;
  __syncthreads();
  if (ry == 0 && n < N) {
    float t = 0.0f;
    for (int k = 0; k < 8; ++k) t += red[k][threadIdx.x & 31];
    atomicAdd(out + n, t);
  }
}

__global__ void adam_kernel(int n, float* __restrict__ p, const float* __restrict__ grad, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ p16, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g, vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    p16[i] = __float2bfloat16_rn(pi);
  }
}

__global__ void to_bf16_kernel(int n, const float* __restrict__ p, bf16* __restrict__ q) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) q[i] = __float2bfloat16_rn(p[i]);
}

// standardised bf16 network inputs [rows][16] from raw features [rows][9]
__global__ void norm_inputs_kernel(long long rows, const float* __restrict__ f, GbMlpNorm nm, bf16* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows * GB_MLP_KIN;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / GB_MLP_KIN;
    const int j = (int)(i % GB_MLP_KIN);
    const float v = j < GB_MLP_NF ? (f[r * GB_MLP_NF + j] - nm.in_mu[j]) / nm.in_sd[j] : 0.0f;
    x[i] = __float2bfloat16_rn(v);
  }
}

// standardised targets [rows][288] from taumol's taug and fracs [rows][140]
__global__ void norm_targets_kernel(long long rows, const float* __restrict__ tau, const float* __restrict__ frac,
                                    GbMlpNorm nm, float* __restrict__ t) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows * GB_MLP_NOUTP;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / GB_MLP_NOUTP;
    const int j = (int)(i % GB_MLP_NOUTP);
    float v = 0.0f;
    if (j < GB_NGPT_MLP) v = (logf(fmaxf(tau[r * GB_NGPT_MLP + j], GB_MLP_TAU_FLOOR)) - nm.out_mu[j]) / nm.out_sd[j];
    else if (j < GB_MLP_NOUT) v = (frac[r * GB_NGPT_MLP + j - GB_NGPT_MLP] - nm.out_mu[j]) / nm.out_sd[j];
    t[i] = v;
  }
}

// per-column raw features of every layer of one grid, rows = icol * nlay + lay
__global__ void features_kernel(GbMlpGridIn g, double grav, double avogad, float* __restrict__ f) {
  const long long rows = (long long)g.ncol * g.nlay;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
    const long long icol = r / g.nlay;
    const int lay = (int)(r - icol * g.nlay);
    layer_features(g.play, g.plev, g.tlay, g.tlev, g.h2ovmr, g.o3vmr, g.co2vmr, g.ch4vmr, g.n2ovmr, g.ld, icol, lay,
                   grav, avogad, f + r * GB_MLP_NF);
  }
}

// ------------------------------------------------------------------ inference
constexpr int IW = 8;                       // warps per inference block
constexpr int SW_H = GB_MLP_H + 8;          // padded row strides (bf16 elements)
constexpr int SW_O = GB_MLP_NOUTP + 8;
constexpr int SX = GB_MLP_KIN + 8;

struct InferSmem {
  bf16 w1[GB_MLP_KIN * SW_H];
  bf16 w2[GB_MLP_H * SW_H];
  bf16 w3[GB_MLP_H * SW_H];
  bf16 w4[GB_MLP_H * SW_O];
  float b1[GB_MLP_H], b2[GB_MLP_H], b3[GB_MLP_H], b4[GB_MLP_NOUTP];
  float omu[GB_MLP_NOUTP], osd[GB_MLP_NOUTP];
  bf16 x[IW][16 * SX];
};

// silu(acc + bias) of two n8 accumulator tiles -> one k16 operand fragment
__device__ __forceinline__ void to_operand(const float* c0, const float* c1, const float* bias, int n0, int tq,
                                           uint32_t* a) {
  const float bA = bias[n0 + 2 * tq], bB = bias[n0 + 2 * tq + 1];
  const float bC = bias[n0 + 8 + 2 * tq], bD = bias[n0 + 8 + 2 * tq + 1];
  a[0] = pack_bf16(silu(c0[0] + bA), silu(c0[1] + bB));
  a[1] = pack_bf16(silu(c0[2] + bA), silu(c0[3] + bB));
  a[2] = pack_bf16(silu(c1[0] + bC), silu(c1[1] + bD));
  a[3] = pack_bf16(silu(c1[2] + bC), silu(c1[3] + bD));
}

// hidden layer 128 -> 128 on operand fragments held in registers
__device__ __forceinline__ void hidden_layer(const bf16* w, const float* bias, uint32_t (&a)[8][4], int lane) {
  float acc[16][4];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
  for (int kt = 0; kt < 8; ++kt) {
#pragma unroll
    for (int np = 0; np < 8; ++np) {
      uint32_t b0, b1, b2, b3;
      ldsm_x4_t(smem_u32(w + (kt * 16 + (lane & 15)) * SW_H + np * 16 + (lane >> 4) * 8), b0, b1, b2, b3);
      mma16816(acc[2 * np], a[kt], b0, b1);
      mma16816(acc[2 * np + 1], a[kt], b2, b3);
    }
  }
  const int tq = lane & 3;
#pragma unroll
  for (int kt = 0; kt < 8; ++kt) to_operand(acc[2 * kt], acc[2 * kt + 1], bias, kt * 16, tq, a[kt]);
}

__global__ void __launch_bounds__(IW * 32, 1) infer_kernel(GbMlpGridIn g, GbMlpNorm nm, const bf16* __restrict__ p16,
                                                           const float* __restrict__ p32, double grav, double avogad,
                                                           __half* __restrict__ out_tau, __half* __restrict__ out_frac,
                                                           unsigned char* __restrict__ flag) {
  extern __shared__ __align__(16) char smraw[];
  InferSmem& S = *reinterpret_cast<InferSmem*>(smraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // weights (bf16, padded rows), biases and output scaling into shared memory
  for (int i = tid; i < GB_MLP_KIN * GB_MLP_H; i += blockDim.x) S.w1[(i / GB_MLP_H) * SW_H + i % GB_MLP_H] = p16[GB_MLP_OFF_W1 + i];
  for (int i = tid; i < GB_MLP_H * GB_MLP_H; i += blockDim.x) {
    S.w2[(i / GB_MLP_H) * SW_H + i % GB_MLP_H] = p16[GB_MLP_OFF_W2 + i];
    S.w3[(i / GB_MLP_H) * SW_H + i % GB_MLP_H] = p16[GB_MLP_OFF_W3 + i];
  }
  for (int i = tid; i < GB_MLP_H * GB_MLP_NOUTP; i += blockDim.x)
    S.w4[(i / GB_MLP_NOUTP) * SW_O + i % GB_MLP_NOUTP] = p16[GB_MLP_OFF_W4 + i];
  for (int i = tid; i < GB_MLP_H; i += blockDim.x) {
    S.b1[i] = p32[GB_MLP_OFF_B1 + i];
    S.b2[i] = p32[GB_MLP_OFF_B2 + i];
    S.b3[i] = p32[GB_MLP_OFF_B3 + i];
  }
  for (int i = tid; i < GB_MLP_NOUTP; i += blockDim.x) {
    S.b4[i] = p32[GB_MLP_OFF_B4 + i];
    S.omu[i] = nm.out_mu[i];
    S.osd[i] = nm.out_sd[i];
  }
  __syncthreads();
  const long long rows = (long long)g.ncol * g.nlay;
  const long long ntile = (rows + 15) / 16;
  bf16* sx = S.x[warp];
  const int gq = lane >> 2, tq = lane & 3;
  for (long long tile = (long long)blockIdx.x * IW + warp; tile < ntile; tile += (long long)gridDim.x * IW) {
    // rows are layer-major (consecutive rows = consecutive columns of one layer: coalesced loads)
    const long long r0 = tile * 16;
    if (lane < 16) {
      const long long r = r0 + lane;
      float f[GB_MLP_NF];
      bool ok = false;
      if (r < rows) {
        const int lay = (int)(r / g.ncol);
        const long long icol = r - (long long)lay * g.ncol;
        layer_features(g.play, g.plev, g.tlay, g.tlev, g.h2ovmr, g.o3vmr, g.co2vmr, g.ch4vmr, g.n2ovmr, g.ld, icol, lay,
                       grav, avogad, f);
        ok = in_range(f, nm);
        flag[icol * g.nlay + lay] = ok ? 1 : 0;
      } else {
#pragma unroll
        for (int i = 0; i < GB_MLP_NF; ++i) f[i] = nm.in_mu[i];
      }
#pragma unroll
      for (int j = 0; j < GB_MLP_KIN; ++j)
        sx[lane * SX + j] = __float2bfloat16_rn(j < GB_MLP_NF ? (f[j] - nm.in_mu[j]) / nm.in_sd[j] : 0.0f);
    }
    __syncwarp();
    // layer 1: 16 -> 128
    uint32_t a[8][4];
    {
      uint32_t x[4];
      ldsm_x4(smem_u32(sx + (lane & 15) * SX + (lane >> 4) * 8), x[0], x[1], x[2], x[3]);
      float acc[16][4];
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
      for (int np = 0; np < 8; ++np) {
        uint32_t b0, b1, b2, b3;
        ldsm_x4_t(smem_u32(S.w1 + (lane & 15) * SW_H + np * 16 + (lane >> 4) * 8), b0, b1, b2, b3);
        mma16816(acc[2 * np], x, b0, b1);
        mma16816(acc[2 * np + 1], x, b2, b3);
      }
#pragma unroll
      for (int kt = 0; kt < 8; ++kt) to_operand(acc[2 * kt], acc[2 * kt + 1], S.b1, kt * 16, tq, a[kt]);
    }
    hidden_layer(S.w2, S.b2, a, lane);
    hidden_layer(S.w3, S.b3, a, lane);
    // output layer 128 -> 288 in chunks of 32 columns
#pragma unroll 1
    for (int ch = 0; ch < GB_MLP_NOUTP / 32; ++ch) {
      float acc[4][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
      for (int kt = 0; kt < 8; ++kt)
#pragma unroll
        for (int np = 0; np < 2; ++np) {
          uint32_t b0, b1, b2, b3;
          ldsm_x4_t(smem_u32(S.w4 + (kt * 16 + (lane & 15)) * SW_O + ch * 32 + np * 16 + (lane >> 4) * 8), b0, b1, b2, b3);
          mma16816(acc[2 * np], a[kt], b0, b1);
          mma16816(acc[2 * np + 1], a[kt], b2, b3);
        }
#pragma unroll
      for (int ni = 0; ni < 4; ++ni)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const long long r = r0 + gq + 8 * h;
          const int j = ch * 32 + ni * 8 + 2 * tq;
          if (r >= rows || j >= GB_MLP_NOUT) continue;
          const int lay = (int)(r / g.ncol);
          const long long icol = r - (long long)lay * g.ncol;
          const long long o = (icol * g.nlay + lay) * GB_NGPT_MLP;
          const float y0 = (acc[ni][2 * h] + S.b4[j]) * S.osd[j] + S.omu[j];
          const float y1 = (acc[ni][2 * h + 1] + S.b4[j + 1]) * S.osd[j + 1] + S.omu[j + 1];
          if (j < GB_NGPT_MLP)
            *reinterpret_cast<__half2*>(out_tau + o + j) =
                __floats2half2_rn(fminf(__expf(y0), GB_MLP_HALF_MAX), fminf(__expf(y1), GB_MLP_HALF_MAX));
          else
            *reinterpret_cast<__half2*>(out_frac + o + j - GB_NGPT_MLP) = __floats2half2_rn(y0, y1);
        }
    }
    __syncwarp();
  }
}

}  // namespace gbmlp

// ------------------------------------------------------------------ host side
using namespace gbmlp;

size_t gb_mlp_infer_smem() { return sizeof(InferSmem); }

cudaError_t gb_mlp_features(const GbMlpGridIn& g, double grav, double avogad, float* d_feat, cudaStream_t st) {
  const long long rows = (long long)g.ncol * g.nlay;
  if (rows == 0) return cudaSuccess;
  const int blocks = (int)((rows + 255) / 256 < 4096 ? (rows + 255) / 256 : 4096);
  features_kernel<<<blocks, 256, 0, st>>>(g, grav, avogad, d_feat);
  return cudaGetLastError();
}

cudaError_t gb_mlp_norm_inputs(long long rows, const float* d_feat, const GbMlpNorm& nm, bf16* d_x, cudaStream_t st) {
  if (rows == 0) return cudaSuccess;
  norm_inputs_kernel<<<2048, 256, 0, st>>>(rows, d_feat, nm, d_x);
  return cudaGetLastError();
}

cudaError_t gb_mlp_norm_targets(long long rows, const float* d_tau, const float* d_frac, const GbMlpNorm& nm,
                                float* d_t, cudaStream_t st) {
  if (rows == 0) return cudaSuccess;
  norm_targets_kernel<<<4096, 256, 0, st>>>(rows, d_tau, d_frac, nm, d_t);
  return cudaGetLastError();
}

cudaError_t gb_mlp_forward_backward(const MlpBuffers& b, long long rows, const bf16* d_x, const float* d_t,
                                    const float* d_w, float* d_grad, float* d_loss, cudaStream_t st) {
  const int H = GB_MLP_H, O = GB_MLP_NOUTP;
  const int M = (int)rows;
  cudaError_t e;
  GemmArgs a{};
  // forward: Z1/A1, Z2/A2, Z3/A3, Y
  const bf16* W[4] = {b.p16 + GB_MLP_OFF_W1, b.p16 + GB_MLP_OFF_W2, b.p16 + GB_MLP_OFF_W3, b.p16 + GB_MLP_OFF_W4};
  const float* Bs[4] = {b.p32 + GB_MLP_OFF_B1, b.p32 + GB_MLP_OFF_B2, b.p32 + GB_MLP_OFF_B3, b.p32 + GB_MLP_OFF_B4};
  const bf16* in = d_x;
  int kin = GB_MLP_KIN;
  for (int l = 0; l < 3; ++l) {
    a = GemmArgs{};
    a.M = M; a.N = H; a.K = kin;
    a.A = in; a.lda = kin;
    a.B = W[l]; a.ldb = H;
    a.Z = b.z[l]; a.Act = b.act[l]; a.ldz = H; a.bias = Bs[l];
    if ((e = gemm<false, false, EPI_BIAS_SILU>(a, 1, st)) != cudaSuccess) return e;
    in = b.act[l];
    kin = H;
  }
  a = GemmArgs{};
  a.M = M; a.N = O; a.K = H;
  a.A = b.act[2]; a.lda = H;
  a.B = W[3]; a.ldb = O;
  a.C = b.y; a.ldc = O; a.bias = Bs[3];
  if ((e = gemm<false, false, EPI_BIAS_F32>(a, 1, st)) != cudaSuccess) return e;
  loss_kernel<<<1024, 256, 0, st>>>(rows, b.y, d_t, d_w, b.dy, d_loss);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // backward
  if ((e = cudaMemsetAsync(d_grad, 0, GB_MLP_NPARAM * sizeof(float), st)) != cudaSuccess) return e;
  const int splits = (int)((rows + 2047) / 2048);
  const bf16* dZ = b.dy;
  int nout = O;
  float* gW[4] = {d_grad + GB_MLP_OFF_W1, d_grad + GB_MLP_OFF_W2, d_grad + GB_MLP_OFF_W3, d_grad + GB_MLP_OFF_W4};
  float* gB[4] = {d_grad + GB_MLP_OFF_B1, d_grad + GB_MLP_OFF_B2, d_grad + GB_MLP_OFF_B3, d_grad + GB_MLP_OFF_B4};
  for (int l = 3; l >= 0; --l) {
    const bf16* Ain = l == 0 ? d_x : b.act[l - 1];
    const int kin_l = l == 0 ? GB_MLP_KIN : H;
    // dW_l = A_{l-1}^T dZ_l  (reduction over the batch, split across blocks)
    a = GemmArgs{};
    a.M = kin_l; a.N = nout; a.K = M;
    a.A = Ain; a.lda = kin_l;
    a.B = dZ; a.ldb = nout;
    a.C = gW[l]; a.ldc = nout;
    if ((e = gemm<true, false, EPI_ATOMIC>(a, splits, st)) != cudaSuccess) return e;
    colsum_kernel<<<dim3((nout + 31) / 32, (unsigned)((rows + 255) / 256)), 256, 0, st>>>(rows, nout, dZ, gB[l]);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (l == 0) break;
    // dZ_{l-1} = (dZ_l W_l^T) * silu'(Z_{l-1})
    a = GemmArgs{};
    a.M = M; a.N = H; a.K = nout;
    a.A = dZ; a.lda = nout;
    a.B = W[l]; a.ldb = nout;  // W_l is [in][out]: as B^T with B[n][k] = W[n][k]
    a.Z = b.dz[l - 1]; a.ldz = H; a.Zin = b.z[l - 1];
    if ((e = gemm<false, true, EPI_DSILU>(a, 1, st)) != cudaSuccess) return e;
    dZ = b.dz[l - 1];
    nout = H;
  }
  return cudaSuccess;
}

cudaError_t gb_mlp_adam(const MlpBuffers& b, const float* d_grad, float lr, int step, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  adam_kernel<<<(GB_MLP_NPARAM + 255) / 256, 256, 0, st>>>(GB_MLP_NPARAM, b.p32, d_grad, b.m, b.v, b.p16, lr, b1, b2,
                                                           1e-8f, c1, c2);
  return cudaGetLastError();
}

cudaError_t gb_mlp_sync_bf16(const MlpBuffers& b, cudaStream_t st) {
  to_bf16_kernel<<<(GB_MLP_NPARAM + 255) / 256, 256, 0, st>>>(GB_MLP_NPARAM, b.p32, b.p16);
  return cudaGetLastError();
}

cudaError_t gb_mlp_infer(const GbMlpGridIn& g, const GbMlpNorm& nm, const bf16* p16, const float* p32, double grav,
                         double avogad, __half* d_tau, __half* d_frac, unsigned char* d_flag, int nsm, cudaStream_t st) {
  const long long rows = (long long)g.ncol * g.nlay;
  if (rows == 0) return cudaSuccess;
  const size_t sm = sizeof(InferSmem);
  cudaError_t e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const long long tiles = (rows + 15) / 16;
  long long blocks = (tiles + IW - 1) / IW;
  if (blocks > nsm) blocks = nsm;
  infer_kernel<<<(int)blocks, IW * 32, sm, st>>>(g, nm, p16, p32, grav, avogad, d_tau, d_frac, d_flag);
  return cudaGetLastError();
}
