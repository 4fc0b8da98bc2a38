// Inference of the taumol MLP on the 5th-generation tensor cores (tcgen05).
//
// One CTA per SM, persistent over tiles of 128 layers (rows).  The four
// weight matrices live in shared memory for the whole kernel as K-major,
// 128-byte-swizzled bf16 images (prepared once by mlp_tc_images_kernel); the
// 128 x K activation tile is written to shared memory in the same layout by
// the epilogue of the previous layer.  One thread issues tcgen05.mma
// (M = 128, kind::f16, bf16 operands, fp32 accumulators in tensor memory) and
// commits to an mbarrier; sixteen warps then read the accumulators back with
// tcgen05.ld (warp w: TMEM lanes 32*(w%4).., column quarter w/4), apply bias and
// SiLU, and write the next layer's operand tile.  The output layer
// (N = 288 = 2 x 144) is un-standardised and written as binary16 per
// (column, layer) in the layout the column kernel reads.  The next tile's
// features are formed while the output layer's MMAs run, and its raw inputs
// loaded (into registers) a tile ahead.
//
// Every wait on the mbarrier is bounded; a wait that runs out records an
// error flag, and the kernel frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lw_mlp.cuh"
#include "lw_common.h"
#include "lw_mlp.h"

namespace gbtc {

using bf16 = __nv_bfloat16;

constexpr int M = 128;          // rows per tile (TMEM lanes)
constexpr int KIN = 64;         // layer-1 K (9 features, zero padded to one 128-byte row)
constexpr int H = GB_MLP_H;     // 128
constexpr int NO = GB_MLP_NOUTP;  // 288
constexpr int NOH = NO / 2;     // 144 per output MMA
constexpr int NT = 512;         // 16 warps: 4 per TMEM lane quarter
constexpr int TMEM_COLS = 512;

// shared-memory image offsets (bytes; every operand tile starts on 1024 bytes)
constexpr int OFF_W1 = 0;                             // [128 n][64 k]          16 KB
constexpr int OFF_W2 = OFF_W1 + H * 128;              // 2 k-blocks x [128][64] 32 KB
constexpr int OFF_W3 = OFF_W2 + 2 * H * 128;          // 32 KB
constexpr int OFF_W4 = OFF_W3 + 2 * H * 128;          // 2 k-blocks x [288][64] 72 KB
constexpr int IMG_BYTES = OFF_W4 + 2 * NO * 128;      // weight images
constexpr int OFF_X = IMG_BYTES;                      // [128 m][64 k]          16 KB
constexpr int OFF_H = OFF_X + M * 128;                // 2 k-blocks x [128][64] 32 KB
constexpr int OFF_F32 = OFF_H + 2 * M * 128;          // b1 b2 b3 (128 each), output scale and shift (288 each)
constexpr int NF32 = 3 * H + 2 * NO;
constexpr int OFF_BAR = OFF_F32 + NF32 * 4;           // two mbarriers (MMA, weights) + TMEM address
constexpr int SMEM_BYTES = OFF_BAR + 24;
constexpr int BULK = 16384;                           // bytes per bulk copy of the weight images
static_assert(OFF_W2 % 1024 == 0 && OFF_W3 % 1024 == 0 && OFF_W4 % 1024 == 0 && OFF_X % 1024 == 0 &&
                  OFF_H % 1024 == 0 && (NOH * 128) % 1024 == 0,
              "operand tiles must start on 1024-byte boundaries (128-byte swizzle atoms)");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(NT / 32 * 32 * 32 <= OFF_F32 - OFF_X, "the output staging fits in the input and hidden tiles");
static_assert(IMG_BYTES % 16 == 0 && OFF_BAR % 8 == 0, "bulk copies move multiples of 16 bytes; mbarriers are 8-byte aligned");

// byte offset of element (r, k) in a K-major, 128-byte-swizzled tile of R rows
// (k-blocks of 64 elements; 16-byte chunk c of row r sits at chunk c ^ (r & 7))
__host__ __device__ constexpr uint32_t sw128(int R, int r, int k) {
  return (uint32_t)((k >> 6) * (R * 128) + r * 128 + ((((k & 63) >> 3) ^ (r & 7)) << 4) + (k & 7) * 2);
}

// tcgen05 shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row
// groups 1024 bytes apart (stride byte offset), leading byte offset unused
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused with this swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset
  d |= (uint64_t)1 << 46;                        // descriptor version
  d |= (uint64_t)2 << 61;                        // 128-byte swizzle
  return d;
}

// instruction descriptor, kind::f16: bf16 A and B (K-major), fp32 D, M x N
__host__ __device__ constexpr uint32_t idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

// bounded wait for the mbarrier phase with the given parity; false if it ran out
__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); ++i) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 accumulator columns of the warp's 32 lanes, without waiting: the values
// are defined only after wait_ld16 / wait_ld32 on the same registers
__device__ __forceinline__ void ld16_async(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// wait for the thread's tensor-memory loads; the registers they fill are
// read-write operands, so no use of them moves above the wait
__device__ __forceinline__ void wait_ld16(uint32_t* r) {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}
__device__ __forceinline__ void wait_ld32(uint32_t* a, uint32_t* b) {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n"
               : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7]),
                 "+r"(a[8]), "+r"(a[9]), "+r"(a[10]), "+r"(a[11]), "+r"(a[12]), "+r"(a[13]), "+r"(a[14]), "+r"(a[15]),
                 "+r"(b[0]), "+r"(b[1]), "+r"(b[2]), "+r"(b[3]), "+r"(b[4]), "+r"(b[5]), "+r"(b[6]), "+r"(b[7]),
                 "+r"(b[8]), "+r"(b[9]), "+r"(b[10]), "+r"(b[11]), "+r"(b[12]), "+r"(b[13]), "+r"(b[14]), "+r"(b[15])
               :
               : "memory");
}

// layer and column of row r of the layer-major row space (32-bit division
// where the row index fits, the 64-bit one otherwise; both exact)
__device__ __forceinline__ int row_layer(long long r, int ncol, long long& icol) {
  const int lay = r <= 0x7fffffffLL ? (int)((uint32_t)r / (uint32_t)ncol) : (int)(r / ncol);
  icol = r - (long long)lay * ncol;
  return lay;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 2^x by the PTX approximate base-2 exponential
__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;\n" : "=f"(y) : "f"(x));
  return y;
}

// silu(acc + bias) of 32 consecutive hidden units (from n0) of this thread's
// row, into the next layer's operand tile
__device__ __forceinline__ void hidden_epilogue(uint32_t tcol, int row, int n0, const float* bias, char* hbase) {
  uint32_t r[32];  // both 16-column loads in flight before the one wait
  ld16_async(tcol, r);
  ld16_async(tcol + 16, r + 16);
  wait_ld32(r, r + 16);
#pragma unroll
  for (int c16 = 0; c16 < 2; ++c16) {
    float v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[c16 * 16 + i]);
    float b[16];
#pragma unroll
    for (int i = 0; i < 4; ++i) {  // n0 is a multiple of 32 and bias 16-byte aligned
      const float4 q = reinterpret_cast<const float4*>(bias + n0 + c16 * 16)[i];
      b[4 * i] = q.x, b[4 * i + 1] = q.y, b[4 * i + 2] = q.z, b[4 * i + 3] = q.w;
    }
    uint32_t p[8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
      p[i] = gbmlp::pack_bf16(gbmlp::silu(v[2 * i] + b[2 * i]), gbmlp::silu(v[2 * i + 1] + b[2 * i + 1]));
    const int k0 = n0 + c16 * 16;
    *reinterpret_cast<uint4*>(hbase + sw128(M, row, k0)) = make_uint4(p[0], p[1], p[2], p[3]);
    *reinterpret_cast<uint4*>(hbase + sw128(M, row, k0 + 8)) = make_uint4(p[4], p[5], p[6], p[7]);
  }
}

__global__ void __launch_bounds__(NT, 1) infer_tc_kernel(GbMlpGridIn g, GbMlpNorm nm, const uint4* __restrict__ img,
                                                         const float* __restrict__ f32, double grav, double avogad,
                                                         __half* __restrict__ out_tau, __half* __restrict__ out_frac,
                                                         unsigned char* __restrict__ flag, int* __restrict__ err) {
  extern __shared__ __align__(1024) char sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* sf = reinterpret_cast<const float*>(sm + OFF_F32);
  // output j = acc * oscale[j] + oshift[j]: the output bias and un-standardisation
  // folded together, in base-2 logarithm units for taug (j < 140)
  const float *b1 = sf, *b2 = sf + H, *b3 = sf + 2 * H, *oscale = sf + 3 * H, *oshift = oscale + NO;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + OFF_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + OFF_BAR + 16);
  // weight images into shared memory by bulk (TMA) copies completing on an
  // mbarrier; the fp32 vectors by plain loads
  uint64_t* wbar = bar + 1;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(wbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(wbar)), "r"(IMG_BYTES)
                 : "memory");
    for (int off = 0; off < IMG_BYTES; off += BULK) {
      const int n = IMG_BYTES - off < BULK ? IMG_BYTES - off : BULK;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
              smem_addr(sm + off)),
          "l"(reinterpret_cast<const char*>(img) + off), "r"(n), "r"(smem_addr(wbar))
          : "memory");
    }
  }
  for (int i = tid; i < NF32; i += NT) reinterpret_cast<float*>(sm + OFF_F32)[i] = f32[i];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t sbase = smem_addr(sm);
  // the swizzled operand tiles assume a 1024-byte aligned shared-memory window
  bool ok = (sbase & 1023u) == 0;
  ok = wait_parity(smem_addr(wbar), 0) && ok;  // weight images in place
  ok = !__syncthreads_or(!ok);
  const uint32_t bar_a = smem_addr(bar);
  const int q = warp & 3, part = warp >> 2;  // lane quarter, column quarter
  const int row = q * 32 + lane;                                // this thread's tile row in the epilogue
  const uint32_t tlane = tmem + ((uint32_t)(q * 32) << 16);     // TMEM address of the warp's lane quarter
  const long long rows = (long long)g.ncol * g.nlay;
  const long long ntile = (rows + M - 1) / M;
  constexpr int NCH = 2 * (NOH / 16);  // output chunks of 16 columns
  uint32_t phase = 0;
  // inputs of this thread's row of tile t (rows are layer-major: coalesced loads)
  auto fetch = [&](long long t) {
    gbmlp::RawLayer rw{};
    const long long r = t * M + tid;
    if (tid < M && t < ntile && r < rows) {
      long long icol;
      const int lay = row_layer(r, g.ncol, icol);
      rw = gbmlp::load_raw(g.play, g.plev, g.tlay, g.tlev, g.h2ovmr, g.o3vmr, g.co2vmr, g.ch4vmr, g.n2ovmr, g.ld,
                           icol, lay);
    }
    return rw;
  };
  // features of this thread's row of tile t from `raw`, standardised and
  // packed as bf16 pairs into xp (rows past the end get the means); the row's
  // flag (on the network or not) is stored here
  gbmlp::RawLayer raw;
  uint32_t xp[8];
  auto features = [&](long long t) {
    if (tid >= M) return;
    const long long r = t * M + tid;
    float f[GB_MLP_NF];
    if (r < rows) {
      long long icol;
      const int lay = row_layer(r, g.ncol, icol);
      gbmlp::raw_features(raw, grav, avogad, f);
      flag[icol * g.nlay + lay] = gbmlp::in_range(f, nm) ? 1 : 0;
    } else {
#pragma unroll
      for (int i = 0; i < GB_MLP_NF; ++i) f[i] = nm.in_mu[i];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int j0 = 2 * i, j1 = 2 * i + 1;
      const float x0 = j0 < GB_MLP_NF ? (f[j0] - nm.in_mu[j0]) / nm.in_sd[j0] : 0.0f;
      const float x1 = j1 < GB_MLP_NF ? (f[j1] - nm.in_mu[j1]) / nm.in_sd[j1] : 0.0f;
      xp[i] = gbmlp::pack_bf16(x0, x1);
    }
  };
  // The first tile's features before the loop; every later tile's are formed
  // (and its inputs for the tile after it loaded) while the output layer's
  // MMAs of the tile before it run.
  raw = fetch(blockIdx.x);
  features(blockIdx.x);
  raw = fetch(blockIdx.x + gridDim.x);
  // A wait that runs out leaves `ok` false in its warp; every block-wide
  // barrier below is also the vote that ends the kernel in all threads.
  for (long long tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const long long r0 = tile * M;
    if (__syncthreads_or(!ok)) {  // and the previous tile's output staging (input tile) is done
      ok = false;
      break;
    }
    if (tid < M) {
      char* xb = sm + OFF_X;
      *reinterpret_cast<uint4*>(xb + sw128(M, tid, 0)) = make_uint4(xp[0], xp[1], xp[2], xp[3]);
      *reinterpret_cast<uint4*>(xb + sw128(M, tid, 8)) = make_uint4(xp[4], xp[5], xp[6], xp[7]);
#pragma unroll
      for (int c = 2; c < 8; ++c) *reinterpret_cast<uint4*>(xb + sw128(M, tid, 8 * c)) = make_uint4(0, 0, 0, 0);
    }
    // ---- four layers
    for (int l = 0; l < 4; ++l) {
      fence_async_smem();
      fence_before();
      if (__syncthreads_or(!ok)) {
        ok = false;
        break;
      }
      fence_after();
      if (tid == 0) {
        if (l == 0) {
          for (int s = 0; s < KIN / 16; ++s)
            mma(tmem, sdesc(sbase + OFF_X + s * 32), sdesc(sbase + OFF_W1 + s * 32), idesc(M, H), s > 0);
        } else if (l < 3) {
          const int W = l == 1 ? OFF_W2 : OFF_W3;
          for (int s = 0; s < H / 16; ++s) {
            const int kb = s >> 2, ks = (s & 3) * 32;
            mma(tmem, sdesc(sbase + OFF_H + kb * M * 128 + ks), sdesc(sbase + W + kb * H * 128 + ks), idesc(M, H), s > 0);
          }
        } else {
          for (int hh = 0; hh < 2; ++hh)
            for (int s = 0; s < H / 16; ++s) {
              const int kb = s >> 2, ks = (s & 3) * 32;
              mma(tmem + hh * 256, sdesc(sbase + OFF_H + kb * M * 128 + ks),
                  sdesc(sbase + OFF_W4 + kb * NO * 128 + hh * NOH * 128 + ks), idesc(M, NOH), s > 0);
            }
        }
        commit(bar_a);
      }
      if (l == 3) {
        features(tile + gridDim.x);
        raw = fetch(tile + 2 * (long long)gridDim.x);
      }
      ok = wait_parity(bar_a, phase);
      phase ^= 1u;
      fence_after();
      // warp-uniform, since the tensor-memory loads below are .sync.aligned;
      // a warp whose wait ran out skips the epilogue and the next vote ends the kernel
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) continue;
      if (l < 3) {
        hidden_epilogue(tlane + part * 32, row, part * 32, l == 0 ? b1 : (l == 1 ? b2 : b3), sm + OFF_H);
      } else {
        const long long r = r0 + row;
        const bool live = r < rows;
        long long o = 0;
        if (live) {
          long long icol;
          const int lay = row_layer(r, g.ncol, icol);
          o = (icol * g.nlay + lay) * GB_NGPT_MLP;
        }
        // 18 chunks of 16 outputs (two halves of 144); warp quarter `part` takes chunks part, part+4, ...,
        // two per wait for the tensor-memory loads.
        // A chunk goes through shared memory (the free input tile) as
        // binary16: each lane puts its row's 16 values there (four 8-byte
        // groups, group m of row r at slot m ^ ((r >> 2) & 3), so that neither
        // the puts nor the gets conflict on banks), then every store writes 32
        // contiguous bytes (16 outputs) of eight rows instead of 8 bytes of 32.
        uint2* stg = reinterpret_cast<uint2*>(sm + OFF_X) + warp * (32 * 4);
        long long orow[4];
        bool lrow[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {  // the rows this lane stores for: k*8 + lane/4 of the warp's 32
          const int src = k * 8 + (lane >> 2);
          orow[k] = __shfl_sync(0xffffffffu, o, src);
          lrow[k] = __shfl_sync(0xffffffffu, live ? 1 : 0, src) != 0;
        }
        auto chunk_col = [](int c) { return (uint32_t)((c / (NOH / 16)) * 256 + (c % (NOH / 16)) * 16); };
        auto out_chunk = [&](int c, const uint32_t* rv) {
          const int hh = c / (NOH / 16), c16 = c % (NOH / 16);
          const int j0 = hh * NOH + c16 * 16;  // output index of rv[0]
          const float4* sc = reinterpret_cast<const float4*>(oscale + j0);
          const float4* sh = reinterpret_cast<const float4*>(oshift + j0);
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            const float4 a = sc[m], b = sh[m];
            float y0 = fmaf(__uint_as_float(rv[4 * m]), a.x, b.x), y1 = fmaf(__uint_as_float(rv[4 * m + 1]), a.y, b.y);
            float y2 = fmaf(__uint_as_float(rv[4 * m + 2]), a.z, b.z), y3 = fmaf(__uint_as_float(rv[4 * m + 3]), a.w, b.w);
            if (j0 + 4 * m < GB_NGPT_MLP) {  // groups of four never straddle 140
              y0 = fminf(ex2(y0), GB_MLP_HALF_MAX), y1 = fminf(ex2(y1), GB_MLP_HALF_MAX);
              y2 = fminf(ex2(y2), GB_MLP_HALF_MAX), y3 = fminf(ex2(y3), GB_MLP_HALF_MAX);
            }
            const __half2 h01 = __floats2half2_rn(y0, y1), h23 = __floats2half2_rn(y2, y3);
            stg[lane * 4 + (m ^ ((lane >> 2) & 3))] =
                make_uint2(*reinterpret_cast<const uint32_t*>(&h01), *reinterpret_cast<const uint32_t*>(&h23));
          }
          __syncwarp();
          const int q4 = lane & 3, rr = lane >> 2;
          const int j = j0 + 4 * q4;  // first output index of this lane's four
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int r8 = k * 8 + rr;
            const uint2 val = stg[r8 * 4 + (q4 ^ ((r8 >> 2) & 3))];
            if (!lrow[k]) continue;
            if (j + 3 < GB_NGPT_MLP) {
              *reinterpret_cast<uint2*>(out_tau + orow[k] + j) = val;
            } else if (j >= GB_NGPT_MLP && j + 3 < GB_MLP_NOUT) {
              *reinterpret_cast<uint2*>(out_frac + orow[k] + j - GB_NGPT_MLP) = val;
            }  // four-output groups never straddle 140 or 280 (both multiples of 4)
          }
          __syncwarp();
        };
#pragma unroll 1
        for (int c = part; c < NCH; c += 8) {
          uint32_t ra[16], rb[16];
          ld16_async(tlane + chunk_col(c), ra);
          if (c + 4 < NCH) {  // warp-uniform
            ld16_async(tlane + chunk_col(c + 4), rb);
            wait_ld32(ra, rb);
            out_chunk(c, ra);
            out_chunk(c + 4, rb);
          } else {
            wait_ld16(ra);
            out_chunk(c, ra);
          }
        }
      }
    }
  }
  fence_before();
  const bool failed = __syncthreads_or(!ok);  // a warp's wait in the last layer can have run out
  fence_after();
  if (failed && tid == 0) atomicMax(err, GB_COL_TCWAIT);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// K-major 128-byte-swizzled weight images (bf16) from the [in][out] parameter
// blob, and the fp32 vectors (biases, output scaling) the kernel stages
__global__ void images_kernel(const bf16* __restrict__ p16, const float* __restrict__ p32, GbMlpNorm nm,
                              char* __restrict__ img, float* __restrict__ f32) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  // W1: rows n (128), k < 64 (features beyond 16 are zero)
  for (int i = tid; i < H * KIN; i += nth) {
    const int n = i / KIN, k = i % KIN;
    const bf16 v = k < GB_MLP_KIN ? p16[GB_MLP_OFF_W1 + k * H + n] : __float2bfloat16_rn(0.0f);
    *reinterpret_cast<bf16*>(img + OFF_W1 + sw128(H, n, k)) = v;
  }
  for (int i = tid; i < H * H; i += nth) {
    const int n = i / H, k = i % H;
    *reinterpret_cast<bf16*>(img + OFF_W2 + sw128(H, n, k)) = p16[GB_MLP_OFF_W2 + k * H + n];
    *reinterpret_cast<bf16*>(img + OFF_W3 + sw128(H, n, k)) = p16[GB_MLP_OFF_W3 + k * H + n];
  }
  for (int i = tid; i < NO * H; i += nth) {
    const int n = i / H, k = i % H;
    *reinterpret_cast<bf16*>(img + OFF_W4 + sw128(NO, n, k)) = p16[GB_MLP_OFF_W4 + k * NO + n];
  }
  for (int i = tid; i < H; i += nth) {
    f32[i] = p32[GB_MLP_OFF_B1 + i];
    f32[H + i] = p32[GB_MLP_OFF_B2 + i];
    f32[2 * H + i] = p32[GB_MLP_OFF_B3 + i];
  }
  // output i = (acc + b4) * sd + mu = acc * scale + shift, times log2(e) for
  // the log-taug outputs so that the kernel takes 2^x
  for (int i = tid; i < NO; i += nth) {
    const double c = i < GB_NGPT_MLP ? 1.4426950408889634 : 1.0;
    const double sd = nm.out_sd[i];
    f32[3 * H + i] = (float)(sd * c);
    f32[3 * H + NO + i] = (float)(((double)p32[GB_MLP_OFF_B4 + i] * sd + (double)nm.out_mu[i]) * c);
  }
}

}  // namespace gbtc

size_t gb_mlp_tc_image_bytes() { return (size_t)gbtc::IMG_BYTES + (size_t)gbtc::NF32 * 4; }

cudaError_t gb_mlp_tc_images(const __nv_bfloat16* p16, const float* p32, const GbMlpNorm& nm, void* d_img,
                             cudaStream_t st) {
  char* img = static_cast<char*>(d_img);
  gbtc::images_kernel<<<256, 256, 0, st>>>(p16, p32, nm, img, reinterpret_cast<float*>(img + gbtc::IMG_BYTES));
  return cudaGetLastError();
}

cudaError_t gb_mlp_infer_tc(const GbMlpGridIn& g, const GbMlpNorm& nm, const void* d_img, double grav,
                            double avogad, __half* d_tau, __half* d_frac, unsigned char* d_flag, int* d_err, int nsm,
                            cudaStream_t st) {
  const long long rows = (long long)g.ncol * g.nlay;
  if (rows == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(gbtc::infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       gbtc::SMEM_BYTES);
  if (e != cudaSuccess) return e;
  const long long tiles = (rows + gbtc::M - 1) / gbtc::M;
  const int blocks = (int)(tiles < nsm ? tiles : nsm);
  const char* img = static_cast<const char*>(d_img);
  gbtc::infer_tc_kernel<<<blocks, gbtc::NT, gbtc::SMEM_BYTES, st>>>(
      g, nm, reinterpret_cast<const uint4*>(img), reinterpret_cast<const float*>(img + gbtc::IMG_BYTES), grav, avogad,
      d_tau, d_frac, d_flag, d_err);
  return cudaGetLastError();
}
