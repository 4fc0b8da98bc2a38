// Learned stand-in for taumol: a small MLP from per-layer state to the 140
// g-point gas optical depths and Planck fractions (device-side pieces shared
// by the training kernels, the inference kernel and the column kernel).
//
// Network: 9 features -> 128 -> 128 -> 128 -> 280, SiLU between layers.
// Weights and activations are bf16, products accumulate in fp32 on the
// tensor cores (mma.sync m16n8k16).  Outputs 0..139 are standardised
// log(taug), 140..279 standardised Planck fractions (g order of rrtmg).
//
// Features of layer (icol, lay), computed from the rrtmg_lw inputs exactly as
// inatm/setcoef form them (rrtmg_lw_rad.f90:807-867, rrtmg_lw_setcoef.f90:349-362):
//   0 log(pavel)        1 tavel            2 log(colh2o)      3 log(colo3)
//   4 log(colco2)       5 log(colch4)      6 log(coln2o)      7 log(pz(l-1) - pz(l))
//   8 tz(l-1)  (temperature of the layer's lower boundary level)
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#define GB_MLP_NF 9
#define GB_MLP_RANGE_MARGIN 0.02f  // validity range = training range widened by 2% of its width per side
#define GB_MLP_KIN 16     // input width padded to one mma k-step
#define GB_MLP_H 128
#define GB_MLP_NOUT 280
#define GB_MLP_NOUTP 288  // padded to a multiple of 32

// Parameter blob (fp32 master copy and bf16 working copy share the order).
// Weight matrices are row-major [in][out].
#define GB_MLP_OFF_W1 0
#define GB_MLP_OFF_B1 (GB_MLP_OFF_W1 + GB_MLP_KIN * GB_MLP_H)
#define GB_MLP_OFF_W2 (GB_MLP_OFF_B1 + GB_MLP_H)
#define GB_MLP_OFF_B2 (GB_MLP_OFF_W2 + GB_MLP_H * GB_MLP_H)
#define GB_MLP_OFF_W3 (GB_MLP_OFF_B2 + GB_MLP_H)
#define GB_MLP_OFF_B3 (GB_MLP_OFF_W3 + GB_MLP_H * GB_MLP_H)
#define GB_MLP_OFF_W4 (GB_MLP_OFF_B3 + GB_MLP_H)
#define GB_MLP_OFF_B4 (GB_MLP_OFF_W4 + GB_MLP_H * GB_MLP_NOUTP)
#define GB_MLP_NPARAM (GB_MLP_OFF_B4 + GB_MLP_NOUTP)

// Normalisation and validity range, fitted on the training set.
struct GbMlpNorm {
  float in_mu[GB_MLP_KIN], in_sd[GB_MLP_KIN];  // feature standardisation (padding: 0, 1)
  float in_lo[GB_MLP_NF], in_hi[GB_MLP_NF];    // training range; outside -> plain taumol
  float out_mu[GB_MLP_NOUTP], out_sd[GB_MLP_NOUTP];
};

namespace gbmlp {

// The rrtmg_lw inputs one layer's features are made of.
struct RawLayer {
  double play, plev0, plev1, tlay, tlev, h2o, o3, co2, ch4, n2o;
};

// Loads of one layer's inputs (Fortran layout, leading dimension ld); issued
// early by the inference kernel so that their latency hides behind the MMAs.
__device__ __forceinline__ RawLayer load_raw(const double* __restrict__ play, const double* __restrict__ plev,
                                            const double* __restrict__ tlay, const double* __restrict__ tlev,
                                            const double* __restrict__ h2o, const double* __restrict__ o3,
                                            const double* __restrict__ co2, const double* __restrict__ ch4,
                                            const double* __restrict__ n2o, long long ld, long long icol, int lay) {
  const long long o = icol + ld * lay;
  RawLayer r;
  r.play = __ldg(play + o);
  r.plev0 = __ldg(plev + o);
  r.plev1 = __ldg(plev + o + ld);
  r.tlay = __ldg(tlay + o);
  r.tlev = __ldg(tlev + o);
  r.h2o = __ldg(h2o + o);
  r.o3 = __ldg(o3 + o);
  r.co2 = __ldg(co2 + o);
  r.ch4 = __ldg(ch4 + o);
  r.n2o = __ldg(n2o + o);
  return r;
}

// The nine raw features of a layer, formed as inatm/setcoef form the column
// amounts (coldry, 1e-20 scaling, 1e-32 floors for absent gases).
__device__ __forceinline__ void raw_features(const RawLayer& r, double grav, double avogad, float* f) {
  const float pavel = (float)r.play;
  const float tavel = (float)r.tlay;
  const double dpz = r.plev0 - r.plev1;
  const float w1 = (float)r.h2o;
  const float amm = (1.0f - w1) * 28.9660f + w1 * 18.0160f;
  const float coldry = (float)dpz * 1.e3f * (float)avogad / (1.e2f * (float)grav * amm * (1.0f + w1));
  float colh2o = 1.e-20f * coldry * w1;
  float colo3 = 1.e-20f * coldry * (float)r.o3;
  float colco2 = 1.e-20f * coldry * (float)r.co2;
  float colch4 = 1.e-20f * coldry * (float)r.ch4;
  float coln2o = 1.e-20f * coldry * (float)r.n2o;
  const float floor_ = 1.e-32f * coldry;
  if (colo3 == 0.0f) colo3 = floor_;
  if (colco2 == 0.0f) colco2 = floor_;
  if (colch4 == 0.0f) colch4 = floor_;
  if (coln2o == 0.0f) coln2o = floor_;
  f[0] = __logf(pavel);
  f[1] = tavel;
  f[2] = __logf(fmaxf(colh2o, 1.e-30f));
  f[3] = __logf(fmaxf(colo3, 1.e-30f));
  f[4] = __logf(fmaxf(colco2, 1.e-30f));
  f[5] = __logf(fmaxf(colch4, 1.e-30f));
  f[6] = __logf(fmaxf(coln2o, 1.e-30f));
  f[7] = __logf(fmaxf((float)dpz, 1.e-30f));
  f[8] = (float)r.tlev;
}

// Raw features of one layer from the rrtmg_lw inputs.
__device__ __forceinline__ void layer_features(const double* __restrict__ play, const double* __restrict__ plev,
                                               const double* __restrict__ tlay, const double* __restrict__ tlev,
                                               const double* __restrict__ h2o, const double* __restrict__ o3,
                                               const double* __restrict__ co2, const double* __restrict__ ch4,
                                               const double* __restrict__ n2o, long long ld, long long icol,
                                               int lay, double grav, double avogad, float* f) {
  raw_features(load_raw(play, plev, tlay, tlev, h2o, o3, co2, ch4, n2o, ld, icol, lay), grav, avogad, f);
}

__device__ __forceinline__ bool in_range(const float* f, const GbMlpNorm& n) {
  bool ok = true;
#pragma unroll
  for (int i = 0; i < GB_MLP_NF; ++i) ok = ok && f[i] >= n.in_lo[i] && f[i] <= n.in_hi[i];
  return ok;
}

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

// D += A(16x16, bf16) * B(16x8, bf16), fp32 accumulators
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

}  // namespace gbmlp
