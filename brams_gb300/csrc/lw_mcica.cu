// McICA sub-column generator on the GPU (mcica_subcol_gen_lw.f90:183-703,
// mcica_random_numbers.f90:77-306).
//
// The reference draws every random number from one Mersenne-twister (irng=1)
// or KISS (irng=0) sequence in a fixed loop order and marks sub-column isub
// of layer ilev cloudy when CDF >= 1 - cldf (:650).  The GPU reproduces the
// draws bit for bit:
//   * draw generation -- one thread per column for per-column seeds (the
//     reference called with ncol = 1 and seed = base + column), or one block
//     stepping the single sequence 624 words at a time for the reference's
//     all-columns call (draw order isub, column, layer);
//   * CDF construction and the cloudy test in double precision, one thread
//     per (column, sub-column), layers in order (max-random and exponential
//     overlap carry CDF from one layer to the next).
// Draws are kept as doubles exactly as getRandomReal/kissvec return them.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/gb_rrtmg_lw.h"
#include "lw_common.h"
#include "lw_mcica.h"
#include "lw_mt.cuh"

namespace gbm {

// ---------------------------------------------------------------- Mersenne twister
using gbmt::temper;
using gbmt::real;
__device__ __forceinline__ uint32_t mt_temper(uint32_t y) { return gbmt::temper(y); }
__device__ __forceinline__ uint32_t mt_twist(uint32_t u, uint32_t v) { return gbmt::twist(u, v); }
__device__ __forceinline__ double mt_real(uint32_t u) { return gbmt::real(u); }

// Full-state generator for longer per-column sequences.
struct MtState {
  uint32_t s[624];
  int cur;
};
__device__ void mt_init(MtState& m, uint32_t seed) {
  m.s[0] = seed;
  for (int i = 1; i < 624; ++i) m.s[i] = 1812433253u * (m.s[i - 1] ^ (m.s[i - 1] >> 30)) + (uint32_t)i;
  m.cur = 624;
}
__device__ uint32_t mt_next(MtState& m) {
  if (m.cur >= 624) {
    for (int k = 0; k < 227; ++k) m.s[k] = m.s[k + 397] ^ mt_twist(m.s[k], m.s[k + 1]);
    for (int k = 227; k < 623; ++k) m.s[k] = m.s[k - 227] ^ mt_twist(m.s[k], m.s[k + 1]);
    m.s[623] = m.s[396] ^ mt_twist(m.s[623], m.s[0]);
    m.cur = 0;
  }
  return mt_temper(m.s[m.cur++]);
}

// per-column seeds: column c uses seed0 + c; draws[c * ndraw + k]
__global__ void mt_percol_kernel(int ncol, int seed0, int ndraw, double* __restrict__ draws) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  double* out = draws + (long long)c * ndraw;
  uint32_t seed = (uint32_t)(seed0 + c);
  if (ndraw <= 226) {
    uint32_t lo[227];
    gbmt::first_reals(seed, ndraw, lo, out, 1);
    return;
  }
  MtState m;
  mt_init(m, seed);
  for (int k = 0; k < ndraw; ++k) out[k] = mt_real(mt_next(m));
}

// one sequence for the whole call: a single block keeps the 624-word state in
// shared memory and produces it one twist (624 draws) at a time.
__global__ void __launch_bounds__(256) mt_stream_kernel(uint32_t seed, long long ndraw, double* __restrict__ draws) {
  __shared__ uint32_t st[624];
  __shared__ uint32_t nw[624];
  if (threadIdx.x == 0) {
    uint32_t s = seed;
    st[0] = s;
    for (int i = 1; i < 624; ++i) {
      s = 1812433253u * (s ^ (s >> 30)) + (uint32_t)i;
      st[i] = s;
    }
  }
  __syncthreads();
  for (long long base = 0; base < ndraw; base += 624) {
    // nextState (:127-139): words 0..226 from old words, 227..622 from new 0..395, 623 from new 396 and new 0
    for (int k = threadIdx.x; k < 227; k += blockDim.x) nw[k] = st[k + 397] ^ mt_twist(st[k], st[k + 1]);
    __syncthreads();
    for (int k = 227 + threadIdx.x; k < 454; k += blockDim.x) nw[k] = nw[k - 227] ^ mt_twist(st[k], st[k + 1]);
    __syncthreads();
    for (int k = 454 + threadIdx.x; k < 623; k += blockDim.x) nw[k] = nw[k - 227] ^ mt_twist(st[k], st[k + 1]);
    __syncthreads();
    if (threadIdx.x == 0) nw[623] = nw[396] ^ mt_twist(st[623], nw[0]);
    __syncthreads();
    for (int k = threadIdx.x; k < 624; k += blockDim.x) {
      st[k] = nw[k];
      long long d = base + k;
      if (d < ndraw) draws[d] = mt_real(mt_temper(nw[k]));
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- KISS (irng = 0)
struct Kiss {
  uint32_t s1, s2, s3, s4;
  __device__ double next() {
    s1 = 69069u * s1 + 1327217885u;
    uint32_t k = s2;
    k ^= k << 13;
    k ^= k >> 17;
    k ^= k << 5;
    s2 = k;
    s3 = 18000u * (s3 & 65535u) + (s3 >> 16);
    s4 = 30903u * (s4 & 65535u) + (s4 >> 16);
    int32_t kiss = (int32_t)(s1 + s2 + (s3 << 16) + s4);
    return (double)kiss * 2.328306e-10 + 0.5;
  }
};

// kissvec seeds from the fractional part of the bottom four layer pressures
// (:460-474), warmed up changeSeed times; then the column's own sequence.
// skip_per_draw > 0 reproduces icld 4/5, where every kissvec call of the
// reference advances all columns although only column c's value is kept.
__global__ void kiss_percol_kernel(int ncol, long long ld, const double* __restrict__ play, int change_seed,
                                   int seed_step, int ndraw, int ncol_call, int nsub, int* __restrict__ err,
                                   double* __restrict__ draws) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  double p[4];
  for (int l = 0; l < 4; ++l) p[l] = play[c + ld * l] * 1.e2;
  if (p[0] < p[1]) {
    // the reference stops here (status 8); the column's draws are set to 0 so
    // that its sub-columns are the same on every call, not the previous
    // contents of the draw buffer
    atomicMax(err, 8);
    for (int d = 0; d < ndraw; ++d) draws[(long long)c * ndraw + d] = 0.0;
    return;
  }
  Kiss k;
  auto sd = [](double x) { return (uint32_t)(int32_t)((x - (double)(long long)x) * 1000000000.0); };
  k.s1 = sd(p[0]); k.s2 = sd(p[1]); k.s3 = sd(p[2]); k.s4 = sd(p[3]);
  const int warm = change_seed + seed_step * c;
  for (int i = 0; i < warm; ++i) k.next();
  double* out = draws + (long long)c * ndraw;
  if (ncol_call <= 1) {
    for (int d = 0; d < ndraw; ++d) out[d] = k.next();
  } else {
    // icld 4/5 in one call over ncol_call columns: pairs of draws per
    // (isub, column, layer), each advancing every column; keep column c's
    int nlay_pairs = ndraw / 2 / nsub;  // = nlay
    int col_in_call = c % ncol_call;
    int d = 0;
    for (int isub = 0; isub < nsub; ++isub)
      for (int i = 0; i < ncol_call; ++i)
        for (int l = 0; l < nlay_pairs; ++l) {
          double a = k.next(), b = k.next();
          if (i == col_in_call) {
            out[d++] = a;
            out[d++] = b;
          }
        }
  }
}

// ---------------------------------------------------------------- CDF + outputs
// One block per column, one thread per sub-column.  `draw(isub, ilev, which)`
// locates the draw the reference would use for that cell.
__global__ void mcica_fill_kernel(McicaArgs a, const double* __restrict__ draws) {
  const int c = blockIdx.x;
  const int isub = threadIdx.x;
  if (c >= a.ncol || isub >= a.nsub) return;
  const int nlay = a.nlay;
  const long long ld = a.ld;
  auto D = [&](int ilev, int which) -> double {
    long long idx;
    if (a.mode == MCICA_STREAM_MT) {
      // one sequence over the call: loop order isub, column, layer (:476-645)
      long long ncol = a.ncol;
      if (a.icld == 3) idx = (long long)isub * ncol + c;
      else if (a.icld <= 2) idx = ((long long)isub * ncol + c) * nlay + ilev;
      else idx = 2 * (((long long)isub * ncol + c) * nlay + ilev) + which;
      return draws[idx];
    }
    // per-column sequences (MT with per-column seeds, or KISS)
    long long base = (long long)c * a.ndraw_per_col;
    if (a.icld == 3) idx = isub;
    else if (a.icld <= 2) idx = (long long)isub * nlay + ilev;
    else idx = 2 * ((long long)isub * nlay + ilev) + which;
    if (a.mode == MCICA_PERCOL_KISS && a.icld <= 2) idx = (long long)isub * nlay + ilev;
    return draws[base + idx];
  };
  auto cldf_at = [&](int ilev) {
    double v = a.cldfrac[c + ld * ilev];
    return v < 1.0e-20 ? 0.0 : v;
  };
  double cdf_prev = 0.0;
  for (int ilev = 0; ilev < nlay; ++ilev) {
    double cdf;
    if (a.icld == 3) {
      cdf = D(0, 0);
    } else if (a.icld <= 2) {
      cdf = D(ilev, 0);
      if (a.icld == 2 && ilev > 0) {
        double cp = cldf_at(ilev - 1);
        cdf = (cdf_prev > 1.0 - cp) ? cdf_prev : cdf * (1.0 - cp);  // :528-537
      }
    } else {
      cdf = D(ilev, 0);
      double cdf2 = D(ilev, 1);
      if (ilev > 0 && cdf2 < a.alpha[c + ld * ilev]) cdf = cdf_prev;  // :626-630, 639-643
    }
    cdf_prev = cdf;
    bool cloudy = cdf >= 1.0 - cldf_at(ilev);
    long long o = (long long)isub + a.nsub * ((long long)c + ld * ilev);
    long long oc = c + ld * ilev;
    // the band of the sub-column's optical properties (mcica_subcol_gen_sw.f90:
    // n = ngb(isubcol) - ngbm; the longwave one uses ngb itself)
    const long long ob = (a.ngb[isub] - a.band0 - 1) + (long long)a.nbnd * (c + ld * (long long)ilev);
    if (cloudy) {
      a.cldfmcl[o] = 1.0;
      a.clwpmcl[o] = a.clwp[oc];
      a.ciwpmcl[o] = a.ciwp[oc];
      a.taucmcl[o] = a.tauc[ob];
      if (a.ssacmcl) {
        a.ssacmcl[o] = a.ssac[ob];
        a.asmcmcl[o] = a.asmc[ob];
        a.fsfcmcl[o] = a.fsfc[ob];
      }
    } else {
      a.cldfmcl[o] = 0.0;
      a.clwpmcl[o] = 0.0;
      a.ciwpmcl[o] = 0.0;
      a.taucmcl[o] = 0.0;
      if (a.ssacmcl) {
        a.ssacmcl[o] = 1.0;
        a.asmcmcl[o] = 0.0;
        a.fsfcmcl[o] = 0.0;
      }
    }
  }
  // reicmcl / relqmcl copies (:264-265)
  if (isub == 0) {
    for (int ilev = 0; ilev < nlay; ++ilev) {
      long long oc = c + ld * ilev;
      a.reicmcl[oc] = a.rei[oc];
      a.relqmcl[oc] = a.rel[oc];
    }
  }
}

}  // namespace gbm

cudaError_t gb_mcica_launch(const McicaArgs& a, double* d_draws, int* d_err, cudaStream_t stream,
                            bool seed_per_column) {
  if (a.ncol <= 0) return cudaSuccess;
  const int per = a.icld == 3 ? 1 : (a.icld <= 2 ? a.nlay : 2 * a.nlay);
  const int ndraw = a.nsub * per;
  if (a.mode == MCICA_PERCOL_MT) {
    gbm::mt_percol_kernel<<<(a.ncol + 127) / 128, 128, 0, stream>>>(a.ncol, a.seed, ndraw, d_draws);
  } else if (a.mode == MCICA_STREAM_MT) {
    gbm::mt_stream_kernel<<<1, 256, 0, stream>>>((uint32_t)a.seed, (long long)ndraw * a.ncol, d_draws);
  } else {
    gbm::kiss_percol_kernel<<<(a.ncol + 127) / 128, 128, 0, stream>>>(
        a.ncol, a.ld, a.play, a.seed, seed_per_column ? 1 : 0, ndraw, a.icld >= 4 ? a.ncol_call : 1, a.nsub, d_err,
        d_draws);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  McicaArgs b = a;
  b.ndraw_per_col = ndraw;
  gbm::mcica_fill_kernel<<<a.ncol, 160, 0, stream>>>(b, d_draws);
  return cudaGetLastError();
}

cudaError_t gb_mcica_percol_mt(int ncol, unsigned seed0, int ndraw, double* d_draws, cudaStream_t stream) {
  if (ncol <= 0) return cudaSuccess;
  gbm::mt_percol_kernel<<<(ncol + 127) / 128, 128, 0, stream>>>(ncol, (int)seed0, ndraw, d_draws);
  return cudaGetLastError();
}

size_t gb_mcica_draw_count(int ncol, int nlay, int icld, int nsub) {
  const int per = icld == 3 ? 1 : (icld <= 2 ? nlay : 2 * nlay);
  return (size_t)nsub * per * (size_t)ncol;
}

// ----------------------------------------------------------------------------
// Allocation-free McICA entry point.
//
// Some callers must not allocate device memory while a model runs: a host
// model whose device memory is owned by another runtime (an OpenACC or
// OpenMP-offload data region, or a pooled allocator that forbids allocations
// outside its pool), and time-stepping codes that cannot afford the implicit
// device-wide synchronisation of cudaMalloc/cudaFree in the middle of a step.
// gb_mcica_subcol_lw_noalloc serves them: its draw buffer is this fixed
// file-scope array, so a call allocates nothing.  Every GPU that loads the
// library holds the array until the process exits.
//
// Layout: the first 256 bytes hold the status word, the rest holds draws.
// All calls share the array and it keeps the previous call's contents: the
// status word is cleared at the start of every call, and every draw slot a
// call reads is written by that call first (a column whose KISS seeding
// fails gets zero draws and status 8).  Calls whose kernels overlap on
// the GPU (different streams without ordering, or several host threads)
// race on the array and must be serialised by the caller.
static __device__ __align__(256) double g_mcica_scratch[GB_MCICA_NOALLOC_STATUS_DOUBLES + GB_MCICA_NOALLOC_MAX_DRAWS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_mcica_scratch on the current device.  In host code the
// array's name stands for a host-side shadow, not a device address, so the
// address is queried once per device (with that device current) and cached.
cudaError_t scratch_on_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_mcica_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}
}  // namespace

extern "C" int gb_mcica_subcol_lw_noalloc(void* stream, int ncol, int nlay, int icld, int permuteseed, int* irng,
                                          const double* play, const double* cldfrac, const double* ciwp,
                                          const double* clwp, const double* rei, const double* rel,
                                          const double* tauc, const double* alpha, double* cldfmcl,
                                          double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl,
                                          double* taucmcl, int64_t ld, int seed_per_column, int* d_status) {
  if (!irng) return GB_LW_E_ARGS;
  if (icld == 0) return GB_LW_OK;
  if (icld < 0 || icld > 5) return GB_LW_E_ICLD;
  if (ncol < 0 || nlay < 1 || ld < ncol) return GB_LW_E_ARGS;
  if (*irng != 0) *irng = 1;
  if (icld >= 4 && !alpha) return GB_LW_E_ARGS;
  if (*irng == 0 && nlay < 4) return GB_LW_E_ARGS;
  if (!play || !cldfrac || !ciwp || !clwp || !rei || !rel || !tauc || !cldfmcl || !ciwpmcl || !clwpmcl ||
      !reicmcl || !relqmcl || !taucmcl)
    return GB_LW_E_ARGS;
  if (ncol == 0) return GB_LW_OK;
  if (gb_mcica_draw_count(ncol, nlay, icld) > (size_t)GB_MCICA_NOALLOC_MAX_DRAWS) return GB_LW_E_SCRATCH;
  double* scratch = nullptr;
  if (scratch_on_current_device(&scratch) != cudaSuccess) return GB_LW_E_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  int* status = reinterpret_cast<int*>(scratch);
  if (cudaMemsetAsync(status, 0, sizeof(int), s) != cudaSuccess) return GB_LW_E_CUDA;
  McicaArgs a{};
  a.mode = *irng == 0 ? MCICA_PERCOL_KISS : (seed_per_column ? MCICA_PERCOL_MT : MCICA_STREAM_MT);
  a.ncol = ncol;
  a.nlay = nlay;
  a.icld = icld;
  a.seed = permuteseed;
  a.ncol_call = seed_per_column ? 1 : ncol;
  a.ld = ld;
  a.play = play; a.cldfrac = cldfrac; a.ciwp = ciwp; a.clwp = clwp; a.rei = rei; a.rel = rel;
  a.tauc = tauc; a.alpha = alpha;
  a.cldfmcl = cldfmcl; a.ciwpmcl = ciwpmcl; a.clwpmcl = clwpmcl; a.taucmcl = taucmcl;
  a.reicmcl = reicmcl; a.relqmcl = relqmcl;
  // g-point -> band map (rrtmg_lw_init.f90:359-374): band b owns ng(b) consecutive g-points
  static const int ng_list[16] = GB_NG_LIST;
  for (int b = 0, g = 0; b < 16; ++b)
    for (int k = 0; k < ng_list[b]; ++k) a.ngb[g++] = b + 1;
  if (gb_mcica_launch(a, scratch + GB_MCICA_NOALLOC_STATUS_DOUBLES, status, s, seed_per_column != 0) != cudaSuccess)
    return GB_LW_E_CUDA;
  if (d_status && cudaMemcpyAsync(d_status, status, sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return GB_LW_E_CUDA;
  return GB_LW_OK;
}
