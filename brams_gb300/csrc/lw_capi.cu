// C ABI of the GB300 RRTMG_LW solver (declared in include/gb_rrtmg_lw.h).
//
// gb_rrtmg_lw streams host columns through the device in chunks: for chunk k
// the inputs are copied (cudaMemcpy2DAsync, one copy per argument array,
// pitch = the caller's leading dimension) on stream k%2, the column kernel
// runs on the same stream and the outputs are copied back, so copies of one
// chunk overlap the kernel of the other.  gb_rrtmg_lw_device runs the kernel
// directly on caller-owned device arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gb_rrtmg_lw.h"
#include "lw_common.h"
#include "lw_mcica.h"
#include "lw_solver.h"
#include "lw_tables.h"
#include "lw_context.h"

#include <dlfcn.h>

static_assert(sizeof(gb_lw_grid) == 368, "gb_lw_grid layout is part of the ABI (Python mirror: GridDesc)");

struct gb_lw_graph {
  gb_lw_context* ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  float* gas = nullptr;      // taumol hand-over planes
  double* draws = nullptr;  // McICA draws of the fused-cloud grids
  long long* fall = nullptr;  // hand-over list of a batch with learned gas optics
  unsigned* nfall = nullptr;
};

int gb_ctx_fail(gb_lw_context* c, cudaError_t e, const char* where) {
  if (c) c->last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return GB_LW_E_CUDA;
}

namespace {

int cuda_fail(gb_lw_context* c, cudaError_t e, const char* where) { return gb_ctx_fail(c, e, where); }
#define CK(call)                                      \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return cuda_fail(ctx, _e, #call); \
  } while (0)

std::string default_table_dir() {
  Dl_info info;
  if (dladdr((void*)&default_table_dir, &info) && info.dli_fname) {
    std::string p = info.dli_fname;
    size_t s = p.find_last_of('/');
    std::string dir = s == std::string::npos ? "." : p.substr(0, s);
    // library lives in brams_gb300/_lib/, tables in brams_gb300/data/
    return dir + "/../data";
  }
  return "brams_gb300/data";
}

// inputs of one chunk, packed per array with leading dimension = chunk columns
struct InLayout {
  size_t play, plev, tlay, tlev, tsfc, gas[10], emis, reic, relq, tauaer, cldf, tauc, ciwp, clwp, total;
};
InLayout in_layout(int C, int nlay) {
  InLayout L;
  size_t o = 0;
  auto take = [&](size_t n) { size_t r = o; o += (n + 31) & ~size_t(31); return r; };
  L.play = take((size_t)C * nlay);
  L.plev = take((size_t)C * (nlay + 1));
  L.tlay = take((size_t)C * nlay);
  L.tlev = take((size_t)C * (nlay + 1));
  L.tsfc = take(C);
  for (int k = 0; k < 10; ++k) L.gas[k] = take((size_t)C * nlay);
  L.emis = take((size_t)C * 16);
  L.reic = take((size_t)C * nlay);
  L.relq = take((size_t)C * nlay);
  L.tauaer = take((size_t)C * nlay * 16);
  L.cldf = take((size_t)GB_NGPT * C * nlay);
  L.tauc = take((size_t)GB_NGPT * C * nlay);
  L.ciwp = take((size_t)GB_NGPT * C * nlay);
  L.clwp = take((size_t)GB_NGPT * C * nlay);
  L.total = o;
  return L;
}
struct OutLayout {
  size_t uflx, dflx, uflxc, dflxc, duflx, duflxc, hr, hrc, status, total;
};
OutLayout out_layout(int C, int nlay) {
  OutLayout L;
  size_t o = 0;
  auto take = [&](size_t n) { size_t r = o; o += (n + 31) & ~size_t(31); return r; };
  L.uflx = take((size_t)C * (nlay + 1));
  L.dflx = take((size_t)C * (nlay + 1));
  L.uflxc = take((size_t)C * (nlay + 1));
  L.dflxc = take((size_t)C * (nlay + 1));
  L.duflx = take((size_t)C * (nlay + 1));
  L.duflxc = take((size_t)C * (nlay + 1));
  L.hr = take((size_t)C * nlay);
  L.hrc = take((size_t)C * nlay);
  L.status = take(C);  // ints stored in double slots
  L.total = o;
  return L;
}

int ensure_chunks(gb_lw_context* ctx, int C, int nlay) {
  if (ctx->chunk_cols >= C && ctx->chunk_nlay == nlay && ctx->bufs[0].in) return 0;
  for (auto& b : ctx->bufs) {
    cudaFree(b.in);
    cudaFree(b.out);
    b.in = b.out = nullptr;
  }
  InLayout li = in_layout(C, nlay);
  OutLayout lo = out_layout(C, nlay);
  for (auto& b : ctx->bufs) {
    if (cudaMalloc(&b.in, li.total * 8) != cudaSuccess || cudaMalloc(&b.out, lo.total * 8) != cudaSuccess) {
      ctx->last_error = "device allocation of chunk buffers failed";
      cudaGetLastError();
      return GB_LW_E_NOMEM;
    }
    b.in_elems = li.total;
    b.out_elems = lo.total;
  }
  ctx->chunk_cols = C;
  ctx->chunk_nlay = nlay;
  return 0;
}

// strided 2-D copy of `rows` rows of `width` doubles with source/destination pitches (in doubles)
cudaError_t copy2d(double* dst, size_t dpitch, const double* src, size_t spitch, size_t width, size_t rows,
                   cudaMemcpyKind kind, cudaStream_t s) {
  if (width == 0 || rows == 0) return cudaSuccess;
  return cudaMemcpy2DAsync(dst, dpitch * 8, src, spitch * 8, width * 8, rows, kind, s);
}

// a taumol hand-over buffer of at least `bytes` (grown on demand)
int ensure_buffer(gb_lw_context* ctx, float** buf, size_t* have, size_t bytes) {
  if (*buf && *have >= bytes) return 0;
  cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  if (cudaMalloc(buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    *buf = nullptr;
    ctx->last_error = "device allocation of the gas-optics hand-over planes failed";
    return GB_LW_E_NOMEM;
  }
  *have = bytes;
  return 0;
}

// points a descriptor at a hand-over buffer of `bytes` (slots of nsmax layers)
void attach_gas(LwBatch& b, float* buf, size_t bytes) {
  b.gstride = (long long)b.nsmax * GB_NGPT;
  b.gslots = (long long)(bytes / (3 * sizeof(float) * (size_t)b.gstride));
  b.gtau = buf;
  b.gfrac = buf + (size_t)b.gslots * b.gstride;
  b.gcld = buf + (size_t)2 * b.gslots * b.gstride;
}

// hand-over bytes a batch of `ncols` columns at `nlay` layers is solved with
size_t gas_need(int nlay, long long ncols) { return gb_lw_gas_bytes(nlay, gb_lw_gas_slots(nlay, ncols)); }

bool flags_ok(int idrv, int inflglw, int iceflglw, int liqflglw) {
  return (idrv == 0 || idrv == 1) && inflglw >= 0 && inflglw <= 2 && iceflglw >= 0 && iceflglw <= 3 &&
         liqflglw >= 0 && liqflglw <= 1;
}

// Kind of a batch for the tuned-shape table: bit 0 fused-cloud grids, bit 1 learned gas optics.
int batch_kind(const LwBatch& b) {
  int k = 0;
  for (int i = 0; i < b.ngrid; ++i) {
    if (b.g[i].cloud_mode == LW_CLOUD_FUSED && b.g[i].icld >= 1) k |= GB_LW_KIND_FUSED;
    if (b.g[i].sur_flag) k |= GB_LW_KIND_LEARNED;
  }
  return k;
}

// Default shape: variant 0 at as many resident blocks as fit.  Batches with
// learned gas optics index the shapes of the transfer kernel on the
// network's outputs.
gb_lw_tuning default_tuning(gb_lw_context* ctx, int nlay, int kind) {
  gb_lw_tuning t{};
  const bool lean = kind & GB_LW_KIND_LEARNED;
  t.variant = 0;
  t.threads = gb_lw_variant(t.variant, lean).threads;
  t.min_blocks = gb_lw_variant(t.variant, lean).min_blocks;
  const int occ = std::max(1, gb_lw_slots(nlay, t.variant, lean) / std::max(1, ctx->num_sms));
  t.blocks_per_sm = std::min(occ, t.min_blocks);
  t.blocks = t.blocks_per_sm * ctx->num_sms;
  t.ms = 0.0;
  return t;
}

gb_lw_tuning tuning_for(gb_lw_context* ctx, int nlay, int kind) {
  const int key = nlay * 4 + kind;
  for (size_t i = 0; i < ctx->tuned_nlay.size(); ++i)
    if (ctx->tuned_nlay[i] == key) return ctx->tuned[i];
  return default_tuning(ctx, nlay, kind);
}

void store_tuning(gb_lw_context* ctx, int nlay, int kind, const gb_lw_tuning& t) {
  const int key = nlay * 4 + kind;
  for (size_t i = 0; i < ctx->tuned_nlay.size(); ++i)
    if (ctx->tuned_nlay[i] == key) {
      ctx->tuned[i] = t;
      return;
    }
  ctx->tuned_nlay.push_back(key);
  ctx->tuned.push_back(t);
}

// One grid through the launch shape tuned (or defaulted) for its layer count
// and kind, with the hand-over buffer `k` of the context (grown on demand).
int launch_one(gb_lw_context* ctx, const LwArgs& a, int k, cudaStream_t stream) {
  if (a.ncol <= 0) return GB_LW_OK;
  LwBatch b;
  b.ngrid = 1;
  b.nsmax = a.nlay;
  b.col0[0] = 0;
  b.col0[1] = a.ncol;
  b.g[0] = a;
  int rc = ensure_buffer(ctx, &ctx->d_gas[k], &ctx->gas_bytes[k], gas_need(a.nlay, a.ncol));
  if (rc) return rc;
  attach_gas(b, ctx->d_gas[k], ctx->gas_bytes[k]);
  const gb_lw_tuning t = tuning_for(ctx, a.nlay, batch_kind(b));
  cudaError_t e = gb_lw_launch_batch(b, ctx->d_tables, t.variant, t.blocks, stream);
  return e == cudaSuccess ? GB_LW_OK : gb_ctx_fail(ctx, e, "column kernels");
}

// A batch with learned gas optics gets the context's hand-over list (room
// for every column of the batch); other batches run the full kernel alone.
int attach_fall(gb_lw_context* ctx, LwBatch& b) {
  b.fall = nullptr;
  b.nfall = nullptr;
  if (!(batch_kind(b) & GB_LW_KIND_LEARNED)) return 0;
  const size_t need = (size_t)b.col0[b.ngrid];
  if (need > ctx->fall_elems || !ctx->d_nfall) {
    cudaFree(ctx->d_fall);
    ctx->d_fall = nullptr;
    ctx->fall_elems = 0;
    if (!ctx->d_nfall && cudaMalloc(&ctx->d_nfall, sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      ctx->d_nfall = nullptr;
      ctx->last_error = "device allocation of the hand-over list failed";
      return GB_LW_E_NOMEM;
    }
    if (cudaMalloc(&ctx->d_fall, need * sizeof(long long)) != cudaSuccess) {
      cudaGetLastError();
      ctx->last_error = "device allocation of the hand-over list failed";
      return GB_LW_E_NOMEM;
    }
    ctx->fall_elems = need;
  }
  b.fall = ctx->d_fall;
  b.nfall = ctx->d_nfall;
  return 0;
}

}  // namespace

// Validates the grids of a batched call and fills the launch descriptor.
// frac < 1 keeps only that fraction of each grid's columns (autotuner sample).
int gb_ctx_make_batch(gb_lw_context* ctx, int ngrid, const gb_lw_grid* grids, double frac, LwBatch& b) {
  if (ngrid < 1 || ngrid > GB_LW_MAX_GRIDS || !grids) return GB_LW_E_ARGS;
  b = LwBatch{};
  b.ngrid = ngrid;
  b.nsmax = 1;
  b.col0[0] = 0;
  for (int i = 0; i < ngrid; ++i) {
    const gb_lw_grid& g = grids[i];
    if (g.ncol < 0 || g.nlay < 1 || g.nlay > GB_MAXLAY || g.ld_in < g.ncol || g.ld_out < g.ncol) return GB_LW_E_ARGS;
    if (!flags_ok(g.idrv, g.inflglw, g.iceflglw, g.liqflglw)) return GB_LW_E_ARGS;
    int icld = (g.icld < 0 || g.icld > 3) ? 2 : g.icld;  // rrtmg_lw_rad.f90:465
    const bool fused = g.cloud_mode == GB_LW_CLOUD_FUSED;
    if (g.cloud_mode != GB_LW_CLOUD_SUBCOL && !fused) return GB_LW_E_ARGS;
    if (fused && icld != 0 && icld != 3) return GB_LW_E_ARGS;
    const double* req[] = {g.play, g.plev, g.tlay, g.tlev, g.tsfc, g.h2ovmr, g.o3vmr, g.co2vmr, g.ch4vmr,
                           g.n2ovmr, g.o2vmr, g.cfc11vmr, g.cfc12vmr, g.cfc22vmr, g.ccl4vmr, g.emis,
                           g.tauaer, g.uflx, g.dflx, g.hr, g.uflxc, g.dflxc, g.hrc};
    if (g.ncol > 0) {
      for (const double* p : req)
        if (!p) return GB_LW_E_ARGS;
      if (icld >= 1 && (!g.reicmcl || !g.relqmcl)) return GB_LW_E_ARGS;
      if (icld >= 1 && !fused && (!g.cldfmcl || !g.taucmcl || !g.ciwpmcl || !g.clwpmcl)) return GB_LW_E_ARGS;
      if (icld >= 1 && fused && (!g.cldfrac || !g.ciwp || !g.clwp || !g.tauc)) return GB_LW_E_ARGS;
      if (g.idrv == 1 && (!g.duflx_dt || !g.duflxc_dt)) return GB_LW_E_ARGS;
    }
    int nc = g.ncol;
    if (frac < 1.0 && nc > 0) nc = std::max(1, std::min(nc, (int)std::ceil(frac * nc)));
    LwArgs& a = b.g[i];
    a = LwArgs{};
    a.ncol = nc; a.nlay = g.nlay; a.ld = g.ld_in; a.ldo = g.ld_out;
    a.icld = icld; a.idrv = g.idrv; a.inflag = g.inflglw; a.iceflag = g.iceflglw; a.liqflag = g.liqflglw;
    a.cloud_mode = fused ? LW_CLOUD_FUSED : LW_CLOUD_SUBCOL;
    a.seed0 = g.seed0;
    a.play = g.play; a.plev = g.plev; a.tlay = g.tlay; a.tlev = g.tlev; a.tsfc = g.tsfc;
    a.h2ovmr = g.h2ovmr; a.o3vmr = g.o3vmr; a.co2vmr = g.co2vmr; a.ch4vmr = g.ch4vmr; a.n2ovmr = g.n2ovmr;
    a.o2vmr = g.o2vmr; a.cfc11vmr = g.cfc11vmr; a.cfc12vmr = g.cfc12vmr; a.cfc22vmr = g.cfc22vmr;
    a.ccl4vmr = g.ccl4vmr; a.emis = g.emis; a.tauaer = g.tauaer;
    a.cldfmcl = g.cldfmcl; a.taucmcl = g.taucmcl; a.ciwpmcl = g.ciwpmcl; a.clwpmcl = g.clwpmcl;
    a.cldfrac = g.cldfrac; a.ciwp = g.ciwp; a.clwp = g.clwp; a.tauc = g.tauc;
    a.reicmcl = g.reicmcl; a.relqmcl = g.relqmcl;
    a.uflx = g.uflx; a.dflx = g.dflx; a.hr = g.hr; a.uflxc = g.uflxc; a.dflxc = g.dflxc; a.hrc = g.hrc;
    a.duflx_dt = g.duflx_dt; a.duflxc_dt = g.duflxc_dt;
    a.col_err = g.d_col_status;
    a.err_flag = ctx->d_err;
    a.sur_tau = reinterpret_cast<const __half*>(g.sur_tau);
    a.sur_frac = reinterpret_cast<const __half*>(g.sur_frac);
    a.sur_flag = g.sur_flag;
    if ((g.sur_tau != nullptr) != (g.sur_frac != nullptr) || (g.sur_tau != nullptr) != (g.sur_flag != nullptr))
      return GB_LW_E_ARGS;
    b.col0[i + 1] = b.col0[i] + nc;
    b.nsmax = std::max(b.nsmax, g.nlay);
  }
  if (gb_lw_smem_bytes(b.nsmax) > ctx->max_smem) {
    ctx->last_error = "nlay too large for one thread block's shared memory";
    return GB_LW_E_ARGS;
  }
  return 0;
}

// hand-over planes for a descriptor's columns from the context's batch buffer
static int attach_batch_gas(gb_lw_context* ctx, LwBatch& b) {
  int rc = ensure_buffer(ctx, &ctx->d_bgas, &ctx->bgas_bytes, gas_need(b.nsmax, b.col0[b.ngrid]));
  if (rc) return rc;
  attach_gas(b, ctx->d_bgas, ctx->bgas_bytes);
  return 0;
}


size_t gb_ctx_fused_draws(const LwBatch& b) {
  size_t n = 0;
  for (int i = 0; i < b.ngrid; ++i)
    if (b.g[i].cloud_mode == LW_CLOUD_FUSED && b.g[i].icld >= 1) n += (size_t)b.g[i].ncol * GB_NGPT;
  return n;
}

int gb_ctx_make_draws(gb_lw_context* ctx, LwBatch& b, double* buf, cudaStream_t stream) {
  size_t off = 0;
  for (int i = 0; i < b.ngrid; ++i) {
    LwArgs& a = b.g[i];
    if (a.cloud_mode != LW_CLOUD_FUSED || a.icld < 1) continue;
    cudaError_t e = gb_mcica_percol_mt(a.ncol, a.seed0, GB_NGPT, buf + off, stream);
    if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "McICA draws");
    a.draws = buf + off;
    off += (size_t)a.ncol * GB_NGPT;
  }
  return GB_LW_OK;
}

int gb_ctx_launch_batch(gb_lw_context* ctx, LwBatch& b, cudaStream_t stream) {
  if (b.col0[b.ngrid] == 0) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  const gb_lw_tuning t = tuning_for(ctx, b.nsmax, batch_kind(b));
  int rc = attach_batch_gas(ctx, b);
  if (rc) return rc;
  const size_t nd = gb_ctx_fused_draws(b);
  if (nd > ctx->fdraws_elems) {
    cudaFree(ctx->d_fdraws);
    ctx->d_fdraws = nullptr;
    ctx->fdraws_elems = 0;
    if (cudaMalloc(&ctx->d_fdraws, nd * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      ctx->last_error = "device allocation of the McICA draws failed";
      return GB_LW_E_NOMEM;
    }
    ctx->fdraws_elems = nd;
  }
  if (nd) {
    rc = gb_ctx_make_draws(ctx, b, ctx->d_fdraws, stream);
    if (rc) return rc;
  }
  if ((rc = attach_fall(ctx, b)) != 0) return rc;
  cudaError_t e = gb_lw_launch_batch(b, ctx->d_tables, t.variant, t.blocks, stream);
  if (e != cudaSuccess) return gb_ctx_fail(ctx, e, "batched launch");
  return GB_LW_OK;
}

namespace {
struct ConstHold {
  std::vector<unsigned char> bytes;
  int holders = 0;
};
std::mutex g_const_mu;
std::map<std::pair<int, int>, ConstHold> g_const;  // (kind, device) -> the bytes live contexts hold
}  // namespace

bool gb_const_acquire(int kind, int device, const void* bytes, size_t n, bool* upload) {
  std::lock_guard<std::mutex> lk(g_const_mu);
  ConstHold& h = g_const[{kind, device}];
  const unsigned char* b = static_cast<const unsigned char*>(bytes);
  if (h.holders > 0 && (h.bytes.size() != n || std::memcmp(h.bytes.data(), b, n) != 0)) return false;
  *upload = h.holders == 0;
  if (h.holders == 0) h.bytes.assign(b, b + n);
  ++h.holders;
  return true;
}

void gb_const_release(int kind, int device) {
  std::lock_guard<std::mutex> lk(g_const_mu);
  auto it = g_const.find({kind, device});
  if (it != g_const.end() && it->second.holders > 0) --it->second.holders;
}

extern "C" {

int gb_rrtmg_lw_ini(double cpdair, const char* table_dir, int device, gb_lw_context** out) {
  if (!out) return GB_LW_E_ARGS;
  *out = nullptr;
  gb_lw_context* ctx = new gb_lw_context();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    int r = cuda_fail(ctx, e, "cudaSetDevice");
    std::fprintf(stderr, "gb_rrtmg_lw_ini: %s\n", ctx->last_error.c_str());
    delete ctx;
    return r;
  }
  std::string dir = table_dir ? table_dir : default_table_dir();
  ctx->table_dir = dir;
  std::string ref = dir + "/lw_ref_tables.gblw", kt = dir + "/lw_ktables.gblw";
  std::vector<float> blob;
  std::vector<double> cloud64;
  std::string err;
  if (!gb_build_tables(ref.c_str(), kt.c_str(), cpdair, ctx->tabs, blob, err, &cloud64)) {
    std::fprintf(stderr, "gb_rrtmg_lw_ini: %s\n", err.c_str());
    delete ctx;
    return GB_LW_E_TABLES;
  }
  ctx->absliq0 = cloud64[ctx->tabs.c64_absliq0];
  ctx->abscld1 = cloud64[ctx->tabs.c64_abscld1];
  bool upload = false;
  if (!gb_const_acquire(GB_CONST_LW, device, &ctx->tabs, sizeof(GbTables), &upload)) {
    std::fprintf(stderr,
                 "gb_rrtmg_lw_ini: another context on device %d holds different longwave tables "
                 "(cpdair or table files); the contexts of a device must agree on them\n",
                 device);
    delete ctx;
    return GB_LW_E_TABLES;
  }
  ctx->lw_const_held = true;
  int dev_smem = 0;
  cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  ctx->max_smem = (size_t)dev_smem;
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaMalloc(&ctx->d_tables, blob.size() * 4) != cudaSuccess || cudaMalloc(&ctx->d_err, 8) != cudaSuccess ||
      cudaMalloc(&ctx->d_cloud64, cloud64.size() * 8) != cudaSuccess) {
    cudaGetLastError();
    gb_rrtmg_lw_free(ctx);
    return GB_LW_E_NOMEM;
  }
  ctx->d_err_host = ctx->d_err + 1;
  if (cudaMemcpy(ctx->d_tables, blob.data(), blob.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->d_cloud64, cloud64.data(), cloud64.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(ctx->d_err, 0, 8) != cudaSuccess || (upload && gb_lw_set_tables(ctx->tabs) != cudaSuccess) ||
      cudaStreamCreateWithFlags(&ctx->streams[0], cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->streams[1], cudaStreamNonBlocking) != cudaSuccess) {
    std::fprintf(stderr, "gb_rrtmg_lw_ini: %s\n", cudaGetErrorString(cudaGetLastError()));
    gb_rrtmg_lw_free(ctx);
    return GB_LW_E_CUDA;
  }
  *out = ctx;
  return GB_LW_OK;
}

int gb_rrtmg_lw_free(gb_lw_context* ctx) {
  if (!ctx) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  for (auto& b : ctx->bufs) {
    cudaFree(b.in);
    cudaFree(b.out);
  }
  for (auto& s : ctx->streams)
    if (s) cudaStreamDestroy(s);
  cudaFree(ctx->d_tables);
  cudaFree(ctx->d_err);
  cudaFree(ctx->d_draws);
  for (auto& p : ctx->d_gas) cudaFree(p);
  cudaFree(ctx->d_bgas);
  cudaFree(ctx->d_sur);
  cudaFree(ctx->d_sur_flag);
  cudaFree(ctx->d_fdraws);
  cudaFree(ctx->d_fall);
  cudaFree(ctx->d_nfall);
  cudaFree(ctx->d_cloud64);
  cudaFree(ctx->d_band);
  cudaFree(ctx->d_ncb);
  cudaFree(ctx->d_sw_tables);
  cudaFree(ctx->d_sw_tables_f);
  cudaFree(ctx->d_sw_scratch);
  if (ctx->lw_const_held) gb_const_release(GB_CONST_LW, ctx->device);
  if (ctx->sw_const_held) gb_const_release(GB_CONST_SW, ctx->device);
  delete ctx;
  return GB_LW_OK;
}

int gb_rrtmg_lw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int* icld, int idrv,
                       const double* play, const double* plev, const double* tlay, const double* tlev,
                       const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                       const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                       const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                       const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
                       const double* cldfmcl, const double* taucmcl, const double* ciwpmcl,
                       const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                       const double* tauaer, double* uflx, double* dflx, double* hr, double* uflxc,
                       double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt, int64_t ld_in,
                       int64_t ld_out, int* d_col_status) {
  if (!ctx || !icld) return GB_LW_E_ARGS;
  if (*icld < 0 || *icld > 3) *icld = 2;  // rrtmg_lw_rad.f90:465
  if (ncol < 0 || nlay < 1 || nlay > GB_MAXLAY || ld_in < ncol || ld_out < ncol) return GB_LW_E_ARGS;
  if (!flags_ok(idrv, inflglw, iceflglw, liqflglw)) return GB_LW_E_ARGS;
  if (gb_lw_smem_bytes(nlay) > ctx->max_smem) {
    ctx->last_error = "nlay too large for one thread block's shared memory";
    return GB_LW_E_ARGS;
  }
  if (ncol == 0) return GB_LW_OK;
  const double* req[] = {play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
                         cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, tauaer, uflx, dflx, hr, uflxc, dflxc, hrc};
  for (const double* p : req)
    if (!p) return GB_LW_E_ARGS;
  if (*icld >= 1 && (!cldfmcl || !taucmcl || !ciwpmcl || !clwpmcl || !reicmcl || !relqmcl)) return GB_LW_E_ARGS;
  if (idrv == 1 && (!duflx_dt || !duflxc_dt)) return GB_LW_E_ARGS;
  LwArgs a{};
  a.ncol = ncol;
  a.nlay = nlay;
  a.ld = ld_in;
  a.ldo = ld_out;
  a.icld = *icld;
  a.idrv = idrv;
  a.inflag = inflglw;
  a.iceflag = iceflglw;
  a.liqflag = liqflglw;
  a.play = play; a.plev = plev; a.tlay = tlay; a.tlev = tlev; a.tsfc = tsfc;
  a.h2ovmr = h2ovmr; a.o3vmr = o3vmr; a.co2vmr = co2vmr; a.ch4vmr = ch4vmr; a.n2ovmr = n2ovmr; a.o2vmr = o2vmr;
  a.cfc11vmr = cfc11vmr; a.cfc12vmr = cfc12vmr; a.cfc22vmr = cfc22vmr; a.ccl4vmr = ccl4vmr; a.emis = emis;
  a.cldfmcl = cldfmcl; a.taucmcl = taucmcl; a.ciwpmcl = ciwpmcl; a.clwpmcl = clwpmcl;
  a.reicmcl = reicmcl; a.relqmcl = relqmcl; a.tauaer = tauaer;
  a.uflx = uflx; a.dflx = dflx; a.hr = hr; a.uflxc = uflxc; a.dflxc = dflxc; a.hrc = hrc;
  a.duflx_dt = duflx_dt; a.duflxc_dt = duflxc_dt;
  a.col_err = d_col_status;
  a.err_flag = ctx->d_err;
  cudaSetDevice(ctx->device);
  return launch_one(ctx, a, 0, (cudaStream_t)stream);
}

int gb_rrtmg_lw_sync_status(gb_lw_context* ctx, void* stream) {
  if (!ctx) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  int h = 0;
  CK(cudaMemcpyAsync(&h, ctx->d_err, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  CK(cudaMemsetAsync(ctx->d_err, 0, 4, (cudaStream_t)stream));
  CK(cudaStreamSynchronize((cudaStream_t)stream));
  return h;
}

int gb_rrtmg_lw(gb_lw_context* ctx, int ncol, int nlay, int* icld, int idrv, const double* play,
                const double* plev, const double* tlay, const double* tlev, const double* tsfc,
                const double* h2ovmr, const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                const double* n2ovmr, const double* o2vmr, const double* cfc11vmr,
                const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
                const double* emis, int inflglw, int iceflglw, int liqflglw, const double* cldfmcl,
                const double* taucmcl, const double* ciwpmcl, const double* clwpmcl,
                const double* reicmcl, const double* relqmcl, const double* tauaer, double* uflx,
                double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc, double* duflx_dt,
                double* duflxc_dt, int64_t ld_in, int64_t ld_out) {
  if (!ctx || !icld) return GB_LW_E_ARGS;
  if (*icld < 0 || *icld > 3) *icld = 2;
  if (ncol < 0 || nlay < 1 || nlay > GB_MAXLAY || ld_in < ncol || ld_out < ncol) return GB_LW_E_ARGS;
  if (!flags_ok(idrv, inflglw, iceflglw, liqflglw)) return GB_LW_E_ARGS;
  if (gb_lw_smem_bytes(nlay) > ctx->max_smem) return GB_LW_E_ARGS;
  if (ncol == 0) return GB_LW_OK;
  const bool clouds = *icld >= 1;
  if (clouds && (!cldfmcl || !taucmcl || !ciwpmcl || !clwpmcl || !reicmcl || !relqmcl)) return GB_LW_E_ARGS;
  if (idrv == 1 && (!duflx_dt || !duflxc_dt)) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  // chunk size: about 2 GB of inputs per chunk buffer
  const size_t per_col = (size_t)(600 * nlay + 64) * 8;
  int C = (int)std::max<size_t>(1, std::min<size_t>((size_t)ncol, (size_t)(2ull << 30) / per_col));
  int rc = ensure_chunks(ctx, C, nlay);
  if (rc) return rc;
  const InLayout li = in_layout(C, nlay);
  const OutLayout lo = out_layout(C, nlay);
  CK(cudaMemsetAsync(ctx->d_err_host, 0, 4, ctx->streams[0]));
  CK(cudaStreamSynchronize(ctx->streams[0]));
  const double* gas_src[10] = {h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr};
  int nchunks = (ncol + C - 1) / C;
  for (int k = 0; k < nchunks; ++k) {
    const int c0 = k * C, nc = std::min(C, ncol - c0);
    cudaStream_t s = ctx->streams[k & 1];
    double* I = ctx->bufs[k & 1].in;
    double* O = ctx->bufs[k & 1].out;
    const size_t P = C;  // device pitch
    auto H2D = [&](size_t doff, const double* src, size_t rows) {
      return copy2d(I + doff, P, src + c0, (size_t)ld_in, nc, rows, cudaMemcpyHostToDevice, s);
    };
    CK(H2D(li.play, play, nlay));
    CK(H2D(li.plev, plev, nlay + 1));
    CK(H2D(li.tlay, tlay, nlay));
    CK(H2D(li.tlev, tlev, nlay + 1));
    CK(H2D(li.tsfc, tsfc, 1));
    for (int g = 0; g < 10; ++g) CK(H2D(li.gas[g], gas_src[g], nlay));
    CK(H2D(li.emis, emis, 16));
    CK(H2D(li.tauaer, tauaer, (size_t)nlay * 16));
    if (clouds) {
      CK(H2D(li.reic, reicmcl, nlay));
      CK(H2D(li.relq, relqmcl, nlay));
      auto MC = [&](size_t doff, const double* src) {
        return copy2d(I + doff, (size_t)GB_NGPT * P, src + (size_t)GB_NGPT * c0, (size_t)GB_NGPT * ld_in,
                      (size_t)GB_NGPT * nc, nlay, cudaMemcpyHostToDevice, s);
      };
      CK(MC(li.cldf, cldfmcl));
      CK(MC(li.tauc, taucmcl));
      CK(MC(li.ciwp, ciwpmcl));
      CK(MC(li.clwp, clwpmcl));
    }
    LwArgs a{};
    a.ncol = nc;
    a.nlay = nlay;
    a.ld = P;
    a.ldo = P;
    a.icld = *icld;
    a.idrv = idrv;
    a.inflag = inflglw;
    a.iceflag = iceflglw;
    a.liqflag = liqflglw;
    a.play = I + li.play; a.plev = I + li.plev; a.tlay = I + li.tlay; a.tlev = I + li.tlev; a.tsfc = I + li.tsfc;
    a.h2ovmr = I + li.gas[0]; a.o3vmr = I + li.gas[1]; a.co2vmr = I + li.gas[2]; a.ch4vmr = I + li.gas[3];
    a.n2ovmr = I + li.gas[4]; a.o2vmr = I + li.gas[5]; a.cfc11vmr = I + li.gas[6]; a.cfc12vmr = I + li.gas[7];
    a.cfc22vmr = I + li.gas[8]; a.ccl4vmr = I + li.gas[9]; a.emis = I + li.emis;
    a.reicmcl = I + li.reic; a.relqmcl = I + li.relq; a.tauaer = I + li.tauaer;
    a.cldfmcl = I + li.cldf; a.taucmcl = I + li.tauc; a.ciwpmcl = I + li.ciwp; a.clwpmcl = I + li.clwp;
    a.uflx = O + lo.uflx; a.dflx = O + lo.dflx; a.uflxc = O + lo.uflxc; a.dflxc = O + lo.dflxc;
    a.duflx_dt = O + lo.duflx; a.duflxc_dt = O + lo.duflxc; a.hr = O + lo.hr; a.hrc = O + lo.hrc;
    a.col_err = nullptr;
    a.err_flag = ctx->d_err_host;
    rc = launch_one(ctx, a, k & 1, s);
    if (rc) return rc;
    auto D2H = [&](double* dst, size_t soff, size_t rows) {
      return copy2d(dst + c0, (size_t)ld_out, O + soff, P, nc, rows, cudaMemcpyDeviceToHost, s);
    };
    CK(D2H(uflx, lo.uflx, nlay + 1));
    CK(D2H(dflx, lo.dflx, nlay + 1));
    CK(D2H(uflxc, lo.uflxc, nlay + 1));
    CK(D2H(dflxc, lo.dflxc, nlay + 1));
    CK(D2H(hr, lo.hr, nlay));
    CK(D2H(hrc, lo.hrc, nlay));
    if (idrv == 1) {
      CK(D2H(duflx_dt, lo.duflx, nlay + 1));
      CK(D2H(duflxc_dt, lo.duflxc, nlay + 1));
    }
  }
  CK(cudaStreamSynchronize(ctx->streams[0]));
  CK(cudaStreamSynchronize(ctx->streams[1]));
  int h = 0;
  CK(cudaMemcpy(&h, ctx->d_err_host, 4, cudaMemcpyDeviceToHost));
  return h;
}

namespace {

// grows a device array of the context to at least `n` elements of `size` bytes
int ensure_elems(gb_lw_context* ctx, void** p, size_t* have, size_t n, size_t size, const char* what) {
  if (*p && *have >= n) return 0;
  cudaFree(*p);
  *p = nullptr;
  *have = 0;
  if (cudaMalloc(p, n * size) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    ctx->last_error = std::string("device allocation failed: ") + what;
    return GB_LW_E_NOMEM;
  }
  *have = n;
  return 0;
}

// argument checks shared by the non-McICA entry points
int nomcica_check(gb_lw_context* ctx, int ncol, int nlay, int* icld, int idrv, int inflglw, int iceflglw,
                  int liqflglw, int64_t ld_in, int64_t ld_out) {
  if (!ctx || !icld) return GB_LW_E_ARGS;
  if (*icld < 0 || *icld > 3) *icld = 2;  // rrtmg_lw_rad.nomcica.f90:456
  if (ncol < 0 || nlay < 1 || nlay > GB_MAXLAY || ld_in < ncol || ld_out < ncol) return GB_LW_E_ARGS;
  if (!flags_ok(idrv, inflglw, iceflglw, liqflglw)) return GB_LW_E_ARGS;
  if (gb_lw_smem_bytes(nlay) > ctx->max_smem) {
    ctx->last_error = "nlay too large for one thread block's shared memory";
    return GB_LW_E_ARGS;
  }
  return 0;
}

// one grid of band clouds: cldprop into the context's band buffers, then the
// band-cloud kernel (status into `err`, per-column codes into col_err)
int nomcica_launch(gb_lw_context* ctx, LwArgs a, const double* cldfr, const double* taucld, const double* cicewp,
                   const double* cliqwp, const double* reice, const double* reliq, int k, cudaStream_t stream) {
  a.cloud_mode = LW_CLOUD_BAND;
  if (a.icld >= 1) {
    int rc = ensure_elems(ctx, reinterpret_cast<void**>(&ctx->d_band), &ctx->band_elems, (size_t)16 * a.ld * a.nlay,
                          sizeof(double), "band cloud depths");
    if (!rc)
      rc = ensure_elems(ctx, reinterpret_cast<void**>(&ctx->d_ncb), &ctx->ncb_elems, (size_t)a.ld, sizeof(int),
                        "cloud-band counts");
    if (!rc)
      rc = gb_ctx_cldprop(ctx, stream, a.ncol, a.nlay, a.inflag, a.iceflag, a.liqflag, cldfr, taucld, cicewp, cliqwp,
                          reice, reliq, ctx->d_band, a.ld, a.col_err, ctx->d_ncb, a.err_flag);
    if (rc) return rc;
    a.cldfrac = cldfr;
    a.tauc = ctx->d_band;
    a.ncbands = ctx->d_ncb;
  } else if (a.col_err) {
    CK(cudaMemsetAsync(a.col_err, 0, sizeof(int) * (size_t)a.ncol, stream));
  }
  return launch_one(ctx, a, k, stream);
}

}  // namespace

int gb_rrtmg_lw_nomcica_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int* icld, int idrv,
                               const double* play, const double* plev, const double* tlay, const double* tlev,
                               const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                               const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                               const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                               const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
                               const double* cldfr, const double* taucld, const double* cicewp, const double* cliqwp,
                               const double* reice, const double* reliq, const double* tauaer, double* uflx,
                               double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc, double* duflx_dt,
                               double* duflxc_dt, int64_t ld_in, int64_t ld_out, int* d_col_status) {
  int rc = nomcica_check(ctx, ncol, nlay, icld, idrv, inflglw, iceflglw, liqflglw, ld_in, ld_out);
  if (rc || ncol == 0) return rc;
  const double* req[] = {play, plev, tlay, tlev, tsfc, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr,
                         cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr, emis, tauaer, uflx, dflx, hr, uflxc, dflxc, hrc};
  for (const double* p : req)
    if (!p) return GB_LW_E_ARGS;
  if (*icld >= 1 && (!cldfr || !taucld || !cicewp || !cliqwp || !reice || !reliq)) return GB_LW_E_ARGS;
  if (idrv == 1 && (!duflx_dt || !duflxc_dt)) return GB_LW_E_ARGS;
  LwArgs a{};
  a.ncol = ncol;
  a.nlay = nlay;
  a.ld = ld_in;
  a.ldo = ld_out;
  a.icld = *icld;
  a.idrv = idrv;
  a.inflag = inflglw;
  a.iceflag = iceflglw;
  a.liqflag = liqflglw;
  a.play = play; a.plev = plev; a.tlay = tlay; a.tlev = tlev; a.tsfc = tsfc;
  a.h2ovmr = h2ovmr; a.o3vmr = o3vmr; a.co2vmr = co2vmr; a.ch4vmr = ch4vmr; a.n2ovmr = n2ovmr; a.o2vmr = o2vmr;
  a.cfc11vmr = cfc11vmr; a.cfc12vmr = cfc12vmr; a.cfc22vmr = cfc22vmr; a.ccl4vmr = ccl4vmr; a.emis = emis;
  a.tauaer = tauaer;
  a.uflx = uflx; a.dflx = dflx; a.hr = hr; a.uflxc = uflxc; a.dflxc = dflxc; a.hrc = hrc;
  a.duflx_dt = duflx_dt; a.duflxc_dt = duflxc_dt;
  a.col_err = d_col_status;
  a.err_flag = ctx->d_err;
  cudaSetDevice(ctx->device);
  return nomcica_launch(ctx, a, cldfr, taucld, cicewp, cliqwp, reice, reliq, 0, (cudaStream_t)stream);
}

int gb_rrtmg_lw_nomcica(gb_lw_context* ctx, int ncol, int nlay, int* icld, int idrv, const double* play,
                        const double* plev, const double* tlay, const double* tlev, const double* tsfc,
                        const double* h2ovmr, const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                        const double* n2ovmr, const double* o2vmr, const double* cfc11vmr, const double* cfc12vmr,
                        const double* cfc22vmr, const double* ccl4vmr, const double* emis, int inflglw,
                        int iceflglw, int liqflglw, const double* cldfr, const double* taucld,
                        const double* cicewp, const double* cliqwp, const double* reice, const double* reliq,
                        const double* tauaer, double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc,
                        double* hrc, double* duflx_dt, double* duflxc_dt, int64_t ld_in, int64_t ld_out) {
  int rc = nomcica_check(ctx, ncol, nlay, icld, idrv, inflglw, iceflglw, liqflglw, ld_in, ld_out);
  if (rc || ncol == 0) return rc;
  const bool clouds = *icld >= 1;
  if (clouds && (!cldfr || !taucld || !cicewp || !cliqwp || !reice || !reliq)) return GB_LW_E_ARGS;
  if (idrv == 1 && (!duflx_dt || !duflxc_dt)) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  // chunks of the same buffers as gb_rrtmg_lw; the band clouds take the
  // space of the McICA arrays: cldfr, cicewp, cliqwp and taucld in the
  // cldfmcl area, cldprop's depths in the taucmcl area
  const size_t per_col = (size_t)(600 * nlay + 64) * 8;
  int C = (int)std::max<size_t>(1, std::min<size_t>((size_t)ncol, (size_t)(2ull << 30) / per_col));
  rc = ensure_chunks(ctx, C, nlay);
  if (rc) return rc;
  const InLayout li = in_layout(C, nlay);
  const OutLayout lo = out_layout(C, nlay);
  CK(cudaMemsetAsync(ctx->d_err_host, 0, 4, ctx->streams[0]));
  CK(cudaStreamSynchronize(ctx->streams[0]));
  const double* gas_src[10] = {h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr};
  const size_t lay = (size_t)C * nlay;
  const int nchunks = (ncol + C - 1) / C;
  for (int k = 0; k < nchunks; ++k) {
    const int c0 = k * C, nc = std::min(C, ncol - c0);
    cudaStream_t s = ctx->streams[k & 1];
    double* I = ctx->bufs[k & 1].in;
    double* O = ctx->bufs[k & 1].out;
    const size_t P = C;
    auto H2D = [&](size_t doff, const double* src, size_t rows) {
      return copy2d(I + doff, P, src + c0, (size_t)ld_in, nc, rows, cudaMemcpyHostToDevice, s);
    };
    CK(H2D(li.play, play, nlay));
    CK(H2D(li.plev, plev, nlay + 1));
    CK(H2D(li.tlay, tlay, nlay));
    CK(H2D(li.tlev, tlev, nlay + 1));
    CK(H2D(li.tsfc, tsfc, 1));
    for (int g = 0; g < 10; ++g) CK(H2D(li.gas[g], gas_src[g], nlay));
    CK(H2D(li.emis, emis, 16));
    CK(H2D(li.tauaer, tauaer, (size_t)nlay * 16));
    const size_t cf_o = li.cldf, ci_o = li.cldf + lay, cw_o = li.cldf + 2 * lay, tc_o = li.cldf + 3 * lay;
    if (clouds) {
      CK(H2D(cf_o, cldfr, nlay));
      CK(H2D(ci_o, cicewp, nlay));
      CK(H2D(cw_o, cliqwp, nlay));
      CK(H2D(li.reic, reice, nlay));
      CK(H2D(li.relq, reliq, nlay));
      CK(copy2d(I + tc_o, 16 * P, taucld + (size_t)16 * c0, (size_t)16 * ld_in, (size_t)16 * nc, nlay,
                cudaMemcpyHostToDevice, s));
    }
    LwArgs a{};
    a.ncol = nc;
    a.nlay = nlay;
    a.ld = P;
    a.ldo = P;
    a.icld = *icld;
    a.idrv = idrv;
    a.inflag = inflglw;
    a.iceflag = iceflglw;
    a.liqflag = liqflglw;
    a.play = I + li.play; a.plev = I + li.plev; a.tlay = I + li.tlay; a.tlev = I + li.tlev; a.tsfc = I + li.tsfc;
    a.h2ovmr = I + li.gas[0]; a.o3vmr = I + li.gas[1]; a.co2vmr = I + li.gas[2]; a.ch4vmr = I + li.gas[3];
    a.n2ovmr = I + li.gas[4]; a.o2vmr = I + li.gas[5]; a.cfc11vmr = I + li.gas[6]; a.cfc12vmr = I + li.gas[7];
    a.cfc22vmr = I + li.gas[8]; a.ccl4vmr = I + li.gas[9]; a.emis = I + li.emis; a.tauaer = I + li.tauaer;
    a.uflx = O + lo.uflx; a.dflx = O + lo.dflx; a.uflxc = O + lo.uflxc; a.dflxc = O + lo.dflxc;
    a.duflx_dt = O + lo.duflx; a.duflxc_dt = O + lo.duflxc; a.hr = O + lo.hr; a.hrc = O + lo.hrc;
    a.col_err = nullptr;
    a.err_flag = ctx->d_err_host;
    if (clouds) {
      // cldprop's outputs in the chunk's own buffers (the chunks of the two streams overlap)
      a.cloud_mode = LW_CLOUD_BAND;
      double* band = I + li.tauc;
      int* ncb = reinterpret_cast<int*>(I + li.ciwp);
      rc = gb_ctx_cldprop(ctx, s, nc, nlay, inflglw, iceflglw, liqflglw, I + cf_o, I + tc_o, I + ci_o, I + cw_o,
                          I + li.reic, I + li.relq, band, (int64_t)P, nullptr, ncb, ctx->d_err_host);
      if (rc) return rc;
      a.cldfrac = I + cf_o;
      a.tauc = band;
      a.ncbands = ncb;
      rc = launch_one(ctx, a, k & 1, s);
    } else {
      rc = nomcica_launch(ctx, a, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, k & 1, s);
    }
    if (rc) return rc;
    auto D2H = [&](double* dst, size_t soff, size_t rows) {
      return copy2d(dst + c0, (size_t)ld_out, O + soff, P, nc, rows, cudaMemcpyDeviceToHost, s);
    };
    CK(D2H(uflx, lo.uflx, nlay + 1));
    CK(D2H(dflx, lo.dflx, nlay + 1));
    CK(D2H(uflxc, lo.uflxc, nlay + 1));
    CK(D2H(dflxc, lo.dflxc, nlay + 1));
    CK(D2H(hr, lo.hr, nlay));
    CK(D2H(hrc, lo.hrc, nlay));
    if (idrv == 1) {
      CK(D2H(duflx_dt, lo.duflx, nlay + 1));
      CK(D2H(duflxc_dt, lo.duflxc, nlay + 1));
    }
  }
  CK(cudaStreamSynchronize(ctx->streams[0]));
  CK(cudaStreamSynchronize(ctx->streams[1]));
  int h = 0;
  CK(cudaMemcpy(&h, ctx->d_err_host, 4, cudaMemcpyDeviceToHost));
  return h;
}

int gb_mcica_subcol_lw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int icld, int permuteseed,
                              int* irng, const double* play, const double* cldfrac, const double* ciwp,
                              const double* clwp, const double* rei, const double* rel, const double* tauc,
                              const double* alpha, double* cldfmcl, double* ciwpmcl, double* clwpmcl,
                              double* reicmcl, double* relqmcl, double* taucmcl, int64_t ld,
                              int seed_per_column) {
  if (!ctx || !irng) return GB_LW_E_ARGS;
  if (icld == 0) return GB_LW_OK;  // mcica_subcol_gen_lw.f90:257
  if (icld < 0 || icld > 5) return GB_LW_E_ICLD;
  if (ncol < 0 || nlay < 1 || ld < ncol) return GB_LW_E_ARGS;
  if (*irng != 0) *irng = 1;  // :444
  if (icld >= 4 && !alpha) return GB_LW_E_ARGS;
  if (*irng == 0 && nlay < 4) return GB_LW_E_ARGS;
  if (ncol == 0) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  size_t need = gb_mcica_draw_count(ncol, nlay, icld);
  if (need > ctx->draws_elems) {
    cudaFree(ctx->d_draws);
    ctx->d_draws = nullptr;
    ctx->draws_elems = 0;
    if (cudaMalloc(&ctx->d_draws, need * 8) != cudaSuccess) {
      cudaGetLastError();
      return GB_LW_E_NOMEM;
    }
    ctx->draws_elems = need;
  }
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
  for (int g = 0; g < GB_NGPT; ++g) a.ngb[g] = ctx->tabs.ngb[g];
  CK(gb_mcica_launch(a, ctx->d_draws, ctx->d_err, (cudaStream_t)stream, seed_per_column != 0));
  return GB_LW_OK;
}

int gb_mcica_subcol_lw(gb_lw_context* ctx, int ncol, int nlay, int icld, int permuteseed, int* irng,
                       const double* play, const double* cldfrac, const double* ciwp, const double* clwp,
                       const double* rei, const double* rel, const double* tauc, const double* alpha,
                       double* cldfmcl, double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl,
                       double* taucmcl, int64_t ld, int seed_per_column) {
  if (!ctx || !irng) return GB_LW_E_ARGS;
  if (icld == 0) return GB_LW_OK;
  if (icld < 0 || icld > 5) return GB_LW_E_ICLD;
  if (ncol < 0 || nlay < 1 || ld < ncol) return GB_LW_E_ARGS;
  if (ncol == 0) return GB_LW_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->streams[0];
  // device copies with leading dimension ncol
  const size_t n2 = (size_t)ncol * nlay, nm = (size_t)GB_NGPT * n2;
  double* d = nullptr;
  size_t total = 7 * n2 + 16 * n2 + 4 * nm + 2 * n2;
  if (cudaMalloc(&d, total * 8) != cudaSuccess) {
    cudaGetLastError();
    return GB_LW_E_NOMEM;
  }
  double *dplay = d, *dcf = d + n2, *dci = d + 2 * n2, *dcl = d + 3 * n2, *dre = d + 4 * n2, *drl = d + 5 * n2,
         *dal = d + 6 * n2, *dtc = d + 7 * n2, *o_cf = dtc + 16 * n2, *o_ci = o_cf + nm, *o_cl = o_ci + nm,
         *o_tc = o_cl + nm, *o_re = o_tc + nm, *o_rl = o_re + n2;
  int rc = GB_LW_OK;
  auto fail = [&](cudaError_t e, const char* w) {
    rc = cuda_fail(ctx, e, w);
  };
  struct Cp { double* dst; const double* src; size_t w, rows; } cps[] = {
      {dplay, play, (size_t)ncol, (size_t)nlay}, {dcf, cldfrac, (size_t)ncol, (size_t)nlay},
      {dci, ciwp, (size_t)ncol, (size_t)nlay}, {dcl, clwp, (size_t)ncol, (size_t)nlay},
      {dre, rei, (size_t)ncol, (size_t)nlay}, {drl, rel, (size_t)ncol, (size_t)nlay}};
  for (auto& c : cps) {
    cudaError_t e = copy2d(c.dst, c.w, c.src, (size_t)ld, c.w, c.rows, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { fail(e, "mcica H2D"); break; }
  }
  if (rc == GB_LW_OK && alpha) {
    cudaError_t e = copy2d(dal, ncol, alpha, (size_t)ld, ncol, nlay, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) fail(e, "mcica H2D alpha");
  }
  if (rc == GB_LW_OK) {
    cudaError_t e = copy2d(dtc, (size_t)16 * ncol, tauc, (size_t)16 * ld, (size_t)16 * ncol, nlay, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) fail(e, "mcica H2D tauc");
  }
  if (rc == GB_LW_OK) {
    rc = gb_mcica_subcol_lw_device(ctx, s, ncol, nlay, icld, permuteseed, irng, dplay, dcf, dci, dcl, dre, drl, dtc,
                                   alpha ? dal : nullptr, o_cf, o_ci, o_cl, o_re, o_rl, o_tc, ncol, seed_per_column);
  }
  if (rc == GB_LW_OK) {
    struct Back { double* dst; const double* src; size_t w; } bk[] = {
        {cldfmcl, o_cf, (size_t)GB_NGPT * ncol}, {ciwpmcl, o_ci, (size_t)GB_NGPT * ncol},
        {clwpmcl, o_cl, (size_t)GB_NGPT * ncol}, {taucmcl, o_tc, (size_t)GB_NGPT * ncol}};
    for (auto& b : bk) {
      cudaError_t e = copy2d(b.dst, (size_t)GB_NGPT * ld, b.src, b.w, b.w, nlay, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) { fail(e, "mcica D2H"); break; }
    }
    if (rc == GB_LW_OK) {
      cudaError_t e = copy2d(reicmcl, (size_t)ld, o_re, ncol, ncol, nlay, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = copy2d(relqmcl, (size_t)ld, o_rl, ncol, ncol, nlay, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) fail(e, "mcica D2H radii");
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  if (rc == GB_LW_OK && e != cudaSuccess) rc = cuda_fail(ctx, e, "mcica sync");
  int h = 0;
  if (rc == GB_LW_OK) {
    cudaMemcpy(&h, ctx->d_err, 4, cudaMemcpyDeviceToHost);
    cudaMemset(ctx->d_err, 0, 4);
    rc = h;
  }
  cudaFree(d);
  return rc;
}

int gb_rrtmg_lw_gas_optics_diag(gb_lw_context* ctx, int ncol, int nlay, const double* play, const double* plev,
                                const double* tlay, const double* tlev, const double* tsfc, const double* h2ovmr,
                                const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                                const double* n2ovmr, const double* o2vmr, const double* cfc11vmr,
                                const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
                                const double* emis, const double* tauaer, float* taut, float* fracs) {
  if (!ctx || ncol <= 0 || nlay < 1 || nlay > GB_MAXLAY || !taut || !fracs) return GB_LW_E_ARGS;
  (void)tlev;
  (void)tsfc;
  (void)emis;
  cudaSetDevice(ctx->device);
  const size_t n2 = (size_t)ncol * nlay, n3 = (size_t)ncol * (nlay + 1);
  const double* src2[] = {play, tlay, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr};
  double* d = nullptr;
  float* dt = nullptr;
  if (cudaMalloc(&d, (12 * n2 + n3) * 8) != cudaSuccess || cudaMalloc(&dt, 2 * n2 * GB_NGPT * 4) != cudaSuccess) {
    cudaFree(d);
    cudaGetLastError();
    return GB_LW_E_NOMEM;
  }
  double* dev2[12];
  for (int k = 0; k < 12; ++k) {
    dev2[k] = d + k * n2;
    cudaMemcpy(dev2[k], src2[k], n2 * 8, cudaMemcpyHostToDevice);
  }
  double* dplev = d + 12 * n2;
  cudaMemcpy(dplev, plev, n3 * 8, cudaMemcpyHostToDevice);
  LwBatch b;
  b.ngrid = 1;
  b.nsmax = nlay;
  b.col0[0] = 0;
  b.col0[1] = ncol;
  LwArgs& a = b.g[0];
  a = LwArgs{};
  a.ncol = ncol; a.nlay = nlay; a.ld = ncol; a.ldo = ncol;
  a.play = dev2[0]; a.tlay = dev2[1]; a.h2ovmr = dev2[2]; a.o3vmr = dev2[3]; a.co2vmr = dev2[4];
  a.ch4vmr = dev2[5]; a.n2ovmr = dev2[6]; a.o2vmr = dev2[7]; a.cfc11vmr = dev2[8]; a.cfc12vmr = dev2[9];
  a.cfc22vmr = dev2[10]; a.ccl4vmr = dev2[11]; a.plev = dplev;
  a.err_flag = ctx->d_err_host;
  // the taumol kernel writes column i, layer l at row i * nlay + l
  b.gstride = (long long)nlay * GB_NGPT;
  b.gslots = ncol;
  b.gtau = dt;
  b.gfrac = dt + n2 * GB_NGPT;
  int rc = GB_LW_OK;
  cudaError_t e = gb_lw_launch_gas(b, ctx->d_tables, 0, ncol, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(taut, dt, n2 * GB_NGPT * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(fracs, dt + n2 * GB_NGPT, n2 * GB_NGPT * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = cuda_fail(ctx, e, "gas optics diagnostics");
  if (rc == GB_LW_OK) {
    // taut = taug + the aerosol optical depth of the g-point's band (rrtmg_lw_rad.f90:548-553), in fp32
    for (int i = 0; i < ncol; ++i)
      for (int l = 0; l < nlay; ++l)
        for (int g = 0; g < GB_NGPT; ++g) {
          const int ib = ctx->tabs.ngb[g] - 1;
          taut[((size_t)i * nlay + l) * GB_NGPT + g] += (float)tauaer[i + (size_t)ncol * (l + (size_t)nlay * ib)];
        }
  }
  cudaFree(d);
  cudaFree(dt);
  return rc;
}

int gb_rrtmg_lw_batch_device(gb_lw_context* ctx, void* stream, int ngrid, const gb_lw_grid* grids) {
  if (!ctx) return GB_LW_E_ARGS;
  LwBatch b;
  int rc = gb_ctx_make_batch(ctx, ngrid, grids, 1.0, b);
  if (rc) return rc;
  return gb_ctx_launch_batch(ctx, b, (cudaStream_t)stream);
}

int gb_rrtmg_lw_tuning_get(gb_lw_context* ctx, int nlay, int kind, gb_lw_tuning* out) {
  if (!ctx || !out || nlay < 1 || nlay > GB_MAXLAY || kind < 0 || kind > 3) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  *out = tuning_for(ctx, nlay, kind);
  return GB_LW_OK;
}

int gb_rrtmg_lw_num_variants(void) { return gb_lw_num_variants(); }

int gb_rrtmg_lw_tuning_set(gb_lw_context* ctx, int nlay, int kind, const gb_lw_tuning* shape) {
  if (!ctx || !shape || nlay < 1 || nlay > GB_MAXLAY || kind < 0 || kind > 3) return GB_LW_E_ARGS;
  if (shape->variant < 0 || shape->variant >= gb_lw_num_variants()) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  const bool lean = kind & GB_LW_KIND_LEARNED;
  const int occ = gb_lw_slots(nlay, shape->variant, lean) / std::max(1, ctx->num_sms);
  if (shape->blocks_per_sm < 1 || shape->blocks_per_sm > occ) {
    ctx->last_error = "blocks_per_sm exceeds what fits on an SM for this nlay and variant";
    return GB_LW_E_ARGS;
  }
  gb_lw_tuning t{};
  t.variant = shape->variant;
  t.threads = gb_lw_variant(t.variant, lean).threads;
  t.min_blocks = gb_lw_variant(t.variant, lean).min_blocks;
  t.blocks_per_sm = shape->blocks_per_sm;
  t.blocks = t.blocks_per_sm * ctx->num_sms;
  t.ms = shape->ms;
  store_tuning(ctx, nlay, kind, t);
  return GB_LW_OK;
}

int gb_rrtmg_lw_autotune(gb_lw_context* ctx, void* stream, int ngrid, const gb_lw_grid* grids, int sample_cols,
                         int reps, gb_lw_tuning* best) {
  if (!ctx) return GB_LW_E_ARGS;
  LwBatch full;
  int rc = gb_ctx_make_batch(ctx, ngrid, grids, 1.0, full);
  if (rc) return rc;
  const long long total = full.col0[ngrid];
  if (total == 0) return GB_LW_E_ARGS;
  const double frac = sample_cols > 0 && sample_cols < total ? (double)sample_cols / (double)total : 1.0;
  LwBatch b;
  rc = gb_ctx_make_batch(ctx, ngrid, grids, frac, b);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  reps = std::max(1, reps);
  // candidate shapes: every variant at 1 .. max resident blocks per SM
  struct Cand { int v, per; };
  std::vector<Cand> cands;
  int max_blocks = 1;
  const bool lean = batch_kind(b) & GB_LW_KIND_LEARNED;
  for (int v = 0; v < gb_lw_num_variants(); ++v) {
    const int occ = gb_lw_slots(b.nsmax, v, lean) / std::max(1, ctx->num_sms);
    for (int per = 1; per <= occ; ++per) {
      cands.push_back({v, per});
      max_blocks = std::max(max_blocks, per * ctx->num_sms);
    }
  }
  if (cands.empty()) return GB_LW_E_ARGS;
  (void)max_blocks;
  if ((rc = attach_batch_gas(ctx, b)) != 0) return rc;
  if ((rc = attach_fall(ctx, b)) != 0) return rc;
  // the fused-cloud draws are made once: every candidate times the column kernel alone
  const size_t nd = gb_ctx_fused_draws(b);
  if (nd > ctx->fdraws_elems) {
    cudaFree(ctx->d_fdraws);
    ctx->d_fdraws = nullptr;
    ctx->fdraws_elems = 0;
    if (cudaMalloc(&ctx->d_fdraws, nd * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return GB_LW_E_NOMEM;
    }
    ctx->fdraws_elems = nd;
  }
  if (nd && (rc = gb_ctx_make_draws(ctx, b, ctx->d_fdraws, st)) != 0) return rc;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  gb_lw_tuning bt{};
  bt.ms = 1e30;
  ctx->last_tune.clear();
  cudaError_t err = cudaSuccess;
  for (const Cand& c : cands) {
    const int nb = c.per * ctx->num_sms;
    err = gb_lw_launch_batch(b, ctx->d_tables, c.v, nb, st);  // warm-up
    if (err == cudaSuccess) err = cudaEventRecord(e0, st);
    for (int r = 0; r < reps && err == cudaSuccess; ++r) err = gb_lw_launch_batch(b, ctx->d_tables, c.v, nb, st);
    if (err == cudaSuccess) err = cudaEventRecord(e1, st);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err != cudaSuccess) break;
    const double per_launch = ms / reps;
    gb_lw_tuning rec{};
    rec.variant = c.v;
    rec.threads = gb_lw_variant(c.v, lean).threads;
    rec.min_blocks = gb_lw_variant(c.v, lean).min_blocks;
    rec.blocks_per_sm = c.per;
    rec.blocks = nb;
    rec.ms = per_launch;
    ctx->last_tune.push_back(rec);
    if (per_launch < bt.ms) {
      bt.variant = c.v;
      bt.threads = gb_lw_variant(c.v, lean).threads;
      bt.min_blocks = gb_lw_variant(c.v, lean).min_blocks;
      bt.blocks_per_sm = c.per;
      bt.blocks = nb;
      bt.ms = per_launch;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return cuda_fail(ctx, err, "autotune");
  store_tuning(ctx, b.nsmax, batch_kind(b), bt);
  if (best) *best = bt;
  return GB_LW_OK;
}

int gb_rrtmg_lw_autotune_report(gb_lw_context* ctx, gb_lw_tuning* out, int max) {
  if (!ctx || (max > 0 && !out)) return GB_LW_E_ARGS;
  const int n = (int)ctx->last_tune.size();
  for (int i = 0; i < n && i < max; ++i) out[i] = ctx->last_tune[i];
  return n;
}

int gb_rrtmg_lw_batch_graph_create(gb_lw_context* ctx, int ngrid, const gb_lw_grid* grids, gb_lw_graph** out) {
  if (!ctx || !out) return GB_LW_E_ARGS;
  *out = nullptr;
  LwBatch b;
  int rc = gb_ctx_make_batch(ctx, ngrid, grids, 1.0, b);
  if (rc) return rc;
  if (b.col0[ngrid] == 0) return GB_LW_E_ARGS;
  cudaSetDevice(ctx->device);
  const gb_lw_tuning t = tuning_for(ctx, b.nsmax, batch_kind(b));
  gb_lw_graph* g = new gb_lw_graph();
  g->ctx = ctx;
  const size_t gbytes = gas_need(b.nsmax, b.col0[ngrid]);
  if (cudaMalloc(&g->gas, gbytes) != cudaSuccess) {
    cudaGetLastError();
    delete g;
    return GB_LW_E_NOMEM;
  }
  attach_gas(b, g->gas, gbytes);
  const size_t nd = gb_ctx_fused_draws(b);
  if (nd && cudaMalloc(&g->draws, nd * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    gb_rrtmg_lw_graph_destroy(g);
    return GB_LW_E_NOMEM;
  }
  if (batch_kind(b) & GB_LW_KIND_LEARNED) {  // the graph owns its hand-over list
    if (cudaMalloc(&g->fall, (size_t)b.col0[ngrid] * sizeof(long long)) != cudaSuccess ||
        cudaMalloc(&g->nfall, sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      gb_rrtmg_lw_graph_destroy(g);
      return GB_LW_E_NOMEM;
    }
    b.fall = g->fall;
    b.nfall = g->nfall;
  }
  cudaStream_t s = ctx->streams[0];
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    cudaError_t le = cudaSuccess;
    if (nd && gb_ctx_make_draws(ctx, b, g->draws, s) != GB_LW_OK) le = cudaErrorLaunchFailure;
    if (le == cudaSuccess) le = gb_lw_launch_batch(b, ctx->d_tables, t.variant, t.blocks, s);
    e = cudaStreamEndCapture(s, &g->graph);
    if (le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    gb_rrtmg_lw_graph_destroy(g);
    return cuda_fail(ctx, e, "batch graph capture");
  }
  *out = g;
  return GB_LW_OK;
}

int gb_rrtmg_lw_graph_launch(gb_lw_graph* g, void* stream) {
  if (!g || !g->exec) return GB_LW_E_ARGS;
  gb_lw_context* ctx = g->ctx;
  cudaSetDevice(ctx->device);
  CK(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return GB_LW_OK;
}

int gb_rrtmg_lw_graph_destroy(gb_lw_graph* g) {
  if (!g) return GB_LW_OK;
  cudaSetDevice(g->ctx->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  cudaFree(g->gas);
  cudaFree(g->draws);
  cudaFree(g->fall);
  cudaFree(g->nfall);
  delete g;
  return GB_LW_OK;
}

const char* gb_rrtmg_lw_strerror(int code) {
  switch (code) {
    case GB_LW_OK: return "ok";
    case GB_LW_E_INFLAG1: return "INFLAG = 1 OPTION NOT AVAILABLE WITH MCICA";
    case GB_LW_E_ICE_SMALL: return "ICE RADIUS TOO SMALL";
    case GB_LW_E_ICE_BOUNDS: return "ICE RADIUS OUT OF BOUNDS";
    case GB_LW_E_DGE_BOUNDS: return "ICE GENERALIZED EFFECTIVE SIZE OUT OF BOUNDS";
    case GB_LW_E_LIQ_BOUNDS: return "LIQUID EFFECTIVE RADIUS OUT OF BOUNDS";
    case GB_LW_E_ICLD: return "MCICA_SUBCOL_LW: INVALID ICLD";
    case GB_LW_E_KISS_PMID: return "MCICA_SUBCOL: KISSVEC SEED GENERATOR REQUIRES PMID FROM BOTTOM FOUR LAYERS.";
    case GB_LW_E_LAYTROP: return "pressure must decrease with layer index";
    case GB_LW_E_BADVAL: return "non-positive or non-finite layer pressure or temperature";
    case GB_LW_E_TCWAIT: return "learned gas optics: a tensor-core wait ran out";
    case GB_LW_E_ARGS: return "invalid arguments";
    case GB_LW_E_CUDA: return "CUDA error";
    case GB_LW_E_TABLES: return "table files missing or malformed";
    case GB_LW_E_NOMEM: return "allocation failed";
    case GB_LW_E_SCRATCH: return "call exceeds the fixed scratch of gb_mcica_subcol_lw_noalloc (4,194,304 draws)";
  }
  return "unknown status";
}

const char* gb_rrtmg_lw_last_error(gb_lw_context* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

}  // extern "C"
