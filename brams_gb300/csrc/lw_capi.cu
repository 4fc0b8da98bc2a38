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
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gb_rrtmg_lw.h"
#include "lw_common.h"
#include "lw_mcica.h"
#include "lw_solver.h"
#include "lw_tables.h"

#include <dlfcn.h>

struct ChunkBufs {
  double* in = nullptr;   // all inputs of one chunk, packed
  double* out = nullptr;  // all outputs of one chunk, packed
  size_t in_elems = 0, out_elems = 0;
};

struct gb_lw_context {
  int device = 0;
  GbTables tabs;
  float* d_tables = nullptr;
  int* d_err = nullptr;      // max status of device calls
  int* d_err_host = nullptr; // status of the current host call
  cudaStream_t streams[2] = {nullptr, nullptr};
  ChunkBufs bufs[2];
  int chunk_cols = 0, chunk_nlay = 0;
  double* d_draws = nullptr;
  size_t draws_elems = 0;
  std::string last_error;
  size_t max_smem = 0;
};

namespace {

int cuda_fail(gb_lw_context* c, cudaError_t e, const char* where) {
  if (c) c->last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return GB_LW_E_CUDA;
}
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

bool flags_ok(int idrv, int inflglw, int iceflglw, int liqflglw) {
  return (idrv == 0 || idrv == 1) && inflglw >= 0 && inflglw <= 2 && iceflglw >= 0 && iceflglw <= 3 &&
         liqflglw >= 0 && liqflglw <= 1;
}

}  // namespace

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
  std::string ref = dir + "/lw_ref_tables.gblw", kt = dir + "/lw_ktables.gblw";
  std::vector<float> blob;
  std::string err;
  if (!gb_build_tables(ref.c_str(), kt.c_str(), cpdair, ctx->tabs, blob, err)) {
    std::fprintf(stderr, "gb_rrtmg_lw_ini: %s\n", err.c_str());
    delete ctx;
    return GB_LW_E_TABLES;
  }
  int dev_smem = 0;
  cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  ctx->max_smem = (size_t)dev_smem;
  if (cudaMalloc(&ctx->d_tables, blob.size() * 4) != cudaSuccess || cudaMalloc(&ctx->d_err, 8) != cudaSuccess) {
    cudaGetLastError();
    gb_rrtmg_lw_free(ctx);
    return GB_LW_E_NOMEM;
  }
  ctx->d_err_host = ctx->d_err + 1;
  if (cudaMemcpy(ctx->d_tables, blob.data(), blob.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(ctx->d_err, 0, 8) != cudaSuccess || gb_lw_set_tables(ctx->tabs) != cudaSuccess ||
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
  CK(gb_lw_launch(a, ctx->d_tables, (cudaStream_t)stream));
  return GB_LW_OK;
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
    CK(gb_lw_launch(a, ctx->d_tables, s));
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
  cudaSetDevice(ctx->device);
  const size_t n2 = (size_t)ncol * nlay, n3 = (size_t)ncol * (nlay + 1);
  const double* src2[] = {play, tlay, h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr, cfc11vmr, cfc12vmr, cfc22vmr, ccl4vmr};
  size_t total = 12 * n2 + 2 * n3 + ncol + 16 * (size_t)ncol + 16 * n2 + 6 * n3 + 2 * n2;
  double* d = nullptr;
  float* dt = nullptr;
  if (cudaMalloc(&d, total * 8) != cudaSuccess || cudaMalloc(&dt, 2 * n2 * GB_NGPT * 4) != cudaSuccess) {
    cudaFree(d);
    cudaGetLastError();
    return GB_LW_E_NOMEM;
  }
  double* p = d;
  double* dev2[12];
  for (int k = 0; k < 12; ++k) {
    dev2[k] = p;
    cudaMemcpy(p, src2[k], n2 * 8, cudaMemcpyHostToDevice);
    p += n2;
  }
  double* dplev = p; cudaMemcpy(p, plev, n3 * 8, cudaMemcpyHostToDevice); p += n3;
  double* dtlev = p; cudaMemcpy(p, tlev, n3 * 8, cudaMemcpyHostToDevice); p += n3;
  double* dtsfc = p; cudaMemcpy(p, tsfc, ncol * 8, cudaMemcpyHostToDevice); p += ncol;
  double* demis = p; cudaMemcpy(p, emis, 16 * (size_t)ncol * 8, cudaMemcpyHostToDevice); p += 16 * (size_t)ncol;
  double* dtau = p; cudaMemcpy(p, tauaer, 16 * n2 * 8, cudaMemcpyHostToDevice); p += 16 * n2;
  double* o = p;
  LwArgs a{};
  a.ncol = ncol; a.nlay = nlay; a.ld = ncol; a.ldo = ncol;
  a.icld = 0; a.idrv = 1; a.inflag = 2; a.iceflag = 3; a.liqflag = 1;
  a.play = dev2[0]; a.tlay = dev2[1]; a.h2ovmr = dev2[2]; a.o3vmr = dev2[3]; a.co2vmr = dev2[4];
  a.ch4vmr = dev2[5]; a.n2ovmr = dev2[6]; a.o2vmr = dev2[7]; a.cfc11vmr = dev2[8]; a.cfc12vmr = dev2[9];
  a.cfc22vmr = dev2[10]; a.ccl4vmr = dev2[11];
  a.plev = dplev; a.tlev = dtlev; a.tsfc = dtsfc; a.emis = demis; a.tauaer = dtau;
  a.uflx = o; a.dflx = o + n3; a.uflxc = o + 2 * n3; a.dflxc = o + 3 * n3; a.duflx_dt = o + 4 * n3;
  a.duflxc_dt = o + 5 * n3; a.hr = o + 6 * n3; a.hrc = o + 6 * n3 + n2;
  a.err_flag = ctx->d_err_host;
  a.dbg_taut = dt;
  a.dbg_fracs = dt + n2 * GB_NGPT;
  int rc = GB_LW_OK;
  cudaError_t e = gb_lw_launch(a, ctx->d_tables, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(taut, dt, n2 * GB_NGPT * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(fracs, dt + n2 * GB_NGPT, n2 * GB_NGPT * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = cuda_fail(ctx, e, "gas optics diagnostics");
  cudaFree(d);
  cudaFree(dt);
  return rc;
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
