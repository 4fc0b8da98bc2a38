/*
 * gb_rrtmg_lw.h -- C ABI of the GB300-native RRTMG_LW longwave column solver.
 *
 * Drop-in boundary for BRAMS's radiation driver: each entry point replaces
 * one routine of the reference (luflarois/brams, src/rrtmg/RRTMG_LW/src/)
 * and keeps its argument list, units and Fortran (column-major) layouts.
 * All reals are double precision as in the reference (kind_rb).  Arrays that
 * the reference declares (ncol, ...) take an explicit leading dimension
 * (ld_in / ld_out >= ncol), so callers can pass BRAMS's wider allocations
 * (e.g. outputs allocated (nofcols, nlay+2), rtm_driver.f90:913-922).
 *
 * Return value: 0 on success.  Positive values are the reference's STOP
 * conditions (GB_LW_E_*), reported instead of stopping the process;
 * negative values are argument, memory or CUDA errors.
 *
 * Threading: a context may be used by one host thread at a time, and its
 * calls share the context's device scratch (taumol hand-over planes, McICA
 * draws, the shortwave kernel's slot records, grown on demand), so the
 * *_device calls of one context must not overlap on the device: issue them
 * on one stream, or order the streams (events).  Separate contexts run
 * concurrently.
 */
#ifndef GB_RRTMG_LW_H
#define GB_RRTMG_LW_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_lw_context gb_lw_context;

/* status codes */
#define GB_LW_OK 0
#define GB_LW_E_INFLAG1 2      /* cldprmc: 'INFLAG = 1 OPTION NOT AVAILABLE WITH MCICA'   */
#define GB_LW_E_ICE_SMALL 3    /* cldprmc/cldprop: 'ICE RADIUS TOO SMALL'               */
#define GB_LW_E_ICE_BOUNDS 4   /* cldprmc/cldprop: 'ICE RADIUS OUT OF BOUNDS'           */
#define GB_LW_E_DGE_BOUNDS 5   /* cldprmc/cldprop: 'ICE GENERALIZED EFFECTIVE SIZE ...'  */
#define GB_LW_E_LIQ_BOUNDS 6   /* cldprmc/cldprop: 'LIQUID EFFECTIVE RADIUS OUT OF BOUNDS' */
#define GB_LW_E_ICLD 7         /* mcica_subcol_lw: 'INVALID ICLD'                        */
#define GB_LW_E_KISS_PMID 8    /* generate_stochastic_clouds: KISS seed needs pmid(1) >= pmid(2) */
#define GB_LW_E_LAYTROP 9      /* pressure does not decrease with layer index            */
#define GB_LW_E_BADVAL 11      /* non-positive or non-finite layer pressure/temperature  */
#define GB_LW_E_TCWAIT 12      /* learned gas optics: a tensor-core wait ran out          */
#define GB_LW_E_SW_OPTICS 13   /* cldprmc_sw: cloud optics out of range (the reference's other STOPs) */
#define GB_LW_E_SW_UNSUPPORTED 14 /* option the SW path does not implement (see gb_rrtmg_sw)  */
#define GB_LW_E_ARGS (-1)      /* invalid sizes, flags or null pointers                  */
#define GB_LW_E_CUDA (-2)      /* CUDA runtime error (see gb_rrtmg_lw_last_error)        */
#define GB_LW_E_TABLES (-3)    /* table files missing or malformed, or unlike another live context's on the device */
#define GB_LW_E_NOMEM (-4)     /* device or pinned-host allocation failed                */
#define GB_LW_E_SCRATCH (-5)   /* call too large for the fixed scratch of gb_mcica_subcol_lw_noalloc */

/* Replaces rrtmg_lw_ini(cpdair) (rrtmg_lw_init.f90:47; called from
 * mem_rrtm.f90:114).  Loads the tables from table_dir (NULL: the directory
 * installed next to this library) onto CUDA device `device` and returns a
 * context.  cpdair is the specific heat of dry air used in heatfac
 * (BRAMS: cp = 1004.).  The kernels keep part of the tables in constant
 * memory, one copy per device: every live context of a device must be made
 * from the same table files and cpdair (the reference, too, holds one set of
 * tables per process).  A context whose tables differ from those of a live
 * context on its device is refused with GB_LW_E_TABLES; once the last such
 * context is freed, the device takes the next context's tables. */
int gb_rrtmg_lw_ini(double cpdair, const char* table_dir, int device, gb_lw_context** ctx);

/* Releases all device memory, streams and events of the context. */
int gb_rrtmg_lw_free(gb_lw_context* ctx);

/* Replaces rrtmg_lw (rrtmg_lw_rad.f90:99-108, called at rtm_driver.f90:1313)
 * for HOST arrays.  icld is in/out as in the reference (values outside 0..3
 * become 2).  Layout (ld = ld_in for inputs, ld_out for outputs):
 *   play tlay h2ovmr o3vmr co2vmr ch4vmr n2ovmr o2vmr cfc11vmr cfc12vmr
 *   cfc22vmr ccl4vmr reicmcl relqmcl             (ld, nlay)
 *   plev tlev                                     (ld, nlay+1)
 *   tsfc (ncol), emis (ld, 16), tauaer (ld, nlay, 16)
 *   cldfmcl taucmcl ciwpmcl clwpmcl               (140, ld, nlay)
 *   uflx dflx uflxc dflxc duflx_dt duflxc_dt      (ld_out, nlay+1)
 *   hr hrc                                        (ld_out, nlay)
 * duflx_dt / duflxc_dt are written only when idrv == 1 (may be NULL
 * otherwise); the McICA arrays may be NULL when icld == 0.  Columns are
 * streamed to the GPU in chunks; page-locked host buffers are copied by DMA
 * while earlier chunks compute. */
int gb_rrtmg_lw(gb_lw_context* ctx, int ncol, int nlay, int* icld, int idrv,
                const double* play, const double* plev, const double* tlay, const double* tlev,
                const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
                const double* cldfmcl, const double* taucmcl, const double* ciwpmcl,
                const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                const double* tauaer, double* uflx, double* dflx, double* hr, double* uflxc,
                double* dflxc, double* hrc, double* duflx_dt, double* duflxc_dt,
                int64_t ld_in, int64_t ld_out);

/* Same computation on DEVICE arrays, enqueued on `stream` (a cudaStream_t,
 * NULL for the default stream) without host synchronisation.  Per-column
 * status codes go to d_col_status (device, ncol ints) when not NULL; the
 * maximum status of all calls since the last gb_rrtmg_lw_sync_status is
 * kept on the device. */
int gb_rrtmg_lw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int* icld, int idrv,
                       const double* play, const double* plev, const double* tlay,
                       const double* tlev, const double* tsfc, const double* h2ovmr,
                       const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                       const double* n2ovmr, const double* o2vmr, const double* cfc11vmr,
                       const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
                       const double* emis, int inflglw, int iceflglw, int liqflglw,
                       const double* cldfmcl, const double* taucmcl, const double* ciwpmcl,
                       const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                       const double* tauaer, double* uflx, double* dflx, double* hr,
                       double* uflxc, double* dflxc, double* hrc, double* duflx_dt,
                       double* duflxc_dt, int64_t ld_in, int64_t ld_out, int* d_col_status);

/* Replaces rrtmg_lw of the non-McICA build (rrtmg_lw_rad.nomcica.f90:99-108)
 * for HOST arrays: the state arguments of gb_rrtmg_lw, then band-level
 * clouds as that driver takes them: cldfr cicewp cliqwp reice reliq (ld,
 * nlay) and taucld (16, ld, nlay; read for inflglw 0, summed by cldprop's
 * cloud test otherwise).  Per column it runs cldprop
 * (rrtmg_lw_cldprop.f90:50-295), setcoef, taumol and the transfer with the
 * driver's overlap choice (:546-560): icld 1 random overlap (rtrn,
 * rrtmg_lw_rtrn.f90), 2 and 3 maximum/random overlap (rtrnmr,
 * rrtmg_lw_rtrnmr.f90), 0 clear sky; values outside 0..3 become 2 (:456).
 * The cloud arrays may be NULL when icld == 0. */
int gb_rrtmg_lw_nomcica(gb_lw_context* ctx, int ncol, int nlay, int* icld, int idrv,
                        const double* play, const double* plev, const double* tlay, const double* tlev,
                        const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                        const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                        const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                        const double* ccl4vmr, const double* emis, int inflglw, int iceflglw, int liqflglw,
                        const double* cldfr, const double* taucld, const double* cicewp, const double* cliqwp,
                        const double* reice, const double* reliq, const double* tauaer, double* uflx,
                        double* dflx, double* hr, double* uflxc, double* dflxc, double* hrc,
                        double* duflx_dt, double* duflxc_dt, int64_t ld_in, int64_t ld_out);

/* Same on DEVICE arrays on `stream`, with the status handling of
 * gb_rrtmg_lw_device (cldprop's radius stops included in d_col_status). */
int gb_rrtmg_lw_nomcica_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int* icld, int idrv,
                               const double* play, const double* plev, const double* tlay,
                               const double* tlev, const double* tsfc, const double* h2ovmr,
                               const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                               const double* n2ovmr, const double* o2vmr, const double* cfc11vmr,
                               const double* cfc12vmr, const double* cfc22vmr, const double* ccl4vmr,
                               const double* emis, int inflglw, int iceflglw, int liqflglw,
                               const double* cldfr, const double* taucld, const double* cicewp,
                               const double* cliqwp, const double* reice, const double* reliq,
                               const double* tauaer, double* uflx, double* dflx, double* hr,
                               double* uflxc, double* dflxc, double* hrc, double* duflx_dt,
                               double* duflxc_dt, int64_t ld_in, int64_t ld_out, int* d_col_status);

/* Waits for `stream` and returns (then clears) the maximum column status of
 * the device calls made since the previous call. */
int gb_rrtmg_lw_sync_status(gb_lw_context* ctx, void* stream);

/* Replaces mcica_subcol_lw (mcica_subcol_gen_lw.f90:183-185, called at
 * rtm_driver.f90:1262) for HOST arrays.  icld 0..5, irng 0 (KISS) or 1
 * (Mersenne twister); draws are bit-identical to the reference's.
 *   play cldfrac ciwp clwp rei rel alpha          (ld, nlay)
 *   tauc                                          (16, ld, nlay)
 *   cldfmcl ciwpmcl clwpmcl taucmcl               (140, ld, nlay)
 *   reicmcl relqmcl                               (ld, nlay)
 * seed_per_column = 0 reproduces one reference call over all columns
 * (seed = permuteseed); 1 reproduces one reference call per column with
 * seed = permuteseed + (column index, 0-based).  alpha may be NULL unless
 * icld is 4 or 5. */
int gb_mcica_subcol_lw(gb_lw_context* ctx, int ncol, int nlay, int icld, int permuteseed,
                       int* irng, const double* play, const double* cldfrac, const double* ciwp,
                       const double* clwp, const double* rei, const double* rel,
                       const double* tauc, const double* alpha, double* cldfmcl,
                       double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl,
                       double* taucmcl, int64_t ld, int seed_per_column);

/* Same on DEVICE arrays, enqueued on `stream`. */
int gb_mcica_subcol_lw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int icld,
                              int permuteseed, int* irng, const double* play,
                              const double* cldfrac, const double* ciwp, const double* clwp,
                              const double* rei, const double* rel, const double* tauc,
                              const double* alpha, double* cldfmcl, double* ciwpmcl,
                              double* clwpmcl, double* reicmcl, double* relqmcl,
                              double* taucmcl, int64_t ld, int seed_per_column);

/* cldprop (rrtmg_lw_cldprop.f90:50-295) on DEVICE arrays for ncol columns, as
 * BRAMS calls it per column before McICA (rtm_driver.f90:1250-1258):
 * cldfrac, ciwp, clwp, rei, rel are (ld, nlay); tauc (16, ld, nlay) is the
 * reference's input tauc (required for inflag 0, may be NULL otherwise);
 * taucloud (16, ld, nlay) receives the band cloud optical depths in the
 * layout mcica_subcol_lw and the fused-cloud solver take (bands a layer does
 * not fill are 0).  fp64 throughout, like the reference.  A radius outside
 * the bounds the reference STOPs on sets d_col_status (may be NULL) to the
 * largest such code of the column and the context's status; the offending
 * layer's output is 0. */
int gb_cldprop_lw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int inflag, int iceflag,
                         int liqflag, const double* cldfrac, const double* tauc, const double* ciwp,
                         const double* clwp, const double* rei, const double* rel, double* taucloud,
                         int64_t ld, int* d_col_status);

/* BRAMS's column packing for rrtmg_lw on DEVICE arrays: the statements of
 * radrrtmdrv (rtm_driver.f90:978-1076, 1176-1231) that turn the model state
 * of the subdomain i = ia..iz, j = ja..jz (1-based, columns j outer and i
 * inner) into the solver's inputs.  Model fields are BRAMS's default-real
 * (float) arrays: pi0, pp, theta, rv, cldf, lwl, iwl, rel, rei are
 * (mzp, mxp, myp); rlongup, albedt are (mxp, myp).  Outputs are the
 * rrtmg_lw arrays with leading dimension ld >= ncol and nlay = mzp - 1
 * layers: play, tlay, h2ovmr, the fixed gases, cldfrac, ciwp, clwp, reic
 * (clamped as the driver does for iceflgsw 1-3), relq (ld, nlay); plev,
 * tlev (ld, nlay+1); tsfc (ld); emis (ld, 16), 0 when firsttime is nonzero
 * as on the driver's first call.  Float operations round as the driver's
 * default-real statements do before they meet real(8) values.  o3vmr and
 * tauaer are not written (ozone climatology and CARMA stay with the
 * caller). */
int gb_rtm_pack_lw_device(gb_lw_context* ctx, void* stream, int mzp, int mxp, int myp, int ia, int iz, int ja, int jz,
                          int iceflgsw, int firsttime, const float* pi0, const float* pp, const float* theta,
                          const float* rv, const float* rlongup, const float* albedt, const float* cldf,
                          const float* lwl, const float* iwl, const float* rel, const float* rei, double* play,
                          double* plev, double* tlay, double* tlev, double* tsfc, double* h2ovmr, double* co2vmr,
                          double* ch4vmr, double* n2ovmr, double* o2vmr, double* cfc11vmr, double* cfc12vmr,
                          double* cfc22vmr, double* ccl4vmr, double* emis, double* cldfrac, double* ciwp,
                          double* clwp, double* reic, double* relq, int64_t ld);

/* BRAMS's zonal ozone climatology for the packed columns, on HOST arrays
 * (rtm_driver.f90:1120-1173 with InitGetoz_rrtm :2062-2636 and getoz_rrtm
 * :2638-2823): from each column's interface pressures plev (ld, mzp) (the
 * rrtmg_lw plev, mzp = nlay + 1 levels), its grid latitude glat (degrees,
 * BRAMS's float field) and the day of the year, o3vmr (ld_out, mzp - 1) in
 * the driver's layer order, as the driver forms it without chemistry ozone.
 * gb_rtm_ozone_load reads the climatology (brams_ozone.gblw) from
 * table_dir. */
typedef struct gb_rtm_ozone gb_rtm_ozone;
int gb_rtm_ozone_load(const char* table_dir, gb_rtm_ozone** out);
int gb_rtm_ozone_free(gb_rtm_ozone* oz);
int gb_rtm_ozone_lw(const gb_rtm_ozone* oz, int ncol, int mzp, const double* plev, int64_t ld, const float* glat,
                    int doy, double* o3vmr, int64_t ld_out);

/* The driver's write-back (rtm_driver.f90:1443-1456) on DEVICE arrays:
 * fthrd(k, i, j) = (swhr + hr)(column, k-1) / 86400 for k = 2..mzp-1, copied
 * to k = 1 and k = mzp, and rlong(i, j) = dflx(column, 1), into BRAMS's float
 * fields fthrd (mzp, mxp, myp) and rlong (mxp, myp).  hr (and swhr, NULL for
 * none) have leading dimension ld_hr, dflx ld_flx. */
int gb_rtm_unpack_lw_device(gb_lw_context* ctx, void* stream, int mzp, int mxp, int myp, int ia, int iz, int ja,
                            int jz, const double* hr, const double* swhr, const double* dflx, int64_t ld_hr,
                            int64_t ld_flx, float* fthrd, float* rlong);

/* The shortwave-only parts of the same packing and write-back on DEVICE
 * arrays: coszen(column) = cosz(i, j) and the four albedos asdir asdif aldir
 * aldif = albedt(i, j), 0 when firsttime is nonzero (rtm_driver.f90:989,
 * 992-996), all (ncol) with the columns in the packing order; and
 * rshort(i, j) = swdflx(column, 1), 0 where that flux is below 0.5 W m-2
 * (:1448-1449).  cosz, albedt and rshort are BRAMS's float fields
 * (mxp, myp); swdflx is the first level of rrtmg_sw's output (its first
 * ncol values). */
int gb_rtm_pack_sw_device(gb_lw_context* ctx, void* stream, int mxp, int myp, int ia, int iz, int ja, int jz,
                          int firsttime, const float* cosz, const float* albedt, double* coszen, double* asdir,
                          double* asdif, double* aldir, double* aldif);
int gb_rtm_unpack_sw_device(gb_lw_context* ctx, void* stream, int mxp, int myp, int ia, int iz, int ja, int jz,
                            const double* swdflx, float* rshort);

/* Diagnostics (no counterpart in the reference's interface): runs the same
 * column kernel on host arrays (tight layout, ld = ncol) and also returns
 * the gas-plus-aerosol optical depth taut and the Planck fraction of every
 * (column, layer, g-point) in single precision, g fastest:
 * taut[(icol*nlay + lay)*140 + g].  Used to check taumol band by band. */
int gb_rrtmg_lw_gas_optics_diag(gb_lw_context* ctx, int ncol, int nlay, const double* play,
                                const double* plev, const double* tlay, const double* tlev,
                                const double* tsfc, const double* h2ovmr, const double* o3vmr,
                                const double* co2vmr, const double* ch4vmr, const double* n2ovmr,
                                const double* o2vmr, const double* cfc11vmr,
                                const double* cfc12vmr, const double* cfc22vmr,
                                const double* ccl4vmr, const double* emis, const double* tauaer,
                                float* taut, float* fracs);

/* Allocation-free variant of gb_mcica_subcol_lw_device.  It has no
 * counterpart in the reference: it exists for callers that cannot allocate
 * device memory during a run -- models whose device memory belongs to
 * another runtime (OpenACC / OpenMP-offload data regions, pooled allocators)
 * and time-stepping codes that cannot take the device-wide synchronisation
 * that cudaMalloc/cudaFree may cause.  The caller passes device inputs and
 * outputs as for gb_mcica_subcol_lw_device; no context is needed.  Draws go
 * to a fixed array inside the library of 4 Mi doubles (32 MiB, held by every
 * GPU that loads the library until exit), so
 *   140 * ncol          (icld 3)
 *   140 * ncol * nlay   (icld 1, 2)
 *   280 * ncol * nlay   (icld 4, 5)
 * must not exceed 4,194,304; larger calls return GB_LW_E_SCRATCH.  The first
 * call on a device looks up the array's device address (once per device,
 * with that device current); make that first call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race,
 * so order them (one stream, or events).  The reference's STOP status of the
 * call (e.g. GB_LW_E_KISS_PMID) is copied to d_status (device int) when not
 * NULL.  Enqueued on `stream` without host synchronisation. */
int gb_mcica_subcol_lw_noalloc(void* stream, int ncol, int nlay, int icld, int permuteseed,
                               int* irng, const double* play, const double* cldfrac,
                               const double* ciwp, const double* clwp, const double* rei,
                               const double* rel, const double* tauc, const double* alpha,
                               double* cldfmcl, double* ciwpmcl, double* clwpmcl,
                               double* reicmcl, double* relqmcl, double* taucmcl, int64_t ld,
                               int seed_per_column, int* d_status);

/* ---------------------------------------------------------------------------
 * Batched calls (no counterpart in the reference, which BRAMS calls once per
 * grid and MPI rank, rtm_driver.f90:1313): several grids -- nested grids,
 * ensemble members -- with their own column and layer counts are solved in
 * ONE persistent kernel launch.  Each grid is described by device arrays in
 * the layouts of gb_rrtmg_lw_device.
 *
 * cloud_mode GB_LW_CLOUD_SUBCOL: McICA sub-column arrays as for
 *   gb_rrtmg_lw_device (cldfmcl, taucmcl, ciwpmcl, clwpmcl, reicmcl,
 *   relqmcl).
 * cloud_mode GB_LW_CLOUD_FUSED: the kernel generates the sub-columns itself
 *   from layer clouds, exactly as gb_mcica_subcol_lw with icld 3, irng 1 and
 *   seed_per_column 1 (column c seeded seed0 + c) followed by rrtmg_lw would:
 *   cldfrac ciwp clwp (ld, nlay), tauc (16, ld, nlay), and reicmcl/relqmcl
 *   carry the layer radii rei/rel (ld, nlay).  Requires icld 0 or 3.  The
 *   (140, ncol, nlay) arrays are never formed.
 */
#define GB_LW_CLOUD_SUBCOL 0
#define GB_LW_CLOUD_FUSED 1
#define GB_LW_MAX_GRIDS 32
#define GB_LW_NGPT 140 /* g-points (parrrtm.f90 ngptlw) */

typedef struct gb_lw_grid {
  int ncol, nlay, icld, idrv, inflglw, iceflglw, liqflglw;
  int cloud_mode;
  uint32_t seed0;
  int64_t ld_in, ld_out;
  const double *play, *plev, *tlay, *tlev, *tsfc, *h2ovmr, *o3vmr, *co2vmr, *ch4vmr, *n2ovmr,
      *o2vmr, *cfc11vmr, *cfc12vmr, *cfc22vmr, *ccl4vmr, *emis, *tauaer;
  const double *cldfmcl, *taucmcl, *ciwpmcl, *clwpmcl;   /* GB_LW_CLOUD_SUBCOL */
  const double *cldfrac, *ciwp, *clwp, *tauc;            /* GB_LW_CLOUD_FUSED  */
  const double *reicmcl, *relqmcl;
  double *uflx, *dflx, *hr, *uflxc, *dflxc, *hrc, *duflx_dt, *duflxc_dt;
  int* d_col_status; /* optional, ncol ints */
  /* optional learned gas optics (gb_lw_mlp_infer): taug and Planck fractions
   * [(icol*nlay + lay)*140 + g] as IEEE binary16 bit patterns and a per-layer
   * flag [icol*nlay + lay]; layers whose flag is 0 (inputs outside the
   * network's training range) use taumol.  NULL: taumol everywhere. */
  const uint16_t *sur_tau, *sur_frac;
  const uint8_t* sur_flag;
} gb_lw_grid;

/* Launch shape of the batched kernel: compiled variant (threads per column
 * block, register budget) and resident blocks per SM of the persistent grid. */
typedef struct gb_lw_tuning {
  int variant, threads, min_blocks, blocks_per_sm, blocks;
  double ms; /* measured time of the tuned shape on the sample batch (autotune only) */
} gb_lw_tuning;

/* All grids in one launch on `stream` (ngrid <= GB_LW_MAX_GRIDS), with the
 * shape the context's autotuner chose for this batch (largest nlay), or the
 * default shape.  Same status handling as gb_rrtmg_lw_device. */
int gb_rrtmg_lw_batch_device(gb_lw_context* ctx, void* stream, int ngrid, const gb_lw_grid* grids);

/* Times every compiled variant and persistent-grid size on a sample of the
 * batch (each grid cut to the same fraction of its columns, about
 * sample_cols columns in all; <= 0 for the whole batch), `reps` launches
 * each after a warm-up, keeps the fastest for batches of this largest
 * nlay and kind (GB_LW_KIND_*) and returns it in *best.  Overwrites the
 * outputs of the sampled columns. */
int gb_rrtmg_lw_autotune(gb_lw_context* ctx, void* stream, int ngrid, const gb_lw_grid* grids,
                         int sample_cols, int reps, gb_lw_tuning* best);

/* Every candidate of the last gb_rrtmg_lw_autotune call with its time (up to
 * max into out); returns the number of candidates. */
int gb_rrtmg_lw_autotune_report(gb_lw_context* ctx, gb_lw_tuning* out, int max);

/* Shapes are kept per largest layer count and batch kind: GB_LW_KIND_FUSED
 * if any grid generates its McICA clouds in the kernel, | GB_LW_KIND_LEARNED
 * if any grid uses learned gas optics.  _get returns the shape
 * gb_rrtmg_lw_batch_device would use (tuned, pinned or the default); _set
 * pins one (variant and blocks_per_sm are used, the rest is derived).  For
 * the GB_LW_KIND_LEARNED kinds the variant is one of the learned-only
 * kernel's shapes (that kernel solves the columns wholly on the network; the
 * full kernel, in a second launch, the rest). */
#define GB_LW_KIND_FUSED 1
#define GB_LW_KIND_LEARNED 2
int gb_rrtmg_lw_tuning_get(gb_lw_context* ctx, int nlay, int kind, gb_lw_tuning* out);
int gb_rrtmg_lw_tuning_set(gb_lw_context* ctx, int nlay, int kind, const gb_lw_tuning* shape);
/* Number of compiled kernel variants (valid gb_lw_tuning.variant values). */
int gb_rrtmg_lw_num_variants(void);

/* CUDA graph of one batched launch: the descriptor and the gas-optics
 * hand-over buffer owned by the graph are fixed at creation, so the caller
 * updates the input arrays in place between replays (a time-stepping model's
 * resident state).  The graph holds the batch's kernels (one persistent
 * launch for taumol batches). */
typedef struct gb_lw_graph gb_lw_graph;
int gb_rrtmg_lw_batch_graph_create(gb_lw_context* ctx, int ngrid, const gb_lw_grid* grids,
                                   gb_lw_graph** graph);
int gb_rrtmg_lw_graph_launch(gb_lw_graph* graph, void* stream);
int gb_rrtmg_lw_graph_destroy(gb_lw_graph* graph);

/* ---------------------------------------------------------------------------
 * RRTMG_SW, the shortwave scheme BRAMS calls right after the longwave one
 * (rtm_driver.f90:1386).  gb_rrtmg_sw_ini replaces rrtmg_sw_ini
 * (rrtmg_sw_init.f90:47): it loads sw_tables.gbsw (the reference's
 * k-distribution data reduced to 112 g-points) of table_dir (NULL: the
 * context's table directory) into the context.  gb_rrtmg_sw replaces
 * rrtmg_sw (rrtmg_sw_rad.f90:243-255) with its argument order: layer arrays
 * (ld, nlay), plev/tlev (ld, nlay+1), tsfc and the albedos and coszen (ncol),
 * McICA arrays cldfmcl taucmcl ssacmcl asmcmcl fsfcmcl ciwpmcl clwpmcl
 * (112, ld, nlay) and reicmcl relqmcl (ld, nlay), aerosols tauaer ssaaer
 * asmaer (ld, nlay, 14); outputs swuflx swdflx swuflxc swdflxc (ld_out,
 * nlay+1), swhr swhrc (ld_out, nlay).  icld and iaer are in/out as in the
 * reference.  The solar-variability option isolvar must be negative (BRAMS
 * passes -1) and iaer 0 or 10 (ecaer, for iaer 6, is not read); cloud
 * options inflag 0 or 2 with iceflag 1-3 and liqflag 1 (the reference
 * leaves the coefficients of ice option 0 and liquid option 0 unset).  The
 * arithmetic is the context's shortwave precision (gb_rrtmg_sw_set_precision:
 * fp32 solution with fp64 sums by default, or fp64 throughout).  As in
 * gb_rrtmg_lw_ini, the live contexts of a device must load the same
 * shortwave tables and cpdair: otherwise GB_LW_E_TABLES, and the context is
 * left without shortwave tables.  tlev, tsfc
 * and n2ovmr are not used by the reference's
 * shortwave computation and may be NULL. */
int gb_rrtmg_sw_ini(gb_lw_context* ctx, double cpdair, const char* table_dir);
/* Precision of the shortwave column kernel of this context: 32 (the
 * default) runs the gas optics, cloud optics and two-stream solution in fp32
 * and keeps fp64 for the layer coefficients, the flux accumulation over
 * g-points and the heating rates (fluxes within 0.05 W m-2 and heating rates
 * within 0.01 K/day of the fp64 reference); 64 runs everything in fp64, as
 * the reference does.  Returns GB_LW_E_ARGS for any other value.  No
 * reference counterpart: the reference's precision is fixed at build time. */
int gb_rrtmg_sw_set_precision(gb_lw_context* ctx, int bits);
int gb_rrtmg_sw(gb_lw_context* ctx, int ncol, int nlay, int* icld, int* iaer, const double* play,
                const double* plev, const double* tlay, const double* tlev, const double* tsfc,
                const double* h2ovmr, const double* o3vmr, const double* co2vmr, const double* ch4vmr,
                const double* n2ovmr, const double* o2vmr, const double* asdir, const double* asdif,
                const double* aldir, const double* aldif, const double* coszen, double adjes, int dyofyr,
                double scon, int isolvar, int inflgsw, int iceflgsw, int liqflgsw, const double* cldfmcl,
                const double* taucmcl, const double* ssacmcl, const double* asmcmcl, const double* fsfcmcl,
                const double* ciwpmcl, const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                const double* tauaer, const double* ssaaer, const double* asmaer, const double* ecaer,
                double* swuflx, double* swdflx, double* swhr, double* swuflxc, double* swdflxc, double* swhrc,
                int64_t ld_in, int64_t ld_out);
/* Same on DEVICE arrays on `stream`, with the status handling of
 * gb_rrtmg_lw_device. */
int gb_rrtmg_sw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int* icld, int* iaer,
                       const double* play, const double* plev, const double* tlay, const double* tlev,
                       const double* tsfc, const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                       const double* ch4vmr, const double* n2ovmr, const double* o2vmr, const double* asdir,
                       const double* asdif, const double* aldir, const double* aldif, const double* coszen,
                       double adjes, int dyofyr, double scon, int isolvar, int inflgsw, int iceflgsw, int liqflgsw,
                       const double* cldfmcl, const double* taucmcl, const double* ssacmcl, const double* asmcmcl,
                       const double* fsfcmcl, const double* ciwpmcl, const double* clwpmcl, const double* reicmcl,
                       const double* relqmcl, const double* tauaer, const double* ssaaer, const double* asmaer,
                       const double* ecaer, double* swuflx, double* swdflx, double* swhr, double* swuflxc,
                       double* swdflxc, double* swhrc, int64_t ld_in, int64_t ld_out, int* d_col_status);

/* Replaces mcica_subcol_sw (mcica_subcol_gen_sw.f90:181-296, called at
 * rtm_driver.f90:1373) for HOST arrays: as gb_mcica_subcol_lw with 112
 * sub-columns, band optical properties tauc ssac asmc fsfc (14, ld, nlay)
 * and the McICA outputs cldfmcl ciwpmcl clwpmcl taucmcl ssacmcl asmcmcl
 * fsfcmcl (112, ld, nlay), reicmcl relqmcl (ld, nlay).  Draws are bit-equal
 * to the reference's for icld 1-5, both generators and both seeding modes. */
int gb_mcica_subcol_sw(gb_lw_context* ctx, int ncol, int nlay, int icld, int permuteseed, int* irng,
                       const double* play, const double* cldfrac, const double* ciwp, const double* clwp,
                       const double* rei, const double* rel, const double* tauc, const double* ssac,
                       const double* asmc, const double* fsfc, const double* alpha, double* cldfmcl,
                       double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl, double* taucmcl,
                       double* ssacmcl, double* asmcmcl, double* fsfcmcl, int64_t ld, int seed_per_column);
/* Same on DEVICE arrays on `stream`. */
int gb_mcica_subcol_sw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int icld, int permuteseed,
                              int* irng, const double* play, const double* cldfrac, const double* ciwp,
                              const double* clwp, const double* rei, const double* rel, const double* tauc,
                              const double* ssac, const double* asmc, const double* fsfc, const double* alpha,
                              double* cldfmcl, double* ciwpmcl, double* clwpmcl, double* reicmcl, double* relqmcl,
                              double* taucmcl, double* ssacmcl, double* asmcmcl, double* fsfcmcl, int64_t ld,
                              int seed_per_column);
/* cldprop_sw (rrtmg_sw_cldprop.f90:53-365) on DEVICE arrays for ncol
 * columns, as BRAMS calls it per column before mcica_subcol_sw
 * (rtm_driver.f90:1356-1368): cldfrac, ciwp, clwp, rei, rel are (ld, nlay);
 * tauc, ssac, asmc, fsfc (14, ld, nlay) are the reference's inflag-0 inputs
 * (required for inflag 0; otherwise NULL reads as zeros, which the driver
 * passes).  Outputs, (14, ld, nlay) with the band fastest -- the layout
 * gb_mcica_subcol_sw takes as tauc ssac asmc: taucloud (delta-scaled),
 * ssacloud, asmcloud (delta-scaled) and taucldorig (may be NULL); a clear
 * layer gets 0, 1, 0 and the input tauc.  fp64 with the reference's
 * operations.  A layer the reference STOPs on keeps the clear values and
 * sets d_col_status (may be NULL) to the code of that STOP (radius bounds,
 * GB_LW_E_SW_OPTICS, GB_LW_E_SW_UNSUPPORTED for ice option 0 or liquid
 * option 0 with a nonzero path), and the context's status.  Needs the
 * shortwave tables (gb_rrtmg_sw_ini). */
int gb_cldprop_sw_device(gb_lw_context* ctx, void* stream, int ncol, int nlay, int inflag, int iceflag, int liqflag,
                         const double* cldfrac, const double* tauc, const double* ssac, const double* asmc,
                         const double* fsfc, const double* ciwp, const double* clwp, const double* rei,
                         const double* rel, double* taucloud, double* ssacloud, double* asmcloud, double* taucldorig,
                         int64_t ld, int* d_col_status);

/* ---------------------------------------------------------------------------
 * Multi-GPU column shards (host only; no device call).  BRAMS gives each MPI
 * rank the columns of its own subdomain (rtm_driver.f90:830, nofcols) and
 * each rank calls rrtmg_lw on those; the ranks exchange nothing.  A caller
 * that drives several GPUs from one batch lays the batch's grids end to end
 * and gives rank r the contiguous run of columns whose cumulative work
 * (columns x layers) lies in [r/nranks, (r+1)/nranks) of the total:
 * gb_rrtmg_lw_shard_plan returns that run as per-grid column ranges
 * [c0[i], c1[i]) (empty where c0 == c1), and gb_rrtmg_lw_grid_slice cuts a
 * grid descriptor to columns [c0, c1) by pointer offsets (leading dimensions
 * kept, seed0 advanced by c0 so that McICA draws do not depend on the
 * split).  Each rank passes its non-empty slices to gb_rrtmg_lw_batch_device
 * on its own device; the outputs land in place. */
int gb_rrtmg_lw_shard_plan(int ngrid, const int* ncol, const int* nlay, int nranks, int rank, int64_t* c0,
                           int64_t* c1);
int gb_rrtmg_lw_grid_slice(const gb_lw_grid* grid, int64_t c0, int64_t c1, gb_lw_grid* out);

/* ---------------------------------------------------------------------------
 * Learned gas optics (no counterpart in the reference): a small MLP that maps
 * per-layer state to the 140 g-point gas optical depths and Planck fractions
 * that taumol (rrtmg_lw_taumol.f90) computes, used in place of taumol for
 * layers inside its training range and trained on this library's own taumol.
 *   features (9 per layer): log p, T, log column H2O, O3, CO2, CH4, N2O
 *     (molecules cm-2 * 1e-20, as setcoef forms them), log layer pressure
 *     thickness, temperature of the layer's lower boundary level;
 *   network: 9 -> 128 -> 128 -> 128 -> 280, SiLU, bf16 weights and
 *     activations, fp32 accumulation on the tensor cores;
 *   outputs: standardised log taug (140) and Planck fractions (140).
 * Device arrays are row-major; "rows" index (column, layer) pairs as
 * icol*nlay + lay.  Parameters are exchanged as GB_LW_MLP_NPARAM floats
 * (W1[16][128] b1 W2[128][128] b2 W3[128][128] b3 W4[128][288] b4), the
 * normalisation as GB_LW_MLP_NNORM floats (in_mu[16] in_sd[16] in_lo[9]
 * in_hi[9] out_mu[288] out_sd[288]). */
#define GB_LW_MLP_NPARAM 72352
#define GB_LW_MLP_NNORM 626
typedef struct gb_lw_mlp gb_lw_mlp;

/* New network with seeded random weights on the context's device. */
int gb_lw_mlp_create(gb_lw_context* ctx, uint64_t seed, gb_lw_mlp** mlp);
int gb_lw_mlp_destroy(gb_lw_mlp* mlp);
int gb_lw_mlp_save(gb_lw_mlp* mlp, const char* path);
int gb_lw_mlp_load(gb_lw_context* ctx, const char* path, gb_lw_mlp** mlp);
/* Host copies of the fp32 parameters / normalisation (either may be NULL). */
int gb_lw_mlp_get_params(gb_lw_mlp* mlp, float* params, float* norm);
int gb_lw_mlp_set_params(gb_lw_mlp* mlp, const float* params, const float* norm);
/* Inference engine of gb_lw_mlp_infer: GB_LW_MLP_TCGEN05 (default; tcgen05
 * MMAs with tensor-memory accumulators) or GB_LW_MLP_MMA_SYNC (warp-level
 * mma.sync, the network's reference GPU implementation). */
#define GB_LW_MLP_MMA_SYNC 0
#define GB_LW_MLP_TCGEN05 1
int gb_lw_mlp_set_engine(gb_lw_mlp* mlp, int engine);
/* Weight of each of the 280 outputs in the training loss (default 1). */
int gb_lw_mlp_set_loss_weights(gb_lw_mlp* mlp, const float* w280);

/* Training samples from the plain taumol of one grid (device arrays as in
 * gb_lw_grid; the grid's flux outputs are overwritten): raw features
 * d_feat[rows][9], taug d_tau[rows][140] and Planck fractions
 * d_frac[rows][140], rows = ncol*nlay. */
int gb_lw_mlp_samples(gb_lw_context* ctx, void* stream, const gb_lw_grid* grid, float* d_feat, float* d_tau,
                      float* d_frac);
/* Fits the input/output standardisation and the validity range on a sample
 * set: the min/max of every feature, widened by 2% of that width on each side
 * so that layers at the edge of the training set (the model-top layer) stay
 * on the network. */
int gb_lw_mlp_fit_norm(gb_lw_mlp* mlp, void* stream, int64_t rows, const float* d_feat, const float* d_tau,
                       const float* d_frac);
/* Network inputs d_x (bf16 [rows][16]) and targets d_t (fp32 [rows][288],
 * may be NULL) from samples. */
int gb_lw_mlp_prepare(gb_lw_mlp* mlp, void* stream, int64_t rows, const float* d_feat, const float* d_tau,
                      const float* d_frac, void* d_x, float* d_t);
/* Loss (mean weighted square error of the standardised outputs) and its
 * gradient w.r.t. every parameter (d_grad: GB_LW_MLP_NPARAM floats, NULL =
 * internal) for one batch; rows must be a multiple of 8. */
int gb_lw_mlp_gradients(gb_lw_mlp* mlp, void* stream, int64_t rows, const void* d_x, const float* d_t,
                        float* d_grad, float* d_loss);
/* One Adam step (beta 0.9/0.999) on one batch. */
int gb_lw_mlp_train_step(gb_lw_mlp* mlp, void* stream, int64_t rows, const void* d_x, const float* d_t, float lr,
                         float* d_loss);
/* Standardised outputs d_y[rows][288] of the training forward pass. */
int gb_lw_mlp_forward(gb_lw_mlp* mlp, void* stream, int64_t rows, const void* d_x, float* d_y);
/* Inference for one grid: taug and Planck fractions [(icol*nlay + lay)*140 + g]
 * in binary16 (taug clamped to 65504, the largest finite value; 2 bytes each
 * instead of 4 halves what the column kernel reads) and the per-layer flag
 * (1 inside the training range) for gb_lw_grid's sur_* fields. */
int gb_lw_mlp_infer(gb_lw_mlp* mlp, void* stream, const gb_lw_grid* grid, uint16_t* d_tau, uint16_t* d_frac,
                    uint8_t* d_flag);
/* gb_rrtmg_lw_batch_device with learned gas optics: inference for every grid
 * into context buffers (561 bytes per column-layer), then the one batched
 * launch; out-of-range layers use taumol. */
int gb_rrtmg_lw_batch_surrogate(gb_lw_context* ctx, void* stream, int ngrid, const gb_lw_grid* grids,
                                gb_lw_mlp* mlp);

/* Human-readable text of a status code (static storage). */
const char* gb_rrtmg_lw_strerror(int code);
/* Detail of the last failing call on this context (CUDA error text etc.). */
const char* gb_rrtmg_lw_last_error(gb_lw_context* ctx);

#ifdef __cplusplus
}
#endif

#endif /* GB_RRTMG_LW_H */
