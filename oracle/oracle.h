/*
 * CPU oracle for the RRTMG_LW column solver -- TEST INFRASTRUCTURE ONLY.
 *
 * A double-precision C++ restatement of the reference Fortran
 * (luflarois/brams, src/rrtmg/RRTMG_LW), statement for statement, used as the
 * checker for the CUDA library and as the timed CPU baseline.  Nothing in the
 * product library links against or calls this code.
 *
 * All arrays use the reference's Fortran layout: column-major, first index
 * fastest, with the exact extents of the rrtmg_lw argument list
 * (rrtmg_lw_rad.f90:99-108, declarations :216-332).
 *
 * Parity note: the reference Fortran cannot be compiled here (no Fortran
 * compiler) and its k-distribution data module is absent, so this oracle is
 * pinned by project-made known-answer tests (analytic limits, MT19937
 * published outputs, table round trips), not by reference outputs.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* rrtmg_lw_ini (rrtmg_lw_init.f90:47): loads the table container files and
 * builds tau/exp/tfn lookup tables and heatfac.  Returns 0 on success. */
int ora_init(double cpdair, const char* ref_tables_path, const char* k_tables_path);

/* rrtmg_lw (rrtmg_lw_rad.f90:99): full column solver.  Returns 0 on success,
 * nonzero where the reference would STOP (see ora_error_string).
 * duflx_dt/duflxc_dt may be NULL when idrv == 0.  nthreads <= 1 runs the
 * column loop serially; larger values split columns over std::threads. */
int ora_rrtmg_lw(int ncol, int nlay, int* icld, int idrv,
                 const double* play, const double* plev, const double* tlay,
                 const double* tlev, const double* tsfc,
                 const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                 const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                 const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                 const double* ccl4vmr, const double* emis,
                 int inflglw, int iceflglw, int liqflglw,
                 const double* cldfmcl, const double* taucmcl, const double* ciwpmcl,
                 const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                 const double* tauaer,
                 double* uflx, double* dflx, double* hr, double* uflxc, double* dflxc,
                 double* hrc, double* duflx_dt, double* duflxc_dt, int nthreads);

/* Per-column intermediates of one column (1-based icol): taug/taut/fracs
 * (nlay,140), planklay (nlay,16), planklev (0:nlay,16), plankbnd(16),
 * taucmc (140,nlay) after cldprmc, laytrop.  Any pointer may be NULL. */
int ora_column_intermediates(int ncol, int nlay, int icol, int icld,
                             const double* play, const double* plev, const double* tlay,
                             const double* tlev, const double* tsfc,
                             const double* h2ovmr, const double* o3vmr, const double* co2vmr,
                             const double* ch4vmr, const double* n2ovmr, const double* o2vmr,
                             const double* cfc11vmr, const double* cfc12vmr, const double* cfc22vmr,
                             const double* ccl4vmr, const double* emis,
                             int inflglw, int iceflglw, int liqflglw,
                             const double* cldfmcl, const double* taucmcl, const double* ciwpmcl,
                             const double* clwpmcl, const double* reicmcl, const double* relqmcl,
                             const double* tauaer,
                             double* taug, double* fracs, double* taut, double* planklay,
                             double* planklev, double* plankbnd, double* taucmc, int* laytrop);

/* cldprop (rrtmg_lw_cldprop.f90:50) for one column of nlay layers.
 * taucloud is (nlay,16); returns ncbands through *ncbands. */
int ora_cldprop(int nlayers, int inflag, int iceflag, int liqflag,
                const double* cldfrac, const double* tauc /* (16,nlay) */,
                const double* ciwp, const double* clwp, const double* rei,
                const double* rel, int* ncbands, double* taucloud);

/* mcica_subcol_lw (mcica_subcol_gen_lw.f90:183) with the reference's draw
 * order.  alpha is (ncol,nlay) (used for icld 4/5 only, may be NULL else).
 * Outputs cldfmcl/ciwpmcl/clwpmcl/taucmcl (140,ncol,nlay), reicmcl/relqmcl
 * (ncol,nlay).  irng is in/out as in the reference (clamped to 0/1). */
int ora_mcica_subcol_lw(int ncol, int nlay, int icld, int permuteseed, int* irng,
                        const double* play, const double* cldfrac, const double* ciwp,
                        const double* clwp, const double* rei, const double* rel,
                        const double* tauc /* (16,ncol,nlay) */, const double* alpha,
                        double* cldfmcl, double* ciwpmcl, double* clwpmcl,
                        double* reicmcl, double* relqmcl, double* taucmcl);

/* Mersenne twister of mcica_random_numbers.f90:77-306: the first n outputs of
 * getRandomInt (as uint32) and getRandomReal for a scalar seed. */
void ora_mt_draws(int32_t seed, int n, uint32_t* ints, double* reals);

/* KISS generator kissvec (mcica_subcol_gen_lw.f90:711-743) for one column. */
void ora_kiss_draws(int32_t s1, int32_t s2, int32_t s3, int32_t s4, int n, double* reals);

/* Lookup tables of rrtmg_lw_ini (0:ntbl): tau_tbl, exp_tbl, tfn_tbl. */
void ora_get_tables(double* tau_tbl, double* exp_tbl, double* tfn_tbl, double* heatfac,
                    double* fluxfac);

const char* ora_error_string(int code);

#ifdef __cplusplus
}
#endif
