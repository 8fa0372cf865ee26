/*
 * mge_oracle.h -- CPU FP64 restatement of code_mge's multigrid Runge-Kutta
 * residual cycle.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it as the checker.
 * The GPU product never links, loads or calls this library.
 *
 * Parity status: UNPINNED against the reference binary.  The reference is
 * Fortran 90 whose build needs an absent library ($(HOME)/fcode), absent
 * plugin sources and absent include files; no Fortran compiler exists on
 * either machine, and the reference ships no golden vectors for this path.
 * This restatement follows the Fortran line by line (loop order, expression
 * order, quirks); the functions cite the file:line they restate.
 *
 * The entry points mirror include/mge_gpu.h one for one with an mgeo_
 * prefix, so a test drives the oracle and the GPU library with the same call
 * sequence and compares the resulting fields.
 */
#ifndef MGE_ORACLE_H
#define MGE_ORACLE_H
#include "../include/mge_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mgeo_ctx mgeo_ctx;

int  mgeo_init(const mge_params* prm, mgeo_ctx** out);
void mgeo_destroy(mgeo_ctx* ctx);
const char* mgeo_last_error(const mgeo_ctx* ctx);
int  mgeo_add_block(mgeo_ctx* ctx, const mge_block_desc* desc, int level, int serial);
int  mgeo_commit(mgeo_ctx* ctx);
int  mgeo_init_flow(mgeo_ctx* ctx);
int  mgeo_upload_state(mgeo_ctx* ctx, int level, int serial, const double* w);
int  mgeo_download_field(mgeo_ctx* ctx, int level, int serial, const char* name,
                         double* out, size_t count);
int  mgeo_timestep(mgeo_ctx* ctx, int level, int serial);
int  mgeo_euler(mgeo_ctx* ctx, int level, int serial, int itime, int ncyc,
                int mgl, int mlvl, int lres, int lfir);
int  mgeo_euler_partial(mgeo_ctx* ctx, int level, int serial, int itime, int ncyc,
                        int mgl, int mlvl, int lres, int lfir, int nstage);
int  mgeo_movco(mgeo_ctx* ctx, int mgl);
int  mgeo_movfin(mgeo_ctx* ctx, int mgl, int mlvl);
int  mgeo_bc_overlap(mgeo_ctx* ctx, int mgl);
int  mgeo_get_rtrms(mgeo_ctx* ctx, int level, int serial, int ncyc, double* out);
int  mgeo_solve(mgeo_ctx* ctx, const mge_solve_opts* opts, double* rtrms_hist,
                int hist_len, int* cycles_done, mge_forces* forces);
int  mgeo_cycle(mgeo_ctx* ctx, int mlvl, int ncyc, double* max_res);
int  mgeo_forces_compute(mgeo_ctx* ctx, int level, const mge_solve_opts* opts,
                         mge_forces* out);
int  mgeo_upload_solut(mgeo_ctx* ctx, int level, int serial, double p_tot, double* solut,
                       size_t count, int* nval_out);
int  mgeo_time_advance(mgeo_ctx* ctx, int* itime_out);
int  mgeo_move_surface(mgeo_ctx* ctx, int level, int serial, const double* disp, const double* norv,
                       const double* vel, double vel_fs);
int  mgeo_get_surface(mgeo_ctx* ctx, int level, int serial, double* pnew);
/* threads used by the loops of the oracle (1 = the serial mgsol analogue) */
void mgeo_set_threads(int n);
int  mgeo_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
