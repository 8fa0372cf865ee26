/*
 * mge_gpu.h -- C-ABI of the GB300 multigrid Runge-Kutta residual cycle.
 *
 * This is the drop-in boundary for code_mge's solver/euler call chain.  Every
 * entry point is plain C: pointers, sizes and POD structs, no C++ or torch
 * types, so the unchanged Fortran driver can bind it through ISO_C_BINDING.
 *
 * Array layout of every per-cell field crossing this boundary is the Fortran
 * layout of the reference's mgrid arrays (make_flow.f90:36-56):
 *     w(0:ib,0:jb,0:kb,1:5)   column-major, i fastest, variable slowest,
 *     ib = nx+3, jb = ny+3, kb = nz+3   (two ghost layers on every face,
 *     physical cells i = 2..il with il = nx+1, psmoo.f90:125-127).
 * A C caller indexes it as w[v*N + i + (ib+1)*(j + (jb+1)*k)] with
 * N = (ib+1)*(jb+1)*(kb+1) and v = 0..4.
 *
 * Level numbering follows solver.f90: level 1 is the coarsest grid and level
 * nlevel the finest; the full-multigrid loop runs mlvl = 1..nlevel.
 *
 * Return codes: MGE_OK (0) or one of the negative MGE_E* codes below.  The
 * reference stops the program on the matching condition; the Fortran shim
 * turns a nonzero code back into that stop.
 */
#ifndef MGE_GPU_H
#define MGE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGE_ABI_VERSION 2

/* status codes */
#define MGE_OK           0
#define MGE_ENAN        -1  /* NaN residual (solver.f90:180) or NaN wsol (bc_cutcell.f90:147-156) */
#define MGE_ENEGPRESS   -2  /* c^2 < 0 or NaN in timestep (timestep.f90:45-48) */
#define MGE_EZERORHO    -3  /* |rho| < 1e-8 at a cut cell (efluxb.f90:61-64) */
#define MGE_EBADCFG     -4  /* bad distype/dissip/bctype/sizes (euler.f90:213, dflux.f90:107, bcond.f90:26-31) */
#define MGE_ENOMEM      -5  /* device memory exhausted / admission refused */
#define MGE_ETIMEOUT    -6  /* a bounded device wait gave up */
#define MGE_ECUDA       -7  /* any other CUDA runtime error */
#define MGE_ENOTFOUND   -8  /* unknown level/serial/case handle */

/* character-valued typepara switches, encoded as ints */
#define MGE_EQN_EULER    0  /* eqntype 'e' */
#define MGE_EQN_NS       1  /* eqntype 'n' */
#define MGE_DIS_CENTRAL  0  /* distype 'c'  : JST central flux + dflux */
#define MGE_DIS_ROE1     1  /* distype 'r1' : first-order Roe flux */
#define MGE_DIS_ROE2     2  /* distype 'r2' : MUSCL second-order Roe flux */
#define MGE_DISSIP_SCALAR 0 /* dissip 'scalar' */
#define MGE_DISSIP_MATRIX 1 /* dissip 'matrix' (dflux_matrix) */

#define MGE_PREC_FP64    0  /* plain: every level and kernel in FP64 */
#define MGE_PREC_MIXED   1  /* FP32 coarse levels, IRS and time step; FP64 finest R(w), update, norms, forces */
#define MGE_PREC_REFINED 2  /* what a mixed solve refines to: FP64 on every level; the finest level keeps
                               the mixed form's FP32 time step and IRS and its FP64 residual form */

#define MGE_MAX_STAGE   8
#define MGE_MAX_LEVEL  16
#define MGE_MAX_CLOUD   8

/*
 * Solver parameters: the typepara globals that input_param.f90:17-114 fills
 * from the job sheet, after its own post-processing (cfl made positive with
 * vt recording the sign, vis4 already divided by 32, free-stream state
 * non-dimensionalised with rho0 = 1 and p0 = 1/(gamma M^2)).
 * mge_params_default() fills the same derived quantities from
 * (gamma, mach, alpha, beta) the way input_param.f90:44-69 does.
 */
typedef struct mge_params {
  int    mstage;                  /* number of RK stages (imstage) */
  double cstp[MGE_MAX_STAGE];     /* stage coefficients alpha_m */
  double cdis[MGE_MAX_STAGE];     /* dissipation blending per stage */
  double cfl;                     /* |cfl| */
  int    vt;                      /* 1: global time step dtim, 0: local vdtim */
  double vis2, vis4;              /* k2 and k4 (vis4 already /32) */
  double smoo;                    /* implicit residual smoothing coefficient */
  int    mgtype;                  /* 1: V cycle, 2: W cycle */
  int    eqntype;                 /* MGE_EQN_* */
  int    distype;                 /* MGE_DIS_* */
  int    dissip;                  /* MGE_DISSIP_* */
  double gamma;
  double rm, alpha, beta;         /* free-stream Mach and angles (radians) */
  double rho0, p0, c0, ei0, u0, v0, w0, h0;
  double viscl;                   /* laminar viscosity (NS) */
  double prlmean;                 /* laminar Prandtl number (NS) */
  double gas_const;               /* gas constant used for temperature (NS) */
  double limfac, epsentr;         /* Roe limiter / Harten entropy fix */
  int    wall_adiabatic;          /* NS cut-cell wall: 1 adiabatic no-slip */
  int    irs_variant;             /* 0: psmoo_old (what euler calls), 1: psmoo + progon3 */
  int    precision;               /* MGE_PREC_* */
  int    nlevel;                  /* number of multigrid levels */
  int    mcyc[MGE_MAX_LEVEL];     /* cycles per FMG level (mcyc) */
  double conv_drop;               /* exit when ini_res/max_res > conv_drop (1e6, solver.f90:238) */
  int    execmode;                /* 0 steady, 1 unsteady dual time stepping (BDF2 in physical time) */
  double dtstep;                  /* physical time step, non-dimensional (input_param.f90:90-96) */
} mge_params;

/*
 * One uniform Cartesian block (an mgrid of the reference) with its cut-cell
 * records.  All pointers are borrowed for the duration of mge_add_block only.
 */
typedef struct mge_block_desc {
  int    nx, ny, nz;              /* physical cells (mgrid%ncell) */
  double h[3];                    /* cell sizes */
  double origin[3];               /* coordinate of the lower corner of cell (2,2,2) */
  double cellvolume;
  double si[3], sj[3], sk[3];     /* face vectors (init_metric.f90:111-177, uniform block) */
  int    bctype[6];               /* -20 far, -50 symmetry, -60 periodic, -80 wall, 0 none */
  double facenvec[6][3];          /* outward face normal per face (bc_far.f90:99) */
  const int32_t* blank;           /* (0:ib,0:jb,0:kb) 0 = solid; NULL = all fluid */
  /* cut-cell mirror records z(1:nmir) (txcut, efluxb.f90:30-48, bc_cutcell.f90:41-84) */
  int    nmir;
  const int32_t* ccid;            /* [nmir][3] cut (fluid) cell */
  const int32_t* scid;            /* [nmir][3] solid neighbour */
  const int32_t* faceid;          /* [nmir] 1..6: solid at -i,-j,-k (1,2,3) or +i,+j,+k (4,5,6) */
  const int32_t* zz;              /* [nmir] axis 1..3 */
  const int32_t* npoint;          /* [nmir] cloud size (<= MGE_MAX_CLOUD) */
  const int32_t* ijkdex;          /* [nmir][MGE_MAX_CLOUD][3] cloud cells */
  const double*  coef;            /* [nmir][MGE_MAX_CLOUD] cloud weights */
  const double*  nvec;            /* [nmir][3] wall normal (need not be unit) */
  const double*  qb;              /* [nmir][3] wall velocity; NULL = fixed wall */
  const double*  area;            /* [nmir] wall-face area for force integration; NULL = face area */
  /* parent (next coarser level) relation; parent = -1 for the coarsest level */
  int    parent;                  /* serial of the parent block on level-1 */
  int    ratio[3];                /* h_parent / h per axis (1 or 2) */
  int    offset[3];               /* origin = parent origin + offset * h_parent */
  /* the records' ray-surface intersection points z(m)%psurf, the base of the
   * moved points of mge_move_surface; NULL = zeros */
  const double*  psurf;           /* [nmir][3] */
} mge_block_desc;

/* Cut-cell wall forces (new: the reference has no Cl/Cd integrator): the
 * pressure on every wall face of the records and, for Navier-Stokes, the
 * wall's viscous stress as the solver's no-slip wall flux defines it. */
typedef struct mge_forces {
  double force[3];
  double moment[3];
  double cl, cd;
} mge_forces;

/* Options of a whole-hierarchy solve (solver.f90:109-292 on the device) */
typedef struct mge_solve_opts {
  int    max_cycles_total;        /* safety cap on finest cycles; 0 = mcyc only */
  double ref_area;                /* reference area for Cl/Cd */
  double moment_center[3];
  int    use_graph;               /* capture the multigrid cycle in a CUDA graph */
  double refine_drop;             /* mixed form: switch to FP64 once the residual has dropped by this factor (0: never) */
} mge_solve_opts;

typedef struct mge_ctx mge_ctx;

/* Library identity */
int         mge_abi_version(void);
const char* mge_build_info(void);

/* Fill derived free-stream quantities the way input_param.f90:44-69 does. */
void mge_params_default(mge_params* prm, double gamma, double mach,
                        double alpha, double beta);

/* Context lifetime.  Replaces make_flow allocation (make_flow.f90:36-56). */
int  mge_init(const mge_params* prm, int device, mge_ctx** out);
void mge_destroy(mge_ctx* ctx);
const char* mge_last_error(const mge_ctx* ctx);

/* Add one block at (level, serial); serial counts from 1 per level. */
int mge_add_block(mge_ctx* ctx, const mge_block_desc* desc, int level, int serial);

/* Finish setup: allocate device fields, upload metrics and records. */
int mge_commit(mge_ctx* ctx);

/* Free-stream start, then depvars + bc_cutcell + bcond (init_flow.f90:46-96). */
int mge_init_flow(mge_ctx* ctx);

/* Host <-> device state in the Fortran layout above. p may be NULL.
 * mge_upload_state then does what init_flow.f90:46-66 does after read_solut:
 * depvars, bc_cutcell (the records' solid state from the new cells; a NaN
 * there returns MGE_ENAN as bc_cutcell.f90:147-156 stops) and bcond. */
int mge_upload_state(mge_ctx* ctx, int level, int serial, const double* w);
int mge_download_state(mge_ctx* ctx, int level, int serial, double* w, double* p);
/* Download any per-cell field by name: "w","p","dw","fw","wn","ws","wr","qf",
 * "vdtim","lam" (radi+radj+radk), "blank"(as double), "marker"(as double). */
int mge_download_field(mge_ctx* ctx, int level, int serial, const char* name,
                       double* out, size_t count);

/* Per-call drop-in entry points (solver.f90:154-155,199,204,218-219,228,258). */
int mge_timestep(mge_ctx* ctx, int level, int serial);                 /* timestep.f90 */
int mge_euler(mge_ctx* ctx, int level, int serial, int itime, int ncyc,
              int mgl, int mlvl, int lres, int lfir);                  /* euler.f90 */
int mge_movco(mge_ctx* ctx, int mgl);                                  /* movco.f90 */
int mge_movfin(mge_ctx* ctx, int mgl, int mlvl);                       /* movfin.f90 */
int mge_bc_overlap(mge_ctx* ctx, int mgl);                             /* bc_overlap.f90 */

/* Residual history entry rtrms(ncyc) of a block (euler.f90:431-447). */
int mge_get_rtrms(mge_ctx* ctx, int level, int serial, int ncyc, double* out);

/* Whole solve on the device: FMG level loop, V/W cycles, convergence exit.
 * rtrms_hist receives max_res per finest cycle (job_res.dat), up to hist_len. */
int mge_solve(mge_ctx* ctx, const mge_solve_opts* opts, double* rtrms_hist,
              int hist_len, int* cycles_done, mge_forces* forces);

/* One multigrid cycle (the body of solver.f90's lop0 loop, lines 126-234) at
 * FMG level mlvl, replayed from a CUDA graph captured on the first call for
 * that level; *max_res receives the residual of the cycle (solver.f90:164-176). */
int mge_cycle(mge_ctx* ctx, int mlvl, int ncyc, double* max_res);

/* Asynchronous form of mge_cycle for driving many cases at once: enqueue one
 * cycle (and the read-back of its residual) on the context's stream and
 * return; mge_cycle_poll returns 1 while it runs, then MGE_OK with *max_res
 * (or the error of the cycle).  mge_prolong_async enqueues the FMG
 * prolongation from level mlvl to mlvl+1 (solver.f90:256-259). */
int mge_cycle_async(mge_ctx* ctx, int mlvl);
int mge_cycle_poll(mge_ctx* ctx, int ncyc, double* max_res);
int mge_prolong_async(mge_ctx* ctx, int mlvl);

/* Lockstep cycles of a group of cases (the batched sweep and the serving
 * loop).  One multigrid cycle at FMG level mlvl for every case of the
 * group: each phase of the cycle (time step, each stage's prep, face,
 * record, combine passes, the line sweeps, the boundary passes, the
 * transfers) is one launch over the block of that level of every case; on a
 * level whose blocks hold at most MGE_GROUP_COOP_MAX_CELLS cells in all
 * (environment, 300,000 by default) the whole update of every case is one
 * persistent cooperative launch instead.  The whole cycle is one captured
 * CUDA graph, so the launches of a cycle do not grow with the number of
 * cases.  The reference's solver loops the
 * blocks of one case (solver.f90:151-157); this runs that loop over the
 * blocks of many cases at once, which has no counterpart there.  The cases
 * must share the level count, the multigrid and stage schedule, the CFL
 * number and the scheme (JST central, steady, psmoo_old smoothing), have one
 * block per level, and be in the same precision form; their sizes, bodies
 * and flow conditions may differ.  Each case's results are those of its own
 * per-phase cycle with the line sweeps in global memory.  _async returns at
 * once (MGE_EBADCFG when the cases cannot run together, with the reason in
 * mge_last_error of the first case); _poll returns 1 while the cycle runs,
 * then 0 with each case's finest-level residual in max_res[q] and its stop
 * (0 or an MGE_ code, the reason in that case's mge_last_error) in
 * rc_out[q].  A case takes part in one cycle at a time, group or single. */
int mge_group_cycle_async(mge_ctx* const* cases, int n, int mlvl);
int mge_group_cycle_poll(mge_ctx* const* cases, int n, int ncyc, double* max_res, int* rc_out);

/* Switch a committed context between MGE_PREC_FP64, MGE_PREC_MIXED and
 * MGE_PREC_REFINED in place (the coarse levels' state is converted; graphs
 * are re-captured).  The mixed form's FP32 coarse corrections carry rounding
 * of the size of the coarse truncation error, so its residual stalls near a
 * 1e-7 drop; switching to MGE_PREC_REFINED there (FP64 coarse levels) ends
 * the stall and finishes the solve at FP64 accuracy.
 *
 * On the finest level, the mixed and refined forms evaluate the JST central
 * residual of the Euler equations in a contracted FP64 form: fused
 * multiply-adds, the cell flux as velocity times state, and the convective
 * part as the central difference 0.5*(F(q-1) - F(q+1)) of the cell fluxes
 * instead of the difference of two averaged face fluxes.  It is the same
 * FP64 quantity up to a few roundings, not the reference's bit pattern
 * (MGE_PREC_FP64 keeps that).  MGE_FAST_RESIDUAL=0 in the environment turns
 * it off. */
int mge_set_precision(mge_ctx* ctx, int precision);

/* Launch forms the autotuner chose for a block at mge_init_flow: *coop = 1
 * when timestep + euler run as one cooperative launch; irs3[d] = 1 when the
 * direction-d line sweeps use shared-memory tiles. */
int mge_tuned(mge_ctx* ctx, int level, int serial, int* coop, int* irs3);

/* Free and total memory of a device (admission control of the serving loop). */
int mge_device_mem(int device, size_t* free_bytes, size_t* total_bytes);

/* Cap the grid of the one-launch euler of small blocks (0: all resident
 * blocks), so that cases running side by side can share the GPU. */
int mge_set_coop_ctas(mge_ctx* ctx, int max_ctas);

/* Profiling hook: one timestep + euler update of (level, 1) as a single
 * cooperative launch, recording the device time of every phase between its
 * grid-wide barriers into us_out (microseconds); returns the phase count. */
int mge_coop_trace(mge_ctx* ctx, int level, double* us_out, int nout);

/* Device time (CUDA events on the context's stream) of the last mge_cycle. */
double mge_last_cycle_ms(const mge_ctx* ctx);

/* Kernels this library has launched through mge_cycle (graph kernel nodes). */
long long mge_launch_count(const mge_ctx* ctx);

/* Profiling hook: run one timestep + full euler update on (level, 1) `reps`
 * times outside any graph, timing each kernel kind with CUDA events; writes
 * the average ms per launch of {timestep, prep, face, rec, combine, irs_i,
 * irs_j, irs_k_update, cutcell, bcond, rtrms} into ms_out[0..10] ("rec" is
 * the cut-cell wall-term pass), and, when nout allows, the face pass of stage
 * m (1-based) into ms_out[10 + m], the prep pass of stage m into
 * ms_out[10 + mstage + m] and the combine pass into ms_out[10 + 2*mstage + m].
 * Advances the state of that level. */
int mge_kernel_times(mge_ctx* ctx, int level, int reps, double* ms_out, int nout);

/* Residual norm rtrms (the quantity of euler.f90:431-447) of one block from
 * device arrays the caller owns, for callers that cannot allocate device
 * memory.  No counterpart in the reference: it exists so that a caller that
 * may not call cudaMalloc (for example inside a stream capture it does not
 * control, or under a fixed device-memory budget) can still get the norm.
 * It allocates nothing: its partial sums live in a static 32 KiB device
 * array, which limits it to nx*ny*nz <= 8,388,608 cells (MGE_EBADCFG beyond).
 * dw_rho: density residual dw(:,:,:,1); vdtim: local time steps; blank:
 * int32 blanking as the reference's integer blank array holds it (not the
 * one-byte blank a context keeps on the device), all in the
 * (0:ib,0:jb,0:kb) layout; dtim: the global time step, read when vt = 1;
 * norm_out: one device double; stream: a cudaStream_t or NULL.
 * Every call made outside a stream capture looks up the array's device
 * address afresh (a device reset may move it); a call inside a capture uses
 * the address of the last call made outside one, so make one call on each
 * device before any capture (MGE_EBADCFG otherwise).  An error already
 * pending on the calling thread is returned as MGE_ECUDA, not cleared, and
 * nothing is launched.  All calls share the array: calls that overlap on
 * the GPU race. */
int mge_residual_norm_noalloc(const double* dw_rho, const double* vdtim, const int32_t* blank,
                              int nx, int ny, int nz, double cfl, int vt, double dtim,
                              double* norm_out, void* stream);

/* upload_solut.f90:203-237 (blk2mgrid.f90:14-26 calls it per block): the
 * cell-centre output variables rho, u, v, w, cp, mach, pt-loss of the
 * physical cells (Navier-Stokes adds the energy and three zero gradients),
 * computed on the device in FP64 and copied into
 * solut(2:il,2:jl,2:kl,1:nval), Fortran order.  *nval_out = 7 or 11;
 * count >= nval*nx*ny*nz.  p_tot: the free-stream total pressure the
 * reference's pt-loss is relative to. */
int mge_upload_solut(mge_ctx* ctx, int level, int serial, double p_tot, double* solut,
                     size_t count, int* nval_out);

/* write_solut / read_solut (wsolut.f90:49-92, rsolut.f90:1-41): every block
 * of the context, in mge_add_block order, as the reference's restart text:
 * "(5I5)" code, low(1:4), upp(1:4), then "(5f16.7)" w(0:ib,0:jb,0:kb,1:5).
 * codes[q] is the code of the q-th block added (ncodes = 0: codes 1..n).
 * Reading checks each block's code and upper bounds (the reference stops on a
 * mismatch: MGE_EBADCFG here) and uploads the state. */
int mge_write_restart(mge_ctx* ctx, const char* path, const int* codes, int ncodes);
int mge_read_restart(mge_ctx* ctx, const char* path, const int* codes, int ncodes);

/* solver.f90:263-276,286, the end of a physical time step of the unsteady
 * mode (execmode 1): w2 = w1, w1 = w on every block, and the step counter
 * the following cycles use advances (*itime_out receives it).  The counter
 * starts at 0 at mge_init_flow; the transient source of euler.f90:249-275
 * applies from itime 1 on. */
int mge_time_advance(mge_ctx* ctx, int* itime_out);

/* movsurf.f90:28-35 for one block, called where solver.f90:117 calls it (at
 * the start of each physical step, approxbc on), with the kinematics the
 * reference's FSI framework supplies per record, host arrays [nmir][3] in
 * mge_add_block's record order:
 *   pnew = psurf + disp   (movsurf.f90:31; read back by mge_get_surface)
 *   wall normal = norv    (bc_cutcell.f90:49; normalised where it is used,
 *                          bc_cutcell.f90:57-58, so it need not be unit)
 *   qb = vel / vel_fs     (bc_cutcell.f90:50; vel_fs is input_param.f90:51's
 *                          rm*sqrt(gamma*gas_pmean/gas_rhomean))
 * The new normal and wall velocity take effect from the next stage on, in
 * the cut-cell state, the wall fluxes and the no-slip wall.  The reference's
 * approxbc-off state is the descriptor's nvec and qb; a context goes back to
 * it by a call with disp 0, norv = nvec and vel = qb*vel_fs.  Ordered after
 * the work already queued on the context; MGE_EBADCFG while the context is
 * part of a group cycle in flight, or when vel_fs is not positive. */
int mge_move_surface(mge_ctx* ctx, int level, int serial, const double* disp, const double* norv,
                     const double* vel, double vel_fs);

/* The records' moved points pnew [nmir][3] (psurf before the first
 * mge_move_surface). */
int mge_get_surface(mge_ctx* ctx, int level, int serial, double* pnew);

/* The same text for one block, without a context or a GPU: returns the bytes
 * of the text (writing at most cap-1 of them and a NUL into buf when buf is
 * not null); and the parse of one block from text, returning the bytes it
 * consumed or a negative MGE_E* code. */
long long mge_restart_format(int code, int ib, int jb, int kb, const double* w, char* buf,
                             long long cap);
long long mge_restart_parse(const char* text, long long len, int code, int ib, int jb, int kb,
                            double* w);

/* Cut-cell wall force integration on a level: pressure, plus the viscous
 * wall stress for Navier-Stokes (new: no counterpart in the reference). */
int mge_forces_compute(mge_ctx* ctx, int level, const mge_solve_opts* opts,
                       mge_forces* out);

/* Debug / parity: run only stages 1..nstage of one euler call (no rtrms). */
int mge_euler_partial(mge_ctx* ctx, int level, int serial, int itime, int ncyc,
                      int mgl, int mlvl, int lres, int lfir, int nstage);

/* Device bytes held by the context (admission control). */
size_t mge_device_bytes(const mge_ctx* ctx);

/* Synchronise the context's stream; returns the first deferred device error. */
int mge_sync(mge_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* MGE_GPU_H */
