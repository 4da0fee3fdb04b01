/*
 * wolfd2_gpu.h -- C-ABI of the GB300 (sm_103a) projection-method time step.
 *
 * The library replaces the hot-path subroutines of the wolfd2 Fortran code.
 * Every drop-in entry point takes the same arguments as the Fortran routine
 * it replaces, in the same order and by reference (F77 implicit interfaces
 * pass everything by address), preceded by a context handle.  Arrays are the
 * Fortran driver's own static arrays: REAL*8 (0:mnx,0:mny) column-major,
 * INTEGER*4 region tables (mgri,mgrj[,4]), REAL*8 dBCVal(mgri,mgrj,4,4).
 * mnx/mny/mgri/mgrj are the driver's compile-time sizes (include/config.f)
 * and are given once to wolfd2gpu_create.
 *
 * Data movement: metric arrays and region tables are uploaded once by
 * wolfd2gpu_create / wolfd2gpu_set_metrics (they are constant after Grid and
 * SetUpBCs).  Field arguments of the drop-ins are copied host->device on
 * entry and device->host on exit, so each call is a self-contained
 * replacement.  The device-resident path (wolfd2gpu_load_fields,
 * wolfd2gpu_step, wolfd2gpu_store_fields) keeps the fields on the GPU and
 * runs the whole time-loop body of main.f:690-972 per step.
 *
 * Errors: every function returns an int status, 0 on success (see
 * W2_E_* below).  Convergence results come back through the same out
 * arguments as the reference (nSorConv, the nAuxMomentum value).
 * Threading: one host thread per context; calls on a context are
 * serialised on the context's CUDA stream.
 */
#ifndef WOLFD2_GPU_H
#define WOLFD2_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define W2_OK              0
#define W2_E_ARG           1  /* bad argument or size                          */
#define W2_E_CUDA          2  /* CUDA runtime error                           */
#define W2_E_TIMEOUT       3  /* a device-side wait ran out its time limit    */
#define W2_E_DIVERGED      4  /* max step difference > 1e12 (main.f:969-972)  */
#define W2_E_BCFLAG        5  /* invalid boundary flag (bound_cond.f 'stop')  */
#define W2_E_UNSUPPORTED   6  /* configuration outside this library's scope   */
#define W2_E_FALLBACK      7  /* chain recurrence needed the sequential path  */
#define W2_E_SIZE          8  /* larger than the fixed scratch of the
                                 allocation-free entry point               */

/* Region / boundary enums, identical to include/wolfd2.h:15-60 of the
 * reference. */
#define W2_RM_BLOCKG 0
#define W2_RM_INTERN 1
#define W2_RM_POROUS 2
#define W2_BM_INTERN 0
#define W2_BM_WALL1  1
#define W2_BM_WALL2  2
#define W2_BM_INLET  3
#define W2_BM_OUTLT1 4
#define W2_BM_OUTLT2 5
#define W2_WEST  1
#define W2_EAST  2
#define W2_SOUTH 3
#define W2_NORTH 4

/* Arithmetic of the hot path. */
#define W2_PREC_FP64  0   /* plain FP64, op-by-op as the reference source  */
#define W2_PREC_MIXED 1   /* red/black Poisson sweeps in FP32 on the
                             correction equation, FP64 residual and
                             correction (iterative refinement); npsolver 5
                             or 6 on any grid (rows that round to the unit
                             stencil in FP32 take the tile kernel, others
                             -- non-square cells, blockages, curvilinear
                             grids -- the general-row kernel)            */

typedef struct w2_ctx w2_ctx;

/* Metric arrays in the argument order of grid.f:Grid (src/grid.f:31-42):
 * rau rbu rbv rgv ran rbn rgn rac rbc rgc dju djv djc djn xen yen xzn yzn
 * xec yec xzc yzc xeu yeu xzv yzv xzu yzu xev yev -- 30 host pointers,
 * each REAL*8 (0:mnx,0:mny). */
#define W2_NMETRIC 30

/* Create a context for an nx x ny natural-point grid.  Uploads the region
 * tables (output of SetUpBCs, src/bound_cond.f:34-443) and, where nRegType
 * has porous regions, their porosity and Dupuit-Forchheimer constants
 * (output of PorRegCnst, src/bound_cond.f:1883-1986; may be NULL without
 * porous regions).  Porous regions run in the drop-in nAuxMomentum, the
 * FP64 step, the mixed step (its FP32 momentum on the tables rounded to
 * FP32) and ensembles; the adjoint returns W2_E_UNSUPPORTED for them.  Fields are
 * zero.  No reference counterpart (the reference keeps these as static
 * arrays). */
int wolfd2gpu_create(w2_ctx **ctx, int mnx, int mny, int mgri, int mgrj,
                     int nx, int ny, const int *nReg, const int *nRegBrd,
                     const int *nRegType, const int *nMomBdTp,
                     const double *dBCVal, const double *dPRporos,
                     const double *dPRporc1, const double *dPRporc2);
int wolfd2gpu_destroy(w2_ctx *ctx);

/* Upload the 30 metric arrays computed by the driver's Grid
 * (src/grid.f:368-535), in the order listed above. */
int wolfd2gpu_set_metrics(w2_ctx *ctx, const double *const *metrics);

/* Compute the metric arrays on the device from natural grid points gx, gy
 * (0:mnx,0:mny) with nodes (1..nx,1..ny) filled and already divided by
 * dlref: MirrorPts + FullGrid + Metric, src/grid.f:258-535.  If metrics_out
 * is non-NULL the 30 arrays are also copied back to those host arrays. */
int wolfd2gpu_grid_metric(w2_ctx *ctx, const double *gx, const double *gy,
                          double *const *metrics_out);

/* ---- Drop-in replacements (arguments as in the reference) ------------ */

/* nAuxMomentum, src/momentum.f:33-48: returns the number of Q-L iterations
 * (or -1) through *nQLiter.  The reference's metric arguments are not in
 * this signature: the copies uploaded at set-up are used (the Fortran
 * replacement routine accepts and drops them).  Non-zero
 * density d, dn (EqState output) adds the buoyancy term of YMomentum
 * (momentum.f:703, divided by fr); d = dn = NULL means zero density. */
int wolfd2gpu_naux_momentum(w2_ctx *ctx, const int *nx, const int *ny,
                            const int *mqiter, const double *dk,
                            const double *re, const double *fr,
                            const double *qtol, const double *d,
                            const double *dn, const double *un,
                            const double *vn, double *us, double *vs,
                            int *nQLiter);

/* Ppe, src/pressure.f:30-38: solves for p in place; nSorConv out. */
int wolfd2gpu_ppe(w2_ctx *ctx, const int *nx, const int *ny,
                  const int *lCartesGrid, const int *nPpeSolver,
                  const int *msorit, int *nSorConv, const double *dk,
                  const double *sortol, const double *sorrel, const double *u,
                  const double *v, double *p);

/* Project, src/utility.f:253-259. */
int wolfd2gpu_project(w2_ctx *ctx, const int *nx, const int *ny,
                      const double *dk, const double *p, double *u, double *v);

/* VelBoundCond, src/bound_cond.f:511-513. */
int wolfd2gpu_vel_bound_cond(w2_ctx *ctx, const int *nx, const int *ny,
                             double *u, double *v);

/* PresBoundCond, src/bound_cond.f:853-856. */
int wolfd2gpu_pres_bound_cond(w2_ctx *ctx, const int *nx, const int *ny,
                              double *p);

/* VelOutflowBCs, src/bound_cond.f:1656-1659. */
int wolfd2gpu_vel_outflow_bcs(w2_ctx *ctx, const int *nx, const int *ny,
                              double *u, double *v);

/* DiffMaxNorm, src/utility.f:446: *result = max |un - u| over the
 * reference's index range. */
int wolfd2gpu_diff_max_norm(w2_ctx *ctx, const int *nx, const int *ny,
                            const double *un, const double *u,
                            double *result);

/* Filter, src/utility.f:33-36, velocity components (ncomp 1 = u, 2 = v). */
int wolfd2gpu_filter(w2_ctx *ctx, const int *nx, const int *ny,
                     const int *ncomp, const double *fp, double *qu);

/* ---- Thermal energy (drop-ins; main.f:839-855 with nthermen = 1) --------
 * Thermal region tables as the reference passes them: nTRgType(mgri,mgrj)
 * (0 no source, 1 heat generation, 2 fixed temperature), nTemBdTp(mgri,mgrj,4)
 * (0 interface, 1 fixed temperature, 2 heat flux), dTRgVal(mgri,mgrj),
 * dHGSTval(mgri,mgrj); face temperatures are dBCVal(...,4) given to
 * wolfd2gpu_create.  An unknown flag returns W2_E_BCFLAG (the reference
 * stops).  Metric arguments are the uploaded ones. */

/* TempBoundCond, src/bound_cond.f:1030-1033. */
int wolfd2gpu_temp_bound_cond(w2_ctx *ctx, const int *nx, const int *ny,
                              const int *nTRgType, const int *nTemBdTp,
                              const double *dTRgVal, double *t);

/* ThermEnergy, src/thermal.f:24-34: t (the starred temperature) updated in
 * place from un, vn, u, v, tn. */
int wolfd2gpu_therm_energy(w2_ctx *ctx, const int *nx, const int *ny,
                           const int *nTRgType, const int *nTemBdTp,
                           const double *dk, const double *pe,
                           const double *dTRgVal, const double *dHGSTval,
                           const double *un, const double *vn, const double *u,
                           const double *v, const double *tn, double *t);

/* Filter, src/utility.f:33-36, of the temperature (ncomp = _T_): the
 * Shuman filter on every region whose nTRgType is not 1. */
int wolfd2gpu_filter_t(w2_ctx *ctx, const int *nx, const int *ny, const int *nTRgType,
                       const double *fp, double *t);

/* EqState, src/thermal.f:288-290: den on i, j = 2..n (other entries kept). */
int wolfd2gpu_eq_state(w2_ctx *ctx, const int *nx, const int *ny,
                       const double *uref, const double *densref,
                       const double *tmax, const double *tref,
                       const double *rconst, const double *p, const double *t,
                       double *den);

/* SmallScale, src/small_scale.f:31-49 (Additive Turbulent Decomposition):
 * the small-scale fields uss, vss, pss, tss, updated in place, from the
 * large-scale u1, v1, t1 (all (0:mnx,0:mny) host arrays); arguments in the
 * reference's order without the region tables, dBCVal and metrics (the ones
 * given to wolfd2gpu_create and uploaded); fp is fp(1..4) of the reference
 * (u, v, unused, t).  The map iterates and cell areas persist in the
 * context between calls, as the reference keeps them (SAVE); initflg <= 0
 * seeds them (and zeroes uss, vss, tss), initflg < 0 returns after that.
 * nSorConv (no counterpart in the reference's argument list) receives the
 * small-scale Ppe's count.  pow, tanh and atanh are CUDA's, an ulp or so
 * from the host's, and the chaotic maps amplify such differences.  An
 * outlet on the grid's edge, where the reference's SmlSclBC would write
 * outside its arrays, returns W2_E_UNSUPPORTED. */
int wolfd2gpu_small_scale(w2_ctx *ctx, const int *nx, const int *ny, const int *initflg,
                          const int *nthermen, const int *lCartesGrid, const int *nTRgType,
                          const int *nTemBdTp, const int *nPpeSolver, const int *msorit,
                          const double *dlref, const double *uref, const double *tref,
                          const double *tmax, const double *dka, const double *re,
                          const double *pe, const double *sortol, const double *sorrel,
                          const double *fp, const double *cu0, const double *TsCoef,
                          const double *HsCoef, const double *TemCoef, const double *bnumc,
                          const double *rmax, const double *rlc, const double *dTRgVal,
                          const double *u1, const double *v1, const double *t1, double *uss,
                          double *vss, double *pss, double *tss, int *nSorConv);

/* ---- Device-resident time loop ---------------------------------------- */

/* Thermal switches and constants of the time loop (ReadParam, parse.f:118-159;
 * pe = re * Prandtl, file_manip.f:158; EqState's uref, densref, tmax, tref,
 * rconst). */
typedef struct {
  int nthermen, neqstate, nmeiter;
  double dmeittol, pe, uref, densref, tmax, tref, rconst;
  int nfiltt;         /* Filter of t after the iterations (main.f:889-893) */
  double fpt;
} w2_thermal;

/* Switch the device-resident time loop to main.f's path with the energy
 * equation (nthermen = 1) and/or the equation of state (neqstate = 1):
 * momentum/energy iterations (up to nmeiter, ended by dmeittol, main.f:736-879)
 * with ThermEnergy, EqState and the buoyancy term of YMomentum, then
 * TempBoundCond (and Filter of t with nfiltt = 1).  Tables as for
 * wolfd2gpu_therm_energy.  tp = NULL (or both switches 0) returns to the
 * plain loop.  The temperature and density start
 * at zero; wolfd2gpu_load_thermal / wolfd2gpu_store_thermal move them
 * ((0:mnx,0:mny) host arrays, d may be NULL).  Plain FP64 only, no Filter. */
int wolfd2gpu_set_thermal(w2_ctx *ctx, const w2_thermal *tp, const int *nTRgType,
                          const int *nTemBdTp, const double *dTRgVal,
                          const double *dHGSTval);
int wolfd2gpu_load_thermal(w2_ctx *ctx, const double *t, const double *d);
int wolfd2gpu_store_thermal(w2_ctx *ctx, double *t, double *d);

/* Snapshots streamed from the device (no reference counterpart; the output
 * and restart path of main.f copies the host arrays).  wolfd2gpu_snapshot
 * queues copies of the current time level -- u, v, p, and t, d (may be NULL)
 * with the energy equation -- into (0:mnx,0:mny) host arrays on a copy stream
 * and returns at once; steps called after it run while the copy proceeds,
 * and the first work that overwrites that level waits for it.  Use
 * page-locked host arrays for a copy that overlaps the steps.
 * wolfd2gpu_snapshot_wait blocks until the arrays are filled (then write
 * the Plot3D solution or restart file from them). */
int wolfd2gpu_snapshot(w2_ctx *ctx, double *u, double *v, double *p, double *t,
                       double *d);
int wolfd2gpu_snapshot_wait(w2_ctx *ctx);

/* Run parameters of the time loop (main.f with nthermen = 0). */
typedef struct {
  double dk, re, fr, qtol, sortol, sorrel, fpu, fpv;
  int mqiter, npsolver, msorit, nfiltu, nfiltv, lcartes;
  int precision;      /* W2_PREC_*                                        */
  int refine_sweeps;  /* mixed: FP32 sweeps per refinement pass (0=auto) */
  double refine_tol;  /* reserved, pass 0                                */
} w2_params;

/* Per-step results of main.f:753-966. */
typedef struct {
  int nQLiter, nSorConv;
  double dif[4];      /* DiffMaxNorm of (pn,p), (un,u), (vn,v), (tn,t)  */
  double divmax;      /* max |Divergence(u,v)| (pressure.f:287-299) over
                         the pressure cells of the projected field; no
                         counterpart in the reference                    */
  double divmax_int;  /* the same over the interior cells: the four
                         neighbours are Poisson unknowns and the four
                         faces are set by Project, so the divergence is
                         dk times the Poisson residual.  Cells touching a
                         boundary also carry the fixed face values and
                         the ghost pressures Ppe holds frozen during the
                         solve, which no tolerance removes             */
} w2_stepstat;

/* Copy u, v, p (0:mnx,0:mny host arrays) to / from the device state. */
int wolfd2gpu_load_fields(w2_ctx *ctx, const double *u, const double *v,
                          const double *p);
int wolfd2gpu_store_fields(w2_ctx *ctx, double *u, double *v, double *p);

/* Cold-start projection, main.f:606-641; *nSorConv out. */
int wolfd2gpu_cold_start(w2_ctx *ctx, const w2_params *prm, int *nSorConv);

/* nsteps passes of the time loop body, main.f:693-972, on device-resident
 * fields.  stats (may be NULL) receives one record per step.  Returns
 * W2_E_DIVERGED at the first step whose max difference exceeds 1e12. */
int wolfd2gpu_step(w2_ctx *ctx, const w2_params *prm, int nsteps,
                   w2_stepstat *stats);

/* CUDA graphs for wolfd2gpu_step (on by default; no reference counterpart).
 * When enabled, a call's launch sequence is captured once and replayed by
 * later calls that bake in the same launches: same starting time level,
 * step count, parameters, and device state (any re-tuning, metric upload or
 * face profile makes a new capture).  Profiling (wolfd2gpu_profile) uses
 * direct launches. */
int wolfd2gpu_set_graph(w2_ctx *ctx, int enable);

/* ---- Adjoint (no reference counterpart) --------------------------------
 * wolfd2gpu_step_counts: nsteps plain steps with the iteration counts fixed
 * per step (counts[2s] Q-L iterations, counts[2s+1] SOR sweeps; no
 * convergence test stops them earlier): the map whose derivative the adjoint
 * gives, for finite-difference checks.
 * wolfd2gpu_adjoint: from the loaded fields, runs nsteps plain FP64 steps
 * (checkpointing the fields every `every` steps and recording each step's
 * counts into counts[2*nsteps] when not NULL), evaluates
 *   J = 0.5 * weight * (sum of u^2 over i=1..nx, j=2..ny
 *                       + sum of v^2 over i=2..nx, j=1..ny)
 * at the final step, and returns dJ/du, dJ/dv, dJ/dp of the initial fields
 * ((0:mnx,0:mny) host arrays, any of them may be NULL) and dJ/d(face values)
 * of the face profile (ireg, jreg, face, var) in gprof[0..nprof) (positions
 * as wolfd2gpu_set_face_profile).  The derivative is that of the step with
 * the recorded counts held fixed; the context ends at the final state.
 * Limits: ppe_solver rb_sor (5), Cartesian grids, no Filter. */
int wolfd2gpu_step_counts(w2_ctx *ctx, const w2_params *prm, int nsteps,
                          const int *counts, w2_stepstat *stats);
int wolfd2gpu_adjoint(w2_ctx *ctx, const w2_params *prm, int nsteps, int every,
                      double weight, double *J, double *gu, double *gv, double *gp,
                      int ireg, int jreg, int face, int var, double *gprof, int nprof,
                      int *counts);

/* Self-test of the device-wait limit (no reference counterpart): runs a
 * grid barrier that one of its two blocks never reaches; the waiting block
 * gives up after the limit (4 s) and the call returns W2_E_TIMEOUT with the
 * barrier state cleared, the context still usable.  Nothing faults or hangs. */
int wolfd2gpu_selftest_wait(w2_ctx *ctx);

/* Synchronise the context stream; returns the first pending error. */
int wolfd2gpu_sync(w2_ctx *ctx);

/* Last error message of this context (static storage of the context). */
const char *wolfd2gpu_last_error(w2_ctx *ctx);

/* Library configuration knobs (segment length and warm-up of the chain
 * recurrence, threads per block, blocks per SM); 0 keeps the default.
 * blocks_per_sm = -1 selects the one-colour-per-barrier red/black sweep,
 * -2 forces the tiled two-sweeps-per-barrier form at any grid size, -3 runs
 * that form in 1024-thread blocks (two points in flight per thread instead
 * of four in 512-thread blocks), -4 returns to 512-thread blocks.  For the
 * mixed Poisson solve with general rows, -5 selects the form with one grid
 * barrier per colour on Cartesian grids too, -6 returns to the tiled form
 * (four sweeps per grid barrier; the default on Cartesian grids).
 * Takes effect on the next launch. */
int wolfd2gpu_tune(w2_ctx *ctx, int chain_seg, int chain_warm, int threads,
                   int blocks_per_sm);

/* Per-position values on one region face (no counterpart in the reference,
 * whose faces carry one constant per variable; used for the parabolic
 * inflow and the lid profile of the benchmark decks): the inlet or
 * moving-wall value of variable var (1 = u, 2 = v) at position pos along the
 * face -- j on west/east faces, i on south/north faces -- becomes
 * values[pos], pos = 0..n-1 (n = ny+2 or nx+2).  values = NULL restores the
 * region constant dBCVal.  At most 16 profiles per context. */
int wolfd2gpu_set_face_profile(w2_ctx *ctx, int ireg, int jreg, int face, int var,
                               const double *values, int n);

/* Precision of the drop-in wolfd2gpu_ppe on this context (W2_PREC_*) and
 * FP32 sweeps per refinement pass (0 = auto).  No counterpart in the
 * reference, whose Ppe is FP64 only. */
int wolfd2gpu_set_precision(w2_ctx *ctx, int precision, int refine_sweeps);

/* Mixed Poisson kernel shape: sweeps between grid barriers (4 or 8; the
 * halo is twice that), the largest block the tile planner may use
 * (64..512 threads; 0 keeps the current value), and the tile mode: 0 = one
 * tile per block when the grid allows it, else several tiles per block;
 * 1 = always several tiles per block; 2 = the same on at most 16 blocks
 * (a test shape); 3 = one tile per block, two blocks per SM (at most 256
 * threads each).  Tiles are re-planned. */
int wolfd2gpu_tune_mixed(w2_ctx *ctx, int sweeps_per_barrier, int threads,
                         int mode);

/* Staging of the mixed Poisson boxes in the several-tiles-per-block mode
 * (the 4096 x 1024 channel, ensembles): enable = 1 (default) loads each
 * tile's boxes with TMA tensor copies, 0 with per-thread vector loads.  The
 * results are the same bit for bit.  No counterpart in the reference. */
int wolfd2gpu_set_tma(w2_ctx *ctx, int enable);

/* Device pointers of the resident u, v, p fields and the device leading
 * dimension (elements), for callers that bring their own device buffers. */
int wolfd2gpu_device_fields(w2_ctx *ctx, double **u, double **v, double **p,
                            int *ld);

/* Kernel launches issued so far by this context (for accounting). */
long long wolfd2gpu_launch_count(w2_ctx *ctx);

/* Chain-solver statistics since the last call (then reset): the most
 * verification rounds any chain solve needed (at most the segment count;
 * one more than that would mean the sequential guard walk ran) and the
 * number of such guard walks (0 in a correct build). */
int wolfd2gpu_chain_stats(w2_ctx *ctx, int *max_rounds, int *fallbacks);

/* The context's CUDA stream (a cudaStream_t), for callers that time or
 * order work against it. */
void *wolfd2gpu_stream(w2_ctx *ctx);

/* Per-kernel timing with CUDA events recorded on the context stream around
 * every launch of the time loop.  Kinds: */
#define W2_K_MOMENTUM 0  /* nAuxMomentum persistent kernel        */
#define W2_K_PPE      1  /* Ppe persistent kernel                 */
#define W2_K_POST     2  /* Project + boundary rows + step norms  */
#define W2_K_BC       3  /* one-block boundary programs           */
#define W2_K_COPY     4  /* time-level copies                     */
#define W2_K_THERM    5  /* ThermEnergy and EqState               */
#define W2_K_NKINDS   6
int wolfd2gpu_profile(w2_ctx *ctx, int enable);
/* Accumulated device time (ms) and launch count of one kind since the last
 * wolfd2gpu_profile(ctx, 1); synchronises the context stream. */
int wolfd2gpu_profile_read(w2_ctx *ctx, int kind, double *total_ms,
                           long long *count);

/* ---- Ensembles (no reference counterpart) -----------------------------
 * Many independent cases advanced together: one launch per stage covers
 * every case, each case on its own group of the launch's blocks (a ragged
 * partition sized by the cases' cells), with its own barriers, convergence
 * tests and iteration counts.  Each case is an ordinary context, set up as
 * usual (metrics, regions, fields).  One call steps every case in the same
 * precision: W2_PREC_MIXED (rb_sor or rb_sorp in every case; unit-row
 * cases on the multi-tile kernel, which needs a Cartesian grid, the others
 * on the general-row kernel) or W2_PREC_FP64 (any grid and any of the six
 * Poisson solvers, per case).  Filter (nfiltu, nfiltv) runs per case.
 * Per case, results are bit-identical to wolfd2gpu_step on that context
 * alone.
 *
 * wolfd2gpu_ens_create: cases[n]; threads per block (0: 128) and Poisson
 *   sweeps per barrier (0: 4) of every launch.  The contexts must outlive
 *   the ensemble; their own calls must not overlap an ensemble call.
 * wolfd2gpu_ens_step: prm[n] (one per case), nsteps steps; stats (may be
 *   NULL) receives n*nsteps records, case-major.  Returns W2_E_DIVERGED if
 *   a case's max step difference exceeds 1e12 (the case halts; the others
 *   continue) and the first device error otherwise.
 * wolfd2gpu_ens_graph: when enabled, one step's launch sequence is captured
 *   in a CUDA graph on the first call and replayed every step.
 * wolfd2gpu_ens_info: blocks of the momentum and (mixed) Poisson launches
 *   (the plain Poisson launch uses the momentum partition), device
 *   milliseconds of the last ens_step call (CUDA events around its steps),
 *   and kernel launches so far. */
typedef struct w2_ens w2_ens;
int wolfd2gpu_ens_create(w2_ens **out, w2_ctx *const *cases, int n, int threads,
                         int sweeps_per_barrier);
int wolfd2gpu_ens_step(w2_ens *ens, const w2_params *prm, int nsteps,
                       w2_stepstat *stats);
int wolfd2gpu_ens_graph(w2_ens *ens, int enable);
int wolfd2gpu_ens_info(w2_ens *ens, int *blocks_momentum, int *blocks_poisson,
                       double *last_ms, long long *launches);
/* Per-stage device time of direct (not graph) ensemble launches, CUDA
 * events on the ensemble's stream: enable (resets the sums), then read the
 * total milliseconds and launch count of a stage. */
enum { W2_ENS_COPY = 0, W2_ENS_MOMENTUM = 1, W2_ENS_BC = 2, W2_ENS_PPE = 3, W2_ENS_POST = 4,
       W2_ENS_NSTAGES = 5 };
int wolfd2gpu_ens_profile(w2_ens *ens, int enable);
int wolfd2gpu_ens_profile_read(w2_ens *ens, int stage, double *total_ms, long long *count);
const char *wolfd2gpu_ens_error(w2_ens *ens);
int wolfd2gpu_ens_destroy(w2_ens *ens);

/* ---- Allocation-free entry point ---------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * -- a driver that gives all device memory to its own pool at start-up, or
 * code that must not reach the allocator inside its solve loop -- and so
 * cannot create a w2_ctx.  Runs red/black point SOR (nPpeSolver 5 or 6,
 * pressure.f:457-656, with the divergence and b = div/dk of Ppe) on device
 * arrays the caller owns, all in the reference layout with leading dimension
 * ld (elements) and rows j = 0..ny+1: metrics rau, rgv, xeu, yeu, xzv, yzv,
 * velocities u, v, and p (updated in place).  The only scratch is a fixed
 * static device array of W2_NOALLOC_MAX_POINTS doubles plus barrier state
 * (about 9.6 MB, held by every device that loads the library until the
 * process exits); the call makes no allocation.  Limits: Cartesian grids,
 * no blockage regions, ld*(ny+2) <= W2_NOALLOC_MAX_POINTS (else W2_E_SIZE).
 * Every call looks up the scratch's address on the current device
 * (cudaGetSymbolAddress, which allocates nothing).  All calls share the
 * scratch: calls that overlap on the GPU race, so serialise them.
 * stream is a cudaStream_t (NULL = legacy default stream); the call
 * synchronises it and copies its status to the host before returning
 * nSorConv, so it cannot be used inside stream or graph capture. */
#define W2_NOALLOC_MAX_POINTS 1200000
int wolfd2gpu_ppe_rbsor_noalloc(int nx, int ny, int ld, int lCartesGrid,
                                int nPpeSolver, int msorit, double dk,
                                double sortol, double sorrel,
                                const double *rau, const double *rgv,
                                const double *xeu, const double *yeu,
                                const double *xzv, const double *yzv,
                                const double *u, const double *v, double *p,
                                int *nSorConv, void *stream);

#ifdef __cplusplus
}
#endif
#endif
