/*
 * wolfd2_oracle.h -- CPU oracle for the wolfd2 projection-method time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran routines on the hot path (momentum.f, pressure.f, utility.f,
 * bound_cond.f, thermal.f and the time-loop body of main.f).  It exists so the tests,
 * the smoke check and the CPU-baseline leg of the benchmark can check the
 * CUDA library against an independent implementation.  Nothing in the
 * product (wolfd2_gb300/, include/) links or calls it.
 *
 * Parity pinning: the reference ships no tests, golden vectors or sample
 * decks, and no Fortran compiler exists on the build or GPU machines, so the
 * restatement cannot be checked against the compiled reference.  It is
 * checked instead against a mechanical Fortran-77-to-C translation of the
 * reference's own source files (oracle/f77c.py, output in oracle/_ref/, built
 * only where the reference source tree is present) -- see the tests.  Where
 * that translation is absent, parity is unpinned.
 *
 * Storage follows the reference: every field is REAL*8 (0:mnx,0:mny),
 * column-major, element (i,j) at offset i + j*(mnx+1).  Region tables keep
 * their Fortran shapes: nRegBrd(mgri,mgrj,4), nRegType(mgri,mgrj),
 * nMomBdTp(mgri,mgrj,4), dBCVal(mgri,mgrj,4,4), porous coefficients
 * (mgri,mgrj).  All work arrays live in an oracle context, zero-initialised
 * once and persistent across calls, which reproduces the static storage the
 * reference's large local arrays get from gfortran (some entries, e.g.
 * cj1(nx+1,j), are read but never written and must stay zero).
 *
 * Build: cc -O2 -ffp-contract=off (op-by-op IEEE double, no FMA), see
 * oracle/Makefile.
 */
#ifndef WOLFD2_ORACLE_H
#define WOLFD2_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct w2o_ctx w2o_ctx;

/* Region / boundary tables, Fortran layout (see include/wolfd2.h). */
typedef struct {
  int mgri, mgrj;          /* leading dimensions (20, 10 in config.f) */
  const int *nReg;         /* nReg(2)                                  */
  const int *nRegBrd;      /* nRegBrd(mgri,mgrj,4)                     */
  const int *nRegType;     /* nRegType(mgri,mgrj)                      */
  const int *nMomBdTp;     /* nMomBdTp(mgri,mgrj,4)                    */
  const double *dBCVal;    /* dBCVal(mgri,mgrj,4,4)                    */
  const double *dPRporos;  /* dPRporos(mgri,mgrj)                      */
  const double *dPRporc1;
  const double *dPRporc2;
  /* Per-position face values (no counterpart in the reference): NULL, or
   * mgri*mgrj*4*2 pointers, entry ((ir-1) + (jr-1)*mgri + (face-1)*mgri*mgrj)*2
   * + (var-1) (var 1 = u, 2 = v), each NULL or the values at position pos
   * along the face (j on west/east, i on south/north faces).  They replace
   * dBCVal in VelBoundCond's inlet and moving-wall rows. */
  const double *const *prof;
} w2o_regions;

/* The 30 metric arrays produced by grid.f:Metric, each (0:mnx,0:mny). */
typedef struct {
  double *ran, *rbn, *rgn, *rac, *rbc, *rgc, *rau, *rbu, *rbv, *rgv;
  double *dju, *djv, *djc, *djn;
  double *xen, *yen, *xzn, *yzn, *xec, *yec, *xzc, *yzc;
  double *xeu, *yeu, *xzv, *yzv, *xzu, *yzu, *xev, *yev;
} w2o_metrics;

/* The metric arrays rounded to single precision (the FP32 momentum's input). */
typedef struct {
  float *ran, *rbn, *rgn, *rac, *rbc, *rgc, *rau, *rbu, *rbv, *rgv;
  float *dju, *djv, *djc, *djn;
  float *xen, *yen, *xzn, *yzn, *xec, *yec, *xzc, *yzc;
  float *xeu, *yeu, *xzv, *yzv, *xzu, *yzu, *xev, *yev;
} w2o_metrics32;

w2o_ctx *w2o_create(int mnx, int mny);
void w2o_destroy(w2o_ctx *c);

/* grid.f:31-127 minus file reading: gx,gy hold nodes (1..nx,1..ny), already
 * divided by dlref; mirror points are added in place. */
void w2o_grid(w2o_ctx *c, int nx, int ny, double *gx, double *gy,
              w2o_metrics *m);

/* momentum.f:33-193 */
int w2o_naux_momentum(w2o_ctx *c, int nx, int ny, int mqiter,
                      const w2o_regions *r, double dk, double re, double fr,
                      double qtol, const w2o_metrics *m, const double *d,
                      const double *dn, const double *un, const double *vn,
                      double *us, double *vs);

/* nAuxMomentum in single precision: every operation of w2o_naux_momentum in
 * IEEE single (FP32 fields and metrics, literals and dk, re, fr rounded to
 * single); the stopping test compares against qtol in double. */
int w2o_naux_momentum_f32(w2o_ctx *c, int nx, int ny, int mqiter,
                          const w2o_regions *r, double dk, double re,
                          double fr, double qtol, const w2o_metrics32 *m,
                          const float *d, const float *dn, const float *un,
                          const float *vn, float *us, float *vs);
void w2o_vel_outflow_bcs_f32(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                             float *u, float *v);

/* pressure.f:30-249; returns nSorConv */
int w2o_ppe(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
            int lcartes, int npsolver, int msorit, double dk, double sortol,
            double sorrel, const w2o_metrics *m, const double *u,
            const double *v, double *p);

/* utility.f:253-440 */
void w2o_project(w2o_ctx *c, int nx, int ny, const w2o_regions *r, double dk,
                 const w2o_metrics *m, const double *p, double *u, double *v);

/* bound_cond.f:511-847, 853-1024, 1656-1874 */
void w2o_vel_bound_cond(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                        double *u, double *v);
void w2o_pres_bound_cond(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                         double *p);
void w2o_vel_outflow_bcs(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                         double *u, double *v);

/* utility.f:33-247 (ncomp 1=u, 2=v) */
void w2o_filter(w2o_ctx *c, int nx, int ny, int ncomp, const w2o_regions *r,
                double fp, double *q);

/* utility.f:446-507 */
double w2o_diff_max_norm(w2o_ctx *c, int nx, int ny, const double *un,
                         const double *u);
double w2o_dmax_norm(w2o_ctx *c, int nx, int ny, const double *u);

/* Thermal region and boundary tables, Fortran layout (mgri, mgrj of the
 * regions): nTRgType(mgri,mgrj) (RT_NOSRCE 0, RT_HEATGN 1, RT_TEMPER 2),
 * nTemBdTp(mgri,mgrj,4) (BT_INTERN 0, BT_TEMPER 1, BT_HTFLUX 2),
 * dTRgVal(mgri,mgrj), dHGSTval(mgri,mgrj).  Face values are dBCVal's
 * variable 4 (_T_). */
typedef struct {
  const int *nTRgType;
  const int *nTemBdTp;
  const double *dTRgVal;
  const double *dHGSTval;
} w2o_thermal;

/* bound_cond.f:1030-1186 */
void w2o_temp_bound_cond(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                         const w2o_thermal *th, double *t);

/* thermal.f:24-280 (t: the starred temperature, updated in place) */
void w2o_therm_energy(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                      const w2o_thermal *th, double dk, double pe,
                      const w2o_metrics *m, const double *un, const double *vn,
                      const double *u, const double *v, const double *tn,
                      double *t);

/* thermal.f:288-329 */
void w2o_eq_state(w2o_ctx *c, int nx, int ny, double uref, double densref, double tmax,
                  double tref, double rconst, const double *p, const double *t, double *den);

/* momentum.f:1307-1339 (exported for unit tests) */
void w2o_alt_trid_lu(int n, double *a /* a(3,n) */, double *b);

/* Time-loop parameters (main.f with nsmallscl = 0). */
typedef struct {
  double dk, re, fr, qtol, sortol, sorrel, fpu, fpv;
  int mqiter, npsolver, msorit, nfiltu, nfiltv, lcartes;
} w2o_params;

/* Thermal switches and constants of the time loop (ReadParam, parse.f:118-159
 * defaults; pe = re * Prandtl, file_manip.f:158). */
typedef struct {
  int nthermen, neqstate, nmeiter;
  double dmeittol, pe, uref, densref, tmax, tref, rconst;
  int nfiltt;    /* Filter of t after the iterations (main.f:889-893) */
  double fpt;
} w2o_thermal_params;

/* Filter of a scalar (utility.f:33-247, ncomp = _T_): every region whose
 * nTRgType is not 1 (the reference compares with BT_TEMPER = 1). */
void w2o_filter_t(w2o_ctx *c, int nx, int ny, const w2o_regions *r, const w2o_thermal *th,
                  double fp, double *q);

/* Fields of the time loop, each (0:mnx,0:mny). */
typedef struct {
  double *u, *v, *p, *t, *un, *vn, *pn, *tn, *us, *vs, *ts, *d, *dn;
} w2o_fields;

/* main.f:606-641 (cold-start projection) */
int w2o_cold_start(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                   const w2o_params *prm, const w2o_metrics *m,
                   w2o_fields *f);

/* main.f:690-972 for one step; returns 0, or 1 when 'Solution diverged'. */
int w2o_step(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
             const w2o_params *prm, const w2o_metrics *m, w2o_fields *f,
             int *nQLiter, int *nSorConv, double dif[4]);

/* The same with the thermal energy equation: momentum/energy iterations
 * (main.f:736-879: ThermEnergy, EqState, the ME convergence test), and
 * TempBoundCond after them.  th/tp NULL or nthermen = 0 is w2o_step. */
int w2o_step_thermal(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                     const w2o_thermal *th, const w2o_thermal_params *tp,
                     const w2o_params *prm, const w2o_metrics *m, w2o_fields *f,
                     int *nQLiter, int *nSorConv, double dif[4]);

/* Small-scale (ATD) model parameters: parse.f's ss* keywords (defaults
 * parse.f:144-178), the reference scales, and main.f's dk passed as dka. */
typedef struct {
  int npsolver, msorit, lcartes;   /* nssPpeSlvr, mssSorIt, lCartesGrid   */
  double dlref, uref, tref, tmax, dka, re, pe, sortol, sorrel;
  double fp[4];                    /* ssFiltPar(_U_.._T_); fp[2] unused   */
  double cu0, tscoef, hscoef, temcoef, bnumc, rmax, rlc;
} w2o_atd_params;

/* What small_scale.f keeps between calls (its SAVE): the three logistic-map
 * iterates per cell for each of u, v, t, the cell areas and their sum, and
 * the work arrays (whose unwritten borders stay zero). */
typedef struct w2o_atd w2o_atd;
w2o_atd *w2o_atd_create(int mnx, int mny);
void w2o_atd_destroy(w2o_atd *s);

/* bound_cond.f:1211-1500 (image-point conditions of the small scales;
 * PresBoundCond for p).  A west or south outlet on the grid's edge, where
 * the reference writes outside its arrays, stops with a message. */
void w2o_sml_scl_bc(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                    const w2o_thermal *th, double *u, double *v, double *p,
                    double *t);

/* small_scale.f:31-578.  initflg <= 0 seeds the maps and the areas and
 * zeroes uss, vss, tss (initflg < 0 stops there); u1, v1, t1 are the large
 * scales.  Returns the small-scale Ppe's nSorConv (0 when initflg < 0). */
int w2o_small_scale(w2o_ctx *c, w2o_atd *s, int nx, int ny, int initflg,
                    const w2o_regions *r, const w2o_thermal *th,
                    const w2o_atd_params *ap, const w2o_metrics *m,
                    const double *u1, const double *v1, const double *t1,
                    double *uss, double *vss, double *pss, double *tss);

/* The small scales carried by the time loop (main.f's nsmallscl = 1): the
 * model's saved state and parameters, uss, vss, pss, tss and their level-n
 * copies usn, vsn, tsn, each (0:mnx,0:mny).  Seed them after the cold start
 * with w2o_small_scale(initflg 0) on u, v, t. */
typedef struct {
  w2o_atd *state;
  const w2o_atd_params *ap;
  double *uss, *vss, *pss, *tss, *usn, *vsn, *tsn;
} w2o_atd_run;

/* w2o_step_thermal with the small scales (main.f:708-730, 898-940): added to
 * the level-n fields before the iterations, removed from the new fields and
 * recomputed by SmallScale after them, then added back; a NULL run is
 * w2o_step_thermal.  The thermal tables th are required with a run. */
int w2o_step_atd(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                 const w2o_thermal *th, const w2o_thermal_params *tp,
                 const w2o_params *prm, const w2o_metrics *m, w2o_fields *f,
                 const w2o_atd_run *a, int *nQLiter, int *nSorConv, double dif[4]);

#ifdef __cplusplus
}
#endif
#endif
