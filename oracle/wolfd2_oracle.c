/*
 * wolfd2_oracle.c -- TEST INFRASTRUCTURE: CPU restatement of the reference's
 * projection-method time step.  See wolfd2_oracle.h for the scope, the
 * storage conventions and the parity-pinning status.
 *
 * Every routine names the reference file:line it restates.  Expressions keep
 * the reference's evaluation order (Fortran evaluates same-precedence
 * operators left to right and this file is compiled without FMA
 * contraction), so results are the IEEE-double results of the reference
 * source as written.
 */
#include "wolfd2_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* Region and boundary enums, include/wolfd2.h:15-60 */
enum { RM_BLOCKG = 0, RM_INTERN = 1, RM_POROUS = 2 };
enum { BM_INTERN = 0, BM_WALL1 = 1, BM_WALL2 = 2, BM_INLET = 3,
       BM_OUTLT1 = 4, BM_OUTLT2 = 5 };
enum { WEST = 1, EAST = 2, SOUTH = 3, NORTH = 4 };
enum { VU = 1, VV = 2, VP = 3, VT = 4 };
enum { RT_NOSRCE = 0, RT_HEATGN = 1, RT_TEMPER = 2 };
enum { BT_INTERN = 0, BT_TEMPER = 1, BT_HTFLUX = 2 };

/* Persistent work storage (the reference's static locals). */
typedef struct {
  double *cj1, *cj2, *c1s, *c2s, *c1n, *c2n, *cps, *cpn, *cpj;
  double *cnvs, *difs, *cnvn, *difn;
  double *a; /* a(3,mn) */
  double *b; /* b(mn)   */
} w2o_mom_ws;

typedef struct {
  float *cj1, *cj2, *c1s, *c2s, *c1n, *c2n, *cps, *cpn, *cpj;
  float *cnvs, *difs, *cnvn, *difn;
  float *a, *b;
} w2o_mom_ws32;

struct w2o_ctx {
  int mnx, mny;
  size_t ld, nf; /* leading dimension mnx+1 and field size */
  size_t mn;     /* mnx*mny (chain workspace length) */
  w2o_mom_ws wx, wy;       /* XMomentum / YMomentum statics            */
  double *dus, *dvs;       /* nAuxMomentum statics                     */
  w2o_mom_ws32 wx32, wy32; /* the same in single precision             */
  float *dus32, *dvs32;
  double *div, *pa, *pb;   /* Ppe statics: div, a(mn,5), b(mn)         */
  double *rbp_pn;          /* SlorRBP static pn(0:mnx,0:mny)           */
  double *qh;              /* Filter static qh                         */
  double *xu, *yu, *xv, *yv, *xc, *yc; /* Grid statics              */
  double *lin;             /* aline/bline/plold for the line solvers   */
  double *rbp_dif;         /* SorRBP dif(0:nx+1,0:ny+1)                */
  double *th_cu1, *th_cv1, *th_cun, *th_cvn, *th_s; /* ThermEnergy statics */
  double *th_a, *th_b;     /* ThermEnergy a(3,mn), b(mn)               */
};

#define IX(i, j) ((size_t)(i) + (size_t)(j) * c->ld)
#define F(a, i, j) (a)[IX(i, j)]

/* Region-table accessors (Fortran column-major, 1-based). */
#define RBRD(r, ir, jr, s) \
  (r)->nRegBrd[((ir)-1) + ((jr)-1) * (r)->mgri + ((s)-1) * (r)->mgri * (r)->mgrj]
#define RTYP(r, ir, jr) (r)->nRegType[((ir)-1) + ((jr)-1) * (r)->mgri]
#define MBTP(r, ir, jr, s) \
  (r)->nMomBdTp[((ir)-1) + ((jr)-1) * (r)->mgri + ((s)-1) * (r)->mgri * (r)->mgrj]
#define BCV(r, ir, jr, s, var)                                            \
  (r)->dBCVal[((ir)-1) + ((jr)-1) * (r)->mgri + ((s)-1) * (r)->mgri * (r)->mgrj + \
              ((var)-1) * (r)->mgri * (r)->mgrj * 4]
#define RPAR(arr, r, ir, jr) (r)->arr[((ir)-1) + ((jr)-1) * (r)->mgri]
/* A face value at position pos: the per-position profile when one is set
 * (test shim for inflow and lid profiles), else the region constant. */
#define PKEY(r, ir, jr, s, var) \
  ((((ir)-1) + ((jr)-1) * (r)->mgri + ((s)-1) * (r)->mgri * (r)->mgrj) * 2 + ((var)-1))
#define BCVP(r, ir, jr, s, var, pos)                                   \
  (((r)->prof && (r)->prof[PKEY(r, ir, jr, s, var)])                   \
       ? (r)->prof[PKEY(r, ir, jr, s, var)][pos]                       \
       : BCV(r, ir, jr, s, var))

static void die(const char *msg, int ir, int jr) {
  fprintf(stderr, "%s in region %d,%d\n", msg, ir, jr);
  exit(2);
}

static double *zalloc(size_t n) {
  double *p = (double *)calloc(n ? n : 1, sizeof(double));
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    exit(3);
  }
  return p;
}

static void mom_ws_init(w2o_mom_ws *w, size_t nf, size_t mn) {
  w->cj1 = zalloc(nf); w->cj2 = zalloc(nf); w->c1s = zalloc(nf);
  w->c2s = zalloc(nf); w->c1n = zalloc(nf); w->c2n = zalloc(nf);
  w->cps = zalloc(nf); w->cpn = zalloc(nf); w->cpj = zalloc(nf);
  w->cnvs = zalloc(nf); w->difs = zalloc(nf); w->cnvn = zalloc(nf);
  w->difn = zalloc(nf);
  w->a = zalloc(3 * mn); w->b = zalloc(mn);
}

static float *zalloc32(size_t n) {
  float *p = (float *)calloc(n ? n : 1, sizeof(float));
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    exit(3);
  }
  return p;
}

static void mom_ws32_init(w2o_mom_ws32 *w, size_t nf, size_t mn) {
  w->cj1 = zalloc32(nf); w->cj2 = zalloc32(nf); w->c1s = zalloc32(nf);
  w->c2s = zalloc32(nf); w->c1n = zalloc32(nf); w->c2n = zalloc32(nf);
  w->cps = zalloc32(nf); w->cpn = zalloc32(nf); w->cpj = zalloc32(nf);
  w->cnvs = zalloc32(nf); w->difs = zalloc32(nf); w->cnvn = zalloc32(nf);
  w->difn = zalloc32(nf);
  w->a = zalloc32(3 * mn); w->b = zalloc32(mn);
}

static void mom_ws32_free(w2o_mom_ws32 *w) {
  free(w->cj1); free(w->cj2); free(w->c1s); free(w->c2s); free(w->c1n);
  free(w->c2n); free(w->cps); free(w->cpn); free(w->cpj); free(w->cnvs);
  free(w->difs); free(w->cnvn); free(w->difn); free(w->a); free(w->b);
}

static void mom_ws_free(w2o_mom_ws *w) {
  free(w->cj1); free(w->cj2); free(w->c1s); free(w->c2s); free(w->c1n);
  free(w->c2n); free(w->cps); free(w->cpn); free(w->cpj); free(w->cnvs);
  free(w->difs); free(w->cnvn); free(w->difn); free(w->a); free(w->b);
}

w2o_ctx *w2o_create(int mnx, int mny) {
  w2o_ctx *c = (w2o_ctx *)calloc(1, sizeof(w2o_ctx));
  c->mnx = mnx; c->mny = mny;
  c->ld = (size_t)mnx + 1;
  c->nf = c->ld * ((size_t)mny + 1);
  c->mn = (size_t)mnx * (size_t)mny;
  mom_ws_init(&c->wx, c->nf, c->mn);
  mom_ws_init(&c->wy, c->nf, c->mn);
  c->dus = zalloc(c->nf); c->dvs = zalloc(c->nf);
  mom_ws32_init(&c->wx32, c->nf, c->mn);
  mom_ws32_init(&c->wy32, c->nf, c->mn);
  c->dus32 = zalloc32(c->nf); c->dvs32 = zalloc32(c->nf);
  c->div = zalloc(c->nf); c->pa = zalloc(5 * c->mn); c->pb = zalloc(c->mn);
  c->rbp_pn = zalloc(c->nf); c->qh = zalloc(c->nf);
  c->xu = zalloc(c->nf); c->yu = zalloc(c->nf); c->xv = zalloc(c->nf);
  c->yv = zalloc(c->nf); c->xc = zalloc(c->nf); c->yc = zalloc(c->nf);
  size_t mnl = (size_t)(mnx > mny ? mnx : mny);
  c->lin = zalloc(5 * mnl);
  c->rbp_dif = zalloc(c->nf);
  c->th_cu1 = zalloc(c->nf); c->th_cv1 = zalloc(c->nf);
  c->th_cun = zalloc(c->nf); c->th_cvn = zalloc(c->nf);
  c->th_s = zalloc(c->nf);
  c->th_a = zalloc(3 * c->mn); c->th_b = zalloc(c->mn);
  return c;
}

void w2o_destroy(w2o_ctx *c) {
  if (!c) return;
  mom_ws_free(&c->wx); mom_ws_free(&c->wy);
  mom_ws32_free(&c->wx32); mom_ws32_free(&c->wy32);
  free(c->dus32); free(c->dvs32);
  free(c->dus); free(c->dvs); free(c->div); free(c->pa); free(c->pb);
  free(c->rbp_pn); free(c->qh); free(c->xu); free(c->yu); free(c->xv);
  free(c->yv); free(c->xc); free(c->yc); free(c->lin); free(c->rbp_dif);
  free(c->th_cu1); free(c->th_cv1); free(c->th_cun); free(c->th_cvn);
  free(c->th_s); free(c->th_a); free(c->th_b);
  free(c);
}

/* ------------------------------------------------------------------ */
/* grid.f                                                              */
/* ------------------------------------------------------------------ */

void w2o_grid(w2o_ctx *c, int nx, int ny, double *x, double *y,
              w2o_metrics *m) {
  int i, j;
  /* MirrorPts, grid.f:258-306 */
  for (i = 1; i <= nx; i++) {
    F(x, i, 0) = 2.0 * F(x, i, 1) - F(x, i, 2);
    F(x, i, ny + 1) = 2.0 * F(x, i, ny) - F(x, i, ny - 1);
    F(y, i, 0) = 2.0 * F(y, i, 1) - F(y, i, 2);
    F(y, i, ny + 1) = 2.0 * F(y, i, ny) - F(y, i, ny - 1);
  }
  for (j = 1; j <= ny; j++) {
    F(x, 0, j) = 2.0 * F(x, 1, j) - F(x, 2, j);
    F(x, nx + 1, j) = 2.0 * F(x, nx, j) - F(x, nx - 1, j);
    F(y, 0, j) = 2.0 * F(y, 1, j) - F(y, 2, j);
    F(y, nx + 1, j) = 2.0 * F(y, nx, j) - F(y, nx - 1, j);
  }
  F(x, 0, 0) = 2.0 * F(x, 1, 1) - F(x, 2, 2);
  F(y, 0, 0) = 2.0 * F(y, 1, 1) - F(y, 2, 2);
  F(x, 0, ny + 1) = 2.0 * F(x, 1, ny) - F(x, 2, ny - 1);
  F(y, 0, ny + 1) = 2.0 * F(y, 1, ny) - F(y, 2, ny - 1);
  F(x, nx + 1, 0) = 2.0 * F(x, nx, 1) - F(x, nx - 1, 2);
  F(y, nx + 1, 0) = 2.0 * F(y, nx, 1) - F(y, nx - 1, 2);
  F(x, nx + 1, ny + 1) = 2.0 * F(x, nx, ny) - F(x, nx - 1, ny - 1);
  F(y, nx + 1, ny + 1) = 2.0 * F(y, nx, ny) - F(y, nx - 1, ny - 1);

  /* FullGrid, grid.f:312-362 */
  double *xu = c->xu, *yu = c->yu, *xv = c->xv, *yv = c->yv, *xc = c->xc,
         *yc = c->yc;
  for (j = 1; j <= ny + 1; j++)
    for (i = 0; i <= nx + 1; i++) {
      F(xu, i, j) = 0.5 * (F(x, i, j) + F(x, i, j - 1));
      F(yu, i, j) = 0.5 * (F(y, i, j) + F(y, i, j - 1));
    }
  for (j = 0; j <= ny + 1; j++)
    for (i = 1; i <= nx + 1; i++) {
      F(xv, i, j) = 0.5 * (F(x, i, j) + F(x, i - 1, j));
      F(yv, i, j) = 0.5 * (F(y, i, j) + F(y, i - 1, j));
    }
  for (j = 1; j <= ny + 1; j++)
    for (i = 1; i <= nx + 1; i++) {
      F(xc, i, j) = 0.5 * (F(xu, i, j) + F(xu, i - 1, j));
      F(yc, i, j) = 0.5 * (F(yv, i, j) + F(yv, i, j - 1));
    }

  /* Metric, grid.f:368-535 */
  double g11, g12, g22;
  for (j = 1; j <= ny; j++)
    for (i = 1; i <= nx; i++) {
      F(m->xzn, i, j) = F(xv, i + 1, j) - F(xv, i, j);
      F(m->xen, i, j) = F(xu, i, j + 1) - F(xu, i, j);
      F(m->yzn, i, j) = F(yv, i + 1, j) - F(yv, i, j);
      F(m->yen, i, j) = F(yu, i, j + 1) - F(yu, i, j);
      F(m->djn, i, j) = 1.0 / (F(m->xzn, i, j) * F(m->yen, i, j) -
                               F(m->xen, i, j) * F(m->yzn, i, j));
      g11 = F(m->xzn, i, j) * F(m->xzn, i, j) + F(m->yzn, i, j) * F(m->yzn, i, j);
      g12 = F(m->xzn, i, j) * F(m->xen, i, j) + F(m->yzn, i, j) * F(m->yen, i, j);
      g22 = F(m->xen, i, j) * F(m->xen, i, j) + F(m->yen, i, j) * F(m->yen, i, j);
      F(m->ran, i, j) = F(m->djn, i, j) * g22;
      F(m->rbn, i, j) = -F(m->djn, i, j) * g12 * 0.25;
      F(m->rgn, i, j) = F(m->djn, i, j) * g11;
    }
  for (j = 1; j <= ny; j++)
    for (i = 1; i <= nx; i++) {
      F(m->xzu, i, j) = F(xc, i + 1, j) - F(xc, i, j);
      F(m->xeu, i, j) = F(x, i, j) - F(x, i, j - 1);
      F(m->yzu, i, j) = F(yc, i + 1, j) - F(yc, i, j);
      F(m->yeu, i, j) = F(y, i, j) - F(y, i, j - 1);
      F(m->dju, i, j) = 1.0 / (F(m->xzu, i, j) * F(m->yeu, i, j) -
                               F(m->xeu, i, j) * F(m->yzu, i, j));
      g11 = F(m->xzu, i, j) * F(m->xzu, i, j) + F(m->yzu, i, j) * F(m->yzu, i, j);
      g12 = F(m->xzu, i, j) * F(m->xeu, i, j) + F(m->yzu, i, j) * F(m->yeu, i, j);
      g22 = F(m->xeu, i, j) * F(m->xeu, i, j) + F(m->yeu, i, j) * F(m->yeu, i, j);
      (void)g11;
      F(m->rau, i, j) = F(m->dju, i, j) * g22;
      F(m->rbu, i, j) = -F(m->dju, i, j) * g12 * 0.25;
    }
  for (j = 1; j <= ny; j++)
    for (i = 1; i <= nx; i++) {
      F(m->xzv, i, j) = F(x, i, j) - F(x, i - 1, j);
      F(m->xev, i, j) = F(xc, i, j + 1) - F(xc, i, j);
      F(m->yzv, i, j) = F(y, i, j) - F(y, i - 1, j);
      F(m->yev, i, j) = F(yc, i, j + 1) - F(yc, i, j);
      F(m->djv, i, j) = 1.0 / (F(m->xzv, i, j) * F(m->yev, i, j) -
                               F(m->xev, i, j) * F(m->yzv, i, j));
      g11 = F(m->xzv, i, j) * F(m->xzv, i, j) + F(m->yzv, i, j) * F(m->yzv, i, j);
      g12 = F(m->xzv, i, j) * F(m->xev, i, j) + F(m->yzv, i, j) * F(m->yev, i, j);
      g22 = F(m->xev, i, j) * F(m->xev, i, j) + F(m->yev, i, j) * F(m->yev, i, j);
      (void)g22;
      F(m->rbv, i, j) = -F(m->djv, i, j) * g12 * 0.25;
      F(m->rgv, i, j) = F(m->djv, i, j) * g11;
    }
  for (j = 1; j <= ny; j++)
    for (i = 1; i <= nx; i++) {
      F(m->xzc, i, j) = F(xu, i, j) - F(xu, i - 1, j);
      F(m->xec, i, j) = F(xv, i, j) - F(xv, i, j - 1);
      F(m->yzc, i, j) = F(yu, i, j) - F(yu, i - 1, j);
      F(m->yec, i, j) = F(yv, i, j) - F(yv, i, j - 1);
      F(m->djc, i, j) = 1.0 / (F(m->xzc, i, j) * F(m->yec, i, j) -
                               F(m->xec, i, j) * F(m->yzc, i, j));
      g11 = F(m->xzc, i, j) * F(m->xzc, i, j) + F(m->yzc, i, j) * F(m->yzc, i, j);
      g12 = F(m->xzc, i, j) * F(m->xec, i, j) + F(m->yzc, i, j) * F(m->yec, i, j);
      g22 = F(m->xec, i, j) * F(m->xec, i, j) + F(m->yec, i, j) * F(m->yec, i, j);
      F(m->rac, i, j) = F(m->djc, i, j) * g22;
      F(m->rbc, i, j) = -F(m->djc, i, j) * g12 * 0.25;
      F(m->rgc, i, j) = F(m->djc, i, j) * g11;
    }
}

/* ------------------------------------------------------------------ */
/* momentum.f                                                          */
/* ------------------------------------------------------------------ */

/* DiffMaxNorm, utility.f:446-473 */
double w2o_diff_max_norm(w2o_ctx *c, int nx, int ny, const double *un,
                         const double *u) {
  double diff = fabs(F(un, 2, 2) - F(u, 2, 2));
  for (int j = 2; j <= ny - 1; j++)
    for (int i = 2; i <= nx - 1; i++) {
      double a = fabs(F(un, i, j) - F(u, i, j));
      if (a > diff) diff = a;
    }
  return diff;
}

/* nAuxMomentum and its helpers in FP64 (the reference's precision) and in
 * FP32 (the checker of the GPU's single-precision momentum). */
#define REAL double
#define R(x) ((double)(x))
#define FN(x) x
#define RABS fabs
#define RSQRT sqrt
#define MOMWS w2o_mom_ws
#define METRICS w2o_metrics
#define MOM_WX wx
#define MOM_WY wy
#define MOM_DUS dus
#define MOM_DVS dvs
#include "momentum_impl.h"
#undef REAL
#undef R
#undef FN
#undef RABS
#undef RSQRT
#undef MOMWS
#undef METRICS
#undef MOM_WX
#undef MOM_WY
#undef MOM_DUS
#undef MOM_DVS

#define REAL float
#define R(x) ((float)(x))
#define FN(x) x##_f32
#define RABS fabsf
#define RSQRT sqrtf
#define MOMWS w2o_mom_ws32
#define METRICS w2o_metrics32
#define MOM_WX wx32
#define MOM_WY wy32
#define MOM_DUS dus32
#define MOM_DVS dvs32
#include "momentum_impl.h"
#undef REAL
#undef R
#undef FN
#undef RABS
#undef RSQRT
#undef MOMWS
#undef METRICS
#undef MOM_WX
#undef MOM_WY
#undef MOM_DUS
#undef MOM_DVS

/* ------------------------------------------------------------------ */
/* thermal.f and TempBoundCond                                         */
/* ------------------------------------------------------------------ */

#define TRT(t, r, ir, jr) (t)->nTRgType[((ir)-1) + ((jr)-1) * (r)->mgri]
#define TBT(t, r, ir, jr, s) \
  (t)->nTemBdTp[((ir)-1) + ((jr)-1) * (r)->mgri + ((s)-1) * (r)->mgri * (r)->mgrj]
#define TRV(arr, r, ir, jr) (arr)[((ir)-1) + ((jr)-1) * (r)->mgri]

/* TempBoundCond, bound_cond.f:1030-1186: fixed-temperature regions (interior
 * value, then image points across each face), else per face: interface,
 * fixed temperature (image) or heat flux (ghost = value + inner). */
void w2o_temp_bound_cond(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                         const w2o_thermal *th, double *t) {
  (void)nx; (void)ny;
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      const int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      const int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      int i, j;
      if (TRT(th, r, ireg, jreg) == RT_TEMPER) {
        const double tv = TRV(th->dTRgVal, r, ireg, jreg);
        for (j = jS + 1; j <= jN; j++)
          for (i = iW + 1; i <= iE; i++) F(t, i, j) = tv;
        for (j = jS + 1; j <= jN; j++) F(t, iW + 1, j) = 2.0 * BCV(r, ireg, jreg, WEST, VT) - F(t, iW, j);
        for (j = jS + 1; j <= jN; j++) F(t, iE, j) = 2.0 * BCV(r, ireg, jreg, EAST, VT) - F(t, iE + 1, j);
        for (i = iW + 1; i <= iE; i++) F(t, i, jS + 1) = 2.0 * BCV(r, ireg, jreg, SOUTH, VT) - F(t, i, jS);
        for (i = iW + 1; i <= iE; i++) F(t, i, jN) = 2.0 * BCV(r, ireg, jreg, NORTH, VT) - F(t, i, jN + 1);
        continue;
      }
      switch (TBT(th, r, ireg, jreg, WEST)) {
        case BT_INTERN: break;
        case BT_TEMPER:
          for (j = jS + 1; j <= jN; j++) F(t, iW, j) = 2.0 * BCV(r, ireg, jreg, WEST, VT) - F(t, iW + 1, j);
          break;
        case BT_HTFLUX:
          for (j = jS + 1; j <= jN; j++) F(t, iW, j) = BCV(r, ireg, jreg, WEST, VT) + F(t, iW + 1, j);
          break;
        default: die("Wrong nTemBdTp W flag", ireg, jreg);
      }
      switch (TBT(th, r, ireg, jreg, EAST)) {
        case BT_INTERN: break;
        case BT_TEMPER:
          for (j = jS + 1; j <= jN; j++) F(t, iE + 1, j) = 2.0 * BCV(r, ireg, jreg, EAST, VT) - F(t, iE, j);
          break;
        case BT_HTFLUX:
          for (j = jS + 1; j <= jN; j++) F(t, iE + 1, j) = BCV(r, ireg, jreg, EAST, VT) + F(t, iE, j);
          break;
        default: die("Wrong nTemBdTp E flag", ireg, jreg);
      }
      switch (TBT(th, r, ireg, jreg, SOUTH)) {
        case BT_INTERN: break;
        case BT_TEMPER:
          for (i = iW + 1; i <= iE; i++) F(t, i, jS) = 2.0 * BCV(r, ireg, jreg, SOUTH, VT) - F(t, i, jS + 1);
          break;
        case BT_HTFLUX:
          for (i = iW + 1; i <= iE; i++) F(t, i, jS) = BCV(r, ireg, jreg, SOUTH, VT) + F(t, i, jS + 1);
          break;
        default: die("Wrong nTemBdTp S flag", ireg, jreg);
      }
      switch (TBT(th, r, ireg, jreg, NORTH)) {
        case BT_INTERN: break;
        case BT_TEMPER:
          for (i = iW + 1; i <= iE; i++) F(t, i, jN + 1) = 2.0 * BCV(r, ireg, jreg, NORTH, VT) - F(t, i, jN);
          break;
        case BT_HTFLUX:
          for (i = iW + 1; i <= iE; i++) F(t, i, jN + 1) = BCV(r, ireg, jreg, NORTH, VT) + F(t, i, jN);
          break;
        default: die("Wrong nTemBdTp N flag", ireg, jreg);
      }
    }
}

/* ThermEnergy, thermal.f:24-280.  Two split steps on ONE chain of the
 * (nx-1)(ny-1) interior points in i-fastest order (ind = (j-2)(nx-1)+i-1)
 * for both splits: split 1 holds the upwinded i-direction rows, split 2 the
 * j-direction coefficients on the same i-fastest chain, as the reference
 * writes them, with identity rows in fixed-temperature regions. */
void w2o_therm_energy(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                      const w2o_thermal *th, double dk, double pe,
                      const w2o_metrics *m, const double *un, const double *vn,
                      const double *u, const double *v, const double *tn,
                      double *t) {
  double *cu1 = c->th_cu1, *cv1 = c->th_cv1, *cun = c->th_cun, *cvn = c->th_cvn, *sg = c->th_s;
  double *a = c->th_a, *b = c->th_b;
#define TA(k, ind) a[((k)-1) + 3 * (size_t)((ind)-1)]
#define TB(ind) b[(ind)-1]
  const double pe1 = 1.0 / pe;
  int i, j;
  w2o_temp_bound_cond(c, nx, ny, r, th, t);
  conv_coef(c, nx, ny, 6, 0, m->xzc, m->xec, m->yzc, m->yec, u, v, cu1, cv1);
  conv_coef(c, nx, ny, 3, 0, m->xzv, m->xeu, m->yzv, m->yeu, un, vn, cun, cvn);
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      const int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      const int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      const double sv = TRT(th, r, ireg, jreg) == RT_HEATGN ? TRV(th->dHGSTval, r, ireg, jreg) : 0.0;
      for (j = jS + 1; j <= jN; j++)
        for (i = iW + 1; i <= iE; i++) F(sg, i, j) = sv;
    }
  /* split 1 */
  for (j = 2; j <= ny; j++)
    for (i = 2; i <= nx; i++) {
      const int ind = (j - 2) * (nx - 1) + i - 1;
      const double rkj = dk * F(m->djc, i, j) * 0.5;
      const double rw = F(m->rau, i - 1, j), ro = F(m->rau, i, j);
      if (F(cu1, i, j) >= 0.0) {
        TA(1, ind) = rkj * (-F(cu1, i - 1, j) - pe1 * rw);
        TA(2, ind) = 1.0 + rkj * (F(cu1, i, j) + pe1 * (ro + rw));
        TA(3, ind) = rkj * (-pe1 * ro);
      } else {
        TA(1, ind) = rkj * (-pe1 * rw);
        TA(2, ind) = 1.0 + rkj * (-F(cu1, i, j) + pe1 * (ro + rw));
        TA(3, ind) = rkj * (F(cu1, i + 1, j) - pe1 * ro);
      }
      const double cc = -F(cvn, i, j - 1) * F(tn, i, j - 1) - F(cun, i - 1, j) * F(tn, i - 1, j) +
                        (F(cun, i, j) - F(cun, i - 1, j) + F(cvn, i, j) - F(cvn, i, j - 1)) * F(tn, i, j) +
                        F(cun, i, j) * F(tn, i + 1, j) + F(cvn, i, j) * F(tn, i, j + 1);
      const double dd =
          F(m->rau, i, j) * (F(tn, i + 1, j) - F(tn, i, j)) -
          F(m->rau, i - 1, j) * (F(tn, i, j) - F(tn, i - 1, j)) +
          F(m->rbu, i, j) * (F(tn, i + 1, j + 1) + F(tn, i, j + 1) - F(tn, i + 1, j - 1) - F(tn, i, j - 1)) -
          F(m->rbu, i - 1, j) * (F(tn, i, j + 1) + F(tn, i - 1, j + 1) - F(tn, i, j - 1) - F(tn, i - 1, j - 1)) +
          F(m->rbv, i, j) * (F(tn, i + 1, j + 1) + F(tn, i + 1, j) - F(tn, i - 1, j + 1) - F(tn, i - 1, j)) -
          F(m->rbv, i, j - 1) * (F(tn, i + 1, j) + F(tn, i + 1, j - 1) - F(tn, i - 1, j) - F(tn, i - 1, j - 1)) +
          F(m->rgv, i, j) * (F(tn, i, j + 1) - F(tn, i, j)) -
          F(m->rgv, i, j - 1) * (F(tn, i, j) - F(tn, i, j - 1));
      TB(ind) = dk * F(sg, i, j) * 0.5 + 2.0 * rkj * (-cc + pe1 * dd);
    }
  w2o_alt_trid_lu((nx - 1) * (ny - 1), a, b);
  /* split 2: same chain order, j-direction coefficients */
  for (j = 2; j <= ny; j++)
    for (i = 2; i <= nx; i++) {
      const int ind = (j - 2) * (nx - 1) + i - 1;
      const double rkj = dk * F(m->djc, i, j) * 0.5;
      const double rs = F(m->rgv, i, j - 1), ro = F(m->rgv, i, j);
      if (F(cv1, i, j) >= 0.0) {
        TA(1, ind) = rkj * (-F(cv1, i, j - 1) - pe1 * rs);
        TA(2, ind) = 1.0 + rkj * (F(cv1, i, j) + pe1 * (ro + rs));
        TA(3, ind) = rkj * (-pe1 * ro);
      } else {
        TA(1, ind) = rkj * (-pe1 * rs);
        TA(2, ind) = 1.0 + rkj * (-F(cv1, i, j) + pe1 * (ro + rs));
        TA(3, ind) = rkj * (F(cv1, i, j + 1) - pe1 * ro);
      }
    }
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      if (TRT(th, r, ireg, jreg) != RT_TEMPER) continue;
      const int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      const int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      for (j = jS + 1; j <= jN; j++)
        for (i = iW + 1; i <= iE; i++) {
          const int ind = (j - 2) * (nx - 1) + i - 1;
          TA(1, ind) = 0.0;
          TA(2, ind) = 1.0;
          TA(3, ind) = 0.0;
          TB(ind) = 0.0;
        }
    }
  w2o_alt_trid_lu((nx - 1) * (ny - 1), a, b);
  for (j = 2; j <= ny; j++)
    for (i = 2; i <= nx; i++) F(t, i, j) = F(t, i, j) + TB((j - 2) * (nx - 1) + i - 1);
#undef TA
#undef TB
}

/* EqState, thermal.f:288-329: den = (p densref uref^2 + pref) /
 * (densref rconst (t (tmax - tref) + tref)) - 1 on i, j = 2..n, flushed to
 * zero below 1e-10 in magnitude. */
void w2o_eq_state(w2o_ctx *c, int nx, int ny, double uref, double densref, double tmax,
                  double tref, double rconst, const double *p, const double *t, double *den) {
  const double pref = densref * rconst * tref;
  for (int j = 2; j <= ny; j++)
    for (int i = 2; i <= nx; i++) {
      const double c1 = F(p, i, j) * densref * (uref * uref) + pref;
      const double c2 = densref * rconst * (F(t, i, j) * (tmax - tref) + tref);
      F(den, i, j) = c1 / c2 - 1.0;
      if (fabs(F(den, i, j)) < 1.0e-10) F(den, i, j) = 0.0;
    }
}

/* ------------------------------------------------------------------ */
/* pressure.f                                                          */
/* ------------------------------------------------------------------ */

#define PA(ind, k) c->pa[((ind)-1) + (size_t)((k)-1) * c->mn]
#define PB(ind) c->pb[(ind)-1]

/* Divergence nloc=1, pressure.f:265-300 */
static void divergence1(w2o_ctx *c, int nx, int ny, const double *xet,
                        const double *yet, const double *xzi,
                        const double *yzi, const double *u, const double *v,
                        double *div) {
  double ucij, uci1j, vcij, vcij1;
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      ucij = F(yet, i, j) * F(u, i, j) -
             F(xet, i, j) * (F(v, i + 1, j) + F(v, i, j) + F(v, i + 1, j - 1) +
                             F(v, i, j - 1)) / 4.0;
      uci1j = F(yet, i - 1, j) * F(u, i - 1, j) -
              F(xet, i - 1, j) * (F(v, i, j) + F(v, i - 1, j) + F(v, i, j - 1) +
                                  F(v, i - 1, j - 1)) / 4.0;
      vcij = F(xzi, i, j) * F(v, i, j) -
             F(yzi, i, j) * (F(u, i, j + 1) + F(u, i - 1, j + 1) + F(u, i, j) +
                             F(u, i - 1, j)) / 4.0;
      vcij1 = F(xzi, i, j - 1) * F(v, i, j - 1) -
              F(yzi, i, j - 1) * (F(u, i, j) + F(u, i - 1, j) + F(u, i, j - 1) +
                                  F(u, i - 1, j - 1)) / 4.0;
      F(div, i, j) = ucij - uci1j + vcij - vcij1;
    }
}

/* RhsPpe, pressure.f:329-378 */
static void rhs_ppe(w2o_ctx *c, int nx, int ny, int lcartes, double dk,
                    const w2o_metrics *m, const double *div, const double *p) {
  int i, j, ind;
  for (j = 2; j <= ny; j++)
    for (i = 2; i <= nx; i++) {
      ind = (j - 2) * (nx - 1) + i - 1;
      PB(ind) = F(div, i, j) / dk;
    }
  if (!lcartes) {
    const double *rbu = m->rbu, *rbv = m->rbv;
    for (j = 2; j <= ny; j++)
      for (i = 2; i <= nx; i++) {
        ind = (j - 2) * (nx - 1) + i - 1;
        PB(ind) = PB(ind) -
                  (F(rbu, i, j) * (F(p, i + 1, j + 1) + F(p, i, j + 1) -
                                   F(p, i + 1, j - 1) - F(p, i, j - 1)) -
                   F(rbu, i - 1, j) * (F(p, i, j + 1) + F(p, i - 1, j + 1) -
                                       F(p, i, j - 1) - F(p, i - 1, j - 1)) +
                   F(rbv, i, j) * (F(p, i + 1, j + 1) + F(p, i + 1, j) -
                                   F(p, i - 1, j + 1) - F(p, i - 1, j)) -
                   F(rbv, i, j - 1) * (F(p, i + 1, j) + F(p, i + 1, j - 1) -
                                       F(p, i - 1, j) - F(p, i - 1, j - 1)));
      }
  }
}

/* One point update shared by Sor/SorRB/SorRBP (pressure.f:434-439);
 * returns |delta| and updates p in place. */
static inline double sor_point(w2o_ctx *c, int nx, double *p, int i, int j,
                               double sorrel) {
  int ind = (j - 2) * (nx - 1) + i - 1;
  double sum = PB(ind) - PA(ind, 1) * F(p, i, j - 1) - PA(ind, 2) * F(p, i - 1, j) -
               PA(ind, 4) * F(p, i + 1, j) - PA(ind, 5) * F(p, i, j + 1);
  sum = sum / PA(ind, 3) - F(p, i, j);
  F(p, i, j) = F(p, i, j) + sorrel * sum;
  return fabs(sum);
}

/* Sor, pressure.f:384-450 */
static int sor(w2o_ctx *c, int nx, int ny, int lcartes, int msorit, double dk,
               double sortol, double sorrel, const w2o_metrics *m,
               const double *div, double *p) {
  if (lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
  for (int it = 1; it <= msorit; it++) {
    if (!lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
    double dif = 0.0;
    for (int j = 2; j <= ny; j++)
      for (int i = 2; i <= nx; i++) {
        double s = sor_point(c, nx, p, i, j, sorrel);
        dif = (s > dif) ? s : dif;
      }
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

/* SorRB, pressure.f:457-541 */
static int sor_rb(w2o_ctx *c, int nx, int ny, int lcartes, int msorit,
                  double dk, double sortol, double sorrel,
                  const w2o_metrics *m, const double *div, double *p) {
  if (lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
  for (int it = 1; it <= msorit; it++) {
    if (!lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
    double dif = 0.0;
    for (int j = 2; j <= ny; j++)
      for (int i = 2 + j % 2; i <= nx; i += 2) {
        double s = sor_point(c, nx, p, i, j, sorrel);
        dif = (s > dif) ? s : dif;
      }
    for (int j = 2; j <= ny; j++)
      for (int i = 2 + (j + 1) % 2; i <= nx; i += 2) {
        double s = sor_point(c, nx, p, i, j, sorrel);
        dif = (s > dif) ? s : dif;
      }
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

/* SorRBP, pressure.f:548-656 (per-point dif array, then its max) */
static int sor_rbp(w2o_ctx *c, int nx, int ny, int lcartes, int msorit,
                   double dk, double sortol, double sorrel,
                   const w2o_metrics *m, const double *div, double *p) {
  double *dif = c->rbp_dif;
  if (lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
  for (int it = 1; it <= msorit; it++) {
    if (!lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) F(dif, i, j) = 0.0;
    for (int j = 2; j <= ny; j++)
      for (int i = 2 + j % 2; i <= nx; i += 2) {
        double s = sor_point(c, nx, p, i, j, sorrel);
        F(dif, i, j) = (s > F(dif, i, j)) ? s : F(dif, i, j);
      }
    for (int j = 2; j <= ny; j++)
      for (int i = 2 + (j + 1) % 2; i <= nx; i += 2) {
        double s = sor_point(c, nx, p, i, j, sorrel);
        F(dif, i, j) = (s > F(dif, i, j)) ? s : F(dif, i, j);
      }
    double difmax = 0.0;
    for (int j = 2; j <= ny; j++)
      for (int i = 2; i <= nx; i++)
        difmax = (F(dif, i, j) > difmax) ? F(dif, i, j) : difmax;
    if (it > 1 && difmax < sortol) return it;
  }
  return 0;
}

/* Line solve of line nl (j = nl) along i, shared by Slor / SlorRB with
 * ndir = 1 (pressure.f:750-790, 905-945).  Returns the line's max |delta|. */
static double slor_line(w2o_ctx *c, int nx, double *p, int nl, double sorrel) {
  int ncomps = nx - 1;
  size_t mnl = (size_t)(c->mnx > c->mny ? c->mnx : c->mny);
  double *aline = c->lin, *bline = c->lin + 3 * mnl, *plold = c->lin + 4 * mnl;
  double dif = 0.0;
  for (int nc = 2; nc <= ncomps + 1; nc++) {
    int ind = (nl - 2) * ncomps + nc - 1;
    plold[nc - 2] = F(p, nc, nl);
    double plprev = F(p, nc, nl - 1), plnext = F(p, nc, nl + 1);
    aline[0 + 3 * (nc - 2)] = PA(ind, 2);
    aline[1 + 3 * (nc - 2)] = PA(ind, 3);
    aline[2 + 3 * (nc - 2)] = PA(ind, 4);
    bline[nc - 2] = PB(ind) - (PA(ind, 1) * plprev + PA(ind, 5) * plnext);
  }
  w2o_alt_trid_lu(ncomps, aline, bline);
  for (int nc = 1; nc <= ncomps; nc++) {
    double sum = bline[nc - 1] - plold[nc - 1];
    bline[nc - 1] = plold[nc - 1] + sorrel * sum;
    sum = fabs(sum);
    dif = (sum > dif) ? sum : dif;
  }
  for (int nc = 2; nc <= ncomps + 1; nc++) F(p, nc, nl) = bline[nc - 2];
  return dif;
}

/* Slor with ndir = 1, pressure.f:673-802 */
static int slor(w2o_ctx *c, int nx, int ny, int lcartes, int msorit,
                double dk, double sortol, double sorrel, const w2o_metrics *m,
                const double *div, double *p) {
  int nlines = ny - 1;
  if (lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
  for (int it = 1; it <= msorit; it++) {
    double dif = 0.0;
    if (!lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
    for (int nl = 2; nl <= nlines + 1; nl++) {
      double s = slor_line(c, nx, p, nl, sorrel);
      dif = (s > dif) ? s : dif;
    }
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

/* SlorRB with ndir = 1, pressure.f:819-959 */
static int slor_rb(w2o_ctx *c, int nx, int ny, int lcartes, int msorit,
                   double dk, double sortol, double sorrel,
                   const w2o_metrics *m, const double *div, double *p) {
  int nlines = ny - 1;
  if (lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
  for (int it = 1; it <= msorit; it++) {
    double dif = 0.0;
    for (int k = 2; k <= 3; k++) {
      if (!lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
      for (int nl = k; nl <= nlines + 1; nl += 2) {
        double s = slor_line(c, nx, p, nl, sorrel);
        dif = (s > dif) ? s : dif;
      }
    }
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

/* SlorRBP, pressure.f:976-1138 */
static int slor_rbp(w2o_ctx *c, int nx, int ny, int lcartes, int msorit,
                    double dk, double sortol, double sorrel,
                    const w2o_metrics *m, const double *div, double *p) {
  int nlines = ny - 1, ncomps = nx - 1;
  size_t mnl = (size_t)(c->mnx > c->mny ? c->mnx : c->mny);
  double *aline = c->lin, *bline = c->lin + 3 * mnl;
  double *pn = c->rbp_pn;
  if (lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
  for (int it = 1; it <= msorit; it++) {
    for (int nl = 1; nl <= nlines + 2; nl++)
      for (int nc = 1; nc <= ncomps + 2; nc++) F(pn, nc, nl) = F(p, nc, nl);
    for (int color = 2; color <= 3; color++) {
      if (!lcartes) rhs_ppe(c, nx, ny, lcartes, dk, m, div, p);
      for (int nl = color; nl <= nlines + 1; nl += 2) {
        for (int nc = 2; nc <= ncomps + 1; nc++) {
          int ind = (nl - 2) * ncomps + nc - 1;
          aline[0 + 3 * (nc - 2)] = PA(ind, 2);
          aline[1 + 3 * (nc - 2)] = PA(ind, 3);
          aline[2 + 3 * (nc - 2)] = PA(ind, 4);
          bline[nc - 2] = PB(ind) - (PA(ind, 1) * F(p, nc, nl - 1) +
                                     PA(ind, 5) * F(p, nc, nl + 1));
        }
        w2o_alt_trid_lu(ncomps, aline, bline);
        for (int nc = 2; nc <= ncomps + 1; nc++) F(p, nc, nl) = bline[nc - 2];
      }
      for (int nl = color; nl <= nlines + 1; nl += 2)
        for (int nc = 2; nc <= ncomps + 1; nc++)
          F(p, nc, nl) = F(pn, nc, nl) + sorrel * (F(p, nc, nl) - F(pn, nc, nl));
    }
    double dif = 0.0;
    for (int nl = 2; nl <= nlines + 1; nl++)
      for (int nc = 2; nc <= ncomps + 1; nc++) {
        double s = fabs(F(pn, nc, nl) - F(p, nc, nl));
        dif = (s > dif) ? s : dif;
      }
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

static void ppe_identity(w2o_ctx *c, int ind) {
  PA(ind, 1) = 0.0; PA(ind, 2) = 0.0; PA(ind, 3) = 1.0;
  PA(ind, 4) = 0.0; PA(ind, 5) = 0.0;
}

/* Ppe, pressure.f:30-249 */
int w2o_ppe(w2o_ctx *c, int nx, int ny, const w2o_regions *r, int lcartes,
            int npsolver, int msorit, double dk, double sortol, double sorrel,
            const w2o_metrics *m, const double *u, const double *v, double *p) {
  int i, j, ind;
  double *div = c->div;
  divergence1(c, nx, ny, m->xeu, m->yeu, m->xzv, m->yzv, u, v, div);
  for (j = 2; j <= ny; j++)
    for (i = 2; i <= nx; i++) {
      ind = (j - 2) * (nx - 1) + i - 1;
      PA(ind, 1) = F(m->rgv, i, j - 1);
      PA(ind, 2) = F(m->rau, i - 1, j);
      PA(ind, 3) = -F(m->rau, i, j) - F(m->rau, i - 1, j) - F(m->rgv, i, j) -
                   F(m->rgv, i, j - 1);
      PA(ind, 4) = F(m->rau, i, j);
      PA(ind, 5) = F(m->rgv, i, j);
    }
  /* Blockage rows, pressure.f:109-196 */
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      if (RTYP(r, ireg, jreg) != RM_BLOCKG) continue;
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      for (j = jS + 2; j <= jN - 1; j++)
        for (i = iW + 2; i <= iE - 1; i++) {
          ppe_identity(c, (j - 2) * (nx - 1) + i - 1);
          F(div, i, j) = 0.0;
        }
      if (ireg > 1 && RTYP(r, ireg - 1, jreg) == RM_BLOCKG)
        for (j = jS + 1; j <= jN; j++) {
          ppe_identity(c, (j - 2) * (nx - 1) + iW);
          F(div, iW + 1, j) = 0.0;
        }
      if (ireg < r->nReg[0] && RTYP(r, ireg + 1, jreg) == RM_BLOCKG)
        for (j = jS + 1; j <= jN; j++) {
          ppe_identity(c, (j - 2) * (nx - 1) + iE - 1);
          F(div, iE, j) = 0.0;
        }
      if (jreg > 1 && RTYP(r, ireg, jreg - 1) == RM_BLOCKG)
        for (i = iW + 1; i <= iE; i++) {
          ppe_identity(c, (jS - 1) * (nx - 1) + i - 1);
          F(div, i, jS + 1) = 0.0;
        }
      if (jreg < r->nReg[1] && RTYP(r, ireg, jreg + 1) == RM_BLOCKG)
        for (i = iW + 1; i <= iE; i++) {
          ppe_identity(c, (jN - 2) * (nx - 1) + i - 1);
          F(div, i, jN) = 0.0;
        }
    }
  int nconv = 0;
  switch (npsolver) {
    case 1: nconv = sor(c, nx, ny, lcartes, msorit, dk, sortol, sorrel, m, div, p); break;
    case 2: nconv = slor(c, nx, ny, lcartes, msorit, dk, sortol, sorrel, m, div, p); break;
    case 3: nconv = slor_rb(c, nx, ny, lcartes, msorit, dk, sortol, sorrel, m, div, p); break;
    case 4: nconv = slor_rbp(c, nx, ny, lcartes, msorit, dk, sortol, sorrel, m, div, p); break;
    case 5: nconv = sor_rb(c, nx, ny, lcartes, msorit, dk, sortol, sorrel, m, div, p); break;
    case 6: nconv = sor_rbp(c, nx, ny, lcartes, msorit, dk, sortol, sorrel, m, div, p); break;
    default: fprintf(stderr, "Wrong nPpeSolver flag passed to Ppe\n");
  }
  if (nconv < 1) nconv = msorit;
  return nconv;
}
#undef PA
#undef PB

/* ------------------------------------------------------------------ */
/* utility.f                                                           */
/* ------------------------------------------------------------------ */

/* Project, utility.f:253-440 */
void w2o_project(w2o_ctx *c, int nx, int ny, const w2o_regions *r, double dk,
                 const w2o_metrics *m, const double *p, double *u, double *v) {
  (void)nx; (void)ny;
  double pzi, pet, djk;
  const double *dju = m->dju, *djv = m->djv, *yeu = m->yeu, *xzv = m->xzv,
               *yzu = m->yzu, *xev = m->xev;
#define UPD_U(i, j)                                                                  \
  do {                                                                               \
    pzi = F(p, (i) + 1, j) - F(p, i, j);                                             \
    pet = (F(p, (i) + 1, (j) + 1) + F(p, i, (j) + 1) - F(p, (i) + 1, (j)-1) -        \
           F(p, i, (j)-1)) / 4.0;                                                    \
    djk = F(dju, i, j) * dk;                                                         \
    F(u, i, j) = F(u, i, j) - djk * (F(yeu, i, j) * pzi - F(yzu, i, j) * pet);       \
  } while (0)
#define UPD_V(i, j)                                                                  \
  do {                                                                               \
    pzi = (F(p, (i) + 1, (j) + 1) + F(p, (i) + 1, j) - F(p, (i)-1, (j) + 1) -        \
           F(p, (i)-1, j)) / 4.0;                                                    \
    pet = F(p, i, (j) + 1) - F(p, i, j);                                             \
    djk = F(djv, i, j) * dk;                                                         \
    F(v, i, j) = F(v, i, j) - djk * (-F(xev, i, j) * pzi + F(xzv, i, j) * pet);      \
  } while (0)
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      if (RTYP(r, ireg, jreg) == RM_BLOCKG) continue;
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      for (int j = jS + 1; j <= jN; j++)
        for (int i = iW + 1; i <= iE - 1; i++) UPD_U(i, j);
      int t = MBTP(r, ireg, jreg, WEST);
      if (t == BM_OUTLT1)
        for (int j = jS + 1; j <= jN; j++) UPD_U(iW, j);
      t = MBTP(r, ireg, jreg, EAST);
      if (t == BM_INTERN || t == BM_OUTLT1)
        for (int j = jS + 1; j <= jN; j++) UPD_U(iE, j);
    }
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      if (RTYP(r, ireg, jreg) == RM_BLOCKG) continue;
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      for (int j = jS + 1; j <= jN - 1; j++)
        for (int i = iW + 1; i <= iE; i++) UPD_V(i, j);
      int t = MBTP(r, ireg, jreg, SOUTH);
      if (t == BM_OUTLT1)
        for (int i = iW + 1; i <= iE; i++) UPD_V(i, jS);
      t = MBTP(r, ireg, jreg, NORTH);
      if (t == BM_INTERN || t == BM_OUTLT1)
        for (int i = iW + 1; i <= iE; i++) UPD_V(i, jN);
    }
#undef UPD_U
#undef UPD_V
}

/* Filter, utility.f:33-247 (velocity components only) */
void w2o_filter(w2o_ctx *c, int nx, int ny, int ncomp, const w2o_regions *r,
                double fp, double *qu) {
  double *qh = c->qh;
  for (int j = 0; j <= ny + 1; j++)
    for (int i = 0; i <= nx + 1; i++) F(qh, i, j) = F(qu, i, j);
#define FILT(i, j)                                                                 \
  F(qh, i, j) = (F(qu, i, (j)-1) + F(qu, (i)-1, j) + F(qu, i, (j) + 1) +            \
                 F(qu, (i) + 1, j) + fp * F(qu, i, j)) / (fp + 4.0)
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      if (RTYP(r, ireg, jreg) == RM_BLOCKG) continue;
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      if (ncomp == VU) {
        for (int j = jS + 1; j <= jN; j++)
          for (int i = iW + 1; i <= iE - 1; i++) FILT(i, j);
        if (MBTP(r, ireg, jreg, WEST) == BM_OUTLT1)
          for (int j = jS + 1; j <= jN; j++) FILT(iW, j);
        int t = MBTP(r, ireg, jreg, EAST);
        if (t == BM_INTERN || t == BM_OUTLT1)
          for (int j = jS + 1; j <= jN; j++) FILT(iE, j);
      } else {
        for (int j = jS + 1; j <= jN - 1; j++)
          for (int i = iW + 1; i <= iE; i++) FILT(i, j);
        if (MBTP(r, ireg, jreg, SOUTH) == BM_OUTLT1)
          for (int i = iW + 1; i <= iE; i++) FILT(i, jS);
        int t = MBTP(r, ireg, jreg, NORTH);
        if (t == BM_INTERN || t == BM_OUTLT1)
          for (int i = iW + 1; i <= iE; i++) FILT(i, jN);
      }
    }
#undef FILT
  for (int j = 0; j <= ny + 1; j++)
    for (int i = 0; i <= nx + 1; i++) F(qu, i, j) = F(qh, i, j);
}

void w2o_filter_t(w2o_ctx *c, int nx, int ny, const w2o_regions *r, const w2o_thermal *th,
                  double fp, double *qu) {
  double *qh = c->qh;
  for (int j = 0; j <= ny + 1; j++)
    for (int i = 0; i <= nx + 1; i++) F(qh, i, j) = F(qu, i, j);
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      if (th->nTRgType[(ireg - 1) + (jreg - 1) * r->mgri] == BT_TEMPER) continue;
      const int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      const int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      for (int j = jS + 1; j <= jN; j++)
        for (int i = iW + 1; i <= iE; i++)
          F(qh, i, j) = (F(qu, i, j - 1) + F(qu, i - 1, j) + F(qu, i, j + 1) + F(qu, i + 1, j) +
                         fp * F(qu, i, j)) / (fp + 4.0);
    }
  for (int j = 0; j <= ny + 1; j++)
    for (int i = 0; i <= nx + 1; i++) F(qu, i, j) = F(qh, i, j);
}

/* ------------------------------------------------------------------ */
/* bound_cond.f                                                        */
/* ------------------------------------------------------------------ */

/* VelBoundCond, bound_cond.f:511-847 */
void w2o_vel_bound_cond(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                        double *u, double *v) {
  (void)nx; (void)ny;
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      int i, j;
      switch (MBTP(r, ireg, jreg, WEST)) {
        case BM_INTERN: break;
        case BM_WALL1:
          for (j = jS; j <= jN; j++) F(u, iW, j) = 0.0;
          for (j = jS + 1; j <= jN; j++)
            F(v, iW, j) = 2.0 * BCVP(r, ireg, jreg, WEST, VV, j) - F(v, iW + 1, j);
          break;
        case BM_WALL2:
          for (j = jS; j <= jN; j++) F(u, iW, j) = 0.0;
          for (j = jS + 1; j <= jN; j++) F(v, iW, j) = F(v, iW + 1, j);
          break;
        case BM_INLET:
          for (j = jS; j <= jN; j++) F(u, iW, j) = BCVP(r, ireg, jreg, WEST, VU, j);
          for (j = jS + 1; j <= jN; j++)
            F(v, iW, j) = 2.0 * BCVP(r, ireg, jreg, WEST, VV, j) - F(v, iW + 1, j);
          break;
        case BM_OUTLT1:
          for (j = jS; j <= jN; j++) F(u, iW - 1, j) = BCV(r, ireg, jreg, WEST, VU) + F(u, iW, j);
          for (j = jS + 1; j <= jN; j++) F(v, iW, j) = -F(v, iW + 1, j);
          break;
        case BM_OUTLT2:
          for (j = jS + 1; j <= jN; j++)
            F(u, iW, j) = F(u, iW + 1, j) + F(v, iW + 1, j) - F(v, iW + 1, j - 1);
          for (j = jS + 1; j <= jN; j++)
            F(v, iW, j) = -F(v, iW, j - 1) + 5.0 * (F(v, iW + 1, j) - F(v, iW + 1, j - 1)) +
                          8.0 * (F(u, iW + 1, j) - F(u, iW, j));
          break;
        default: die("Wrong nBdTypeW flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, EAST)) {
        case BM_INTERN: break;
        case BM_WALL1:
          for (j = jS; j <= jN; j++) F(u, iE, j) = 0.0;
          for (j = jS + 1; j <= jN; j++)
            F(v, iE + 1, j) = 2.0 * BCVP(r, ireg, jreg, EAST, VV, j) - F(v, iE, j);
          break;
        case BM_WALL2:
          for (j = jS; j <= jN; j++) F(u, iE, j) = 0.0;
          for (j = jS + 1; j <= jN; j++) F(v, iE + 1, j) = F(v, iE, j);
          break;
        case BM_INLET:
          for (j = jS; j <= jN; j++) F(u, iE, j) = BCVP(r, ireg, jreg, EAST, VU, j);
          for (j = jS + 1; j <= jN; j++)
            F(v, iE + 1, j) = 2.0 * BCVP(r, ireg, jreg, EAST, VV, j) - F(v, iE, j);
          break;
        case BM_OUTLT1:
          for (j = jS; j <= jN; j++) F(u, iE + 1, j) = BCV(r, ireg, jreg, EAST, VU) + F(u, iE, j);
          for (j = jS + 1; j <= jN; j++) F(v, iE + 1, j) = -F(v, iE, j);
          break;
        case BM_OUTLT2:
          for (j = jS + 1; j <= jN; j++)
            F(u, iE, j) = F(u, iE - 1, j) - (F(v, iE, j) - F(v, iE, j - 1));
          for (j = jS + 1; j <= jN - 1; j++)
            F(v, iE + 1, j) = F(v, iE + 1, j - 1) + 3.0 * (F(v, iE, j - 1) - F(v, iE, j)) -
                              4.0 * (F(u, iE, j) - F(u, iE - 1, j));
          break;
        default: die("Wrong nBdTypeE flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, SOUTH)) {
        case BM_INTERN: break;
        case BM_WALL1:
          for (i = iW + 1; i <= iE; i++)
            F(u, i, jS) = 2.0 * BCVP(r, ireg, jreg, SOUTH, VU, i) - F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS) = 0.0;
          break;
        case BM_WALL2:
          for (i = iW + 1; i <= iE; i++) F(u, i, jS) = F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS) = 0.0;
          break;
        case BM_INLET:
          for (i = iW + 1; i <= iE; i++)
            F(u, i, jS) = 2.0 * BCVP(r, ireg, jreg, SOUTH, VU, i) - F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS) = BCVP(r, ireg, jreg, SOUTH, VV, i);
          break;
        case BM_OUTLT1:
          for (i = iW + 1; i <= iE; i++) F(u, i, jS) = -F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS) = BCV(r, ireg, jreg, SOUTH, VV) + F(v, i, jS);
          break;
        case BM_OUTLT2:
          for (i = iW + 1; i <= iE; i++)
            F(v, i, jS) = F(v, i, jS + 1) + (F(u, i, jS + 1) - F(u, i - 1, jS + 1));
          for (i = iW + 1; i <= iE - 1; i++)
            F(u, i, jS) = F(u, i - 1, jS) + 3.0 * (F(u, i - 1, jS + 1) - F(u, i, jS + 1)) -
                          4.0 * (F(v, i, jS + 1) - F(v, i, jS));
          break;
        default: die("Wrong nBdTypeS flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, NORTH)) {
        case BM_INTERN: break;
        case BM_WALL1:
          for (i = iW + 1; i <= iE; i++)
            F(u, i, jN + 1) = 2.0 * BCVP(r, ireg, jreg, NORTH, VU, i) - F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN) = 0.0;
          break;
        case BM_WALL2:
          for (i = iW + 1; i <= iE; i++) F(u, i, jN + 1) = F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN) = 0.0;
          break;
        case BM_INLET:
          for (i = iW + 1; i <= iE; i++)
            F(u, i, jN + 1) = 2.0 * BCVP(r, ireg, jreg, NORTH, VU, i) - F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN) = BCVP(r, ireg, jreg, NORTH, VV, i);
          break;
        case BM_OUTLT1:
          for (i = iW + 1; i <= iE; i++) F(u, i, jN + 1) = -F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN + 1) = BCV(r, ireg, jreg, NORTH, VV) + F(v, i, jN);
          break;
        case BM_OUTLT2:
          for (i = iW; i <= iE; i++)
            F(v, i, jN) = F(v, i, jN - 1) - (F(u, i, jN) - F(u, i - 1, jN));
          for (i = iW + 1; i <= iE - 1; i++)
            F(u, i, jN + 1) = F(u, i - 1, jN + 1) + 3.0 * (F(u, i - 1, jN) - F(u, i, jN)) -
                              4.0 * (F(v, i, jN) - F(v, i, jN - 1));
          break;
        default: die("Wrong nBdTypeN flag", ireg, jreg);
      }
    }
}

/* PresBoundCond, bound_cond.f:853-1024 */
void w2o_pres_bound_cond(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                         double *p) {
  (void)nx; (void)ny;
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      int i, j, t;
      if (RTYP(r, ireg, jreg) == RM_BLOCKG) {
        for (j = jS + 1; j <= jN; j++)
          for (i = iW + 1; i <= iE; i++) F(p, i, j) = 0.0;
        for (j = jS + 1; j <= jN; j++) F(p, iW + 1, j) = BCV(r, ireg, jreg, WEST, VP) + F(p, iW, j);
        for (j = jS + 1; j <= jN; j++) F(p, iE, j) = BCV(r, ireg, jreg, EAST, VP) + F(p, iE + 1, j);
        for (i = iW + 1; i <= iE; i++) F(p, i, jS + 1) = BCV(r, ireg, jreg, SOUTH, VP) + F(p, i, jS);
        for (i = iW + 1; i <= iE; i++) F(p, i, jN) = BCV(r, ireg, jreg, NORTH, VP) + F(p, i, jN + 1);
        continue;
      }
      t = MBTP(r, ireg, jreg, WEST);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        for (j = jS + 1; j <= jN; j++) F(p, iW, j) = BCV(r, ireg, jreg, WEST, VP) + F(p, iW + 1, j);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        for (j = jS + 1; j <= jN; j++) F(p, iW, j) = 2.0 * BCV(r, ireg, jreg, WEST, VP) - F(p, iW + 1, j);
      } else if (t != BM_INTERN) die("Wrong nBdTypeW flag", ireg, jreg);
      t = MBTP(r, ireg, jreg, EAST);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        for (j = jS + 1; j <= jN; j++) F(p, iE + 1, j) = BCV(r, ireg, jreg, EAST, VP) + F(p, iE, j);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        for (j = jS + 1; j <= jN; j++) F(p, iE + 1, j) = 2.0 * BCV(r, ireg, jreg, EAST, VP) - F(p, iE, j);
      } else if (t != BM_INTERN) die("Wrong nBdTypeE flag", ireg, jreg);
      t = MBTP(r, ireg, jreg, SOUTH);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        for (i = iW + 1; i <= iE; i++) F(p, i, jS) = BCV(r, ireg, jreg, SOUTH, VP) + F(p, i, jS + 1);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        for (i = iW + 1; i <= iE; i++) F(p, i, jS) = 2.0 * BCV(r, ireg, jreg, SOUTH, VP) - F(p, i, jS + 1);
      } else if (t != BM_INTERN) die("Wrong nBdTypeS flag", ireg, jreg);
      t = MBTP(r, ireg, jreg, NORTH);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        for (i = iW + 1; i <= iE; i++) F(p, i, jN + 1) = BCV(r, ireg, jreg, NORTH, VP) + F(p, i, jN);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        for (i = iW + 1; i <= iE; i++) F(p, i, jN + 1) = 2.0 * BCV(r, ireg, jreg, NORTH, VP) - F(p, i, jN);
      } else if (t != BM_INTERN) die("Wrong nBdTypeN flag", ireg, jreg);
    }
}

/* ------------------------------------------------------------------ */
/* main.f                                                              */
/* ------------------------------------------------------------------ */

/* Cold start, main.f:606-641 */
int w2o_cold_start(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                   const w2o_params *prm, const w2o_metrics *m,
                   w2o_fields *f) {
  w2o_vel_bound_cond(c, nx, ny, r, f->u, f->v);
  int nconv = w2o_ppe(c, nx, ny, r, prm->lcartes, prm->npsolver, prm->msorit,
                      prm->dk, prm->sortol, prm->sorrel, m, f->u, f->v, f->p);
  w2o_pres_bound_cond(c, nx, ny, r, f->p);
  w2o_project(c, nx, ny, r, prm->dk, m, f->p, f->u, f->v);
  w2o_vel_bound_cond(c, nx, ny, r, f->u, f->v);
  return nconv;
}

/* One pass of the time loop, main.f:690-972 (nthermen = nsmallscl = 0, so the
 * momentum/energy loop runs once, main.f:736). */
int w2o_step(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
             const w2o_params *prm, const w2o_metrics *m, w2o_fields *f,
             int *nQLiter, int *nSorConv, double dif[4]) {
  return w2o_step_thermal(c, nx, ny, r, NULL, NULL, prm, m, f, nQLiter, nSorConv, dif);
}

int w2o_step_thermal(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                     const w2o_thermal *th, const w2o_thermal_params *tp,
                     const w2o_params *prm, const w2o_metrics *m, w2o_fields *f,
                     int *nQLiter, int *nSorConv, double dif[4]) {
  return w2o_step_atd(c, nx, ny, r, th, tp, prm, m, f, NULL, nQLiter, nSorConv, dif);
}

int w2o_step_atd(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                 const w2o_thermal *th, const w2o_thermal_params *tp,
                 const w2o_params *prm, const w2o_metrics *m, w2o_fields *f,
                 const w2o_atd_run *a, int *nQLiter, int *nSorConv, double dif[4]) {
  int i, j;
  const int therm = th && tp && tp->nthermen == 1;
  const int eqs = th && tp && tp->neqstate == 1;
  /* main.f:736: without the energy equation one pass */
  int nme = tp ? tp->nmeiter : 1;
  if (!therm && nme > 0) nme = 1;
  for (j = 0; j <= ny + 1; j++)
    for (i = 0; i <= nx + 1; i++) {
      F(f->pn, i, j) = F(f->p, i, j);
      F(f->un, i, j) = F(f->u, i, j);
      F(f->vn, i, j) = F(f->v, i, j);
      F(f->tn, i, j) = F(f->t, i, j);
      F(f->dn, i, j) = F(f->d, i, j);
    }
  if (a) /* main.f:708-730: keep the small scales of level n, add them to it */
    for (j = 0; j <= ny + 1; j++)
      for (i = 0; i <= nx + 1; i++) {
        F(a->usn, i, j) = F(a->uss, i, j);
        F(a->vsn, i, j) = F(a->vss, i, j);
        F(a->tsn, i, j) = F(a->tss, i, j);
        F(f->un, i, j) = F(f->un, i, j) + F(a->uss, i, j);
        F(f->vn, i, j) = F(f->vn, i, j) + F(a->vss, i, j);
        F(f->tn, i, j) = F(f->tn, i, j) + F(a->tss, i, j);
      }
  for (int l = 1; l <= nme; l++) {
    for (j = 0; j <= ny + 1; j++)
      for (i = 0; i <= nx + 1; i++) {
        F(f->us, i, j) = F(f->u, i, j);
        F(f->vs, i, j) = F(f->v, i, j);
        F(f->ts, i, j) = F(f->t, i, j);
      }
    *nQLiter = w2o_naux_momentum(c, nx, ny, prm->mqiter, r, prm->dk, prm->re,
                                 prm->fr, prm->qtol, m, f->d, f->dn, f->un,
                                 f->vn, f->us, f->vs);
    if (prm->nfiltu == 1) w2o_filter(c, nx, ny, VU, r, prm->fpu, f->us);
    if (prm->nfiltv == 1) w2o_filter(c, nx, ny, VV, r, prm->fpv, f->vs);
    w2o_vel_bound_cond(c, nx, ny, r, f->us, f->vs);
    w2o_pres_bound_cond(c, nx, ny, r, f->p);
    *nSorConv = w2o_ppe(c, nx, ny, r, prm->lcartes, prm->npsolver, prm->msorit,
                        prm->dk, prm->sortol, prm->sorrel, m, f->us, f->vs, f->p);
    w2o_pres_bound_cond(c, nx, ny, r, f->p);
    w2o_project(c, nx, ny, r, prm->dk, m, f->p, f->us, f->vs);
    w2o_vel_bound_cond(c, nx, ny, r, f->us, f->vs);
    w2o_pres_bound_cond(c, nx, ny, r, f->p);
    if (therm)
      w2o_therm_energy(c, nx, ny, r, th, prm->dk, tp->pe, m, f->un, f->vn, f->us, f->vs, f->tn, f->ts);
    if (eqs)
      w2o_eq_state(c, nx, ny, tp->uref, tp->densref, tp->tmax, tp->tref, tp->rconst, f->p, f->ts, f->d);
    /* main.f:857-859, the momentum/energy convergence test's norms */
    double me[3];
    me[0] = w2o_diff_max_norm(c, nx, ny, f->u, f->us);
    me[1] = w2o_diff_max_norm(c, nx, ny, f->v, f->vs);
    me[2] = w2o_diff_max_norm(c, nx, ny, f->t, f->ts);
    for (j = 0; j <= ny + 1; j++)
      for (i = 0; i <= nx + 1; i++) {
        F(f->u, i, j) = F(f->us, i, j);
        F(f->v, i, j) = F(f->vs, i, j);
        F(f->t, i, j) = F(f->ts, i, j);
      }
    /* difmax = max(dif(1),dif(2),dif(3)) (main.f:873) */
    double mx = me[0];
    if (me[1] > mx) mx = me[1];
    if (me[2] > mx) mx = me[2];
    if (l > 1 && mx < tp->dmeittol) break;
  }
  if (therm && tp->nfiltt == 1) w2o_filter_t(c, nx, ny, r, th, tp->fpt, f->t);
  if (a) { /* main.f:898-940: small scales of level n+1 from the large scales */
    for (j = 0; j <= ny + 1; j++)
      for (i = 0; i <= nx + 1; i++) {
        F(f->u, i, j) = F(f->u, i, j) - F(a->usn, i, j);
        F(f->v, i, j) = F(f->v, i, j) - F(a->vsn, i, j);
        F(f->t, i, j) = F(f->t, i, j) - F(a->tsn, i, j);
      }
    w2o_small_scale(c, a->state, nx, ny, 1, r, th, a->ap, m, f->u, f->v, f->t, a->uss,
                    a->vss, a->pss, a->tss);
    for (j = 0; j <= ny + 1; j++)
      for (i = 0; i <= nx + 1; i++) {
        F(f->u, i, j) = F(f->u, i, j) + F(a->uss, i, j);
        F(f->v, i, j) = F(f->v, i, j) + F(a->vss, i, j);
        F(f->t, i, j) = F(f->t, i, j) + F(a->tss, i, j);
      }
  }
  w2o_vel_bound_cond(c, nx, ny, r, f->u, f->v);
  w2o_pres_bound_cond(c, nx, ny, r, f->p);
  if (therm) w2o_temp_bound_cond(c, nx, ny, r, th, f->t);
  dif[0] = w2o_diff_max_norm(c, nx, ny, f->pn, f->p);
  dif[1] = w2o_diff_max_norm(c, nx, ny, f->un, f->u);
  dif[2] = w2o_diff_max_norm(c, nx, ny, f->vn, f->v);
  dif[3] = w2o_diff_max_norm(c, nx, ny, f->tn, f->t);
  double difmax = dif[0];
  for (int k = 1; k < 4; k++) difmax = dif[k] > difmax ? dif[k] : difmax;
  return difmax > 1.0e12 ? 1 : 0;
}

/* ------------------------------------------------------------------------
 * Small-scale (ATD) model: SmlSclBC (bound_cond.f:1211-1500) and SmallScale
 * (small_scale.f:31-578), the second caller of Ppe and Project.
 * ---------------------------------------------------------------------- */

void w2o_sml_scl_bc(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                    const w2o_thermal *th, double *u, double *v, double *p,
                    double *t) {
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      const int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      const int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      int i, j;
      /* image points: wall faces mirror (no-slip) or copy (no-stress) the
       * tangential component and zero the normal one */
      switch (MBTP(r, ireg, jreg, WEST)) {
        case BM_INTERN: break;
        case BM_WALL1: case BM_INLET:
          for (j = jS; j <= jN; j++) F(u, iW, j) = 0.0;
          for (j = jS + 1; j <= jN; j++) F(v, iW, j) = -F(v, iW + 1, j);
          break;
        case BM_WALL2:
          for (j = jS; j <= jN; j++) F(u, iW, j) = 0.0;
          for (j = jS + 1; j <= jN; j++) F(v, iW, j) = F(v, iW + 1, j);
          break;
        case BM_OUTLT1:
          if (iW < 1) die("SmlSclBC: west outlet writes column iW-1 outside the array", ireg, jreg);
          for (j = jS; j <= jN; j++) F(u, iW - 1, j) = F(u, iW, j);
          for (j = jS + 1; j <= jN; j++) F(v, iW, j) = -F(v, iW + 1, j);
          break;
        case BM_OUTLT2:
          for (j = jS; j <= jN; j++) {
            if (j < 1) die("SmlSclBC: west outlet reads row j-1 outside the array", ireg, jreg);
            F(u, iW, j) = F(u, iW + 1, j) - F(v, iW, j) + F(v, iW, j - 1);
          }
          for (j = jS + 1; j <= jN; j++)
            F(v, iW, j) = -F(v, iW, j - 1) + 5.0 * (F(v, iW + 1, j) - F(v, iW + 1, j - 1)) +
                          8.0 * (F(u, iW + 1, j) - F(u, iW, j));
          break;
        default: die("Wrong nBdTypeW flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, EAST)) {
        case BM_INTERN: break;
        case BM_WALL1: case BM_INLET:
          for (j = jS; j <= jN; j++) F(u, iE, j) = 0.0;
          for (j = jS + 1; j <= jN; j++) F(v, iE + 1, j) = -F(v, iE, j);
          break;
        case BM_WALL2:
          for (j = jS; j <= jN; j++) F(u, iE, j) = 0.0;
          for (j = jS + 1; j <= jN; j++) F(v, iE + 1, j) = F(v, iE, j);
          break;
        case BM_OUTLT1: /* the u row assigns u(iE+1,j) to itself */
          for (j = jS + 1; j <= jN; j++) F(v, iE + 1, j) = -F(v, iE, j);
          break;
        case BM_OUTLT2:
          for (j = jS + 1; j <= jN; j++) F(u, iE, j) = F(u, iE - 1, j) - (F(v, iE, j) - F(v, iE, j - 1));
          for (j = jS + 1; j <= jN - 1; j++)
            F(v, iE + 1, j) = F(v, iE + 1, j - 1) + 3.0 * (F(v, iE, j - 1) - F(v, iE, j)) -
                              4.0 * (F(u, iE, j) - F(u, iE - 1, j));
          break;
        default: die("Wrong nBdTypeE flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, SOUTH)) {
        case BM_INTERN: break;
        case BM_WALL1: case BM_INLET:
          for (i = iW + 1; i <= iE; i++) F(u, i, jS) = -F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS) = 0.0;
          break;
        case BM_WALL2:
          for (i = iW + 1; i <= iE; i++) F(u, i, jS) = F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS) = 0.0;
          break;
        case BM_OUTLT1:
          if (jS < 1) die("SmlSclBC: south outlet writes row jS-1 outside the array", ireg, jreg);
          for (i = iW + 1; i <= iE; i++) F(u, i, jS) = -F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS - 1) = F(v, i, jS);
          break;
        case BM_OUTLT2:
          if (jS < 1 || iW < 1) die("SmlSclBC: south outlet reaches outside the array", ireg, jreg);
          for (i = iW + 1; i <= iE; i++)
            F(u, i, jS - 1) = F(u, i - 1, jS - 1) + 5.0 * (F(u, i, jS) - F(u, i - 1, jS)) +
                              8.0 * (F(v, i, jS) - F(v, i - 1, jS - 1));
          for (i = iW; i <= iE; i++) F(v, i, jS - 1) = F(v, i, jS) - F(u, i, jS) - F(u, i - 1, jS);
          break;
        default: die("Wrong nBdTypeS flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, NORTH)) {
        case BM_INTERN: break;
        case BM_WALL1: case BM_INLET:
          for (i = iW + 1; i <= iE; i++) F(u, i, jN + 1) = -F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN) = 0.0;
          break;
        case BM_WALL2:
          for (i = iW + 1; i <= iE; i++) F(u, i, jN + 1) = F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN) = 0.0;
          break;
        case BM_OUTLT1:
          for (i = iW + 1; i <= iE; i++) F(u, i, jN + 1) = -F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN + 1) = F(v, i, jN);
          break;
        case BM_OUTLT2:
          if (iW < 1) die("SmlSclBC: north outlet reads column iW-1 outside the array", ireg, jreg);
          for (i = iW; i <= iE; i++) F(v, i, jN) = F(v, i, jN - 1) - (F(u, i, jN) - F(u, i - 1, jN));
          for (i = iW + 1; i <= iE - 1; i++)
            F(u, i, jN + 1) = F(u, i - 1, jN + 1) + 3.0 * (F(u, i - 1, jN) - F(u, i, jN)) -
                              4.0 * (F(v, i, jN) - F(v, i, jN - 1));
          break;
        default: die("Wrong nBdTypeN flag", ireg, jreg);
      }
    }
  /* the pressure takes the large-scale pressure conditions */
  w2o_pres_bound_cond(c, nx, ny, r, p);
  /* small-scale temperature: homogeneous image conditions */
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      const int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      const int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      int i, j;
      if (TRT(th, r, ireg, jreg) == RT_TEMPER) {
        for (j = jS + 1; j <= jN; j++)
          for (i = iW + 1; i <= iE; i++) F(t, i, j) = 0.0;
        for (j = jS + 1; j <= jN; j++) F(t, iW + 1, j) = -F(t, iW, j);
        for (j = jS + 1; j <= jN; j++) F(t, iE, j) = -F(t, iE + 1, j);
        for (i = iW + 1; i <= iE; i++) F(t, i, jS + 1) = -F(t, i, jS);
        for (i = iW + 1; i <= iE; i++) F(t, i, jN) = -F(t, i, jN + 1);
        continue;
      }
      for (int face = WEST; face <= NORTH; face++) {
        const int bt = TBT(th, r, ireg, jreg, face);
        if (bt == BT_INTERN) continue;
        if (bt != BT_TEMPER && bt != BT_HTFLUX) die("Wrong nTemBdTp flag", ireg, jreg);
        const double sg = bt == BT_TEMPER ? -1.0 : 1.0;
        if (face == WEST)
          for (j = jS + 1; j <= jN; j++) F(t, iW, j) = sg * F(t, iW + 1, j);
        else if (face == EAST)
          for (j = jS + 1; j <= jN; j++) F(t, iE + 1, j) = sg * F(t, iE, j);
        else if (face == SOUTH)
          for (i = iW + 1; i <= iE; i++) F(t, i, jS) = sg * F(t, i, jS + 1);
        else
          for (i = iW + 1; i <= iE; i++) F(t, i, jN + 1) = sg * F(t, i, jN);
      }
    }
}

/* small_scale.f keeps every local between calls (a bare SAVE): the map
 * iterates and the cell areas carry information from call to call, and the
 * work arrays keep whatever their never-written borders hold (zero). */
struct w2o_atd {
  size_t nf;
  double *umap, *vmap, *tmap;  /* (0:mnx,0:mny,3) */
  double *area, tarea;
  double *xz, *xe, *yz, *ye, *rj, *ul, *vl, *tl, *uc, *vc, *uf, *vf, *tf;
};

w2o_atd *w2o_atd_create(int mnx, int mny) {
  w2o_atd *s = (w2o_atd *)calloc(1, sizeof(w2o_atd));
  s->nf = (size_t)(mnx + 1) * (size_t)(mny + 1);
  double **arr[] = {&s->area, &s->xz, &s->xe, &s->yz, &s->ye, &s->rj, &s->ul, &s->vl,
                    &s->tl, &s->uc, &s->vc, &s->uf, &s->vf, &s->tf};
  for (size_t k = 0; k < sizeof(arr) / sizeof(arr[0]); k++) *arr[k] = (double *)calloc(s->nf, sizeof(double));
  s->umap = (double *)calloc(3 * s->nf, sizeof(double));
  s->vmap = (double *)calloc(3 * s->nf, sizeof(double));
  s->tmap = (double *)calloc(3 * s->nf, sizeof(double));
  return s;
}

void w2o_atd_destroy(w2o_atd *s) {
  if (!s) return;
  double *arr[] = {s->area, s->xz, s->xe, s->yz, s->ye, s->rj, s->ul, s->vl, s->tl,
                   s->uc, s->vc, s->uf, s->vf, s->tf, s->umap, s->vmap, s->tmap};
  for (size_t k = 0; k < sizeof(arr) / sizeof(arr[0]); k++) free(arr[k]);
  free(s);
}

/* one step of the logistic map x <- r A x (1 - B |x|) of small_scale.f */
static inline double atd_map(double rm, double x) {
  const double A = 4.82842712474, B = 1.47839783948;
  return rm * A * x * (1.0 - B * fabs(x));
}

int w2o_small_scale(w2o_ctx *c, w2o_atd *s, int nx, int ny, int initflg,
                    const w2o_regions *r, const w2o_thermal *th,
                    const w2o_atd_params *ap, const w2o_metrics *m,
                    const double *u1, const double *v1, const double *t1,
                    double *uss, double *vss, double *pss, double *tss) {
  const double rc = 0.20710678119;
  const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  const double piosr2 = acos(-1.0) / sqrt(2.0);
  const double hs = ap->dlref * ap->hscoef, dk = ap->dka * ap->dlref / ap->uref;
  const double pr = ap->pe / ap->re, rnu = ap->uref * ap->dlref / ap->re, dkappa = rnu / pr;
  const double dl = ap->dlref;
  const size_t nf = s->nf;
  if (initflg <= 0) {
    /* seed the three maps per variable, sweeping j fastest */
    double um = 0.92, vm = 0.31, tm = 0.50;
    for (int i = 0; i <= nx + 1; i++)
      for (int j = 0; j <= ny + 1; j++) {
        for (int l = 0; l < 3; l++) {
          um = atd_map(rc, um);
          vm = atd_map(rc, vm);
          tm = atd_map(rc, tm);
          s->umap[IX(i, j) + l * nf] = um;
          s->vmap[IX(i, j) + l * nf] = vm;
          s->tmap[IX(i, j) + l * nf] = tm;
        }
        F(uss, i, j) = 0.0;
        F(vss, i, j) = 0.0;
        F(tss, i, j) = 0.0;
      }
    s->tarea = 0.0;
    for (int i = 1; i <= nx; i++)
      for (int j = 1; j <= ny; j++) {
        F(s->area, i, j) = 1.0 / F(m->djc, i, j);
        s->tarea = s->tarea + F(s->area, i, j);
      }
    if (initflg < 0) return 0;
  }
  /* dimensional metrics, cell-centred large-scale fields, contravariant
   * velocity; the copies that will be low-pass filtered */
  for (int i = 1; i <= nx; i++)
    for (int j = 1; j <= ny; j++) {
      F(s->xz, i, j) = dl * F(m->xzc, i, j);
      F(s->xe, i, j) = dl * F(m->xec, i, j);
      F(s->yz, i, j) = dl * F(m->yzc, i, j);
      F(s->ye, i, j) = dl * F(m->yec, i, j);
      F(s->rj, i, j) = F(m->djc, i, j) / (dl * dl);
      F(s->vl, i, j) = ap->uref * (F(v1, i, j) + F(v1, i, j - 1)) * 0.5;
      F(s->ul, i, j) = ap->uref * (F(u1, i, j) + F(u1, i - 1, j)) * 0.5;
      F(s->tl, i, j) = (ap->tmax - ap->tref) * F(t1, i, j) + ap->tref;
      F(s->uc, i, j) = F(s->ye, i, j) * F(s->ul, i, j) - F(s->xe, i, j) * F(s->vl, i, j);
      F(s->vc, i, j) = F(s->xz, i, j) * F(s->vl, i, j) - F(s->yz, i, j) * F(s->ul, i, j);
      F(s->uf, i, j) = F(s->uc, i, j);
      F(s->vf, i, j) = F(s->vc, i, j);
      F(s->tf, i, j) = F(s->tl, i, j);
    }
  w2o_temp_bound_cond(c, nx, ny, r, th, s->tf);
  w2o_filter(c, nx, ny, VU, r, ap->fp[0], s->uf);
  w2o_filter(c, nx, ny, VV, r, ap->fp[1], s->vf);
  w2o_filter_t(c, nx, ny, r, th, ap->fp[3], s->tf);
  /* high-pass parts: field minus its Shuman-filtered copy */
  for (int i = 1; i <= nx; i++)
    for (int j = 1; j <= ny; j++) {
      F(s->uf, i, j) = F(s->uc, i, j) - F(s->uf, i, j);
      F(s->vf, i, j) = F(s->vc, i, j) - F(s->vf, i, j);
      F(s->tf, i, j) = F(s->tl, i, j) - F(s->tf, i, j);
    }
#define CD_I(a) ((F(a, i + 1, j) - F(a, i - 1, j)) * 0.5)
#define CD_J(a) ((F(a, i, j + 1) - F(a, i, j - 1)) * 0.5)
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      const int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      const int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      if (RTYP(r, ireg, jreg) == RM_BLOCKG || TRT(th, r, ireg, jreg) == RT_TEMPER) continue;
      for (int i = iW + 1; i <= iE; i++)
        for (int j = jS + 1; j <= jN; j++) {
          const double xz = F(s->xz, i, j), xe = F(s->xe, i, j), yz = F(s->yz, i, j);
          const double ye = F(s->ye, i, j), rj = F(s->rj, i, j);
          const double hxy = sqrt(xz * xz + yz * yz + xe * xe + ye * ye);
          /* |grad u| and |grad T| of the unfiltered large scales (physical
           * derivatives through the inverse Jacobian) */
          double uz = CD_I(s->ul), ue = CD_J(s->ul), vz = CD_I(s->vl), ve = CD_J(s->vl);
          double q1 = rj * (ye * uz - yz * ue), q2 = rj * (xz * ue - xe * uz);
          double q3 = rj * (ye * vz - yz * ve), q4 = rj * (xz * ve - xe * vz);
          const double delu2n = sqrt(q1 * q1 + q2 * q2 + q3 * q3 + q4 * q4);
          double tz = CD_I(s->tl), te = CD_J(s->tl);
          q1 = rj * (ye * tz - yz * te);
          q2 = rj * (xz * te - xe * tz);
          const double delt2n = sqrt(q1 * q1 + q2 * q2);
          const double reh = delu2n * (hxy * hxy) / rnu, peh = pr * reh;
          if (!(peh > 3.0)) continue;
          const double cuU = ap->cu0 * ap->temcoef, cuV = ap->cu0, cuT = ap->cu0;
          int nmap = 0;
          if (ap->cu0 > (double)1.0e-10f) {
            const double ts = ap->tscoef * piosr2 * pow(reh, third) / (ap->cu0 * delu2n);
            nmap = (int)(1.0 + dk / ts);
          }
          if (nmap > 50) nmap = 50;
          const double bnum = sqrt(15.0) * pow((hs * hs) * delu2n / rnu, sixth);
          const double rmap = ap->rmax * tanh(pow(bnum / ap->bnumc, ap->rlc) * atanh(rc / ap->rmax));
          /* anisotropy: gradients of the high-pass parts */
          uz = CD_I(s->uf); ue = CD_J(s->uf);
          vz = CD_I(s->vf); ve = CD_J(s->vf);
          tz = CD_I(s->tf); te = CD_J(s->tf);
          const double gu1 = rj * (ye * uz - yz * ue), gu2 = rj * (xz * ue - xe * uz);
          const double gv1 = rj * (ye * vz - yz * ve), gv2 = rj * (xz * ve - xe * vz);
          const double gt1 = rj * (ye * tz - yz * te), gt2 = rj * (xz * te - xe * tz);
          const double gu = sqrt(gu1 * gu1 + gu2 * gu2), gv = sqrt(gv1 * gv1 + gv2 * gv2);
          const double gt = sqrt(gt1 * gt1 + gt2 * gt2);
          const double grd = sqrt(gu * gu + gv * gv + gt * gt);
          const double s1 = gu / grd, s2 = gv / grd;
          const double a1 = xz * s1 + xe * s2, a2 = yz * s1 + ye * s2;
          const double rnrmjs = sqrt(a1 * a1 + a2 * a2);
          const double zeta1 = sqrt(2.0) * s1 / rnrmjs, zeta2 = sqrt(2.0) * s2 / rnrmjs;
          double alf11 = 0.0, alf12 = 0.0, alf21 = 0.0, alf22 = 0.0;
          double alf31 = 0.0, alf32 = 0.0, alf33 = 0.0;
          if (fabs(gu) > 0.0) { alf11 = gu1 / gu; alf12 = gu2 / gu; }
          if (fabs(gv) > 0.0) { alf21 = gv1 / gv; alf22 = gv2 / gv; }
          if (fabs(gt) > 0.0) {
            alf31 = gu1 / gt;
            alf32 = gu2 / gt;
            alf33 = sqrt(gt1 * gt1 + gt2 * gt2) / gt;
          }
          /* advance the nine chaotic maps nmap times and keep them */
          double mp[9];
          for (int l = 0; l < 3; l++) {
            mp[l] = s->umap[IX(i, j) + l * nf];
            mp[3 + l] = s->vmap[IX(i, j) + l * nf];
            mp[6 + l] = s->tmap[IX(i, j) + l * nf];
          }
          for (int k = 0; k < nmap; k++)
            for (int l = 0; l < 9; l++) mp[l] = atd_map(rmap, mp[l]);
          for (int l = 0; l < 3; l++) {
            s->umap[IX(i, j) + l * nf] = mp[l];
            s->vmap[IX(i, j) + l * nf] = mp[3 + l];
            s->tmap[IX(i, j) + l * nf] = mp[6 + l];
          }
          /* both velocity combinations draw on the u maps */
          const double um = alf11 * mp[0] + alf12 * mp[1];
          const double vm = alf21 * mp[0] + alf22 * mp[1];
          const double tm = alf31 * mp[6] + alf32 * mp[7] + alf33 * mp[8];
          const double sq = sqrt(rnu * delu2n), r6 = pow(reh, sixth);
          double av = cuV * r6 * sq;
          double at = pow(3.0 * pow(cuT, 4.0) * peh / pr, sixth) * sqrt(dkappa);
          at = at * delt2n / sqrt(delu2n) * ap->temcoef;
          const double ascale = sqrt(F(s->area, i, j) / s->tarea);
          const double h3 = pow(hxy, third);
          (void)cuU; /* its amplitude is computed and not used */
          av = av * ascale * h3;
          at = at * ascale * h3;
          /* the u component takes av, as the v component does */
          const double uscon = av * zeta1 * um, vscon = av * zeta2 * vm;
          double us = rj * (xz * uscon + ye * vscon) / ap->uref;
          double vs = rj * (ye * vscon + yz * uscon) / ap->uref;
          double tsv = (at * tm * 1.0) / (ap->tmax - ap->tref);
          F(uss, i, j) = fabs(us) < 1.0e-14 ? 0.0 : us;
          F(vss, i, j) = fabs(vs) < 1.0e-14 ? 0.0 : vs;
          F(tss, i, j) = fabs(tsv) < 1.0e-14 ? 0.0 : tsv;
        }
    }
#undef CD_I
#undef CD_J
  w2o_sml_scl_bc(c, nx, ny, r, th, uss, vss, pss, tss);
  for (int j = 0; j <= ny; j++)
    for (int i = 0; i <= nx; i++) F(pss, i, j) = 0.0;
  w2o_sml_scl_bc(c, nx, ny, r, th, uss, vss, pss, tss);
  const int nsor = w2o_ppe(c, nx, ny, r, ap->lcartes, ap->npsolver, ap->msorit, ap->dka,
                           ap->sortol, ap->sorrel, m, uss, vss, pss);
  w2o_sml_scl_bc(c, nx, ny, r, th, uss, vss, pss, tss);
  w2o_project(c, nx, ny, r, ap->dka, m, pss, uss, vss);
  return nsor;
}
