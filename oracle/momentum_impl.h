/*
 * momentum_impl.h -- TEST INFRASTRUCTURE: the oracle's nAuxMomentum
 * (momentum.f:33-1339, with DMaxNorm utility.f:479-507 and VelOutflowBCs
 * bound_cond.f:1656-1874), written once for a floating type REAL and
 * included twice by wolfd2_oracle.c:
 *   REAL = double, FN(x) = x      -- the FP64 restatement of the reference;
 *   REAL = float,  FN(x) = x_f32  -- the same operations in IEEE single, the
 *                                    checker of the GPU's FP32 momentum.
 * Literals are R(x) = (REAL)(x), so single-precision instances evaluate in
 * single precision throughout (no promotion to double); region constants and
 * the step parameters dk, re, fr enter as R(value).  qtol stays double: the
 * stopping test compares the REAL maximum, widened, against it.
 *
 * Expects from the includer: REAL, R, FN, RABS, RSQRT, MOMWS (work storage
 * type), METRICS (metric pointer struct), MOM_WX / MOM_WY / MOM_DUS / MOM_DVS
 * (the context's storage for this type), and the F/RBRD/RTYP/MBTP/BCV/RPAR
 * accessors and die() of wolfd2_oracle.c.
 */

/* VelOutflowBCs, bound_cond.f:1656-1874 */
void FN(w2o_vel_outflow_bcs)(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                         REAL *u, REAL *v) {
  (void)nx; (void)ny;
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      int i, j;
      switch (MBTP(r, ireg, jreg, WEST)) {
        case BM_INTERN: case BM_WALL1: case BM_WALL2: case BM_INLET: break;
        case BM_OUTLT1:
          for (j = jS; j <= jN; j++) F(u, iW - 1, j) = R(BCV(r, ireg, jreg, WEST, VU)) + F(u, iW, j);
          for (j = jS + 1; j <= jN; j++) F(v, iW, j) = -F(v, iW + 1, j);
          break;
        case BM_OUTLT2:
          for (j = jS + 1; j <= jN; j++)
            F(u, iW, j) = F(u, iW + 1, j) - F(v, iW + 1, j) + F(v, iW + 1, j - 1);
          for (j = jS + 1; j <= jN; j++)
            F(v, iW, j) = -F(v, iW, j - 1) + R(5.0) * (F(v, iW + 1, j) - F(v, iW + 1, j - 1)) +
                          R(8.0) * (F(u, iW + 1, j) - F(u, iW, j));
          break;
        default: die("Wrong nBdTypeW flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, EAST)) {
        case BM_INTERN: case BM_WALL1: case BM_WALL2: case BM_INLET: break;
        case BM_OUTLT1:
          for (j = jS; j <= jN; j++) F(u, iE + 1, j) = R(BCV(r, ireg, jreg, EAST, VU)) + F(u, iE, j);
          for (j = jS + 1; j <= jN; j++) F(v, iE + 1, j) = -F(v, iE, j);
          break;
        case BM_OUTLT2:
          for (j = jS + 1; j <= jN; j++)
            F(u, iE, j) = F(u, iE - 1, j) - (F(v, iE, j) - F(v, iE, j - 1));
          for (j = jS + 1; j <= jN - 1; j++)
            F(v, iE + 1, j) = F(v, iE + 1, j - 1) + R(3.0) * (F(v, iE, j - 1) - F(v, iE, j)) -
                              R(4.0) * (F(u, iE, j) - F(u, iE - 1, j));
          break;
        default: die("Wrong nBdTypeE flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, SOUTH)) {
        case BM_INTERN: case BM_WALL1: case BM_WALL2: case BM_INLET: break;
        case BM_OUTLT1:
          for (i = iW + 1; i <= iE; i++) F(u, i, jS) = -F(u, i, jS + 1);
          for (i = iW; i <= iE; i++) F(v, i, jS) = R(BCV(r, ireg, jreg, SOUTH, VV)) + F(v, i, jS);
          break;
        case BM_OUTLT2:
          for (i = iW + 1; i <= iE; i++)
            F(v, i, jS) = F(v, i, jS + 1) + (F(u, i, jS + 1) - F(u, i - 1, jS + 1));
          for (i = iW + 1; i <= iE - 1; i++)
            F(u, i, jS) = F(u, i - 1, jS) + R(3.0) * (F(u, i - 1, jS + 1) - F(u, i, jS + 1)) -
                          R(4.0) * (F(v, i, jS + 1) - F(v, i, jS));
          break;
        default: die("Wrong nBdTypeS flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, NORTH)) {
        case BM_INTERN: case BM_WALL1: case BM_WALL2: case BM_INLET: break;
        case BM_OUTLT1:
          for (i = iW + 1; i <= iE; i++) F(u, i, jN + 1) = -F(u, i, jN);
          for (i = iW; i <= iE; i++) F(v, i, jN + 1) = R(BCV(r, ireg, jreg, NORTH, VV)) + F(v, i, jN);
          break;
        case BM_OUTLT2:
          for (i = iW; i <= iE; i++)
            F(v, i, jN) = F(v, i, jN - 1) - (F(u, i, jN) - F(u, i - 1, jN));
          for (i = iW + 1; i <= iE - 1; i++)
            F(u, i, jN + 1) = F(u, i - 1, jN + 1) + R(3.0) * (F(u, i - 1, jN) - F(u, i, jN)) -
                              R(4.0) * (F(v, i, jN) - F(v, i, jN - 1));
          break;
        default: die("Wrong nBdTypeN flag", ireg, jreg);
      }
    }
}

/* AltTridLU, momentum.f:1307-1339.  a is a(3,n) column-major: a(k,i) at
 * a[(k-1) + 3*(i-1)].  Row 1's super-diagonal is divided by the ORIGINAL
 * diagonal of row 2 (momentum.f:1319). */
void FN(w2o_alt_trid_lu)(int n, REAL *a, REAL *b) {
#define A(k, i) a[((k)-1) + 3 * (size_t)((i)-1)]
#define B(i) b[(i)-1]
  int i;
  A(3, 1) = A(3, 1) / A(2, 2);
  B(1) = B(1) / A(2, 1);
  for (i = 2; i <= n - 1; i++) {
    A(2, i) = A(2, i) - (A(1, i) * A(3, i - 1));
    A(3, i) = A(3, i) / A(2, i);
    B(i) = (B(i) - A(1, i) * B(i - 1)) / A(2, i);
  }
  A(2, n) = A(2, n) - (A(1, n) * A(3, n - 1));
  B(n) = (B(n) - A(1, n) * B(n - 1)) / A(2, n);
  for (i = n - 1; i >= 1; i--) B(i) = B(i) - (A(3, i) * B(i + 1));
#undef A
#undef B
}

/* ConvCoef, momentum.f:864-981 (cases 1, 2, 4, 5 of the momentum
 * equations; 3 and 6 of the thermal energy equation). */
static void FN(conv_coef)(w2o_ctx *c, int nx, int ny, int ncomp, int njacob,
                      const REAL *xzi, const REAL *xet, const REAL *yzi,
                      const REAL *yet, const REAL *u, const REAL *v,
                      REAL *cc1, REAL *cc2) {
  int i, j;
  REAL djac = R(1.0);
  if (njacob == 1) djac = R(2.0);
  switch (ncomp) {
    case 1:
      for (j = 1; j <= ny + 1; j++)
        for (i = 1; i <= nx + 1; i++)
          F(cc1, i, j) = (djac * F(yet, i, j) * (F(u, i, j) + F(u, i - 1, j)) -
                          F(xet, i, j) * (F(v, i, j) + F(v, i, j - 1))) * R(0.5);
      for (j = 1; j <= ny; j++)
        for (i = 1; i <= nx; i++)
          F(cc2, i, j) = (F(xzi, i, j) * (F(v, i + 1, j) + F(v, i, j)) -
                          djac * F(yzi, i, j) * (F(u, i, j + 1) + F(u, i, j))) * R(0.5);
      break;
    case 2:
      for (j = 1; j <= ny; j++)
        for (i = 1; i <= nx; i++)
          F(cc1, i, j) = (F(yet, i, j) * (F(u, i, j + 1) + F(u, i, j)) -
                          djac * F(xet, i, j) * (F(v, i + 1, j) + F(v, i, j))) * R(0.5);
      for (j = 1; j <= ny + 1; j++)
        for (i = 1; i <= nx + 1; i++)
          F(cc2, i, j) = (djac * F(xzi, i, j) * (F(v, i, j) + F(v, i, j - 1)) -
                          F(yzi, i, j) * (F(u, i, j) + F(u, i - 1, j))) * R(0.5);
      break;
    case 4:
      for (j = 1; j <= ny; j++)
        for (i = 0; i <= nx; i++) {
          F(cc1, i, j) = djac * F(yet, i, j) * F(u, i, j) -
                         F(xet, i, j) * (F(v, i + 1, j) + F(v, i, j) +
                                         F(v, i + 1, j - 1) + F(v, i, j - 1)) / R(4.0);
          F(cc2, i, j) = F(xzi, i, j) * (F(v, i + 1, j) + F(v, i, j) +
                                         F(v, i + 1, j - 1) + F(v, i, j - 1)) / R(4.0) -
                         djac * F(yzi, i, j) * F(u, i, j);
        }
      break;
    case 5:
      for (j = 0; j <= ny; j++)
        for (i = 1; i <= nx; i++) {
          F(cc1, i, j) = F(yet, i, j) * (F(u, i, j + 1) + F(u, i - 1, j + 1) +
                                         F(u, i, j) + F(u, i - 1, j)) / R(4.0) -
                         djac * F(xet, i, j) * F(v, i, j);
          F(cc2, i, j) = djac * F(xzi, i, j) * F(v, i, j) -
                         F(yzi, i, j) * (F(u, i, j + 1) + F(u, i - 1, j + 1) +
                                         F(u, i, j) + F(u, i - 1, j)) / R(4.0);
        }
      break;
    case 3:
      for (j = 1; j <= ny; j++)
        for (i = 1; i <= nx; i++) {
          F(cc1, i, j) = (F(yet, i, j) * F(u, i, j) -
                          F(xet, i, j) * (F(v, i + 1, j) + F(v, i, j) + F(v, i + 1, j - 1) +
                                          F(v, i, j - 1)) / R(4.0)) * R(0.5);
          F(cc2, i, j) = (F(xzi, i, j) * F(v, i, j) -
                          F(yzi, i, j) * (F(u, i, j + 1) + F(u, i - 1, j + 1) + F(u, i, j) +
                                          F(u, i - 1, j)) / R(4.0)) * R(0.5);
        }
      break;
    case 6:
      for (j = 1; j <= ny + 1; j++)
        for (i = 1; i <= nx + 1; i++) {
          F(cc1, i, j) = (F(yet, i, j) * (F(u, i, j) + F(u, i - 1, j)) -
                          F(xet, i, j) * (F(v, i, j) + F(v, i, j - 1))) * R(0.5);
          F(cc2, i, j) = (F(xzi, i, j) * (F(v, i, j) + F(v, i, j - 1)) -
                          F(yzi, i, j) * (F(u, i, j) + F(u, i - 1, j))) * R(0.5);
        }
      break;
    default:
      die("Error: Wrong component flag passed to ConvCoef", ncomp, 0);
  }
}

/* DConvU, momentum.f:987-1009 */
static void FN(dconv_u)(w2o_ctx *c, int nx, int ny, const REAL *c1,
                    const REAL *c2, const REAL *u, REAL *cv) {
  for (int j = 2; j <= ny; j++)
    for (int i = 1; i <= nx; i++)
      F(cv, i, j) = -F(c2, i, j - 1) * F(u, i, j - 1) - F(c1, i, j) * F(u, i - 1, j) +
                    (F(c1, i + 1, j) - F(c1, i, j) + F(c2, i, j) - F(c2, i, j - 1)) *
                        F(u, i, j) +
                    F(c1, i + 1, j) * F(u, i + 1, j) + F(c2, i, j) * F(u, i, j + 1);
}

/* DDiffU, momentum.f:1015-1045 */
static void FN(ddiff_u)(w2o_ctx *c, int nx, int ny, const REAL *ac,
                    const REAL *bc, const REAL *bn, const REAL *gn,
                    const REAL *u, REAL *d) {
  REAL s1, s2;
  for (int j = 2; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      s1 = F(ac, i + 1, j) * (F(u, i + 1, j) - F(u, i, j)) -
           F(ac, i, j) * (F(u, i, j) - F(u, i - 1, j)) +
           F(bc, i + 1, j) * (F(u, i + 1, j + 1) + F(u, i, j + 1) -
                              F(u, i + 1, j - 1) - F(u, i, j - 1)) -
           F(bc, i, j) * (F(u, i, j + 1) + F(u, i - 1, j + 1) - F(u, i, j - 1) -
                          F(u, i - 1, j - 1));
      s2 = F(bn, i, j) * (F(u, i + 1, j + 1) + F(u, i + 1, j) -
                          F(u, i - 1, j + 1) - F(u, i - 1, j)) -
           F(bn, i, j - 1) * (F(u, i + 1, j) + F(u, i + 1, j - 1) -
                              F(u, i - 1, j) - F(u, i - 1, j - 1)) +
           F(gn, i, j) * (F(u, i, j + 1) - F(u, i, j)) -
           F(gn, i, j - 1) * (F(u, i, j) - F(u, i, j - 1));
      F(d, i, j) = s1 + s2;
    }
}

/* DConvV, momentum.f:1051-1073 */
static void FN(dconv_v)(w2o_ctx *c, int nx, int ny, const REAL *c1,
                    const REAL *c2, const REAL *v, REAL *cv) {
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx; i++)
      F(cv, i, j) = -F(c2, i, j) * F(v, i, j - 1) - F(c1, i - 1, j) * F(v, i - 1, j) +
                    (F(c1, i, j) - F(c1, i - 1, j) + F(c2, i, j + 1) - F(c2, i, j)) *
                        F(v, i, j) +
                    F(c1, i, j) * F(v, i + 1, j) + F(c2, i, j + 1) * F(v, i, j + 1);
}

/* DDiffV, momentum.f:1079-1109 */
static void FN(ddiff_v)(w2o_ctx *c, int nx, int ny, const REAL *an,
                    const REAL *bc, const REAL *bn, const REAL *gc,
                    const REAL *v, REAL *d) {
  REAL s1, s2;
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx; i++) {
      s1 = F(an, i, j) * (F(v, i + 1, j) - F(v, i, j)) -
           F(an, i - 1, j) * (F(v, i, j) - F(v, i - 1, j)) +
           F(bn, i, j) * (F(v, i + 1, j + 1) + F(v, i, j + 1) -
                          F(v, i + 1, j - 1) - F(v, i, j - 1)) -
           F(bn, i - 1, j) * (F(v, i, j + 1) + F(v, i - 1, j + 1) -
                              F(v, i, j - 1) - F(v, i - 1, j - 1));
      s2 = F(bc, i, j + 1) * (F(v, i + 1, j + 1) + F(v, i + 1, j) -
                              F(v, i - 1, j + 1) - F(v, i - 1, j)) -
           F(bc, i, j) * (F(v, i + 1, j) + F(v, i + 1, j - 1) - F(v, i - 1, j) -
                          F(v, i - 1, j - 1)) +
           F(gc, i, j + 1) * (F(v, i, j + 1) - F(v, i, j)) -
           F(gc, i, j) * (F(v, i, j) - F(v, i, j - 1));
      F(d, i, j) = s1 + s2;
    }
}

/* PorosCoef, momentum.f:1115-1226 */
static void FN(poros_coef)(w2o_ctx *c, int nx, int ny, int ncomp, int njacob,
                       const w2o_regions *r, const REAL *u, const REAL *v,
                       REAL *cp) {
  (void)nx; (void)ny;
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      if (RTYP(r, ireg, jreg) != RM_POROUS) {
        for (int j = jS; j <= jN; j++)
          for (int i = iW; i <= iE; i++) F(cp, i, j) = R(0.0);
        continue;
      }
      REAL porc1 = R(RPAR(dPRporc1, r, ireg, jreg));
      REAL porc2 = R(RPAR(dPRporc2, r, ireg, jreg));
      REAL unorm, unrm1, t;
      if (ncomp == 1) {
        for (int j = jS + 1; j <= jN; j++)
          for (int i = iW; i <= iE; i++) {
            /* the reference divides only the last v term by 4 */
            t = F(v, i, j) + F(v, i + 1, j) + F(v, i, j - 1) + F(v, i + 1, j - 1) / R(4.0);
            unorm = RSQRT(F(u, i, j) * F(u, i, j) + t * t);
            unrm1 = R(0.0);
            if (unorm > R(1.0e-8)) unrm1 = (F(u, i, j) * F(u, i, j)) / unorm;
            if (njacob == 1) unorm = unrm1 + unorm;
            F(cp, i, j) = porc1 + porc2 * unorm;
          }
      } else if (ncomp == 2) {
        for (int j = jS; j <= jN; j++)
          for (int i = iW + 1; i <= iE; i++) {
            t = (F(u, i - 1, j + 1) + F(u, i, j + 1) + F(u, i - 1, j) + F(u, i, j)) / R(4.0);
            unorm = RSQRT(t * t + F(v, i, j) * F(v, i, j));
            unrm1 = R(0.0);
            if (unorm > R(1.0e-8)) unrm1 = (F(v, i, j) * F(v, i, j)) / unorm;
            if (njacob == 1) unorm = unrm1 + unorm;
            F(cp, i, j) = porc1 + porc2 * unorm;
          }
      } else {
        die("Error: Wrong ncomp flag passed to PorosCoef", ncomp, 0);
      }
    }
}

/* Porosity division of convective coefficients, momentum.f:296-324 (X) and
 * 621-649 (Y). */
static void FN(poros_scale)(w2o_ctx *c, const w2o_regions *r, MOMWS *w,
                        int yflag) {
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      if (RTYP(r, ireg, jreg) != RM_POROUS) continue;
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      REAL por = R(RPAR(dPRporos, r, ireg, jreg));
      int j0 = yflag ? jS : jS + 1, i0 = yflag ? iW + 1 : iW;
      for (int j = j0; j <= jN; j++)
        for (int i = i0; i <= iE; i++) {
          F(w->cj1, i, j) = F(w->cj1, i, j) / por;
          F(w->cj2, i, j) = F(w->cj2, i, j) / por;
          F(w->c1s, i, j) = F(w->c1s, i, j) / por;
          F(w->c2s, i, j) = F(w->c2s, i, j) / por;
          F(w->c1n, i, j) = F(w->c1n, i, j) / por;
          F(w->c2n, i, j) = F(w->c2n, i, j) / por;
        }
    }
}

#define CA(k, ind) w->a[((k)-1) + 3 * (size_t)((ind)-1)]
#define CB(ind) w->b[(ind)-1]

static void FN(set_identity_row)(MOMWS *w, int ind) {
  CA(1, ind) = R(0.0); CA(2, ind) = R(1.0); CA(3, ind) = R(0.0); CB(ind) = R(0.0);
}

/* XMomentum, momentum.f:199-514 */
static void FN(x_momentum)(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                       double dk, double re, const METRICS *m,
                       const REAL *us, const REAL *vs, const REAL *un,
                       const REAL *vn, REAL *dus) {
  MOMWS *w = &c->MOM_WX;
  int i, j, ind;
  REAL re1 = R(1.0) / R(re), dk2 = R(dk) * R(0.5), rkj;

  FN(conv_coef)(c, nx, ny, 4, 1, m->xzu, m->xeu, m->yzu, m->yeu, us, vs, w->cj1, w->cj2);
  FN(conv_coef)(c, nx, ny, 1, 0, m->xzn, m->xec, m->yzn, m->yec, us, vs, w->c1s, w->c2s);
  FN(conv_coef)(c, nx, ny, 1, 0, m->xzn, m->xec, m->yzn, m->yec, un, vn, w->c1n, w->c2n);
  FN(poros_scale)(c, r, w, 0);

  FN(dconv_u)(c, nx, ny, w->c1s, w->c2s, us, w->cnvs);
  FN(dconv_u)(c, nx, ny, w->c1n, w->c2n, un, w->cnvn);
  FN(ddiff_u)(c, nx, ny, m->rac, m->rbc, m->rbn, m->rgn, us, w->difs);
  FN(ddiff_u)(c, nx, ny, m->rac, m->rbc, m->rbn, m->rgn, un, w->difn);

  FN(poros_coef)(c, nx, ny, 1, 1, r, us, vs, w->cpj);
  FN(poros_coef)(c, nx, ny, 1, 0, r, us, vs, w->cps);
  FN(poros_coef)(c, nx, ny, 1, 0, r, un, vn, w->cpn);

  /* First split step, momentum.f:350-384 */
  for (j = 2; j <= ny; j++)
    for (i = 1; i <= nx; i++) {
      ind = (j - 2) * nx + i;
      rkj = dk2 * F(m->dju, i, j);
      if (F(w->cj1, i, j) >= R(0.0)) {
        CA(1, ind) = rkj * (-F(w->cj1, i - 1, j) - re1 * F(m->rac, i, j));
        CA(2, ind) = R(1.0) + rkj * (F(w->cj1, i, j) +
                                  re1 * (F(m->rac, i + 1, j) + F(m->rac, i, j))) +
                     dk2 * F(w->cpj, i, j);
        CA(3, ind) = rkj * (-re1 * F(m->rac, i + 1, j));
      } else {
        CA(1, ind) = rkj * (-re1 * F(m->rac, i, j));
        CA(2, ind) = R(1.0) + rkj * (-F(w->cj1, i, j) +
                                  re1 * (F(m->rac, i + 1, j) + F(m->rac, i, j))) +
                     dk2 * F(w->cpj, i, j);
        CA(3, ind) = rkj * (F(w->cj1, i + 1, j) - re1 * F(m->rac, i + 1, j));
      }
      CB(ind) = F(un, i, j) - F(us, i, j) +
                rkj * (-F(w->cnvs, i, j) - F(w->cnvn, i, j)) +
                rkj * re1 * (F(w->difs, i, j) + F(w->difn, i, j)) -
                dk2 * (F(w->cps, i, j) * F(us, i, j) + F(w->cpn, i, j) * F(un, i, j));
    }
  FN(w2o_alt_trid_lu)(nx * (ny - 1), w->a, w->b);

  /* Second split step, momentum.f:396-428 */
  for (j = 2; j <= ny; j++)
    for (i = 1; i <= nx; i++) {
      ind = (j - 2) * nx + i;
      rkj = dk2 * F(m->dju, i, j);
      if (F(w->cj2, i, j) >= R(0.0)) {
        CA(1, ind) = rkj * (-F(w->cj2, i, j - 1) - re1 * F(m->rgn, i, j - 1));
        CA(2, ind) = R(1.0) + rkj * (F(w->cj2, i, j) +
                                  re1 * (F(m->rgn, i, j) + F(m->rgn, i, j - 1))) +
                     dk2 * F(w->cpj, i, j);
        CA(3, ind) = rkj * (-re1 * F(m->rgn, i, j));
      } else {
        CA(1, ind) = rkj * (-re1 * F(m->rgn, i, j - 1));
        CA(2, ind) = R(1.0) + rkj * (-F(w->cj2, i, j) +
                                  re1 * (F(m->rgn, i, j) + F(m->rgn, i, j - 1))) +
                     dk2 * F(w->cpj, i, j);
        CA(3, ind) = rkj * (F(w->cj2, i, j + 1) - re1 * F(m->rgn, i, j));
      }
    }

  /* Blockage and W/E boundary identity rows, momentum.f:434-496 */
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      if (RTYP(r, ireg, jreg) == RM_BLOCKG)
        for (j = jS + 1; j <= jN; j++)
          for (i = iW; i <= iE; i++) FN(set_identity_row)(w, (j - 2) * nx + i);
      switch (MBTP(r, ireg, jreg, WEST)) {
        case BM_INTERN: case BM_OUTLT1: case BM_OUTLT2: break;
        case BM_WALL1: case BM_WALL2: case BM_INLET:
          for (j = jS + 1; j <= jN; j++) FN(set_identity_row)(w, (j - 2) * nx + iW);
          break;
        default: die("Wrong nBdTypeW flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, EAST)) {
        case BM_INTERN: case BM_OUTLT1: case BM_OUTLT2: break;
        case BM_WALL1: case BM_WALL2: case BM_INLET:
          for (j = jS + 1; j <= jN; j++) FN(set_identity_row)(w, (j - 2) * nx + iE);
          break;
        default: die("Wrong nBdTypeE flag", ireg, jreg);
      }
    }
  FN(w2o_alt_trid_lu)(nx * (ny - 1), w->a, w->b);

  for (j = 2; j <= ny; j++)
    for (i = 1; i <= nx; i++) F(dus, i, j) = CB((j - 2) * nx + i);
}

/* YMomentum, momentum.f:520-838 */
static void FN(y_momentum)(w2o_ctx *c, int nx, int ny, const w2o_regions *r,
                       double dk, double re, double fr, const METRICS *m,
                       const REAL *d, const REAL *dn, const REAL *us,
                       const REAL *vs, const REAL *un, const REAL *vn,
                       REAL *dvs) {
  MOMWS *w = &c->MOM_WY;
  int i, j, ind;
  REAL re1 = R(1.0) / R(re), dk2 = R(dk) * R(0.5), fr1 = R(1.0) / R(fr), rkj, buoy;
  (void)fr1;

  FN(conv_coef)(c, nx, ny, 5, 1, m->xzv, m->xev, m->yzv, m->yev, us, vs, w->cj1, w->cj2);
  FN(conv_coef)(c, nx, ny, 2, 0, m->xzc, m->xen, m->yzc, m->yen, us, vs, w->c1s, w->c2s);
  FN(conv_coef)(c, nx, ny, 2, 0, m->xzc, m->xen, m->yzc, m->yen, un, vn, w->c1n, w->c2n);
  FN(poros_scale)(c, r, w, 1);

  FN(dconv_v)(c, nx, ny, w->c1s, w->c2s, vs, w->cnvs);
  FN(dconv_v)(c, nx, ny, w->c1n, w->c2n, vn, w->cnvn);
  FN(ddiff_v)(c, nx, ny, m->ran, m->rbc, m->rbn, m->rgc, vs, w->difs);
  FN(ddiff_v)(c, nx, ny, m->ran, m->rbc, m->rbn, m->rgc, vn, w->difn);

  FN(poros_coef)(c, nx, ny, 2, 1, r, us, vs, w->cpj);
  FN(poros_coef)(c, nx, ny, 2, 0, r, us, vs, w->cps);
  FN(poros_coef)(c, nx, ny, 2, 0, r, un, vn, w->cpn);

  /* First split step, momentum.f:675-711 */
  for (j = 1; j <= ny; j++)
    for (i = 2; i <= nx; i++) {
      ind = (j - 1) * (nx - 1) + i - 1;
      rkj = dk2 * F(m->djv, i, j);
      if (F(w->cj1, i, j) >= R(0.0)) {
        CA(1, ind) = rkj * (-F(w->cj1, i - 1, j) - re1 * F(m->ran, i - 1, j));
        CA(2, ind) = rkj * (F(w->cj1, i, j) +
                            re1 * (F(m->ran, i, j) + F(m->ran, i - 1, j))) +
                     dk2 * F(w->cpj, i, j) + R(1.0);
        CA(3, ind) = rkj * (-re1 * F(m->ran, i, j));
      } else {
        CA(1, ind) = rkj * (-re1 * F(m->ran, i - 1, j));
        CA(2, ind) = rkj * (-F(w->cj1, i, j) +
                            re1 * (F(m->ran, i, j) + F(m->ran, i - 1, j))) +
                     dk2 * F(w->cpj, i, j) + R(1.0);
        CA(3, ind) = rkj * (F(w->cj1, i + 1, j) - re1 * F(m->ran, i, j));
      }
      buoy = R(dk) * (F(d, i, j + 1) + F(d, i, j) + F(dn, i, j + 1) + F(dn, i, j)) /
             (R(4.0) * R(fr));
      CB(ind) = F(vn, i, j) - F(vs, i, j) +
                rkj * (-F(w->cnvs, i, j) - F(w->cnvn, i, j)) +
                rkj * re1 * (F(w->difs, i, j) + F(w->difn, i, j)) -
                dk2 * (F(w->cps, i, j) * F(vs, i, j) + F(w->cpn, i, j) * F(vn, i, j)) -
                buoy;
    }
  FN(w2o_alt_trid_lu)((nx - 1) * ny, w->a, w->b);

  /* Second split step, momentum.f:723-754 */
  for (j = 1; j <= ny; j++)
    for (i = 2; i <= nx; i++) {
      ind = (j - 1) * (nx - 1) + i - 1;
      rkj = dk2 * F(m->djv, i, j);
      if (F(w->cj2, i, j) >= R(0.0)) {
        CA(1, ind) = rkj * (-F(w->cj2, i, j - 1) - re1 * F(m->rgc, i, j));
        CA(2, ind) = rkj * (F(w->cj2, i, j) +
                            re1 * (F(m->rgc, i, j + 1) + F(m->rgc, i, j))) +
                     dk2 * F(w->cpj, i, j) + R(1.0);
        CA(3, ind) = rkj * (-re1 * F(m->rgc, i, j + 1));
      } else {
        CA(1, ind) = rkj * (-re1 * F(m->rgc, i, j));
        CA(2, ind) = rkj * (-F(w->cj2, i, j) +
                            re1 * (F(m->rgc, i, j + 1) + F(m->rgc, i, j))) +
                     dk2 * F(w->cpj, i, j) + R(1.0);
        CA(3, ind) = rkj * (F(w->cj2, i, j + 1) - re1 * F(m->rgc, i, j + 1));
      }
    }

  /* Blockage and S/N boundary identity rows, momentum.f:760-821 */
  for (int jreg = 1; jreg <= r->nReg[1]; jreg++)
    for (int ireg = 1; ireg <= r->nReg[0]; ireg++) {
      int iW = RBRD(r, ireg, jreg, WEST), iE = RBRD(r, ireg, jreg, EAST);
      int jS = RBRD(r, ireg, jreg, SOUTH), jN = RBRD(r, ireg, jreg, NORTH);
      if (RTYP(r, ireg, jreg) == RM_BLOCKG)
        for (j = jS; j <= jN; j++)
          for (i = iW + 1; i <= iE; i++) FN(set_identity_row)(w, (j - 1) * (nx - 1) + i - 1);
      switch (MBTP(r, ireg, jreg, SOUTH)) {
        case BM_INTERN: case BM_OUTLT1: case BM_OUTLT2: break;
        case BM_WALL1: case BM_WALL2: case BM_INLET:
          for (i = iW + 1; i <= iE; i++) FN(set_identity_row)(w, (jS - 1) * (nx - 1) + i - 1);
          break;
        default: die("Wrong nBdTypeS flag", ireg, jreg);
      }
      switch (MBTP(r, ireg, jreg, NORTH)) {
        case BM_INTERN: case BM_OUTLT1: case BM_OUTLT2: break;
        case BM_WALL1: case BM_WALL2: case BM_INLET:
          for (i = iW + 1; i <= iE; i++) FN(set_identity_row)(w, (jN - 1) * (nx - 1) + i - 1);
          break;
        default: die("Wrong nBdTypeN flag", ireg, jreg);
      }
    }
  FN(w2o_alt_trid_lu)((nx - 1) * ny, w->a, w->b);

  for (j = 1; j <= ny; j++)
    for (i = 2; i <= nx; i++) F(dvs, i, j) = CB((j - 1) * (nx - 1) + i - 1);
}
#undef CA
#undef CB

/* DMaxNorm, utility.f:479-507 */
double FN(w2o_dmax_norm)(w2o_ctx *c, int nx, int ny, const REAL *u) {
  REAL diff = RABS(F(u, 5, 5));
  for (int j = 2; j <= ny - 1; j++)
    for (int i = 2; i <= nx - 1; i++) {
      REAL a = RABS(F(u, i, j));
      if (a > diff) diff = a;
    }
  return diff;
}

/* nAuxMomentum, momentum.f:33-193 */
int FN(w2o_naux_momentum)(w2o_ctx *c, int nx, int ny, int mqiter,
                      const w2o_regions *r, double dk, double re, double fr,
                      double qtol, const METRICS *m, const REAL *d,
                      const REAL *dn, const REAL *un, const REAL *vn,
                      REAL *us, REAL *vs) {
  int i, j, mm;
  for (j = 1; j <= ny + 1; j++)
    for (i = 1; i <= nx + 1; i++) {
      F(us, i, j) = F(un, i, j);
      F(vs, i, j) = F(vn, i, j);
    }
  for (mm = 1; mm <= mqiter; mm++) {
    FN(w2o_vel_outflow_bcs)(c, nx, ny, r, us, vs);
    for (j = 0; j <= ny + 1; j++)
      for (i = 0; i <= nx + 1; i++) {
        F(c->MOM_DUS, i, j) = R(0.0);
        F(c->MOM_DVS, i, j) = R(0.0);
      }
    FN(x_momentum)(c, nx, ny, r, dk, re, m, us, vs, un, vn, c->MOM_DUS);
    FN(y_momentum)(c, nx, ny, r, dk, re, fr, m, d, dn, us, vs, un, vn, c->MOM_DVS);
    for (j = 1; j <= ny; j++)
      for (i = 1; i <= nx; i++) {
        F(us, i, j) = F(us, i, j) + F(c->MOM_DUS, i, j);
        F(vs, i, j) = F(vs, i, j) + F(c->MOM_DVS, i, j);
      }
    REAL d1 = FN(w2o_dmax_norm)(c, nx, ny, c->MOM_DUS);
    REAL d2 = FN(w2o_dmax_norm)(c, nx, ny, c->MOM_DVS);
    REAL difmax = d2 > d1 ? d2 : d1;  /* max(dif(1),dif(2)): dif(1) unless dif(2) is larger */
    if (difmax <= qtol) return mm;
  }
  return -1;
}

