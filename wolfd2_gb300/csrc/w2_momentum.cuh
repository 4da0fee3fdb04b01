// w2_momentum.cuh -- nAuxMomentum (momentum.f:33-193) on the device.
//
// One Newton-Kantorovich (Q-L) iteration is four phases of a persistent
// kernel:
//   M1  convective face coefficients of ConvCoef (cases 4, 1 for x; 5, 2 for
//       y) from us/vs and un/vn, each value computed once;
//   M2  per row: DConv/DDiff stencils of the starred and time-level-n fields
//       and the split-1 and split-2 tridiagonal rows of XMomentum
//       (momentum.f:350-428) and YMomentum (momentum.f:675-754), written in
//       chain order, with the boundary/blockage identity rows of split 2;
//   C   the four chain solves (x and y chains together, split 1 then 2);
//   M4  us += dus, vs += dvs and the DMaxNorm test against qtol.
// Expressions keep the reference's operand order; the translation unit is
// compiled without FMA contraction, so every value is the IEEE-double value
// of the reference expression.  Non-porous regions contribute exact zeros
// (PorosCoef writes 0, so dk2*cpj adds +0 to a value >= 1 and the RHS terms
// vanish); porous decks are rejected on the host.
#pragma once
#include "w2_chain.cuh"
#include "w2_bc.cuh"

namespace w2 {

// ---- M1: ConvCoef outputs ---------------------------------------------
__device__ void mom_conv_coef(const Dev &d, const double *us, const double *vs,
                              const double *un, const double *vn) {
  const int nx = d.nx, ny = d.ny;
  const Metrics &m = d.m;
  const int W = nx + 2, H = ny + 2;
  for (int idx = gtid(); idx < W * H; idx += gthreads()) {
    const int i = idx % W, j = idx / W;
    const size_t o = IX(d, i, j);
    // XMomentum: ConvCoef(4, njacob=1) with xzu, xeu, yzu, yeu (momentum.f:942-950)
    if (i <= nx && j >= 1 && j <= ny) {
      const double vsum = vs[IX(d, i + 1, j)] + vs[o] + vs[IX(d, i + 1, j - 1)] + vs[IX(d, i, j - 1)];
      d.cj1x[o] = 2.0 * m.yeu[o] * us[o] - m.xeu[o] * vsum / 4.0;
      d.cj2x[o] = m.xzu[o] * vsum / 4.0 - 2.0 * m.yzu[o] * us[o];
    }
    // XMomentum: ConvCoef(1, njacob=0) with xzn, xec, yzn, yec (momentum.f:901-913)
    if (i >= 1 && j >= 1) {
      d.c1sx[o] = (m.yec[o] * (us[o] + us[IX(d, i - 1, j)]) - m.xec[o] * (vs[o] + vs[IX(d, i, j - 1)])) * 0.5;
      d.c1nx[o] = (m.yec[o] * (un[o] + un[IX(d, i - 1, j)]) - m.xec[o] * (vn[o] + vn[IX(d, i, j - 1)])) * 0.5;
      if (i <= nx && j <= ny) {
        d.c2sx[o] = (m.xzn[o] * (vs[IX(d, i + 1, j)] + vs[o]) - m.yzn[o] * (us[IX(d, i, j + 1)] + us[o])) * 0.5;
        d.c2nx[o] = (m.xzn[o] * (vn[IX(d, i + 1, j)] + vn[o]) - m.yzn[o] * (un[IX(d, i, j + 1)] + un[o])) * 0.5;
      }
    }
    // YMomentum: ConvCoef(5, njacob=1) with xzv, xev, yzv, yev (momentum.f:953-961)
    if (i >= 1 && i <= nx && j <= ny) {
      const double usum = us[IX(d, i, j + 1)] + us[IX(d, i - 1, j + 1)] + us[o] + us[IX(d, i - 1, j)];
      d.cj1y[o] = m.yev[o] * usum / 4.0 - 2.0 * m.xev[o] * vs[o];
      d.cj2y[o] = 2.0 * m.xzv[o] * vs[o] - m.yzv[o] * usum / 4.0;
    }
    // YMomentum: ConvCoef(2, njacob=0) with xzc, xen, yzc, yen (momentum.f:916-928)
    if (i >= 1 && j >= 1) {
      if (i <= nx && j <= ny) {
        d.c1sy[o] = (m.yen[o] * (us[IX(d, i, j + 1)] + us[o]) - m.xen[o] * (vs[IX(d, i + 1, j)] + vs[o])) * 0.5;
        d.c1ny[o] = (m.yen[o] * (un[IX(d, i, j + 1)] + un[o]) - m.xen[o] * (vn[IX(d, i + 1, j)] + vn[o])) * 0.5;
      }
      d.c2sy[o] = (m.xzc[o] * (vs[o] + vs[IX(d, i, j - 1)]) - m.yzc[o] * (us[o] + us[IX(d, i - 1, j)])) * 0.5;
      d.c2ny[o] = (m.xzc[o] * (vn[o] + vn[IX(d, i, j - 1)]) - m.yzc[o] * (un[o] + un[IX(d, i - 1, j)])) * 0.5;
    }
  }
}

// DConvU, momentum.f:1000-1006
__device__ __forceinline__ double dconv_u(const Dev &d, const double *c1, const double *c2,
                                          const double *u, int i, int j) {
  const size_t o = IX(d, i, j), os = IX(d, i, j - 1), oe = IX(d, i + 1, j);
  return -c2[os] * u[os] - c1[o] * u[IX(d, i - 1, j)] +
         (c1[oe] - c1[o] + c2[o] - c2[os]) * u[o] + c1[oe] * u[oe] + c2[o] * u[IX(d, i, j + 1)];
}

// DDiffU, momentum.f:1030-1042
__device__ __forceinline__ double ddiff_u(const Dev &d, const double *ac, const double *bc,
                                          const double *bn, const double *gn, const double *u,
                                          int i, int j) {
#define Uu(a, b) u[IX(d, a, b)]
  const double s1 = ac[IX(d, i + 1, j)] * (Uu(i + 1, j) - Uu(i, j)) -
                    ac[IX(d, i, j)] * (Uu(i, j) - Uu(i - 1, j)) +
                    bc[IX(d, i + 1, j)] * (Uu(i + 1, j + 1) + Uu(i, j + 1) - Uu(i + 1, j - 1) - Uu(i, j - 1)) -
                    bc[IX(d, i, j)] * (Uu(i, j + 1) + Uu(i - 1, j + 1) - Uu(i, j - 1) - Uu(i - 1, j - 1));
  const double s2 = bn[IX(d, i, j)] * (Uu(i + 1, j + 1) + Uu(i + 1, j) - Uu(i - 1, j + 1) - Uu(i - 1, j)) -
                    bn[IX(d, i, j - 1)] * (Uu(i + 1, j) + Uu(i + 1, j - 1) - Uu(i - 1, j) - Uu(i - 1, j - 1)) +
                    gn[IX(d, i, j)] * (Uu(i, j + 1) - Uu(i, j)) -
                    gn[IX(d, i, j - 1)] * (Uu(i, j) - Uu(i, j - 1));
#undef Uu
  return s1 + s2;
}

// DConvV, momentum.f:1064-1070
__device__ __forceinline__ double dconv_v(const Dev &d, const double *c1, const double *c2,
                                          const double *v, int i, int j) {
  const size_t o = IX(d, i, j), ow = IX(d, i - 1, j), on = IX(d, i, j + 1);
  return -c2[o] * v[IX(d, i, j - 1)] - c1[ow] * v[ow] + (c1[o] - c1[ow] + c2[on] - c2[o]) * v[o] +
         c1[o] * v[IX(d, i + 1, j)] + c2[on] * v[on];
}

// DDiffV, momentum.f:1094-1106
__device__ __forceinline__ double ddiff_v(const Dev &d, const double *an, const double *bc,
                                          const double *bn, const double *gc, const double *v,
                                          int i, int j) {
#define Vv(a, b) v[IX(d, a, b)]
  const double s1 = an[IX(d, i, j)] * (Vv(i + 1, j) - Vv(i, j)) -
                    an[IX(d, i - 1, j)] * (Vv(i, j) - Vv(i - 1, j)) +
                    bn[IX(d, i, j)] * (Vv(i + 1, j + 1) + Vv(i, j + 1) - Vv(i + 1, j - 1) - Vv(i, j - 1)) -
                    bn[IX(d, i - 1, j)] * (Vv(i, j + 1) + Vv(i - 1, j + 1) - Vv(i, j - 1) - Vv(i - 1, j - 1));
  const double s2 = bc[IX(d, i, j + 1)] * (Vv(i + 1, j + 1) + Vv(i + 1, j) - Vv(i - 1, j + 1) - Vv(i - 1, j)) -
                    bc[IX(d, i, j)] * (Vv(i + 1, j) + Vv(i + 1, j - 1) - Vv(i - 1, j) - Vv(i - 1, j - 1)) +
                    gc[IX(d, i, j + 1)] * (Vv(i, j + 1) - Vv(i, j)) -
                    gc[IX(d, i, j)] * (Vv(i, j) - Vv(i, j - 1));
#undef Vv
  return s1 + s2;
}

// ---- M2: stencils and tridiagonal rows --------------------------------
__device__ void mom_assemble(const Dev &d, double dk, double re, const double *us,
                             const double *vs, const double *un, const double *vn) {
  const int nx = d.nx, ny = d.ny;
  const Metrics &m = d.m;
  const double re1 = 1.0 / re, dk2 = dk * 0.5;
  // X rows: i = 1..nx, j = 2..ny, ind = (j-2)*nx + i-1
  const int nX = nx * (ny - 1);
  const int nY = (nx - 1) * ny;
  for (int t = gtid(); t < nX + nY; t += gthreads()) {
    if (t < nX) {
      const int i = t % nx + 1, j = t / nx + 2;
      const size_t o = IX(d, i, j);
      const double rkj = dk2 * m.dju[o];
      const double cnvs = dconv_u(d, d.c1sx, d.c2sx, us, i, j);
      const double cnvn = dconv_u(d, d.c1nx, d.c2nx, un, i, j);
      const double difs = ddiff_u(d, m.rac, m.rbc, m.rbn, m.rgn, us, i, j);
      const double difn = ddiff_u(d, m.rac, m.rbc, m.rbn, m.rgn, un, i, j);
      const double cj1 = d.cj1x[o], racp = m.rac[IX(d, i + 1, j)], rac0 = m.rac[o];
      double a1, a2, a3;
      if (cj1 >= 0.0) {
        a1 = rkj * (-d.cj1x[IX(d, i - 1, j)] - re1 * rac0);
        a2 = 1.0 + rkj * (cj1 + re1 * (racp + rac0));
        a3 = rkj * (-re1 * racp);
      } else {
        a1 = rkj * (-re1 * rac0);
        a2 = 1.0 + rkj * (-cj1 + re1 * (racp + rac0));
        a3 = rkj * (d.cj1x[IX(d, i + 1, j)] - re1 * racp);
      }
      d.x1.a1[t] = a1;
      d.x1.a2[t] = a2;
      d.x1.a3[t] = a3;
      d.x1.b[t] =
          un[o] - us[o] + rkj * (-cnvs - cnvn) + rkj * re1 * (difs + difn);
      // split 2 (momentum.f:396-428) with identity rows (momentum.f:432-496)
      if (d.mask[o] & MK_XID) {
        a1 = 0.0; a2 = 1.0; a3 = 0.0;
      } else {
        const double cj2 = d.cj2x[o], rgn0 = m.rgn[o], rgns = m.rgn[IX(d, i, j - 1)];
        if (cj2 >= 0.0) {
          a1 = rkj * (-d.cj2x[IX(d, i, j - 1)] - re1 * rgns);
          a2 = 1.0 + rkj * (cj2 + re1 * (rgn0 + rgns));
          a3 = rkj * (-re1 * rgn0);
        } else {
          a1 = rkj * (-re1 * rgns);
          a2 = 1.0 + rkj * (-cj2 + re1 * (rgn0 + rgns));
          a3 = rkj * (d.cj2x[IX(d, i, j + 1)] - re1 * rgn0);
        }
      }
      d.x2.a1[t] = a1;
      d.x2.a2[t] = a2;
      d.x2.a3[t] = a3;
    } else {
      // Y rows: i = 2..nx, j = 1..ny, ind = (j-1)*(nx-1) + i-2
      const int q = t - nX;
      const int i = q % (nx - 1) + 2, j = q / (nx - 1) + 1;
      const size_t o = IX(d, i, j);
      const double rkj = dk2 * m.djv[o];
      const double cnvs = dconv_v(d, d.c1sy, d.c2sy, vs, i, j);
      const double cnvn = dconv_v(d, d.c1ny, d.c2ny, vn, i, j);
      const double difs = ddiff_v(d, m.ran, m.rbc, m.rbn, m.rgc, vs, i, j);
      const double difn = ddiff_v(d, m.ran, m.rbc, m.rbn, m.rgc, vn, i, j);
      const double cj1 = d.cj1y[o], ran0 = m.ran[o], ranw = m.ran[IX(d, i - 1, j)];
      double a1, a2, a3;
      if (cj1 >= 0.0) {
        a1 = rkj * (-d.cj1y[IX(d, i - 1, j)] - re1 * ranw);
        a2 = rkj * (cj1 + re1 * (ran0 + ranw)) + 1.0;
        a3 = rkj * (-re1 * ran0);
      } else {
        a1 = rkj * (-re1 * ranw);
        a2 = rkj * (-cj1 + re1 * (ran0 + ranw)) + 1.0;
        a3 = rkj * (d.cj1y[IX(d, i + 1, j)] - re1 * ran0);
      }
      d.y1.a1[q] = a1;
      d.y1.a2[q] = a2;
      d.y1.a3[q] = a3;
      d.y1.b[q] =
          vn[o] - vs[o] + rkj * (-cnvs - cnvn) + rkj * re1 * (difs + difn);
      if (d.mask[o] & MK_YID) {
        a1 = 0.0; a2 = 1.0; a3 = 0.0;
      } else {
        const double cj2 = d.cj2y[o], rgc0 = m.rgc[o], rgcn = m.rgc[IX(d, i, j + 1)];
        if (cj2 >= 0.0) {
          a1 = rkj * (-d.cj2y[IX(d, i, j - 1)] - re1 * rgc0);
          a2 = rkj * (cj2 + re1 * (rgcn + rgc0)) + 1.0;
          a3 = rkj * (-re1 * rgcn);
        } else {
          a1 = rkj * (-re1 * rgc0);
          a2 = rkj * (-cj2 + re1 * (rgcn + rgc0)) + 1.0;
          a3 = rkj * (d.cj2y[IX(d, i, j + 1)] - re1 * rgcn);
        }
      }
      d.y2.a1[q] = a1;
      d.y2.a2[q] = a2;
      d.y2.a3[q] = a3;
    }
  }
}

// ---- M4: update and DMaxNorm (momentum.f:171-188, utility.f:479-507) --
__device__ void mom_update(const Dev &d, double *us, double *vs, unsigned long long *slot) {
  const int nx = d.nx, ny = d.ny;
  double mx = 0.0;
  for (int t = gtid(); t < nx * ny; t += gthreads()) {
    const int i = t % nx + 1, j = t / nx + 1;
    const size_t o = IX(d, i, j);
    const double du = (j >= 2) ? d.x2.x[(j - 2) * nx + i - 1] : 0.0;
    const double dv = (i >= 2) ? d.y2.x[(j - 1) * (nx - 1) + i - 2] : 0.0;
    us[o] = us[o] + du;
    vs[o] = vs[o] + dv;
    const bool in = (i >= 2 && i <= nx - 1 && j >= 2 && j <= ny - 1) || (i == 5 && j == 5);
    if (in) mx = dmax(dmax(mx, fabs(du)), fabs(dv));
  }
  block_max_to(slot, mx);
}

// The whole nAuxMomentum.  Returns nQLiter (or -1) in *out; false on error.
__device__ bool naux_momentum(const Dev &d, int mqiter, double dk, double re, double qtol,
                              const double *un, const double *vn, double *us, double *vs,
                              int *out) {
  Sync *sy = d.sync;
  int result = -1;
  for (int it = 1; it <= mqiter; ++it) {
    if (d.has_outflow) {
      if (blockIdx.x == 0 && !vel_outflow_bcs_block(d, us, vs) && threadIdx.x == 0)
        set_error(sy, W2_E_BCFLAG);
      if (!grid_sync(sy)) return false;
    }
    mom_conv_coef(d, us, vs, un, vn);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (it == 1) sy->red[1] = 0ull;
      sy->red[(it + 1) % 3] = 0ull;
    }
    if (!grid_sync(sy)) return false;
    mom_assemble(d, dk, re, us, vs, un, vn);
    if (!grid_sync(sy)) return false;
    if (!solve_chains(d, d.x1, d.y1, 2)) return false;
    if (!solve_chains(d, d.x2, d.y2, 2)) return false;
    mom_update(d, us, vs, &sy->red[it % 3]);
    if (!grid_sync(sy)) return false;
    const double difmax = slot_value(&sy->red[it % 3]);
    if (difmax <= qtol) {
      result = it;
      break;
    }
  }
  *out = result;
  return true;
}

}  // namespace w2
