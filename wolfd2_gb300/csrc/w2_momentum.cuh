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
// compiled without FMA contraction, so every value is the IEEE value of the
// reference expression in the arithmetic type T: double on the plain path,
// float (single-precision fields, metrics and chains) on the mixed one.  Non-porous regions contribute exact zeros
// (PorosCoef writes 0, so dk2*cpj adds +0 to a value >= 1 and the RHS terms
// vanish); porous decks are rejected on the host.
#pragma once
#include "w2_chain.cuh"
#include "w2_bc.cuh"

namespace w2 {

template <class T>
__device__ __forceinline__ T tmax(T a, T b) { return b > a ? b : a; }

// The FP64 view of the momentum inputs and work arrays held by Dev.
__device__ __forceinline__ MomView<double> mom_view64(const Dev &d) {
  const Metrics &m = d.m;
  MomView<double> v;
  v.yeu = m.yeu; v.xeu = m.xeu; v.xzu = m.xzu; v.yzu = m.yzu;
  v.yec = m.yec; v.xec = m.xec; v.xzn = m.xzn; v.yzn = m.yzn;
  v.yev = m.yev; v.xev = m.xev; v.xzv = m.xzv; v.yzv = m.yzv;
  v.yen = m.yen; v.xen = m.xen; v.xzc = m.xzc; v.yzc = m.yzc;
  v.dju = m.dju; v.djv = m.djv; v.rac = m.rac; v.rbc = m.rbc;
  v.rbn = m.rbn; v.rgn = m.rgn; v.ran = m.ran; v.rgc = m.rgc;
  v.cj1x = d.cj1x; v.cj2x = d.cj2x; v.c1sx = d.c1sx; v.c2sx = d.c2sx; v.c1nx = d.c1nx; v.c2nx = d.c2nx;
  v.cj1y = d.cj1y; v.cj2y = d.cj2y; v.c1sy = d.c1sy; v.c2sy = d.c2sy; v.c1ny = d.c1ny; v.c2ny = d.c2ny;
  v.x1 = d.x1; v.x2 = d.x2; v.y1 = d.y1; v.y2 = d.y2;
  return v;
}

// ---- M1: ConvCoef outputs ---------------------------------------------
template <class T>
__device__ void mom_conv_coef(const Dev &d, const MomView<T> &V, const T *us, const T *vs,
                              const T *un, const T *vn) {
  const int nx = d.nx, ny = d.ny;
    const int W = nx + 2, H = ny + 2;
  for (int idx = gtid(); idx < W * H; idx += gthreads()) {
    const int i = idx % W, j = idx / W;
    const size_t o = IX(d, i, j);
    // XMomentum: ConvCoef(4, njacob=1) with xzu, xeu, yzu, yeu (momentum.f:942-950)
    if (i <= nx && j >= 1 && j <= ny) {
      const T vsum = vs[IX(d, i + 1, j)] + vs[o] + vs[IX(d, i + 1, j - 1)] + vs[IX(d, i, j - 1)];
      V.cj1x[o] = T(2.0) * V.yeu[o] * us[o] - V.xeu[o] * vsum / T(4.0);
      V.cj2x[o] = V.xzu[o] * vsum / T(4.0) - T(2.0) * V.yzu[o] * us[o];
    }
    // XMomentum: ConvCoef(1, njacob=0) with xzn, xec, yzn, yec (momentum.f:901-913)
    if (i >= 1 && j >= 1) {
      V.c1sx[o] = (V.yec[o] * (us[o] + us[IX(d, i - 1, j)]) - V.xec[o] * (vs[o] + vs[IX(d, i, j - 1)])) * T(0.5);
      V.c1nx[o] = (V.yec[o] * (un[o] + un[IX(d, i - 1, j)]) - V.xec[o] * (vn[o] + vn[IX(d, i, j - 1)])) * T(0.5);
      if (i <= nx && j <= ny) {
        V.c2sx[o] = (V.xzn[o] * (vs[IX(d, i + 1, j)] + vs[o]) - V.yzn[o] * (us[IX(d, i, j + 1)] + us[o])) * T(0.5);
        V.c2nx[o] = (V.xzn[o] * (vn[IX(d, i + 1, j)] + vn[o]) - V.yzn[o] * (un[IX(d, i, j + 1)] + un[o])) * T(0.5);
      }
    }
    // YMomentum: ConvCoef(5, njacob=1) with xzv, xev, yzv, yev (momentum.f:953-961)
    if (i >= 1 && i <= nx && j <= ny) {
      const T usum = us[IX(d, i, j + 1)] + us[IX(d, i - 1, j + 1)] + us[o] + us[IX(d, i - 1, j)];
      V.cj1y[o] = V.yev[o] * usum / T(4.0) - T(2.0) * V.xev[o] * vs[o];
      V.cj2y[o] = T(2.0) * V.xzv[o] * vs[o] - V.yzv[o] * usum / T(4.0);
    }
    // YMomentum: ConvCoef(2, njacob=0) with xzc, xen, yzc, yen (momentum.f:916-928)
    if (i >= 1 && j >= 1) {
      if (i <= nx && j <= ny) {
        V.c1sy[o] = (V.yen[o] * (us[IX(d, i, j + 1)] + us[o]) - V.xen[o] * (vs[IX(d, i + 1, j)] + vs[o])) * T(0.5);
        V.c1ny[o] = (V.yen[o] * (un[IX(d, i, j + 1)] + un[o]) - V.xen[o] * (vn[IX(d, i + 1, j)] + vn[o])) * T(0.5);
      }
      V.c2sy[o] = (V.xzc[o] * (vs[o] + vs[IX(d, i, j - 1)]) - V.yzc[o] * (us[o] + us[IX(d, i - 1, j)])) * T(0.5);
      V.c2ny[o] = (V.xzc[o] * (vn[o] + vn[IX(d, i, j - 1)]) - V.yzc[o] * (un[o] + un[IX(d, i - 1, j)])) * T(0.5);
    }
  }
}

// DConvU, momentum.f:1000-1006
template <class T>
__device__ __forceinline__ T dconv_u(const Dev &d, const T *c1, const T *c2,
                                          const T *u, int i, int j) {
  const size_t o = IX(d, i, j), os = IX(d, i, j - 1), oe = IX(d, i + 1, j);
  return -c2[os] * u[os] - c1[o] * u[IX(d, i - 1, j)] +
         (c1[oe] - c1[o] + c2[o] - c2[os]) * u[o] + c1[oe] * u[oe] + c2[o] * u[IX(d, i, j + 1)];
}

// DDiffU, momentum.f:1030-1042
template <class T>
__device__ __forceinline__ T ddiff_u(const Dev &d, const T *ac, const T *bc,
                                          const T *bn, const T *gn, const T *u,
                                          int i, int j) {
#define Uu(a, b) u[IX(d, a, b)]
  const T s1 = ac[IX(d, i + 1, j)] * (Uu(i + 1, j) - Uu(i, j)) -
                    ac[IX(d, i, j)] * (Uu(i, j) - Uu(i - 1, j)) +
                    bc[IX(d, i + 1, j)] * (Uu(i + 1, j + 1) + Uu(i, j + 1) - Uu(i + 1, j - 1) - Uu(i, j - 1)) -
                    bc[IX(d, i, j)] * (Uu(i, j + 1) + Uu(i - 1, j + 1) - Uu(i, j - 1) - Uu(i - 1, j - 1));
  const T s2 = bn[IX(d, i, j)] * (Uu(i + 1, j + 1) + Uu(i + 1, j) - Uu(i - 1, j + 1) - Uu(i - 1, j)) -
                    bn[IX(d, i, j - 1)] * (Uu(i + 1, j) + Uu(i + 1, j - 1) - Uu(i - 1, j) - Uu(i - 1, j - 1)) +
                    gn[IX(d, i, j)] * (Uu(i, j + 1) - Uu(i, j)) -
                    gn[IX(d, i, j - 1)] * (Uu(i, j) - Uu(i, j - 1));
#undef Uu
  return s1 + s2;
}

// DConvV, momentum.f:1064-1070
template <class T>
__device__ __forceinline__ T dconv_v(const Dev &d, const T *c1, const T *c2,
                                          const T *v, int i, int j) {
  const size_t o = IX(d, i, j), ow = IX(d, i - 1, j), on = IX(d, i, j + 1);
  return -c2[o] * v[IX(d, i, j - 1)] - c1[ow] * v[ow] + (c1[o] - c1[ow] + c2[on] - c2[o]) * v[o] +
         c1[o] * v[IX(d, i + 1, j)] + c2[on] * v[on];
}

// DDiffV, momentum.f:1094-1106
template <class T>
__device__ __forceinline__ T ddiff_v(const Dev &d, const T *an, const T *bc,
                                          const T *bn, const T *gc, const T *v,
                                          int i, int j) {
#define Vv(a, b) v[IX(d, a, b)]
  const T s1 = an[IX(d, i, j)] * (Vv(i + 1, j) - Vv(i, j)) -
                    an[IX(d, i - 1, j)] * (Vv(i, j) - Vv(i - 1, j)) +
                    bn[IX(d, i, j)] * (Vv(i + 1, j + 1) + Vv(i, j + 1) - Vv(i + 1, j - 1) - Vv(i, j - 1)) -
                    bn[IX(d, i - 1, j)] * (Vv(i, j + 1) + Vv(i - 1, j + 1) - Vv(i, j - 1) - Vv(i - 1, j - 1));
  const T s2 = bc[IX(d, i, j + 1)] * (Vv(i + 1, j + 1) + Vv(i + 1, j) - Vv(i - 1, j + 1) - Vv(i - 1, j)) -
                    bc[IX(d, i, j)] * (Vv(i + 1, j) + Vv(i + 1, j - 1) - Vv(i - 1, j) - Vv(i - 1, j - 1)) +
                    gc[IX(d, i, j + 1)] * (Vv(i, j + 1) - Vv(i, j)) -
                    gc[IX(d, i, j)] * (Vv(i, j) - Vv(i, j - 1));
#undef Vv
  return s1 + s2;
}

// ---- M2: stencils and tridiagonal rows --------------------------------
template <class T>
__device__ void mom_assemble(const Dev &d, const MomView<T> &V, double dk, double re, const T *us,
                             const T *vs, const T *un, const T *vn) {
  const int nx = d.nx, ny = d.ny;
    const T re1 = T(1.0) / T(re), dk2 = T(dk) * T(0.5);
  // X rows: i = 1..nx, j = 2..ny, ind = (j-2)*nx + i-1
  const int nX = nx * (ny - 1);
  const int nY = (nx - 1) * ny;
  for (int t = gtid(); t < nX + nY; t += gthreads()) {
    if (t < nX) {
      const int i = t % nx + 1, j = t / nx + 2;
      const size_t o = IX(d, i, j);
      const T rkj = dk2 * V.dju[o];
      const T cnvs = dconv_u(d, V.c1sx, V.c2sx, us, i, j);
      const T cnvn = dconv_u(d, V.c1nx, V.c2nx, un, i, j);
      const T difs = ddiff_u(d, V.rac, V.rbc, V.rbn, V.rgn, us, i, j);
      const T difn = ddiff_u(d, V.rac, V.rbc, V.rbn, V.rgn, un, i, j);
      const T cj1 = V.cj1x[o], racp = V.rac[IX(d, i + 1, j)], rac0 = V.rac[o];
      T a1, a2, a3;
      if (cj1 >= T(0.0)) {
        a1 = rkj * (-V.cj1x[IX(d, i - 1, j)] - re1 * rac0);
        a2 = T(1.0) + rkj * (cj1 + re1 * (racp + rac0));
        a3 = rkj * (-re1 * racp);
      } else {
        a1 = rkj * (-re1 * rac0);
        a2 = T(1.0) + rkj * (-cj1 + re1 * (racp + rac0));
        a3 = rkj * (V.cj1x[IX(d, i + 1, j)] - re1 * racp);
      }
      V.x1.a1[t] = a1;
      V.x1.a2[t] = a2;
      V.x1.a3[t] = a3;
      V.x1.b[t] =
          un[o] - us[o] + rkj * (-cnvs - cnvn) + rkj * re1 * (difs + difn);
      // split 2 (momentum.f:396-428) with identity rows (momentum.f:432-496)
      if (d.mask[o] & MK_XID) {
        a1 = T(0.0); a2 = T(1.0); a3 = T(0.0);
      } else {
        const T cj2 = V.cj2x[o], rgn0 = V.rgn[o], rgns = V.rgn[IX(d, i, j - 1)];
        if (cj2 >= T(0.0)) {
          a1 = rkj * (-V.cj2x[IX(d, i, j - 1)] - re1 * rgns);
          a2 = T(1.0) + rkj * (cj2 + re1 * (rgn0 + rgns));
          a3 = rkj * (-re1 * rgn0);
        } else {
          a1 = rkj * (-re1 * rgns);
          a2 = T(1.0) + rkj * (-cj2 + re1 * (rgn0 + rgns));
          a3 = rkj * (V.cj2x[IX(d, i, j + 1)] - re1 * rgn0);
        }
      }
      V.x2.a1[t] = a1;
      V.x2.a2[t] = a2;
      V.x2.a3[t] = a3;
    } else {
      // Y rows: i = 2..nx, j = 1..ny, ind = (j-1)*(nx-1) + i-2
      const int q = t - nX;
      const int i = q % (nx - 1) + 2, j = q / (nx - 1) + 1;
      const size_t o = IX(d, i, j);
      const T rkj = dk2 * V.djv[o];
      const T cnvs = dconv_v(d, V.c1sy, V.c2sy, vs, i, j);
      const T cnvn = dconv_v(d, V.c1ny, V.c2ny, vn, i, j);
      const T difs = ddiff_v(d, V.ran, V.rbc, V.rbn, V.rgc, vs, i, j);
      const T difn = ddiff_v(d, V.ran, V.rbc, V.rbn, V.rgc, vn, i, j);
      const T cj1 = V.cj1y[o], ran0 = V.ran[o], ranw = V.ran[IX(d, i - 1, j)];
      T a1, a2, a3;
      if (cj1 >= T(0.0)) {
        a1 = rkj * (-V.cj1y[IX(d, i - 1, j)] - re1 * ranw);
        a2 = rkj * (cj1 + re1 * (ran0 + ranw)) + T(1.0);
        a3 = rkj * (-re1 * ran0);
      } else {
        a1 = rkj * (-re1 * ranw);
        a2 = rkj * (-cj1 + re1 * (ran0 + ranw)) + T(1.0);
        a3 = rkj * (V.cj1y[IX(d, i + 1, j)] - re1 * ran0);
      }
      V.y1.a1[q] = a1;
      V.y1.a2[q] = a2;
      V.y1.a3[q] = a3;
      V.y1.b[q] =
          vn[o] - vs[o] + rkj * (-cnvs - cnvn) + rkj * re1 * (difs + difn);
      if (d.mask[o] & MK_YID) {
        a1 = T(0.0); a2 = T(1.0); a3 = T(0.0);
      } else {
        const T cj2 = V.cj2y[o], rgc0 = V.rgc[o], rgcn = V.rgc[IX(d, i, j + 1)];
        if (cj2 >= T(0.0)) {
          a1 = rkj * (-V.cj2y[IX(d, i, j - 1)] - re1 * rgc0);
          a2 = rkj * (cj2 + re1 * (rgcn + rgc0)) + T(1.0);
          a3 = rkj * (-re1 * rgcn);
        } else {
          a1 = rkj * (-re1 * rgc0);
          a2 = rkj * (-cj2 + re1 * (rgcn + rgc0)) + T(1.0);
          a3 = rkj * (V.cj2y[IX(d, i, j + 1)] - re1 * rgcn);
        }
      }
      V.y2.a1[q] = a1;
      V.y2.a2[q] = a2;
      V.y2.a3[q] = a3;
    }
  }
}

// ---- M4: update and DMaxNorm (momentum.f:171-188, utility.f:479-507) --
template <class T>
__device__ void mom_update(const Dev &d, const MomView<T> &V, T *us, T *vs, unsigned long long *slot) {
  const int nx = d.nx, ny = d.ny;
  T mx = T(0.0);
  for (int t = gtid(); t < nx * ny; t += gthreads()) {
    const int i = t % nx + 1, j = t / nx + 1;
    const size_t o = IX(d, i, j);
    const T du = (j >= 2) ? V.x2.x[(j - 2) * nx + i - 1] : T(0.0);
    const T dv = (i >= 2) ? V.y2.x[(j - 1) * (nx - 1) + i - 2] : T(0.0);
    us[o] = us[o] + du;
    vs[o] = vs[o] + dv;
    const bool in = (i >= 2 && i <= nx - 1 && j >= 2 && j <= ny - 1) || (i == 5 && j == 5);
    if (in) mx = tmax(tmax(mx, fabs(du)), fabs(dv));
  }
  block_max_to(slot, mx);
}

// The whole nAuxMomentum.  Returns nQLiter (or -1) in *out; false on error.
template <class T>
__device__ bool naux_momentum(const Dev &d, const MomView<T> &V, int mqiter, double dk, double re, double qtol,
                              const T *un, const T *vn, T *us, T *vs,
                              int *out) {
  Sync *sy = d.sync;
  int result = -1;
  for (int it = 1; it <= mqiter; ++it) {
    if (d.has_outflow) {
      if (blockIdx.x == 0 && !vel_outflow_bcs_block(d, us, vs) && threadIdx.x == 0)
        set_error(sy, W2_E_BCFLAG);
      if (!grid_sync(sy)) return false;
    }
    mom_conv_coef(d, V, us, vs, un, vn);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (it == 1) sy->red[1] = 0ull;
      sy->red[(it + 1) % 3] = 0ull;
    }
    if (!grid_sync(sy)) return false;
    mom_assemble(d, V, dk, re, us, vs, un, vn);
    if (!grid_sync(sy)) return false;
    if (!solve_chains(d, V.x1, V.y1, 2)) return false;
    if (!solve_chains(d, V.x2, V.y2, 2)) return false;
    mom_update(d, V, us, vs, &sy->red[it % 3]);
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
