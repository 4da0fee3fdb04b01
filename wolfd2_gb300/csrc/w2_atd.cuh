// w2_atd.cuh -- the small-scale model of Additive Turbulent Decomposition on
// the device: SmallScale (small_scale.f:31-578) and SmlSclBC
// (bound_cond.f:1211-1500).
//
// SmallScale forms cell-centred large-scale fields, their Shuman-filtered
// high-pass parts, and in every cell above the Peclet threshold advances
// nine logistic maps (three per variable) up to 50 times; the map values,
// projected on the directions of the high-pass gradients, give the small
// scales uss, vss, tss.  It then projects (uss, vss) with its own Ppe and
// Project.  The routine keeps every local between calls (a bare SAVE): the
// map iterates and cell areas carry from call to call, and its work arrays
// keep whatever their never-written entries hold (zero).  AtdState is that
// saved state, in device memory.
//
// Arithmetic is the reference's operand order in FP64 with no contraction.
// pow, tanh and atanh are CUDA's, which differ from the host libm's by an
// ulp or so; the chaotic maps amplify such differences, so results match
// the oracle to a tolerance that grows with the number of map iterations.
#pragma once
#include "w2_thermal.cuh"

namespace w2 {

struct AtdParams {
  double dlref, uref, tref, tmax, dka, re, pe;
  double fpu, fpv, fpt;
  double cu0, tscoef, hscoef, temcoef, bnumc, rmax, rlc;
};

struct AtdState {
  double *map[9];     // umap(.,.,1..3), vmap(.,.,1..3), tmap(.,.,1..3)
  double *area, *tarea;
  double *xz, *xe, *yz, *ye, *rj, *ul, *vl, *tl, *uc, *vc, *uf, *vf, *tf, *ff;
};

// One step of the logistic map x <- r A x (1 - B |x|) of small_scale.f.
__device__ __forceinline__ double atd_map(double rm, double x) {
  const double A = 4.82842712474, B = 1.47839783948;
  return rm * A * x * (1.0 - B * fabs(x));
}

// Dimensional metrics, cell-centred large-scale fields and contravariant
// velocity on i, j = 1..n (small_scale.f:246-276); tf = tl, to be filtered.
__global__ void k_atd_prep(Dev d, AtdState S, AtdParams P, const double *u1, const double *v1,
                           const double *t1) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny;
  const Metrics &m = d.m;
  const double dl = P.dlref;
  for (int t = gtid(); t < nx * ny; t += gthreads()) {
    const int i = t % nx + 1, j = t / nx + 1;
    const size_t o = IX(d, i, j);
    S.xz[o] = dl * m.xzc[o];
    S.xe[o] = dl * m.xec[o];
    S.yz[o] = dl * m.yzc[o];
    S.ye[o] = dl * m.yec[o];
    S.rj[o] = m.djc[o] / (dl * dl);
    S.vl[o] = P.uref * (v1[o] + v1[IX(d, i, j - 1)]) * 0.5;
    S.ul[o] = P.uref * (u1[o] + u1[IX(d, i - 1, j)]) * 0.5;
    S.tl[o] = (P.tmax - P.tref) * t1[o] + P.tref;
    S.uc[o] = S.ye[o] * S.ul[o] - S.xe[o] * S.vl[o];
    S.vc[o] = S.xz[o] * S.vl[o] - S.yz[o] * S.ul[o];
    S.tf[o] = S.tl[o];
  }
}

// High-pass part: the field minus its filtered copy, on i, j = 1..n; `hp`
// receives it, `a` is the field, `f` the filtered copy.
__global__ void k_atd_highpass(Dev d, const double *a, const double *f, double *hp) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < nx * ny; t += gthreads()) {
    const size_t o = IX(d, t % nx + 1, t / nx + 1);
    hp[o] = a[o] - f[o];
  }
}

// The small scales of one cell (small_scale.f:309-520).
__device__ void atd_cell(const Dev &d, const AtdState &S, const AtdParams &P, int i, int j, double *uss,
                         double *vss, double *tss) {
  const double rc = 0.20710678119;
  const double third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  const double piosr2 = acos(-1.0) / sqrt(2.0);
  const double hs = P.dlref * P.hscoef, dk = P.dka * P.dlref / P.uref;
  const double pr = P.pe / P.re, rnu = P.uref * P.dlref / P.re, dkappa = rnu / pr;
  const size_t o = IX(d, i, j), oe = IX(d, i + 1, j), ow = IX(d, i - 1, j), on = IX(d, i, j + 1),
               os = IX(d, i, j - 1);
#define CD_I(a) ((a[oe] - a[ow]) * 0.5)
#define CD_J(a) ((a[on] - a[os]) * 0.5)
  const double xz = S.xz[o], xe = S.xe[o], yz = S.yz[o], ye = S.ye[o], rj = S.rj[o];
  const double hxy = sqrt(xz * xz + yz * yz + xe * xe + ye * ye);
  double uz = CD_I(S.ul), ue = CD_J(S.ul), vz = CD_I(S.vl), ve = CD_J(S.vl);
  double q1 = rj * (ye * uz - yz * ue), q2 = rj * (xz * ue - xe * uz);
  double q3 = rj * (ye * vz - yz * ve), q4 = rj * (xz * ve - xe * vz);
  const double delu2n = sqrt(q1 * q1 + q2 * q2 + q3 * q3 + q4 * q4);
  double tz = CD_I(S.tl), te = CD_J(S.tl);
  q1 = rj * (ye * tz - yz * te);
  q2 = rj * (xz * te - xe * tz);
  const double delt2n = sqrt(q1 * q1 + q2 * q2);
  const double reh = delu2n * (hxy * hxy) / rnu, peh = pr * reh;
  if (!(peh > 3.0)) return;
  const double cuV = P.cu0, cuT = P.cu0;
  int nmap = 0;
  if (P.cu0 > (double)1.0e-10f) {
    const double ts = P.tscoef * piosr2 * pow(reh, third) / (P.cu0 * delu2n);
    nmap = (int)(1.0 + dk / ts);
  }
  if (nmap > 50) nmap = 50;
  const double bnum = sqrt(15.0) * pow((hs * hs) * delu2n / rnu, sixth);
  const double rmap = P.rmax * tanh(pow(bnum / P.bnumc, P.rlc) * atanh(rc / P.rmax));
  uz = CD_I(S.uf);
  ue = CD_J(S.uf);
  vz = CD_I(S.vf);
  ve = CD_J(S.vf);
  tz = CD_I(S.tf);
  te = CD_J(S.tf);
#undef CD_I
#undef CD_J
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
  double alf11 = 0.0, alf12 = 0.0, alf21 = 0.0, alf22 = 0.0, alf31 = 0.0, alf32 = 0.0, alf33 = 0.0;
  if (fabs(gu) > 0.0) {
    alf11 = gu1 / gu;
    alf12 = gu2 / gu;
  }
  if (fabs(gv) > 0.0) {
    alf21 = gv1 / gv;
    alf22 = gv2 / gv;
  }
  if (fabs(gt) > 0.0) {
    alf31 = gu1 / gt;
    alf32 = gu2 / gt;
    alf33 = sqrt(gt1 * gt1 + gt2 * gt2) / gt;
  }
  // advance the nine maps nmap times and keep them
  double mp[9];
#pragma unroll
  for (int l = 0; l < 9; ++l) mp[l] = S.map[l][o];
  for (int k = 0; k < nmap; ++k)
#pragma unroll
    for (int l = 0; l < 9; ++l) mp[l] = atd_map(rmap, mp[l]);
#pragma unroll
  for (int l = 0; l < 9; ++l) S.map[l][o] = mp[l];
  // both velocity combinations draw on the u maps (small_scale.f:463-466)
  const double um = alf11 * mp[0] + alf12 * mp[1];
  const double vm = alf21 * mp[0] + alf22 * mp[1];
  const double tm = alf31 * mp[6] + alf32 * mp[7] + alf33 * mp[8];
  const double sq = sqrt(rnu * delu2n), r6 = pow(reh, sixth);
  double av = cuV * r6 * sq;
  double at = pow(3.0 * pow(cuT, 4.0) * peh / pr, sixth) * sqrt(dkappa);
  at = at * delt2n / sqrt(delu2n) * P.temcoef;
  const double ascale = sqrt(S.area[o] / *S.tarea);
  const double h3 = pow(hxy, third);
  av = av * ascale * h3;
  at = at * ascale * h3;
  // the u component takes av, as the v component does (small_scale.f:498)
  const double uscon = av * zeta1 * um, vscon = av * zeta2 * vm;
  const double us = rj * (xz * uscon + ye * vscon) / P.uref;
  const double vs = rj * (ye * vscon + yz * uscon) / P.uref;
  const double tsv = (at * tm * 1.0) / (P.tmax - P.tref);
  uss[o] = fabs(us) < 1.0e-14 ? 0.0 : us;
  vss[o] = fabs(vs) < 1.0e-14 ? 0.0 : vs;
  tss[o] = fabs(tsv) < 1.0e-14 ? 0.0 : tsv;
}

// The region loop of small_scale.f:309-520: every cell (iW+1..iE, jS+1..jN)
// of every region that is neither a blockage nor of fixed temperature.
__global__ void k_atd_cells(Dev d, AtdState S, AtdParams P, ThermTables tt, double *uss, double *vss,
                            double *tss) {
  vgrid_set(0, gridDim.x);
  const Regions &r = d.r;
  for (int jr = 1; jr <= r.nrj; ++jr)
    for (int ir = 1; ir <= r.nri; ++ir) {
      if (r.RT(ir, jr) == RM_BLOCKG || t_rt(d, tt, ir, jr) == RT_TEMPER) continue;
      const int iW = r.B(ir, jr, WEST), iE = r.B(ir, jr, EAST);
      const int jS = r.B(ir, jr, SOUTH), jN = r.B(ir, jr, NORTH);
      const int w = iE - iW, h = jN - jS;
      for (int t = gtid(); t < w * h; t += gthreads())
        atd_cell(d, S, P, iW + 1 + t % w, jS + 1 + t / w, uss, vss, tss);
    }
}

// pss = 0 on i = 0..nx, j = 0..ny (small_scale.f:536-540).
__global__ void k_atd_zero_p(Dev d, double *p) {
  vgrid_set(0, gridDim.x);
  const int W = d.nx + 1, H = d.ny + 1;
  for (int t = gtid(); t < W * H; t += gthreads()) p[IX(d, t % W, t / W)] = 0.0;
}

// SmlSclBC (bound_cond.f:1211-1500) by one block: the velocity image rows
// region by region and face by face on thread 0 (several are recurrences,
// and later loops read what earlier ones wrote), PresBoundCond on the whole
// block, then the small-scale temperature's homogeneous image rows.  An
// unknown flag sets W2_E_BCFLAG; an outlet on the grid's edge, where the
// reference would write outside its arrays, sets W2_E_UNSUPPORTED.
__global__ void k_atd_bc(Dev d, ThermTables tt, double *u, double *v, double *p, double *t) {
  vgrid_set(0, gridDim.x);
  const Regions &r = d.r;
  Sync *sy = d.sync;
#define UF(i, j) u[IX(d, i, j)]
#define VF(i, j) v[IX(d, i, j)]
#define TF(i, j) t[IX(d, i, j)]
  __shared__ int bad;
  if (threadIdx.x == 0) {
    bad = 0;
    for (int jreg = 1; jreg <= r.nrj && !bad; jreg++)
      for (int ireg = 1; ireg <= r.nri && !bad; ireg++) {
        const int iW = r.B(ireg, jreg, WEST), iE = r.B(ireg, jreg, EAST);
        const int jS = r.B(ireg, jreg, SOUTH), jN = r.B(ireg, jreg, NORTH);
        int i, j;
        switch (r.BT(ireg, jreg, WEST)) {
          case BM_INTERN: break;
          case BM_WALL1: case BM_INLET:
            for (j = jS; j <= jN; j++) UF(iW, j) = 0.0;
            for (j = jS + 1; j <= jN; j++) VF(iW, j) = -VF(iW + 1, j);
            break;
          case BM_WALL2:
            for (j = jS; j <= jN; j++) UF(iW, j) = 0.0;
            for (j = jS + 1; j <= jN; j++) VF(iW, j) = VF(iW + 1, j);
            break;
          case BM_OUTLT1:
            if (iW < 1) { bad = W2_E_UNSUPPORTED; break; }
            for (j = jS; j <= jN; j++) UF(iW - 1, j) = UF(iW, j);
            for (j = jS + 1; j <= jN; j++) VF(iW, j) = -VF(iW + 1, j);
            break;
          case BM_OUTLT2:
            if (jS < 1) { bad = W2_E_UNSUPPORTED; break; }
            for (j = jS; j <= jN; j++) UF(iW, j) = UF(iW + 1, j) - VF(iW, j) + VF(iW, j - 1);
            for (j = jS + 1; j <= jN; j++)
              VF(iW, j) = -VF(iW, j - 1) + 5.0 * (VF(iW + 1, j) - VF(iW + 1, j - 1)) +
                          8.0 * (UF(iW + 1, j) - UF(iW, j));
            break;
          default: bad = W2_E_BCFLAG;
        }
        if (bad) break;
        switch (r.BT(ireg, jreg, EAST)) {
          case BM_INTERN: break;
          case BM_WALL1: case BM_INLET:
            for (j = jS; j <= jN; j++) UF(iE, j) = 0.0;
            for (j = jS + 1; j <= jN; j++) VF(iE + 1, j) = -VF(iE, j);
            break;
          case BM_WALL2:
            for (j = jS; j <= jN; j++) UF(iE, j) = 0.0;
            for (j = jS + 1; j <= jN; j++) VF(iE + 1, j) = VF(iE, j);
            break;
          case BM_OUTLT1:  // the u row assigns u(iE+1,j) to itself
            for (j = jS + 1; j <= jN; j++) VF(iE + 1, j) = -VF(iE, j);
            break;
          case BM_OUTLT2:
            for (j = jS + 1; j <= jN; j++) UF(iE, j) = UF(iE - 1, j) - (VF(iE, j) - VF(iE, j - 1));
            for (j = jS + 1; j <= jN - 1; j++)
              VF(iE + 1, j) = VF(iE + 1, j - 1) + 3.0 * (VF(iE, j - 1) - VF(iE, j)) -
                              4.0 * (UF(iE, j) - UF(iE - 1, j));
            break;
          default: bad = W2_E_BCFLAG;
        }
        if (bad) break;
        switch (r.BT(ireg, jreg, SOUTH)) {
          case BM_INTERN: break;
          case BM_WALL1: case BM_INLET:
            for (i = iW + 1; i <= iE; i++) UF(i, jS) = -UF(i, jS + 1);
            for (i = iW; i <= iE; i++) VF(i, jS) = 0.0;
            break;
          case BM_WALL2:
            for (i = iW + 1; i <= iE; i++) UF(i, jS) = UF(i, jS + 1);
            for (i = iW; i <= iE; i++) VF(i, jS) = 0.0;
            break;
          case BM_OUTLT1:
            if (jS < 1) { bad = W2_E_UNSUPPORTED; break; }
            for (i = iW + 1; i <= iE; i++) UF(i, jS) = -UF(i, jS + 1);
            for (i = iW; i <= iE; i++) VF(i, jS - 1) = VF(i, jS);
            break;
          case BM_OUTLT2:
            if (jS < 1 || iW < 1) { bad = W2_E_UNSUPPORTED; break; }
            for (i = iW + 1; i <= iE; i++)
              UF(i, jS - 1) = UF(i - 1, jS - 1) + 5.0 * (UF(i, jS) - UF(i - 1, jS)) +
                              8.0 * (VF(i, jS) - VF(i - 1, jS - 1));
            for (i = iW; i <= iE; i++) VF(i, jS - 1) = VF(i, jS) - UF(i, jS) - UF(i - 1, jS);
            break;
          default: bad = W2_E_BCFLAG;
        }
        if (bad) break;
        switch (r.BT(ireg, jreg, NORTH)) {
          case BM_INTERN: break;
          case BM_WALL1: case BM_INLET:
            for (i = iW + 1; i <= iE; i++) UF(i, jN + 1) = -UF(i, jN);
            for (i = iW; i <= iE; i++) VF(i, jN) = 0.0;
            break;
          case BM_WALL2:
            for (i = iW + 1; i <= iE; i++) UF(i, jN + 1) = UF(i, jN);
            for (i = iW; i <= iE; i++) VF(i, jN) = 0.0;
            break;
          case BM_OUTLT1:
            for (i = iW + 1; i <= iE; i++) UF(i, jN + 1) = -UF(i, jN);
            for (i = iW; i <= iE; i++) VF(i, jN + 1) = VF(i, jN);
            break;
          case BM_OUTLT2:
            if (iW < 1) { bad = W2_E_UNSUPPORTED; break; }
            for (i = iW; i <= iE; i++) VF(i, jN) = VF(i, jN - 1) - (UF(i, jN) - UF(i - 1, jN));
            for (i = iW + 1; i <= iE - 1; i++)
              UF(i, jN + 1) = UF(i - 1, jN + 1) + 3.0 * (UF(i - 1, jN) - UF(i, jN)) -
                              4.0 * (VF(i, jN) - VF(i, jN - 1));
            break;
          default: bad = W2_E_BCFLAG;
        }
      }
    if (bad) set_error(sy, bad);
  }
  __syncthreads();
  if (bad) return;
  // the pressure takes the large-scale pressure conditions
  if (!pres_bound_cond_block(d, p)) {
    if (threadIdx.x == 0) set_error(sy, W2_E_BCFLAG);
    return;
  }
  __syncthreads();
  // the small-scale temperature: homogeneous image conditions
  if (threadIdx.x == 0) {
    for (int jreg = 1; jreg <= r.nrj && !bad; jreg++)
      for (int ireg = 1; ireg <= r.nri && !bad; ireg++) {
        const int iW = r.B(ireg, jreg, WEST), iE = r.B(ireg, jreg, EAST);
        const int jS = r.B(ireg, jreg, SOUTH), jN = r.B(ireg, jreg, NORTH);
        int i, j;
        if (t_rt(d, tt, ireg, jreg) == RT_TEMPER) {
          for (j = jS + 1; j <= jN; j++)
            for (i = iW + 1; i <= iE; i++) TF(i, j) = 0.0;
          for (j = jS + 1; j <= jN; j++) TF(iW + 1, j) = -TF(iW, j);
          for (j = jS + 1; j <= jN; j++) TF(iE, j) = -TF(iE + 1, j);
          for (i = iW + 1; i <= iE; i++) TF(i, jS + 1) = -TF(i, jS);
          for (i = iW + 1; i <= iE; i++) TF(i, jN) = -TF(i, jN + 1);
          continue;
        }
        for (int face = WEST; face <= NORTH; face++) {
          const int bt = t_bt(d, tt, ireg, jreg, face);
          if (bt == BT_INTERN) continue;
          if (bt != BT_TEMPER && bt != BT_HTFLUX) {
            bad = W2_E_BCFLAG;
            break;
          }
          const double sg = bt == BT_TEMPER ? -1.0 : 1.0;
          if (face == WEST)
            for (j = jS + 1; j <= jN; j++) TF(iW, j) = sg * TF(iW + 1, j);
          else if (face == EAST)
            for (j = jS + 1; j <= jN; j++) TF(iE + 1, j) = sg * TF(iE, j);
          else if (face == SOUTH)
            for (i = iW + 1; i <= iE; i++) TF(i, jS) = sg * TF(i, jS + 1);
          else
            for (i = iW + 1; i <= iE; i++) TF(i, jN + 1) = sg * TF(i, jN);
        }
      }
    if (bad) set_error(sy, bad);
  }
#undef UF
#undef VF
#undef TF
}

}  // namespace w2
