// w2_adjoint.cuh -- discrete adjoint of the plain FP64 time step.
//
// The adjoint is that of the step as computed, with each step's iteration
// counts held at the values of the forward run (nQLiter Q-L iterations,
// nSorConv SOR sweeps): for those counts the step is a smooth map of the
// velocities, pressures and boundary values, and these kernels apply its
// transpose.  Reverse order of a step (forward order in w2_kernels.cuh /
// w2_api.cu issue_steps):
//   tail    boundary rows and Project: the boundary programs are replayed on
//           the host into a list of linear assignments (adj_bc_ops), applied
//           here in reverse; Project's transpose scatters into the pressure;
//   Ppe     red/black SOR is affine in p and b: its transpose runs the half
//           sweeps in reverse colour order, each a gather from the colour
//           that the forward half sweep updated; b = div/dk and Divergence
//           are transposed after the sweeps;
//   Q-L     each iteration is recomputed from its taped iterate (assembly,
//           both chain solves); the split-2 then split-1 chain solves are
//           transposed (AltTridLU's quirked first row included) and solved
//           with the same exact chain solver, and the row coefficients'
//           adjoints are scattered back through ConvCoef, DConv and DDiff.
// Scatters use FP64 atomics; results are deterministic up to the order of
// those additions.
#pragma once
#include "w2_kernels.cuh"

namespace w2 {

// ---- boundary programs as assignment lists ---------------------------------

// Op k: target tgt[k] = const + sum_q coef[6k+q] * field[src[6k+q]]
// (+ pcoef[k] * face value prof[k] when prof[k] >= 0).  Codes are field * nf
// + cell, fields 0 u, 1 v, 2 p.  Ops of one stage are independent.
constexpr int kAdjSrc = 6;  // sources per op at most

struct AdjBCList {
  const int *stage;   // nstages + 1 op offsets
  int nstages;
  const int *tgt, *src, *nsrc, *prof;
  const double *coef, *pcoef;
  double *tmp;        // one value per op
  size_t nf;
};

__device__ __forceinline__ double *adj_field(double *lu, double *lv, double *lp, size_t nf, int code,
                                             size_t &idx) {
  const int f = (int)((size_t)code / nf);
  idx = (size_t)code - (size_t)f * nf;
  return f == 0 ? lu : (f == 1 ? lv : lp);
}

// The transpose of one boundary program (one block).
__global__ void k_adj_bc(AdjBCList L, double *lu, double *lv, double *lp, double *lprof) {
  for (int s = L.nstages - 1; s >= 0; --s) {
    const int a = L.stage[s], b = L.stage[s + 1];
    for (int k = a + (int)threadIdx.x; k < b; k += (int)blockDim.x) {
      size_t o;
      double *f = adj_field(lu, lv, lp, L.nf, L.tgt[k], o);
      L.tmp[k] = f[o];
      f[o] = 0.0;
    }
    __syncthreads();
    for (int k = a + (int)threadIdx.x; k < b; k += (int)blockDim.x) {
      const double t = L.tmp[k];
      if (t == 0.0) continue;
      for (int q = 0; q < L.nsrc[k]; ++q) {
        size_t o;
        double *f = adj_field(lu, lv, lp, L.nf, L.src[kAdjSrc * k + q], o);
        atomicAdd(&f[o], L.coef[kAdjSrc * k + q] * t);
      }
      if (L.prof[k] >= 0 && lprof) atomicAdd(&lprof[L.prof[k]], L.pcoef[k] * t);
    }
    __syncthreads();
  }
}

// ---- Project (utility.f:253-440) -------------------------------------------
__global__ void k_adj_project(Dev d, double dk, const double *lu, const double *lv, double *lp) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny, W = nx + 2, H = ny + 2;
  const Metrics &m = d.m;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const int i = t % W, j = t / W;
    const size_t o = IX(d, i, j);
    const uint16_t mk = d.mask[o];
    if (mk & MK_PU) {
      const double l = lu[o];
      if (l != 0.0) {
        const double djk = m.dju[o] * dk;
        // u -= djk*(yeu*pzi - yzu*pet), pzi = p(i+1,j)-p(i,j), pet = (p(i+1,j+1)+p(i,j+1)-p(i+1,j-1)-p(i,j-1))/4
        const double gz = -djk * m.yeu[o] * l, ge = djk * m.yzu[o] * l * 0.25;
        atomicAdd(&lp[IX(d, i + 1, j)], gz);
        atomicAdd(&lp[o], -gz);
        atomicAdd(&lp[IX(d, i + 1, j + 1)], ge);
        atomicAdd(&lp[IX(d, i, j + 1)], ge);
        atomicAdd(&lp[IX(d, i + 1, j - 1)], -ge);
        atomicAdd(&lp[IX(d, i, j - 1)], -ge);
      }
    }
    if (mk & MK_PV) {
      const double l = lv[o];
      if (l != 0.0) {
        const double djk = m.djv[o] * dk;
        // v -= djk*(-xev*pzi + xzv*pet), pzi = (p(i+1,j+1)+p(i+1,j)-p(i-1,j+1)-p(i-1,j))/4, pet = p(i,j+1)-p(i,j)
        const double gz = djk * m.xev[o] * l * 0.25, ge = -djk * m.xzv[o] * l;
        atomicAdd(&lp[IX(d, i + 1, j + 1)], gz);
        atomicAdd(&lp[IX(d, i + 1, j)], gz);
        atomicAdd(&lp[IX(d, i - 1, j + 1)], -gz);
        atomicAdd(&lp[IX(d, i - 1, j)], -gz);
        atomicAdd(&lp[IX(d, i, j + 1)], ge);
        atomicAdd(&lp[o], -ge);
      }
    }
  }
}

// ---- Ppe: red/black SOR (pressure.f:457-532) and Divergence ---------------

// Transposed SOR coefficients, fixed for a call: for each unknown x,
// q3 = sorrel/a3(x) and qk = sorrel*ak(x)/a3(x) (k = 1, 2, 4, 5), the
// factors by which x's update reads b and each neighbour.  Evaluated as the
// sweep itself groups them, so the products below round as before.
struct AdjPpeCoef {
  double *q1, *q2, *q3, *q4, *q5;
};

__global__ void k_adj_ppe_coef(Dev d, double sorrel, AdjPpeCoef q) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t x = IX(d, i, j);
    const double a3 = d.pa3[x];
    q.q3[x] = sorrel / a3;
    q.q1[x] = sorrel * d.pa1[x] / a3;
    q.q2[x] = sorrel * d.pa2[x] / a3;
    q.q4[x] = sorrel * d.pa4[x] / a3;
    q.q5[x] = sorrel * d.pa5[x] / a3;
  }
}

// Gather of point (i, j), whose colour is not `par`, from the unknowns of
// colour `par` that it neighbours: sum over such x of dp_x_new/dp_y * lambda_x.
__device__ __forceinline__ double adj_rb_gather(const Dev &d, const AdjPpeCoef &q, const double *lp, int i,
                                                int j) {
  double g = 0.0;
  auto unk = [&](int a, int b) { return a >= 2 && a <= d.nx && b >= 2 && b <= d.ny; };
  // x north of y: y is x's south, coefficient a1(x)
  if (unk(i, j + 1)) {
    const size_t x = IX(d, i, j + 1);
    g -= q.q1[x] * lp[x];
  }
  // x east of y: y is x's west, a2(x)
  if (unk(i + 1, j)) {
    const size_t x = IX(d, i + 1, j);
    g -= q.q2[x] * lp[x];
  }
  // x west of y: y is x's east, a4(x)
  if (unk(i - 1, j)) {
    const size_t x = IX(d, i - 1, j);
    g -= q.q4[x] * lp[x];
  }
  // x south of y: y is x's north, a5(x)
  if (unk(i, j - 1)) {
    const size_t x = IX(d, i, j - 1);
    g -= q.q5[x] * lp[x];
  }
  return g;
}

// Transpose of nsor red/black sweeps (colour 0 then 1 per sweep) with fixed
// count, then of b = div/dk and Divergence.  lp: in, the adjoint of p after
// the sweeps; out, of p before them.  lb: scratch (the adjoint of b).
// lus, lvs: += the divergence's transpose.  q: from k_adj_ppe_coef with the
// same sorrel.
__global__ void __launch_bounds__(kMaxThreads) k_adj_ppe(Dev d, int nsor, double sorrel, double dk,
                                                         AdjPpeCoef q, double *lp, double *lb, double *lus,
                                                         double *lvs) {
  vgrid_set(0, gridDim.x);
  Sync *sy = d.sync;
  const int nx = d.nx, ny = d.ny, W = nx + 1, H = ny + 1;  // points i, j = 1..nx+1, 1..ny+1
  const double om = 1.0 - sorrel;
  for (int t = gtid(); t < (nx + 2) * (ny + 2); t += gthreads()) lb[IX(d, t % (nx + 2), t / (nx + 2))] = 0.0;
  if (!grid_sync(sy)) return;
  for (int h = 2 * nsor - 1; h >= 0; --h) {
    const int par = h & 1;
    const bool first = h == 2 * nsor - 1;
    for (int t = gtid(); t < W * H; t += gthreads()) {
      const int i = t % W + 1, j = t / W + 1;
      const size_t o = IX(d, i, j);
      const bool isu = i >= 2 && i <= nx && j >= 2 && j <= ny;
      if (((i + j) & 1) == par) {
        // the colour's own points: an unknown's update read b; a boundary
        // point of this colour neighbours no unknown of it
        if (isu) lb[o] += q.q3[o] * lp[o];
      } else {
        const double g = adj_rb_gather(d, q, lp, i, j);
        if (isu) lp[o] = (first ? lp[o] : om * lp[o]) + g;
        else lp[o] += g;
      }
    }
    if (!grid_sync(sy)) return;
  }
  // the first forward half sweep (colour 0) also scaled its own points
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    if (((i + j) & 1) == 0 && nsor > 0) lp[IX(d, i, j)] *= om;
  }
  // b = div/dk on the unknowns (Cartesian RhsPpe), Divergence nloc = 1
  const Metrics &m = d.m;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    if (d.mask[o] & MK_DIVZ) continue;
    const double l = lb[o] / dk;
    if (l == 0.0) continue;
    const size_t ow = IX(d, i - 1, j), os = IX(d, i, j - 1);
    // + ucij
    atomicAdd(&lus[o], m.yeu[o] * l);
    const double xa = -m.xeu[o] / 4.0 * l;
    atomicAdd(&lvs[IX(d, i + 1, j)], xa);
    atomicAdd(&lvs[o], xa);
    atomicAdd(&lvs[IX(d, i + 1, j - 1)], xa);
    atomicAdd(&lvs[os], xa);
    // - uci1j
    atomicAdd(&lus[ow], -m.yeu[ow] * l);
    const double xb = m.xeu[ow] / 4.0 * l;
    atomicAdd(&lvs[o], xb);
    atomicAdd(&lvs[ow], xb);
    atomicAdd(&lvs[os], xb);
    atomicAdd(&lvs[IX(d, i - 1, j - 1)], xb);
    // + vcij
    atomicAdd(&lvs[o], m.xzv[o] * l);
    const double ya = -m.yzv[o] / 4.0 * l;
    atomicAdd(&lus[IX(d, i, j + 1)], ya);
    atomicAdd(&lus[IX(d, i - 1, j + 1)], ya);
    atomicAdd(&lus[o], ya);
    atomicAdd(&lus[ow], ya);
    // - vcij1
    atomicAdd(&lvs[os], -m.xzv[os] * l);
    const double yb = m.yzv[os] / 4.0 * l;
    atomicAdd(&lus[o], yb);
    atomicAdd(&lus[ow], yb);
    atomicAdd(&lus[os], yb);
    atomicAdd(&lus[IX(d, i - 1, j - 1)], yb);
  }
}

// ---- Q-L iteration ----------------------------------------------------------

struct AdjIter {
  const double *us, *vs, *un, *vn;  // the iterate and level n
  double *lus, *lvs, *lun, *lvn;    // adjoints (lus, lvs: in lambda of us^k, out of us^(k-1))
  double *sa1x, *sa2x, *sa3x, *sx1;  // split-1 X rows and solution, saved
  double *sa1y, *sa2y, *sa3y, *sy1;
  Chain tx, ty;                     // transposed systems (own storage)
  double dk, re;
};

// Grid point of X chain row t (i = 1..nx, j = 2..ny) and Y chain row q.
__device__ __forceinline__ void xrow_ij(const Dev &d, int t, int &i, int &j) {
  i = t % d.nx + 1;
  j = t / d.nx + 2;
}
__device__ __forceinline__ void yrow_ij(const Dev &d, int q, int &i, int &j) {
  i = q % (d.nx - 1) + 2;
  j = q / (d.nx - 1) + 1;
}

// Transposed system of the effective matrix of a chain (row 0's super
// diagonal a3(0)*a2(0)/a2(1)), set up for the quirked solver: its row 0
// super input is chosen so that the quirk yields the wanted value.
__device__ __forceinline__ void adj_transpose_row(const Chain &c, const double *a1, const double *a2,
                                                  const double *a3, int k, double &t1, double &t2,
                                                  double &t3) {
  const int n = c.n;
  const double a2k = a2[cpos(c, k)];
  t2 = a2k;
  t1 = 0.0;
  t3 = 0.0;
  if (k >= 1) {
    if (k == 1) {
      const int p0 = cpos(c, 0);
      t1 = a3[p0] * a2[p0] / a2k;
    } else {
      t1 = a3[cpos(c, k - 1)];
    }
  }
  if (k <= n - 2) {
    const double a1n = a1[cpos(c, k + 1)];
    if (k == 0) t3 = a1n * a2[cpos(c, 1)] / a2k;
    else t3 = a1n;
  }
}

// Adjoints of the row coefficients of a solved chain (effective matrix, x the
// solution, lb = A^-T lambda_x): la1, la2, la3 of row k, quirk included.
__device__ __forceinline__ void adj_coef(const Chain &c, const double *a2, const double *a3,
                                         const double *x, const double *lb, int k, double &la1,
                                         double &la2, double &la3) {
  const int n = c.n;
  const int p = cpos(c, k);
  const double l = lb[p];
  la1 = k >= 1 ? -l * x[cpos(c, k - 1)] : 0.0;
  la2 = -l * x[p];
  la3 = 0.0;
  if (k <= n - 2) {
    const double xn = x[cpos(c, k + 1)];
    if (k == 0) {
      const int p1 = cpos(c, 1);
      const double ls = -l * xn;  // adjoint of the effective super a3(0)*a2(0)/a2(1)
      la3 = ls * a2[p] / a2[p1];
      la2 += ls * a3[p] / a2[p1];
    } else {
      la3 = -l * xn;
    }
  }
  if (k == 1) {
    // row 1's diagonal enters row 0's effective super
    const int p0 = cpos(c, 0);
    const double ls0 = -lb[p0] * x[p];
    la2 += -ls0 * a3[p0] * a2[p0] / (a2[p] * a2[p]);
  }
}

// ConvCoef adjoints: scatter lambda of a face coefficient into the fields.
__device__ __forceinline__ void adj_conv_x4(const Dev &d, const MomView<double> &V, double *lus,
                                            double *lvs, int i, int j, double l1, double l2) {
  if (!(i <= d.nx && j >= 1 && j <= d.ny) || (l1 == 0.0 && l2 == 0.0)) return;
  atomicAdd(&lus[IX(d, i, j)], 2.0 * V.yeu(i, j) * l1 - 2.0 * V.yzu(i, j) * l2);
  const double lv = -V.xeu(i, j) / 4.0 * l1 + V.xzu(i, j) / 4.0 * l2;
  atomicAdd(&lvs[IX(d, i + 1, j)], lv);
  atomicAdd(&lvs[IX(d, i, j)], lv);
  atomicAdd(&lvs[IX(d, i + 1, j - 1)], lv);
  atomicAdd(&lvs[IX(d, i, j - 1)], lv);
}

__device__ __forceinline__ void adj_conv_y5(const Dev &d, const MomView<double> &V, double *lus,
                                            double *lvs, int i, int j, double l1, double l2) {
  if (!(i >= 1 && i <= d.nx && j <= d.ny) || (l1 == 0.0 && l2 == 0.0)) return;
  atomicAdd(&lvs[IX(d, i, j)], -2.0 * V.xev(i, j) * l1 + 2.0 * V.xzv(i, j) * l2);
  const double lu = V.yev(i, j) / 4.0 * l1 - V.yzv(i, j) / 4.0 * l2;
  atomicAdd(&lus[IX(d, i, j + 1)], lu);
  atomicAdd(&lus[IX(d, i - 1, j + 1)], lu);
  atomicAdd(&lus[IX(d, i, j)], lu);
  atomicAdd(&lus[IX(d, i - 1, j)], lu);
}

__device__ __forceinline__ void adj_conv_x1_c1(const Dev &d, const MomView<double> &V, double *lu,
                                               double *lv, int i, int j, double l) {
  if (i < 1 || j < 1 || l == 0.0) return;
  const double a = 0.5 * V.yec(i, j) * l, b = -0.5 * V.xec(i, j) * l;
  atomicAdd(&lu[IX(d, i, j)], a);
  atomicAdd(&lu[IX(d, i - 1, j)], a);
  atomicAdd(&lv[IX(d, i, j)], b);
  atomicAdd(&lv[IX(d, i, j - 1)], b);
}

__device__ __forceinline__ void adj_conv_x1_c2(const Dev &d, const MomView<double> &V, double *lu,
                                               double *lv, int i, int j, double l) {
  if (i < 1 || j < 1 || i > d.nx || j > d.ny || l == 0.0) return;
  const double a = 0.5 * V.xzn(i, j) * l, b = -0.5 * V.yzn(i, j) * l;
  atomicAdd(&lv[IX(d, i + 1, j)], a);
  atomicAdd(&lv[IX(d, i, j)], a);
  atomicAdd(&lu[IX(d, i, j + 1)], b);
  atomicAdd(&lu[IX(d, i, j)], b);
}

__device__ __forceinline__ void adj_conv_y2_c1(const Dev &d, const MomView<double> &V, double *lu,
                                               double *lv, int i, int j, double l) {
  if (i < 1 || j < 1 || i > d.nx || j > d.ny || l == 0.0) return;
  const double a = 0.5 * V.yen(i, j) * l, b = -0.5 * V.xen(i, j) * l;
  atomicAdd(&lu[IX(d, i, j + 1)], a);
  atomicAdd(&lu[IX(d, i, j)], a);
  atomicAdd(&lv[IX(d, i + 1, j)], b);
  atomicAdd(&lv[IX(d, i, j)], b);
}

__device__ __forceinline__ void adj_conv_y2_c2(const Dev &d, const MomView<double> &V, double *lu,
                                               double *lv, int i, int j, double l) {
  if (i < 1 || j < 1 || l == 0.0) return;
  const double a = 0.5 * V.xzc(i, j) * l, b = -0.5 * V.yzc(i, j) * l;
  atomicAdd(&lv[IX(d, i, j)], a);
  atomicAdd(&lv[IX(d, i, j - 1)], a);
  atomicAdd(&lu[IX(d, i, j)], b);
  atomicAdd(&lu[IX(d, i - 1, j)], b);
}

// DDiffU transpose (momentum.f:1030-1042): l * d(ddiff_u)/du scattered.
__device__ __forceinline__ void adj_ddiff_u(const Dev &d, const MRef<double> &ac, const MRef<double> &bc,
                                            const MRef<double> &bn, const MRef<double> &gn, double *lu,
                                            int i, int j, double l) {
  if (l == 0.0) return;
#define AU(a, b, c) atomicAdd(&lu[IX(d, a, b)], (c) * l)
  const double acp = ac(i + 1, j), ac0 = ac(i, j), bcp = bc(i + 1, j), bc0 = bc(i, j);
  const double bn0 = bn(i, j), bns = bn(i, j - 1), gn0 = gn(i, j), gns = gn(i, j - 1);
  AU(i + 1, j, acp - bns + bn0);
  AU(i, j, -acp - ac0 - gn0 - gns);
  AU(i - 1, j, ac0 - bn0 + bns);
  AU(i + 1, j + 1, bcp + bn0);
  AU(i, j + 1, bcp - bc0 + gn0);
  AU(i + 1, j - 1, -bcp - bns);
  AU(i, j - 1, -bcp + bc0 + gns);
  AU(i - 1, j + 1, -bc0 - bn0);
  AU(i - 1, j - 1, bc0 + bns);
#undef AU
}

// DDiffV transpose (momentum.f:1094-1106)
__device__ __forceinline__ void adj_ddiff_v(const Dev &d, const MRef<double> &an, const MRef<double> &bc,
                                            const MRef<double> &bn, const MRef<double> &gc, double *lv,
                                            int i, int j, double l) {
  if (l == 0.0) return;
#define AV(a, b, c) atomicAdd(&lv[IX(d, a, b)], (c) * l)
  const double an0 = an(i, j), anw = an(i - 1, j), bn0 = bn(i, j), bnw = bn(i - 1, j);
  const double bcn = bc(i, j + 1), bc0 = bc(i, j), gcn = gc(i, j + 1), gc0 = gc(i, j);
  AV(i + 1, j, an0 + bcn - bc0);
  AV(i, j, -an0 - anw - gcn - gc0);
  AV(i - 1, j, anw - bcn + bc0);
  AV(i + 1, j + 1, bn0 + bcn);
  AV(i, j + 1, bn0 - bnw + gcn);
  AV(i + 1, j - 1, -bn0 - bc0);
  AV(i, j - 1, -bn0 + bnw + gc0);
  AV(i - 1, j + 1, -bnw - bcn);
  AV(i - 1, j - 1, bnw + bc0);
#undef AV
}

// Split-1 X row (i, j) transpose: coefficient adjoints la1..la3 and rhs
// adjoint lb into us, vs, un, vn (momentum.f:350-384).
__device__ void adj_xrow1(const Dev &d, const MomView<double> &V, const AdjIter &A, int i, int j,
                          double la1, double la2, double la3, double lb) {
  const double *us = A.us, *vs = A.vs, *un = A.un, *vn = A.vn;
  const double re1 = 1.0 / A.re, dk2 = A.dk * 0.5;
  const size_t o = IX(d, i, j);
  const double rkj = dk2 * V.dju(i, j);
  double c1, c2;
  conv_x4(d, V, us, vs, i, j, c1, c2);
  double l_c1w = 0.0, l_c1o = 0.0, l_c1e = 0.0;
  if (c1 >= 0.0) {
    l_c1w = -rkj * la1;
    l_c1o = rkj * la2;
  } else {
    l_c1o = -rkj * la2;
    l_c1e = rkj * la3;
  }
  adj_conv_x4(d, V, A.lus, A.lvs, i - 1, j, l_c1w, 0.0);
  adj_conv_x4(d, V, A.lus, A.lvs, i, j, l_c1o, 0.0);
  adj_conv_x4(d, V, A.lus, A.lvs, i + 1, j, l_c1e, 0.0);
  if (lb == 0.0) return;
  // b = un - us + rkj*(-cnvs - cnvn) + rkj*re1*(difs + difn)
  atomicAdd(&A.lun[o], lb);
  atomicAdd(&A.lus[o], -lb);
  const double lc = -rkj * lb, ld = rkj * re1 * lb;
  adj_ddiff_u(d, V.rac, V.rbc, V.rbn, V.rgn, A.lus, i, j, ld);
  adj_ddiff_u(d, V.rac, V.rbc, V.rbn, V.rgn, A.lun, i, j, ld);
  // cnv = dconv_u(c2(i,j-1), c1(i,j), c1(i+1,j), c2(i,j), u)
  for (int side = 0; side < 2; ++side) {
    const double *u = side ? un : us, *v = side ? vn : vs;
    double *lu = side ? A.lun : A.lus, *lv = side ? A.lvn : A.lvs;
    const double c2s = conv_x1_c2(d, V, u, v, i, j - 1), c1o = conv_x1_c1(d, V, u, v, i, j);
    const double c1e = conv_x1_c1(d, V, u, v, i + 1, j), c2o = conv_x1_c2(d, V, u, v, i, j);
    const double uo = u[o], us_ = u[IX(d, i, j - 1)], uw = u[IX(d, i - 1, j)], ue = u[IX(d, i + 1, j)],
                 un_ = u[IX(d, i, j + 1)];
    atomicAdd(&lu[IX(d, i, j - 1)], -c2s * lc);
    atomicAdd(&lu[IX(d, i - 1, j)], -c1o * lc);
    atomicAdd(&lu[o], (c1e - c1o + c2o - c2s) * lc);
    atomicAdd(&lu[IX(d, i + 1, j)], c1e * lc);
    atomicAdd(&lu[IX(d, i, j + 1)], c2o * lc);
    adj_conv_x1_c2(d, V, lu, lv, i, j - 1, (-us_ - uo) * lc);
    adj_conv_x1_c1(d, V, lu, lv, i, j, (-uw - uo) * lc);
    adj_conv_x1_c1(d, V, lu, lv, i + 1, j, (uo + ue) * lc);
    adj_conv_x1_c2(d, V, lu, lv, i, j, (uo + un_) * lc);
  }
}

// Split-1 Y row (i, j) transpose (momentum.f:675-711).
__device__ void adj_yrow1(const Dev &d, const MomView<double> &V, const AdjIter &A, int i, int j,
                          double la1, double la2, double la3, double lb) {
  const double *us = A.us, *vs = A.vs, *un = A.un, *vn = A.vn;
  const double re1 = 1.0 / A.re, dk2 = A.dk * 0.5;
  const size_t o = IX(d, i, j);
  const double rkj = dk2 * V.djv(i, j);
  double c1, c2;
  conv_y5(d, V, us, vs, i, j, c1, c2);
  double l_c1w = 0.0, l_c1o = 0.0, l_c1e = 0.0;
  if (c1 >= 0.0) {
    l_c1w = -rkj * la1;
    l_c1o = rkj * la2;
  } else {
    l_c1o = -rkj * la2;
    l_c1e = rkj * la3;
  }
  adj_conv_y5(d, V, A.lus, A.lvs, i - 1, j, l_c1w, 0.0);
  adj_conv_y5(d, V, A.lus, A.lvs, i, j, l_c1o, 0.0);
  adj_conv_y5(d, V, A.lus, A.lvs, i + 1, j, l_c1e, 0.0);
  if (lb == 0.0) return;
  atomicAdd(&A.lvn[o], lb);
  atomicAdd(&A.lvs[o], -lb);
  const double lc = -rkj * lb, ld = rkj * re1 * lb;
  adj_ddiff_v(d, V.ran, V.rbc, V.rbn, V.rgc, A.lvs, i, j, ld);
  adj_ddiff_v(d, V.ran, V.rbc, V.rbn, V.rgc, A.lvn, i, j, ld);
  // cnv = dconv_v(c2(i,j), c1(i-1,j), c1(i,j), c2(i,j+1), v)
  for (int side = 0; side < 2; ++side) {
    const double *u = side ? un : us, *v = side ? vn : vs;
    double *lu = side ? A.lun : A.lus, *lv = side ? A.lvn : A.lvs;
    const double c2o = conv_y2_c2(d, V, u, v, i, j), c1w = conv_y2_c1(d, V, u, v, i - 1, j);
    const double c1o = conv_y2_c1(d, V, u, v, i, j), c2n = conv_y2_c2(d, V, u, v, i, j + 1);
    const double vo = v[o], vs_ = v[IX(d, i, j - 1)], vw = v[IX(d, i - 1, j)], ve = v[IX(d, i + 1, j)],
                 vn_ = v[IX(d, i, j + 1)];
    atomicAdd(&lv[IX(d, i, j - 1)], -c2o * lc);
    atomicAdd(&lv[IX(d, i - 1, j)], -c1w * lc);
    atomicAdd(&lv[o], (c1o - c1w + c2n - c2o) * lc);
    atomicAdd(&lv[IX(d, i + 1, j)], c1o * lc);
    atomicAdd(&lv[IX(d, i, j + 1)], c2n * lc);
    adj_conv_y2_c2(d, V, lu, lv, i, j, (-vs_ - vo) * lc);
    adj_conv_y2_c1(d, V, lu, lv, i - 1, j, (-vw - vo) * lc);
    adj_conv_y2_c1(d, V, lu, lv, i, j, (vo + ve) * lc);
    adj_conv_y2_c2(d, V, lu, lv, i, j + 1, (vo + vn_) * lc);
  }
}

// Split-2 rows (momentum.f:396-428, 723-754) transpose: coefficient
// adjoints into us, vs through cj2 (identity rows have none).
__device__ void adj_xrow2(const Dev &d, const MomView<double> &V, const AdjIter &A, int i, int j,
                          double la1, double la2, double la3) {
  if (d.mask[IX(d, i, j)] & MK_XID) return;
  const double rkj = A.dk * 0.5 * V.dju(i, j);
  double c1, c2;
  conv_x4(d, V, A.us, A.vs, i, j, c1, c2);
  if (c2 >= 0.0) {
    adj_conv_x4(d, V, A.lus, A.lvs, i, j - 1, 0.0, -rkj * la1);
    adj_conv_x4(d, V, A.lus, A.lvs, i, j, 0.0, rkj * la2);
  } else {
    adj_conv_x4(d, V, A.lus, A.lvs, i, j, 0.0, -rkj * la2);
    adj_conv_x4(d, V, A.lus, A.lvs, i, j + 1, 0.0, rkj * la3);
  }
}

__device__ void adj_yrow2(const Dev &d, const MomView<double> &V, const AdjIter &A, int i, int j,
                          double la1, double la2, double la3) {
  if (d.mask[IX(d, i, j)] & MK_YID) return;
  const double rkj = A.dk * 0.5 * V.djv(i, j);
  double c1, c2;
  conv_y5(d, V, A.us, A.vs, i, j, c1, c2);
  if (c2 >= 0.0) {
    adj_conv_y5(d, V, A.lus, A.lvs, i, j - 1, 0.0, -rkj * la1);
    adj_conv_y5(d, V, A.lus, A.lvs, i, j, 0.0, rkj * la2);
  } else {
    adj_conv_y5(d, V, A.lus, A.lvs, i, j, 0.0, -rkj * la2);
    adj_conv_y5(d, V, A.lus, A.lvs, i, j + 1, 0.0, rkj * la3);
  }
}

// The transpose of one Q-L iteration (us^(k-1) -> us^k), with the iteration
// recomputed from its taped iterate first.
__global__ void __launch_bounds__(kMaxThreads, 1) k_adj_iter(Dev d, AdjIter A) {
  vgrid_set(0, gridDim.x);
  Sync *sy = d.sync;
  const MomView<double> &V = d.f64;
  const int nx = d.nx, ny = d.ny, nX = nx * (ny - 1), nY = (nx - 1) * ny;
  // recompute: ConvCoef, split-1 rows, split-1 solves
  mom_conv_coef(d, V, A.us, A.vs, A.un, A.vn);
  if (!grid_sync(sy)) return;
  mom_assemble1(d, V, A.dk, A.re, A.us, A.vs, A.un, A.vn);
  if (!grid_sync(sy)) return;
  if (!solve_chains(d, V.x1, V.y1, 2)) return;
  // keep the split-1 rows and solutions (the split-2 rows take their storage)
  for (int t = gtid(); t < nX + nY; t += gthreads()) {
    if (t < nX) {
      const int p = cpos(V.x1, t);
      A.sa1x[p] = V.x1.a1[p]; A.sa2x[p] = V.x1.a2[p]; A.sa3x[p] = V.x1.a3[p]; A.sx1[p] = V.x1.x[p];
    } else {
      const int p = cpos(V.y1, t - nX);
      A.sa1y[p] = V.y1.a1[p]; A.sa2y[p] = V.y1.a2[p]; A.sa3y[p] = V.y1.a3[p]; A.sy1[p] = V.y1.x[p];
    }
  }
  if (!grid_sync(sy)) return;
  mom_assemble2(d, V, A.dk, A.re, A.us, A.vs);
  if (!grid_sync(sy)) return;
  if (!solve_chains(d, V.x2, V.y2, 2)) return;
  // transposed split-2 systems, rhs = lambda of dus / dvs
  for (int t = gtid(); t < nX + nY; t += gthreads()) {
    int i, j;
    if (t < nX) {
      xrow_ij(d, t, i, j);
      const int p = cpos(A.tx, t);
      double t1, t2, t3;
      adj_transpose_row(V.x2, V.x2.a1, V.x2.a2, V.x2.a3, t, t1, t2, t3);
      A.tx.a1[p] = t1; A.tx.a2[p] = t2; A.tx.a3[p] = t3;
      A.tx.b[p] = A.lus[IX(d, i, j)];
    } else {
      const int q = t - nX;
      yrow_ij(d, q, i, j);
      const int p = cpos(A.ty, q);
      double t1, t2, t3;
      adj_transpose_row(V.y2, V.y2.a1, V.y2.a2, V.y2.a3, q, t1, t2, t3);
      A.ty.a1[p] = t1; A.ty.a2[p] = t2; A.ty.a3[p] = t3;
      A.ty.b[p] = A.lvs[IX(d, i, j)];
    }
  }
  if (!grid_sync(sy)) return;
  if (!solve_chains(d, A.tx, A.ty, 2)) return;
  // split-2 coefficient adjoints into the fields; transposed split-1 systems
  // with rhs = lambda of the split-1 solution (0 on identity rows)
  for (int t = gtid(); t < nX + nY; t += gthreads()) {
    int i, j;
    double la1, la2, la3;
    if (t < nX) {
      xrow_ij(d, t, i, j);
      const int p = cpos(A.tx, t);
      adj_coef(V.x2, V.x2.a2, V.x2.a3, V.x2.x, A.tx.x, t, la1, la2, la3);
      adj_xrow2(d, V, A, i, j, la1, la2, la3);
      double t1, t2, t3;
      adj_transpose_row(V.x1, A.sa1x, A.sa2x, A.sa3x, t, t1, t2, t3);
      A.tx.a1[p] = t1; A.tx.a2[p] = t2; A.tx.a3[p] = t3;
      A.tx.b[p] = (d.mask[IX(d, i, j)] & MK_XID) ? 0.0 : A.tx.x[p];
    } else {
      const int q = t - nX;
      yrow_ij(d, q, i, j);
      const int p = cpos(A.ty, q);
      adj_coef(V.y2, V.y2.a2, V.y2.a3, V.y2.x, A.ty.x, q, la1, la2, la3);
      adj_yrow2(d, V, A, i, j, la1, la2, la3);
      double t1, t2, t3;
      adj_transpose_row(V.y1, A.sa1y, A.sa2y, A.sa3y, q, t1, t2, t3);
      A.ty.a1[p] = t1; A.ty.a2[p] = t2; A.ty.a3[p] = t3;
      A.ty.b[p] = (d.mask[IX(d, i, j)] & MK_YID) ? 0.0 : A.ty.x[p];
    }
  }
  if (!grid_sync(sy)) return;
  if (!solve_chains(d, A.tx, A.ty, 2)) return;
  // split-1 coefficient and rhs adjoints into the fields
  for (int t = gtid(); t < nX + nY; t += gthreads()) {
    int i, j;
    double la1, la2, la3;
    if (t < nX) {
      xrow_ij(d, t, i, j);
      adj_coef(V.x1, A.sa2x, A.sa3x, A.sx1, A.tx.x, t, la1, la2, la3);
      adj_xrow1(d, V, A, i, j, la1, la2, la3, A.tx.x[cpos(A.tx, t)]);
    } else {
      const int q = t - nX;
      yrow_ij(d, q, i, j);
      adj_coef(V.y1, A.sa2y, A.sa3y, A.sy1, A.ty.x, q, la1, la2, la3);
      adj_yrow1(d, V, A, i, j, la1, la2, la3, A.ty.x[cpos(A.ty, q)]);
    }
  }
}

// a += b, c += e on every cell.
__global__ void k_axpy2(Dev d, double *a, const double *b, double *c, const double *e) {
  vgrid_set(0, gridDim.x);
  const int W = d.nx + 2, H = d.ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const size_t o = IX(d, t % W, t / W);
    a[o] += b[o];
    c[o] += e[o];
  }
}

// 0.5 * w * sum of u^2 over the X unknowns (i = 1..nx, j = 2..ny) and v^2 over
// the Y unknowns (i = 2..nx, j = 1..ny) into *J (atomic); lu = w u, lv = w v
// there and 0 elsewhere.
__global__ void k_adj_objective(Dev d, double w, const double *u, const double *v, double *lu, double *lv,
                                double *J) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny, W = nx + 2, H = ny + 2;
  double s = 0.0;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const int i = t % W, j = t / W;
    const size_t o = IX(d, i, j);
    const bool xu = i >= 1 && i <= nx && j >= 2 && j <= ny;
    const bool yv = i >= 2 && i <= nx && j >= 1 && j <= ny;
    lu[o] = xu ? w * u[o] : 0.0;
    lv[o] = yv ? w * v[o] : 0.0;
    if (xu) s += u[o] * u[o];
    if (yv) s += v[o] * v[o];
  }
  s *= 0.5 * w;
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(J, s);
}

}  // namespace w2
