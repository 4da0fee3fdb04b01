// w2_thermal.cuh -- the thermal energy equation on the device: ThermEnergy
// (thermal.f:24-280) with its TempBoundCond (bound_cond.f:1030-1186), and
// EqState (thermal.f:288-329).
//
// ThermEnergy is one persistent kernel of these phases:
//   T0  block 0 applies TempBoundCond to t (regions in the reference's
//       order, one face loop at a time); every block forms the convective
//       coefficients ConvCoef(6) of (u, v) and ConvCoef(3) of (un, vn);
//   T1  split-1 rows on the chain of the (nx-1)(ny-1) interior points in
//       i-fastest order: upwinded i-direction coefficients, right-hand side
//       dk s/2 + 2 rkj (-c + d/pe) from the 9-point stencil of tn;
//   C1  the chain solve (the exact parallel AltTridLU of w2_chain.cuh, with
//       the first-row quirk);
//   T2  split-2 rows: the j-direction coefficients written on the SAME
//       i-fastest chain (as the reference does: its second AltTridLU couples
//       ind-1 and ind+1, i.e. i-neighbours, with j-direction values), right-
//       hand side the split-1 solution, identity rows in fixed-temperature
//       regions;
//   C2  the chain solve;
//   T3  t += solution on the interior.
// Expressions keep the reference's operand order (no FMA contraction in
// this translation unit), so t matches the reference bit for bit.
//
// The time step with the energy equation (main.f:690-972, nthermen = 1) is
// the plain step's launches inside momentum/energy iterations: k_copy_th,
// then per iteration [k_me_begin from the second on] k_naux, k_bc, the Ppe
// kernel, k_me_post, k_therm, k_eq_state, k_me_norms; then k_step_tail_th.
// Iterations after the convergence test fired skip their launches on the
// device (Dev::me_gate, Sync::me_done), so a step is one fixed launch
// sequence and can be captured in a CUDA graph.
#pragma once
#include "w2_kernels.cuh"

namespace w2 {

enum { RT_NOSRCE = 0, RT_HEATGN = 1, RT_TEMPER = 2 };
enum { BT_INTERN = 0, BT_TEMPER = 1, BT_HTFLUX = 2 };

// Thermal region tables, Fortran layout (mgri, mgrj of the momentum tables).
struct ThermTables {
  const int *trt;     // nTRgType(mgri,mgrj)
  const int *tbt;     // nTemBdTp(mgri,mgrj,4)
  const double *trv;  // dTRgVal(mgri,mgrj)
  const double *hgs;  // dHGSTval(mgri,mgrj)
};

struct ThermArgs {
  ThermTables tt;
  double dk, pe;
  const double *un, *vn, *u, *v, *tn;
  double *t;
  double *cu1, *cv1, *cun, *cvn;  // ConvCoef outputs (field layout)
  Chain ch;                       // (nx-1)(ny-1) rows, b included
};

__device__ __forceinline__ int t_rt(const Dev &d, const ThermTables &tt, int ir, int jr) {
  return tt.trt[(ir - 1) + (jr - 1) * d.r.mgri];
}
__device__ __forceinline__ int t_bt(const Dev &d, const ThermTables &tt, int ir, int jr, int s) {
  return tt.tbt[(ir - 1) + (jr - 1) * d.r.mgri + (s - 1) * d.r.mgri * d.r.mgrj];
}
__device__ __forceinline__ double t_val(const Dev &d, const double *a, int ir, int jr) {
  return a[(ir - 1) + (jr - 1) * d.r.mgri];
}
// Face temperature dBCVal(ir, jr, s, _T_).
__device__ __forceinline__ double t_bcv(const Dev &d, int ir, int jr, int s) {
  return d.r.bcv[(ir - 1) + (jr - 1) * d.r.mgri + (s - 1) * d.r.mgri * d.r.mgrj +
                 3 * d.r.mgri * d.r.mgrj * 4];
}

// TempBoundCond by one block: regions in the reference's order (j outer),
// each face loop finished before the next starts, since later loops read
// values earlier ones wrote.  The host has checked every nTemBdTp flag.
__device__ void temp_bc_block(const Dev &d, const ThermTables &tt, double *t) {
  const int T = blockDim.x;
  for (int jr = 1; jr <= d.r.nrj; ++jr)
    for (int ir = 1; ir <= d.r.nri; ++ir) {
      const int iW = d.r.B(ir, jr, 1), iE = d.r.B(ir, jr, 2), jS = d.r.B(ir, jr, 3), jN = d.r.B(ir, jr, 4);
      const int w = iE - iW, h = jN - jS;  // interior width (i = iW+1..iE), height
      if (t_rt(d, tt, ir, jr) == RT_TEMPER) {
        const double tv = t_val(d, tt.trv, ir, jr);
        for (int q = threadIdx.x; q < w * h; q += T) t[IX(d, iW + 1 + q % w, jS + 1 + q / w)] = tv;
        __syncthreads();
        const double bw = t_bcv(d, ir, jr, 1), be = t_bcv(d, ir, jr, 2);
        const double bs = t_bcv(d, ir, jr, 3), bn = t_bcv(d, ir, jr, 4);
        for (int q = threadIdx.x; q < h; q += T) t[IX(d, iW + 1, jS + 1 + q)] = 2.0 * bw - t[IX(d, iW, jS + 1 + q)];
        __syncthreads();
        for (int q = threadIdx.x; q < h; q += T) t[IX(d, iE, jS + 1 + q)] = 2.0 * be - t[IX(d, iE + 1, jS + 1 + q)];
        __syncthreads();
        for (int q = threadIdx.x; q < w; q += T) t[IX(d, iW + 1 + q, jS + 1)] = 2.0 * bs - t[IX(d, iW + 1 + q, jS)];
        __syncthreads();
        for (int q = threadIdx.x; q < w; q += T) t[IX(d, iW + 1 + q, jN)] = 2.0 * bn - t[IX(d, iW + 1 + q, jN + 1)];
        __syncthreads();
        continue;
      }
      // west, east: ghost column iW / iE+1 from column iW+1 / iE
      for (int s = 1; s <= 4; ++s) {
        const int bt = t_bt(d, tt, ir, jr, s);
        if (bt == BT_INTERN) continue;
        const double bv = t_bcv(d, ir, jr, s);
        const bool ew = s <= 2;
        const int n = ew ? h : w;
        for (int q = threadIdx.x; q < n; q += T) {
          size_t g, in;
          if (s == 1) { g = IX(d, iW, jS + 1 + q); in = IX(d, iW + 1, jS + 1 + q); }
          else if (s == 2) { g = IX(d, iE + 1, jS + 1 + q); in = IX(d, iE, jS + 1 + q); }
          else if (s == 3) { g = IX(d, iW + 1 + q, jS); in = IX(d, iW + 1 + q, jS + 1); }
          else { g = IX(d, iW + 1 + q, jN + 1); in = IX(d, iW + 1 + q, jN); }
          t[g] = bt == BT_TEMPER ? 2.0 * bv - t[in] : bv + t[in];
        }
        __syncthreads();
      }
    }
}

// Region of interior point (i, j): the one whose interior (iW, iE] x (jS, jN]
// holds it.  Regions tile the interior, so one always does.
__device__ __forceinline__ void region_of(const Dev &d, int i, int j, int &ir, int &jr) {
  ir = 1;
  while (ir < d.r.nri && i > d.r.B(ir, 1, 2)) ++ir;
  jr = 1;
  while (jr < d.r.nrj && j > d.r.B(1, jr, 4)) ++jr;
}

__global__ void __launch_bounds__(kMaxThreads, 1) k_therm(Dev d, ThermArgs A) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  Sync *sy = d.sync;
  const int nx = d.nx, ny = d.ny;
  const Metrics &m = d.m;
  // ---- T0
  if (vblock() == 0) temp_bc_block(d, A.tt, A.t);
  {
    // ConvCoef case 6 (xzc, xec, yzc, yec; u, v) on i, j = 1..n+1
    const int W = nx + 1, H = ny + 1;
    for (int q = gtid(); q < W * H; q += gthreads()) {
      const int i = q % W + 1, j = q / W + 1;
      const size_t o = IX(d, i, j), w = IX(d, i - 1, j), s = IX(d, i, j - 1);
      A.cu1[o] = (m.yec[o] * (A.u[o] + A.u[w]) - m.xec[o] * (A.v[o] + A.v[s])) * 0.5;
      A.cv1[o] = (m.xzc[o] * (A.v[o] + A.v[s]) - m.yzc[o] * (A.u[o] + A.u[w])) * 0.5;
    }
    // ConvCoef case 3 (xzv, xeu, yzv, yeu; un, vn) on i, j = 1..n
    for (int q = gtid(); q < nx * ny; q += gthreads()) {
      const int i = q % nx + 1, j = q / nx + 1;
      const size_t o = IX(d, i, j);
      const double *un = A.un, *vn = A.vn;
      A.cun[o] = (m.yeu[o] * un[o] - m.xeu[o] * (vn[IX(d, i + 1, j)] + vn[o] + vn[IX(d, i + 1, j - 1)] +
                                                  vn[IX(d, i, j - 1)]) / 4.0) * 0.5;
      A.cvn[o] = (m.xzv[o] * vn[o] - m.yzv[o] * (un[IX(d, i, j + 1)] + un[IX(d, i - 1, j + 1)] + un[o] +
                                                  un[IX(d, i - 1, j)]) / 4.0) * 0.5;
    }
  }
  if (!grid_sync(sy)) return;
  const double pe1 = 1.0 / A.pe, dk = A.dk;
  const int n = (nx - 1) * (ny - 1);
  // ---- T1
  for (int k = gtid(); k < n; k += gthreads()) {
    const int i = k % (nx - 1) + 2, j = k / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const int p = cpos(A.ch, k);
    const double rkj = dk * m.djc[o] * 0.5;
    const double rw = m.rau[IX(d, i - 1, j)], ro = m.rau[o];
    const double cu = A.cu1[o];
    double a1, a2, a3;
    if (cu >= 0.0) {
      a1 = rkj * (-A.cu1[IX(d, i - 1, j)] - pe1 * rw);
      a2 = 1.0 + rkj * (cu + pe1 * (ro + rw));
      a3 = rkj * (-pe1 * ro);
    } else {
      a1 = rkj * (-pe1 * rw);
      a2 = 1.0 + rkj * (-cu + pe1 * (ro + rw));
      a3 = rkj * (A.cu1[IX(d, i + 1, j)] - pe1 * ro);
    }
    const double *tn = A.tn;
    const size_t e = IX(d, i + 1, j), w = IX(d, i - 1, j), s = IX(d, i, j - 1), nn = IX(d, i, j + 1);
    const size_t ne = IX(d, i + 1, j + 1), se = IX(d, i + 1, j - 1), nw = IX(d, i - 1, j + 1),
                 sw = IX(d, i - 1, j - 1);
    const double cc = -A.cvn[s] * tn[s] - A.cun[w] * tn[w] +
                      (A.cun[o] - A.cun[w] + A.cvn[o] - A.cvn[s]) * tn[o] + A.cun[o] * tn[e] +
                      A.cvn[o] * tn[nn];
    const double dd = m.rau[o] * (tn[e] - tn[o]) - m.rau[w] * (tn[o] - tn[w]) +
                      m.rbu[o] * (tn[ne] + tn[nn] - tn[se] - tn[s]) -
                      m.rbu[w] * (tn[nn] + tn[nw] - tn[s] - tn[sw]) +
                      m.rbv[o] * (tn[ne] + tn[e] - tn[nw] - tn[w]) -
                      m.rbv[s] * (tn[e] + tn[se] - tn[w] - tn[sw]) + m.rgv[o] * (tn[nn] - tn[o]) -
                      m.rgv[s] * (tn[o] - tn[s]);
    int ir, jr;
    region_of(d, i, j, ir, jr);
    const double sv = t_rt(d, A.tt, ir, jr) == RT_HEATGN ? t_val(d, A.tt.hgs, ir, jr) : 0.0;
    A.ch.a1[p] = a1;
    A.ch.a2[p] = a2;
    A.ch.a3[p] = a3;
    A.ch.b[p] = dk * sv * 0.5 + 2.0 * rkj * (-cc + pe1 * dd);
  }
  if (!grid_sync(sy)) return;
  // ---- C1
  if (!solve_chains(d, A.ch, A.ch, 1)) return;
  // ---- T2 (rows at the same storage positions; the solve's last barrier
  // has passed, so the rows of C1 are dead)
  for (int k = gtid(); k < n; k += gthreads()) {
    const int i = k % (nx - 1) + 2, j = k / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const int p = cpos(A.ch, k);
    int ir, jr;
    region_of(d, i, j, ir, jr);
    double a1, a2, a3, b;
    if (t_rt(d, A.tt, ir, jr) == RT_TEMPER) {
      a1 = 0.0;
      a2 = 1.0;
      a3 = 0.0;
      b = 0.0;
    } else {
      const double rkj = dk * m.djc[o] * 0.5;
      const double rs = m.rgv[IX(d, i, j - 1)], ro = m.rgv[o];
      const double cv = A.cv1[o];
      if (cv >= 0.0) {
        a1 = rkj * (-A.cv1[IX(d, i, j - 1)] - pe1 * rs);
        a2 = 1.0 + rkj * (cv + pe1 * (ro + rs));
        a3 = rkj * (-pe1 * ro);
      } else {
        a1 = rkj * (-pe1 * rs);
        a2 = 1.0 + rkj * (-cv + pe1 * (ro + rs));
        a3 = rkj * (A.cv1[IX(d, i, j + 1)] - pe1 * ro);
      }
      b = A.ch.x[p];
    }
    A.ch.a1[p] = a1;
    A.ch.a2[p] = a2;
    A.ch.a3[p] = a3;
    A.ch.b[p] = b;
  }
  if (!grid_sync(sy)) return;
  // ---- C2
  if (!solve_chains(d, A.ch, A.ch, 1)) return;
  // ---- T3
  for (int k = gtid(); k < n; k += gthreads()) {
    const int i = k % (nx - 1) + 2, j = k / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    A.t[o] = A.t[o] + A.ch.x[cpos(A.ch, k)];
  }
}

// TempBoundCond alone (one block).
__global__ void k_temp_bc(Dev d, ThermTables tt, double *t) {
  vgrid_set(0, gridDim.x);
  temp_bc_block(d, tt, t);
}

// EqState on i, j = 2..n.
__global__ void k_eq_state(Dev d, double uref, double densref, double tmax, double tref, double rconst,
                           const double *p, const double *t, double *den) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  const int nx = d.nx, ny = d.ny;
  const double pref = densref * rconst * tref;
  for (int q = gtid(); q < (nx - 1) * (ny - 1); q += gthreads()) {
    const int i = q % (nx - 1) + 2, j = q / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const double c1 = p[o] * densref * (uref * uref) + pref;
    const double c2 = densref * rconst * (t[o] * (tmax - tref) + tref);
    double r = c1 / c2 - 1.0;
    if (fabs(r) < 1.0e-10) r = 0.0;
    den[o] = r;
  }
}

// Filter of a scalar (utility.f:33-247 with ncomp = _T_): the Shuman filter
// on the interior of every region whose nTRgType is not 1 (the reference
// compares nTRgType with BT_TEMPER, whose value is 1), from qu into qh; the
// other points copy qu.  The caller copies qh back to qu.
__global__ void k_filter_t(Dev d, ThermTables tt, double fp, const double *qu, double *qh) {
  vgrid_set(0, gridDim.x);
  if (d.sync->halt) return;
  const int W = d.nx + 2, H = d.ny + 2;
  for (int q = gtid(); q < W * H; q += gthreads()) {
    const int i = q % W, j = q / W;
    const size_t o = IX(d, i, j);
    double r = qu[o];
    if (i >= 2 && i <= d.nx && j >= 2 && j <= d.ny) {
      int ir, jr;
      region_of(d, i, j, ir, jr);
      if (t_rt(d, tt, ir, jr) != BT_TEMPER)
        r = (qu[IX(d, i, j - 1)] + qu[IX(d, i - 1, j)] + qu[IX(d, i, j + 1)] + qu[IX(d, i + 1, j)] + fp * qu[o]) /
            (fp + 4.0);
    }
    qh[o] = r;
  }
}

// ---- the time step with the energy equation --------------------------------

// Time levels (main.f:696-704) and the first iterates (main.f:741-747, with
// nAuxMomentum's us = un): us = un, vs = vn, p = pn, ts = tn on the whole
// array, dn = d; the momentum/energy iterations start unconverged.
__global__ void k_copy_th(Dev d, double *us, const double *un, double *vs, const double *vn, double *p,
                          const double *pn, double *ts, const double *tn, double *dn, const double *den) {
  vgrid_set(0, gridDim.x);
  if (d.sync->halt) return;
  if (vblock() == 0 && threadIdx.x == 0) d.sync->me_done = 0;
  const int W = d.nx + 2, H = d.ny + 2;
  for (int q = gtid(); q < W * H; q += gthreads()) {
    const size_t o = IX(d, q % W, q / W);
    us[o] = un[o];
    vs[o] = vn[o];
    p[o] = pn[o];
    ts[o] = tn[o];
    dn[o] = den[o];
  }
}

// Iteration l >= 2: keep the previous iterates (u, v, t before this pass,
// for the convergence norms), then nAuxMomentum's us(1..nx+1,1..ny+1) = un
// (momentum.f:114-119); ts = t is the array itself.
__global__ void k_me_begin(Dev d, const double *un, const double *vn, double *us, double *vs,
                           const double *ts, double *up, double *vp, double *tp) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  const int W = d.nx + 2, H = d.ny + 2;
  for (int q = gtid(); q < W * H; q += gthreads()) {
    const int i = q % W, j = q / W;
    const size_t o = IX(d, i, j);
    up[o] = us[o];
    vp[o] = vs[o];
    tp[o] = ts[o];
    if (i >= 1 && j >= 1) {
      us[o] = un[o];
      vs[o] = vn[o];
    }
  }
}

// After Ppe in an iteration (main.f:818-836): PresBoundCond, Project,
// VelBoundCond, PresBoundCond.
__global__ void __launch_bounds__(kMaxThreads) k_me_post(Dev d, double dk, double *p, double *u, double *v) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  Sync *sy = d.sync;
  if (vblock() == 0 && !pres_bound_cond_block(d, p) && threadIdx.x == 0) set_error(sy, W2_E_BCFLAG);
  if (!grid_sync(sy)) return;
  project_grid(d, dk, p, u, v);
  if (!grid_sync(sy)) return;
  if (vblock() == 0) {
    const bool ok = vel_bound_cond_block(d, u, v) && pres_bound_cond_block(d, p);
    if (!ok && threadIdx.x == 0) set_error(sy, W2_E_BCFLAG);
  }
}

// The iteration's convergence norms (main.f:857-877): DiffMaxNorm of the
// previous and new u, v, t; from iteration 2 on, max < dmeittol ends the
// iterations.
__global__ void __launch_bounds__(kMaxThreads) k_me_norms(Dev d, int l, double tol, const double *up,
                                                         const double *vp, const double *tp,
                                                         const double *us, const double *vs,
                                                         const double *ts) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  Sync *sy = d.sync;
  if (vblock() == 0 && threadIdx.x == 0) sy->red[41] = sy->red[42] = sy->red[43] = 0ull;
  if (!grid_sync(sy)) return;
  block_max_to(&sy->red[41], diff_norm_local(d, up, us));
  block_max_to(&sy->red[42], diff_norm_local(d, vp, vs));
  block_max_to(&sy->red[43], diff_norm_local(d, tp, ts));
  if (!grid_sync(sy)) return;
  if (vblock() == 0 && threadIdx.x == 0) {
    double mx = slot_value(&sy->red[41]);
    const double m2 = slot_value(&sy->red[42]), m3 = slot_value(&sy->red[43]);
    if (m2 > mx) mx = m2;
    if (m3 > mx) mx = m3;
    if (l > 1 && mx < tol) sy->me_done = 1;
  }
}

// After the iterations (main.f:881-972 without Filter of t): VelBoundCond,
// PresBoundCond, TempBoundCond on the new level, the step norms of p, u, v, t
// and the divergence test.
__global__ void __launch_bounds__(kMaxThreads) k_step_tail_th(Dev d, ThermTables tt, int therm, double *p,
                                                             const double *pn, const double *un,
                                                             const double *vn, double *u, double *v,
                                                             const double *tn, double *t, StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (d.sync->halt) return;
  Sync *sy = d.sync;
  if (vblock() == 0) {
    const bool ok = vel_bound_cond_block(d, u, v) && pres_bound_cond_block(d, p);
    if (!ok && threadIdx.x == 0) set_error(sy, W2_E_BCFLAG);
    if (therm) temp_bc_block(d, tt, t);
    if (threadIdx.x == 0) sy->red[6] = sy->red[7] = sy->red[8] = sy->red[16] = sy->red[44] = sy->red[45] = 0ull;
  }
  if (!grid_sync(sy)) return;
  block_max_to(&sy->red[6], diff_norm_local(d, pn, p));
  block_max_to(&sy->red[7], diff_norm_local(d, un, u));
  block_max_to(&sy->red[8], diff_norm_local(d, vn, v));
  block_max_to(&sy->red[44], diff_norm_local(d, tn, t));
  div_check_to(d, u, v);
  if (!grid_sync(sy)) return;
  if (vblock() == 0 && threadIdx.x == 0) {
    out->dif[0] = slot_value(&sy->red[6]);
    out->dif[1] = slot_value(&sy->red[7]);
    out->dif[2] = slot_value(&sy->red[8]);
    out->dif[3] = slot_value(&sy->red[44]);
    out->divmax = slot_value(&sy->red[16]);
    out->divmax_int = slot_value(&sy->red[45]);
    const double mx = dmax(dmax(dmax(out->dif[0], out->dif[1]), out->dif[2]), out->dif[3]);
    if (mx > 1.0e12) sy->halt = 1;
  }
}

}  // namespace w2
