// w2_kernels.cuh -- __global__ entry points of the plain FP64 path.
#pragma once
#include "w2_bc.cuh"
#include "w2_momentum.cuh"
#include "w2_ppe.cuh"
#include "w2_ppe_mixed.cuh"
#include "w2_ppe_mixg.cuh"
#include "w2_ppe_tiled.cuh"

namespace w2 {

constexpr int kMaxThreads = 512;

// Per-launch step record written by the kernels.
struct StepOut {
  int nql, nsor;
  double dif[4];
  double divmax;  // max |Divergence(u,v)| on the pressure cells after the step
  double divmax_int;  // the same over the interior cells (div_check_local)
};

// ---- grid metrics (grid.f:258-535) ------------------------------------
__global__ void k_mirror(Dev d, double *x, double *y) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny;
#define X(i, j) x[IX(d, i, j)]
#define Y(i, j) y[IX(d, i, j)]
  for (int i = 1 + threadIdx.x; i <= nx; i += blockDim.x) {
    X(i, 0) = 2.0 * X(i, 1) - X(i, 2);
    X(i, ny + 1) = 2.0 * X(i, ny) - X(i, ny - 1);
    Y(i, 0) = 2.0 * Y(i, 1) - Y(i, 2);
    Y(i, ny + 1) = 2.0 * Y(i, ny) - Y(i, ny - 1);
  }
  for (int j = 1 + threadIdx.x; j <= ny; j += blockDim.x) {
    X(0, j) = 2.0 * X(1, j) - X(2, j);
    X(nx + 1, j) = 2.0 * X(nx, j) - X(nx - 1, j);
    Y(0, j) = 2.0 * Y(1, j) - Y(2, j);
    Y(nx + 1, j) = 2.0 * Y(nx, j) - Y(nx - 1, j);
  }
  if (threadIdx.x == 0) {
    X(0, 0) = 2.0 * X(1, 1) - X(2, 2);
    Y(0, 0) = 2.0 * Y(1, 1) - Y(2, 2);
    X(0, ny + 1) = 2.0 * X(1, ny) - X(2, ny - 1);
    Y(0, ny + 1) = 2.0 * Y(1, ny) - Y(2, ny - 1);
    X(nx + 1, 0) = 2.0 * X(nx, 1) - X(nx - 1, 2);
    Y(nx + 1, 0) = 2.0 * Y(nx, 1) - Y(nx - 1, 2);
    X(nx + 1, ny + 1) = 2.0 * X(nx, ny) - X(nx - 1, ny - 1);
    Y(nx + 1, ny + 1) = 2.0 * Y(nx, ny) - Y(nx - 1, ny - 1);
  }
}

__global__ void k_fullgrid_uv(Dev d, const double *x, const double *y, double *xu, double *yu,
                              double *xv, double *yv) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny, W = nx + 2, H = ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const int i = t % W, j = t / W;
    const size_t o = IX(d, i, j);
    if (j >= 1) {
      xu[o] = 0.5 * (x[o] + x[IX(d, i, j - 1)]);
      yu[o] = 0.5 * (y[o] + y[IX(d, i, j - 1)]);
    }
    if (i >= 1) {
      xv[o] = 0.5 * (x[o] + x[IX(d, i - 1, j)]);
      yv[o] = 0.5 * (y[o] + y[IX(d, i - 1, j)]);
    }
  }
}

__global__ void k_fullgrid_c(Dev d, const double *xu, const double *yv, double *xc, double *yc) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx + 1) * (ny + 1); t += gthreads()) {
    const int i = t % (nx + 1) + 1, j = t / (nx + 1) + 1;
    const size_t o = IX(d, i, j);
    xc[o] = 0.5 * (xu[o] + xu[IX(d, i - 1, j)]);
    yc[o] = 0.5 * (yv[o] + yv[IX(d, i, j - 1)]);
  }
}

struct MetricOut {
  double *ran, *rbn, *rgn, *rac, *rbc, *rgc, *rau, *rbu, *rbv, *rgv;
  double *dju, *djv, *djc, *djn;
  double *xen, *yen, *xzn, *yzn, *xec, *yec, *xzc, *yzc;
  double *xeu, *yeu, *xzv, *yzv, *xzu, *yzu, *xev, *yev;
};

__global__ void k_metric(Dev d, MetricOut m, const double *xn, const double *yn, const double *xu,
                         const double *yu, const double *xv, const double *yv, const double *xc,
                         const double *yc) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < nx * ny; t += gthreads()) {
    const int i = t % nx + 1, j = t / nx + 1;
    const size_t o = IX(d, i, j);
    double g11, g12, g22;
    // natural points (N), grid.f:425-448
    m.xzn[o] = xv[IX(d, i + 1, j)] - xv[o];
    m.xen[o] = xu[IX(d, i, j + 1)] - xu[o];
    m.yzn[o] = yv[IX(d, i + 1, j)] - yv[o];
    m.yen[o] = yu[IX(d, i, j + 1)] - yu[o];
    m.djn[o] = 1.0 / (m.xzn[o] * m.yen[o] - m.xen[o] * m.yzn[o]);
    g11 = m.xzn[o] * m.xzn[o] + m.yzn[o] * m.yzn[o];
    g12 = m.xzn[o] * m.xen[o] + m.yzn[o] * m.yen[o];
    g22 = m.xen[o] * m.xen[o] + m.yen[o] * m.yen[o];
    m.ran[o] = m.djn[o] * g22;
    m.rbn[o] = -m.djn[o] * g12 * 0.25;
    m.rgn[o] = m.djn[o] * g11;
    // U cells, grid.f:451-477
    m.xzu[o] = xc[IX(d, i + 1, j)] - xc[o];
    m.xeu[o] = xn[o] - xn[IX(d, i, j - 1)];
    m.yzu[o] = yc[IX(d, i + 1, j)] - yc[o];
    m.yeu[o] = yn[o] - yn[IX(d, i, j - 1)];
    m.dju[o] = 1.0 / (m.xzu[o] * m.yeu[o] - m.xeu[o] * m.yzu[o]);
    g12 = m.xzu[o] * m.xeu[o] + m.yzu[o] * m.yeu[o];
    g22 = m.xeu[o] * m.xeu[o] + m.yeu[o] * m.yeu[o];
    m.rau[o] = m.dju[o] * g22;
    m.rbu[o] = -m.dju[o] * g12 * 0.25;
    // V cells, grid.f:480-506
    m.xzv[o] = xn[o] - xn[IX(d, i - 1, j)];
    m.xev[o] = xc[IX(d, i, j + 1)] - xc[o];
    m.yzv[o] = yn[o] - yn[IX(d, i - 1, j)];
    m.yev[o] = yc[IX(d, i, j + 1)] - yc[o];
    m.djv[o] = 1.0 / (m.xzv[o] * m.yev[o] - m.xev[o] * m.yzv[o]);
    g11 = m.xzv[o] * m.xzv[o] + m.yzv[o] * m.yzv[o];
    g12 = m.xzv[o] * m.xev[o] + m.yzv[o] * m.yev[o];
    m.rbv[o] = -m.djv[o] * g12 * 0.25;
    m.rgv[o] = m.djv[o] * g11;
    // P cells, grid.f:509-532
    m.xzc[o] = xu[o] - xu[IX(d, i - 1, j)];
    m.xec[o] = xv[o] - xv[IX(d, i, j - 1)];
    m.yzc[o] = yu[o] - yu[IX(d, i - 1, j)];
    m.yec[o] = yv[o] - yv[IX(d, i, j - 1)];
    m.djc[o] = 1.0 / (m.xzc[o] * m.yec[o] - m.xec[o] * m.yzc[o]);
    g11 = m.xzc[o] * m.xzc[o] + m.yzc[o] * m.yzc[o];
    g12 = m.xzc[o] * m.xec[o] + m.yzc[o] * m.yec[o];
    g22 = m.xec[o] * m.xec[o] + m.yec[o] * m.yec[o];
    m.rac[o] = m.djc[o] * g22;
    m.rbc[o] = -m.djc[o] * g12 * 0.25;
    m.rgc[o] = m.djc[o] * g11;
  }
#undef X
#undef Y
}

__global__ void k_ppe_coef(Dev d) {
  vgrid_set(0, gridDim.x);
  ppe_coefficients(d);
}
__global__ void k_ppe_check(Dev d, int *flag) {
  vgrid_set(0, gridDim.x);
  ppe_check_unit(d, flag);
}

// ---- field copies -------------------------------------------------------
__device__ __forceinline__ void copy3_body(const Dev &d, double *a, const double *a0, double *b,
                                           const double *b0, double *c, const double *c0) {
  const int W = d.nx + 2, H = d.ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const size_t o = IX(d, t % W, t / W);
    a[o] = a0[o];
    b[o] = b0[o];
    if (c) c[o] = c0[o];
  }
}

__global__ void k_copy3(Dev d, double *a, const double *a0, double *b, const double *b0,
                        double *c, const double *c0) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  copy3_body(d, a, a0, b, b0, c, c0);
}

// us(1..nx+1,1..ny+1) = un, vs = vn (momentum.f:114-119)
__global__ void k_naux_init(Dev d, const double *un, const double *vn, double *us, double *vs) {
  vgrid_set(0, gridDim.x);
  const int W = d.nx + 1, H = d.ny + 1;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const size_t o = IX(d, t % W + 1, t / W + 1);
    us[o] = un[o];
    vs[o] = vn[o];
  }
}

// ---- nAuxMomentum --------------------------------------------------------
__global__ void __launch_bounds__(kMaxThreads, 1) k_naux(Dev d, int mqiter, double dk, double re,
                                                      double qtol, const double *un,
                                                      const double *vn, double *us, double *vs,
                                                      StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  int res = -1;
  if (!naux_momentum<double>(d, d.f64, mqiter, dk, re, qtol, un, vn, us, vs, &res)) return;
  if (vblock() == 0 && threadIdx.x == 0) out->nql = res;
}

// nAuxMomentum in single precision (mixed path) on un32, vn32 -> us32, vs32,
// then us, vs = the FP32 results widened to FP64 on every cell.  POR: the
// porous terms are compiled in (a case with porous regions; without them
// the kernel keeps the registers those terms would take).
template <bool POR = false>
__device__ __forceinline__ void naux32_body(const Dev &d, int mqiter, double dk, double re, double qtol,
                                            const float *un, const float *vn, float *us, float *vs,
                                            double *us64, double *vs64, StepOut *out) {
  int res = -1;
  if (!naux_momentum<float, POR>(d, d.f32, mqiter, dk, re, qtol, un, vn, us, vs, &res)) return;
  if (vblock() == 0 && threadIdx.x == 0) out->nql = res;
  const int W = d.nx + 2, H = d.ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const size_t o = IX(d, t % W, t / W);
    us64[o] = (double)us[o];
    vs64[o] = (double)vs[o];
  }
}

__global__ void __launch_bounds__(kMaxThreads, 1) k_naux32(Dev d, int mqiter, double dk, double re,
                                                        double qtol, const float *un,
                                                        const float *vn, float *us, float *vs,
                                                        double *us64, double *vs64, StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  naux32_body(d, mqiter, dk, re, qtol, un, vn, us, vs, us64, vs64, out);
}

// The same with the porous terms of momentum.f:296-324, 621-649 and
// 1115-1226 in single precision.
__global__ void __launch_bounds__(kMaxThreads, 1) k_naux32_por(Dev d, int mqiter, double dk, double re,
                                                            double qtol, const float *un,
                                                            const float *vn, float *us, float *vs,
                                                            double *us64, double *vs64, StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  naux32_body<true>(d, mqiter, dk, re, qtol, un, vn, us, vs, us64, vs64, out);
}

// Time-level copies of the mixed step: p = pn, and the single-precision
// momentum inputs un32 = (float)un, vn32 = (float)vn, us32 = un32,
// vs32 = vn32 on every cell.
__device__ __forceinline__ void copy_mixed_body(const Dev &d, double *p, const double *pn,
                                                const double *un, const double *vn, float *un32,
                                                float *vn32, float *us32, float *vs32) {
  const int W = d.nx + 2, H = d.ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const size_t o = IX(d, t % W, t / W);
    p[o] = pn[o];
    const float a = (float)un[o], b = (float)vn[o];
    un32[o] = a;
    us32[o] = a;
    vn32[o] = b;
    vs32[o] = b;
  }
}

__global__ void k_copy_mixed(Dev d, double *p, const double *pn, const double *un,
                             const double *vn, float *un32, float *vn32, float *us32,
                             float *vs32) {
  vgrid_set(0, gridDim.x);
  copy_mixed_body(d, p, pn, un, vn, un32, vn32, us32, vs32);
}

// Metric array rounded to single precision.
__global__ void k_to_f32(Dev d, const double *src, float *dst) {
  vgrid_set(0, gridDim.x);
  const int W = d.nx + 2, H = d.ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const size_t o = IX(d, t % W, t / W);
    dst[o] = (float)src[o];
  }
}

// ---- boundary programs (one block) -------------------------------------
enum : int { BC_VEL = 1, BC_PRES = 2, BC_OUTFLOW = 4 };

__device__ __forceinline__ void bc_body(const Dev &d, int ops, double *u, double *v, double *p) {
  bool ok = true;
  if (ops & BC_OUTFLOW) ok = ok && vel_outflow_bcs_block(d, u, v);
  if (ops & BC_VEL) ok = ok && vel_bound_cond_block(d, u, v);
  if (ops & BC_PRES) ok = ok && pres_bound_cond_block(d, p);
  if (!ok && threadIdx.x == 0) set_error(d.sync, W2_E_BCFLAG);
}

__global__ void k_bc(Dev d, int ops, double *u, double *v, double *p) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  bc_body(d, ops, u, v, p);
}

// ---- Ppe -----------------------------------------------------------------
// Multi-block form (solvers 3, 4, 5, 6) and single-block form (1, 2: the
// first block of the virtual grid solves, the others only help with the
// divergence and right-hand side).
__device__ __forceinline__ void ppe_body(const Dev &d, int lcartes, int npsolver, int msorit, double dk,
                                         double sortol, double sorrel, const double *u, const double *v,
                                         double *p, StepOut *out) {
  Sync *sy = d.sync;
  ppe_divergence(d, u, v);
  if (!grid_sync(sy)) return;
  if (lcartes) {
    ppe_rhs_grid(d, lcartes, dk, p);
    if (!grid_sync(sy)) return;
  }
  int nconv = 0;
  if (npsolver == 1 || npsolver == 2) {
    if (vblock() == 0) {
      nconv = npsolver == 1 ? sor_lex_block(d, p, lcartes, msorit, dk, sortol, sorrel)
                            : slor_block(d, p, lcartes, msorit, dk, sortol, sorrel);
    }
  } else if (npsolver >= 3 && npsolver <= 6) {
    nconv = ppe_parallel(d, p, npsolver, lcartes, msorit, dk, sortol, sorrel);
    if (nconv < 0) return;
  }
  if (vblock() == 0 && threadIdx.x == 0) out->nsor = nconv < 1 ? msorit : nconv;
}

__global__ void __launch_bounds__(kMaxThreads) k_ppe(Dev d, int lcartes, int npsolver, int msorit,
                                                     double dk, double sortol, double sorrel,
                                                     const double *u, const double *v, double *p,
                                                     StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  ppe_body(d, lcartes, npsolver, msorit, dk, sortol, sorrel, u, v, p, out);
}

// Red/black SOR with two sweeps per grid barrier (unit-stencil rows,
// sorrel = 1); dynamic shared memory holds the staged tile.
template <int NB>
__device__ __forceinline__ void ppe_tiled_body(const Dev &d, const TileGeom &g, int lcartes, int msorit,
                                               double dk, double sortol, double sorrel, const double *u,
                                               const double *v, double *p, StepOut *out) {
  if (step_skip(d)) return;
  Sync *sy = d.sync;
  ppe_divergence(d, u, v);
  if (!grid_sync(sy)) return;
  ppe_rhs_grid(d, lcartes, dk, p);
  if (!grid_sync(sy)) return;
  const int nconv = ppe_rb_tiled<NB>(d, g, p, d.ppn, d.qh, msorit, sortol, sorrel);
  if (nconv < 0) return;
  if (vblock() == 0 && threadIdx.x == 0) out->nsor = nconv < 1 ? msorit : nconv;
}

// Red/black SOR on shared-memory tiles: 512-thread blocks with four points
// of a thread in flight, or (k_ppe_tiled_w) 1024-thread blocks with two.
__global__ void __launch_bounds__(kMaxThreads, 1) k_ppe_tiled(Dev d, TileGeom g, int lcartes,
                                                           int msorit, double dk, double sortol,
                                                           double sorrel, const double *u, const double *v,
                                                           double *p, StepOut *out) {
  vgrid_set(0, gridDim.x);
  ppe_tiled_body<4>(d, g, lcartes, msorit, dk, sortol, sorrel, u, v, p, out);
}
__global__ void __launch_bounds__(1024, 1) k_ppe_tiled_w(Dev d, TileGeom g, int lcartes, int msorit,
                                                         double dk, double sortol, double sorrel,
                                                         const double *u, const double *v, double *p,
                                                         StepOut *out) {
  vgrid_set(0, gridDim.x);
  ppe_tiled_body<2>(d, g, lcartes, msorit, dk, sortol, sorrel, u, v, p, out);
}

// Mixed-precision red/black SOR (FP32 sweeps, FP64 residual and correction)
// with K sweeps per grid barrier; RES: one tile per block resident in shared
// memory, else blocks loop over tiles.
template <int K, bool RES>
__global__ void __launch_bounds__(kMixedThreads, 1) k_ppe_mixed(Dev d, MixedGeom g, MixedArgs a,
                                                      StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  const int nconv = ppe_mixed<K, RES>(d, g, a);
  if (nconv < 0) return;
  if (vblock() == 0 && threadIdx.x == 0) out->nsor = nconv < 1 ? a.msorit : nconv;
}

// Mixed-precision red/black SOR with the grid's own rows (any Cartesian
// grid, blockages, curvilinear grids): one grid barrier per colour.
__global__ void __launch_bounds__(kMaxThreads) k_ppe_mixg(Dev d, MixgArgs a, StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  const int nconv = ppe_mixg(d, a);
  if (nconv < 0) return;
  if (vblock() == 0 && threadIdx.x == 0) out->nsor = nconv < 1 ? a.msorit : nconv;
}

// Its FP32 coefficient planes, formed once per metric upload.
__global__ void k_mixg_coef(Dev d, MixgArgs a) {
  vgrid_set(0, gridDim.x);
  mixg_coefficients(d, a);
}

// The tiled form for Cartesian grids: kMixgtK sweeps per grid barrier on
// halo'd tiles in shared memory.
__global__ void __launch_bounds__(kMixgtThreads, 1) k_ppe_mixgt(Dev d, MixgtGeom g, MixgtArgs a, StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  const int nconv = ppe_mixgt(d, g, a);
  if (nconv < 0) return;
  if (vblock() == 0 && threadIdx.x == 0) out->nsor = nconv < 1 ? a.msorit : nconv;
}

// Its FP32 rows c1..c5 in field layout, the diagonal as its FP32
// reciprocal (every unknown; zeros elsewhere from the allocation).
__global__ void k_mixgt_coef(Dev d, float *c1, float *c2, float *c3, float *c4, float *c5) {
  vgrid_set(0, gridDim.x);
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const size_t o = IX(d, t % (nx - 1) + 2, t / (nx - 1) + 2);
    c1[o] = (float)d.pa1[o];
    c2[o] = (float)d.pa2[o];
    c3[o] = 1.0f / (float)d.pa3[o];
    c4[o] = (float)d.pa4[o];
    c5[o] = (float)d.pa5[o];
  }
}

// ---- Project (utility.f:253-440), masked -------------------------------
__device__ void project_grid(const Dev &d, double dk, const double *p, double *u, double *v) {
  const int nx = d.nx, ny = d.ny, W = nx + 2, H = ny + 2;
  const Metrics &m = d.m;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const int i = t % W, j = t / W;
    const size_t o = IX(d, i, j);
    const uint16_t mk = d.mask[o];
    if (mk & MK_PU) {
      const double pzi = p[IX(d, i + 1, j)] - p[o];
      const double pet = (p[IX(d, i + 1, j + 1)] + p[IX(d, i, j + 1)] - p[IX(d, i + 1, j - 1)] -
                          p[IX(d, i, j - 1)]) / 4.0;
      const double djk = m.dju[o] * dk;
      u[o] = u[o] - djk * (m.yeu[o] * pzi - m.yzu[o] * pet);
    }
    if (mk & MK_PV) {
      const double pzi = (p[IX(d, i + 1, j + 1)] + p[IX(d, i + 1, j)] - p[IX(d, i - 1, j + 1)] -
                          p[IX(d, i - 1, j)]) / 4.0;
      const double pet = p[IX(d, i, j + 1)] - p[o];
      const double djk = m.djv[o] * dk;
      v[o] = v[o] - djk * (-m.xev[o] * pzi + m.xzv[o] * pet);
    }
  }
}

__global__ void k_project(Dev d, double dk, const double *p, double *u, double *v) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  project_grid(d, dk, p, u, v);
}

// DiffMaxNorm (utility.f:446-473) into red[slot]
__device__ double diff_norm_local(const Dev &d, const double *a, const double *b) {
  const int nx = d.nx, ny = d.ny;
  double mx = 0.0;
  for (int t = gtid(); t < (nx - 2) * (ny - 2); t += gthreads()) {
    const int i = t % (nx - 2) + 2, j = t / (nx - 2) + 2;
    const size_t o = IX(d, i, j);
    mx = dmax(mx, fabs(a[o] - b[o]));
  }
  if (gtid() == 0) {
    // DiffMaxNorm starts from |delta(2,2)| (utility.f:446-473): a NaN there
    // keeps the norm NaN (its bits rank above every finite value in the
    // slot's max), so a NaN solution is reported as the reference reports
    // it; NaNs elsewhere are skipped, as its max skips them
    const double d22 = fabs(a[IX(d, 2, 2)] - b[IX(d, 2, 2)]);
    mx = (d22 != d22) ? d22 : dmax(mx, d22);
  }
  return mx;
}

__global__ void k_diff_norm(Dev d, const double *a, const double *b, unsigned long long *slot) {
  vgrid_set(0, gridDim.x);
  block_max_to(slot, diff_norm_local(d, a, b));
}

// Discrete divergence check on the pressure cells (2..nx, 2..ny) outside
// blockages: max |Divergence(u,v)| of the projected field, FP64, into
// `all`; into `inner`, the same over the interior cells -- those whose four
// neighbours are unknowns of the Poisson equation (i, j = 3..n-1) and whose
// four faces are all updated by Project.  There the divergence is dk times
// the Poisson residual, the part a converged solve drives to zero.  In a
// cell touching a boundary it also holds the face value the boundary
// conditions fix and the change of the ghost pressure that Ppe keeps frozen
// during the solve (PresBoundCond runs before and after it, main.f:793-816),
// which no solver tolerance removes.
__device__ void div_check_local(const Dev &d, const double *u, const double *v, double &all,
                                double &inner) {
  const int nx = d.nx, ny = d.ny;
  double mx = 0.0, mi = 0.0;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const uint16_t mk = d.mask[o];
    if (mk & MK_DIVZ) continue;
    const double a = fabs(div_point(d, u, v, i, j));
    mx = dmax(mx, a);
    if (i >= 3 && i <= nx - 1 && j >= 3 && j <= ny - 1 && (mk & MK_PU) && (mk & MK_PV) &&
        (d.mask[IX(d, i - 1, j)] & MK_PU) && (d.mask[IX(d, i, j - 1)] & MK_PV))
      mi = dmax(mi, a);
  }
  all = mx;
  inner = mi;
}

// Both divergence maxima of the projected field into slots 16 (all cells)
// and 45 (interior cells).
__device__ __forceinline__ void div_check_to(const Dev &d, const double *u, const double *v) {
  double all, inner;
  div_check_local(d, u, v, all, inner);
  block_max_to(&d.sync->red[16], all);
  block_max_to(&d.sync->red[45], inner);
}

// Tail of one step, main.f:813-972: PresBoundCond, Project, boundary
// conditions of the starred and new fields, the three step norms, the
// divergence guard and the discrete divergence check.
__device__ __forceinline__ void step_post_body(const Dev &d, double dk, double *p, const double *pn,
                                               const double *un, const double *vn, double *u,
                                               double *v, StepOut *out) {
  Sync *sy = d.sync;
  if (vblock() == 0) {
    if (!pres_bound_cond_block(d, p) && threadIdx.x == 0) set_error(sy, W2_E_BCFLAG);
  }
  if (vblock() == 0 && threadIdx.x == 0) sy->red[6] = sy->red[7] = sy->red[8] = sy->red[16] = sy->red[45] = 0ull;
  if (!grid_sync(sy)) return;
  project_grid(d, dk, p, u, v);
  if (!grid_sync(sy)) return;
  if (vblock() == 0) {
    bool ok = vel_bound_cond_block(d, u, v) && pres_bound_cond_block(d, p);
    // u = us etc. (main.f:864-870) is a buffer swap on the host; then
    // main.f:946-953 applies the conditions again to the new level.
    ok = ok && vel_bound_cond_block(d, u, v) && pres_bound_cond_block(d, p);
    if (!ok && threadIdx.x == 0) set_error(sy, W2_E_BCFLAG);
  }
  if (!grid_sync(sy)) return;
  block_max_to(&sy->red[6], diff_norm_local(d, pn, p));
  block_max_to(&sy->red[7], diff_norm_local(d, un, u));
  block_max_to(&sy->red[8], diff_norm_local(d, vn, v));
  div_check_to(d, u, v);
  if (!grid_sync(sy)) return;
  if (vblock() == 0 && threadIdx.x == 0) {
    out->dif[0] = slot_value(&sy->red[6]);
    out->dif[1] = slot_value(&sy->red[7]);
    out->dif[2] = slot_value(&sy->red[8]);
    out->dif[3] = 0.0;
    out->divmax = slot_value(&sy->red[16]);
    out->divmax_int = slot_value(&sy->red[45]);
    double mx = dmax(dmax(out->dif[0], out->dif[1]), out->dif[2]);
    if (mx > 1.0e12) sy->halt = 1;
  }
}

__global__ void __launch_bounds__(kMaxThreads) k_step_post(Dev d, double dk, double *p,
                                                           const double *pn, const double *un,
                                                           const double *vn, double *u,
                                                           double *v, StepOut *out) {
  vgrid_set(0, gridDim.x);
  if (step_skip(d)) return;
  step_post_body(d, dk, p, pn, un, vn, u, v, out);
}

// ---- self-test of the device-wait limit ------------------------------------
// Two blocks; block 1 leaves at once, so the grid barrier block 0 waits on
// never completes: the wait runs out its time limit, sets W2_E_TIMEOUT and
// returns.  A host-made failure: nothing faults, traps or hangs.
__global__ void k_selftest_wait(Dev d) {
  vgrid_set(0, gridDim.x);
  if (vblock() != 0) return;
  grid_sync(d.sync);
}

// ---- Filter (utility.f:33-247), velocity components ---------------------
// The filtered value of cell (i, j) where the mask bit is set, else the
// value itself.
__device__ __forceinline__ double filter_point(const Dev &d, int bit, double fp, const double *qu, int i,
                                               int j) {
  const size_t o = IX(d, i, j);
  if (d.mask[o] & bit)
    return (qu[IX(d, i, j - 1)] + qu[IX(d, i - 1, j)] + qu[IX(d, i, j + 1)] + qu[IX(d, i + 1, j)] +
            fp * qu[o]) / (fp + 4.0);
  return qu[o];
}

__global__ void k_filter(Dev d, int bit, double fp, const double *qu, double *qh) {
  vgrid_set(0, gridDim.x);
  const int W = d.nx + 2, H = d.ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const int i = t % W, j = t / W;
    qh[IX(d, i, j)] = filter_point(d, bit, fp, qu, i, j);
  }
}

}  // namespace w2
