// w2_ppe.cuh -- the pseudo-pressure Poisson equation (pressure.f:30-1138).
//
// Coefficients a(ind,1..5) (pressure.f:97-196) depend only on the metrics and
// the region tables, so they are formed once per metric upload in field
// layout (pa1..pa5 at (i,j)).  Per Ppe call the divergence (nloc = 1) and the
// right-hand side b = div/dk (+ cross terms on non-Cartesian grids) are
// formed, then the selected relaxation runs with its own stopping rule
// "m > 1 and dif < sortol".  Ghost values of p are left exactly as
// PresBoundCond set them before the call (the reference never refreshes
// them during the iterations).
//
//   Sor (1)           lexicographic point SOR: one block, rows as threads,
//                     skewed one column per row so that each anti-diagonal
//                     step sees exactly the new/old neighbour values of the
//                     sequential loop (pressure.f:431-441);
//   Slor (2)          line SOR, lines in sequence, one thread per line;
//   SlorRB (3)        red/black line SOR, lines of one colour in parallel;
//   SlorRBP (4)       red/black line SOR with deferred relaxation;
//   SorRB/SorRBP (5,6) red/black point SOR, points of one colour in
//                     parallel; both produce identical numbers (the per-point
//                     dif array of SorRBP has the same maximum).
#pragma once
#include "w2_common.cuh"
#include "w2_bc.cuh"

namespace w2 {

// Coefficients, pressure.f:97-196 (identity rows from the mask).
__device__ void ppe_coefficients(const Dev &d) {
  const int nx = d.nx, ny = d.ny;
  const Metrics &m = d.m;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    if (d.mask[o] & MK_PID) {
      d.pa1[o] = 0.0; d.pa2[o] = 0.0; d.pa3[o] = 1.0; d.pa4[o] = 0.0; d.pa5[o] = 0.0;
    } else {
      const double rau0 = m.rau[o], rauw = m.rau[IX(d, i - 1, j)];
      const double rgv0 = m.rgv[o], rgvs = m.rgv[IX(d, i, j - 1)];
      d.pa1[o] = rgvs;
      d.pa2[o] = rauw;
      d.pa3[o] = -rau0 - rauw - rgv0 - rgvs;
      d.pa4[o] = rau0;
      d.pa5[o] = rgv0;
    }
  }
}

// Flags any row whose coefficients are not the unit stencil (identity rows
// of blockages excluded from the check; the unit form is used only when
// there are none).
// flag bit 0: some row is not exactly (1,1,-4,1,1) (or is an identity row);
// bit 1: some row does not round to it in FP32 (or is an identity row).
__device__ void ppe_check_unit(const Dev &d, int *flag) {
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const bool id = (d.mask[o] & MK_PID) != 0;
    if (id || d.pa1[o] != 1.0 || d.pa2[o] != 1.0 || d.pa3[o] != -4.0 || d.pa4[o] != 1.0 ||
        d.pa5[o] != 1.0)
      atomicOr(flag, 1);
    if (id || (float)d.pa1[o] != 1.0f || (float)d.pa2[o] != 1.0f || (float)d.pa3[o] != -4.0f ||
        (float)d.pa4[o] != 1.0f || (float)d.pa5[o] != 1.0f)
      atomicOr(flag, 2);
  }
}

// Divergence nloc = 1 at cell (i,j), pressure.f:287-299.
__device__ __forceinline__ double div_point(const Dev &d, const double *u, const double *v,
                                            int i, int j) {
  const Metrics &m = d.m;
  const size_t o = IX(d, i, j), ow = IX(d, i - 1, j), os = IX(d, i, j - 1);
  const double ucij = m.yeu[o] * u[o] -
                      m.xeu[o] * (v[IX(d, i + 1, j)] + v[o] + v[IX(d, i + 1, j - 1)] + v[os]) / 4.0;
  const double uci1j = m.yeu[ow] * u[ow] -
                       m.xeu[ow] * (v[o] + v[ow] + v[os] + v[IX(d, i - 1, j - 1)]) / 4.0;
  const double vcij = m.xzv[o] * v[o] -
                      m.yzv[o] * (u[IX(d, i, j + 1)] + u[IX(d, i - 1, j + 1)] + u[o] + u[ow]) / 4.0;
  const double vcij1 = m.xzv[os] * v[os] -
                       m.yzv[os] * (u[o] + u[ow] + u[os] + u[IX(d, i - 1, j - 1)]) / 4.0;
  return ucij - uci1j + vcij - vcij1;
}

// Divergence nloc = 1 on i,j = 1..nx,1..ny, then blockage zeroing.
__device__ void ppe_divergence(const Dev &d, const double *u, const double *v) {
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < nx * ny; t += gthreads()) {
    const int i = t % nx + 1, j = t / nx + 1;
    const size_t o = IX(d, i, j);
    d.div[o] = (d.mask[o] & MK_DIVZ) ? 0.0 : div_point(d, u, v, i, j);
  }
}

// RhsPpe, pressure.f:354-375 (one point).
__device__ __forceinline__ double rhs_point(const Dev &d, int lcartes, double dk,
                                            const double *p, int i, int j) {
  const size_t o = IX(d, i, j);
  double b = d.div[o] / dk;
  if (!lcartes) {
    const double *rbu = d.m.rbu, *rbv = d.m.rbv;
#define Pp(a, c) p[IX(d, a, c)]
    b = b - (rbu[o] * (Pp(i + 1, j + 1) + Pp(i, j + 1) - Pp(i + 1, j - 1) - Pp(i, j - 1)) -
             rbu[IX(d, i - 1, j)] * (Pp(i, j + 1) + Pp(i - 1, j + 1) - Pp(i, j - 1) - Pp(i - 1, j - 1)) +
             rbv[o] * (Pp(i + 1, j + 1) + Pp(i + 1, j) - Pp(i - 1, j + 1) - Pp(i - 1, j)) -
             rbv[IX(d, i, j - 1)] * (Pp(i + 1, j) + Pp(i + 1, j - 1) - Pp(i - 1, j) - Pp(i - 1, j - 1)));
#undef Pp
  }
  return b;
}

__device__ void ppe_rhs_grid(const Dev &d, int lcartes, double dk, const double *p) {
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    d.pb[IX(d, i, j)] = rhs_point(d, lcartes, dk, p, i, j);
  }
}

__device__ void ppe_rhs_block(const Dev &d, int lcartes, double dk, const double *p) {
  const int nx = d.nx, ny = d.ny;
  for (int t = threadIdx.x; t < (nx - 1) * (ny - 1); t += blockDim.x) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    d.pb[IX(d, i, j)] = rhs_point(d, lcartes, dk, p, i, j);
  }
}

// One point of Sor/SorRB/SorRBP, pressure.f:434-439: returns |delta|.
__device__ __forceinline__ double sor_point(const Dev &d, double *p, int i, int j, double sorrel) {
  const size_t o = IX(d, i, j);
  double sum = d.pb[o] - d.pa1[o] * p[IX(d, i, j - 1)] - d.pa2[o] * p[IX(d, i - 1, j)] -
               d.pa4[o] * p[IX(d, i + 1, j)] - d.pa5[o] * p[IX(d, i, j + 1)];
  sum = sum / d.pa3[o] - p[o];
  p[o] = p[o] + sorrel * sum;
  return sum;
}

// Unit-stencil form of sor_point for rows whose coefficients are exactly
// (a1,a2,a3,a4,a5) = (1,1,-4,1,1) -- every row of a uniform grid whose
// spacing is a power of two.  1*x == x and x/(-4) == x*(-0.25) hold bit for
// bit in IEEE double (exact scaling), and with sorrel == 1 the relaxation
// p + 1*sum == p + sum, so this is the same arithmetic in 7 FP64 operations
// instead of 12 plus a division.
__device__ __forceinline__ double sor_point_unit(const Dev &d, double *p, int i, int j) {
  const size_t o = IX(d, i, j);
  double sum = d.pb[o] - p[IX(d, i, j - 1)] - p[IX(d, i - 1, j)] - p[IX(d, i + 1, j)] -
               p[IX(d, i, j + 1)];
  sum = sum * -0.25 - p[o];
  p[o] = p[o] + sum;
  return sum;
}

// Red/black colour sweep over (i+j) % 2 == parity, pressure.f:505-532.
template <bool UNIT>
__device__ double rb_color(const Dev &d, double *p, int parity, double sorrel) {
  const int nx = d.nx, ny = d.ny;
  const int nh = (nx - 2) / 2 + 1;  // points per row of one colour (max)
  // max of |delta| >= 0 kept as IEEE bit patterns: integer compares, same
  // order as the doubles, and no FP64 pipe slot
  unsigned long long mx = 0ull;
  for (int t = gtid(); t < nh * (ny - 1); t += gthreads()) {
    const int j = t / nh + 2;
    const int i = 2 + ((j + parity) & 1) + 2 * (t % nh);
    if (i > nx) continue;
    const double a = UNIT ? sor_point_unit(d, p, i, j) : sor_point(d, p, i, j, sorrel);
    const unsigned long long b = abs_bits(a);
    mx = b > mx ? b : mx;
  }
  return __longlong_as_double((long long)mx);
}

// ---- line solves along i (ndir = 1) ------------------------------------
// Line nl = j: unknowns p(2..nx, j), aline = (a2, a3, a4), bline = b -
// (a1 p(i,j-1) + a5 p(i,j+1)); AltTridLU with the first-row quirk.
// Writes the solved line to p; when `relax` the reference's in-line
// over-relaxation (pressure.f:933-939) is applied and max|delta| returned.
__device__ double line_solve(const Dev &d, double *p, int j, double sorrel, bool relax) {
  const int nx = d.nx, n = nx - 1;
  double *a3p = d.la3p + IX(d, 0, j), *bp = d.lbp + IX(d, 0, j);
#define BL(i) (d.pb[IX(d, i, j)] - (d.pa1[IX(d, i, j)] * p[IX(d, i, j - 1)] + \
                                    d.pa5[IX(d, i, j)] * p[IX(d, i, j + 1)]))
  // row 1 (i = 2): quirk a3'(1) = a3(1) / a2(2)
  double s3 = d.pa4[IX(d, 2, j)] / d.pa3[IX(d, 3, j)];
  double sb = BL(2) / d.pa3[IX(d, 2, j)];
  a3p[2] = s3;
  bp[2] = sb;
  for (int k = 2; k <= n; ++k) {
    const int i = k + 1;
    const size_t o = IX(d, i, j);
    const double a1 = d.pa2[o];
    const double a2p = d.pa3[o] - a1 * s3;
    const double nb = (BL(i) - a1 * sb) / a2p;
    if (k < n) s3 = d.pa4[o] / a2p;
    sb = nb;
    a3p[i] = s3;
    bp[i] = sb;
  }
#undef BL
  // back substitution into bp (x), then relaxation
  double xn = bp[nx];
  for (int i = nx - 1; i >= 2; --i) {
    xn = bp[i] - a3p[i] * xn;
    bp[i] = xn;
  }
  double mx = 0.0;
  for (int i = 2; i <= nx; ++i) {
    const size_t o = IX(d, i, j);
    if (relax) {
      const double old = p[o];
      double sum = bp[i] - old;
      p[o] = old + sorrel * sum;
      mx = dmax(mx, fabs(sum));
    } else {
      p[o] = bp[i];
    }
  }
  return mx;
}

// Lexicographic point SOR by one block (Sor, pressure.f:384-450).
// Thread t owns rows 2+t, 2+t+T, ...; at step s it updates column
// i = s - j + 4 of each of its rows, so (i,j-1) and (i-1,j) are already new
// and (i+1,j), (i,j+1) still old -- the exact sequential order.
__device__ int sor_lex_block(const Dev &d, double *p, int lcartes, int msorit, double dk,
                             double sortol, double sorrel) {
  const int nx = d.nx, ny = d.ny;
  __shared__ double red[32];
  for (int it = 1; it <= msorit; ++it) {
    if (!lcartes) {
      ppe_rhs_block(d, lcartes, dk, p);
      __syncthreads();
    }
    double mx = 0.0;
    const int nsteps = (nx - 2) + (ny - 2) + 1;
    for (int s = 0; s < nsteps; ++s) {
      for (int j = 2 + (int)threadIdx.x; j <= ny; j += blockDim.x) {
        const int i = s - j + 4;
        if (i >= 2 && i <= nx) mx = dmax(mx, fabs(sor_point(d, p, i, j, sorrel)));
      }
      __syncthreads();
    }
    // block max
    for (int o = 16; o > 0; o >>= 1) mx = dmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    double dif = 0.0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) dif = dmax(dif, red[w]);
    __syncthreads();
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

// Slor (2), lines in order, by thread 0 of one block.
__device__ int slor_block(const Dev &d, double *p, int lcartes, int msorit, double dk,
                          double sortol, double sorrel) {
  __shared__ double difsh;
  for (int it = 1; it <= msorit; ++it) {
    if (!lcartes) {
      ppe_rhs_block(d, lcartes, dk, p);
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      double dif = 0.0;
      for (int j = 2; j <= d.ny; ++j) dif = dmax(dif, line_solve(d, p, j, sorrel, true));
      difsh = dif;
    }
    __syncthreads();
    const double dif = difsh;
    __syncthreads();
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

// Multi-block solvers: returns nConv (0 = not converged) or -1 on error.
__device__ int ppe_parallel(const Dev &d, double *p, int npsolver, int lcartes, int msorit,
                            double dk, double sortol, double sorrel) {
  Sync *sy = d.sync;
  const int nx = d.nx, ny = d.ny;
  for (int it = 1; it <= msorit; ++it) {
    unsigned long long *slot = &sy->red[3 + it % 3];
    if (vblock() == 0 && threadIdx.x == 0) {
      if (it == 1) sy->red[3 + 1] = 0ull;
      sy->red[3 + (it + 1) % 3] = 0ull;
    }
    if (npsolver == 5 || npsolver == 6) {
      if (!lcartes) {
        ppe_rhs_grid(d, lcartes, dk, p);
        if (!grid_sync(sy)) return -1;
      }
      const bool unit = d.ppe_unit && sorrel == 1.0;
      double mx = unit ? rb_color<true>(d, p, 0, sorrel) : rb_color<false>(d, p, 0, sorrel);
      if (!grid_sync(sy)) return -1;
      mx = dmax(mx, unit ? rb_color<true>(d, p, 1, sorrel) : rb_color<false>(d, p, 1, sorrel));
      block_max_to(slot, mx);
      if (!grid_sync(sy)) return -1;
    } else if (npsolver == 3) {
      // SlorRB: colour k = 2 (lines 2,4,..) then k = 3 (lines 3,5,..)
      double mx = 0.0;
      for (int k = 2; k <= 3; ++k) {
        if (!lcartes) {
          ppe_rhs_grid(d, lcartes, dk, p);
          if (!grid_sync(sy)) return -1;
        }
        const int nl = (ny - k) / 2 + 1;
        for (int t = gtid(); t < nl; t += gthreads()) mx = dmax(mx, line_solve(d, p, k + 2 * t, sorrel, true));
        if (!grid_sync(sy)) return -1;
      }
      block_max_to(slot, mx);
      if (!grid_sync(sy)) return -1;
    } else if (npsolver == 4) {
      // SlorRBP: pn = p over (1..nx,1..ny); solve colour, relax colour
      for (int t = gtid(); t < nx * ny; t += gthreads()) {
        const int i = t % nx + 1, j = t / nx + 1;
        d.ppn[IX(d, i, j)] = p[IX(d, i, j)];
      }
      if (!grid_sync(sy)) return -1;
      for (int k = 2; k <= 3; ++k) {
        if (!lcartes) {
          ppe_rhs_grid(d, lcartes, dk, p);
          if (!grid_sync(sy)) return -1;
        }
        const int nl = (ny - k) / 2 + 1;
        for (int t = gtid(); t < nl; t += gthreads()) line_solve(d, p, k + 2 * t, sorrel, false);
        if (!grid_sync(sy)) return -1;
        for (int t = gtid(); t < nl * (nx - 1); t += gthreads()) {
          const int j = k + 2 * (t / (nx - 1)), i = t % (nx - 1) + 2;
          const size_t o = IX(d, i, j);
          p[o] = d.ppn[o] + sorrel * (p[o] - d.ppn[o]);
        }
        if (!grid_sync(sy)) return -1;
      }
      double mx = 0.0;
      for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
        const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
        const size_t o = IX(d, i, j);
        mx = dmax(mx, fabs(d.ppn[o] - p[o]));
      }
      block_max_to(slot, mx);
      if (!grid_sync(sy)) return -1;
    } else {
      return 0;
    }
    const double dif = slot_value(slot);
    if (it > 1 && dif < sortol) return it;
  }
  return 0;
}

}  // namespace w2
