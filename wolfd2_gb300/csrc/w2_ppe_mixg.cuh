// w2_ppe_mixg.cuh -- mixed-precision Ppe with the grid's own Poisson rows:
// the red/black point iteration of SorRB/SorRBP (pressure.f:457-656) in FP32
// on the correction equation, for every grid the unit-stencil kernel
// (w2_ppe_mixed.cuh) does not take -- cells of any shape and spacing, the
// identity rows of blockages (pressure.f:109-196) and, with lcartes = 0,
// curvilinear grids whose right-hand side carries RhsPpe's cross terms
// (pressure.f:360-375).
//
// A refinement pass forms r = RhsPpe(p) - A p in FP64 with the rows a1..a5
// of pressure.f:97-196, relaxes A e = r from e = 0 in FP32 with the rows
// rounded to FP32 (c_k = (float)a_k) and adds e to p in FP64.  A sweep
// first forms r' = r - (cross terms of e, FP32) when lcartes = 0 -- the
// reference forms its right-hand side once per sweep from the current p --
// then updates the black points, then the red ones:
//   s = r' - c1 eS - c2 eW - c4 eE - c5 eN;  s = s * (1/c3) - e;  e = e + sorrel s
// with max |s| as the sweep's dif, 1/c3 the FP32 reciprocal of the rounded
// diagonal, formed once with the coefficients (the reference divides; the
// product is one rounding of a slightly different FP32 operator, and the
// next pass's FP64 residual corrects it like any FP32 error).  Sweep counts,
// the stopping rule (sweep m > 1 and dif < sortol) and the pass lengths are
// those of the unit-stencil kernel; on unit rows every operation rounds as
// the unit form does (1 x == x, 1/-4 == -0.25 exactly).
//
// Layout: colour-split FP32 planes in global memory (they stay in L2: 8
// floats a cell, each in the plane of the cell's colour).  Cell (i, j) lives in the plane of its colour (i+j)&1 at
// j*gw + (i >> 1), so the points of one colour in a row are contiguous and
// a point's east/west neighbours are the other plane's entries k and k-1 or
// k+1.  Cells off the unknowns hold e = 0 (the ghost pressures stay frozen
// during the iteration, so their correction is zero) and are never written.
// One grid barrier separates the colours, one ends the sweep (and, with
// lcartes = 0, one follows the cross-term pass).  Single cases on Cartesian
// grids run the tiled form at the end of this file by default, K sweeps
// per grid barrier; ensembles run this form on every general-row case.
#pragma once
#include "w2_ppe.cuh"
#include "w2_ppe_mixed.cuh"

namespace w2 {

// Plane indices (each a pair: colour 0, colour 1).
enum : int { MG_E = 0, MG_R = 2, MG_RR = 4, MG_C1 = 6, MG_C2 = 8, MG_C3 = 10, MG_C4 = 12,
             MG_C5 = 14, MG_PLANES = 16 };

struct MixgArgs {
  int lcartes, msorit, inner;  // inner: FP32 sweeps per refinement pass
  double dk, sortol;
  float relax;                 // sorrel
  const double *u, *v;
  double *p;
  float *buf;                  // MG_PLANES planes of gw x (ny + 2) floats
  int gw;                      // floats per plane row (a multiple of 32)
  const float *rbu, *rbv;      // FP32 rbu, rbv in field layout (lcartes = 0)
};

__host__ __device__ inline int mixg_gw(int nx) { return ((nx + 1) / 2 + 1 + 31) / 32 * 32; }

__device__ __forceinline__ float *mixg_plane(const MixgArgs &a, int ny, int q) {
  return a.buf + (size_t)q * a.gw * (ny + 2);
}
__device__ __forceinline__ int mixg_pos(const MixgArgs &a, int i, int j) { return j * a.gw + (i >> 1); }

// The rows rounded to FP32 into the coefficient planes, the diagonal as its
// FP32 reciprocal (every unknown; the planes' other cells stay as the
// allocation's zeros).
__device__ void mixg_coefficients(const Dev &d, const MixgArgs &a) {
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const int c = (i + j) & 1, x = mixg_pos(a, i, j);
    mixg_plane(a, ny, MG_C1 + c)[x] = (float)d.pa1[o];
    mixg_plane(a, ny, MG_C2 + c)[x] = (float)d.pa2[o];
    mixg_plane(a, ny, MG_C3 + c)[x] = 1.0f / (float)d.pa3[o];
    mixg_plane(a, ny, MG_C4 + c)[x] = (float)d.pa4[o];
    mixg_plane(a, ny, MG_C5 + c)[x] = (float)d.pa5[o];
  }
}

// r = RhsPpe(p) - A p in FP64 on the unknowns (the divergence in d.div),
// rounded into the r planes; e = 0.  A p in mixed_ap's order.
__device__ void mixg_residual(const Dev &d, const MixgArgs &a) {
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const double bb = rhs_point(d, a.lcartes, a.dk, a.p, i, j);
    const double ap = d.pa1[o] * a.p[o - d.ld] + d.pa2[o] * a.p[o - 1] + d.pa4[o] * a.p[o + 1] +
                      d.pa5[o] * a.p[o + d.ld] + d.pa3[o] * a.p[o];
    const int c = (i + j) & 1, x = mixg_pos(a, i, j);
    mixg_plane(a, ny, MG_R + c)[x] = (float)(bb - ap);
    mixg_plane(a, ny, MG_E + c)[x] = 0.0f;
  }
}

// p += e on the unknowns, FP64.
__device__ void mixg_correct(const Dev &d, const MixgArgs &a) {
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    a.p[o] = a.p[o] + (double)mixg_plane(a, ny, MG_E + ((i + j) & 1))[mixg_pos(a, i, j)];
  }
}

// lcartes = 0: r' = r - the cross terms of e (RhsPpe's form, pressure.f:
// 360-375, in FP32 with rbu, rbv rounded to FP32) into the r' planes, in
// batches of kMixgBatch points whose loads all issue before any store.
constexpr int kMixgBatch = 4;

__device__ void mixg_cross(const Dev &d, const MixgArgs &a) {
  const int nx = d.nx, ny = d.ny, n = (nx - 1) * (ny - 1), T = gthreads();
  const float *__restrict__ E0 = mixg_plane(a, ny, MG_E);
  const float *__restrict__ E1 = mixg_plane(a, ny, MG_E + 1);
  const float *__restrict__ rbu = a.rbu;
  const float *__restrict__ rbv = a.rbv;
  auto e = [&](int i, int j) { return ((i + j) & 1 ? E1 : E0)[mixg_pos(a, i, j)]; };
  for (int t0 = gtid(); t0 < n; t0 += kMixgBatch * T) {
    float x[kMixgBatch];
    int i[kMixgBatch], j[kMixgBatch];
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      const int t = min(t0 + q * T, n - 1);
      i[q] = t % (nx - 1) + 2;
      j[q] = t / (nx - 1) + 2;
      const size_t o = IX(d, i[q], j[q]);
      const int ii = i[q], jj = j[q];
      x[q] = rbu[o] * (e(ii + 1, jj + 1) + e(ii, jj + 1) - e(ii + 1, jj - 1) - e(ii, jj - 1)) -
             rbu[o - 1] * (e(ii, jj + 1) + e(ii - 1, jj + 1) - e(ii, jj - 1) - e(ii - 1, jj - 1)) +
             rbv[o] * (e(ii + 1, jj + 1) + e(ii + 1, jj) - e(ii - 1, jj + 1) - e(ii - 1, jj)) -
             rbv[o - d.ld] * (e(ii + 1, jj) + e(ii + 1, jj - 1) - e(ii - 1, jj) - e(ii - 1, jj - 1));
    }
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      if (t0 + q * T >= n) break;
      const int c = (i[q] + j[q]) & 1, p = mixg_pos(a, i[q], j[q]);
      mixg_plane(a, ny, MG_RR + c)[p] = mixg_plane(a, ny, MG_R + c)[p] - x[q];
    }
  }
}

// Half-sweep of colour c: row j's points of that colour sit at i = 2k + par
// (par = (c + j) & 1, k = 1 .. (nx - par) / 2), their west/east neighbours
// at the other plane's k - 1 + par and k + par, north/south at k one row up
// or down.  A thread takes kMixgBatch points at a time and loads all their
// operands before it updates any (points of one colour never read each
// other), so their L2 round trips overlap; a point past the end reads the
// plane's cell (1, 1) and writes nothing.  Returns max |s| as IEEE bits.
__device__ unsigned int mixg_half(const Dev &d, const MixgArgs &a, int c, float relax) {
  const int nx = d.nx, ny = d.ny, nk = nx >> 1, gw = a.gw, total = nk * (ny - 1), T = gthreads();
  const float *__restrict__ R = mixg_plane(a, ny, (a.lcartes ? MG_R : MG_RR) + c);
  const float *__restrict__ C1 = mixg_plane(a, ny, MG_C1 + c);
  const float *__restrict__ C2 = mixg_plane(a, ny, MG_C2 + c);
  const float *__restrict__ C3 = mixg_plane(a, ny, MG_C3 + c);
  const float *__restrict__ C4 = mixg_plane(a, ny, MG_C4 + c);
  const float *__restrict__ C5 = mixg_plane(a, ny, MG_C5 + c);
  const float *__restrict__ Eo = mixg_plane(a, ny, MG_E + (c ^ 1));
  float *__restrict__ Ec = mixg_plane(a, ny, MG_E + c);
  unsigned int mx = 0u;
  // (j, k) of point t, advanced by T points at a time without a division
  const int dj = T / nk, dk = T % nk;
  int t = gtid(), j = 2 + t / nk, k = 1 + t % nk;
  while (t < total) {
    int x[kMixgBatch], par[kMixgBatch];
    bool ok[kMixgBatch];
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      par[q] = (c + j) & 1;
      ok[q] = t < total && 2 * k + par[q] <= nx;
      x[q] = ok[q] ? j * gw + k : gw + 1;
      if (!ok[q]) par[q] = 0;
      t += T;
      k += dk;
      j += dj;
      if (k > nk) {
        k -= nk;
        ++j;
      }
    }
    float r[kMixgBatch], c1[kMixgBatch], c2[kMixgBatch], c3[kMixgBatch], c4[kMixgBatch], c5[kMixgBatch];
    float e0[kMixgBatch], es[kMixgBatch], ew[kMixgBatch], ee[kMixgBatch], en[kMixgBatch];
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      r[q] = R[x[q]];
      c1[q] = C1[x[q]];
      c2[q] = C2[x[q]];
      c3[q] = C3[x[q]];
      c4[q] = C4[x[q]];
      c5[q] = C5[x[q]];
      e0[q] = Ec[x[q]];
      es[q] = Eo[x[q] - gw];
      ew[q] = Eo[x[q] - 1 + par[q]];
      ee[q] = Eo[x[q] + par[q]];
      en[q] = Eo[x[q] + gw];
    }
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      float s = r[q] - c1[q] * es[q];
      s = s - c2[q] * ew[q];
      s = s - c4[q] * ee[q];
      s = s - c5[q] * en[q];
      s = s * c3[q];
      s = s - e0[q];
      if (ok[q]) {
        Ec[x[q]] = e0[q] + relax * s;
        const unsigned int b = __float_as_uint(s) & 0x7fffffffu;
        mx = b > mx ? b : mx;
      }
    }
  }
  return mx;
}

// Block max of FP32 bit patterns into a slot holding double bits.
__device__ __forceinline__ void mixg_block_max(unsigned int v, unsigned long long *slot) {
  __shared__ unsigned int wm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = __reduce_max_sync(0xffffffffu, v);
  if (lane == 0) wm[w] = v;
  __syncthreads();
  if (w == 0) {
    v = __reduce_max_sync(0xffffffffu, lane < nw ? wm[lane] : 0u);
    if (lane == 0 && v) atomicMax(slot, (unsigned long long)__double_as_longlong((double)__uint_as_float(v)));
  }
  __syncthreads();
}

// The whole Ppe: Divergence (blockage cells zeroed), then refinement passes
// until the stopping rule fires or msorit sweeps are done.  Returns nConv
// (0 = not converged) or -1 on a barrier error.  The per-sweep maxima use the
// PPE ring red[3..5]: sweep m writes slot m % 3 and, before its first
// barrier, block 0 clears slot (m + 1) % 3, which every block read before
// the barriers of sweep m - 1.
__device__ int ppe_mixg(const Dev &d, const MixgArgs &a) {
  Sync *sy = d.sync;
  unsigned long long *ring = &sy->red[3];
  if (vblock() == 0 && threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) ring[k] = 0ull;
  ppe_divergence(d, a.u, a.v);
  if (!grid_sync(sy)) return -1;
  int m = 0, result = 0;
  bool done = false;
  while (!done) {
    mixg_residual(d, a);
    if (!grid_sync(sy)) return -1;
    int in_pass = 0;
    while (true) {
      ++m;
      unsigned long long *slot = ring + m % 3;
      if (vblock() == 0 && threadIdx.x == 0) ring[(m + 1) % 3] = 0ull;
      if (!a.lcartes) {
        mixg_cross(d, a);
        if (!grid_sync(sy)) return -1;
      }
      unsigned int mx = mixg_half(d, a, 0, a.relax);
      if (!grid_sync(sy)) return -1;
      const unsigned int m1 = mixg_half(d, a, 1, a.relax);
      mx = m1 > mx ? m1 : mx;
      mixg_block_max(mx, slot);
      if (!grid_sync(sy)) return -1;
      if (m > 1 && slot_value(slot) < a.sortol) {
        result = m;
        done = true;
        break;
      }
      ++in_pass;
      if (m >= a.msorit) {
        done = true;
        break;
      }
      if (in_pass >= a.inner) break;
    }
    mixg_correct(d, a);
    if (!grid_sync(sy)) return -1;
  }
  return result;
}


// ---- tiled form (Cartesian grids) ------------------------------------------
// The same iteration on halo'd tiles in shared memory, K sweeps per grid
// barrier, as the plain tiled sweep does it (w2_ppe_tiled.cuh): each block
// stages, for every tile it owns, the tile grown by H = 2K cells of e, r and
// c1..c5 (natural (i, j) layout, FP32), runs the colour half-sweeps on
// boxes that shrink by one cell per half-sweep -- black on the tile grown
// by H-1, red on H-2, ... -- so that every point of the box it covers sees
// exactly the values a global sweep would, then writes its tile's e.  e is
// double-buffered in global memory between groups.  lcartes = 0 keeps the
// one-colour-per-barrier kernel above (its cross terms need e on the
// diagonals of every point at the start of each sweep).
constexpr int kMixgtK = 4;
constexpr int kMixgtH = 2 * kMixgtK;
constexpr int kMixgtThreads = 512;
constexpr int kMixgtPlanes = 7;  // e, r, c1..c5

struct MixgtGeom {
  int tx, ty;    // tile size in unknowns
  int ntx, nty;  // tiles per direction
};

struct MixgtArgs {
  int msorit, inner;
  double dk, sortol;
  float relax;
  const double *u, *v;
  double *p;
  const float *c[5];  // c1..c5 in field layout, zero off the unknowns
  float *r;           // r in field layout, zero off the unknowns
  float *e[2];        // e, double-buffered, zero off the unknowns
};

__host__ __device__ inline size_t mixgt_smem_bytes(int tx, int ty) {
  return (size_t)kMixgtPlanes * (tx + 2 * kMixgtH) * (ty + 2 * kMixgtH) * sizeof(float);
}

// r = RhsPpe(p) - A p (Cartesian: div/dk - A p) in FP64 on the unknowns.
__device__ void mixgt_residual(const Dev &d, const MixgtArgs &a) {
  const int nx = d.nx, ny = d.ny;
  for (int t = gtid(); t < (nx - 1) * (ny - 1); t += gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = IX(d, i, j);
    const double bb = rhs_point(d, 1, a.dk, a.p, i, j);
    const double ap = d.pa1[o] * a.p[o - d.ld] + d.pa2[o] * a.p[o - 1] + d.pa4[o] * a.p[o + 1] +
                      d.pa5[o] * a.p[o + d.ld] + d.pa3[o] * a.p[o];
    a.r[o] = (float)(bb - ap);
  }
}

// A tile's own unknowns and its box.
struct MixgtBox {
  int oi0, oi1, oj0, oj1;  // own tile, clipped to the unknowns
  int gi0, gj0, bw, bh;    // box origin and size
};

__device__ __forceinline__ MixgtBox mixgt_box(const Dev &d, const MixgtGeom &g, int tile) {
  MixgtBox b;
  const int ti = tile % g.ntx, tj = tile / g.ntx;
  b.oi0 = 2 + ti * g.tx;
  b.oj0 = 2 + tj * g.ty;
  b.oi1 = min(d.nx, b.oi0 + g.tx - 1);
  b.oj1 = min(d.ny, b.oj0 + g.ty - 1);
  b.gi0 = b.oi0 - kMixgtH;
  b.gj0 = b.oj0 - kMixgtH;
  b.bw = g.tx + 2 * kMixgtH;
  b.bh = g.ty + 2 * kMixgtH;
  return b;
}

// Stage the box: e from ein (zeros when ein is null), r, c1..c5; zeros
// outside the stored field.
__device__ void mixgt_stage(const Dev &d, const MixgtArgs &a, const MixgtBox &b, const float *ein,
                            float *S) {
  const int n = b.bw * b.bh, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const float *c1 = a.c[0], *c2 = a.c[1], *c3 = a.c[2], *c4 = a.c[3], *c5 = a.c[4], *r = a.r;
  for (int jj = threadIdx.x >> 5; jj < b.bh; jj += nw) {
    const int j = b.gj0 + jj;
    const bool jin = j >= 0 && j <= d.ny + 1;
    for (int ii = lane; ii < b.bw; ii += 32) {
      const int i = b.gi0 + ii, t = jj * b.bw + ii;
      const bool in = jin && i >= 0 && i <= d.nx + 1;
      const size_t o = in ? IX(d, i, j) : 0;
      S[t] = (in && ein) ? ein[o] : 0.0f;
      S[n + t] = in ? r[o] : 0.0f;
      S[2 * n + t] = in ? c1[o] : 0.0f;
      S[3 * n + t] = in ? c2[o] : 0.0f;
      S[4 * n + t] = in ? c3[o] : 0.0f;
      S[5 * n + t] = in ? c4[o] : 0.0f;
      S[6 * n + t] = in ? c5[o] : 0.0f;
    }
  }
}

// Half-sweep of colour c over the box [bi0,bi1] x [bj0,bj1] (clipped to the
// unknowns) of the staged planes; the colour's points numbered row by row,
// kMixgBatch of a thread's points loaded before any is updated.  Returns
// max |s| (IEEE bits) over the own tile's points.
__device__ unsigned int mixgt_half(float *S, const MixgtBox &b, int bi0, int bi1, int bj0, int bj1, int c,
                                   float relax) {
  unsigned int mx = 0u;
  const int rows = bj1 - bj0 + 1;
  if (rows <= 0 || bi1 < bi0) return 0u;
  const int n = b.bw * b.bh, bw = b.bw;
  float *E = S;
  const float *R = S + n, *C1 = S + 2 * n, *C2 = S + 3 * n, *C3 = S + 4 * n, *C4 = S + 5 * n,
              *C5 = S + 6 * n;
  const int wmax = (bi1 - bi0) / 2 + 1, total = rows * wmax, T = blockDim.x;
  // (j, k) of point t, advanced by T points at a time without a division
  const int dj = T / wmax, dk = T % wmax;
  int t = threadIdx.x, j = bj0 + t / wmax, k = t % wmax;
  while (t < total) {
    int x[kMixgBatch];
    bool ok[kMixgBatch], own[kMixgBatch];
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      const int i = bi0 + 2 * k + ((bi0 + j + c) & 1);
      ok[q] = t < total && i <= bi1;
      own[q] = ok[q] && i >= b.oi0 && i <= b.oi1 && j >= b.oj0 && j <= b.oj1;
      x[q] = ok[q] ? (i - b.gi0) + (j - b.gj0) * bw : bw + 1;
      t += T;
      k += dk;
      j += dj;
      if (k >= wmax) {
        k -= wmax;
        ++j;
      }
    }
    float r[kMixgBatch], c1[kMixgBatch], c2[kMixgBatch], c3[kMixgBatch], c4[kMixgBatch], c5[kMixgBatch];
    float e0[kMixgBatch], es[kMixgBatch], ew[kMixgBatch], ee[kMixgBatch], en[kMixgBatch];
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      r[q] = R[x[q]];
      c1[q] = C1[x[q]];
      c2[q] = C2[x[q]];
      c3[q] = C3[x[q]];
      c4[q] = C4[x[q]];
      c5[q] = C5[x[q]];
      e0[q] = E[x[q]];
      es[q] = E[x[q] - bw];
      ew[q] = E[x[q] - 1];
      ee[q] = E[x[q] + 1];
      en[q] = E[x[q] + bw];
    }
#pragma unroll
    for (int q = 0; q < kMixgBatch; ++q) {
      float s = r[q] - c1[q] * es[q];
      s = s - c2[q] * ew[q];
      s = s - c4[q] * ee[q];
      s = s - c5[q] * en[q];
      s = s * c3[q];
      s = s - e0[q];
      if (ok[q]) E[x[q]] = e0[q] + relax * s;
      if (own[q]) {
        const unsigned int bb = __float_as_uint(s) & 0x7fffffffu;
        mx = bb > mx ? bb : mx;
      }
    }
  }
  return mx;
}

// ns sweeps of every tile this block owns, from ein (null: e = 0) to eout;
// per-sweep maxima into slots (null: not recorded).
__device__ void mixgt_group(const Dev &d, const MixgtGeom &g, const MixgtArgs &a, int ns, const float *ein,
                            float *eout, unsigned long long *slots) {
  extern __shared__ __align__(16) float mgt_smem[];
  __shared__ unsigned int redm[kMixgtK][32];
  unsigned int mxs[kMixgtK];
#pragma unroll
  for (int s = 0; s < kMixgtK; ++s) mxs[s] = 0u;
  const int ntiles = g.ntx * g.nty;
  for (int tile = vblock(); tile < ntiles; tile += vblocks()) {
    const MixgtBox b = mixgt_box(d, g, tile);
    mixgt_stage(d, a, b, ein, mgt_smem);
    __syncthreads();
    for (int s = 0; s < ns; ++s) {
      for (int c = 0; c < 2; ++c) {
        const int grow = kMixgtH - 1 - 2 * s - c;
        const int bi0 = max(2, b.oi0 - grow), bi1 = min(d.nx, b.oi1 + grow);
        const int bj0 = max(2, b.oj0 - grow), bj1 = min(d.ny, b.oj1 + grow);
        const unsigned int m = mixgt_half(mgt_smem, b, bi0, bi1, bj0, bj1, c, a.relax);
#pragma unroll
        for (int q = 0; q < kMixgtK; ++q)
          if (q == s) mxs[q] = m > mxs[q] ? m : mxs[q];
        __syncthreads();
      }
    }
    const int tw = b.oi1 - b.oi0 + 1, th = b.oj1 - b.oj0 + 1;
    for (int t = threadIdx.x; t < tw * th; t += blockDim.x) {
      const int i = b.oi0 + t % tw, j = b.oj0 + t / tw;
      eout[IX(d, i, j)] = mgt_smem[(i - b.gi0) + (j - b.gj0) * b.bw];
    }
    __syncthreads();
  }
  if (!slots) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int s = 0; s < kMixgtK; ++s) {
    const unsigned int v = __reduce_max_sync(0xffffffffu, mxs[s]);
    if (lane == 0) redm[s][w] = v;
  }
  __syncthreads();
  if (w < ns) {
    const unsigned int v = __reduce_max_sync(0xffffffffu, lane < nw ? redm[w][lane] : 0u);
    if (lane == 0 && v)
      atomicMax(&slots[w], (unsigned long long)__double_as_longlong((double)__uint_as_float(v)));
  }
  __syncthreads();
}

// p += e on the own tiles of this block, FP64.
__device__ void mixgt_correct(const Dev &d, const MixgtGeom &g, const MixgtArgs &a, const float *e) {
  const int ntiles = g.ntx * g.nty;
  for (int tile = vblock(); tile < ntiles; tile += vblocks()) {
    const MixgtBox b = mixgt_box(d, g, tile);
    const int tw = b.oi1 - b.oi0 + 1, th = b.oj1 - b.oj0 + 1;
    for (int t = threadIdx.x; t < tw * th; t += blockDim.x) {
      const size_t o = IX(d, b.oi0 + t % tw, b.oj0 + t / tw);
      a.p[o] = a.p[o] + (double)e[o];
    }
  }
}

// The whole Ppe on tiles (Cartesian grids).  Per-sweep maxima in the ring
// red[kMixedRing ..] of three groups of kMixgtK slots: group q writes set
// q % 3 and, before its barrier, block 0 clears set (q + 1) % 3, last read
// by every block before the barrier of group q - 1.  When the stopping rule
// fires on sweep s < ns of a group, the group's input buffer is intact and
// the tiles are swept again from it for s + 1 sweeps.  Returns nConv (0 =
// not converged) or -1 on a barrier error.
__device__ int ppe_mixgt(const Dev &d, const MixgtGeom &g, const MixgtArgs &a) {
  Sync *sy = d.sync;
  unsigned long long *ring = &sy->red[kMixedRing];
  if (vblock() == 0 && threadIdx.x == 0)
    for (int k = 0; k < 3 * kMixgtK; ++k) ring[k] = 0ull;
  ppe_divergence(d, a.u, a.v);
  if (!grid_sync(sy)) return -1;
  int m = 0, result = 0, grp = 0;
  bool done = false;
  while (!done) {
    mixgt_residual(d, a);
    if (!grid_sync(sy)) return -1;
    int q = 0, in_pass = 0;
    const float *efinal = nullptr;
    while (true) {
      const int ns = min(kMixgtK, min(a.inner - in_pass, a.msorit - m));
      unsigned long long *slots = ring + (grp % 3) * kMixgtK;
      if (vblock() == 0 && threadIdx.x == 0) {
        unsigned long long *next = ring + ((grp + 1) % 3) * kMixgtK;
        for (int k = 0; k < kMixgtK; ++k) next[k] = 0ull;
      }
      const float *ein = q == 0 ? nullptr : a.e[(q + 1) & 1];
      float *eout = a.e[q & 1];
      mixgt_group(d, g, a, ns, ein, eout, slots);
      if (!grid_sync(sy)) return -1;
      int conv = -1;
      for (int s = 0; s < ns; ++s) {
        if (m + s + 1 > 1 && slot_value(&slots[s]) < a.sortol) {
          conv = s;
          break;
        }
      }
      ++grp;
      ++q;
      efinal = eout;
      if (conv >= 0) {
        result = m + conv + 1;
        if (conv < ns - 1) mixgt_group(d, g, a, conv + 1, ein, eout, nullptr);
        done = true;
        break;
      }
      m += ns;
      in_pass += ns;
      if (m >= a.msorit) {
        done = true;
        break;
      }
      if (in_pass >= a.inner) break;
    }
    mixgt_correct(d, g, a, efinal);
    if (!grid_sync(sy)) return -1;
  }
  return result;
}

}  // namespace w2
