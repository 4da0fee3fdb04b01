// w2_ppe_tiled.cuh -- red/black point SOR (SorRB/SorRBP, pressure.f:457-656)
// with two sweeps per grid barrier, for unit-stencil rows.
//
// Each block owns a rectangular tile of the unknowns p(2..nx, 2..ny) and
// stages the tile plus a halo of H = 2*K cells (K = sweeps per barrier) of
// p and b in shared memory.  Within a group of K sweeps it runs the colour
// half-sweeps on shrinking boxes around the tile -- black on the tile grown
// by H-1, red on H-2, black on H-3, ... -- so every half-sweep on the box it
// covers sees exactly the neighbour values the global sweep would: the halo
// cells are recomputed redundantly from the same inputs with the same
// arithmetic.  p is double-buffered in global memory (a group reads one
// buffer and writes the other), so tiles never see a neighbour's partial
// update.  The per-sweep maximum of |delta| is taken over each tile's own
// points and combined across blocks, and the reference's stopping rule
// (m > 1 and dif < sortol) is evaluated sweep by sweep after the barrier;
// when it fires on the first sweep of a group, the state saved after that
// sweep is the answer.  Results are bit-identical to one global sweep at a
// time.
#pragma once
#include "w2_ppe.cuh"

namespace w2 {

constexpr int kSweepsPerSync = 2;
constexpr int kHalo = 2 * kSweepsPerSync;

struct TileGeom {
  int tx, ty;    // tile size in unknowns
  int ntx, nty;  // tiles per direction
  double one, mone;  // 1 and -1, given at launch (see tile_half_sweep)
};

// x * -0.25, exactly: for x normal with an exponent field >= 3 the product is
// x with its sign flipped and 2 taken from its exponent field, done on the
// integer pipe; a zero flips its sign; everything else (products that would
// be subnormal, infinities, NaN) takes the FP64 multiply.
__device__ __forceinline__ double mul_neg_quarter(double x) {
  const unsigned long long b = dbits(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - 3u < 2044u)
    return __longlong_as_double((long long)((b ^ 0x8000000000000000ull) - (2ull << 52)));
  if ((b & 0x7fffffffffffffffull) == 0ull) return __longlong_as_double((long long)(b ^ 0x8000000000000000ull));
  return x * -0.25;
}

// Half-sweep of one colour over box [bi0,bi1] x [bj0,bj1] (grid indices,
// already clipped to the unknowns) of the shared tile (origin gi0, gj0,
// row length W).  The colour's points are numbered row by row; thread t takes
// points t, t+T, t+2T, ... in batches of four whose operands are all loaded
// before any is updated (points of one colour never read each other), and the
// row/column of the next point is advanced incrementally.  Returns max
// |delta| (as IEEE bits) over points inside the own tile.  RELAX: the
// update is p + sorrel*sum (pressure.f:531); without it sorrel is 1 and
// 1*sum == sum bit for bit, so the product is left out.
// The FP64 pipe bounds this loop.  Every addition and subtraction is issued
// as a fused multiply-add with a factor of +1 or -1 (one = 1, mone = -1,
// launch parameters the compiler cannot fold): x*(+-1) is exact, so
// fma(x, -1, y) rounds exactly as y - x and fma(x, 1, y) as y + x, and the
// GB300 issues FP64 FMAs at a higher rate than FP64 adds.  The product by
// -1/4 is an exponent edit (mul_neg_quarter).
template <bool RELAX, int NB>
__device__ __forceinline__ unsigned long long tile_half_sweep(
    double *P, const double *Bt, int W, int gi0, int gj0, int bi0, int bi1, int bj0, int bj1,
    int parity, int oi0, int oi1, int oj0, int oj1, double relax, double one, double mone) {
  unsigned long long mx = 0ull;
  const int rows = bj1 - bj0 + 1;
  if (rows <= 0 || bi1 < bi0) return 0ull;
  const int wmax = (bi1 - bi0) / 2 + 1;  // slots per row (last may be empty)
  const int total = rows * wmax;
  const int T = blockDim.x;
  const int dj = T / wmax, dk = T % wmax;
  int t = threadIdx.x;
  int j = bj0 + t / wmax, k = t % wmax;
  while (t < total) {
    int o[NB];
    bool ok[NB], own[NB];
    double b[NB], s_[NB], w_[NB], e_[NB], n_[NB], c_[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int i = bi0 + 2 * k + (((bi0 + j + parity) & 1));
      ok[q] = (t < total) && (i <= bi1);
      own[q] = ok[q] && i >= oi0 && i <= oi1 && j >= oj0 && j <= oj1;
      o[q] = ok[q] ? (i - gi0) + (j - gj0) * W : W + 1;
      t += T;
      k += dk;
      j += dj;
      if (k >= wmax) {
        k -= wmax;
        ++j;
      }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      b[q] = Bt[o[q]];
      s_[q] = P[o[q] - W];
      w_[q] = P[o[q] - 1];
      e_[q] = P[o[q] + 1];
      n_[q] = P[o[q] + W];
      c_[q] = P[o[q]];
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      // sum = b - s - w - e - n; sum = sum / a3 - c (a3 = -4); p = c + sorrel * sum
      double sum = __fma_rn(s_[q], mone, b[q]);
      sum = __fma_rn(w_[q], mone, sum);
      sum = __fma_rn(e_[q], mone, sum);
      sum = __fma_rn(n_[q], mone, sum);
      sum = __fma_rn(c_[q], mone, mul_neg_quarter(sum));
      if (ok[q]) P[o[q]] = RELAX ? __fma_rn(relax * sum, one, c_[q]) : __fma_rn(sum, one, c_[q]);
      if (own[q]) {
        const unsigned long long bb = abs_bits(sum);
        mx = bb > mx ? bb : mx;
      }
    }
  }
  return mx;
}

// One group of up to K sweeps on every tile this block owns: read pin,
// write pout (and pmid after the first sweep), record per-sweep maxima.
// NB points of a thread are in flight at once.
template <bool RELAX, int NB>
__device__ void tiled_group(const Dev &d, const TileGeom &g, const double *pin, double *pout,
                            double *pmid, int nsweeps, unsigned long long *slots, double relax) {
  extern __shared__ double smem[];
  const int W = g.tx + 2 * kHalo, Hh = g.ty + 2 * kHalo;
  double *P = smem, *Bt = smem + W * Hh;
  __shared__ unsigned long long red[kSweepsPerSync][32];
  const int ntiles = g.ntx * g.nty;
  for (int tile = vblock(); tile < ntiles; tile += vblocks()) {
    const int ti = tile % g.ntx, tj = tile / g.ntx;
    const int oi0 = 2 + ti * g.tx, oj0 = 2 + tj * g.ty;
    const int oi1 = min(d.nx, oi0 + g.tx - 1), oj1 = min(d.ny, oj0 + g.ty - 1);
    const int gi0 = oi0 - kHalo, gj0 = oj0 - kHalo;
    // stage p and b on the box grown by H, clipped to the stored field
    for (int t = threadIdx.x; t < W * Hh; t += blockDim.x) {
      const int i = gi0 + t % W, j = gj0 + t / W;
      if (i >= 0 && i <= d.nx + 1 && j >= 0 && j <= d.ny + 1) {
        const size_t o = IX(d, i, j);
        P[t] = pin[o];
        Bt[t] = d.pb[o];
      }
    }
    __syncthreads();
    unsigned long long mxs[kSweepsPerSync];
    for (int s = 0; s < kSweepsPerSync; ++s) mxs[s] = 0ull;
    for (int s = 0; s < nsweeps; ++s) {
      for (int c = 0; c < 2; ++c) {
        const int e = kHalo - 1 - 2 * s - c;  // box growth for this half-sweep
        const int bi0 = max(2, oi0 - e), bi1 = min(d.nx, oi1 + e);
        const int bj0 = max(2, oj0 - e), bj1 = min(d.ny, oj1 + e);
        const unsigned long long m = tile_half_sweep<RELAX, NB>(P, Bt, W, gi0, gj0, bi0, bi1, bj0, bj1,
                                                            c, oi0, oi1, oj0, oj1, relax, g.one,
                                                            g.mone);
        mxs[s] = m > mxs[s] ? m : mxs[s];
        __syncthreads();
      }
      if (s == 0 && nsweeps > 1 && pmid != nullptr) {
        for (int t = threadIdx.x; t < (oi1 - oi0 + 1) * (oj1 - oj0 + 1); t += blockDim.x) {
          const int w = oi1 - oi0 + 1;
          const int i = oi0 + t % w, j = oj0 + t / w;
          pmid[IX(d, i, j)] = P[(i - gi0) + (j - gj0) * W];
        }
      }
    }
    for (int t = threadIdx.x; t < (oi1 - oi0 + 1) * (oj1 - oj0 + 1); t += blockDim.x) {
      const int w = oi1 - oi0 + 1;
      const int i = oi0 + t % w, j = oj0 + t / w;
      pout[IX(d, i, j)] = P[(i - gi0) + (j - gj0) * W];
    }
    // block max per sweep -> global slots
    for (int s = 0; s < nsweeps; ++s) {
      unsigned long long b = mxs[s];
      for (int o = 16; o > 0; o >>= 1) {
        unsigned long long t2 = __shfl_down_sync(0xffffffffu, b, o);
        b = t2 > b ? t2 : b;
      }
      if ((threadIdx.x & 31) == 0) red[s][threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      const int nw = (blockDim.x + 31) >> 5;
      for (int s = 0; s < nsweeps; ++s) {
        unsigned long long b = threadIdx.x < nw ? red[s][threadIdx.x] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
          unsigned long long t2 = __shfl_down_sync(0xffffffffu, b, o);
          b = t2 > b ? t2 : b;
        }
        if (threadIdx.x == 0 && b) atomicMax(&slots[s], b);
      }
    }
    __syncthreads();
  }
}

// Red/black SOR by groups of K sweeps.  p is the caller's field; pb2 and pm
// are scratch fields.  Returns nConv (0 = not converged) or -1 on error.
template <int NB>
__device__ int ppe_rb_tiled(const Dev &d, const TileGeom &g, double *p, double *p2, double *pm,
                            int msorit, double sortol, double sorrel) {
  Sync *sy = d.sync;
  const int W = d.nx + 2, H = d.ny + 2;
  // scratch buffers start as copies of p (ghost values included)
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const size_t o = IX(d, t % W, t / W);
    p2[o] = p[o];
    pm[o] = p[o];
  }
  double *bufs[2] = {p, p2};
  int cur = 0, result = 0;
  double *final_src = p;
  // per-sweep maxima: a ring of three groups of K slots.  Group g uses slot
  // set g % 3 and, before its barrier, clears set (g+1) % 3 -- last read by
  // every block before group g-1's barrier -- so one barrier per group
  // orders both the clear and the reads.
  unsigned long long *ring = &sy->red[10];
  if (vblock() == 0 && threadIdx.x == 0)
    for (int k = 0; k < 3 * kSweepsPerSync; ++k) ring[k] = 0ull;
  if (!grid_sync(sy)) return -1;
  int grp = 0;
  for (int m0 = 1; m0 <= msorit; m0 += kSweepsPerSync, ++grp) {
    const int ns = min(kSweepsPerSync, msorit - m0 + 1);
    unsigned long long *slots = ring + (grp % 3) * kSweepsPerSync;
    if (vblock() == 0 && threadIdx.x == 0) {
      unsigned long long *next = ring + ((grp + 1) % 3) * kSweepsPerSync;
      for (int k = 0; k < kSweepsPerSync; ++k) next[k] = 0ull;
    }
    if (sorrel == 1.0)
      tiled_group<false, NB>(d, g, bufs[cur], bufs[cur ^ 1], pm, ns, slots, sorrel);
    else
      tiled_group<true, NB>(d, g, bufs[cur], bufs[cur ^ 1], pm, ns, slots, sorrel);
    if (!grid_sync(sy)) return -1;
    int conv_s = -1;
    for (int s2 = 0; s2 < ns; ++s2) {
      const int m = m0 + s2;
      const double dif = slot_value(&slots[s2]);
      if (m > 1 && dif < sortol) {
        conv_s = s2;
        result = m;
        break;
      }
    }
    cur ^= 1;
    final_src = (conv_s >= 0 && conv_s < ns - 1) ? pm : bufs[cur];
    if (conv_s >= 0) break;
  }
  if (final_src != p) {
    for (int t = gtid(); t < (d.nx - 1) * (d.ny - 1); t += gthreads()) {
      const int i = t % (d.nx - 1) + 2, j = t / (d.nx - 1) + 2;
      p[IX(d, i, j)] = final_src[IX(d, i, j)];
    }
  }
  if (!grid_sync(sy)) return -1;
  return result;
}

}  // namespace w2
