// w2_ppe_mixed.cuh -- mixed-precision Ppe: the red/black point iteration of
// SorRB/SorRBP (pressure.f:457-656) run in FP32 on the correction equation,
// with the residual and the correction accumulated in FP64.
//
// One refinement pass forms r = b - A p in FP64 (b = div/dk from
// Divergence/RhsPpe, pressure.f:287-299 and 354-359), relaxes A e = r from
// e = 0 with the reference's point update -- black points (i+j even) first,
// then red, relaxation factor sorrel -- in FP32, and adds e to p in FP64.
// In exact arithmetic n sweeps on e followed by p += e are n sweeps on p, so
// the sweep count, the per-sweep maximum |delta| and the stopping rule
// (sweep m > 1 and dif < sortol, at most msorit sweeps, pressure.f:493-497)
// are the reference's; the rounding of the sweeps is FP32.  Each pass runs
// `inner` sweeps; every pass restarts e from an FP64 residual, so FP32
// rounding never accumulates beyond one pass.
//
// Layout.  Every block owns one tile of the unknowns (2..nx, 2..ny) and
// keeps in shared memory the tile grown by a halo of H = 2K cells, where K is
// the number of sweeps between grid barriers.  The box is stored as two
// colour planes (colour 0: i+j even) of hw = bw/2 entries per row, so the
// points of one colour are contiguous and every neighbour of a point is in
// the other plane at the same or the adjacent index: a warp's loads of one
// operand hit 32 consecutive words.  Within a group of K sweeps the
// half-sweeps run on shrinking boxes around the tile (grown by H-1, H-2, ...,
// 0), so the tile's own points see exactly the values a global sweep would.
// Between groups only the halo ring changes hands: each block writes the
// band of its tile within H of the edge to a global FP32 buffer and reads
// its ring from the neighbours' bands (two buffers, alternating by group).
#pragma once
#include "w2_ppe.cuh"

namespace w2 {

constexpr int kMixedMaxK = 8;
constexpr int kMixedRing = 17;  // Sync::red[17 .. 17 + 3K): per-sweep maxima

struct MixedGeom {
  int tx, ty;    // tile size in unknowns (tx even)
  int ntx, nty;  // tiles per direction, ntx*nty <= blocks
};

struct MixedArgs {
  int lcartes, msorit, inner;  // inner: FP32 sweeps per refinement pass
  double dk, sortol;
  float relax;                 // sorrel
  const double *u, *v;
  double *p;
  float *ebuf0, *ebuf1;        // band exchange, field layout
};

// A block's box: its tile grown by H, as two colour planes per array.
struct MixedBox {
  float *E[2], *E0[2], *R[2];
  int gi0, gj0, bw, bh, hw;
  int oi0, oi1, oj0, oj1;
  __device__ __forceinline__ int at(int i, int j) const {
    return (j - gj0) * hw + ((i - gi0) >> 1);
  }
  __device__ __forceinline__ bool own(int i, int j) const {
    return i >= oi0 && i <= oi1 && j >= oj0 && j <= oj1;
  }
};

// Half-sweep of one colour over the box [bi0,bi1] x [bj0,bj1] (grid
// indices, clipped to the unknowns).  Thread t takes the colour's points
// t, t+T, ... numbered row by row, four at a time with all loads issued
// before any update.  Returns max |delta| over the own tile as FP32 bits.
__device__ __forceinline__ unsigned int mixed_half_sweep(const MixedBox &b, int bi0, int bi1,
                                                         int bj0, int bj1, int colour,
                                                         float relax, bool track) {
  unsigned int mx = 0u;
  const int rows = bj1 - bj0 + 1;
  if (rows <= 0 || bi1 < bi0) return 0u;
  const int wmax = (bi1 - bi0) / 2 + 1;
  const int total = rows * wmax;
  const int T = blockDim.x;
  const int dj = T / wmax, dk = T % wmax;
  float *Ec = b.E[colour];
  const float *Eo = b.E[colour ^ 1];
  const float *Rc = b.R[colour];
  const int hw = b.hw;
  int t = threadIdx.x;
  int j = bj0 + t / wmax, k = t % wmax;
  constexpr int NB = 4;
  while (t < total) {
    int o[NB], par[NB];
    bool ok[NB], own[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int i = bi0 + 2 * k + ((bi0 + j + colour) & 1);
      ok[q] = (t < total) && (i <= bi1);
      own[q] = ok[q] && b.own(i, j);
      const int ii = i - b.gi0;
      o[q] = ok[q] ? (j - b.gj0) * hw + (ii >> 1) : hw + 1;
      par[q] = ok[q] ? (ii & 1) : 0;
      t += T;
      k += dk;
      j += dj;
      if (k >= wmax) {
        k -= wmax;
        ++j;
      }
    }
    float c_[NB], r_[NB], s_[NB], n_[NB], w_[NB], e_[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      c_[q] = Ec[o[q]];
      r_[q] = Rc[o[q]];
      s_[q] = Eo[o[q] - hw];
      n_[q] = Eo[o[q] + hw];
      w_[q] = Eo[o[q] - 1 + par[q]];
      e_[q] = Eo[o[q] + par[q]];
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      float sum = r_[q] - s_[q] - w_[q] - e_[q] - n_[q];
      sum = sum * -0.25f - c_[q];
      if (ok[q]) Ec[o[q]] = c_[q] + relax * sum;
      if (track && own[q]) {
        const unsigned int bb = __float_as_uint(fabsf(sum));
        mx = bb > mx ? bb : mx;
      }
    }
  }
  return mx;
}

// ns (<= K) sweeps on the box: colour half-sweeps on boxes shrinking from
// the tile grown by H-1 to the tile itself.  With redm, each warp keeps its
// running maximum of sweep s in redm[s][warp] (zeroed by the caller).
template <int K>
__device__ __forceinline__ void mixed_sweeps(const Dev &d, const MixedBox &b, int ns,
                                             float relax, unsigned int (*redm)[32]) {
  constexpr int H = 2 * K;
#pragma unroll 1
  for (int s = 0; s < ns; ++s) {
#pragma unroll 1
    for (int c = 0; c < 2; ++c) {
      const int e = H - 1 - 2 * s - c;
      const int bi0 = max(2, b.oi0 - e), bi1 = min(d.nx, b.oi1 + e);
      const int bj0 = max(2, b.oj0 - e), bj1 = min(d.ny, b.oj1 + e);
      const unsigned int m = mixed_half_sweep(b, bi0, bi1, bj0, bj1, c, relax, redm != nullptr);
      if (redm) {
        const unsigned int v = __reduce_max_sync(0xffffffffu, m);
        if ((threadIdx.x & 31) == 0) {
          unsigned int &slot = redm[s][threadIdx.x >> 5];
          slot = v > slot ? v : slot;
        }
      }
      __syncthreads();
    }
  }
}

// r = b - A p in FP64 on the whole box (zero off the unknowns), e = 0.
__device__ void mixed_residual(const Dev &d, const MixedBox &b, const double *p) {
  const int n = b.bw * b.bh;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = b.gi0 + t % b.bw, j = b.gj0 + t / b.bw;
    float r = 0.0f;
    if (i >= 2 && i <= d.nx && j >= 2 && j <= d.ny) {
      const size_t o = IX(d, i, j);
      const double ap = p[o - d.ld] + p[o - 1] + p[o + 1] + p[o + d.ld] - 4.0 * p[o];
      r = (float)(d.pb[o] - ap);
    }
    const int c = (i + j) & 1, x = b.at(i, j);
    b.R[c][x] = r;
    b.E[c][x] = 0.0f;
  }
}

// p += e on the own tile, FP64.
__device__ void mixed_correct(const Dev &d, const MixedBox &b, double *p) {
  const int tw = b.oi1 - b.oi0 + 1, th = b.oj1 - b.oj0 + 1;
  for (int t = threadIdx.x; t < tw * th; t += blockDim.x) {
    const int i = b.oi0 + t % tw, j = b.oj0 + t / tw;
    const size_t o = IX(d, i, j);
    p[o] = p[o] + (double)b.E[(i + j) & 1][b.at(i, j)];
  }
}

// One group of ns sweeps: ring from the neighbours' bands (ein, null in the
// first group of a pass, when e is still zero everywhere), snapshot, sweeps,
// own band to eout, per-sweep block maxima into slots.
template <int K>
__device__ void mixed_group(const Dev &d, const MixedBox &b, int ns, float relax,
                            const float *ein, float *eout, unsigned long long *slots) {
  constexpr int H = 2 * K;
  __shared__ unsigned int redm[K][32];
  if (ein) {
    const int n = b.bw * b.bh;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const int i = b.gi0 + t % b.bw, j = b.gj0 + t / b.bw;
      if (i >= 2 && i <= d.nx && j >= 2 && j <= d.ny && !b.own(i, j))
        b.E[(i + j) & 1][b.at(i, j)] = ein[IX(d, i, j)];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < b.bh * b.hw; t += blockDim.x) {
    b.E0[0][t] = b.E[0][t];
    b.E0[1][t] = b.E[1][t];
  }
  for (int t = threadIdx.x; t < K * 32; t += blockDim.x) redm[t / 32][t % 32] = 0u;
  __syncthreads();
  mixed_sweeps<K>(d, b, ns, relax, redm);
  const int tw = b.oi1 - b.oi0 + 1, th = b.oj1 - b.oj0 + 1;
  for (int t = threadIdx.x; t < tw * th; t += blockDim.x) {
    const int i = b.oi0 + t % tw, j = b.oj0 + t / tw;
    if (i - b.oi0 < H || b.oi1 - i < H || j - b.oj0 < H || b.oj1 - j < H)
      eout[IX(d, i, j)] = b.E[(i + j) & 1][b.at(i, j)];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int s = wid; s < ns; s += nw) {
    const unsigned int v = __reduce_max_sync(0xffffffffu, lane < nw ? redm[s][lane] : 0u);
    if (lane == 0 && v)
      atomicMax(&slots[s], (unsigned long long)__double_as_longlong((double)__uint_as_float(v)));
  }
  __syncthreads();
}

// Back to the snapshot taken at the start of the last group, then ns sweeps:
// the state after sweep ns when the stopping rule fired inside a group.
template <int K>
__device__ void mixed_redo(const Dev &d, const MixedBox &b, int ns, float relax) {
  for (int t = threadIdx.x; t < b.bh * b.hw; t += blockDim.x) {
    b.E[0][t] = b.E0[0][t];
    b.E[1][t] = b.E0[1][t];
  }
  __syncthreads();
  mixed_sweeps<K>(d, b, ns, relax, nullptr);
}

// Bytes of dynamic shared memory for a tile of tx x ty unknowns.
__host__ __device__ inline size_t mixed_smem_bytes(int K, int tx, int ty) {
  const size_t bw = (size_t)tx + 4 * K, bh = (size_t)ty + 4 * K;
  return 6 * bh * (bw / 2) * sizeof(float);
}

// The whole mixed Ppe: Divergence and b = div/dk in FP64, then refinement
// passes until the stopping rule fires or msorit sweeps are done.  Returns
// nConv (0 = not converged) or -1 on a barrier error.
template <int K>
__device__ int ppe_mixed(const Dev &d, const MixedGeom &g, const MixedArgs &a) {
  constexpr int H = 2 * K;
  Sync *sy = d.sync;
  unsigned long long *ring = &sy->red[kMixedRing];
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int k = 0; k < 3 * K; ++k) ring[k] = 0ull;
  ppe_divergence(d, a.u, a.v);
  if (!grid_sync(sy)) return -1;
  ppe_rhs_grid(d, a.lcartes, a.dk, a.p);
  if (!grid_sync(sy)) return -1;

  extern __shared__ double smem[];
  float *fs = reinterpret_cast<float *>(smem);
  const bool has = (int)blockIdx.x < g.ntx * g.nty;
  MixedBox b;
  {
    const int ti = blockIdx.x % g.ntx, tj = blockIdx.x / g.ntx;
    b.oi0 = 2 + ti * g.tx;
    b.oj0 = 2 + tj * g.ty;
    b.oi1 = min(d.nx, b.oi0 + g.tx - 1);
    b.oj1 = min(d.ny, b.oj0 + g.ty - 1);
    b.gi0 = b.oi0 - H;
    b.gj0 = b.oj0 - H;
    b.bw = g.tx + 2 * H;
    b.bh = g.ty + 2 * H;
    b.hw = b.bw / 2;
    const int plane = b.bh * b.hw;
    b.E[0] = fs;
    b.E[1] = fs + plane;
    b.E0[0] = fs + 2 * plane;
    b.E0[1] = fs + 3 * plane;
    b.R[0] = fs + 4 * plane;
    b.R[1] = fs + 5 * plane;
  }
  int m = 0, result = 0, grp = 0;
  bool done = false;
  while (!done) {
    if (has) mixed_residual(d, b, a.p);
    __syncthreads();
    int q = 0, in_pass = 0;
    while (true) {
      const int ns = min(K, min(a.inner - in_pass, a.msorit - m));
      unsigned long long *slots = ring + (grp % 3) * K;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long *next = ring + ((grp + 1) % 3) * K;
        for (int k = 0; k < K; ++k) next[k] = 0ull;
      }
      const float *ein = q == 0 ? nullptr : ((q & 1) ? a.ebuf0 : a.ebuf1);
      float *eout = (q & 1) ? a.ebuf1 : a.ebuf0;
      if (has) mixed_group<K>(d, b, ns, a.relax, ein, eout, slots);
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
      if (conv >= 0) {
        result = m + conv + 1;
        if (has && conv < ns - 1) mixed_redo<K>(d, b, conv + 1, a.relax);
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
    if (has) mixed_correct(d, b, a.p);
    if (!grid_sync(sy)) return -1;
  }
  return result;
}

}  // namespace w2
