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
// Layout.  Every block owns one tile of tx x ty unknowns and keeps in shared
// memory the tile grown by a halo of H = 2K cells, K being the sweeps run
// between grid barriers.  The box is stored as two colour planes (colour 0:
// i+j even) of hw = bw/2 entries per row: the points of one colour are
// contiguous and every neighbour of a point sits in the other plane at the
// same or the adjacent index.  Each thread owns a fixed list of (row, slot)
// positions of the box, built once per launch, holding per colour the
// point's distance to the box frame.  Half-sweep h (1-based within a group)
// updates the points at distance >= h: the frame's values are those of the
// group start, so after h half-sweeps only the points closer than h to the
// frame can be stale, and after 2K half-sweeps the tile (distance >= H) is
// exactly what a global sweep gives.  Between groups only the halo ring
// changes hands, through a global buffer in the same colour-split layout
// whose rows are aligned so that the ring and band segments move as 16-byte
// vectors: each block writes the band of its tile within H of the edge and
// reads its ring (two buffers, alternating by group).
#pragma once
#include "w2_ppe.cuh"

namespace w2 {

constexpr int kMixedPmax = 16;     // box positions per thread
constexpr int kMixedBatch = 8;     // positions whose operands are loaded together
constexpr int kMixedThreads = 512;
constexpr int kMixedRing = 17;     // Sync::red[17 .. 17 + 3K): per-sweep maxima

struct MixedGeom {
  int tx, ty;    // tile size in unknowns (tx a multiple of 8)
  int ntx, nty;  // tiles per direction, ntx*nty <= blocks
  int gw, gh;    // exchange buffer: floats per colour row, rows
  int P;         // box positions per thread
};

struct MixedArgs {
  int lcartes, msorit, inner;  // inner: FP32 sweeps per refinement pass
  double dk, sortol;
  float relax;                 // sorrel
  const double *u, *v;
  double *p;
  float *xbuf0, *xbuf1;        // exchange buffers: 2 colour planes of gh x gw
};

// Exchange-buffer element of cell (i, j), colour (i+j)&1, for halo H:
// row j + H - 2, float (i + H - 2) >> 1.  A tile (ti, tj)'s box row jj
// starts at row tj*ty + jj, float ti*tx/2, both 16-byte aligned.
struct MixedBox {
  float *E[2], *E0[2], *R[2];  // colour planes, row stride hw
  int gi0, gj0, bw, bh, hw;    // box origin (grid indices) and size
  int oi0, oi1, oj0, oj1;      // own tile, clipped to the unknowns
  int ti, tj;
  __device__ __forceinline__ int at(int i, int j) const {
    return (j - gj0) * hw + ((i - gi0) >> 1);
  }
};

// Packed position: bits 0-15 row*hw + slot, bit 16 row parity of colour 0,
// bits 17-21 / 22-26 distance of the colour-0 / colour-1 point to the box
// frame (0 = not an unknown: never updated).  A thread's unused positions
// point at row 1, slot 1 with distance 0, so that their (unconditional)
// operand loads stay inside the box.
__device__ __forceinline__ unsigned int mixed_unused(const MixedBox &b) {
  return (unsigned int)(b.hw + 1);
}

__device__ __forceinline__ unsigned int mixed_position(const Dev &d, const MixedBox &b, int n,
                                                       int H) {
  const int per_row = b.hw - 1, rows = b.bh - 2;
  if (n >= rows * per_row) return mixed_unused(b);
  const int jj = 1 + n / per_row, slot = n % per_row;
  const int par0 = (b.gj0 + jj) & 1;
  unsigned int w = (unsigned int)(jj * b.hw + slot) | ((unsigned int)par0 << 16);
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int par = par0 ^ c;
    const int ii = 2 * (slot + 1 - par) + par;
    const int i = b.gi0 + ii, j = b.gj0 + jj;
    int dist = 0;
    if (i >= 2 && i <= d.nx && j >= 2 && j <= d.ny) {
      dist = min(min(ii, b.bw - 1 - ii), min(jj, b.bh - 1 - jj));
      dist = min(dist, H);
    }
    w |= (unsigned int)dist << (17 + 5 * c);
  }
  return w;
}

// Half-sweep h of colour c over the thread's positions; returns the max
// |delta| over own points (distance >= H) as FP32 bits.  Every position's
// operands are loaded (all lie inside the box) and only the stores and the
// maximum are predicated, so the loop has no data-dependent branches.
template <int K>
__device__ __forceinline__ unsigned int mixed_half_sweep(const MixedBox &b, const unsigned int *pt,
                                                         int P, int c, int h, float relax) {
  constexpr int H = 2 * K;
  constexpr int NB = kMixedBatch;
  unsigned int mx = 0u;
  float *Ec = b.E[c];
  const float *Eo = b.E[c ^ 1];
  const float *Rc = b.R[c];
  const int hw = b.hw;
  const int shift = 17 + 5 * c;
#pragma unroll
  for (int q0 = 0; q0 < kMixedPmax; q0 += NB) {
    if (q0 >= P) break;
    int o[NB], par[NB], dist[NB];
    float c_[NB], r_[NB], s_[NB], n_[NB], w_[NB], e_[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const unsigned int w = pt[q0 + q];
      par[q] = (int)((w >> 16) & 1u) ^ c;
      dist[q] = (int)((w >> shift) & 31u);
      o[q] = (int)(w & 0xffffu) + 1 - par[q];
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
      const float nv = c_[q] + relax * sum;
      if (dist[q] >= h) Ec[o[q]] = nv;
      const unsigned int bb = (dist[q] >= H) ? __float_as_uint(fabsf(sum)) : 0u;
      mx = bb > mx ? bb : mx;
    }
  }
  return mx;
}

// ns (<= K) sweeps.  With redm, each warp keeps its running maximum of sweep
// s in redm[s][warp] (zeroed by the caller).
template <int K>
__device__ __forceinline__ void mixed_sweeps(const MixedBox &b, const unsigned int *pt, int P,
                                             int ns, float relax, unsigned int (*redm)[32]) {
#pragma unroll 1
  for (int s = 0; s < ns; ++s) {
#pragma unroll 1
    for (int c = 0; c < 2; ++c) {
      const unsigned int m = mixed_half_sweep<K>(b, pt, P, c, 2 * s + c + 1, relax);
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

// The halo ring from the neighbours' bands: box rows [0,H) and [H+ty,bh)
// whole, rows [H,H+ty) the K floats at either end of each colour row.
template <int K>
__device__ void mixed_ring_load(const MixedGeom &g, const MixedBox &b, const float *G) {
  constexpr int H = 2 * K, KV = K / 4;
  const int hv = b.hw / 4;                       // float4 per colour row
  const int n_full = 2 * H * hv, n_side = g.ty * 2 * KV;
  const int per_c = n_full + n_side, total = 2 * per_c;
  const size_t plane = (size_t)g.gh * g.gw;
  const int row0 = b.tj * g.ty, col0 = b.ti * g.tx / 2;
  constexpr int NB = 4;
  for (int f0 = threadIdx.x; f0 < total; f0 += NB * blockDim.x) {
    float4 v[NB];
    int dst[NB], cc[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int f = f0 + q * blockDim.x;
      dst[q] = -1;
      cc[q] = 0;
      if (f < total) {
        const int c = f >= per_c ? 1 : 0;
        int gg = f - c * per_c, jj, kk;
        if (gg < n_full) {
          const int r = gg / hv;
          jj = r < H ? r : r + g.ty;
          kk = 4 * (gg - r * hv);
        } else {
          gg -= n_full;
          const int r = gg / (2 * KV), rem = gg - r * 2 * KV;
          jj = H + r;
          kk = rem < KV ? 4 * rem : b.hw - K + 4 * (rem - KV);
        }
        cc[q] = c;
        dst[q] = jj * b.hw + kk;
        v[q] = *reinterpret_cast<const float4 *>(G + c * plane + (size_t)(row0 + jj) * g.gw + col0 + kk);
      }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q)
      if (dst[q] >= 0) *reinterpret_cast<float4 *>(b.E[cc[q]] + dst[q]) = v[q];
  }
}

// The tile's band within H of its edge to the exchange buffer.
template <int K>
__device__ void mixed_band_store(const MixedGeom &g, const MixedBox &b, float *G) {
  constexpr int H = 2 * K, KV = K / 4;
  const int tv = g.tx / 8;  // float4 per colour row of the tile
  const int total = 2 * g.ty * tv;
  const size_t plane = (size_t)g.gh * g.gw;
  const int row0 = b.tj * g.ty, col0 = b.ti * g.tx / 2;
  for (int f = threadIdx.x; f < total; f += blockDim.x) {
    const int c = f >= g.ty * tv ? 1 : 0;
    const int gg = f - c * g.ty * tv;
    const int r = gg / tv, seg = gg - r * tv;
    if (r < H || r >= g.ty - H || seg < KV || seg >= tv - KV) {
      const int jj = H + r, kk = K + 4 * seg;
      *reinterpret_cast<float4 *>(G + c * plane + (size_t)(row0 + jj) * g.gw + col0 + kk) =
          *reinterpret_cast<const float4 *>(b.E[c] + jj * b.hw + kk);
    }
  }
}

// One group of ns sweeps: ring (not in the first group of a pass, when e is
// still zero everywhere), snapshot, sweeps, band, per-sweep block maxima.
template <int K>
__device__ void mixed_group(const MixedGeom &g, const MixedBox &b, const unsigned int *pt,
                            int ns, float relax, const float *ein, float *eout,
                            unsigned long long *slots) {
  __shared__ unsigned int redm[K][32];
  if (ein) {
    mixed_ring_load<K>(g, b, ein);
    __syncthreads();
  }
  {
    const int n4 = b.bh * b.hw / 4;
    float4 *e0 = reinterpret_cast<float4 *>(b.E[0]), *e1 = reinterpret_cast<float4 *>(b.E[1]);
    float4 *s0 = reinterpret_cast<float4 *>(b.E0[0]), *s1 = reinterpret_cast<float4 *>(b.E0[1]);
    for (int t = threadIdx.x; t < n4; t += blockDim.x) {
      s0[t] = e0[t];
      s1[t] = e1[t];
    }
  }
  for (int t = threadIdx.x; t < K * 32; t += blockDim.x) redm[t / 32][t % 32] = 0u;
  __syncthreads();
  mixed_sweeps<K>(b, pt, g.P, ns, relax, redm);
  mixed_band_store<K>(g, b, eout);
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
__device__ void mixed_redo(const MixedGeom &g, const MixedBox &b, const unsigned int *pt, int ns,
                           float relax) {
  const int n4 = b.bh * b.hw / 4;
  float4 *e0 = reinterpret_cast<float4 *>(b.E[0]), *e1 = reinterpret_cast<float4 *>(b.E[1]);
  const float4 *s0 = reinterpret_cast<const float4 *>(b.E0[0]);
  const float4 *s1 = reinterpret_cast<const float4 *>(b.E0[1]);
  for (int t = threadIdx.x; t < n4; t += blockDim.x) {
    e0[t] = s0[t];
    e1[t] = s1[t];
  }
  __syncthreads();
  mixed_sweeps<K>(b, pt, g.P, ns, relax, nullptr);
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
  b.ti = blockIdx.x % g.ntx;
  b.tj = blockIdx.x / g.ntx;
  b.oi0 = 2 + b.ti * g.tx;
  b.oj0 = 2 + b.tj * g.ty;
  b.oi1 = min(d.nx, b.oi0 + g.tx - 1);
  b.oj1 = min(d.ny, b.oj0 + g.ty - 1);
  b.gi0 = b.oi0 - H;
  b.gj0 = b.oj0 - H;
  b.bw = g.tx + 2 * H;
  b.bh = g.ty + 2 * H;
  b.hw = b.bw / 2;
  {
    const int plane = b.bh * b.hw;
    b.E[0] = fs;
    b.E[1] = fs + plane;
    b.E0[0] = fs + 2 * plane;
    b.E0[1] = fs + 3 * plane;
    b.R[0] = fs + 4 * plane;
    b.R[1] = fs + 5 * plane;
  }
  unsigned int pt[kMixedPmax];
#pragma unroll
  for (int q = 0; q < kMixedPmax; ++q)
    pt[q] = (has && q < g.P) ? mixed_position(d, b, (int)threadIdx.x + q * (int)blockDim.x, H)
                             : mixed_unused(b);

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
      const float *ein = q == 0 ? nullptr : ((q & 1) ? a.xbuf0 : a.xbuf1);
      float *eout = (q & 1) ? a.xbuf1 : a.xbuf0;
      if (has) mixed_group<K>(g, b, pt, ns, a.relax, ein, eout, slots);
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
        if (has && conv < ns - 1) mixed_redo<K>(g, b, pt, conv + 1, a.relax);
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
