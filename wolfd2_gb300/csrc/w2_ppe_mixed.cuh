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
// Layout.  Every block owns one tile of tx x ty unknowns; its box is the tile
// grown by a halo of H = 2K cells, K being the sweeps run between grid
// barriers.  The box is split into two colour planes (colour 0: i+j even) of
// hw = bw/2 columns: in every row, column k of a plane holds the point of
// that colour at i = gi0 + 2k + (row parity), so a point's east/west
// neighbours are the other plane's columns k and k-1 or k+1, and its
// north/south neighbours are the other plane's column k one row up or down.
//
// Registers.  Thread (t, s) owns the column pair k = 2t, 2t+1 of both planes
// over the rows of strip s (at most kMixedRows rows; which rows depends on
// the kernel, see mixed_half_sweep).  A half-sweep of colour c
// first reads the strip's column pair of the other plane into registers (8
// bytes a row), then walks its rows: north/south come from those registers
// (from shared memory at the strip's first and last row), the neighbour
// column beyond the pair from the adjacent lane by one warp shuffle whose
// direction is the row's parity (uniform across the warp; shared memory for
// the lanes at a warp's edge).  The two points of a row are updated
// together by the packed FP32 instructions (add/sub/mul.rn.f32x2), which
// round each lane as the scalar instruction does.  Updates are written through to the
// shared-memory planes, which are what other threads read and what the halo
// exchange moves.  Half-sweep h (1-based within a group) updates the points
// whose distance to the box frame is at least h: the frame keeps its
// group-start values, so after h half-sweeps only points closer than h to it
// can be stale, and after 2K half-sweeps the tile (distance >= H) is exactly
// what a global sweep gives.  Rows closer than h to the frame are skipped
// whole.
//
// Between groups only the halo ring changes hands, through a global buffer
// in the same colour-split layout whose rows are aligned so that ring and
// band segments move as 16-byte vectors: each block writes the band of its
// tile within H of the edge and reads its ring (two buffers, alternating by
// group).
#pragma once
#include "w2_ppe.cuh"
#include "w2_tma.cuh"

namespace w2 {

constexpr int kMixedRows = 8;       // rows of a thread's strip
constexpr int kMixedThreads = 512;  // largest block
constexpr int kMixedRing = 17;      // Sync::red[17 .. 17 + 3K): per-sweep maxima

struct MixedGeom {
  int tx, ty;    // tile size in unknowns (tx a multiple of 8)
  int ntx, nty;  // tiles per direction, ntx*nty <= blocks
  int gw, gh;    // exchange buffer: floats per colour row, rows
  int hwp;       // threads over one strip row (mixed_lanes)
  int resident;  // one tile per block, box kept in shared memory (else multi-tile)
};

struct MixedArgs {
  int lcartes, msorit, inner;  // inner: FP32 sweeps per refinement pass
  double dk, sortol;
  float relax;                 // sorrel
  const double *u, *v;
  double *p;
  float *xbuf0, *xbuf1;        // exchange buffers: 2 colour planes of gh x gw
  float *rbuf;                 // r of every unknown, same layout (multi-tile mode)
  const CUtensorMap *tm;       // multi-tile mode: TMA maps of xbuf0, xbuf1, rbuf
                               // (null: the boxes are staged with vector loads)
};

// Exchange-buffer element of cell (i, j), colour (i+j)&1, for halo H:
// row j + H - 2, float (i + H - 2) >> 1.  A tile (ti, tj)'s box row jj
// starts at row tj*ty + jj, float ti*tx/2, both 16-byte aligned.
struct MixedBox {
  float *E[2], *E0[2], *R[2];  // colour planes in shared memory, row stride hw
  int gi0, gj0, bw, bh, hw;    // box origin (grid indices) and size
  int oi0, oi1, oj0, oj1;      // own tile, clipped to the unknowns
  int ti, tj;
  int k, lane;                 // this thread's first column (pair k, k+1), lane
  int strip, nstrips;          // this thread's strip and the block's strips
  int jlo, jhi;                // box rows of unknowns
  int dc[4];                   // distance to the frame of box columns 2k .. 2k+3
                               // (column k + q/2 in rows of parity q&1)
  unsigned int own4;           // bit q: dc[q] >= H (own tile)
  bool wedge, eedge;           // west/east neighbour column lives in another warp
};

// Distance of box column ii's cells to the left/right frame (0 when the
// column is off the unknowns).
__device__ __forceinline__ int mixed_dcol(const Dev &d, const MixedBox &b, int ii, int H) {
  const int i = b.gi0 + ii;
  if (ii < 0 || ii >= b.bw || i < 2 || i > d.nx) return 0;
  return min(min(ii, b.bw - 1 - ii), H);
}

template <int C, class A>
__device__ __forceinline__ A &pick(A &a0, A &a1) {
  if constexpr (C == 0) return a0;
  else return a1;
}

// Packed FP32 pairs: each lane rounds as the scalar instruction does.
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 x, y, z;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
      "sub.rn.f32x2 z, x, y;\n\tmov.b64 {%0, %1}, z;\n\t}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 x, y, z;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
      "mul.rn.f32x2 z, x, y;\n\tmov.b64 {%0, %1}, z;\n\t}"
      : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

// The planes by 32-bit shared-window address (byte offsets).  Reached
// through the box's pointers, the resident kernel's sweeps came out as
// generic loads and stores (the compiler did not trace the pointers back to
// the shared window there); the multi-tile and ensemble kernels get shared
// loads from the pointers and run faster with them than with these
// volatile forms, so the access form is a template choice (SH).
// The loads name memory too, so that no compiler pass moves them across
// the block barriers or across the other accesses of the planes.
__device__ __forceinline__ float2 lds2(unsigned a) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ float lds1(unsigned a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void sts2(unsigned a, float2 v) {
  asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void sts1(unsigned a, float v) {
  asm volatile("st.shared.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

// The rows of a half-sweep of colour C for a strip whose first row has
// parity P0 (so row r has parity P0 ^ (r & 1), known once unrolled).  eo
// holds the strip's column pair of the other plane, read from shared memory
// at the start of the half-sweep.  In a row of parity 0 the pair's points
// sit at box columns 2k and 2k+2 with west neighbours (k-1, k) and east
// neighbours (k, k+1) of the other plane; in a row of parity 1 at 2k+1 and
// 2k+3 with west (k, k+1) and east (k+1, k+2).  actm bit q: the point at box
// column 2k+q is updated in this half-sweep.
template <int K, int C, int P0, bool SH>
__device__ __forceinline__ unsigned int mixed_rows(const MixedBox &b, int jj0, unsigned int amask,
                                                   unsigned int orow, unsigned int actm, float relax) {
  const unsigned sR = smem_addr(b.R[C]), sE = smem_addr(b.E[C]), sO = smem_addr(b.E[C ^ 1]);
  const char *pR = reinterpret_cast<const char *>(b.R[C]), *pO = reinterpret_cast<const char *>(b.E[C ^ 1]);
  char *pE = reinterpret_cast<char *>(b.E[C]);
  // plane accesses at byte offset o: shared-window forms or through the pointers
  auto ldO2 = [&](unsigned o) {
    if constexpr (SH) return lds2(sO + o);
    else return *reinterpret_cast<const float2 *>(pO + o);
  };
  auto ldO1 = [&](unsigned o) {
    if constexpr (SH) return lds1(sO + o);
    else return *reinterpret_cast<const float *>(pO + o);
  };
  auto ldE2 = [&](unsigned o) {
    if constexpr (SH) return lds2(sE + o);
    else return *reinterpret_cast<const float2 *>(pE + o);
  };
  auto ldR2 = [&](unsigned o) {
    if constexpr (SH) return lds2(sR + o);
    else return *reinterpret_cast<const float2 *>(pR + o);
  };
  auto stE2 = [&](unsigned o, float2 v) {
    if constexpr (SH) sts2(sE + o, v);
    else *reinterpret_cast<float2 *>(pE + o) = v;
  };
  auto stE1 = [&](unsigned o, float v) {
    if constexpr (SH) sts1(sE + o, v);
    else *reinterpret_cast<float *>(pE + o) = v;
  };
  const unsigned hb = 4u * (unsigned)b.hw, base = 4u * (unsigned)(jj0 * b.hw + b.k);
  const float2 q4 = make_float2(-0.25f, -0.25f);
  float2 eo[kMixedRows];
#pragma unroll
  for (int r = 0; r < kMixedRows; ++r) eo[r] = ldO2(base + r * hb);
  unsigned int mx = 0u;
#pragma unroll
  for (int r = 0; r < kMixedRows; ++r) {
    if (!((amask >> r) & 1u)) continue;   // same for the whole warp
    const int par = P0 ^ (r & 1);         // folded once the loop is unrolled
    const unsigned o = base + r * hb;     // byte offset of the pair in a plane
    const float2 ot = eo[r];
    float2 w, e;
    if (par == 0) {
      float nb = __shfl_up_sync(0xffffffffu, ot.y, 1);
      if (b.wedge) nb = ldO1(o - 4u);
      w = make_float2(nb, ot.x);
      e = ot;
    } else {
      float nb = __shfl_down_sync(0xffffffffu, ot.x, 1);
      if (b.eedge) nb = ldO1(o + 8u);
      w = ot;
      e = make_float2(ot.y, nb);
    }
    const float2 sv = (r == 0) ? ldO2(o - hb) : eo[r > 0 ? r - 1 : 0];
    const float2 nv = (r == kMixedRows - 1) ? ldO2(o + hb) : eo[r < kMixedRows - 1 ? r + 1 : r];
    const float2 c0 = ldE2(o);
    float2 sum = f2sub(f2sub(f2sub(f2sub(ldR2(o), sv), w), e), nv);
    sum = f2sub(f2mul(sum, q4), c0);
    // c0 + relax*sum in two roundings, as scalar intrinsics: a packed
    // multiply followed by a packed add came out fused
    const float2 nw = make_float2(__fadd_rn(c0.x, __fmul_rn(relax, sum.x)),
                                  __fadd_rn(c0.y, __fmul_rn(relax, sum.y)));
    const bool a0 = (actm >> par) & 1u, a1 = (actm >> (2 + par)) & 1u;
    if (a0 && a1) {
      stE2(o, nw);
    } else {
      if (a0) stE1(o, nw.x);
      if (a1) stE1(o + 4u, nw.y);
    }
    if ((orow >> r) & 1u) {
      if (a0 && ((b.own4 >> par) & 1u)) {
        const unsigned int bb = __float_as_uint(fabsf(sum.x));
        mx = bb > mx ? bb : mx;
      }
      if (a1 && ((b.own4 >> (2 + par)) & 1u)) {
        const unsigned int bb = __float_as_uint(fabsf(sum.y));
        mx = bb > mx ? bb : mx;
      }
    }
  }
  return mx;
}

// Half-sweep h of colour C over the thread's strip; returns the max |delta|
// over own points (distance >= H) as FP32 bits.  It updates the rows at
// distance >= h from the frame (h .. bh-1-h).  In the multi-tile and
// ensemble kernels (!SH) those rows are dealt out to the block's strips in
// equal runs, so every warp has about the same number of rows whatever h is
// (fixed strips would leave the warps near the frame idle at the barrier
// while the shrinking box passes them by): 27.0 against 32.9 ms per channel
// solve.  The resident kernel keeps fixed strips of kMixedRows rows (1 +
// strip * kMixedRows ..), measured faster there (10.7 against 11.0 ms).  A
// strip's run is uniform per warp and at most kMixedRows rows long: the
// block has enough strips of kMixedRows rows to cover rows 1 .. bh-2.
template <int K, int C, bool SH>
__device__ __forceinline__ unsigned int mixed_half_sweep(const MixedBox &b, int h, float relax) {
  constexpr int H = 2 * K;
  const int span = b.bh - 2 * h;
  if (span <= 0) return 0u;
  int run, jj0;
  if constexpr (SH) {
    run = kMixedRows;
    jj0 = 1 + b.strip * kMixedRows;
  } else {
    run = (span + b.nstrips - 1) / b.nstrips;
    jj0 = h + b.strip * run;
  }
  // rows of unknowns among the run inside h .. bh-1-h, and own rows
  // (distance >= H)
  const int ulo = max(max(b.jlo, jj0), h), uhi = min(min(b.jhi, jj0 + run - 1), b.bh - 1 - h);
  if (uhi < ulo) return 0u;
  const unsigned int amask = ((2u << (uhi - jj0)) - 1u) & ~((1u << (ulo - jj0)) - 1u);
  const int olo = max(ulo, H), ohi = min(uhi, b.bh - 1 - H);
  const unsigned int orow = ohi < olo ? 0u : ((2u << (ohi - jj0)) - 1u) & ~((1u << (olo - jj0)) - 1u);
  unsigned int actm = 0u;
#pragma unroll
  for (int q = 0; q < 4; ++q) actm |= (b.dc[q] >= h ? 1u : 0u) << q;
  if ((C + b.gj0 + jj0) & 1) return mixed_rows<K, C, 1, SH>(b, jj0, amask, orow, actm, relax);
  return mixed_rows<K, C, 0, SH>(b, jj0, amask, orow, actm, relax);
}

// ns (<= K) sweeps.  With redm, each warp keeps its running maximum of
// sweep s in redm[s][warp] (zeroed by the caller).  SH: plane accesses in
// the shared-window forms (resident kernel) or through the box's pointers.
template <int K, bool SH>
__device__ __forceinline__ void mixed_sweeps(const MixedBox &b, int ns, float relax,
                                             unsigned int (*redm)[32]) {
#pragma unroll 1
  for (int s = 0; s < ns; ++s) {
    const unsigned int m0 = mixed_half_sweep<K, 0, SH>(b, 2 * s + 1, relax);
    __syncthreads();
    const unsigned int m1 = mixed_half_sweep<K, 1, SH>(b, 2 * s + 2, relax);
    if (redm) {
      const unsigned int m = m0 > m1 ? m0 : m1;
      const unsigned int v = __reduce_max_sync(0xffffffffu, m);
      if (b.lane == 0) {
        unsigned int &slot = redm[s][threadIdx.x >> 5];
        slot = v > slot ? v : slot;
      }
    }
    __syncthreads();
  }
}

// (A p) at point o in FP64 for the residual of a refinement pass: on
// unit-stencil rows p_s + p_w + p_e + p_n - 4 p, otherwise the coefficients
// of pressure.f:97-106 in the same order, (((a1 p_s + a2 p_w) + a4 p_e) +
// a5 p_n) + a3 p, which is the unit form bit for bit when the a's are
// (1, 1, -4, 1, 1).  The FP32 sweeps run the unit stencil: the rows of any
// uniform square-cell grid round to it in FP32 (ppe_unit32), and the
// residual of the next pass, formed with the FP64 rows, corrects the
// difference.
__device__ __forceinline__ double mixed_ap(const Dev &d, const double *p, size_t o) {
  if (d.ppe_unit) return p[o - d.ld] + p[o - 1] + p[o + 1] + p[o + d.ld] - 4.0 * p[o];
  return d.pa1[o] * p[o - d.ld] + d.pa2[o] * p[o - 1] + d.pa4[o] * p[o + 1] + d.pa5[o] * p[o + d.ld] +
         d.pa3[o] * p[o];
}

// r = b - A p in FP64 on the whole box (zero off the unknowns) into the
// shared R planes; e = 0 in the shared planes.
__device__ __noinline__ void mixed_residual(const Dev &d, const MixedBox &b, const double *p) {
  const int n = b.bw * b.bh;
#pragma unroll 1
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = b.gi0 + t % b.bw, j = b.gj0 + t / b.bw;
    float r = 0.0f;
    if (i >= 2 && i <= d.nx && j >= 2 && j <= d.ny) {
      const size_t o = IX(d, i, j);
      r = (float)(d.pb[o] - mixed_ap(d, p, o));
    }
    const int c = (i + j) & 1, x = (j - b.gj0) * b.hw + ((i - b.gi0) >> 1);
    b.R[c][x] = r;
    b.E[c][x] = 0.0f;
  }
}

// p += e on the own tile, FP64.
__device__ __noinline__ void mixed_correct(const Dev &d, const MixedBox &b, double *p) {
  const int tw = b.oi1 - b.oi0 + 1, th = b.oj1 - b.oj0 + 1;
  for (int t = threadIdx.x; t < tw * th; t += blockDim.x) {
    const int i = b.oi0 + t % tw, j = b.oj0 + t / tw;
    const size_t o = IX(d, i, j);
    p[o] = p[o] + (double)b.E[(i + j) & 1][(j - b.gj0) * b.hw + ((i - b.gi0) >> 1)];
  }
}

// The halo ring from the neighbours' bands: box rows [0,H) and [H+ty,bh)
// whole, rows [H,H+ty) the K floats at either end of each colour row.
template <int K>
__device__ __noinline__ void mixed_ring_load(const MixedGeom &g, const MixedBox &b, const float *G) {
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
__device__ __noinline__ void mixed_band_store(const MixedGeom &g, const MixedBox &b, float *G) {
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

// Shared-memory plane copy (both colours), 16-byte vectors.
__device__ __noinline__ void mixed_copy_planes(const MixedBox &b, float *dst0, float *dst1,
                                               const float *src0, const float *src1) {
  const int n4 = b.bh * b.hw / 4;
  float4 *d0 = reinterpret_cast<float4 *>(dst0), *d1 = reinterpret_cast<float4 *>(dst1);
  const float4 *s0 = reinterpret_cast<const float4 *>(src0);
  const float4 *s1 = reinterpret_cast<const float4 *>(src1);
  for (int t = threadIdx.x; t < n4; t += blockDim.x) {
    d0[t] = s0[t];
    d1[t] = s1[t];
  }
}

// One group of ns sweeps: ring (not in the first group of a pass, when e is
// still zero everywhere), snapshot, sweeps, band, per-sweep block maxima.
template <int K>
__device__ __forceinline__ void mixed_group(const MixedGeom &g, const MixedBox &b, int ns,
                                            float relax, const float *ein, float *eout,
                                            unsigned long long *slots) {
  __shared__ unsigned int redm[K][32];
  if (ein) {
    mixed_ring_load<K>(g, b, ein);
    __syncthreads();
  }
  mixed_copy_planes(b, b.E0[0], b.E0[1], b.E[0], b.E[1]);
  for (int t = threadIdx.x; t < K * 32; t += blockDim.x) redm[t / 32][t % 32] = 0u;
  __syncthreads();
  mixed_sweeps<K, true>(b, ns, relax, redm);
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
__device__ __forceinline__ void mixed_redo(const MixedBox &b, int ns, float relax) {
  mixed_copy_planes(b, b.E[0], b.E[1], b.E0[0], b.E0[1]);
  __syncthreads();
  mixed_sweeps<K, true>(b, ns, relax, nullptr);
}

// Bytes of dynamic shared memory for a tile of tx x ty unknowns: the two
// colour planes of e and of r, and (resident mode) the snapshot of e.
// Multi-tile mode: the r planes start on a 128-byte boundary (a TMA
// destination), after the e planes rounded up to 32 floats.
__host__ __device__ inline size_t mixed_r_offset(size_t plane) { return (2 * plane + 31) & ~(size_t)31; }
__host__ __device__ inline size_t mixed_smem_bytes(int K, int tx, int ty, bool resident = true) {
  const size_t bw = (size_t)tx + 4 * K, bh = (size_t)ty + 4 * K, plane = bh * (bw / 2);
  return (resident ? 6 * plane : mixed_r_offset(plane) + 2 * plane) * sizeof(float);
}

// Threads over one strip row of a tile's box: the plane column pairs
// rounded up to whole warps.
__host__ __device__ inline int mixed_lanes(int K, int tx) {
  const int hw = tx / 2 + 2 * K;  // a multiple of 4: tx is a multiple of 8
  return (hw / 2 + 31) / 32 * 32;
}

// Threads of a block for a tile of tx x ty unknowns: whole warps over the
// plane column pairs times strips of kMixedRows rows over the box rows
// 1..bh-2.
__host__ __device__ inline int mixed_threads(int K, int tx, int ty) {
  const int rows = ty + 4 * K - 2;
  return mixed_lanes(K, tx) * ((rows + kMixedRows - 1) / kMixedRows);
}

// The box of tile `tile` and this thread's place in it.  Resident mode keeps
// planes E, E0, R; multi-tile mode E and R.
template <int K>
__device__ __forceinline__ void mixed_setup(const Dev &d, const MixedGeom &g, MixedBox &b,
                                            int tile, float *fs, bool resident) {
  constexpr int H = 2 * K;
  b.ti = tile % g.ntx;
  b.tj = tile / g.ntx;
  b.oi0 = 2 + b.ti * g.tx;
  b.oj0 = 2 + b.tj * g.ty;
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
  if (resident) {
    b.E0[0] = fs + 2 * plane;
    b.E0[1] = fs + 3 * plane;
    b.R[0] = fs + 4 * plane;
    b.R[1] = fs + 5 * plane;
  } else {
    const int r0 = (int)mixed_r_offset((size_t)plane);
    b.E0[0] = b.E0[1] = nullptr;
    b.R[0] = fs + r0;
    b.R[1] = fs + r0 + plane;
  }
  // lanes past the box's column pairs read the last pair (their values
  // reach only the frame column, which is never updated) and update nothing
  const int t = (int)threadIdx.x % g.hwp, np = b.hw / 2;
  const bool valid = t < np;
  b.k = 2 * min(t, np - 1);
  b.lane = (int)threadIdx.x & 31;
  b.strip = (int)threadIdx.x / g.hwp;
  b.nstrips = (int)blockDim.x / g.hwp;
  b.jlo = max(1, 2 - b.gj0);
  b.jhi = min(b.bh - 2, d.ny - b.gj0);
  b.own4 = 0u;
  for (int q = 0; q < 4; ++q) {
    b.dc[q] = valid ? mixed_dcol(d, b, 2 * b.k + q, H) : 0;
    if (b.dc[q] >= H) b.own4 |= 1u << q;
  }
  b.wedge = b.lane == 0 && valid && b.k >= 2;
  b.eedge = b.lane == 31 && valid && b.k + 2 < b.hw;
}

// Position of cell (i, j) in a colour-split buffer (see MixedBox).
template <int K>
__device__ __forceinline__ size_t mixed_gpos(const MixedGeom &g, int i, int j) {
  constexpr int H = 2 * K;
  return (size_t)((i + j) & 1) * g.gh * g.gw + (size_t)(j + H - 2) * g.gw + ((i + H - 2) >> 1);
}

// ---- multi-tile mode: blocks loop over tiles, staging whole boxes -------

// The whole box of one colour-split buffer into two shared planes (zeros
// when G is null).
template <int K>
__device__ __noinline__ void mixed_box_load(const MixedGeom &g, const MixedBox &b, const float *G,
                                            float *P0, float *P1) {
  const int hv = b.hw / 4, total = 2 * b.bh * hv;
  const size_t plane = (size_t)g.gh * g.gw;
  const int row0 = b.tj * g.ty, col0 = b.ti * g.tx / 2;
  for (int f = threadIdx.x; f < total; f += blockDim.x) {
    const int c = f >= b.bh * hv ? 1 : 0;
    const int gg = f - c * b.bh * hv;
    const int jj = gg / hv, kk = 4 * (gg - jj * hv);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (G) v = *reinterpret_cast<const float4 *>(G + c * plane + (size_t)(row0 + jj) * g.gw + col0 + kk);
    *reinterpret_cast<float4 *>((c ? P1 : P0) + jj * b.hw + kk) = v;
  }
}

// The own tile of the shared e planes to a colour-split buffer.
template <int K>
__device__ __noinline__ void mixed_tile_store(const MixedGeom &g, const MixedBox &b, float *G) {
  const int tv = g.tx / 8, total = 2 * g.ty * tv;
  const size_t plane = (size_t)g.gh * g.gw;
  const int row0 = b.tj * g.ty, col0 = b.ti * g.tx / 2;
  for (int f = threadIdx.x; f < total; f += blockDim.x) {
    const int c = f >= g.ty * tv ? 1 : 0;
    const int gg = f - c * g.ty * tv;
    const int r = gg / tv, seg = gg - r * tv;
    const int jj = 2 * K + r, kk = K + 4 * seg;
    *reinterpret_cast<float4 *>(G + c * plane + (size_t)(row0 + jj) * g.gw + col0 + kk) =
        *reinterpret_cast<const float4 *>(b.E[c] + jj * b.hw + kk);
  }
}

// r = b - A p in FP64 on the own unknowns of a tile, into the r buffer.
template <int K>
__device__ __noinline__ void mixed_residual_tile(const Dev &d, const MixedGeom &g,
                                                 const MixedBox &b, const double *p, float *Rg) {
  const int tw = b.oi1 - b.oi0 + 1, th = b.oj1 - b.oj0 + 1;
  for (int t = threadIdx.x; t < tw * th; t += blockDim.x) {
    const int i = b.oi0 + t % tw, j = b.oj0 + t / tw;
    const size_t o = IX(d, i, j);
    Rg[mixed_gpos<K>(g, i, j)] = (float)(d.pb[o] - mixed_ap(d, p, o));
  }
}

// p += e on the own unknowns of a tile, e from a colour-split buffer.
template <int K>
__device__ __noinline__ void mixed_correct_tile(const Dev &d, const MixedGeom &g,
                                                const MixedBox &b, double *p, const float *G) {
  const int tw = b.oi1 - b.oi0 + 1, th = b.oj1 - b.oj0 + 1;
  for (int t = threadIdx.x; t < tw * th; t += blockDim.x) {
    const int i = b.oi0 + t % tw, j = b.oj0 + t / tw;
    const size_t o = IX(d, i, j);
    p[o] = p[o] + (double)G[mixed_gpos<K>(g, i, j)];
  }
}

// Block maxima of ns sweeps into the global slots.
__device__ __forceinline__ void mixed_flush_maxima(unsigned int (*redm)[32], int ns,
                                                   unsigned long long *slots) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int s = wid; s < ns; s += nw) {
    const unsigned int v = __reduce_max_sync(0xffffffffu, lane < nw ? redm[s][lane] : 0u);
    if (lane == 0 && v)
      atomicMax(&slots[s], (unsigned long long)__double_as_longlong((double)__uint_as_float(v)));
  }
}

// Multi-tile mode: the box of e (zeros when ein is null) and of r into the
// shared planes.  With tensor maps, thread 0 issues one TMA load per buffer
// (both colour planes in one 3-D box) and waits on the block's mbarrier;
// without, every thread moves 16-byte vectors.  Returns false if the wait
// ran out its time limit (the error is set).
template <int K>
__device__ __forceinline__ bool mixed_stage(const MixedGeom &g, const MixedBox &b, const MixedArgs &a,
                                            bool tma, const float *ein, unsigned long long *bar,
                                            unsigned &phase, Sync *sy) {
  if (!tma) {
    mixed_box_load<K>(g, b, ein, b.E[0], b.E[1]);
    mixed_box_load<K>(g, b, a.rbuf, b.R[0], b.R[1]);
    __syncthreads();
    return true;
  }
  __shared__ int ok;
  if (threadIdx.x == 0) {
    const int x = b.ti * g.tx / 2, y = b.tj * g.ty;
    const unsigned box = 2u * (unsigned)b.bh * (unsigned)b.hw * 4u;
    // the planes were last read and written by the block's threads, ordered
    // before this point by the block barrier that ended the previous tile
    fence_proxy_async_smem();
    mbar_expect_tx(bar, ein ? 2u * box : box);
    if (ein) tma_load_3d(b.E[0], a.tm + (ein == a.xbuf0 ? 0 : 1), x, y, 0, bar);
    tma_load_3d(b.R[0], a.tm + 2, x, y, 0, bar);
  }
  if (!ein) mixed_box_load<K>(g, b, nullptr, b.E[0], b.E[1]);
  if (threadIdx.x == 0) ok = mbar_wait(bar, phase, sy) ? 1 : 0;
  __syncthreads();
  phase ^= 1u;
  return ok != 0;
}

// The whole mixed Ppe: Divergence and b = div/dk in FP64, then refinement
// passes until the stopping rule fires or msorit sweeps are done.  One tile
// per block keeps the box resident in shared memory between groups (only the
// halo ring is exchanged); with more tiles than blocks, each block stages
// the whole box of each of its tiles every group.  Returns nConv (0 = not
// converged) or -1 on a barrier error.  RES selects the mode at compile
// time (each mode is its own kernel: together they would not fit the 128
// registers a thread of a 512-thread block has).
template <int K, bool RES>
__device__ int ppe_mixed(const Dev &d, const MixedGeom &g, const MixedArgs &a) {
  Sync *sy = d.sync;
  unsigned long long *ring = &sy->red[kMixedRing];
  if (vblock() == 0 && threadIdx.x == 0)
    for (int k = 0; k < 3 * K; ++k) ring[k] = 0ull;
  ppe_divergence(d, a.u, a.v);
  if (!grid_sync(sy)) return -1;
  ppe_rhs_grid(d, a.lcartes, a.dk, a.p);
  if (!grid_sync(sy)) return -1;

  extern __shared__ __align__(128) double smem[];
  __shared__ unsigned int redm[K][32];
  __shared__ unsigned long long tbar;  // completion of the TMA box loads (multi-tile mode)
  unsigned tphase = 0u;
  float *fs = reinterpret_cast<float *>(smem);
  // TMA destinations must start on 128-byte boundaries: the declaration
  // asks for that alignment of the dynamic base; should a base ever lack
  // it, the boxes are staged with vector loads instead
  const bool tma = !RES && a.tm && (smem_addr(smem) & 127u) == 0u;
  if constexpr (!RES) {
    if (tma && threadIdx.x == 0) mbar_init(&tbar, 1);
    __syncthreads();
  }
  const int ntiles = g.ntx * g.nty;
  constexpr bool resident = RES;
  const bool has = vblock() < ntiles;
  MixedBox b;
  if constexpr (resident) mixed_setup<K>(d, g, b, vblock(), fs, true);

  int m = 0, result = 0, grp = 0;
  bool done = false;
  while (!done) {
    if constexpr (resident) {
      if (has) mixed_residual(d, b, a.p);
      __syncthreads();
    } else {
      for (int tile = vblock(); tile < ntiles; tile += vblocks()) {
        mixed_setup<K>(d, g, b, tile, fs, false);
        mixed_residual_tile<K>(d, g, b, a.p, a.rbuf);
      }
      if (!grid_sync(sy)) return -1;
    }
    int q = 0, in_pass = 0;
    const float *efinal = nullptr;
    while (true) {
      const int ns = min(K, min(a.inner - in_pass, a.msorit - m));
      unsigned long long *slots = ring + (grp % 3) * K;
      if (vblock() == 0 && threadIdx.x == 0) {
        unsigned long long *next = ring + ((grp + 1) % 3) * K;
        for (int k = 0; k < K; ++k) next[k] = 0ull;
      }
      const float *ein = q == 0 ? nullptr : ((q & 1) ? a.xbuf0 : a.xbuf1);
      float *eout = (q & 1) ? a.xbuf1 : a.xbuf0;
      if constexpr (resident) {
        if (has) mixed_group<K>(g, b, ns, a.relax, ein, eout, slots);
      } else {
        for (int t = threadIdx.x; t < K * 32; t += blockDim.x) redm[t / 32][t % 32] = 0u;
        for (int tile = vblock(); tile < ntiles; tile += vblocks()) {
          mixed_setup<K>(d, g, b, tile, fs, false);
          if (!mixed_stage<K>(g, b, a, tma, ein, &tbar, tphase, sy)) return -1;
          mixed_sweeps<K, false>(b, ns, a.relax, redm);
          mixed_tile_store<K>(g, b, eout);
          __syncthreads();
        }
        mixed_flush_maxima(redm, ns, slots);
      }
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
        if (conv < ns - 1) {
          if constexpr (resident) {
            if (has) mixed_redo<K>(b, conv + 1, a.relax);
          } else {
            // the group's input buffer is intact: sweep again from it
            for (int tile = vblock(); tile < ntiles; tile += vblocks()) {
              mixed_setup<K>(d, g, b, tile, fs, false);
              if (!mixed_stage<K>(g, b, a, tma, ein, &tbar, tphase, sy)) return -1;
              mixed_sweeps<K, false>(b, conv + 1, a.relax, nullptr);
              mixed_tile_store<K>(g, b, eout);
              __syncthreads();
            }
          }
        }
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
    if constexpr (resident) {
      if (has) mixed_correct(d, b, a.p);
    } else {
      for (int tile = vblock(); tile < ntiles; tile += vblocks()) {
        mixed_setup<K>(d, g, b, tile, fs, false);
        mixed_correct_tile<K>(d, g, b, a.p, efinal);
      }
    }
    if (!grid_sync(sy)) return -1;
  }
  return result;
}

}  // namespace w2
