// w2_chain.cuh -- exact parallel solve of AltTridLU chains (momentum.f:1307-1339).
//
// The reference solves each momentum split step as ONE Thomas recurrence over
// the concatenation of all grid lines, including a first-row quirk (row 1's
// super-diagonal is divided by row 2's ORIGINAL diagonal).  Neighbouring
// lines couple through the chain wherever the end rows are not identity rows,
// so a per-line solve would change the numbers.
//
// This solver reproduces the sequential recurrence bit for bit with parallel
// work.  The chain is cut into segments of L rows, one thread each, and
// stored segment-interleaved (row r of segment s at r*nseg + s) so that a
// warp's loads at every step of the walks are consecutive words:
//   F1  every segment runs the forward recurrence (factorisation + forward
//       substitution, state (a3', b')) starting `warm` rows early from the
//       state (0, 0), so by its first own row the state has usually converged
//       to the true one (the recurrence contracts);
//   F2  verification rounds: each segment re-runs its rows from the exact end
//       state of its predecessor and stops at the first row whose recomputed
//       state equals the stored one bit for bit -- from there on the stored
//       values ARE the sequential ones.  A segment that never re-joins its
//       stored trajectory publishes a new end state and another round runs.
//       When a round changes nothing, every segment provably holds the values
//       of the sequential recurrence (induction from row 0, which is exact).
//   B1/B2  the same for the back substitution x(k) = b'(k) - a3'(k) x(k+1),
//       running from the last row down.
// Round r leaves segments 0..r+1 exact, so at most nseg rounds run before a
// round changes nothing; the loop is bounded by that count.  A NaN state
// stays NaN through every later row of the recurrence (only +, -, *, /), so
// two NaNs count as equal: the solve then matches the sequential one up to
// NaN payloads, and a diverged flow settles in a few rounds like any other.
// One warp walking the chain sequentially remains as a guard that a correct
// build never reaches (it sets the fallback flag).
#pragma once
#include "w2_common.cuh"

namespace w2 {

// One row of a chain: sub-, main and super-diagonal and right-hand side.
template <class T>
struct ChainRow {
  T a1, a2, a3, b;
};

// Bound of the verification rounds of one solve: every segment count plus
// one settling round (see the induction above).
__device__ __forceinline__ int max_rounds(int nseg0, int nseg1) {
  return (nseg0 > nseg1 ? nseg0 : nseg1) + 1;
}

// Equal bits, or both NaN (integer tests: no floating-point pipe).
__device__ __forceinline__ bool same_state(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a),
                           y = (unsigned long long)__double_as_longlong(b);
  const unsigned long long inf = 0x7ff0000000000000ull, mag = 0x7fffffffffffffffull;
  return x == y || ((x & mag) > inf && (y & mag) > inf);
}
__device__ __forceinline__ bool same_state(float a, float b) {
  const unsigned x = (unsigned)__float_as_int(a), y = (unsigned)__float_as_int(b);
  return x == y || ((x & 0x7fffffffu) > 0x7f800000u && (y & 0x7fffffffu) > 0x7f800000u);
}

// Storage position of chain row k: row r of segment s lives at r*nseg + s,
// so the threads of a warp, one segment each, touch consecutive words at
// every step of their walks.
template <class T>
__device__ __forceinline__ int cpos(const ChainT<T> &c, int k) {
  const int s = k / c.L;
  return (k - s * c.L) * c.nseg + s;
}

// A walk over consecutive chain rows with their storage positions.
struct RowWalk {
  int k, r, s, p;
  __device__ __forceinline__ RowWalk(int k0, int L, int nseg)
      : k(k0), r(k0 % L), s(k0 / L), p((k0 % L) * nseg + k0 / L) {}
  __device__ __forceinline__ void next(int L, int nseg) {
    ++k;
    if (++r == L) {
      r = 0;
      p = ++s;
    } else {
      p += nseg;
    }
  }
  __device__ __forceinline__ void prev(int L, int nseg) {
    --k;
    if (--r < 0) {
      r = L - 1;
      --s;
      p = r * nseg + s;
    } else {
      p -= nseg;
    }
  }
};

// Right-hand side of a row (the split-2 identity rows find theirs zeroed by
// the split-2 assembly).
template <class T>
__device__ __forceinline__ T chain_rhs(const ChainT<T> &c, int p) {
  return c.b[p];
}

// One forward row k >= 1 (stored at p) of AltTridLU: a2' = a2 - a1 a3'(k-1);
// a3' = a3/a2' (not formed on the last row); b' = (b - a1 b'(k-1)) / a2'.
template <class T>
__device__ __forceinline__ void fwd_row(const ChainT<T> &c, int k, int p, T &a3p, T &bp) {
  const T a1 = c.a1[p];
  const T a2p = c.a2[p] - a1 * a3p;
  const T nb = (chain_rhs(c, p) - a1 * bp) / a2p;
  a3p = (k < c.n - 1) ? c.a3[p] / a2p : T(0);
  bp = nb;
}

// Row 0 with the reference's first-row quirk.
template <class T>
__device__ __forceinline__ void fwd_row0(const ChainT<T> &c, T &a3p, T &bp) {
  a3p = c.a3[0] / c.a2[cpos(c, 1)];
  bp = chain_rhs(c, 0) / c.a2[0];
}

// Walks load their rows a batch ahead of the recurrence: each thread copies
// the coefficients of its next rows into its own slots of shared memory with
// cp.async, waits once, then runs the rows from there.  A walk is a chain of
// dependent steps, so this pays one memory latency per batch instead of one
// per row, without holding the batch in registers.  On a uniform stretch of
// flow no segment re-joins its stored trajectory before the end of the grid
// line (the rounded recurrence can settle on either of two neighbouring
// values), so rounds walk whole lines and this latency sets their cost.
// Each row's arithmetic is fwd_row's, or x = b' - a3' x going back.
template <class T>
struct RowBatch {
  static constexpr int n = sizeof(T) == 4 ? 16 : 8;  // rows per batch
  static constexpr int arrays = 6;                    // staged arrays at most
};

// Dynamic shared memory the walks need in a block of `threads` threads.
inline size_t walk_stage_bytes(size_t elem, int threads) {
  return elem * (elem == 4 ? 16 : 8) * 6 * (size_t)threads;
}

// This thread's slots: slot (a, r) at stage[(a * n + r) * blockDim.x].
template <class T>
__device__ __forceinline__ T *walk_stage() {
  extern __shared__ __align__(16) unsigned char w2_walk_smem[];
  return reinterpret_cast<T *>(w2_walk_smem) + threadIdx.x;
}

template <class T>
__device__ __forceinline__ void stage_copy(T *dst, const T *src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(src), "n"((int)sizeof(T))
               : "memory");
}

__device__ __forceinline__ void stage_wait() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;\n" ::: "memory");
}

// Forward rows w.k .. w.k+m-1 (m <= the batch); STORE writes a3' and b'.
template <class T, bool STORE>
__device__ __forceinline__ void fwd_batch(const ChainT<T> &c, RowWalk &w, int m, int L, int ns,
                                          T &a3p, T &bp) {
  constexpr int R = RowBatch<T>::n;
  T *st = walk_stage<T>();
  const int bs = blockDim.x;
  RowWalk v = w;
  for (int r = 0; r < m; ++r) {
    stage_copy(st + (0 * R + r) * bs, c.a1 + v.p);
    stage_copy(st + (1 * R + r) * bs, c.a2 + v.p);
    stage_copy(st + (2 * R + r) * bs, c.a3 + v.p);
    stage_copy(st + (3 * R + r) * bs, c.b + v.p);
    v.next(L, ns);
  }
  stage_wait();
  RowWalk u = w;
  for (int r = 0; r < m; ++r) {
    const T a1 = st[(0 * R + r) * bs];
    const T a2p = st[(1 * R + r) * bs] - a1 * a3p;
    const T nb = (st[(3 * R + r) * bs] - a1 * bp) / a2p;
    a3p = (u.k < c.n - 1) ? st[(2 * R + r) * bs] / a2p : T(0);
    bp = nb;
    if (STORE) {
      c.a3p[u.p] = a3p;
      c.bp[u.p] = bp;
    }
    u.next(L, ns);
  }
  w = v;
}

// Back substitution rows w.k, w.k-1, ... (m of them); STORE writes x.
template <class T, bool STORE>
__device__ __forceinline__ void bwd_batch(const ChainT<T> &c, RowWalk &w, int m, int L, int ns, T &xn) {
  constexpr int R = RowBatch<T>::n;
  T *st = walk_stage<T>();
  const int bs = blockDim.x;
  RowWalk v = w;
  for (int r = 0; r < m; ++r) {
    stage_copy(st + (0 * R + r) * bs, c.bp + v.p);
    stage_copy(st + (1 * R + r) * bs, c.a3p + v.p);
    v.prev(L, ns);
  }
  stage_wait();
  RowWalk u = w;
  for (int r = 0; r < m; ++r) {
    xn = st[(0 * R + r) * bs] - st[(1 * R + r) * bs] * xn;
    if (STORE) c.x[u.p] = xn;
    u.prev(L, ns);
  }
  w = v;
}

template <class T>
__device__ void chain_f1(const ChainT<T> &c, int s, int L, int W) {
  constexpr int R = RowBatch<T>::n;
  const int k0 = s * L, k1 = min(c.n, k0 + L), ns = c.nseg;
  T a3p, bp;
  int kown = k0;
  if (k0 == 0) {
    fwd_row0(c, a3p, bp);
    c.a3p[0] = a3p;
    c.bp[0] = bp;
    kown = 1;
  } else {
    const int kw = k0 - W;
    RowWalk u(kw <= 0 ? 1 : kw, L, ns);
    if (kw <= 0) {
      fwd_row0(c, a3p, bp);
    } else {
      a3p = T(0);
      bp = T(0);
    }
    while (u.k < k0) fwd_batch<T, false>(c, u, min(R, k0 - u.k), L, ns, a3p, bp);
  }
  RowWalk w(kown, L, ns);
  while (w.k < k1) fwd_batch<T, true>(c, w, min(R, k1 - w.k), L, ns, a3p, bp);
  c.ef[2 * s] = a3p;
  c.ef[2 * s + 1] = bp;
}

// Verification round; reads end states from `ein`, writes `eout`.
// Returns true when the segment's end state changed.  The first row runs
// alone (most segments re-join their stored trajectory there), the rest in
// batches.
template <class T>
__device__ bool chain_f2(const ChainT<T> &c, int s, int L, const T *ein, T *eout) {
  constexpr int R = RowBatch<T>::n;
  if (s == 0) {
    eout[0] = ein[0];
    eout[1] = ein[1];
    return false;
  }
  const int k0 = s * L, k1 = min(c.n, k0 + L), ns = c.nseg;
  T a3p = ein[2 * (s - 1)], bp = ein[2 * (s - 1) + 1];
  fwd_row(c, k0, s, a3p, bp);
  if (same_state(a3p, c.a3p[s]) && same_state(bp, c.bp[s])) {
    eout[2 * s] = ein[2 * s];
    eout[2 * s + 1] = ein[2 * s + 1];
    return false;
  }
  c.a3p[s] = a3p;
  c.bp[s] = bp;
  T *st = walk_stage<T>();
  const int bs = blockDim.x;
  for (int k = k0 + 1, p = s + ns; k < k1;) {
    const int m = min(R, k1 - k);
    for (int r = 0; r < m; ++r) {
      const int q = p + r * ns;
      stage_copy(st + (0 * R + r) * bs, c.a1 + q);
      stage_copy(st + (1 * R + r) * bs, c.a2 + q);
      stage_copy(st + (2 * R + r) * bs, c.a3 + q);
      stage_copy(st + (3 * R + r) * bs, c.b + q);
      stage_copy(st + (4 * R + r) * bs, c.a3p + q);
      stage_copy(st + (5 * R + r) * bs, c.bp + q);
    }
    stage_wait();
    for (int r = 0; r < m; ++r) {
      const T a1 = st[(0 * R + r) * bs];
      const T a2p = st[(1 * R + r) * bs] - a1 * a3p;
      const T nb = (st[(3 * R + r) * bs] - a1 * bp) / a2p;
      a3p = (k + r < c.n - 1) ? st[(2 * R + r) * bs] / a2p : T(0);
      bp = nb;
      if (same_state(a3p, st[(4 * R + r) * bs]) && same_state(bp, st[(5 * R + r) * bs])) {
        eout[2 * s] = ein[2 * s];
        eout[2 * s + 1] = ein[2 * s + 1];
        return false;
      }
      c.a3p[p + r * ns] = a3p;
      c.bp[p + r * ns] = bp;
    }
    k += m;
    p += m * ns;
  }
  eout[2 * s] = a3p;
  eout[2 * s + 1] = bp;
  return true;
}

template <class T>
__device__ void chain_b1(const ChainT<T> &c, int s, int L, int W, T *eb) {
  constexpr int R = RowBatch<T>::n;
  const int k0 = s * L, k1 = min(c.n, k0 + L), ns = c.nseg;
  const int plast = cpos(c, c.n - 1);
  T xn;
  int kown;
  if (k1 == c.n) {
    xn = c.bp[plast];
    c.x[plast] = xn;
    kown = c.n - 2;
  } else {
    const int kw = k1 - 1 + W;
    int kstart;
    if (kw >= c.n - 1) {
      xn = c.bp[plast];
      kstart = c.n - 2;
    } else {
      xn = T(0);
      kstart = kw;
    }
    RowWalk u(kstart, L, ns);
    while (u.k >= k1) bwd_batch<T, false>(c, u, min(R, u.k - k1 + 1), L, ns, xn);
    kown = k1 - 1;
  }
  if (kown >= k0) {
    RowWalk w(kown, L, ns);
    while (w.k >= k0) bwd_batch<T, true>(c, w, min(R, w.k - k0 + 1), L, ns, xn);
  }
  eb[s] = c.x[s];
}

template <class T>
__device__ bool chain_b2(const ChainT<T> &c, int s, int L, const T *ein, T *eout) {
  constexpr int R = RowBatch<T>::n;
  const int k0 = s * L, k1 = min(c.n, k0 + L), ns = c.nseg;
  if (k1 == c.n) {
    eout[s] = ein[s];
    return false;
  }
  T xn = ein[s + 1];
  int p = (k1 - 1 - k0) * ns + s;
  xn = c.bp[p] - c.a3p[p] * xn;
  if (same_state(xn, c.x[p])) {
    eout[s] = ein[s];
    return false;
  }
  c.x[p] = xn;
  p -= ns;
  T *st = walk_stage<T>();
  const int bs = blockDim.x;
  for (int k = k1 - 2; k >= k0;) {
    const int m = min(R, k - k0 + 1);
    for (int r = 0; r < m; ++r) {
      const int q = p - r * ns;
      stage_copy(st + (0 * R + r) * bs, c.bp + q);
      stage_copy(st + (1 * R + r) * bs, c.a3p + q);
      stage_copy(st + (2 * R + r) * bs, c.x + q);
    }
    stage_wait();
    for (int r = 0; r < m; ++r) {
      xn = st[(0 * R + r) * bs] - st[(1 * R + r) * bs] * xn;
      if (same_state(xn, st[(2 * R + r) * bs])) {
        eout[s] = ein[s];
        return false;
      }
      c.x[p - r * ns] = xn;
    }
    k -= m;
    p -= m * ns;
  }
  eout[s] = xn;
  return true;
}

// Sequential completion used when verification rounds do not settle: warp 0
// of block 0 walks the chain in chunks of 32 rows, the lanes staging each
// chunk's coefficients through shared memory and lane 0 running the
// recurrence (same arithmetic as fwd_row / the back substitution).
// The guard walk gives up after kGuardLimitNs, well inside the other blocks'
// barrier wait (kWaitLimitNs): it sets W2_E_FALLBACK, which those blocks see
// while they wait, so a chain too long to walk in time ends the launch with
// that status instead of a barrier timeout.
constexpr unsigned long long kGuardLimitNs = 1000000000ull;

// true (on every lane) once the guard walk started at t0 is out of time;
// the first lane to see it sets W2_E_FALLBACK.
__device__ __forceinline__ bool guard_out_of_time(Sync *sy, unsigned long long t0) {
  int late = 0;
  if ((threadIdx.x & 31) == 0 && gtime_ns() - t0 > kGuardLimitNs) {
    set_error(sy, W2_E_FALLBACK);
    late = 1;
  }
  return __shfl_sync(0xffffffffu, late, 0) != 0;
}

template <class T>
__device__ void chain_sequential_warp(const ChainT<T> &c, bool forward, Sync *sy) {
  __shared__ T s1[32], s2[32], s3[32], sb[32], o3[32], ob[32];
  const int lane = threadIdx.x & 31;
  const unsigned long long t0 = gtime_ns();
  if (forward) {
    T a3p = T(0), bp = T(0);
    for (int base = 0; base < c.n; base += 32) {
      if (guard_out_of_time(sy, t0)) return;
      const int k = base + lane, cnt = min(32, c.n - base);
      const int p = k < c.n ? cpos(c, k) : 0;
      if (k < c.n) {
        s1[lane] = c.a1[p];
        s2[lane] = c.a2[p];
        s3[lane] = c.a3[p];
        sb[lane] = chain_rhs(c, p);
      }
      __syncwarp();
      if (lane == 0) {
        for (int q = 0; q < cnt; ++q) {
          const int kk = base + q;
          if (kk == 0) {
            a3p = s3[0] / c.a2[cpos(c, 1)];
            bp = sb[0] / s2[0];
          } else {
            const T a1 = s1[q];
            const T a2p = s2[q] - a1 * a3p;
            const T nb = (sb[q] - a1 * bp) / a2p;
            a3p = (kk < c.n - 1) ? s3[q] / a2p : T(0);
            bp = nb;
          }
          o3[q] = a3p;
          ob[q] = bp;
        }
      }
      __syncwarp();
      if (k < c.n) {
        c.a3p[p] = o3[lane];
        c.bp[p] = ob[lane];
      }
      __syncwarp();
    }
  } else {
    T xn = T(0);
    for (int top = c.n - 1; top >= 0; top -= 32) {
      if (guard_out_of_time(sy, t0)) return;
      const int k = top - lane, cnt = min(32, top + 1);
      const int p = k >= 0 ? cpos(c, k) : 0;
      if (k >= 0) {
        s3[lane] = c.a3p[p];
        sb[lane] = c.bp[p];
      }
      __syncwarp();
      if (lane == 0) {
        for (int q = 0; q < cnt; ++q) {
          const int kk = top - q;
          xn = (kk == c.n - 1) ? sb[q] : sb[q] - s3[q] * xn;
          ob[q] = xn;
        }
      }
      __syncwarp();
      if (k >= 0) c.x[p] = ob[lane];
      __syncwarp();
    }
  }
}

// Views of a chain whose end-state buffers are swapped per round.
template <class T>
__device__ __forceinline__ const T *ef_buf(const ChainT<T> &c, int b) {
  return c.ef + (size_t)b * 2 * c.nseg;
}
template <class T>
__device__ __forceinline__ const T *eb_buf(const ChainT<T> &c, int b) {
  return c.eb + (size_t)b * c.nseg;
}

// Solve up to two independent chains together (segments of both share the
// grid).  Every block must call this.  Returns false if a barrier failed.
// The chains are taken by reference (they live in the kernel's parameter
// space) and each walk names its chain statically, so the walks read the
// array pointers from the parameter bank instead of holding them in
// registers.
template <class T>
__device__ bool solve_chains(const Dev &d, const ChainT<T> &c0, const ChainT<T> &c1, int nchains) {
  Sync *sy = d.sync;
  const int L = d.seg, W = d.warm;
  const int nseg0 = c0.nseg, nseg1 = nchains > 1 ? c1.nseg : 0;
  const int nsegt = nseg0 + nseg1;
  const int nrounds = max_rounds(nseg0, nseg1);
  // ---- F1
  for (int g = gtid(); g < nsegt; g += gthreads()) {
    if (g < nseg0) chain_f1(c0, g, L, W);
    else chain_f1(c1, g - nseg0, L, W);
  }
  // ---- F2 rounds (end-state buffers alternate 0 -> 1 -> 0 ...)
  int cur = 0;
  bool settled = false;
  for (int round = 0; round < nrounds; ++round) {
    if (vblock() == 0 && threadIdx.x == 0) {
      if (round == 0) sy->iout[0] = 0;
      sy->iout[(round + 1) % 3] = 0;
    }
    if (!grid_sync(sy)) return false;
    int any = 0;
    for (int g = gtid(); g < nsegt; g += gthreads()) {
      if (g < nseg0) {
        if (chain_f2(c0, g, L, ef_buf(c0, cur), const_cast<T *>(ef_buf(c0, cur ^ 1)))) any = 1;
      } else {
        if (chain_f2(c1, g - nseg0, L, ef_buf(c1, cur), const_cast<T *>(ef_buf(c1, cur ^ 1)))) any = 1;
      }
    }
    if (any) atomicOr(&sy->iout[round % 3], 1);
    if (!grid_sync(sy)) return false;
    int ch = cuda::atomic_ref<int, cuda::thread_scope_device>(sy->iout[round % 3])
                 .load(cuda::memory_order_acquire);
    cur ^= 1;
    if (!ch) {
      settled = true;
      if (vblock() == 0 && threadIdx.x == 0) atomicMax(&sy->max_rounds, round + 1);
      break;
    }
  }
  if (vblock() == 0 && threadIdx.x == 0 && !settled) atomicMax(&sy->max_rounds, nrounds + 1);
  if (!settled) {
    if (vblock() == 0 && threadIdx.x < 32) {
      // copies: the guard walk must not take the address of parameter space
      const ChainT<T> t0 = c0, t1 = c1;
      chain_sequential_warp(t0, true, sy);
      chain_sequential_warp(t0, false, sy);
      if (nchains > 1) {
        chain_sequential_warp(t1, true, sy);
        chain_sequential_warp(t1, false, sy);
      }
      if (threadIdx.x == 0) atomicAdd(&sy->fallback, 1);
    }
    if (!grid_sync(sy)) return false;
    return true;  // sequential pass produced a3p, bp and x
  }
  // ---- B1
  for (int g = gtid(); g < nsegt; g += gthreads()) {
    if (g < nseg0) chain_b1(c0, g, L, W, const_cast<T *>(eb_buf(c0, 0)));
    else chain_b1(c1, g - nseg0, L, W, const_cast<T *>(eb_buf(c1, 0)));
  }
  cur = 0;
  settled = false;
  for (int round = 0; round < nrounds; ++round) {
    if (vblock() == 0 && threadIdx.x == 0) {
      if (round == 0) sy->iout[3] = 0;
      sy->iout[3 + (round + 1) % 3] = 0;
    }
    if (!grid_sync(sy)) return false;
    int any = 0;
    for (int g = gtid(); g < nsegt; g += gthreads()) {
      if (g < nseg0) {
        if (chain_b2(c0, g, L, eb_buf(c0, cur), const_cast<T *>(eb_buf(c0, cur ^ 1)))) any = 1;
      } else {
        if (chain_b2(c1, g - nseg0, L, eb_buf(c1, cur), const_cast<T *>(eb_buf(c1, cur ^ 1)))) any = 1;
      }
    }
    if (any) atomicOr(&sy->iout[3 + round % 3], 1);
    if (!grid_sync(sy)) return false;
    int ch = cuda::atomic_ref<int, cuda::thread_scope_device>(sy->iout[3 + round % 3])
                 .load(cuda::memory_order_acquire);
    cur ^= 1;
    if (!ch) {
      settled = true;
      if (vblock() == 0 && threadIdx.x == 0) atomicMax(&sy->max_rounds, round + 1);
      break;
    }
  }
  if (!settled) {
    if (vblock() == 0 && threadIdx.x < 32) {
      // forward values are exact here; redo the back substitution serially
      const ChainT<T> t0 = c0, t1 = c1;
      chain_sequential_warp(t0, false, sy);
      if (nchains > 1) chain_sequential_warp(t1, false, sy);
      if (threadIdx.x == 0) atomicAdd(&sy->fallback, 1);
    }
    if (!grid_sync(sy)) return false;
  }
  return true;
}

}  // namespace w2
