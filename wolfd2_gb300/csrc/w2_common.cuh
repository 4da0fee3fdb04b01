// w2_common.cuh -- device-side context, bounded grid barrier and reductions
// shared by every persistent kernel of the wolfd2 GB300 time step.
//
// Field layout on the device: REAL*8 (0:nx+1, 0:ny+1) with i fastest and a
// padded leading dimension ld (a multiple of 32 elements, so every row starts
// on a 256-byte boundary).  Element (i,j) lives at i + j*ld.  Work arrays that
// the reference keeps as static locals are allocated zeroed once and reused,
// which gives the same "never written => 0" entries the reference reads
// (for example cj1(nx+1,j) in momentum.f:374).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cuda/atomic>

#include "../../include/wolfd2_gpu.h"

namespace w2 {

// Bits of the per-cell mask, built on the host from the region tables by
// replaying the reference's region loops.
enum : uint16_t {
  MK_XID = 1u << 0,   // X split-2 identity row   (momentum.f:444-496)
  MK_YID = 1u << 1,   // Y split-2 identity row   (momentum.f:770-821)
  MK_PU = 1u << 2,    // Project updates u(i,j)   (utility.f:301-366)
  MK_PV = 1u << 3,    // Project updates v(i,j)   (utility.f:371-437)
  MK_PID = 1u << 4,   // PPE identity row         (pressure.f:109-196)
  MK_DIVZ = 1u << 5,  // div(i,j) zeroed          (pressure.f:109-196)
  MK_FU = 1u << 6,    // Filter u at (i,j)        (utility.f:79-140)
  MK_FV = 1u << 7,    // Filter v at (i,j)        (utility.f:142-204)
  MK_PCX = 1u << 8,   // X PorosCoef value from a porous region (momentum.f:1186-1196)
  MK_PCY = 1u << 9,   // Y PorosCoef value from a porous region (momentum.f:1200-1209)
};

// Porous regions on the momentum path (FP64, and FP32 in the mixed step),
// from a host replay of the region loops: div[0..1] are the porosities the X division loop
// (momentum.f:296-324) applies to a cell, first and second (1 where it
// applies fewer: a cell on the shared border of two porous regions is
// divided twice), div[2..3] those of the Y loop (momentum.f:621-649);
// c1[k], c2[k] are porc1, porc2 of the porous region whose PorosCoef loop
// writes the cell last (k = 0 X, 1 Y; read where MK_PCX / MK_PCY is set).
struct Porous {
  const double *div[4];
  const double *c1[2], *c2[2];
  // the same tables rounded to FP32, for the mixed path's FP32 momentum
  const float *div32[4];
  const float *c1_32[2], *c2_32[2];
};

// Metric arrays (grid.f:368-535), device copies in the padded layout.
struct Metrics {
  const double *ran, *rbn, *rgn, *rac, *rbc, *rgc, *rau, *rbu, *rbv, *rgv;
  const double *dju, *djv, *djc, *djn;
  const double *xen, *yen, *xzn, *yzn, *xec, *yec, *xzc, *yzc;
  const double *xeu, *yeu, *xzv, *yzv, *xzu, *yzu, *xev, *yev;
};

// Region tables, Fortran layout (include/wolfd2.h, src/main.f:211-239).
struct Regions {
  int nri, nrj, mgri, mgrj;
  const int *brd;     // nRegBrd(mgri,mgrj,4)
  const int *rtype;   // nRegType(mgri,mgrj)
  const int *btype;   // nMomBdTp(mgri,mgrj,4)
  const double *bcv;  // dBCVal(mgri,mgrj,4,4)
  __device__ __forceinline__ int B(int ir, int jr, int s) const {
    return brd[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj];
  }
  __device__ __forceinline__ int RT(int ir, int jr) const {
    return rtype[(ir - 1) + (jr - 1) * mgri];
  }
  __device__ __forceinline__ int BT(int ir, int jr, int s) const {
    return btype[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj];
  }
  __device__ __forceinline__ double BV(int ir, int jr, int s, int var) const {
    return bcv[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj +
               (var - 1) * mgri * mgrj * 4];
  }
};

// A concatenated tridiagonal chain solved by AltTridLU semantics
// (momentum.f:1307-1339): forward elimination over all n rows in order,
// row 1's super-diagonal divided by row 2's original diagonal.  T is the
// arithmetic type (double for the plain path, float for the mixed one).
template <class T>
struct ChainT {
  int n;           // rows
  int nseg;        // segments of L rows (the last may be shorter)
  int L;           // rows per segment; row r of segment s is stored at r*nseg + s
  T *a1, *a2, *a3, *b;             // sub, diag, super, rhs
  T *a3p, *bp, *x;                 // factorised super, forward rhs, solution
  T *ef;           // forward end states: 2 per segment x 2 buffers
  T *eb;           // backward end states: 1 per segment x 2 buffers
};
using Chain = ChainT<double>;

// A metric array as the momentum stencils read it: value(i, j) =
// p[i*si + j*sj].  A full array has (si, sj) = (1, ld); an array that the
// host found to depend on i only (every column equal, bit for bit) is a
// profile over i with sj = 0, one that depends on j only a profile over j
// with si = 0, a constant has si = sj = 0.  On Cartesian grids most metric
// arrays collapse this way, so the stencils stream no metric data.
template <class T>
struct MRef {
  const T *p;
  int si, sj;
  __device__ __forceinline__ T operator()(int i, int j) const { return p[i * si + j * sj]; }
};

// The momentum step's inputs and work arrays in one arithmetic type: the
// metric arrays the stencils read, the ConvCoef outputs and the four chains
// (split 2 reuses the storage of split 1, whose rows are dead by then).
template <class T>
struct MomView {
  MRef<T> yeu, xeu, xzu, yzu, yec, xec, xzn, yzn;
  MRef<T> yev, xev, xzv, yzv, yen, xen, xzc, yzc;
  MRef<T> dju, djv, rac, rbc, rbn, rgn, ran, rgc;
  T *cj1x, *cj2x, *c1sx, *c2sx, *c1nx, *c2nx;  // ConvCoef outputs (FP64 only)
  T *cj1y, *cj2y, *c1sy, *c2sy, *c1ny, *c2ny;
  ChainT<T> x1, x2, y1, y2;
};

// Grid-wide synchronisation state in device memory.
struct Sync {
  unsigned int count;
  unsigned int gen;
  int error;          // sticky W2_E_* code
  int changed;        // chain verification rounds: "some segment moved"
  int fallback;       // chain recurrence needed a sequential pass
  int pad0;
  int halt;           // a step diverged: later stages of the run are skipped
  int max_rounds;     // most verification rounds any chain solve needed
  unsigned long long red[48];  // max-reductions (bit patterns of doubles >= 0):
                               // [0..2] momentum ring, [3..5] PPE ring,
                               // [6..8] step norms, [9] scratch, [10..15]
                               // tiled PPE ring, [16] divergence check,
                               // [17..40] mixed PPE ring, [41..44]
                               // momentum/energy norms, [45] interior
                               // divergence check
  int iout[8];                 // chain verification flags ([0..2] fwd, [3..5] bwd)
  double dout[8];              // small double results
  int me_done;                 // the momentum/energy iterations of this step converged
};

struct Dev {
  int nx, ny, ld;
  Metrics m;
  Regions r;
  const uint16_t *mask;
  // per-position face values: prof_idx[((ir-1) + (jr-1)*mgri + (face-1)*mgri*mgrj)*2
  // + var-1] is -1 or the offset of the values in prof (null: none set)
  const int *prof_idx;
  const double *prof;
  // fields of the device-resident time loop
  double *u, *v, *p, *un, *vn, *pn, *us, *vs;
  // momentum work arrays (X: cj1x..c2nx; Y: cj1y..c2ny)
  double *cj1x, *cj2x, *c1sx, *c2sx, *c1nx, *c2nx;
  double *cj1y, *cj2y, *c1sy, *c2sy, *c1ny, *c2ny;
  Chain x1, x2, y1, y2;
  // PPE: coefficients a(ind,1..5) and rhs/divergence, field layout
  double *pa1, *pa2, *pa3, *pa4, *pa5;
  double *div, *pb, *ppn;
  double *la3p, *lbp;  // line-solver scratch (field layout)
  double *qh;          // filter scratch
  MomView<double> f64; // momentum view of the plain path
  MomView<float> f32;  // single-precision momentum (mixed path)
  Sync *sync;
  int seg, warm;       // chain segment length and warm-up rows
  int has_outflow;     // any OUTLT1/OUTLT2 face (VelOutflowBCs not a no-op)
  int ppe_unit;        // every PPE row is the unit stencil (1,1,-4,1,1)
  int ppe_unit32;      // every PPE row rounds to the unit stencil in FP32 (no
                       // identity rows): any uniform square-cell Cartesian grid
  // density at the starred and time-level-n states for the buoyancy term of
  // YMomentum (momentum.f:703), FP64 path; null when the density is zero
  const double *den, *denn;
  double fr;
  int porous;          // porous regions present (tables in por)
  Porous por;
  int me_gate;         // a launch of momentum/energy iteration >= 2: skipped once they converged
};

__device__ __forceinline__ size_t IX(const Dev &d, int i, int j) {
  return (size_t)i + (size_t)j * (size_t)d.ld;
}

__device__ __forceinline__ unsigned long long gtime_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Time limit of every device-side wait.
constexpr unsigned long long kWaitLimitNs = 4000000000ull;

__device__ __forceinline__ void set_error(Sync *s, int code) {
  atomicCAS(&s->error, 0, code);
}

__device__ __forceinline__ int read_error(Sync *s) {
  return cuda::atomic_ref<int, cuda::thread_scope_device>(s->error).load(
      cuda::memory_order_acquire);
}

// A launch of the time step skips its work once the run has halted (a step
// diverged) or, inside momentum/energy iterations 2.., once they converged.
__device__ __forceinline__ bool step_skip(const Dev &d) {
  return d.sync->halt || (d.me_gate && d.sync->me_done);
}

// ---- virtual grid ---------------------------------------------------------
// The blocks that work on one case: a single-case launch is its own virtual
// grid; an ensemble launch gives each case a group of consecutive blocks.
// Every kernel sets it at entry (vgrid_set), and device routines index,
// reduce and synchronise within it (vblock, vblocks, gtid, gthreads,
// grid_sync).
struct VGrid {
  int first, count;
};
__device__ __forceinline__ VGrid &vgrid_slot() {
  __shared__ VGrid g;
  return g;
}
// Every thread of the block writes the same values, so each thread reads
// back what it wrote without a block barrier.
__device__ __forceinline__ void vgrid_set(int first, int count) { vgrid_slot() = VGrid{first, count}; }
__device__ __forceinline__ int vblock() { return (int)blockIdx.x - vgrid_slot().first; }
__device__ __forceinline__ int vblocks() { return vgrid_slot().count; }
__device__ __forceinline__ int gtid() { return vblock() * (int)blockDim.x + (int)threadIdx.x; }
__device__ __forceinline__ int gthreads() { return vblocks() * (int)blockDim.x; }

// Grid barrier with a time limit.  All blocks of a cooperative launch call
// it the same number of times.  Thread 0 of each block arrives with one
// acquire-release add on the counter (the block's writes are ordered before
// it by the __syncthreads); the last arriver resets the counter and
// publishes the next generation with a release store, and the others poll
// the generation with acquire loads.  No device-wide fences and no sleep in
// the poll: measured 1.9 us per barrier on 152 blocks against 3.0 us with
// them.  A block whose wait runs out its time limit sets the sticky timeout
// error and returns false, as does one that sees an error while it waits;
// its callers leave the kernel, and the remaining blocks end at their next
// wait's limit.  Other errors set during a launch reach the host after it.
static __device__ __noinline__ bool grid_sync(Sync *s) {
  __shared__ int ok;
  __syncthreads();
  if (vblocks() == 1) {
    if (threadIdx.x == 0) ok = (read_error(s) == 0);
    __syncthreads();
    return ok;
  }
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(s->gen), cnt(s->count);
    // the generation cannot move before this block arrives, and this thread
    // last saw its current value (or published it), so a relaxed read is exact
    const unsigned g = gen.load(cuda::memory_order_relaxed);
    int good = 1;
    if (cnt.fetch_add(1u, cuda::memory_order_acq_rel) == (unsigned)vblocks() - 1u) {
      cnt.store(0u, cuda::memory_order_relaxed);
      gen.store(g + 1u, cuda::memory_order_release);
    } else {
      const unsigned long long t0 = gtime_ns();
      unsigned spins = 0;
      while (gen.load(cuda::memory_order_acquire) == g) {
        if ((++spins & 63u) == 0) {
          if (read_error(s) != 0) {
            good = 0;
            break;
          }
          if (gtime_ns() - t0 > kWaitLimitNs) {
            set_error(s, W2_E_TIMEOUT);
            good = 0;
            break;
          }
        }
      }
    }
    ok = good;
  }
  __syncthreads();
  return ok;
}

// Block-wide max of non-negative doubles, then one atomicMax per block on the
// IEEE bit pattern (order-preserving for values >= 0, so the max is exact).
__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// |x| as an IEEE bit pattern by clearing the sign bit: an integer AND, where
// fabs() on a double costs an FP64-pipe instruction on this part.  Bit-equal
// to dbits(fabs(x)) for every x.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return dbits(x) & 0x7fffffffffffffffull;
}

static __device__ __noinline__ void block_max_to(unsigned long long *slot, double v) {
  __shared__ unsigned long long wmax[32];
  unsigned long long b = dbits(v);
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
    b = t > b ? t : b;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wmax[w] = b;
  __syncthreads();
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    b = lane < nw ? wmax[lane] : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
      b = t > b ? t : b;
    }
    if (lane == 0 && b != 0ull) atomicMax(slot, b);
  }
  __syncthreads();
}

__device__ __forceinline__ double slot_value(const unsigned long long *slot) {
  unsigned long long b = cuda::atomic_ref<const unsigned long long, cuda::thread_scope_device>(*slot)
                             .load(cuda::memory_order_relaxed);
  return __longlong_as_double((long long)b);
}

// Max helper matching the reference's dmax1/max on non-NaN values.
__device__ __forceinline__ double dmax(double a, double b) { return b > a ? b : a; }



}  // namespace w2
