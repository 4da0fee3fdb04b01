// w2_noalloc.cu -- allocation-free red/black Ppe on caller-owned device memory.
//
// Some callers cannot call cudaMalloc.  Examples: a driver that hands the
// whole device memory to its own pool at start-up, and code that must not
// touch the allocator once its solve loop is running.  Those callers cannot
// create a w2_ctx, which allocates its work arrays.  This entry point runs
// the same red/black point SOR as wolfd2gpu_ppe with nPpeSolver 5 or 6
// (src/pressure.f:457-656, with the divergence and right-hand side of
// pressure.f:287-299 and 354-359) directly on device arrays the caller
// passes.  Its only scratch -- grid-barrier state, the per-sweep maxima and
// the right-hand side b -- lives in the fixed-size file-scope array below,
// so the call itself allocates nothing.
//
// Limits: Cartesian grids only (lCartesGrid = 1), region layouts without
// blockages (no identity rows), and ld*(ny+2) <= W2_NOALLOC_MAX_POINTS.
// Every call on a device shares the one scratch array and leaves its
// contents behind; each call clears the barrier and reduction state before
// use.  Two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on that array and give wrong results, so
// callers serialise them.  A call waits for its stream and copies its result
// to the host before returning, so it cannot be recorded into a CUDA graph
// by stream capture.
#include <cuda_runtime.h>

#include <cstdio>

#include "w2_common.cuh"

namespace {

constexpr size_t kMaxPoints = W2_NOALLOC_MAX_POINTS;
constexpr size_t kSyncBytes = (sizeof(w2::Sync) + 255) / 256 * 256;
constexpr size_t kScratchBytes = kSyncBytes + kMaxPoints * sizeof(double);

}  // namespace

// The scratch: barrier/reduction state, then b.  About 9.6 MB per device,
// held by every GPU that loads this library until the process exits.
static __device__ __align__(256) unsigned char w2_noalloc_scratch[kScratchBytes];

namespace {

struct NaArgs {
  int nx, ny, ld, msorit;
  double dk, sortol, sorrel;
  const double *rau, *rgv, *xeu, *yeu, *xzv, *yzv, *u, *v;
  double *p;
  unsigned char *scratch;  // device address of w2_noalloc_scratch
};

__device__ __forceinline__ size_t NI(const NaArgs &a, int i, int j) {
  return (size_t)i + (size_t)j * (size_t)a.ld;
}

// One point of SorRB with the coefficients of pressure.f:97-106 formed in
// place from rau and rgv (same expressions, so the same bits as the stored
// a(ind,1..5)).
__device__ __forceinline__ double na_point(const NaArgs &a, const double *b, int i, int j) {
  const size_t o = NI(a, i, j), w = NI(a, i - 1, j), s = NI(a, i, j - 1);
  const double a1 = a.rgv[s], a2 = a.rau[w], a4 = a.rau[o], a5 = a.rgv[o];
  const double a3 = -a.rau[o] - a.rau[w] - a.rgv[o] - a.rgv[s];
  double sum = b[o] - a1 * a.p[s] - a2 * a.p[w] - a4 * a.p[NI(a, i + 1, j)] -
               a5 * a.p[NI(a, i, j + 1)];
  sum = sum / a3 - a.p[o];
  a.p[o] = a.p[o] + a.sorrel * sum;
  return sum;
}

__global__ void __launch_bounds__(512) k_ppe_noalloc(NaArgs a) {
  w2::vgrid_set(0, gridDim.x);
  w2::Sync *sy = reinterpret_cast<w2::Sync *>(a.scratch);
  double *b = reinterpret_cast<double *>(a.scratch + kSyncBytes);
  const int nx = a.nx, ny = a.ny;
  // Divergence nloc = 1 and b = div/dk on the unknowns (2..nx, 2..ny)
  for (int t = w2::gtid(); t < (nx - 1) * (ny - 1); t += w2::gthreads()) {
    const int i = t % (nx - 1) + 2, j = t / (nx - 1) + 2;
    const size_t o = NI(a, i, j), ow = NI(a, i - 1, j), os = NI(a, i, j - 1);
    const double *u = a.u, *v = a.v;
    const double ucij = a.yeu[o] * u[o] -
                        a.xeu[o] * (v[NI(a, i + 1, j)] + v[o] + v[NI(a, i + 1, j - 1)] + v[os]) / 4.0;
    const double uci1j = a.yeu[ow] * u[ow] -
                         a.xeu[ow] * (v[o] + v[ow] + v[os] + v[NI(a, i - 1, j - 1)]) / 4.0;
    const double vcij = a.xzv[o] * v[o] -
                        a.yzv[o] * (u[NI(a, i, j + 1)] + u[NI(a, i - 1, j + 1)] + u[o] + u[ow]) / 4.0;
    const double vcij1 = a.xzv[os] * v[os] -
                         a.yzv[os] * (u[o] + u[ow] + u[os] + u[NI(a, i - 1, j - 1)]) / 4.0;
    const double div = ucij - uci1j + vcij - vcij1;
    b[o] = div / a.dk;
  }
  if (!w2::grid_sync(sy)) return;
  int nconv = 0;
  const int nh = (nx - 2) / 2 + 1;
  for (int it = 1; it <= a.msorit; ++it) {
    unsigned long long *slot = &sy->red[it % 3];
    if (w2::vblock() == 0 && threadIdx.x == 0) sy->red[(it + 1) % 3] = 0ull;
    unsigned long long mx = 0ull;
    for (int parity = 0; parity < 2; ++parity) {
      for (int t = w2::gtid(); t < nh * (ny - 1); t += w2::gthreads()) {
        const int j = t / nh + 2;
        const int i = 2 + ((j + parity) & 1) + 2 * (t % nh);
        if (i > nx) continue;
        const unsigned long long q = w2::abs_bits(na_point(a, b, i, j));
        mx = q > mx ? q : mx;
      }
      if (parity == 0 && !w2::grid_sync(sy)) return;
    }
    w2::block_max_to(slot, __longlong_as_double((long long)mx));
    if (!w2::grid_sync(sy)) return;
    if (it > 1 && w2::slot_value(slot) < a.sortol) {
      nconv = it;
      break;
    }
  }
  if (w2::vblock() == 0 && threadIdx.x == 0) sy->iout[0] = nconv < 1 ? a.msorit : nconv;
}

// The device address of the scratch array on the current device.  In host
// code the array's name is only a host-side stand-in for the symbol, so the
// kernel is given this address instead.  It is looked up on every call (the
// call's set-up, with the caller's device current): the lookup allocates
// nothing and is cheap, and an address cached across calls would go stale
// if the device's primary context were reset in between (cudaDeviceReset
// by anyone in the process), after which the module -- and the array with
// it -- can be loaded at another address.
int scratch_address(void **out) {
  void *ptr = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&ptr, w2_noalloc_scratch);
  if (e != cudaSuccess || ptr == nullptr) {
    fprintf(stderr, "wolfd2gpu_ppe_rbsor_noalloc: cudaGetSymbolAddress failed: %s\n",
            cudaGetErrorString(e));
    return W2_E_CUDA;
  }
  *out = ptr;
  return W2_OK;
}

}  // namespace

extern "C" int wolfd2gpu_ppe_rbsor_noalloc(int nx, int ny, int ld, int lCartesGrid,
                                           int nPpeSolver, int msorit, double dk,
                                           double sortol, double sorrel, const double *rau,
                                           const double *rgv, const double *xeu,
                                           const double *yeu, const double *xzv,
                                           const double *yzv, const double *u,
                                           const double *v, double *p, int *nSorConv,
                                           void *stream) {
  if (nx < 6 || ny < 6 || ld < nx + 2 || msorit < 1 || !nSorConv || !rau || !rgv || !xeu ||
      !yeu || !xzv || !yzv || !u || !v || !p)
    return W2_E_ARG;
  if (nPpeSolver != 5 && nPpeSolver != 6) return W2_E_UNSUPPORTED;
  if (!lCartesGrid) return W2_E_UNSUPPORTED;
  if ((size_t)ld * (size_t)(ny + 2) > kMaxPoints) {
    fprintf(stderr,
            "wolfd2gpu_ppe_rbsor_noalloc: ld*(ny+2) = %zu exceeds the fixed scratch of %zu "
            "points (W2_NOALLOC_MAX_POINTS)\n",
            (size_t)ld * (size_t)(ny + 2), kMaxPoints);
    return W2_E_SIZE;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return W2_E_CUDA;
  void *scr = nullptr;
  int rc = scratch_address(&scr);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // clear the barrier/reduction state left by the previous call
  if (cudaMemsetAsync(scr, 0, sizeof(w2::Sync), st) != cudaSuccess) return W2_E_CUDA;
  int nsm = 0, occ = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)k_ppe_noalloc, threads, 0);
  if (occ < 1) return W2_E_CUDA;
  long work = (long)(nx - 1) * (ny - 1);
  long want = (work + 4095) / 4096;
  if (want > 1) want = want < nsm ? nsm : want;
  int blocks = (int)(want < 1 ? 1 : (want > (long)nsm * (occ < 2 ? occ : 2) ? (long)nsm * (occ < 2 ? occ : 2) : want));
  NaArgs a{nx, ny, ld, msorit, dk, sortol, sorrel, rau, rgv, xeu, yeu, xzv, yzv, u, v, p,
           (unsigned char *)scr};
  void *args[] = {&a};
  if (cudaLaunchCooperativeKernel((const void *)k_ppe_noalloc, dim3(blocks), dim3(threads), args, 0,
                                  st) != cudaSuccess)
    return W2_E_CUDA;
  w2::Sync hs;
  if (cudaMemcpyAsync(&hs, scr, sizeof(w2::Sync), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return W2_E_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return W2_E_CUDA;
  if (hs.error) return hs.error;
  *nSorConv = hs.iout[0];
  return W2_OK;
}
