// w2_ensemble.cuh -- many independent cases advanced together: one launch per
// stage of the time step (mixed, or plain FP64) covers every case.
//
// The launch's blocks are split into one group of consecutive blocks per
// case (a ragged partition, sized by the host to each case's cells).  A block
// finds its case in the group table, makes the group its virtual grid
// (vgrid_set), and runs the single-case stage code on the case's descriptor:
// its Dev (grids, metrics, chains, barrier state), its Poisson tile plan and
// the pointers of both time levels.  Every grid barrier, reduction and
// "block 0" duty is then per case, so cases of different sizes, Reynolds
// numbers and convergence histories run side by side and a case that stops
// early leaves its blocks idle until the launch ends.
//
// The step counter lives in device memory and a one-thread kernel advances
// it after each step, so the launch sequence of a step is the same every
// step and can be captured once in a CUDA graph and replayed.
#pragma once
#include "w2_kernels.cuh"

namespace w2 {

// One case of an ensemble (the ragged per-instance descriptor).
struct EnsCase {
  Dev d;                   // the case's view, chain segments set for its block group
  MixedGeom g;             // its Poisson tile plan (several tiles per block)
  MixedArgs a[2];          // Poisson arguments forming time level 0 / 1
  double *U[2], *V[2], *P[2];
  float *F32[4];           // un, vn, us, vs in single precision
  int cur;                 // time level holding the fields when the call starts
  int mqiter;
  double dk, re, qtol;
  int npsolver, lcartes, msorit;  // plain step's Ppe
  double sortol, sorrel;
  int general;             // Poisson rows not the unit stencil in FP32: the
  MixgArgs ga[2];          // general-row mixed Ppe, forming level 0 / 1
  int nfiltu, nfiltv;      // Filter of us, vs after nAuxMomentum (main.f:783-791)
  double fpu, fpv;
  double *hu, *hv;         // its results before they replace us, vs
};

// Arguments shared by the launches of one ensemble step.
struct EnsLaunch {
  const EnsCase *cs;
  const int *first;        // first block of each case's group (n + 1 entries)
  int n;
  const int *step;         // steps completed in this call
  StepOut *outs;           // n x nsteps records, case-major
  int nsteps;
};

// This block's case: the last group starting at or before blockIdx.x.
__device__ __forceinline__ int ens_enter(const int *first, int n) {
  int lo = 0, hi = n - 1;
  const int b = (int)blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  vgrid_set(first[lo], first[lo + 1] - first[lo]);
  return lo;
}

// Level `a` holds the current fields, `b` receives the new ones.
__device__ __forceinline__ int ens_level(const EnsCase &e, const EnsLaunch &L) {
  return (e.cur + *L.step) & 1;
}

__device__ __forceinline__ StepOut *ens_out(const EnsLaunch &L, int k) {
  return L.outs + (size_t)k * L.nsteps + *L.step;
}

__global__ void ke_copy_mixed(EnsLaunch L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int a = ens_level(e, L), b = a ^ 1;
  copy_mixed_body(e.d, e.P[b], e.P[a], e.U[a], e.V[a], e.F32[0], e.F32[1], e.F32[2], e.F32[3]);
}

template <bool POR>
__device__ __forceinline__ void ens_naux32(const EnsLaunch &L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int b = ens_level(e, L) ^ 1;
  naux32_body<POR>(e.d, e.mqiter, e.dk, e.re, e.qtol, e.F32[0], e.F32[1], e.F32[2], e.F32[3], e.U[b],
                   e.V[b], ens_out(L, k));
}

__global__ void __launch_bounds__(kMaxThreads, 1) ke_naux32(EnsLaunch L) { ens_naux32<false>(L); }

// With the porous terms compiled in: launched when some case has porous
// regions (the others skip the terms at run time).
__global__ void __launch_bounds__(kMaxThreads, 1) ke_naux32_por(EnsLaunch L) { ens_naux32<true>(L); }

// Filter of us and vs after nAuxMomentum (utility.f:33-247, main.f:783-791):
// phase 0 filters into the scratch fields, phase 1 copies them back (the
// filter of a cell reads its neighbours' unfiltered values, so the copy
// waits for the launch boundary).  Cases without Filter do nothing.
__global__ void ke_filter(EnsLaunch L, int phase) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt || !(e.nfiltu || e.nfiltv)) return;
  const int b = ens_level(e, L) ^ 1;
  const Dev &d = e.d;
  const int W = d.nx + 2, H = d.ny + 2;
  for (int t = gtid(); t < W * H; t += gthreads()) {
    const int i = t % W, j = t / W;
    const size_t o = IX(d, i, j);
    if (phase == 0) {
      if (e.nfiltu) e.hu[o] = filter_point(d, MK_FU, e.fpu, e.U[b], i, j);
      if (e.nfiltv) e.hv[o] = filter_point(d, MK_FV, e.fpv, e.V[b], i, j);
    } else {
      if (e.nfiltu) e.U[b][o] = e.hu[o];
      if (e.nfiltv) e.V[b][o] = e.hv[o];
    }
  }
}

// Boundary rows before the Poisson solve (one block per case).
__global__ void ke_bc(EnsLaunch L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int b = ens_level(e, L) ^ 1;
  bc_body(e.d, BC_VEL | BC_PRES, e.U[b], e.V[b], e.P[b]);
}

template <int K>
__global__ void __launch_bounds__(kMixedThreads, 1) ke_ppe_mixed(EnsLaunch L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int b = ens_level(e, L) ^ 1;
  const int msorit = e.general ? e.ga[b].msorit : e.a[b].msorit;
  const int nconv = e.general ? ppe_mixg(e.d, e.ga[b]) : ppe_mixed<K, false>(e.d, e.g, e.a[b]);
  if (nconv < 0) return;
  if (vblock() == 0 && threadIdx.x == 0) ens_out(L, k)->nsor = nconv < 1 ? msorit : nconv;
}

__global__ void __launch_bounds__(kMaxThreads) ke_step_post(EnsLaunch L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int a = ens_level(e, L), b = a ^ 1;
  step_post_body(e.d, e.dk, e.P[b], e.P[a], e.U[a], e.V[a], e.U[b], e.V[b], ens_out(L, k));
}

// ---- plain FP64 step: the single-case stage bodies on each case's group --

__global__ void ke_copy3(EnsLaunch L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int a = ens_level(e, L), b = a ^ 1;
  copy3_body(e.d, e.U[b], e.U[a], e.V[b], e.V[a], e.P[b], e.P[a]);
}

__global__ void __launch_bounds__(kMaxThreads, 1) ke_naux(EnsLaunch L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int a = ens_level(e, L), b = a ^ 1;
  int res = -1;
  if (!naux_momentum<double>(e.d, e.d.f64, e.mqiter, e.dk, e.re, e.qtol, e.U[a], e.V[a], e.U[b], e.V[b], &res))
    return;
  if (vblock() == 0 && threadIdx.x == 0) ens_out(L, k)->nql = res;
}

__global__ void __launch_bounds__(kMaxThreads) ke_ppe(EnsLaunch L) {
  const int k = ens_enter(L.first, L.n);
  const EnsCase &e = L.cs[k];
  if (e.d.sync->halt) return;
  const int b = ens_level(e, L) ^ 1;
  ppe_body(e.d, e.lcartes, e.npsolver, e.msorit, e.dk, e.sortol, e.sorrel, e.U[b], e.V[b], e.P[b],
           ens_out(L, k));
}

__global__ void ke_tick(int *step) { ++*step; }

}  // namespace w2
