// w2_api.cu -- host side of the wolfd2 GB300 library: context, device memory,
// region masks, launches, and the C-ABI declared in include/wolfd2_gpu.h.
//
// Compiled for sm_103a with -fmad=false: the FP64 kernels evaluate every
// reference expression operation by operation, so their results are the
// IEEE-double results of the reference source as written.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "w2_adjoint.cuh"
#include "w2_atd.cuh"
#include "w2_ensemble.cuh"
#include "w2_thermal.cuh"

using namespace w2;

// NVTX range over a public call (header-only NVTX v3: a no-op unless a
// profiler or tracer is attached).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

struct w2_ctx {
  int mnx = 0, mny = 0, mgri = 0, mgrj = 0, nx = 0, ny = 0, ld = 0;
  int device = 0, nsm = 0;
  cudaStream_t st = nullptr;
  size_t nf = 0;  // device field length (elements)
  std::vector<void *> allocs;
  Dev dev{};
  double *met[W2_NMETRIC] = {};
  double *U[2] = {}, *V[2] = {}, *P[2] = {};
  int cur = 0;
  double *stage[6] = {};  // drop-in staging: a, b, c, d, e, f
  AtdState atd{};         // SmallScale's saved state (allocated on its first call)
  double *atd_io[4] = {}; // SmallScale's uss, vss, pss, tss on the device
  StepOut *d_out = nullptr;
  StepOut *h_out = nullptr;  // pinned
  int threads = 256, blocks_per_sm = 2, seg_req = 0, warm_req = 0;
  bool metrics_ok = false, porous = false;
  long long launches = 0;
  char err[512] = {0};
  std::vector<int> tab_brd, tab_rtype, tab_btype;
  std::vector<double> tab_bcv;
  std::vector<double> tab_por, tab_porc1, tab_porc2;  // dPRporos, dPRporc1, dPRporc2
  int nri = 0, nrj = 0;
  // per-kernel event timing (wolfd2gpu_profile)
  bool prof_on = false;
  struct Rec { int kind; cudaEvent_t a, b; };
  std::vector<Rec> prof_pending;
  std::vector<cudaEvent_t> ev_pool;
  double prof_ms[W2_K_NKINDS] = {};
  long long prof_n[W2_K_NKINDS] = {};
  // tiled red/black sweeps
  bool tiled_ok = false;
  int tiled_blocks = 0, tiled_threads = 512;
  int tiled_wide = 0;     // 1024-thread blocks, two points in flight per thread
  size_t tiled_smem = 0;
  TileGeom tg{};
  int use_tiled = 1;
  int use_tma = 1;        // TMA staging of multi-tile mixed Poisson boxes
  // mixed-precision Poisson sweeps
  float *xbuf = nullptr;  // two exchange buffers of 2 colour planes each
  size_t xbuf_floats = 0;
  CUtensorMap *d_tm = nullptr;  // TMA maps of the two exchange buffers and r (multi-tile plans)
  bool tm_ok = false;
  bool mixed_ok = false;
  int mixed_K = 8, mixed_threads = kMixedThreads, mixed_blocks = 0;
  int mixed_mode = 0;  // 0 auto, 1 multi-tile, 2 multi-tile on at most 16 blocks,
                       // 3 one tile per block with two blocks per SM
  size_t mixed_smem = 0;
  MixedGeom mg{};
  // mixed Poisson sweeps with the grid's own rows (grids whose rows are not
  // the unit stencil in FP32, blockages, curvilinear grids), made on first use
  float *mgbuf = nullptr;       // MG_PLANES colour-split planes
  float *mg_rb = nullptr;       // FP32 rbu, rbv in field layout
  bool mg_coef_ok = false;      // coefficient planes of the current metrics
  // its tiled form (Cartesian grids): tile plan, buffers (c1..c5, r, e0, e1
  // in field layout), and the switch between the two forms
  bool mgt_ok = false;
  MixgtGeom mgt{};
  int mgt_blocks = 0;
  size_t mgt_smem = 0;
  float *mgt_buf = nullptr;
  int use_mixgt = 1;
  int prec_dropin = W2_PREC_FP64, refine_dropin = 0;
  // single-precision momentum state (mixed path), made on first use
  bool f32_alloc = false, f32_metrics_ok = false;
  float *F32[4] = {};  // un, vn, us, vs
  // step records of wolfd2gpu_step (persistent, so captured graphs keep their address)
  StepOut *d_outs = nullptr;
  int outs_cap = 0;
  // CUDA graphs of whole wolfd2gpu_step calls, keyed by everything their
  // launches bake in (starting level, step count, parameters, device view,
  // tile plans, launch shapes)
  bool graph_on = true;
  struct Graph { cudaGraphExec_t exec; long long launches; };
  std::vector<std::pair<std::string, Graph>> graphs;
  // adjoint work state (made on first use): the transposed chains and the
  // saved split-1 rows and solutions
  bool adj_alloc = false;
  Chain adj_tx{}, adj_ty{};
  double *adj_rows[8] = {};
  // thermal energy (made on first use): the chain of the (nx-1)(ny-1)
  // interior points and the thermal region tables of the current call
  bool therm_alloc = false;
  Chain therm_ch{};
  int *d_ttab = nullptr;     // nTRgType(mgri,mgrj) then nTemBdTp(mgri,mgrj,4)
  double *d_tval = nullptr;  // dTRgVal(mgri,mgrj) then dHGSTval(mgri,mgrj)
  int *d_trt_filter = nullptr;  // nTRgType of the drop-in Filter of t
  // the time loop with the energy equation (wolfd2gpu_set_thermal): its
  // switches, tables, temperature levels, density d / dn, and the previous
  // iterates of the momentum/energy iterations
  // snapshots (wolfd2gpu_snapshot): a copy stream, the events ordering it
  // after the step that made the level and before the step that overwrites it
  cudaStream_t cst = nullptr;
  cudaEvent_t ev_snap_src = nullptr, ev_snap_done = nullptr;
  int snap_level = -1;  // time level a copy may still be reading, or -1
  bool therm_on = false;
  w2_thermal therm_p{};
  ThermTables therm_tt{};
  double *T[2] = {}, *Dd = nullptr, *Ddn = nullptr, *Up = nullptr, *Vp = nullptr, *Tp = nullptr;
  // per-position face values (wolfd2gpu_set_face_profile)
  int *prof_idx = nullptr;   // device table, -1 = region constant
  double *prof = nullptr;    // device values, kMaxProfiles x prof_len
  int prof_len = 0, prof_used = 0;
  std::vector<int> prof_host;
  // how each momentum metric is read (full array, profile over i or j)
  struct MomMetric {
    int mode = 0;          // MP_FULL, MP_I, MP_J
    std::vector<double> host;  // the profile (MP_I: over i, MP_J: over j)
    double *p64 = nullptr;     // device profile, FP64
    float *p32 = nullptr;      // device profile or full array, FP32
  } mm[24];
};

// cuTensorMapEncodeTiled from the driver the runtime uses (no link to
// libcuda), fetched once.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

bool w2_encode_plane_map(CUtensorMap *map, const float *base, int gw, int gh, int hw, int bh) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || !base || ((uintptr_t)base & 15u) || (gw % 4) || (hw % 4) || hw < 4 || hw > 256 || bh < 1 ||
      bh > 256 || hw > gw || bh > gh)
    return false;
  const cuuint64_t dims[3] = {(cuuint64_t)gw, (cuuint64_t)gh, 2};
  const cuuint64_t strides[2] = {(cuuint64_t)gw * 4, (cuuint64_t)gw * gh * 4};
  const cuuint32_t box[3] = {(cuuint32_t)hw, (cuuint32_t)bh, 2};
  const cuuint32_t es[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The three maps (exchange buffers 0 and 1, r) of a multi-tile mixed plan
// over the buffer xb (3 x 2 planes of gh x gw), into dev[0..2].  False when
// a box breaks the TMA rules.
static bool encode_mixed_maps(CUtensorMap *dev, const float *xb, const MixedGeom &g, int K, cudaStream_t st) {
  // a box's x origin (tile column ti * tx/2 floats) must be a multiple of
  // 16 bytes: tx a multiple of 8, as both planners make it
  if (g.resident || g.tx % 8 != 0) return false;
  const size_t plane2 = 2 * (size_t)g.gh * g.gw;
  const int hw = g.tx / 2 + 2 * K, bh = g.ty + 4 * K;
  CUtensorMap h[3];
  for (int k = 0; k < 3; ++k)
    if (!w2_encode_plane_map(&h[k], xb + k * plane2, g.gw, g.gh, hw, bh)) return false;
  return cudaMemcpyAsync(dev, h, sizeof h, cudaMemcpyHostToDevice, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
}

namespace {

int fail(w2_ctx *c, int code, const char *fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(c, W2_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));   \
  } while (0)

template <class T>
T *dalloc(w2_ctx *c, size_t n) {
  void *p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T));
  c->allocs.push_back(p);
  return (T *)p;
}

// Metric order of the C-ABI (grid.f:Grid argument order).
enum {
  M_RAU, M_RBU, M_RBV, M_RGV, M_RAN, M_RBN, M_RGN, M_RAC, M_RBC, M_RGC, M_DJU, M_DJV, M_DJC,
  M_DJN, M_XEN, M_YEN, M_XZN, M_YZN, M_XEC, M_YEC, M_XZC, M_YZC, M_XEU, M_YEU, M_XZV, M_YZV,
  M_XZU, M_YZU, M_XEV, M_YEV
};

void bind_metrics(w2_ctx *c) {
  Metrics &m = c->dev.m;
  double **a = c->met;
  m.rau = a[M_RAU]; m.rbu = a[M_RBU]; m.rbv = a[M_RBV]; m.rgv = a[M_RGV];
  m.ran = a[M_RAN]; m.rbn = a[M_RBN]; m.rgn = a[M_RGN];
  m.rac = a[M_RAC]; m.rbc = a[M_RBC]; m.rgc = a[M_RGC];
  m.dju = a[M_DJU]; m.djv = a[M_DJV]; m.djc = a[M_DJC]; m.djn = a[M_DJN];
  m.xen = a[M_XEN]; m.yen = a[M_YEN]; m.xzn = a[M_XZN]; m.yzn = a[M_YZN];
  m.xec = a[M_XEC]; m.yec = a[M_YEC]; m.xzc = a[M_XZC]; m.yzc = a[M_YZC];
  m.xeu = a[M_XEU]; m.yeu = a[M_YEU]; m.xzv = a[M_XZV]; m.yzv = a[M_YZV];
  m.xzu = a[M_XZU]; m.yzu = a[M_YZU]; m.xev = a[M_XEV]; m.yev = a[M_YEV];
}

// The 24 metric arrays the momentum stencils read, in MomView order.
const int kMomMetric[24] = {M_YEU, M_XEU, M_XZU, M_YZU, M_YEC, M_XEC, M_XZN, M_YZN,
                            M_YEV, M_XEV, M_XZV, M_YZV, M_YEN, M_XEN, M_XZC, M_YZC,
                            M_DJU, M_DJV, M_RAC, M_RBC, M_RBN, M_RGN, M_RAN, M_RGC};
enum { MP_FULL = 0, MP_I = 1, MP_J = 2 };

// The 24 metric references of a momentum view, in MomView order.
template <class T>
std::vector<MRef<T> *> mom_refs(MomView<T> &v) {
  return {&v.yeu, &v.xeu, &v.xzu, &v.yzu, &v.yec, &v.xec, &v.xzn, &v.yzn,
          &v.yev, &v.xev, &v.xzv, &v.yzv, &v.yen, &v.xen, &v.xzc, &v.yzc,
          &v.dju, &v.djv, &v.rac, &v.rbc, &v.rbn, &v.rgn, &v.ran, &v.rgc};
}

// Host replay of the reference's region loops into per-cell mask bits.
int build_masks(w2_ctx *c, std::vector<uint16_t> &mk) {
  const int nx = c->nx, ny = c->ny, ld = c->ld, mgri = c->mgri, mgrj = c->mgrj;
  mk.assign(c->nf, 0);
  std::vector<uint8_t> pu(c->nf, 0), pv(c->nf, 0);
  auto B = [&](int ir, int jr, int s) { return c->tab_brd[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto RT = [&](int ir, int jr) { return c->tab_rtype[(ir - 1) + (jr - 1) * mgri]; };
  auto BT = [&](int ir, int jr, int s) { return c->tab_btype[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto at = [&](int i, int j) -> uint16_t & { return mk[(size_t)i + (size_t)j * ld]; };
  auto inb = [&](int i, int j) { return i >= 0 && i <= nx + 1 && j >= 0 && j <= ny + 1; };
  for (int jr = 1; jr <= c->nrj; jr++)
    for (int ir = 1; ir <= c->nri; ir++) {
      const int iW = B(ir, jr, W2_WEST), iE = B(ir, jr, W2_EAST);
      const int jS = B(ir, jr, W2_SOUTH), jN = B(ir, jr, W2_NORTH);
      if (iW < 1 || iE > nx || jS < 1 || jN > ny || iW >= iE || jS >= jN)
        return fail(c, W2_E_ARG, "region %d,%d borders out of range", ir, jr);
      for (int s = 1; s <= 4; ++s) {
        int t = BT(ir, jr, s);
        if (t < W2_BM_INTERN || t > W2_BM_OUTLT2)
          return fail(c, W2_E_BCFLAG, "Wrong nBdType flag in region %d,%d", ir, jr);
      }
      const int rt = RT(ir, jr);
      if (rt == W2_RM_POROUS) c->porous = true;
      // X split-2 identity rows, momentum.f:444-496
      if (rt == W2_RM_BLOCKG)
        for (int j = jS + 1; j <= jN; j++)
          for (int i = iW; i <= iE; i++) at(i, j) |= MK_XID;
      int tw = BT(ir, jr, W2_WEST), te = BT(ir, jr, W2_EAST);
      int ts = BT(ir, jr, W2_SOUTH), tn = BT(ir, jr, W2_NORTH);
      auto wall = [](int t) { return t == W2_BM_WALL1 || t == W2_BM_WALL2 || t == W2_BM_INLET; };
      if (wall(tw)) for (int j = jS + 1; j <= jN; j++) at(iW, j) |= MK_XID;
      if (wall(te)) for (int j = jS + 1; j <= jN; j++) at(iE, j) |= MK_XID;
      // Y split-2 identity rows, momentum.f:770-821
      if (rt == W2_RM_BLOCKG)
        for (int j = jS; j <= jN; j++)
          for (int i = iW + 1; i <= iE; i++) at(i, j) |= MK_YID;
      if (wall(ts)) for (int i = iW + 1; i <= iE; i++) at(i, jS) |= MK_YID;
      if (wall(tn)) for (int i = iW + 1; i <= iE; i++) at(i, jN) |= MK_YID;
      if (rt != W2_RM_BLOCKG) {
        // Project / Filter u, utility.f:313-363 and 94-137
        for (int j = jS + 1; j <= jN; j++)
          for (int i = iW + 1; i <= iE - 1; i++) { pu[i + (size_t)j * ld]++; at(i, j) |= MK_FU; }
        if (tw == W2_BM_OUTLT1)
          for (int j = jS + 1; j <= jN; j++) { pu[iW + (size_t)j * ld]++; at(iW, j) |= MK_FU; }
        if (te == W2_BM_INTERN || te == W2_BM_OUTLT1)
          for (int j = jS + 1; j <= jN; j++) { pu[iE + (size_t)j * ld]++; at(iE, j) |= MK_FU; }
        // Project / Filter v, utility.f:384-432 and 157-201
        for (int j = jS + 1; j <= jN - 1; j++)
          for (int i = iW + 1; i <= iE; i++) { pv[i + (size_t)j * ld]++; at(i, j) |= MK_FV; }
        if (ts == W2_BM_OUTLT1)
          for (int i = iW + 1; i <= iE; i++) { pv[i + (size_t)jS * ld]++; at(i, jS) |= MK_FV; }
        if (tn == W2_BM_INTERN || tn == W2_BM_OUTLT1)
          for (int i = iW + 1; i <= iE; i++) { pv[i + (size_t)jN * ld]++; at(i, jN) |= MK_FV; }
      } else {
        // PPE identity rows and div zeroing, pressure.f:109-196
        auto pid = [&](int i, int j) {
          if (inb(i, j) && i >= 2 && i <= nx && j >= 2 && j <= ny) at(i, j) |= MK_PID;
        };
        auto dz = [&](int i, int j) { if (inb(i, j)) at(i, j) |= MK_DIVZ; };
        for (int j = jS + 2; j <= jN - 1; j++)
          for (int i = iW + 2; i <= iE - 1; i++) { pid(i, j); dz(i, j); }
        // a(ind,.) rows addressed through ind in the reference map back to
        // (i,j) = (ind mod (nx-1) + 1, ind div (nx-1) + 2)
        auto pid_ind = [&](int ind) {
          int i = (ind - 1) % (nx - 1) + 2, j = (ind - 1) / (nx - 1) + 2;
          pid(i, j);
        };
        if (ir > 1 && RT(ir - 1, jr) == W2_RM_BLOCKG)
          for (int j = jS + 1; j <= jN; j++) { pid_ind((j - 2) * (nx - 1) + iW); dz(iW + 1, j); }
        if (ir < c->nri && RT(ir + 1, jr) == W2_RM_BLOCKG)
          for (int j = jS + 1; j <= jN; j++) { pid_ind((j - 2) * (nx - 1) + iE - 1); dz(iE, j); }
        if (jr > 1 && RT(ir, jr - 1) == W2_RM_BLOCKG)
          for (int i = iW + 1; i <= iE; i++) { pid_ind((jS - 1) * (nx - 1) + i - 1); dz(i, jS + 1); }
        if (jr < c->nrj && RT(ir, jr + 1) == W2_RM_BLOCKG)
          for (int i = iW + 1; i <= iE; i++) { pid_ind((jN - 2) * (nx - 1) + i - 1); dz(i, jN); }
      }
    }
  for (size_t k = 0; k < c->nf; ++k) {
    if (pu[k] > 1 || pv[k] > 1)
      return fail(c, W2_E_UNSUPPORTED, "overlapping projection faces in the region layout");
    if (pu[k]) mk[k] |= MK_PU;
    if (pv[k]) mk[k] |= MK_PV;
  }
  return W2_OK;
}

// Host replay of the porous region loops of XMomentum/YMomentum
// (momentum.f:296-324, 621-649) and PorosCoef (momentum.f:1157-1214) into
// the per-cell tables of Porous (planes: X divisors 0-1, Y divisors 2-3,
// porc1 X, porc2 X, porc1 Y, porc2 Y) and the MK_PCX / MK_PCY bits.
int build_porous(w2_ctx *c, std::vector<uint16_t> &mk, std::vector<double> &tab) {
  const int mgri = c->mgri, mgrj = c->mgrj, ld = c->ld;
  const size_t nf = c->nf;
  tab.assign(8 * nf, 0.0);
  std::fill(tab.begin(), tab.begin() + 4 * nf, 1.0);
  std::vector<uint8_t> nxd(nf, 0), nyd(nf, 0);
  std::vector<int> wx(nf, 0), wy(nf, 0);  // last PorosCoef writer: 0 zero, else region + 1
  auto B = [&](int ir, int jr, int s) { return c->tab_brd[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto id = [&](int ir, int jr) { return (ir - 1) + (jr - 1) * mgri; };
  auto o = [&](int i, int j) { return (size_t)i + (size_t)j * ld; };
  for (int jr = 1; jr <= c->nrj; jr++)
    for (int ir = 1; ir <= c->nri; ir++) {
      const int iW = B(ir, jr, W2_WEST), iE = B(ir, jr, W2_EAST);
      const int jS = B(ir, jr, W2_SOUTH), jN = B(ir, jr, W2_NORTH);
      if (c->tab_rtype[id(ir, jr)] != W2_RM_POROUS) {
        for (int j = jS; j <= jN; j++)
          for (int i = iW; i <= iE; i++) wx[o(i, j)] = wy[o(i, j)] = 0;
        continue;
      }
      const double por = c->tab_por[id(ir, jr)];
      for (int j = jS + 1; j <= jN; j++)
        for (int i = iW; i <= iE; i++) {
          const size_t k = o(i, j);
          if (nxd[k] == 2) return fail(c, W2_E_UNSUPPORTED, "a cell in three porous regions");
          tab[nxd[k]++ * nf + k] = por;
          wx[k] = id(ir, jr) + 1;
        }
      for (int j = jS; j <= jN; j++)
        for (int i = iW + 1; i <= iE; i++) {
          const size_t k = o(i, j);
          if (nyd[k] == 2) return fail(c, W2_E_UNSUPPORTED, "a cell in three porous regions");
          tab[(2 + nyd[k]++) * nf + k] = por;
          wy[k] = id(ir, jr) + 1;
        }
    }
  for (size_t k = 0; k < nf; ++k) {
    if (wx[k]) {
      mk[k] |= MK_PCX;
      tab[4 * nf + k] = c->tab_porc1[wx[k] - 1];
      tab[5 * nf + k] = c->tab_porc2[wx[k] - 1];
    }
    if (wy[k]) {
      mk[k] |= MK_PCY;
      tab[6 * nf + k] = c->tab_porc1[wy[k] - 1];
      tab[7 * nf + k] = c->tab_porc2[wy[k] - 1];
    }
  }
  return W2_OK;
}

cudaEvent_t ev_get(w2_ctx *c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Bracket a launch with events on the context stream when profiling.
struct ProfScope {
  w2_ctx *c;
  int kind;
  cudaEvent_t a = nullptr;
  ProfScope(w2_ctx *c_, int k) : c(c_), kind(k) {
    if (c->prof_on) {
      a = ev_get(c);
      cudaEventRecord(a, c->st);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEvent_t b = ev_get(c);
      cudaEventRecord(b, c->st);
      c->prof_pending.push_back({kind, a, b});
    }
  }
};

void prof_collect(w2_ctx *c) {
  if (c->prof_pending.empty()) return;
  cudaStreamSynchronize(c->st);
  for (auto &r : c->prof_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      c->prof_ms[r.kind] += ms;
      c->prof_n[r.kind] += 1;
    }
    c->ev_pool.push_back(r.a);
    c->ev_pool.push_back(r.b);
  }
  c->prof_pending.clear();
}

int pick_blocks(w2_ctx *c, const void *kern, long work, size_t smem = 0) {
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, c->threads, smem);
  occ = std::max(1, std::min(occ, c->blocks_per_sm));
  // tiny grids: one block (grid barriers become __syncthreads); otherwise at
  // least one block per SM, up to the co-resident limit
  long want = (work + 4095) / 4096;
  if (want > 1) want = std::max<long>(want, c->nsm);
  long nb = std::max<long>(1, std::min<long>(want, (long)occ * c->nsm));
  return (int)nb;
}

int coop(w2_ctx *c, const void *kern, int blocks, void **args, size_t smem = 0) {
  c->launches++;
  cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(c->threads), args, smem, c->st);
  if (e != cudaSuccess) return fail(c, W2_E_CUDA, "cooperative launch: %s", cudaGetErrorString(e));
  return W2_OK;
}

// Dynamic shared memory of the momentum kernels: the chain walks' stage
// (the FP64 and FP32 stages have the same size per thread).
size_t naux_smem(const w2_ctx *c) { return walk_stage_bytes(sizeof(double), c->threads); }

int check_sync(w2_ctx *c) {
  CK(cudaStreamSynchronize(c->st));
  Sync s;
  CK(cudaMemcpy(&s, c->dev.sync, sizeof(Sync), cudaMemcpyDeviceToHost));
  if (s.error) {
    int code = s.error;
    // clear the sticky error and barrier state so the context stays usable
    Sync z;
    memset(&z, 0, sizeof(z));
    cudaMemcpy(c->dev.sync, &z, sizeof(Sync), cudaMemcpyHostToDevice);
    if (code == W2_E_TIMEOUT) return fail(c, code, "device wait exceeded its time limit");
    if (code == W2_E_BCFLAG) return fail(c, code, "invalid boundary flag");
    return fail(c, code, "device error %d", code);
  }
  return W2_OK;
}

// Chain buffers for a chain of n rows.
// Rows of chain storage: segment-interleaved positions run up to
// L*nseg - 1 < n + L, and L is at most kMaxSeg.
constexpr int kMaxSeg = 4096;

template <class T>
int make_chain(w2_ctx *c, ChainT<T> &ch, int n, bool with_b) {
  const size_t cap = (size_t)n + kMaxSeg;
  ch.n = n;
  ch.a1 = dalloc<T>(c, cap);
  ch.a2 = dalloc<T>(c, cap);
  ch.a3 = dalloc<T>(c, cap);
  ch.b = with_b ? dalloc<T>(c, cap) : nullptr;
  ch.a3p = dalloc<T>(c, cap);
  ch.bp = dalloc<T>(c, cap);
  ch.x = dalloc<T>(c, cap);
  // end-state buffers, sized for the smallest segment length allowed (8)
  const int ms = (n + 7) / 8;
  ch.ef = dalloc<T>(c, (size_t)4 * ms);
  ch.eb = dalloc<T>(c, (size_t)2 * ms);
  if (!ch.a1 || !ch.a2 || !ch.a3 || !ch.a3p || !ch.bp || !ch.x || (with_b && !ch.b) || !ch.ef ||
      !ch.eb)
    return fail(c, W2_E_CUDA, "out of device memory (chains)");
  return W2_OK;
}

// Split-2 chain in the storage of split 1: its rows are assembled after the
// split-1 solve, whose rows and forward states are dead by then; its
// right-hand side is the split-1 solution; only the solution is its own.
template <class T>
int alias_split2(w2_ctx *c, ChainT<T> &c2, const ChainT<T> &c1) {
  c2.n = c1.n;
  c2.a1 = c1.a1; c2.a2 = c1.a2; c2.a3 = c1.a3;
  c2.a3p = c1.a3p; c2.bp = c1.bp;
  c2.ef = c1.ef; c2.eb = c1.eb;
  c2.b = c1.x;
  c2.x = dalloc<T>(c, (size_t)c1.n + kMaxSeg);
  if (!c2.x) return fail(c, W2_E_CUDA, "out of device memory (chains)");
  return W2_OK;
}

// Chain segment length and warm-up for `threads` threads walking the chains,
// applied to every chain view of d (end-state buffers are sized for the
// shortest segment allowed, 8 rows).
void chain_views(Dev &d, int nx, int ny, long threads, int seg_req, int warm_req) {
  const int nX = nx * (ny - 1), nY = (nx - 1) * ny;
  int seg = seg_req > 0 ? seg_req : (int)std::max<long>(8, (nX + nY + threads - 1) / threads);
  seg = std::min(seg, kMaxSeg);
  d.seg = seg;
  d.warm = warm_req > 0 ? warm_req : 64;
  const int nsx = (nX + seg - 1) / seg, nsy = (nY + seg - 1) / seg;
  ChainT<double> *c64[] = {&d.x1, &d.x2, &d.y1, &d.y2, &d.f64.x1, &d.f64.x2, &d.f64.y1, &d.f64.y2};
  ChainT<float> *c32[] = {&d.f32.x1, &d.f32.x2, &d.f32.y1, &d.f32.y2};
  for (int k = 0; k < 8; ++k) {
    c64[k]->L = seg;
    c64[k]->nseg = (k % 4) < 2 ? nsx : nsy;
  }
  for (int k = 0; k < 4; ++k) {
    c32[k]->L = seg;
    c32[k]->nseg = k < 2 ? nsx : nsy;
  }
}

int set_segments(w2_ctx *c) {
  int blocks = pick_blocks(c, (const void *)k_naux, (long)c->nx * c->ny, naux_smem(c));
  chain_views(c->dev, c->nx, c->ny, (long)blocks * c->threads, c->seg_req, c->warm_req);
  return W2_OK;
}

int copy_in(w2_ctx *c, double *dst, const double *src) {
  CK(cudaMemcpy2DAsync(dst, (size_t)c->ld * 8, src, (size_t)(c->mnx + 1) * 8, (size_t)(c->nx + 2) * 8,
                       c->ny + 2, cudaMemcpyHostToDevice, c->st));
  return W2_OK;
}

int copy_out(w2_ctx *c, double *dst, const double *src) {
  CK(cudaMemcpy2DAsync(dst, (size_t)(c->mnx + 1) * 8, src, (size_t)c->ld * 8, (size_t)(c->nx + 2) * 8,
                       c->ny + 2, cudaMemcpyDeviceToHost, c->st));
  return W2_OK;
}

bool dims_match(w2_ctx *c, const int *nx, const int *ny) {
  return nx && ny && *nx == c->nx && *ny == c->ny;
}

int ready(w2_ctx *c) {
  if (!c) return W2_E_ARG;
  if (!c->metrics_ok) return fail(c, W2_E_ARG, "metrics not set (wolfd2gpu_set_metrics or wolfd2gpu_grid_metric)");
  return W2_OK;
}

// A snapshot copy may still read time level snap_level: work on the context
// stream that writes that level (or any level, when `level` is -1) first
// waits for the copy.
void snap_fence(w2_ctx *c, int level = -1) {
  if (c->snap_level < 0) return;
  if (level >= 0 && level != c->snap_level) return;
  cudaStreamWaitEvent(c->st, c->ev_snap_done, 0);
  c->snap_level = -1;
}

// ---- launch helpers on explicit device buffers ---------------------------
int launch_bc(w2_ctx *c, int ops, double *u, double *v, double *p) {
  ProfScope ps(c, W2_K_BC);
  c->launches++;
  k_bc<<<1, c->threads, 0, c->st>>>(c->dev, ops, u, v, p);
  CK(cudaGetLastError());
  return W2_OK;
}

int launch_naux(w2_ctx *c, int mqiter, double dk, double re, double qtol, const double *un,
                const double *vn, double *us, double *vs, const double *den = nullptr,
                const double *denn = nullptr, double fr = 0.0) {
  int blocks = pick_blocks(c, (const void *)k_naux, (long)c->nx * c->ny, naux_smem(c));
  ProfScope ps(c, W2_K_MOMENTUM);
  Dev d = c->dev;
  d.den = den;
  d.denn = denn;
  d.fr = fr;
  StepOut *out = c->d_out;
  void *args[] = {&d, &mqiter, &dk, &re, &qtol, (void *)&un, (void *)&vn, &us, &vs, &out};
  return coop(c, (const void *)k_naux, blocks, args, naux_smem(c));
}

// Tile geometry for the tiled red/black kernel: ntx*nty = k * blocks tiles
// (k as small as the shared-memory limit allows), choosing the split with
// the least redundant halo work per block.
const void *tiled_kernel(const w2_ctx *c) {
  return c->tiled_wide ? (const void *)k_ppe_tiled_w : (const void *)k_ppe_tiled;
}

void plan_tiles(w2_ctx *c) {
  c->tiled_ok = false;
  c->tiled_threads = c->tiled_wide ? 1024 : 512;
  int dev = c->device, maxsmem = 0;
  cudaDeviceGetAttribute(&maxsmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t limit = (size_t)maxsmem - 4096;  // leave room for static shared arrays
  if (cudaFuncSetAttribute(tiled_kernel(c), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)limit) != cudaSuccess)
    return;
  const int NX = c->nx - 1, NY = c->ny - 1;
  double best = 1e300;
  // every split into ntx x nty tiles of at least 8 x 8 unknowns; blocks
  // (one per SM) take ceil(tiles / nsm) tiles each, so the cost of a split is
  // that count times the area swept per tile over a group of sweeps
  for (int ntx = 1; ntx <= NX / 8; ++ntx) {
    const int tx = (NX + ntx - 1) / ntx;
    if ((NX + tx - 1) / tx != ntx) continue;
    for (int nty = 1; nty <= NY / 8; ++nty) {
      const int ty = (NY + nty - 1) / nty;
      if ((NY + ty - 1) / ty != nty) continue;
      const size_t smem = (size_t)(tx + 2 * kHalo) * (ty + 2 * kHalo) * 16;
      if (smem > limit) continue;
      double area = 0.0;
      for (int e = kHalo - 1; e >= 0; --e) area += (double)(tx + 2 * e) * (ty + 2 * e);
      const long per_block = ((long)ntx * nty + c->nsm - 1) / c->nsm;
      const double cost = per_block * area;
      if (cost < best) {
        best = cost;
        c->tg = TileGeom{tx, ty, ntx, nty, 1.0, -1.0};
        c->tiled_smem = smem;
      }
    }
  }
  if (best >= 1e300) return;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tiled_kernel(c), c->tiled_threads,
                                                c->tiled_smem);
  if (occ < 1) return;
  c->tiled_blocks = c->nsm;  // one block per SM, each owning ntiles/nsm tiles
  c->tiled_ok = true;
}

// The tiled kernel pays for its halo work only on large grids (one barrier
// costs about as much as sweeping ~0.15 M points); use_tiled == 2 forces it.
bool tiled_applies(w2_ctx *c, int npsolver, double sorrel) {
  const long cells = (long)(c->nx - 1) * (c->ny - 1);
  const bool big = cells >= (long)c->nsm * 1024;
  (void)sorrel;
  return c->use_tiled && (big || c->use_tiled == 2) && c->tiled_ok && c->dev.ppe_unit &&
         (npsolver == 5 || npsolver == 6);
}

int launch_ppe_tiled(w2_ctx *c, int lcartes, int msorit, double dk, double sortol, double sorrel,
                     const double *u, const double *v, double *p, StepOut *out, const Dev *dv = nullptr) {
  Dev d = dv ? *dv : c->dev;
  TileGeom g = c->tg;
  void *args[] = {&d, &g, &lcartes, &msorit, &dk, &sortol, &sorrel, (void *)&u, (void *)&v, &p, &out};
  c->launches++;
  cudaError_t e = cudaLaunchCooperativeKernel(tiled_kernel(c), dim3(c->tiled_blocks),
                                              dim3(c->tiled_threads), args, c->tiled_smem, c->st);
  if (e != cudaSuccess) return fail(c, W2_E_CUDA, "tiled PPE launch: %s", cudaGetErrorString(e));
  return W2_OK;
}

// ---- single-precision momentum state -----------------------------------------

int grid_blocks(w2_ctx *c);

// FP32 forms of the momentum metrics (profiles where the FP64 ones are,
// rounded full arrays otherwise), FP32 chains (split 2 in the storage of
// split 1, the identity rows shared with the FP64 chains), the FP32 ConvCoef
// arrays and the FP32 fields; allocated on the first mixed step, the metrics
// re-rounded whenever new ones are uploaded.
int ensure_f32(w2_ctx *c) {
  Dev &d = c->dev;
  MomView<float> &v = d.f32;
  if (!c->f32_alloc) {
    for (int k = 0; k < 4; ++k)
      if (!(c->F32[k] = dalloc<float>(c, c->nf))) return fail(c, W2_E_CUDA, "out of device memory (FP32 fields)");
    const int nX = c->nx * (c->ny - 1), nY = (c->nx - 1) * c->ny;
    int rc;
    if ((rc = make_chain(c, v.x1, nX, true)) || (rc = alias_split2(c, v.x2, v.x1)) ||
        (rc = make_chain(c, v.y1, nY, true)) || (rc = alias_split2(c, v.y2, v.y1)))
      return rc;
    v.x1.nseg = d.x1.nseg; v.x2.nseg = d.x2.nseg;
    v.y1.nseg = d.y1.nseg; v.y2.nseg = d.y2.nseg;
    v.x1.L = v.x2.L = v.y1.L = v.y2.L = d.seg;
    float **cc[] = {&v.cj1x, &v.cj2x, &v.c1sx, &v.c2sx, &v.c1nx, &v.c2nx,
                    &v.cj1y, &v.cj2y, &v.c1sy, &v.c2sy, &v.c1ny, &v.c2ny};
    for (float **a : cc)
      if (!(*a = dalloc<float>(c, c->nf))) return fail(c, W2_E_CUDA, "out of device memory (FP32 ConvCoef arrays)");
    c->f32_alloc = true;
  }
  if (!c->f32_metrics_ok) {
    std::vector<MRef<float> *> refs = mom_refs(v);
    const int gb = grid_blocks(c);
    const int W = c->nx + 2, H = c->ny + 2;
    std::vector<double> h64;
    for (int k = 0; k < 24; ++k) {
      w2_ctx::MomMetric &mm = c->mm[k];
      if (mm.mode == MP_FULL) {
        // An array that varies only in its last FP64 bits (a uniform grid
        // whose spacing is not a power of two) can be constant along i or j
        // once rounded to FP32: the FP32 view then reads a profile of the
        // rounded values, which are the values it would read in full.
        if (h64.size() != c->nf) h64.resize(c->nf);
        CK(cudaStreamSynchronize(c->st));
        CK(cudaMemcpy(h64.data(), c->met[kMomMetric[k]], c->nf * sizeof(double), cudaMemcpyDeviceToHost));
        auto f32 = [&](int i, int j) { return (float)h64[(size_t)i + (size_t)j * c->ld]; };
        bool ionly = true, jonly = true;
        for (int j = 0; j < H && (ionly || jonly); ++j)
          for (int i = 0; i < W; ++i) {
            const float x = f32(i, j), xi = f32(i, 0), xj = f32(0, j);
            if (ionly && memcmp(&x, &xi, 4) != 0) ionly = false;
            if (jonly && memcmp(&x, &xj, 4) != 0) jonly = false;
          }
        if (ionly || jonly) {
          const int len = ionly ? W : H;
          std::vector<float> h(len);
          for (int q = 0; q < len; ++q) h[q] = ionly ? f32(q, 0) : f32(0, q);
          if (!(mm.p32 = dalloc<float>(c, std::max(W, H))))
            return fail(c, W2_E_CUDA, "out of device memory (FP32 metrics)");
          CK(cudaMemcpy(mm.p32, h.data(), len * sizeof(float), cudaMemcpyHostToDevice));
          *refs[k] = ionly ? MRef<float>{mm.p32, 1, 0} : MRef<float>{mm.p32, 0, 1};
          continue;
        }
        if (!mm.p32 && !(mm.p32 = dalloc<float>(c, c->nf)))
          return fail(c, W2_E_CUDA, "out of device memory (FP32 metrics)");
        k_to_f32<<<gb, c->threads, 0, c->st>>>(d, c->met[kMomMetric[k]], mm.p32);
        c->launches++;
        *refs[k] = MRef<float>{mm.p32, 1, c->ld};
      } else {
        std::vector<float> h(mm.host.size());
        for (size_t q = 0; q < h.size(); ++q) h[q] = (float)mm.host[q];
        if (!mm.p32 && !(mm.p32 = dalloc<float>(c, h.size())))
          return fail(c, W2_E_CUDA, "out of device memory (FP32 metrics)");
        CK(cudaMemcpy(mm.p32, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
        *refs[k] = mm.mode == MP_I ? MRef<float>{mm.p32, 1, 0} : MRef<float>{mm.p32, 0, 1};
      }
    }
    CK(cudaGetLastError());
    c->f32_metrics_ok = true;
  }
  return W2_OK;
}

// How the momentum stencils read each metric: an array whose value depends
// on i only (every column identical, bit for bit, over the stored extent) is
// read as a profile over i, one that depends on j only as a profile over j,
// anything else in full.  Cartesian grids reduce to profiles, so the
// stencils stream no metric arrays.  Fills the FP64 view; the FP32 view
// follows on the next mixed step.
int momentum_metrics(w2_ctx *c) {
  Dev &d = c->dev;
  const int W = c->nx + 2, H = c->ny + 2;
  const size_t ld = c->ld;
  std::vector<double> h(c->nf);
  std::vector<MRef<double> *> refs = mom_refs(d.f64);
  CK(cudaStreamSynchronize(c->st));
  for (int k = 0; k < 24; ++k) {
    const double *src = c->met[kMomMetric[k]];
    CK(cudaMemcpy(h.data(), src, c->nf * sizeof(double), cudaMemcpyDeviceToHost));
    auto bits = [&](size_t o) {
      uint64_t b;
      memcpy(&b, &h[o], 8);
      return b;
    };
    bool ionly = true, jonly = true;
    for (int j = 0; j < H && (ionly || jonly); ++j)
      for (int i = 0; i < W; ++i) {
        const uint64_t b = bits((size_t)i + (size_t)j * ld);
        if (ionly && b != bits((size_t)i)) ionly = false;
        if (jonly && b != bits((size_t)j * ld)) jonly = false;
      }
    w2_ctx::MomMetric &mm = c->mm[k];
    mm.mode = ionly ? MP_I : (jonly ? MP_J : MP_FULL);
    if (mm.mode == MP_FULL) {
      mm.host.clear();
      *refs[k] = MRef<double>{src, 1, (int)ld};
      continue;
    }
    const int len = mm.mode == MP_I ? W : H;
    mm.host.resize(len);
    for (int q = 0; q < len; ++q) mm.host[q] = mm.mode == MP_I ? h[q] : h[(size_t)q * ld];
    if (!mm.p64 && !(mm.p64 = dalloc<double>(c, std::max(W, H))))
      return fail(c, W2_E_CUDA, "out of device memory (metric profiles)");
    CK(cudaMemcpy(mm.p64, mm.host.data(), len * sizeof(double), cudaMemcpyHostToDevice));
    *refs[k] = mm.mode == MP_I ? MRef<double>{mm.p64, 1, 0} : MRef<double>{mm.p64, 0, 1};
  }
  // an FP32 buffer was sized for the previous mode (profile or full array):
  // ensure_f32 makes new ones
  for (int k = 0; k < 24; ++k) c->mm[k].p32 = nullptr;
  c->f32_metrics_ok = false;
  return W2_OK;
}

// ---- mixed-precision Poisson sweeps ----------------------------------------

const void *mixed_kernel(int K, bool resident) {
  switch (K) {
    case 4: return resident ? (const void *)k_ppe_mixed<4, true> : (const void *)k_ppe_mixed<4, false>;
    case 8: return resident ? (const void *)k_ppe_mixed<8, true> : (const void *)k_ppe_mixed<8, false>;
  }
  return nullptr;
}

// Sweep work of one group of K sweeps on a tx x ty tile: (plane columns
// rounded to warps) x (box rows active in each half-sweep).
double mixed_sweep_work(int K, int tx, int ty) {
  const int H = 2 * K, bh = ty + 2 * H, hwp = mixed_lanes(K, tx);
  double rows = 0.0;
  for (int h = 1; h <= 2 * K; ++h) rows += std::max(0, bh - 2 * h);
  return (double)hwp * rows;
}

// Staging work of one group in multi-tile mode (whole box in, tile out).
double mixed_stage_work(int K, int tx, int ty) {
  const int H = 2 * K, bh = ty + 2 * H, hwp = (tx / 2 + H + 31) / 32 * 32;  // plane columns in warps
  return 4.0 * K * bh * hwp / 8.0;
}

// Tile plan of the mixed Poisson kernel.  Preferred: one tile per block (one
// block per SM, box resident in shared memory), the split of the unknowns
// into at most nsm tiles, tx a multiple of 8, whose block does the least
// sweep work per group of K sweeps -- (plane columns rounded to warps) x (box
// rows active in each half-sweep).  Grids too large for that run in
// multi-tile mode: blocks (as many as fit per SM) loop over more tiles,
// staging each box per group; the split then minimises tiles per block x
// (sweep work + staging).
void plan_mixed(w2_ctx *c) {
  c->mixed_ok = false;
  const int K = c->mixed_K;
  if (!mixed_kernel(K, true)) return;
  int maxsmem = 0;
  cudaDeviceGetAttribute(&maxsmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  const int NX = c->nx - 1, NY = c->ny - 1, H = 2 * K;
  auto sweep_work = [&](int tx, int ty) { return mixed_sweep_work(K, tx, ty); };
  for (int pass = (c->mixed_mode == 1 || c->mixed_mode == 2) ? 1 : 0; pass < 2 && !c->mixed_ok; ++pass) {
    const bool resident = pass == 0;
    // mode 3: resident tiles two to an SM (at most 256 threads each, so the
    // two blocks' 128-register threads fit one SM's register file)
    const int per_sm = (resident && c->mixed_mode == 3) ? 2 : 1;
    const int tmax = per_sm == 2 ? std::min(c->mixed_threads, 256) : c->mixed_threads;
    const void *kf = mixed_kernel(K, resident);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kf) != cudaSuccess || (size_t)maxsmem <= fa.sharedSizeBytes) continue;
    const size_t limit = (size_t)maxsmem - fa.sharedSizeBytes;  // less the static arrays
    if (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit) != cudaSuccess)
      continue;
    double best = 1e300;
    for (int ntx = 1; ntx <= std::max(1, NX / 8); ++ntx) {
      int tx = (NX + ntx - 1) / ntx;
      tx = (tx + 7) / 8 * 8;
      if ((NX + tx - 1) / tx != ntx) continue;
      for (int nty = 1; nty <= std::max(1, NY / 4); ++nty) {
        if (resident && ntx * nty > per_sm * c->nsm) break;
        const int ty = (NY + nty - 1) / nty;
        if ((NY + ty - 1) / ty != nty) continue;
        const size_t smem = mixed_smem_bytes(K, tx, ty, resident);
        const int T = mixed_threads(K, tx, ty);
        if (smem > limit || T > tmax) continue;
        double cost = sweep_work(tx, ty);
        int blocks = c->nsm;
        if (per_sm == 2) {
          int occ = 0;
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kf, T, smem);
          if (occ < 2) continue;
          blocks = 2 * c->nsm;
        }
        if (!resident) {
          int occ = 0;
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kf, T, smem);
          if (occ < 1) continue;
          blocks = c->nsm * occ;
          if (c->mixed_mode == 2) blocks = std::min(blocks, 16);
          const int tpb = (ntx * nty + blocks - 1) / blocks;
          cost = tpb * (cost + mixed_stage_work(K, tx, ty));
        }
        if (cost < best) {
          best = cost;
          c->mg = MixedGeom{tx, ty, ntx, nty, ntx * tx / 2 + H, nty * ty + 2 * H,
                            mixed_lanes(K, tx), resident ? 1 : 0};
          c->mixed_smem = smem;
          c->mixed_blocks = blocks;
        }
      }
    }
    if (best >= 1e300) continue;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kf, mixed_threads(K, c->mg.tx, c->mg.ty),
                                                  c->mixed_smem);
    if (occ < 1) continue;
    c->mixed_ok = true;
  }
  if (!c->mixed_ok) return;
  // exchange buffers and the r buffer: zero wherever no tile writes (cells
  // off the unknowns)
  const size_t need = 6 * (size_t)c->mg.gh * c->mg.gw;
  if (need > c->xbuf_floats) {
    if (c->xbuf) {
      cudaFree(c->xbuf);
      c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void *)c->xbuf), c->allocs.end());
      c->xbuf = nullptr;
      c->xbuf_floats = 0;
    }
    if (!(c->xbuf = dalloc<float>(c, need))) {
      c->mixed_ok = false;
      return;
    }
    c->xbuf_floats = need;
  }
  if (cudaMemset(c->xbuf, 0, c->xbuf_floats * sizeof(float)) != cudaSuccess) c->mixed_ok = false;
  // multi-tile plans stage their boxes with TMA when the maps can be made
  c->tm_ok = false;
  if (c->mixed_ok && !c->mg.resident && c->use_tma) {
    if (!c->d_tm) c->d_tm = dalloc<CUtensorMap>(c, 3);
    c->tm_ok = c->d_tm && encode_mixed_maps(c->d_tm, c->xbuf, c->mg, c->mixed_K, c->st);
  }
}

// The mixed Poisson solve takes npsolver 5/6 on every grid: the unit-stencil
// kernel where the rows round to (1,1,-4,1,1) in FP32 on a Cartesian grid
// without blockages (every uniform square-cell grid), the general-row kernel
// everywhere else.
bool mixed_general(const w2_ctx *c, int lcartes) { return !lcartes || !c->dev.ppe_unit32; }

// Tile plan of the general-row kernel's tiled form: one or more blocks of
// kMixgtThreads per SM, as many as shared memory allows; the split of the
// unknowns into tiles minimising tiles per block x (sweep work of a group
// on the shrinking boxes + staging of the box).
void plan_mixgt(w2_ctx *c) {
  c->mgt_ok = false;
  // rows that round to the unit stencil take the unit kernel on Cartesian grids
  if (c->dev.ppe_unit32) return;
  int maxsmem = 0;
  cudaDeviceGetAttribute(&maxsmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  const void *kf = (const void *)k_ppe_mixgt;
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kf) != cudaSuccess || (size_t)maxsmem <= fa.sharedSizeBytes) return;
  const size_t limit = (size_t)maxsmem - fa.sharedSizeBytes;
  if (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit) != cudaSuccess) return;
  const int NX = c->nx - 1, NY = c->ny - 1, H = kMixgtH, K = kMixgtK;
  double best = 1e300;
  for (int ntx = 1; ntx <= NX; ++ntx) {
    const int tx = (NX + ntx - 1) / ntx;
    if ((NX + tx - 1) / tx != ntx) continue;
    for (int nty = 1; nty <= NY; ++nty) {
      const int ty = (NY + nty - 1) / nty;
      if ((NY + ty - 1) / ty != nty) continue;
      const size_t smem = mixgt_smem_bytes(tx, ty);
      if (smem > limit) continue;
      int occ = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kf, kMixgtThreads, smem);
      if (occ < 1) continue;
      const int tiles = ntx * nty, cap = c->nsm * occ;
      const int tpb = (tiles + cap - 1) / cap;
      const double cost = tpb * ((double)K * (tx + H) * (ty + H) + 2.0 * (tx + 2 * H) * (ty + 2 * H));
      if (cost < best) {
        best = cost;
        c->mgt = MixgtGeom{tx, ty, ntx, nty};
        c->mgt_smem = smem;
        c->mgt_blocks = (tiles + tpb - 1) / tpb;
      }
    }
  }
  c->mgt_ok = best < 1e300;
}

bool mixgt_applies(const w2_ctx *c, int lcartes) { return lcartes && c->use_mixgt && c->mgt_ok; }

int mixed_check(w2_ctx *c, int lcartes, int npsolver) {
  if (npsolver != 5 && npsolver != 6)
    return fail(c, W2_E_UNSUPPORTED, "mixed precision needs ppe_solver rb_sor or rb_sorp (5/6), got %d", npsolver);
  if (mixed_general(c, lcartes)) return W2_OK;
  if (!c->mixed_ok) return fail(c, W2_E_UNSUPPORTED, "no mixed-precision tile plan fits this grid");
  return W2_OK;
}

MixgArgs mixg_args(w2_ctx *c, int lcartes, int msorit, double dk, double sortol, double sorrel, int inner,
                   const double *u, const double *v, double *p) {
  return MixgArgs{lcartes, msorit, inner, dk, sortol, (float)sorrel, u, v, p, c->mgbuf, mixg_gw(c->nx),
                  c->mg_rb, c->mg_rb + c->nf};
}

// The general-row kernel's planes (zeroed: cells off the unknowns keep e =
// 0), its FP32 rbu and rbv, and its coefficient planes for the current
// metrics.
int ensure_mixg(w2_ctx *c) {
  const size_t plane = (size_t)mixg_gw(c->nx) * (c->ny + 2);
  if (!c->mgbuf) {
    if (!(c->mgbuf = dalloc<float>(c, MG_PLANES * plane)) || !(c->mg_rb = dalloc<float>(c, 2 * c->nf)))
      return fail(c, W2_E_CUDA, "out of device memory (mixed Poisson planes)");
    CK(cudaMemsetAsync(c->mgbuf, 0, MG_PLANES * plane * sizeof(float), c->st));
    c->mg_coef_ok = false;
  }
  if (!c->mg_coef_ok) {
    const int gb = grid_blocks(c);
    MixgArgs a = mixg_args(c, 1, 0, 1.0, 0.0, 1.0, 1, nullptr, nullptr, nullptr);
    k_mixg_coef<<<gb, c->threads, 0, c->st>>>(c->dev, a);
    k_to_f32<<<gb, c->threads, 0, c->st>>>(c->dev, c->met[M_RBU], c->mg_rb);
    k_to_f32<<<gb, c->threads, 0, c->st>>>(c->dev, c->met[M_RBV], c->mg_rb + c->nf);
    c->launches += 3;
    if (!c->mgt_buf) {
      if (!(c->mgt_buf = dalloc<float>(c, 8 * c->nf)))
        return fail(c, W2_E_CUDA, "out of device memory (tiled mixed Poisson buffers)");
      CK(cudaMemsetAsync(c->mgt_buf, 0, 8 * c->nf * sizeof(float), c->st));
    }
    float *b = c->mgt_buf;
    const size_t nf = c->nf;
    k_mixgt_coef<<<gb, c->threads, 0, c->st>>>(c->dev, b, b + nf, b + 2 * nf, b + 3 * nf, b + 4 * nf);
    c->launches++;
    CK(cudaGetLastError());
    c->mg_coef_ok = true;
  }
  return W2_OK;
}

int auto_inner(w2_ctx *c, int req) {
  if (req > 0) return req;
  return 16 * c->mixed_K;
}

int launch_ppe_mixed(w2_ctx *c, int lcartes, int msorit, double dk, double sortol, double sorrel,
                     int inner, const double *u, const double *v, double *p, StepOut *out) {
  if (mixed_general(c, lcartes)) {
    if (int rc = ensure_mixg(c)) return rc;
    Dev d = c->dev;
    if (mixgt_applies(c, lcartes)) {
      float *b = c->mgt_buf;
      const size_t nf = c->nf;
      MixgtGeom g = c->mgt;
      MixgtArgs a{msorit, auto_inner(c, inner), dk, sortol, (float)sorrel, u, v, p,
                  {b, b + nf, b + 2 * nf, b + 3 * nf, b + 4 * nf}, b + 5 * nf, {b + 6 * nf, b + 7 * nf}};
      void *args[] = {&d, &g, &a, &out};
      c->launches++;
      cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_ppe_mixgt, dim3(c->mgt_blocks),
                                                  dim3(kMixgtThreads), args, c->mgt_smem, c->st);
      if (e != cudaSuccess) return fail(c, W2_E_CUDA, "tiled mixed PPE launch: %s", cudaGetErrorString(e));
      return W2_OK;
    }
    MixgArgs a = mixg_args(c, lcartes, msorit, dk, sortol, sorrel, auto_inner(c, inner), u, v, p);
    void *args[] = {&d, &a, &out};
    return coop(c, (const void *)k_ppe_mixg, pick_blocks(c, (const void *)k_ppe_mixg, (long)c->nx * c->ny),
                args);
  }
  Dev d = c->dev;
  MixedGeom g = c->mg;
  const size_t plane2 = 2 * (size_t)c->mg.gh * c->mg.gw;
  MixedArgs a{lcartes, msorit, auto_inner(c, inner), dk, sortol, (float)sorrel, u, v, p,
              c->xbuf, c->xbuf + plane2, c->xbuf + 2 * plane2, c->tm_ok ? c->d_tm : nullptr};
  void *args[] = {&d, &g, &a, &out};
  c->launches++;
  const int T = mixed_threads(c->mixed_K, g.tx, g.ty);
  cudaError_t e = cudaLaunchCooperativeKernel(mixed_kernel(c->mixed_K, c->mg.resident != 0), dim3(c->mixed_blocks),
                                              dim3(T), args, c->mixed_smem, c->st);
  if (e != cudaSuccess) return fail(c, W2_E_CUDA, "mixed PPE launch: %s", cudaGetErrorString(e));
  return W2_OK;
}

int launch_ppe(w2_ctx *c, int lcartes, int npsolver, int msorit, double dk, double sortol,
               double sorrel, const double *u, const double *v, double *p) {
  if (c->prec_dropin == W2_PREC_MIXED) {
    int rc = mixed_check(c, lcartes, npsolver);
    if (rc) return rc;
    ProfScope ps(c, W2_K_PPE);
    return launch_ppe_mixed(c, lcartes, msorit, dk, sortol, sorrel, c->refine_dropin, u, v, p, c->d_out);
  }
  if (tiled_applies(c, npsolver, sorrel)) {
    ProfScope ps(c, W2_K_PPE);
    return launch_ppe_tiled(c, lcartes, msorit, dk, sortol, sorrel, u, v, p, c->d_out);
  }
  int blocks = (npsolver == 1 || npsolver == 2) ? 1 : pick_blocks(c, (const void *)k_ppe, (long)c->nx * c->ny);
  ProfScope ps(c, W2_K_PPE);
  Dev d = c->dev;
  StepOut *out = c->d_out;
  void *args[] = {&d, &lcartes, &npsolver, &msorit, &dk, &sortol, &sorrel, (void *)&u, (void *)&v, &p, &out};
  return coop(c, (const void *)k_ppe, blocks, args);
}

int grid_blocks(w2_ctx *c) {
  long work = (long)(c->nx + 2) * (c->ny + 2);
  return (int)std::max<long>(1, std::min<long>((work + c->threads - 1) / c->threads, (long)c->nsm * 8));
}

}  // namespace

extern "C" {

int wolfd2gpu_create(w2_ctx **out, int mnx, int mny, int mgri, int mgrj, int nx, int ny,
                     const int *nReg, const int *nRegBrd, const int *nRegType,
                     const int *nMomBdTp, const double *dBCVal, const double *dPRporos,
                     const double *dPRporc1, const double *dPRporc2) {
  if (!out) return W2_E_ARG;
  *out = nullptr;
  if (nx < 6 || ny < 6 || nx + 1 > mnx || ny + 1 > mny || mgri < 1 || mgrj < 1 || !nReg ||
      !nRegBrd || !nRegType || !nMomBdTp || !dBCVal)
    return W2_E_ARG;
  if (nReg[0] < 1 || nReg[0] > mgri || nReg[1] < 1 || nReg[1] > mgrj) return W2_E_ARG;
  w2_ctx *c = new w2_ctx();
  c->mnx = mnx; c->mny = mny; c->mgri = mgri; c->mgrj = mgrj; c->nx = nx; c->ny = ny;
  c->ld = ((nx + 2 + 31) / 32) * 32;
  c->nf = (size_t)c->ld * (size_t)(ny + 2);
  c->nri = nReg[0]; c->nrj = nReg[1];
  const size_t nt = (size_t)mgri * mgrj;
  c->tab_brd.assign(nRegBrd, nRegBrd + nt * 4);
  c->tab_rtype.assign(nRegType, nRegType + nt);
  c->tab_btype.assign(nMomBdTp, nMomBdTp + nt * 4);
  c->tab_bcv.assign(dBCVal, dBCVal + nt * 16);
  auto bad = [&](int code) { int r = code; wolfd2gpu_destroy(c); return r; };
  for (size_t k = 0; k < nt; ++k)
    if (nRegType[k] == W2_RM_POROUS && (!dPRporos || !dPRporc1 || !dPRporc2)) return bad(W2_E_ARG);
  if (dPRporos && dPRporc1 && dPRporc2) {
    c->tab_por.assign(dPRporos, dPRporos + nt);
    c->tab_porc1.assign(dPRporc1, dPRporc1 + nt);
    c->tab_porc2.assign(dPRporc2, dPRporc2 + nt);
  }
  if (cudaGetDevice(&c->device) != cudaSuccess) return bad(W2_E_CUDA);
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device);
  int coopok = 0;
  cudaDeviceGetAttribute(&coopok, cudaDevAttrCooperativeLaunch, c->device);
  if (!coopok) return bad(W2_E_UNSUPPORTED);
  // A blocking stream: set-up work goes through the legacy default stream
  // (cudaMemset zeroing of every allocation, synchronous uploads whose DMA
  // may still be in flight when they return), and the kernels on this
  // stream must run after it.
  if (cudaStreamCreate(&c->st) != cudaSuccess) return bad(W2_E_CUDA);
  std::vector<uint16_t> mk;
  int rc = build_masks(c, mk);
  std::vector<double> ptab;
  if (!rc && c->porous) rc = build_porous(c, mk, ptab);
  if (rc) { fprintf(stderr, "wolfd2gpu_create: %s\n", c->err); return bad(rc); }
  Dev &d = c->dev;
  if (c->porous) {
    double *pt = dalloc<double>(c, 8 * c->nf);
    if (!pt) return bad(W2_E_CUDA);
    cudaMemcpy(pt, ptab.data(), 8 * c->nf * sizeof(double), cudaMemcpyHostToDevice);
    // the same tables rounded to FP32 for the mixed step's momentum
    std::vector<float> pt32(ptab.size());
    for (size_t q = 0; q < ptab.size(); ++q) pt32[q] = (float)ptab[q];
    float *pf = dalloc<float>(c, 8 * c->nf);
    if (!pf) return bad(W2_E_CUDA);
    cudaMemcpy(pf, pt32.data(), 8 * c->nf * sizeof(float), cudaMemcpyHostToDevice);
    d.porous = 1;
    for (int k = 0; k < 4; ++k) {
      d.por.div[k] = pt + k * c->nf;
      d.por.div32[k] = pf + k * c->nf;
    }
    for (int k = 0; k < 2; ++k) {
      d.por.c1[k] = pt + (4 + 2 * k) * c->nf;
      d.por.c2[k] = pt + (5 + 2 * k) * c->nf;
      d.por.c1_32[k] = pf + (4 + 2 * k) * c->nf;
      d.por.c2_32[k] = pf + (5 + 2 * k) * c->nf;
    }
  }
  d.nx = nx; d.ny = ny; d.ld = c->ld;
  for (int k = 0; k < W2_NMETRIC; ++k)
    if (!(c->met[k] = dalloc<double>(c, c->nf))) return bad(W2_E_CUDA);
  bind_metrics(c);
  int *brd = dalloc<int>(c, nt * 4), *rty = dalloc<int>(c, nt), *bty = dalloc<int>(c, nt * 4);
  double *bcv = dalloc<double>(c, nt * 16);
  uint16_t *dmk = dalloc<uint16_t>(c, c->nf);
  if (!brd || !rty || !bty || !bcv || !dmk) return bad(W2_E_CUDA);
  cudaMemcpy(brd, c->tab_brd.data(), nt * 4 * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(rty, c->tab_rtype.data(), nt * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(bty, c->tab_btype.data(), nt * 4 * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(bcv, c->tab_bcv.data(), nt * 16 * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(dmk, mk.data(), c->nf * sizeof(uint16_t), cudaMemcpyHostToDevice);
  d.r = Regions{c->nri, c->nrj, mgri, mgrj, brd, rty, bty, bcv};
  d.mask = dmk;
  d.has_outflow = 0;
  for (int jr = 1; jr <= c->nrj; ++jr)
    for (int ir = 1; ir <= c->nri; ++ir)
      for (int s = 1; s <= 4; ++s) {
        int t = c->tab_btype[(ir - 1) + (jr - 1) * mgri + (s - 1) * nt];
        if (t == W2_BM_OUTLT1 || t == W2_BM_OUTLT2) d.has_outflow = 1;
      }
  for (int k = 0; k < 2; ++k) {
    if (!(c->U[k] = dalloc<double>(c, c->nf)) || !(c->V[k] = dalloc<double>(c, c->nf)) ||
        !(c->P[k] = dalloc<double>(c, c->nf)))
      return bad(W2_E_CUDA);
  }
  for (int k = 0; k < 6; ++k)
    if (!(c->stage[k] = dalloc<double>(c, c->nf))) return bad(W2_E_CUDA);
  double **wa[] = {&d.cj1x, &d.cj2x, &d.c1sx, &d.c2sx, &d.c1nx, &d.c2nx, &d.cj1y, &d.cj2y,
                   &d.c1sy, &d.c2sy, &d.c1ny, &d.c2ny, &d.pa1, &d.pa2, &d.pa3, &d.pa4,
                   &d.pa5, &d.div, &d.pb, &d.ppn, &d.la3p, &d.lbp, &d.qh};
  for (double **w : wa)
    if (!(*w = dalloc<double>(c, c->nf))) return bad(W2_E_CUDA);
  const int nX = nx * (ny - 1), nY = (nx - 1) * ny;
  if (make_chain(c, d.x1, nX, true) || alias_split2(c, d.x2, d.x1) ||
      make_chain(c, d.y1, nY, true) || alias_split2(c, d.y2, d.y1))
    return bad(W2_E_CUDA);
  d.f64.cj1x = d.cj1x; d.f64.cj2x = d.cj2x; d.f64.c1sx = d.c1sx; d.f64.c2sx = d.c2sx;
  d.f64.c1nx = d.c1nx; d.f64.c2nx = d.c2nx; d.f64.cj1y = d.cj1y; d.f64.cj2y = d.cj2y;
  d.f64.c1sy = d.c1sy; d.f64.c2sy = d.c2sy; d.f64.c1ny = d.c1ny; d.f64.c2ny = d.c2ny;
  d.f64.x1 = d.x1; d.f64.x2 = d.x2; d.f64.y1 = d.y1; d.f64.y2 = d.y2;
  {
    std::vector<MRef<double> *> refs = mom_refs(d.f64);
    for (int k = 0; k < 24; ++k) *refs[k] = MRef<double>{c->met[kMomMetric[k]], 1, (int)c->ld};
  }
  d.sync = dalloc<Sync>(c, 1);
  c->d_out = dalloc<StepOut>(c, 1);
  if (!d.sync || !c->d_out) return bad(W2_E_CUDA);
  if (cudaMallocHost(&c->h_out, sizeof(StepOut)) != cudaSuccess) return bad(W2_E_CUDA);
  c->threads = 256;
  c->blocks_per_sm = 2;
  {
    const int wmax = (int)walk_stage_bytes(sizeof(double), kMaxThreads);
    if (cudaFuncSetAttribute((const void *)k_naux, cudaFuncAttributeMaxDynamicSharedMemorySize, wmax) !=
            cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_naux32, cudaFuncAttributeMaxDynamicSharedMemorySize, wmax) !=
            cudaSuccess ||
        cudaFuncSetAttribute((const void *)k_naux32_por, cudaFuncAttributeMaxDynamicSharedMemorySize, wmax) !=
            cudaSuccess)
      return bad(W2_E_CUDA);
  }
  set_segments(c);
  d.u = c->U[0]; d.v = c->V[0]; d.p = c->P[0];
  if (cudaDeviceSynchronize() != cudaSuccess) return bad(W2_E_CUDA);
  *out = c;
  return W2_OK;
}

int wolfd2gpu_destroy(w2_ctx *c) {
  if (!c) return W2_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  for (auto &r : c->prof_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  for (auto &g : c->graphs) cudaGraphExecDestroy(g.second.exec);
  for (void *p : c->allocs) cudaFree(p);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->cst) {
    cudaStreamSynchronize(c->cst);
    cudaStreamDestroy(c->cst);
  }
  if (c->ev_snap_src) cudaEventDestroy(c->ev_snap_src);
  if (c->ev_snap_done) cudaEventDestroy(c->ev_snap_done);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return W2_OK;
}

const char *wolfd2gpu_last_error(w2_ctx *c) { return c ? c->err : "null context"; }

long long wolfd2gpu_launch_count(w2_ctx *c) { return c ? c->launches : 0; }

void *wolfd2gpu_stream(w2_ctx *c) { return c ? (void *)c->st : nullptr; }

int wolfd2gpu_chain_stats(w2_ctx *c, int *max_rounds, int *fallbacks) {
  if (!c) return W2_E_ARG;
  CK(cudaStreamSynchronize(c->st));
  Sync s;
  CK(cudaMemcpy(&s, c->dev.sync, sizeof(Sync), cudaMemcpyDeviceToHost));
  if (max_rounds) *max_rounds = s.max_rounds;
  if (fallbacks) *fallbacks = s.fallback;
  int zero[2] = {0, 0};
  CK(cudaMemcpy(&c->dev.sync->max_rounds, &zero[0], sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(&c->dev.sync->fallback, &zero[1], sizeof(int), cudaMemcpyHostToDevice));
  return W2_OK;
}

int wolfd2gpu_profile(w2_ctx *c, int enable) {
  if (!c) return W2_E_ARG;
  prof_collect(c);
  for (int k = 0; k < W2_K_NKINDS; ++k) {
    c->prof_ms[k] = 0.0;
    c->prof_n[k] = 0;
  }
  c->prof_on = enable != 0;
  return W2_OK;
}

int wolfd2gpu_profile_read(w2_ctx *c, int kind, double *total_ms, long long *count) {
  if (!c || kind < 0 || kind >= W2_K_NKINDS) return W2_E_ARG;
  prof_collect(c);
  if (total_ms) *total_ms = c->prof_ms[kind];
  if (count) *count = c->prof_n[kind];
  return W2_OK;
}

int wolfd2gpu_tune(w2_ctx *c, int chain_seg, int chain_warm, int threads, int blocks_per_sm) {
  if (!c) return W2_E_ARG;
  if (blocks_per_sm == -1 || blocks_per_sm == -2) {
    // -1: one colour per barrier for red/black SOR; -2: tiled sweeps at any size
    c->use_tiled = blocks_per_sm == -1 ? 0 : 2;
    blocks_per_sm = 0;
  } else if (blocks_per_sm == -5 || blocks_per_sm == -6) {
    // general-row mixed Poisson: one grid barrier per colour (-5) or the
    // tiled form on Cartesian grids (-6, the default)
    c->use_mixgt = blocks_per_sm == -6 ? 1 : 0;
    blocks_per_sm = 0;
  } else if (blocks_per_sm == -3 || blocks_per_sm == -4) {
    // tiled sweeps in 1024-thread blocks (-3) or back to 512-thread blocks (-4)
    c->tiled_wide = blocks_per_sm == -3 ? 1 : 0;
    blocks_per_sm = 0;
    if (c->metrics_ok) plan_tiles(c);
  }
  if (chain_seg < 0 || chain_warm < 0 || threads < 0 || blocks_per_sm < -2) return W2_E_ARG;
  if (chain_seg > 0 && chain_seg < 8) return fail(c, W2_E_ARG, "chain segment length must be >= 8");
  if (threads > 0) {
    if (threads % 32 || threads > kMaxThreads) return fail(c, W2_E_ARG, "threads must be a multiple of 32 <= %d", kMaxThreads);
    c->threads = threads;
  }
  if (blocks_per_sm > 0) c->blocks_per_sm = blocks_per_sm;
  c->seg_req = chain_seg;
  c->warm_req = chain_warm;
  return set_segments(c);
}

static int finish_coefficients(w2_ctx *c) {
  int *flag = &c->dev.sync->iout[7];
  CK(cudaMemsetAsync(flag, 0, sizeof(int), c->st));
  c->launches++;
  k_ppe_check<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, flag);
  CK(cudaGetLastError());
  int h = 1;
  CK(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->dev.ppe_unit = (h & 1) ? 0 : 1;
  c->dev.ppe_unit32 = (h & 2) ? 0 : 1;
  c->mg_coef_ok = false;
  plan_tiles(c);
  plan_mixgt(c);
  plan_mixed(c);
  return momentum_metrics(c);
}

int wolfd2gpu_set_face_profile(w2_ctx *c, int ireg, int jreg, int face, int var,
                               const double *values, int n) {
  if (!c) return W2_E_ARG;
  if (ireg < 1 || ireg > c->mgri || jreg < 1 || jreg > c->mgrj || face < W2_WEST ||
      face > W2_NORTH || var < 1 || var > 2)
    return fail(c, W2_E_ARG, "bad face profile key");
  const int want = (face == W2_WEST || face == W2_EAST) ? c->ny + 2 : c->nx + 2;
  if (values && n != want) return fail(c, W2_E_ARG, "face profile needs %d values, got %d", want, n);
  constexpr int kMaxProfiles = 16;
  const int key = ((ireg - 1) + (jreg - 1) * c->mgri + (face - 1) * c->mgri * c->mgrj) * 2 + (var - 1);
  if (!c->prof_idx) {
    c->prof_host.assign((size_t)c->mgri * c->mgrj * 8, -1);
    c->prof_len = std::max(c->nx, c->ny) + 2;
    if (!(c->prof_idx = dalloc<int>(c, c->prof_host.size())) ||
        !(c->prof = dalloc<double>(c, (size_t)kMaxProfiles * c->prof_len)))
      return fail(c, W2_E_CUDA, "out of device memory (face profiles)");
  }
  if (!values) {
    c->prof_host[key] = -1;
  } else {
    int off = c->prof_host[key];
    if (off < 0) {
      if (c->prof_used >= kMaxProfiles) return fail(c, W2_E_ARG, "at most %d face profiles", kMaxProfiles);
      off = c->prof_used++ * c->prof_len;
      c->prof_host[key] = off;
    }
    CK(cudaMemcpy(c->prof + off, values, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(c->prof_idx, c->prof_host.data(), c->prof_host.size() * sizeof(int),
                cudaMemcpyHostToDevice));
  c->dev.prof_idx = c->prof_idx;
  c->dev.prof = c->prof;
  return W2_OK;
}

int wolfd2gpu_set_precision(w2_ctx *c, int precision, int refine_sweeps) {
  if (!c) return W2_E_ARG;
  if (precision != W2_PREC_FP64 && precision != W2_PREC_MIXED)
    return fail(c, W2_E_ARG, "unknown precision mode %d", precision);
  if (refine_sweeps < 0) return fail(c, W2_E_ARG, "refine_sweeps < 0");
  c->prec_dropin = precision;
  c->refine_dropin = refine_sweeps;
  return W2_OK;
}

int wolfd2gpu_tune_mixed(w2_ctx *c, int sweeps_per_barrier, int threads, int mode) {
  if (!c) return W2_E_ARG;
  if (mode < 0 || mode > 3) return fail(c, W2_E_ARG, "tile mode must be 0, 1, 2 or 3");
  c->mixed_mode = mode;
  if (sweeps_per_barrier != 0 && !mixed_kernel(sweeps_per_barrier, true))
    return fail(c, W2_E_ARG, "sweeps per barrier must be 4 or 8");
  if (threads != 0 && (threads % 32 || threads < 64 || threads > kMixedThreads))
    return fail(c, W2_E_ARG, "thread limit must be a multiple of 32 in 64..%d", kMixedThreads);
  if (sweeps_per_barrier) c->mixed_K = sweeps_per_barrier;
  if (threads) c->mixed_threads = threads;
  if (c->metrics_ok) plan_mixed(c);
  return W2_OK;
}

int wolfd2gpu_set_tma(w2_ctx *c, int enable) {
  if (!c) return W2_E_ARG;
  c->use_tma = enable ? 1 : 0;
  if (c->metrics_ok) plan_mixed(c);
  return W2_OK;
}

int wolfd2gpu_set_metrics(w2_ctx *c, const double *const *metrics) {
  if (!c || !metrics) return W2_E_ARG;
  for (int k = 0; k < W2_NMETRIC; ++k) {
    if (!metrics[k]) return fail(c, W2_E_ARG, "metric %d is null", k);
    int rc = copy_in(c, c->met[k], metrics[k]);
    if (rc) return rc;
  }
  c->launches++;
  k_ppe_coef<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev);
  CK(cudaGetLastError());
  int rc = finish_coefficients(c);
  if (rc) return rc;
  c->metrics_ok = true;
  c->f32_metrics_ok = false;
  return W2_OK;
}

int wolfd2gpu_grid_metric(w2_ctx *c, const double *gx, const double *gy, double *const *metrics_out) {
  if (!c || !gx || !gy) return W2_E_ARG;
  double *x = c->stage[0], *y = c->stage[1], *xu = c->stage[2], *yu = c->stage[3], *xv = c->stage[4],
         *yv = c->stage[5];
  double *xc = c->dev.pa1, *yc = c->dev.pa2;  // free until the PPE coefficients are formed
  for (int k = 0; k < 6; ++k) CK(cudaMemsetAsync(c->stage[k], 0, c->nf * 8, c->st));
  CK(cudaMemsetAsync(xc, 0, c->nf * 8, c->st));
  CK(cudaMemsetAsync(yc, 0, c->nf * 8, c->st));
  for (int k = 0; k < W2_NMETRIC; ++k) CK(cudaMemsetAsync(c->met[k], 0, c->nf * 8, c->st));
  int rc = copy_in(c, x, gx);
  if (!rc) rc = copy_in(c, y, gy);
  if (rc) return rc;
  const int gb = grid_blocks(c);
  k_mirror<<<1, 256, 0, c->st>>>(c->dev, x, y);
  k_fullgrid_uv<<<gb, c->threads, 0, c->st>>>(c->dev, x, y, xu, yu, xv, yv);
  k_fullgrid_c<<<gb, c->threads, 0, c->st>>>(c->dev, xu, yv, xc, yc);
  MetricOut mo;
  double **a = c->met;
  mo.rau = a[M_RAU]; mo.rbu = a[M_RBU]; mo.rbv = a[M_RBV]; mo.rgv = a[M_RGV];
  mo.ran = a[M_RAN]; mo.rbn = a[M_RBN]; mo.rgn = a[M_RGN];
  mo.rac = a[M_RAC]; mo.rbc = a[M_RBC]; mo.rgc = a[M_RGC];
  mo.dju = a[M_DJU]; mo.djv = a[M_DJV]; mo.djc = a[M_DJC]; mo.djn = a[M_DJN];
  mo.xen = a[M_XEN]; mo.yen = a[M_YEN]; mo.xzn = a[M_XZN]; mo.yzn = a[M_YZN];
  mo.xec = a[M_XEC]; mo.yec = a[M_YEC]; mo.xzc = a[M_XZC]; mo.yzc = a[M_YZC];
  mo.xeu = a[M_XEU]; mo.yeu = a[M_YEU]; mo.xzv = a[M_XZV]; mo.yzv = a[M_YZV];
  mo.xzu = a[M_XZU]; mo.yzu = a[M_YZU]; mo.xev = a[M_XEV]; mo.yev = a[M_YEV];
  k_metric<<<gb, c->threads, 0, c->st>>>(c->dev, mo, x, y, xu, yu, xv, yv, xc, yc);
  c->launches += 4;
  CK(cudaGetLastError());
  if (metrics_out)
    for (int k = 0; k < W2_NMETRIC; ++k)
      if (metrics_out[k]) {
        rc = copy_out(c, metrics_out[k], c->met[k]);
        if (rc) return rc;
      }
  CK(cudaMemsetAsync(xc, 0, c->nf * 8, c->st));
  CK(cudaMemsetAsync(yc, 0, c->nf * 8, c->st));
  c->launches++;
  k_ppe_coef<<<gb, c->threads, 0, c->st>>>(c->dev);
  CK(cudaGetLastError());
  rc = finish_coefficients(c);
  if (rc) return rc;
  c->metrics_ok = true;
  c->f32_metrics_ok = false;
  return W2_OK;
}

// ---- drop-ins -------------------------------------------------------------

int wolfd2gpu_naux_momentum(w2_ctx *c, const int *nx, const int *ny, const int *mqiter,
                            const double *dk, const double *re, const double *fr,
                            const double *qtol, const double *d, const double *dn,
                            const double *un, const double *vn, double *us, double *vs,
                            int *nQLiter) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !mqiter || !dk || !re || !qtol || !un || !vn || !us || !vs || !nQLiter)
    return fail(c, W2_E_ARG, "bad argument");
  // density enters only through the buoyancy term of YMomentum
  // (momentum.f:703); all-zero (or absent) density arrays leave it out
  bool buoy = false;
  {
    const double *arrs[2] = {d, dn};
    for (const double *a : arrs)
      if (a)
        for (int j = 0; j <= c->ny + 1 && !buoy; ++j)
          for (int i = 0; i <= c->nx + 1; ++i)
            if (a[i + (size_t)j * (c->mnx + 1)] != 0.0) {
              buoy = true;
              break;
            }
  }
  if (buoy && (!d || !dn || !fr)) return fail(c, W2_E_ARG, "buoyancy needs d, dn and fr");
  double *dun = c->stage[0], *dvn = c->stage[1], *dus = c->stage[2], *dvs = c->stage[3];
  double *dd = c->stage[4], *ddn = c->stage[5];
  if ((rc = copy_in(c, dun, un)) || (rc = copy_in(c, dvn, vn)) || (rc = copy_in(c, dus, us)) ||
      (rc = copy_in(c, dvs, vs)))
    return rc;
  if (buoy && ((rc = copy_in(c, dd, d)) || (rc = copy_in(c, ddn, dn)))) return rc;
  c->launches++;
  k_naux_init<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, dun, dvn, dus, dvs);
  CK(cudaGetLastError());
  if ((rc = launch_naux(c, *mqiter, *dk, *re, *qtol, dun, dvn, dus, dvs, buoy ? dd : nullptr,
                        buoy ? ddn : nullptr, buoy ? *fr : 0.0)))
    return rc;
  if ((rc = copy_out(c, us, dus)) || (rc = copy_out(c, vs, dvs))) return rc;
  CK(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(StepOut), cudaMemcpyDeviceToHost, c->st));
  if ((rc = check_sync(c))) return rc;
  *nQLiter = c->h_out->nql;
  return W2_OK;
}

int wolfd2gpu_ppe(w2_ctx *c, const int *nx, const int *ny, const int *lCartesGrid,
                  const int *nPpeSolver, const int *msorit, int *nSorConv, const double *dk,
                  const double *sortol, const double *sorrel, const double *u, const double *v,
                  double *p) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !lCartesGrid || !nPpeSolver || !msorit || !nSorConv || !dk ||
      !sortol || !sorrel || !u || !v || !p)
    return fail(c, W2_E_ARG, "bad argument");
  double *du = c->stage[0], *dv = c->stage[1], *dp = c->stage[2];
  if ((rc = copy_in(c, du, u)) || (rc = copy_in(c, dv, v)) || (rc = copy_in(c, dp, p))) return rc;
  if ((rc = launch_ppe(c, *lCartesGrid ? 1 : 0, *nPpeSolver, *msorit, *dk, *sortol, *sorrel, du, dv, dp)))
    return rc;
  if ((rc = copy_out(c, p, dp))) return rc;
  CK(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(StepOut), cudaMemcpyDeviceToHost, c->st));
  if ((rc = check_sync(c))) return rc;
  *nSorConv = c->h_out->nsor;
  return W2_OK;
}

int wolfd2gpu_project(w2_ctx *c, const int *nx, const int *ny, const double *dk, const double *p,
                      double *u, double *v) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !dk || !p || !u || !v) return fail(c, W2_E_ARG, "bad argument");
  double *du = c->stage[0], *dv = c->stage[1], *dp = c->stage[2];
  if ((rc = copy_in(c, du, u)) || (rc = copy_in(c, dv, v)) || (rc = copy_in(c, dp, p))) return rc;
  c->launches++;
  k_project<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, *dk, dp, du, dv);
  CK(cudaGetLastError());
  if ((rc = copy_out(c, u, du)) || (rc = copy_out(c, v, dv))) return rc;
  return check_sync(c);
}

static int bc_dropin(w2_ctx *c, const int *nx, const int *ny, int ops, double *u, double *v, double *p) {
  if (!c) return W2_E_ARG;
  if (!dims_match(c, nx, ny)) return fail(c, W2_E_ARG, "bad argument");
  double *du = c->stage[0], *dv = c->stage[1], *dp = c->stage[2];
  int rc;
  if (u && (rc = copy_in(c, du, u))) return rc;
  if (v && (rc = copy_in(c, dv, v))) return rc;
  if (p && (rc = copy_in(c, dp, p))) return rc;
  if ((rc = launch_bc(c, ops, du, dv, dp))) return rc;
  if (u && (rc = copy_out(c, u, du))) return rc;
  if (v && (rc = copy_out(c, v, dv))) return rc;
  if (p && (rc = copy_out(c, p, dp))) return rc;
  return check_sync(c);
}

int wolfd2gpu_vel_bound_cond(w2_ctx *c, const int *nx, const int *ny, double *u, double *v) {
  if (!u || !v) return fail(c, W2_E_ARG, "bad argument");
  return bc_dropin(c, nx, ny, BC_VEL, u, v, nullptr);
}

int wolfd2gpu_pres_bound_cond(w2_ctx *c, const int *nx, const int *ny, double *p) {
  if (!p) return fail(c, W2_E_ARG, "bad argument");
  return bc_dropin(c, nx, ny, BC_PRES, nullptr, nullptr, p);
}

int wolfd2gpu_vel_outflow_bcs(w2_ctx *c, const int *nx, const int *ny, double *u, double *v) {
  if (!u || !v) return fail(c, W2_E_ARG, "bad argument");
  return bc_dropin(c, nx, ny, BC_OUTFLOW, u, v, nullptr);
}

int wolfd2gpu_diff_max_norm(w2_ctx *c, const int *nx, const int *ny, const double *un,
                            const double *u, double *result) {
  if (!c) return W2_E_ARG;
  if (!dims_match(c, nx, ny) || !un || !u || !result) return fail(c, W2_E_ARG, "bad argument");
  int rc;
  double *da = c->stage[0], *db = c->stage[1];
  if ((rc = copy_in(c, da, un)) || (rc = copy_in(c, db, u))) return rc;
  unsigned long long *slot = &c->dev.sync->red[9];
  CK(cudaMemsetAsync(slot, 0, 8, c->st));
  c->launches++;
  k_diff_norm<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, da, db, slot);
  CK(cudaGetLastError());
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, slot, 8, cudaMemcpyDeviceToHost, c->st));
  if ((rc = check_sync(c))) return rc;
  memcpy(result, &bits, 8);
  return W2_OK;
}

int wolfd2gpu_filter(w2_ctx *c, const int *nx, const int *ny, const int *ncomp, const double *fp,
                     double *qu) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !ncomp || !fp || !qu || (*ncomp != 1 && *ncomp != 2))
    return fail(c, W2_E_ARG, "bad argument");
  double *dq = c->stage[0], *dh = c->stage[1];
  if ((rc = copy_in(c, dq, qu))) return rc;
  c->launches++;
  k_filter<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, *ncomp == 1 ? MK_FU : MK_FV, *fp, dq, dh);
  CK(cudaGetLastError());
  if ((rc = copy_out(c, qu, dh))) return rc;
  return check_sync(c);
}

}  // extern "C"

namespace {

// Thermal tables of a call: every flag checked as TempBoundCond's select
// cases do (bound_cond.f:1098-1183, 'stop' on an unknown flag), then
// uploaded.  The chain of the interior points is made on first use.
int therm_prepare(w2_ctx *c, const int *nTRgType, const int *nTemBdTp, const double *dTRgVal,
                  const double *dHGSTval, ThermTables *tt) {
  const int mg = c->mgri * c->mgrj;
  for (int jr = 1; jr <= c->nrj; ++jr)
    for (int ir = 1; ir <= c->nri; ++ir) {
      const int rt = nTRgType[(ir - 1) + (jr - 1) * c->mgri];
      if (rt < RT_NOSRCE || rt > RT_TEMPER)
        return fail(c, W2_E_BCFLAG, "Wrong nTRgType flag in region %d,%d", ir, jr);
      if (rt == RT_TEMPER) continue;
      for (int s = 1; s <= 4; ++s) {
        const int bt = nTemBdTp[(ir - 1) + (jr - 1) * c->mgri + (s - 1) * mg];
        if (bt < BT_INTERN || bt > BT_HTFLUX)
          return fail(c, W2_E_BCFLAG, "Wrong nTemBdTp %c flag in region %d,%d", "WESN"[s - 1], ir, jr);
      }
    }
  if (!c->therm_alloc) {
    const int n = (c->nx - 1) * (c->ny - 1);
    int rc;
    if ((rc = make_chain(c, c->therm_ch, n, true))) return rc;
    if (!(c->d_ttab = dalloc<int>(c, (size_t)5 * mg)) || !(c->d_tval = dalloc<double>(c, (size_t)2 * mg)))
      return fail(c, W2_E_CUDA, "out of device memory (thermal tables)");
    const int wmax = (int)walk_stage_bytes(sizeof(double), kMaxThreads);
    if (cudaFuncSetAttribute((const void *)k_therm, cudaFuncAttributeMaxDynamicSharedMemorySize, wmax) !=
        cudaSuccess)
      return fail(c, W2_E_CUDA, "shared memory attribute (thermal)");
    c->therm_alloc = true;
  }
  CK(cudaMemcpyAsync(c->d_ttab, nTRgType, sizeof(int) * mg, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->d_ttab + mg, nTemBdTp, sizeof(int) * 4 * mg, cudaMemcpyHostToDevice, c->st));
  if (dTRgVal) CK(cudaMemcpyAsync(c->d_tval, dTRgVal, sizeof(double) * mg, cudaMemcpyHostToDevice, c->st));
  if (dHGSTval)
    CK(cudaMemcpyAsync(c->d_tval + mg, dHGSTval, sizeof(double) * mg, cudaMemcpyHostToDevice, c->st));
  // the uploads read pageable host memory: finish them before the caller's
  // arrays can change
  CK(cudaStreamSynchronize(c->st));
  *tt = ThermTables{c->d_ttab, c->d_ttab + mg, c->d_tval, c->d_tval + mg};
  c->therm_ch.L = c->dev.seg;
  c->therm_ch.nseg = (c->therm_ch.n + c->dev.seg - 1) / c->dev.seg;
  return W2_OK;
}

}  // namespace

extern "C" {

int wolfd2gpu_temp_bound_cond(w2_ctx *c, const int *nx, const int *ny, const int *nTRgType,
                              const int *nTemBdTp, const double *dTRgVal, double *t) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !nTRgType || !nTemBdTp || !dTRgVal || !t)
    return fail(c, W2_E_ARG, "bad argument");
  ThermTables tt;
  if ((rc = therm_prepare(c, nTRgType, nTemBdTp, dTRgVal, nullptr, &tt))) return rc;
  double *dt = c->stage[0];
  if ((rc = copy_in(c, dt, t))) return rc;
  c->launches++;
  k_temp_bc<<<1, c->threads, 0, c->st>>>(c->dev, tt, dt);
  CK(cudaGetLastError());
  if ((rc = copy_out(c, t, dt))) return rc;
  return check_sync(c);
}

int wolfd2gpu_therm_energy(w2_ctx *c, const int *nx, const int *ny, const int *nTRgType,
                           const int *nTemBdTp, const double *dk, const double *pe,
                           const double *dTRgVal, const double *dHGSTval, const double *un,
                           const double *vn, const double *u, const double *v, const double *tn,
                           double *t) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !nTRgType || !nTemBdTp || !dk || !pe || !dTRgVal || !dHGSTval || !un ||
      !vn || !u || !v || !tn || !t)
    return fail(c, W2_E_ARG, "bad argument");
  ThermTables tt;
  if ((rc = therm_prepare(c, nTRgType, nTemBdTp, dTRgVal, dHGSTval, &tt))) return rc;
  double *s[6] = {c->stage[0], c->stage[1], c->stage[2], c->stage[3], c->stage[4], c->stage[5]};
  const double *h[6] = {un, vn, u, v, tn, t};
  for (int k = 0; k < 6; ++k)
    if ((rc = copy_in(c, s[k], h[k]))) return rc;
  const Dev &d = c->dev;
  ThermArgs A{tt, *dk, *pe, s[0], s[1], s[2], s[3], s[4], s[5], d.cj1x, d.cj2x, d.c1sx, d.c2sx, c->therm_ch};
  Dev dv = d;
  int blocks = pick_blocks(c, (const void *)k_therm, (long)c->nx * c->ny, naux_smem(c));
  void *args[] = {&dv, &A};
  if ((rc = coop(c, (const void *)k_therm, blocks, args, naux_smem(c)))) return rc;
  if ((rc = copy_out(c, t, s[5]))) return rc;
  return check_sync(c);
}

int wolfd2gpu_filter_t(w2_ctx *c, const int *nx, const int *ny, const int *nTRgType, const double *fp,
                       double *t) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !nTRgType || !fp || !t) return fail(c, W2_E_ARG, "bad argument");
  // only nTRgType matters here; it goes to a table of its own, so the
  // tables of the thermal loop stay as they were
  const int mg = c->mgri * c->mgrj;
  if (!c->d_trt_filter && !(c->d_trt_filter = dalloc<int>(c, mg)))
    return fail(c, W2_E_CUDA, "out of device memory (thermal tables)");
  CK(cudaMemcpyAsync(c->d_trt_filter, nTRgType, sizeof(int) * mg, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  ThermTables tt{c->d_trt_filter, nullptr, nullptr, nullptr};
  double *dq = c->stage[0], *dh = c->stage[1];
  if ((rc = copy_in(c, dq, t))) return rc;
  c->launches++;
  k_filter_t<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, tt, *fp, dq, dh);
  CK(cudaGetLastError());
  if ((rc = copy_out(c, t, dh))) return rc;
  return check_sync(c);
}

int wolfd2gpu_small_scale(w2_ctx *c, const int *nx, const int *ny, const int *initflg,
                          const int *nthermen, const int *lCartesGrid, const int *nTRgType,
                          const int *nTemBdTp, const int *nPpeSolver, const int *msorit,
                          const double *dlref, const double *uref, const double *tref,
                          const double *tmax, const double *dka, const double *re, const double *pe,
                          const double *sortol, const double *sorrel, const double *fp,
                          const double *cu0, const double *TsCoef, const double *HsCoef,
                          const double *TemCoef, const double *bnumc, const double *rmax,
                          const double *rlc, const double *dTRgVal, const double *u1, const double *v1,
                          const double *t1, double *uss, double *vss, double *pss, double *tss,
                          int *nSorConv) {
  (void)nthermen;  // the reference passes it and does not use it
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !initflg || !lCartesGrid || !nTRgType || !nTemBdTp || !nPpeSolver ||
      !msorit || !dlref || !uref || !tref || !tmax || !dka || !re || !pe || !sortol || !sorrel || !fp ||
      !cu0 || !TsCoef || !HsCoef || !TemCoef || !bnumc || !rmax || !rlc || !dTRgVal || !u1 || !v1 || !t1 ||
      !uss || !vss || !pss || !tss || !nSorConv)
    return fail(c, W2_E_ARG, "bad argument");
  if (*nPpeSolver < 1 || *nPpeSolver > 6) return fail(c, W2_E_ARG, "nPpeSolver must be 1..6");
  ThermTables tt;
  if ((rc = therm_prepare(c, nTRgType, nTemBdTp, dTRgVal, nullptr, &tt))) return rc;
  AtdState &S = c->atd;
  if (!S.area) {
    double **arr[] = {&S.area, &S.xz, &S.xe, &S.yz, &S.ye, &S.rj, &S.ul, &S.vl, &S.tl,
                      &S.uc, &S.vc, &S.uf, &S.vf, &S.tf, &S.ff};
    for (double **a : arr)
      if (!(*a = dalloc<double>(c, c->nf))) return fail(c, W2_E_CUDA, "out of device memory (small scales)");
    for (int l = 0; l < 9; ++l)
      if (!(S.map[l] = dalloc<double>(c, c->nf))) return fail(c, W2_E_CUDA, "out of device memory (maps)");
    for (int k = 0; k < 4; ++k)
      if (!(c->atd_io[k] = dalloc<double>(c, c->nf))) return fail(c, W2_E_CUDA, "out of device memory");
    if (!(S.tarea = dalloc<double>(c, 1))) return fail(c, W2_E_CUDA, "out of device memory");
  }
  double *dus = c->atd_io[0], *dvs = c->atd_io[1], *dps = c->atd_io[2], *dts = c->atd_io[3];
  const int NX = c->nx, NY = c->ny;
  const size_t ld = c->ld;
  if (*initflg <= 0) {
    // small_scale.f:198-243 on the host: the maps are seeded along one
    // sequential chain (j fastest), the areas summed in the reference's order
    const double rc0 = 0.20710678119, A = 4.82842712474, B = 1.47839783948;
    double um = 0.92, vm = 0.31, tm = 0.50;
    std::vector<double> h(9 * c->nf, 0.0);
    for (int i = 0; i <= NX + 1; i++)
      for (int j = 0; j <= NY + 1; j++)
        for (int l = 0; l < 3; l++) {
          um = rc0 * A * um * (1.0 - B * std::fabs(um));
          vm = rc0 * A * vm * (1.0 - B * std::fabs(vm));
          tm = rc0 * A * tm * (1.0 - B * std::fabs(tm));
          const size_t o = (size_t)i + (size_t)j * ld;
          h[(size_t)l * c->nf + o] = um;
          h[(size_t)(3 + l) * c->nf + o] = vm;
          h[(size_t)(6 + l) * c->nf + o] = tm;
        }
    for (int l = 0; l < 9; ++l)
      CK(cudaMemcpy(S.map[l], h.data() + (size_t)l * c->nf, c->nf * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<double> djc(c->nf), area(c->nf, 0.0);
    CK(cudaStreamSynchronize(c->st));
    CK(cudaMemcpy(djc.data(), c->met[M_DJC], c->nf * sizeof(double), cudaMemcpyDeviceToHost));
    double tarea = 0.0;
    for (int i = 1; i <= NX; i++)
      for (int j = 1; j <= NY; j++) {
        const size_t o = (size_t)i + (size_t)j * ld;
        area[o] = 1.0 / djc[o];
        tarea = tarea + area[o];
      }
    CK(cudaMemcpy(S.area, area.data(), c->nf * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(S.tarea, &tarea, sizeof(double), cudaMemcpyHostToDevice));
    for (size_t k = 0; k < (size_t)(c->mnx + 1) * (size_t)(c->mny + 1); ++k) {
      const size_t i = k % (size_t)(c->mnx + 1), j = k / (size_t)(c->mnx + 1);
      if (i <= (size_t)NX + 1 && j <= (size_t)NY + 1) uss[k] = vss[k] = tss[k] = 0.0;
    }
    if (*initflg < 0) {
      *nSorConv = 0;
      return W2_OK;
    }
  }
  const AtdParams P{*dlref, *uref, *tref, *tmax, *dka, *re, *pe, fp[0], fp[1], fp[3],
                    *cu0, *TsCoef, *HsCoef, *TemCoef, *bnumc, *rmax, *rlc};
  double *d1 = c->stage[0], *d2 = c->stage[1], *d3 = c->stage[2];
  if ((rc = copy_in(c, d1, u1)) || (rc = copy_in(c, d2, v1)) || (rc = copy_in(c, d3, t1)) ||
      (rc = copy_in(c, dus, uss)) || (rc = copy_in(c, dvs, vss)) || (rc = copy_in(c, dps, pss)) ||
      (rc = copy_in(c, dts, tss)))
    return rc;
  const Dev &d = c->dev;
  const int gb = grid_blocks(c), T = c->threads;
  cudaStream_t st = c->st;
  c->launches += 13;
  k_atd_prep<<<gb, T, 0, st>>>(d, S, P, d1, d2, d3);
  k_temp_bc<<<1, T, 0, st>>>(d, tt, S.tf);
  // the high-pass parts: the field minus its Shuman-filtered copy
  k_filter<<<gb, T, 0, st>>>(d, MK_FU, P.fpu, S.uc, S.ff);
  k_atd_highpass<<<gb, T, 0, st>>>(d, S.uc, S.ff, S.uf);
  k_filter<<<gb, T, 0, st>>>(d, MK_FV, P.fpv, S.vc, S.ff);
  k_atd_highpass<<<gb, T, 0, st>>>(d, S.vc, S.ff, S.vf);
  k_filter_t<<<gb, T, 0, st>>>(d, tt, P.fpt, S.tf, S.ff);
  k_atd_highpass<<<gb, T, 0, st>>>(d, S.tl, S.ff, S.tf);
  k_atd_cells<<<gb, T, 0, st>>>(d, S, P, tt, dus, dvs, dts);
  k_atd_bc<<<1, T, 0, st>>>(d, tt, dus, dvs, dps, dts);
  k_atd_zero_p<<<gb, T, 0, st>>>(d, dps);
  k_atd_bc<<<1, T, 0, st>>>(d, tt, dus, dvs, dps, dts);
  CK(cudaGetLastError());
  if ((rc = check_sync(c))) return rc;
  if ((rc = launch_ppe(c, *lCartesGrid ? 1 : 0, *nPpeSolver, *msorit, *dka, *sortol, *sorrel, dus, dvs, dps)))
    return rc;
  CK(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(StepOut), cudaMemcpyDeviceToHost, st));
  c->launches += 2;
  k_atd_bc<<<1, T, 0, st>>>(d, tt, dus, dvs, dps, dts);
  k_project<<<gb, T, 0, st>>>(d, *dka, dps, dus, dvs);
  CK(cudaGetLastError());
  if ((rc = copy_out(c, uss, dus)) || (rc = copy_out(c, vss, dvs)) || (rc = copy_out(c, pss, dps)) ||
      (rc = copy_out(c, tss, dts)))
    return rc;
  if ((rc = check_sync(c))) return rc;
  *nSorConv = c->h_out->nsor;
  return W2_OK;
}

int wolfd2gpu_eq_state(w2_ctx *c, const int *nx, const int *ny, const double *uref,
                       const double *densref, const double *tmax, const double *tref,
                       const double *rconst, const double *p, const double *t, double *den) {
  int rc = ready(c);
  if (rc) return rc;
  if (!dims_match(c, nx, ny) || !uref || !densref || !tmax || !tref || !rconst || !p || !t || !den)
    return fail(c, W2_E_ARG, "bad argument");
  double *dp = c->stage[0], *dt = c->stage[1], *dd = c->stage[2];
  if ((rc = copy_in(c, dp, p)) || (rc = copy_in(c, dt, t)) || (rc = copy_in(c, dd, den))) return rc;
  c->launches++;
  k_eq_state<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, *uref, *densref, *tmax, *tref, *rconst, dp, dt,
                                                       dd);
  CK(cudaGetLastError());
  if ((rc = copy_out(c, den, dd))) return rc;
  return check_sync(c);
}

int wolfd2gpu_set_thermal(w2_ctx *c, const w2_thermal *tp, const int *nTRgType, const int *nTemBdTp,
                          const double *dTRgVal, const double *dHGSTval) {
  int rc = ready(c);
  if (rc) return rc;
  if (!tp || (tp->nthermen != 1 && tp->neqstate != 1)) {
    c->therm_on = false;
    return W2_OK;
  }
  if (!nTRgType || !nTemBdTp || !dTRgVal || !dHGSTval) return fail(c, W2_E_ARG, "bad argument");
  if (tp->nmeiter < 1 || (tp->nthermen == 1 && !(tp->pe != 0.0)))
    return fail(c, W2_E_ARG, "nmeiter must be >= 1 and pe non-zero");
  if ((rc = therm_prepare(c, nTRgType, nTemBdTp, dTRgVal, dHGSTval, &c->therm_tt))) return rc;
  double **bufs[] = {&c->T[0], &c->T[1], &c->Dd, &c->Ddn, &c->Up, &c->Vp, &c->Tp};
  for (double **b : bufs)
    if (!*b && !(*b = dalloc<double>(c, c->nf))) return fail(c, W2_E_CUDA, "out of device memory (thermal fields)");
  c->therm_p = *tp;
  c->therm_on = true;
  return W2_OK;
}

int wolfd2gpu_load_thermal(w2_ctx *c, const double *t, const double *d) {
  if (!c || !c->therm_on || !t) return fail(c, W2_E_ARG, "thermal loop not set, or t missing");
  int rc;
  snap_fence(c);
  if ((rc = copy_in(c, c->T[c->cur], t))) return rc;
  if (d) {
    if ((rc = copy_in(c, c->Dd, d))) return rc;
  } else {
    CK(cudaMemsetAsync(c->Dd, 0, c->nf * sizeof(double), c->st));
  }
  return W2_OK;
}

int wolfd2gpu_store_thermal(w2_ctx *c, double *t, double *d) {
  if (!c || !c->therm_on) return fail(c, W2_E_ARG, "thermal loop not set");
  int rc;
  if (t && (rc = copy_out(c, t, c->T[c->cur]))) return rc;
  if (d && (rc = copy_out(c, d, c->Dd))) return rc;
  CK(cudaStreamSynchronize(c->st));
  return W2_OK;
}

// ---- device-resident time loop ----------------------------------------------

int wolfd2gpu_load_fields(w2_ctx *c, const double *u, const double *v, const double *p) {
  if (!c || !u || !v || !p) return W2_E_ARG;
  int rc;
  snap_fence(c);
  if ((rc = copy_in(c, c->U[c->cur], u)) || (rc = copy_in(c, c->V[c->cur], v)) ||
      (rc = copy_in(c, c->P[c->cur], p)))
    return rc;
  return W2_OK;
}

// Snapshot of the current time level (u, v, p; t and d with the energy
// equation) into host arrays on a copy stream, ordered after the work issued
// so far; the next steps run meanwhile (the copy engines work beside the
// SMs), and the first launch that overwrites the level waits for the copy.
int wolfd2gpu_snapshot(w2_ctx *c, double *u, double *v, double *p, double *t, double *d) {
  if (!c || !u || !v || !p) return W2_E_ARG;
  if ((t || d) && !c->therm_on) return fail(c, W2_E_ARG, "t, d snapshots need the thermal loop");
  if (!c->cst) {
    if (cudaStreamCreateWithFlags(&c->cst, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_snap_src, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_snap_done, cudaEventDisableTiming) != cudaSuccess)
      return fail(c, W2_E_CUDA, "snapshot stream or events");
  }
  // a previous snapshot into other host buffers must be complete
  if (c->snap_level >= 0) CK(cudaEventSynchronize(c->ev_snap_done));
  CK(cudaEventRecord(c->ev_snap_src, c->st));
  CK(cudaStreamWaitEvent(c->cst, c->ev_snap_src, 0));
  const int L = c->cur;
  const double *src[5] = {c->U[L], c->V[L], c->P[L], c->therm_on ? c->T[L] : nullptr, c->Dd};
  double *dst[5] = {u, v, p, t, d};
  for (int k = 0; k < 5; ++k) {
    if (!dst[k]) continue;
    CK(cudaMemcpy2DAsync(dst[k], (size_t)(c->mnx + 1) * 8, src[k], (size_t)c->ld * 8, (size_t)(c->nx + 2) * 8,
                         c->ny + 2, cudaMemcpyDeviceToHost, c->cst));
  }
  CK(cudaEventRecord(c->ev_snap_done, c->cst));
  c->snap_level = L;
  return W2_OK;
}

// Self-test of the device-wait limit (k_selftest_wait): returns the status
// the host reads after a grid barrier that one block never reaches, which is
// W2_E_TIMEOUT after the limit (4 s); the barrier state is cleared, so the
// context stays usable.
int wolfd2gpu_selftest_wait(w2_ctx *c) {
  if (!c) return W2_E_ARG;
  CK(cudaStreamSynchronize(c->st));
  Dev d = c->dev;
  void *args[] = {&d};
  c->launches++;
  cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_selftest_wait, dim3(2), dim3(32), args, 0, c->st);
  if (e != cudaSuccess) return fail(c, W2_E_CUDA, "cooperative launch: %s", cudaGetErrorString(e));
  return check_sync(c);
}

// Wait until the last snapshot's host arrays are filled.
int wolfd2gpu_snapshot_wait(w2_ctx *c) {
  if (!c) return W2_E_ARG;
  if (c->ev_snap_done) CK(cudaEventSynchronize(c->ev_snap_done));
  return W2_OK;
}

int wolfd2gpu_store_fields(w2_ctx *c, double *u, double *v, double *p) {
  if (!c) return W2_E_ARG;
  int rc;
  if (u && (rc = copy_out(c, u, c->U[c->cur]))) return rc;
  if (v && (rc = copy_out(c, v, c->V[c->cur]))) return rc;
  if (p && (rc = copy_out(c, p, c->P[c->cur]))) return rc;
  CK(cudaStreamSynchronize(c->st));
  return W2_OK;
}

int wolfd2gpu_device_fields(w2_ctx *c, double **u, double **v, double **p, int *ld) {
  if (!c) return W2_E_ARG;
  if (u) *u = c->U[c->cur];
  if (v) *v = c->V[c->cur];
  if (p) *p = c->P[c->cur];
  if (ld) *ld = c->ld;
  return W2_OK;
}

int wolfd2gpu_sync(w2_ctx *c) {
  if (!c) return W2_E_ARG;
  return check_sync(c);
}

static int check_params(w2_ctx *c, const w2_params *prm) {
  if (!prm) return fail(c, W2_E_ARG, "null params");
  if (prm->npsolver < 1 || prm->npsolver > 6 || prm->msorit < 1 || prm->mqiter < 1)
    return fail(c, W2_E_ARG, "bad solver parameters");
  if (prm->precision == W2_PREC_MIXED) {
    if (prm->refine_sweeps < 0) return fail(c, W2_E_ARG, "refine_sweeps < 0");
    return mixed_check(c, prm->lcartes, prm->npsolver);
  }
  if (prm->precision != W2_PREC_FP64)
    return fail(c, W2_E_ARG, "unknown precision mode %d", prm->precision);
  return W2_OK;
}

int wolfd2gpu_cold_start(w2_ctx *c, const w2_params *prm, int *nSorConv) {
  NvtxRange nv("wolfd2gpu_cold_start");
  int rc = ready(c);
  if (rc) return rc;
  if ((rc = check_params(c, prm))) return rc;
  snap_fence(c);
  double *u = c->U[c->cur], *v = c->V[c->cur], *p = c->P[c->cur];
  if ((rc = launch_bc(c, BC_VEL, u, v, p))) return rc;
  if (prm->precision == W2_PREC_MIXED) {
    ProfScope ps(c, W2_K_PPE);
    rc = launch_ppe_mixed(c, prm->lcartes, prm->msorit, prm->dk, prm->sortol, prm->sorrel,
                          prm->refine_sweeps, u, v, p, c->d_out);
  } else {
    rc = launch_ppe(c, prm->lcartes, prm->npsolver, prm->msorit, prm->dk, prm->sortol, prm->sorrel, u, v, p);
  }
  if (rc) return rc;
  if ((rc = launch_bc(c, BC_PRES, u, v, p))) return rc;
  c->launches++;
  k_project<<<grid_blocks(c), c->threads, 0, c->st>>>(c->dev, prm->dk, p, u, v);
  CK(cudaGetLastError());
  if ((rc = launch_bc(c, BC_VEL, u, v, p))) return rc;
  CK(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(StepOut), cudaMemcpyDeviceToHost, c->st));
  if ((rc = check_sync(c))) return rc;
  if (nSorConv) *nSorConv = c->h_out->nsor;
  return W2_OK;
}

}  // extern "C"

namespace {

// The launches of `nsteps` whole steps from time level c->cur (advanced as
// they are issued), step s writing outs[s].
// One step of main.f:690-972 with the energy equation: momentum/energy
// iterations (main.f:736-879) whose launches after convergence skip on the
// device, then the step tail (kernels in w2_thermal.cuh).
int issue_thermal_step(w2_ctx *c, const w2_params *prm, const double *un, const double *vn,
                       const double *pn, double *us, double *vs, double *p, StepOut *o) {
  const w2_thermal &tp = c->therm_p;
  const bool therm = tp.nthermen == 1, eqs = tp.neqstate == 1;
  int nme = tp.nmeiter;
  if (!therm && nme > 0) nme = 1;  // main.f:736
  const int gb = grid_blocks(c);
  const int a = c->cur, b = 1 - a;
  double *tn = c->T[a], *ts = c->T[b];
  Dev d = c->dev;
  int rc = W2_OK;
  {
    ProfScope ps(c, W2_K_COPY);
    c->launches++;
    k_copy_th<<<gb, c->threads, 0, c->st>>>(d, us, un, vs, vn, p, pn, ts, tn, c->Ddn, c->Dd);
    CK(cudaGetLastError());
  }
  for (int l = 1; l <= nme; ++l) {
    Dev dl = d;
    dl.me_gate = l >= 2 ? 1 : 0;
    dl.den = c->Dd;
    dl.denn = c->Ddn;
    dl.fr = prm->fr;
    if (l >= 2) {
      c->launches++;
      k_me_begin<<<gb, c->threads, 0, c->st>>>(dl, un, vn, us, vs, ts, c->Up, c->Vp, c->Tp);
      CK(cudaGetLastError());
    }
    {
      int blocks = pick_blocks(c, (const void *)k_naux, (long)c->nx * c->ny, naux_smem(c));
      ProfScope ps(c, W2_K_MOMENTUM);
      int mq = prm->mqiter;
      double dk = prm->dk, re = prm->re, qtol = prm->qtol;
      void *args[] = {&dl, &mq, &dk, &re, &qtol, (void *)&un, (void *)&vn, &us, &vs, &o};
      if ((rc = coop(c, (const void *)k_naux, blocks, args, naux_smem(c)))) return rc;
    }
    {
      ProfScope ps(c, W2_K_BC);
      c->launches++;
      k_bc<<<1, c->threads, 0, c->st>>>(dl, BC_VEL | BC_PRES, us, vs, p);
      CK(cudaGetLastError());
    }
    {
      ProfScope ps(c, W2_K_PPE);
      if (tiled_applies(c, prm->npsolver, prm->sorrel)) {
        if ((rc = launch_ppe_tiled(c, prm->lcartes, prm->msorit, prm->dk, prm->sortol, prm->sorrel, us, vs, p, o, &dl)))
          return rc;
      } else {
        int blocks = (prm->npsolver == 1 || prm->npsolver == 2)
                         ? 1 : pick_blocks(c, (const void *)k_ppe, (long)c->nx * c->ny);
        int lc = prm->lcartes, ns = prm->npsolver, ms = prm->msorit;
        double dk = prm->dk, st = prm->sortol, sr = prm->sorrel;
        void *args[] = {&dl, &lc, &ns, &ms, &dk, &st, &sr, &us, &vs, &p, &o};
        if ((rc = coop(c, (const void *)k_ppe, blocks, args))) return rc;
      }
    }
    {
      ProfScope ps(c, W2_K_POST);
      int blocks = pick_blocks(c, (const void *)k_me_post, (long)c->nx * c->ny);
      double dk = prm->dk;
      void *args[] = {&dl, &dk, &p, &us, &vs};
      if ((rc = coop(c, (const void *)k_me_post, blocks, args))) return rc;
    }
    if (therm) {
      ProfScope ps(c, W2_K_THERM);
      Chain ch = c->therm_ch;  // segments of the current chain view
      ch.L = d.seg;
      ch.nseg = (ch.n + d.seg - 1) / d.seg;
      ThermArgs A{c->therm_tt, prm->dk, tp.pe, un, vn, us, vs, tn, ts, d.cj1x, d.cj2x, d.c1sx, d.c2sx, ch};
      int blocks = pick_blocks(c, (const void *)k_therm, (long)c->nx * c->ny, naux_smem(c));
      void *args[] = {&dl, &A};
      if ((rc = coop(c, (const void *)k_therm, blocks, args, naux_smem(c)))) return rc;
    }
    if (eqs) {
      ProfScope ps(c, W2_K_THERM);
      c->launches++;
      k_eq_state<<<gb, c->threads, 0, c->st>>>(dl, tp.uref, tp.densref, tp.tmax, tp.tref, tp.rconst, p, ts,
                                               c->Dd);
      CK(cudaGetLastError());
    }
    if (l >= 2 && l < nme) {
      ProfScope ps(c, W2_K_POST);
      int blocks = pick_blocks(c, (const void *)k_me_norms, (long)c->nx * c->ny);
      int ll = l;
      double tol = tp.dmeittol;
      const double *up = c->Up, *vp = c->Vp, *tpv = c->Tp;
      void *args[] = {&dl, &ll, &tol, (void *)&up, (void *)&vp, (void *)&tpv, &us, &vs, &ts};
      if ((rc = coop(c, (const void *)k_me_norms, blocks, args))) return rc;
    }
  }
  if (therm && tp.nfiltt == 1) {
    // main.f:889-893: Filter of t after the iterations
    ProfScope ps(c, W2_K_THERM);
    c->launches++;
    k_filter_t<<<gb, c->threads, 0, c->st>>>(d, c->therm_tt, tp.fpt, ts, d.qh);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ts, d.qh, c->nf * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
  }
  {
    ProfScope ps(c, W2_K_POST);
    int blocks = pick_blocks(c, (const void *)k_step_tail_th, (long)c->nx * c->ny);
    ThermTables tt = c->therm_tt;
    int th = therm ? 1 : 0;
    void *args[] = {&d, &tt, &th, &p, (void *)&pn, (void *)&un, (void *)&vn, &us, &vs, &tn, &ts, &o};
    if ((rc = coop(c, (const void *)k_step_tail_th, blocks, args))) return rc;
  }
  return rc;
}

int issue_steps(w2_ctx *c, const w2_params *prm, int nsteps, StepOut *d_outs) {
  int rc = W2_OK;
  const int gb = grid_blocks(c);
  for (int s = 0; s < nsteps && rc == W2_OK; ++s) {
    const int a = c->cur, b = 1 - a;
    double *un = c->U[a], *vn = c->V[a], *pn = c->P[a];
    double *us = c->U[b], *vs = c->V[b], *p = c->P[b];
    StepOut *o = d_outs + s;
    Dev d = c->dev;
    const bool mixed = prm->precision == W2_PREC_MIXED;
    if (c->therm_on) {
      if ((rc = issue_thermal_step(c, prm, un, vn, pn, us, vs, p, o))) break;
      c->cur = b;
      continue;
    }
    if (mixed) {
      float *un32 = c->F32[0], *vn32 = c->F32[1], *us32 = c->F32[2], *vs32 = c->F32[3];
      {
        ProfScope ps(c, W2_K_COPY);
        c->launches++;
        k_copy_mixed<<<gb, c->threads, 0, c->st>>>(d, p, pn, un, vn, un32, vn32, us32, vs32);
        CK(cudaGetLastError());
      }
      // porous regions: the instance with the porous terms compiled in
      const void *kn = c->porous ? (const void *)k_naux32_por : (const void *)k_naux32;
      int blocks = pick_blocks(c, kn, (long)c->nx * c->ny, naux_smem(c));
      ProfScope ps(c, W2_K_MOMENTUM);
      int mq = prm->mqiter;
      double dk = prm->dk, re = prm->re, qtol = prm->qtol;
      void *args[] = {&d, &mq, &dk, &re, &qtol, &un32, &vn32, &us32, &vs32, &us, &vs, &o};
      if ((rc = coop(c, kn, blocks, args, naux_smem(c)))) break;
    } else {
      ProfScope ps(c, W2_K_COPY);
      c->launches++;
      k_copy3<<<gb, c->threads, 0, c->st>>>(d, us, un, vs, vn, p, pn);
      CK(cudaGetLastError());
    }
    // nAuxMomentum on (un, vn) -> (us, vs); us = un already (main.f:741-747)
    if (!mixed) {
      int blocks = pick_blocks(c, (const void *)k_naux, (long)c->nx * c->ny, naux_smem(c));
      ProfScope ps(c, W2_K_MOMENTUM);
      int mq = prm->mqiter;
      double dk = prm->dk, re = prm->re, qtol = prm->qtol;
      void *args[] = {&d, &mq, &dk, &re, &qtol, &un, &vn, &us, &vs, &o};
      if ((rc = coop(c, (const void *)k_naux, blocks, args, naux_smem(c)))) break;
    }
    if (prm->nfiltu == 1 || prm->nfiltv == 1) {
      double *h = c->stage[5];
      if (prm->nfiltu == 1) {
        k_filter<<<gb, c->threads, 0, c->st>>>(d, MK_FU, prm->fpu, us, h);
        CK(cudaMemcpyAsync(us, h, c->nf * 8, cudaMemcpyDeviceToDevice, c->st));
        c->launches++;
      }
      if (prm->nfiltv == 1) {
        k_filter<<<gb, c->threads, 0, c->st>>>(d, MK_FV, prm->fpv, vs, h);
        CK(cudaMemcpyAsync(vs, h, c->nf * 8, cudaMemcpyDeviceToDevice, c->st));
        c->launches++;
      }
    }
    if ((rc = launch_bc(c, BC_VEL | BC_PRES, us, vs, p))) break;
    if (prm->precision == W2_PREC_MIXED) {
      ProfScope ps(c, W2_K_PPE);
      if ((rc = launch_ppe_mixed(c, prm->lcartes, prm->msorit, prm->dk, prm->sortol, prm->sorrel,
                                 prm->refine_sweeps, us, vs, p, o)))
        break;
    } else if (tiled_applies(c, prm->npsolver, prm->sorrel)) {
      ProfScope ps(c, W2_K_PPE);
      if ((rc = launch_ppe_tiled(c, prm->lcartes, prm->msorit, prm->dk, prm->sortol, prm->sorrel, us, vs, p, o))) break;
    } else {
      int blocks = (prm->npsolver == 1 || prm->npsolver == 2)
                       ? 1 : pick_blocks(c, (const void *)k_ppe, (long)c->nx * c->ny);
      ProfScope ps(c, W2_K_PPE);
      int lc = prm->lcartes, ns = prm->npsolver, ms = prm->msorit;
      double dk = prm->dk, st = prm->sortol, sr = prm->sorrel;
      void *args[] = {&d, &lc, &ns, &ms, &dk, &st, &sr, &us, &vs, &p, &o};
      if ((rc = coop(c, (const void *)k_ppe, blocks, args))) break;
    }
    {
      int blocks = pick_blocks(c, (const void *)k_step_post, (long)c->nx * c->ny);
      ProfScope ps(c, W2_K_POST);
      double dk = prm->dk;
      void *args[] = {&d, &dk, &p, &pn, &un, &vn, &us, &vs, &o};
      if ((rc = coop(c, (const void *)k_step_post, blocks, args))) break;
    }
    c->cur = b;
  }
  return rc;
}

// Cache key of a captured step sequence: the bytes of everything its
// launches bake in.
std::string graph_key(const w2_ctx *c, const w2_params *prm, int nsteps) {
  std::string k;
  auto add = [&](const void *p, size_t n) { k.append((const char *)p, n); };
  const int head[] = {c->cur, nsteps, c->threads, c->blocks_per_sm, c->mixed_K, c->mixed_blocks,
                      c->tiled_blocks, c->tiled_threads, c->use_tiled, (int)c->tiled_ok, (int)c->mixed_ok,
                      c->use_mixgt, (int)c->mgt_ok, c->mgt_blocks};
  add(head, sizeof(head));
  add(prm, sizeof(*prm));
  add(&c->dev, sizeof(c->dev));
  add(&c->mg, sizeof(c->mg));
  add(&c->mgt, sizeof(c->mgt));
  add(&c->tg, sizeof(c->tg));
  const size_t sm[] = {c->mixed_smem, c->tiled_smem};
  add(sm, sizeof(sm));
  add(&c->therm_on, sizeof(c->therm_on));
  if (c->therm_on) {
    add(&c->therm_p, sizeof(c->therm_p));
    add(&c->therm_tt, sizeof(c->therm_tt));
    add(&c->therm_ch, sizeof(c->therm_ch));
    const double *bufs[] = {c->T[0], c->T[1], c->Dd, c->Ddn, c->Up, c->Vp, c->Tp};
    add(bufs, sizeof(bufs));
  }
  return k;
}

}  // namespace

extern "C" {

int wolfd2gpu_set_graph(w2_ctx *c, int enable) {
  if (!c) return W2_E_ARG;
  c->graph_on = enable != 0;
  return W2_OK;
}

int wolfd2gpu_step(w2_ctx *c, const w2_params *prm, int nsteps, w2_stepstat *stats) {
  NvtxRange nv("wolfd2gpu_step");
  int rc = ready(c);
  if (rc) return rc;
  if ((rc = check_params(c, prm))) return rc;
  if (nsteps < 0) return fail(c, W2_E_ARG, "nsteps < 0");
  if (c->therm_on && (prm->precision != W2_PREC_FP64 || prm->nfiltu == 1 || prm->nfiltv == 1))
    return fail(c, W2_E_UNSUPPORTED, "the time loop with the energy equation runs plain FP64 without Filter");
  if (prm->precision == W2_PREC_MIXED && (rc = ensure_f32(c))) return rc;
  // the general-row Poisson planes are made before any launch is captured
  if (prm->precision == W2_PREC_MIXED && mixed_general(c, prm->lcartes) && (rc = ensure_mixg(c))) return rc;
  // one step writes the other level; two or more write both
  if (nsteps >= 2) snap_fence(c);
  else if (nsteps == 1) snap_fence(c, 1 - c->cur);
  std::vector<StepOut> outs((size_t)std::max(nsteps, 1));
  if (nsteps > c->outs_cap) {
    if (c->d_outs) {
      CK(cudaStreamSynchronize(c->st));
      cudaFree(c->d_outs);
      c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void *)c->d_outs), c->allocs.end());
      for (auto &g : c->graphs) cudaGraphExecDestroy(g.second.exec);
      c->graphs.clear();
    }
    if (!(c->d_outs = dalloc<StepOut>(c, nsteps))) return fail(c, W2_E_CUDA, "out of device memory (step records)");
    c->outs_cap = nsteps;
  }
  StepOut *d_outs = c->d_outs;
  if (nsteps > 0 && c->graph_on && !c->prof_on) {
    const int cur0 = c->cur;
    const std::string key = graph_key(c, prm, nsteps);
    const w2_ctx::Graph *hit = nullptr;
    for (auto &g : c->graphs)
      if (g.first == key) hit = &g.second;
    if (!hit) {
      if (c->graphs.size() >= 8) {
        for (auto &g : c->graphs) cudaGraphExecDestroy(g.second.exec);
        c->graphs.clear();
      }
      const long long l0 = c->launches;
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      rc = issue_steps(c, prm, nsteps, d_outs);
      cudaError_t ce = cudaStreamEndCapture(c->st, &g);
      c->cur = cur0;
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (ce != cudaSuccess) return fail(c, W2_E_CUDA, "graph capture: %s", cudaGetErrorString(ce));
      cudaGraphExec_t exec = nullptr;
      ce = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return fail(c, W2_E_CUDA, "graph instantiation: %s", cudaGetErrorString(ce));
      c->graphs.push_back({key, {exec, c->launches - l0}});
      c->launches = l0;
      hit = &c->graphs.back().second;
    }
    CK(cudaGraphLaunch(hit->exec, c->st));
    c->launches += hit->launches;
    c->cur = (cur0 + nsteps) & 1;
  } else {
    rc = issue_steps(c, prm, nsteps, d_outs);
  }
  if (nsteps > 0)
    cudaMemcpyAsync(outs.data(), d_outs, sizeof(StepOut) * nsteps, cudaMemcpyDeviceToHost, c->st);
  int rs = check_sync(c);
  if (rc == W2_OK) rc = rs;
  int diverged_at = -1;
  for (int s = 0; s < nsteps; ++s) {
    double mx = std::max(std::max(std::max(outs[s].dif[0], outs[s].dif[1]), outs[s].dif[2]), outs[s].dif[3]);
    if (stats) {
      stats[s].nQLiter = outs[s].nql;
      stats[s].nSorConv = outs[s].nsor;
      for (int k = 0; k < 4; ++k) stats[s].dif[k] = outs[s].dif[k];
      stats[s].divmax = outs[s].divmax;
      stats[s].divmax_int = outs[s].divmax_int;
    }
    if (diverged_at < 0 && mx > 1.0e12) diverged_at = s;
  }
  if (rc == W2_OK && diverged_at >= 0) {
    // clear the halt flag so the context can be reloaded
    Sync z;
    memset(&z, 0, sizeof(z));
    cudaMemcpy(c->dev.sync, &z, sizeof(Sync), cudaMemcpyHostToDevice);
    return fail(c, W2_E_DIVERGED, "Solution diverged at step %d. Please reduce CFL number.", diverged_at + 1);
  }
  return rc;
}

}  // extern "C"

// ============================================================================
// Ensembles: many independent cases advanced together, one launch per stage
// of the mixed or plain time step (kernels in w2_ensemble.cuh).
// ============================================================================

struct w2_ens {
  std::vector<w2_ctx *> cs;
  int n = 0, K = 4, threads = 256, device = 0, nsm = 0;
  cudaStream_t st = nullptr;
  std::vector<void *> allocs;
  std::vector<EnsCase> h;
  EnsCase *d_cases = nullptr;
  CUtensorMap *d_tm = nullptr;  // 3 TMA maps per case (multi-tile Poisson boxes)
  int *d_first_m = nullptr, *d_first_p = nullptr, *d_first_1 = nullptr, *d_step = nullptr;
  std::vector<int> bm, bp;  // blocks per case: momentum/tail launches, Poisson launch
  int blocks_m = 0, blocks_p = 0;
  size_t smem_m = 0, smem_p = 0;
  StepOut *d_outs = nullptr;
  size_t outs_cap = 0;
  bool mixed_ok = false;    // every case has a mixed Poisson plan
  const char *mixed_why = "";  // why not, when not
  bool graph_on = false;
  cudaGraphExec_t gexec = nullptr;
  int graph_nsteps = -1, graph_prec = -1, graph_filter = -1;
  bool porous = false;     // some case has porous regions (momentum with the porous terms)
  long long launches = 0;
  double last_ms = 0.0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // per-stage event timing of direct (not graph) launches
  bool prof_on = false;
  struct Rec { int kind; cudaEvent_t a, b; };
  std::vector<Rec> prof_pending;
  std::vector<cudaEvent_t> ev_pool;
  double prof_ms[W2_ENS_NSTAGES] = {};
  long long prof_n[W2_ENS_NSTAGES] = {};
  char err[512] = {0};
};

namespace {

int efail(w2_ens *e, int code, const char *fmt, ...) {
  if (e) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(e->err, sizeof(e->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

#define ECK(call)                                                                  \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return efail(e, W2_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));  \
  } while (0)

template <class T>
T *ealloc(w2_ens *e, size_t n) {
  void *p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T));
  e->allocs.push_back(p);
  return (T *)p;
}

// Blocks per case: every case at least one block, the largest work per
// block as small as the total allows (bisection on that ratio), leftover
// blocks to the cases with the most work per block.  Empty if n > total.
std::vector<int> ens_partition(const std::vector<double> &w, int total) {
  const int n = (int)w.size();
  if (n == 0 || n > total) return {};
  auto blocks_for = [&](double r, std::vector<int> *b) {
    long sum = 0;
    for (int k = 0; k < n; ++k) {
      const long q = std::max(1L, (long)std::ceil(w[k] / r));
      if (b) (*b)[k] = (int)q;
      sum += q;
    }
    return sum;
  };
  double lo = 0.0, hi = *std::max_element(w.begin(), w.end()) + 1.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (blocks_for(mid, nullptr) <= total) hi = mid;
    else lo = mid;
  }
  std::vector<int> b(n, 1);
  long sum = blocks_for(hi, &b);
  while (sum < total) {
    int km = 0;
    for (int k = 1; k < n; ++k)
      if (w[k] / b[k] > w[km] / b[km]) km = k;
    ++b[km];
    ++sum;
  }
  return b;
}

// Multi-tile plan of one case's Poisson sweeps on `blocks` blocks of at most
// `tmax` threads and `smax` bytes of dynamic shared memory.
bool ens_plan(const w2_ctx *c, int K, int blocks, int tmax, size_t smax, MixedGeom *mg, size_t *smem) {
  const int NX = c->nx - 1, NY = c->ny - 1, H = 2 * K;
  double best = 1e300;
  for (int ntx = 1; ntx <= std::max(1, NX / 8); ++ntx) {
    int tx = (NX + ntx - 1) / ntx;
    tx = (tx + 7) / 8 * 8;
    if ((NX + tx - 1) / tx != ntx) continue;
    for (int nty = 1; nty <= std::max(1, NY / 4); ++nty) {
      const int ty = (NY + nty - 1) / nty;
      if ((NY + ty - 1) / ty != nty) continue;
      const size_t sm = mixed_smem_bytes(K, tx, ty, false);
      if (sm > smax || mixed_threads(K, tx, ty) > tmax) continue;
      const int tpb = (ntx * nty + blocks - 1) / blocks;
      const double cost = tpb * (mixed_sweep_work(K, tx, ty) + mixed_stage_work(K, tx, ty));
      if (cost < best) {
        best = cost;
        *mg = MixedGeom{tx, ty, ntx, nty, ntx * tx / 2 + H, nty * ty + 2 * H, mixed_lanes(K, tx), 0};
        *smem = sm;
      }
    }
  }
  return best < 1e300;
}

const void *ens_ppe_kernel(int K) {
  switch (K) {
    case 4: return (const void *)ke_ppe_mixed<4>;
    case 8: return (const void *)ke_ppe_mixed<8>;
  }
  return nullptr;
}

cudaEvent_t ens_event(w2_ens *e) {
  if (!e->ev_pool.empty()) {
    cudaEvent_t v = e->ev_pool.back();
    e->ev_pool.pop_back();
    return v;
  }
  cudaEvent_t v = nullptr;
  cudaEventCreate(&v);
  return v;
}

// Events around one stage launch when profiling (never inside a capture).
struct EnsProf {
  w2_ens *e;
  int kind;
  cudaEvent_t a = nullptr;
  EnsProf(w2_ens *e_, int k, bool capturing) : e(e_), kind(k) {
    if (e->prof_on && !capturing) {
      a = ens_event(e);
      cudaEventRecord(a, e->st);
    }
  }
  ~EnsProf() {
    if (!a) return;
    cudaEvent_t b = ens_event(e);
    cudaEventRecord(b, e->st);
    e->prof_pending.push_back({kind, a, b});
  }
};

void ens_prof_collect(w2_ens *e) {
  for (auto &r : e->prof_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      e->prof_ms[r.kind] += ms;
      e->prof_n[r.kind] += 1;
    }
    e->ev_pool.push_back(r.a);
    e->ev_pool.push_back(r.b);
  }
  e->prof_pending.clear();
}

// One step's launches: mixed (Lp: the Poisson partition) or plain FP64
// (every stage on the momentum partition Lm).
int ens_launch_step(w2_ens *e, bool mixed, bool filt, const EnsLaunch &Lm, const EnsLaunch &Lp,
                    const EnsLaunch &L1, bool capturing = false) {
  EnsLaunch am = Lm, ap = Lp;
  void *argm[] = {&am}, *argp[] = {&ap};
  // Filter of us, vs in the cases that ask for it, after nAuxMomentum
  auto filter = [&]() -> int {
    if (!filt) return W2_OK;
    ke_filter<<<e->blocks_m, e->threads, 0, e->st>>>(Lm, 0);
    ke_filter<<<e->blocks_m, e->threads, 0, e->st>>>(Lm, 1);
    ECK(cudaGetLastError());
    if (!capturing) e->launches += 2;
    return W2_OK;
  };
  if (!mixed) {
    {
      EnsProf pr(e, W2_ENS_COPY, capturing);
      ke_copy3<<<e->blocks_m, e->threads, 0, e->st>>>(Lm);
      ECK(cudaGetLastError());
    }
    {
      EnsProf pr(e, W2_ENS_MOMENTUM, capturing);
      ECK(cudaLaunchCooperativeKernel((const void *)ke_naux, dim3(e->blocks_m), dim3(e->threads), argm,
                                      e->smem_m, e->st));
    }
    if (int rc = filter()) return rc;
    {
      EnsProf pr(e, W2_ENS_BC, capturing);
      ke_bc<<<e->n, e->threads, 0, e->st>>>(L1);
      ECK(cudaGetLastError());
    }
    {
      EnsProf pr(e, W2_ENS_PPE, capturing);
      ECK(cudaLaunchCooperativeKernel((const void *)ke_ppe, dim3(e->blocks_m), dim3(e->threads), argm, 0,
                                      e->st));
    }
  } else {
    {
      EnsProf pr(e, W2_ENS_COPY, capturing);
      ke_copy_mixed<<<e->blocks_m, e->threads, 0, e->st>>>(Lm);
      ECK(cudaGetLastError());
    }
    {
      EnsProf pr(e, W2_ENS_MOMENTUM, capturing);
      ECK(cudaLaunchCooperativeKernel(e->porous ? (const void *)ke_naux32_por : (const void *)ke_naux32,
                                      dim3(e->blocks_m), dim3(e->threads), argm,
                                      e->smem_m, e->st));
    }
    if (int rc = filter()) return rc;
    {
      EnsProf pr(e, W2_ENS_BC, capturing);
      ke_bc<<<e->n, e->threads, 0, e->st>>>(L1);
      ECK(cudaGetLastError());
    }
    {
      EnsProf pr(e, W2_ENS_PPE, capturing);
      ECK(cudaLaunchCooperativeKernel(ens_ppe_kernel(e->K), dim3(e->blocks_p), dim3(e->threads), argp,
                                      e->smem_p, e->st));
    }
  }
  {
    EnsProf pr(e, W2_ENS_POST, capturing);
    ECK(cudaLaunchCooperativeKernel((const void *)ke_step_post, dim3(e->blocks_m), dim3(e->threads), argm,
                                    0, e->st));
  }
  ke_tick<<<1, 1, 0, e->st>>>(e->d_step);
  ECK(cudaGetLastError());
  e->launches += 6;
  return W2_OK;
}

}  // namespace

extern "C" {

int wolfd2gpu_ens_create(w2_ens **out, w2_ctx *const *cases, int n, int threads, int sweeps_per_barrier) {
  if (!out || !cases || n < 1) return W2_E_ARG;
  *out = nullptr;
  w2_ens *e = new w2_ens();
  auto bad = [&](int rc) {
    if (rc != W2_OK) fprintf(stderr, "wolfd2gpu_ens_create: %s\n", e->err);
    wolfd2gpu_ens_destroy(e);
    return rc;
  };
  // 128-thread blocks: four per SM, so the ragged partition has 4 x SMs
  // groups to size (with at least one per case, coarser blocks leave the
  // largest cases with too few)
  if (threads == 0) threads = 128;
  if (sweeps_per_barrier == 0) sweeps_per_barrier = 4;
  if (threads % 32 || threads < 64 || threads > kMaxThreads)
    return bad(efail(e, W2_E_ARG, "threads must be a multiple of 32 in 64..%d", kMaxThreads));
  if (!ens_ppe_kernel(sweeps_per_barrier)) return bad(efail(e, W2_E_ARG, "sweeps per barrier must be 4 or 8"));
  e->n = n;
  e->threads = threads;
  e->K = sweeps_per_barrier;
  e->cs.assign(cases, cases + n);
  // cases whose Poisson rows round to the unit stencil in FP32 take the
  // multi-tile unit kernel in the mixed step, the others the general-row one
  for (int k = 0; k < n; ++k) {
    w2_ctx *c = e->cs[k];
    if (!c) return bad(efail(e, W2_E_ARG, "case %d is null", k));
    if (int rc = ready(c)) return bad(efail(e, rc, "case %d: %s", k, c->err));
    if (c->porous) e->porous = true;
    if (c->therm_on)
      return bad(efail(e, W2_E_UNSUPPORTED, "case %d: ensembles do not run the energy equation", k));
    if (k == 0) e->device = c->device;
    else if (c->device != e->device) return bad(efail(e, W2_E_ARG, "cases on different devices"));
  }
  for (int k = 0; k < n; ++k) {
    w2_ctx *c = e->cs[k];
    if (int rc = ensure_f32(c)) return bad(efail(e, rc, "case %d: %s", k, c->err));
    if (!c->dev.ppe_unit32)
      if (int rc = ensure_mixg(c)) return bad(efail(e, rc, "case %d: %s", k, c->err));
    if (cudaStreamSynchronize(c->st) != cudaSuccess) return bad(efail(e, W2_E_CUDA, "case %d: set-up failed", k));
  }
  if (cudaSetDevice(e->device) != cudaSuccess) return bad(efail(e, W2_E_CUDA, "cudaSetDevice"));
  cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, e->device);
  // blocking, like the contexts' streams (ordered after legacy-stream set-up work)
  if (cudaStreamCreate(&e->st) != cudaSuccess ||
      cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess)
    return bad(efail(e, W2_E_CUDA, "stream or event creation failed"));
  std::vector<double> work(n);
  for (int k = 0; k < n; ++k) work[k] = (double)(e->cs[k]->nx - 1) * (e->cs[k]->ny - 1);

  // momentum and step-tail launches (and the plain Poisson launch): blocks
  // by the co-residency of all of them
  e->smem_m = walk_stage_bytes(sizeof(double), threads);
  int occ = 1 << 20;
  for (const void *kf : {(const void *)ke_naux32, (const void *)ke_naux32_por, (const void *)ke_naux}) {
    if (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smem_m) != cudaSuccess)
      return bad(efail(e, W2_E_CUDA, "shared memory attribute (momentum)"));
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kf, threads, e->smem_m);
    occ = std::min(occ, o);
  }
  for (const void *kf : {(const void *)ke_step_post, (const void *)ke_ppe}) {
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kf, threads, 0);
    occ = std::min(occ, o);
  }
  e->blocks_m = occ * e->nsm;
  e->bm = ens_partition(work, e->blocks_m);
  if (e->bm.empty())
    return bad(efail(e, W2_E_UNSUPPORTED, "%d cases need more blocks than the %d that fit", n, e->blocks_m));

  // mixed Poisson launch: as many blocks per SM (up to four) as registers
  // and shared memory allow, each with that share of an SM's shared memory
  const void *kp = ens_ppe_kernel(e->K);
  e->h.resize(n);
  int smem_sm = 0, smem_optin = 0;
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, e->device);
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device);
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kp) != cudaSuccess) return bad(efail(e, W2_E_CUDA, "kernel attributes"));
  for (int per_sm = 4; per_sm >= 1; --per_sm) {
    const size_t smax = std::min<size_t>((size_t)smem_optin, (size_t)smem_sm / per_sm - 1024) - fa.sharedSizeBytes;
    const int total = per_sm * e->nsm;
    std::vector<int> bp = ens_partition(work, total);
    if (bp.empty()) continue;
    std::vector<MixedGeom> g(n);
    size_t smem = 0;
    bool ok = true;
    for (int k = 0; k < n && ok; ++k) {
      if (!e->cs[k]->dev.ppe_unit32) continue;  // general rows: no tiles, no dynamic shared memory
      size_t sk = 0;
      ok = ens_plan(e->cs[k], e->K, bp[k], threads, smax, &g[k], &sk);
      smem = std::max(smem, sk);
    }
    if (!ok) continue;
    if (cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      continue;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kp, threads, smem);
    if (occ < per_sm) continue;
    e->bp = bp;
    e->blocks_p = total;
    e->smem_p = smem;
    for (int k = 0; k < n; ++k) e->h[k].g = g[k];
    break;
  }
  e->mixed_ok = !e->bp.empty();
  if (!e->mixed_ok)
    e->mixed_why = "no Poisson tile plan fits every case in blocks of this many threads and sweeps per barrier";
  if (!e->mixed_ok) {
    // plain steps only: the Poisson table is unused
    e->bp = e->bm;
    e->blocks_p = e->blocks_m;
  }

  // per-case buffers and the parts of the descriptors that do not change
  for (int k = 0; k < n; ++k) {
    w2_ctx *c = e->cs[k];
    EnsCase &h = e->h[k];
    const MixedGeom &g = h.g;
    const size_t plane2 = 2 * (size_t)g.gh * g.gw;
    h.general = c->dev.ppe_unit32 ? 0 : 1;
    float *xb = nullptr;
    if (e->mixed_ok && !h.general && !(xb = ealloc<float>(e, 3 * plane2)))
      return bad(efail(e, W2_E_CUDA, "out of device memory (case %d Poisson buffers)", k));
    const CUtensorMap *tm = nullptr;
    if (e->mixed_ok && !h.general && c->use_tma) {
      if (!e->d_tm && !(e->d_tm = ealloc<CUtensorMap>(e, 3 * (size_t)n)))
        return bad(efail(e, W2_E_CUDA, "out of device memory (tensor maps)"));
      if (encode_mixed_maps(e->d_tm + 3 * k, xb, g, e->K, c->st)) tm = e->d_tm + 3 * k;
    }
    h.d = c->dev;
    chain_views(h.d, c->nx, c->ny, (long)e->bm[k] * threads, c->seg_req, c->warm_req);
    for (int b = 0; b < 2; ++b) {
      h.U[b] = c->U[b];
      h.V[b] = c->V[b];
      h.P[b] = c->P[b];
      h.a[b] = MixedArgs{};
      h.a[b].u = c->U[b];
      h.a[b].v = c->V[b];
      h.a[b].p = c->P[b];
      h.a[b].xbuf0 = xb;
      h.a[b].xbuf1 = xb + plane2;
      h.a[b].rbuf = xb + 2 * plane2;
      h.a[b].tm = tm;
      h.ga[b] = h.general ? mixg_args(c, 1, 0, 1.0, 0.0, 1.0, 1, c->U[b], c->V[b], c->P[b]) : MixgArgs{};
    }
    for (int q = 0; q < 4; ++q) h.F32[q] = c->F32[q];
  }
  std::vector<int> fm(n + 1, 0), fp(n + 1, 0), f1(n + 1, 0);
  for (int k = 0; k < n; ++k) {
    fm[k + 1] = fm[k] + e->bm[k];
    fp[k + 1] = fp[k] + e->bp[k];
    f1[k + 1] = k + 1;
  }
  e->d_cases = ealloc<EnsCase>(e, n);
  e->d_first_m = ealloc<int>(e, n + 1);
  e->d_first_p = ealloc<int>(e, n + 1);
  e->d_first_1 = ealloc<int>(e, n + 1);
  e->d_step = ealloc<int>(e, 1);
  if (!e->d_cases || !e->d_first_m || !e->d_first_p || !e->d_first_1 || !e->d_step)
    return bad(efail(e, W2_E_CUDA, "out of device memory (ensemble tables)"));
  if (cudaMemcpy(e->d_first_m, fm.data(), fm.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->d_first_p, fp.data(), fp.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->d_first_1, f1.data(), f1.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return bad(efail(e, W2_E_CUDA, "table upload"));
  if (cudaDeviceSynchronize() != cudaSuccess) return bad(efail(e, W2_E_CUDA, "set-up failed"));
  *out = e;
  return W2_OK;
}

int wolfd2gpu_ens_graph(w2_ens *e, int enable) {
  if (!e) return W2_E_ARG;
  e->graph_on = enable != 0;
  return W2_OK;
}

int wolfd2gpu_ens_step(w2_ens *e, const w2_params *prm, int nsteps, w2_stepstat *stats) {
  NvtxRange nv("wolfd2gpu_ens_step");
  if (!e || !prm || nsteps < 0) return W2_E_ARG;
  const int n = e->n;
  const bool mixed = prm[0].precision == W2_PREC_MIXED;
  for (int k = 0; k < n; ++k) {
    const w2_params &q = prm[k];
    if (q.precision != W2_PREC_MIXED && q.precision != W2_PREC_FP64)
      return efail(e, W2_E_ARG, "case %d: bad precision %d", k, q.precision);
    if ((q.precision == W2_PREC_MIXED) != mixed)
      return efail(e, W2_E_UNSUPPORTED, "case %d: every case of one call runs in the same precision", k);
    if (mixed && !e->mixed_ok) return efail(e, W2_E_UNSUPPORTED, "%s", e->mixed_why);
    if (mixed && q.npsolver != 5 && q.npsolver != 6)
      return efail(e, W2_E_UNSUPPORTED, "case %d: the mixed step needs rb_sor or rb_sorp", k);
    if (mixed && !q.lcartes && !e->h[k].general)
      return efail(e, W2_E_UNSUPPORTED,
                   "case %d: in an ensemble the mixed step takes lCartesGrid = 0 only on grids whose rows are not "
                   "the unit stencil", k);
    if (q.npsolver < 1 || q.npsolver > 6) return efail(e, W2_E_ARG, "case %d: bad Poisson solver %d", k, q.npsolver);
    if (q.msorit < 1 || q.mqiter < 1 || q.refine_sweeps < 0) return efail(e, W2_E_ARG, "case %d: bad parameters", k);
  }
  if (nsteps == 0) return W2_OK;
  // a snapshot copy of a case must finish before the ensemble's stream writes its fields
  for (int k = 0; k < n; ++k) {
    w2_ctx *c = e->cs[k];
    if (c->snap_level >= 0) {
      ECK(cudaStreamWaitEvent(e->st, c->ev_snap_done, 0));
      c->snap_level = -1;
    }
  }
  // descriptors of this call: parameters, starting levels
  bool filt = false;
  for (int k = 0; k < n; ++k) {
    const w2_params &q = prm[k];
    EnsCase &h = e->h[k];
    h.cur = e->cs[k]->cur;
    h.mqiter = q.mqiter;
    h.dk = q.dk;
    h.re = q.re;
    h.qtol = q.qtol;
    h.npsolver = q.npsolver;
    h.lcartes = q.lcartes;
    h.msorit = q.msorit;
    h.sortol = q.sortol;
    h.sorrel = q.sorrel;
    h.nfiltu = q.nfiltu == 1;
    h.nfiltv = q.nfiltv == 1;
    h.fpu = q.fpu;
    h.fpv = q.fpv;
    h.hu = e->cs[k]->stage[4];
    h.hv = e->cs[k]->stage[5];
    filt = filt || h.nfiltu || h.nfiltv;
    for (int b = 0; b < 2; ++b) {
      MixedArgs &a = h.a[b];
      a.lcartes = q.lcartes;
      a.msorit = q.msorit;
      a.inner = q.refine_sweeps > 0 ? q.refine_sweeps : 16 * e->K;
      a.dk = q.dk;
      a.sortol = q.sortol;
      a.relax = (float)q.sorrel;
      MixgArgs &ga = h.ga[b];
      ga.lcartes = q.lcartes;
      ga.msorit = q.msorit;
      ga.inner = a.inner;
      ga.dk = q.dk;
      ga.sortol = q.sortol;
      ga.relax = (float)q.sorrel;
    }
  }
  ECK(cudaMemcpyAsync(e->d_cases, e->h.data(), sizeof(EnsCase) * n, cudaMemcpyHostToDevice, e->st));
  const size_t need = (size_t)n * nsteps;
  if (need > e->outs_cap) {
    if (e->d_outs) {
      cudaFree(e->d_outs);
      e->allocs.erase(std::remove(e->allocs.begin(), e->allocs.end(), (void *)e->d_outs), e->allocs.end());
    }
    e->d_outs = ealloc<StepOut>(e, need);
    if (!e->d_outs) return efail(e, W2_E_CUDA, "out of device memory (step records)");
    e->outs_cap = need;
    e->graph_nsteps = -1;
  }
  ECK(cudaMemsetAsync(e->d_step, 0, sizeof(int), e->st));
  const EnsLaunch Lm{e->d_cases, e->d_first_m, n, e->d_step, e->d_outs, nsteps};
  const EnsLaunch Lp{e->d_cases, e->d_first_p, n, e->d_step, e->d_outs, nsteps};
  const EnsLaunch L1{e->d_cases, e->d_first_1, n, e->d_step, e->d_outs, nsteps};
  const int prec = mixed ? W2_PREC_MIXED : W2_PREC_FP64;
  if (e->graph_on && (e->graph_nsteps != nsteps || e->graph_prec != prec || e->graph_filter != (int)filt)) {
    if (e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
    cudaGraph_t g = nullptr;
    ECK(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
    const long long l0 = e->launches;
    int rc = ens_launch_step(e, mixed, filt, Lm, Lp, L1, true);
    e->launches = l0;
    cudaError_t ce = cudaStreamEndCapture(e->st, &g);
    if (rc) return rc;
    if (ce != cudaSuccess) return efail(e, W2_E_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&e->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return efail(e, W2_E_CUDA, "graph instantiation: %s", cudaGetErrorString(ce));
    e->graph_nsteps = nsteps;
    e->graph_prec = prec;
    e->graph_filter = (int)filt;
  }
  ECK(cudaEventRecord(e->ev0, e->st));
  for (int s = 0; s < nsteps; ++s) {
    if (e->graph_on) {
      ECK(cudaGraphLaunch(e->gexec, e->st));
      e->launches += filt ? 8 : 6;
    } else if (int rc = ens_launch_step(e, mixed, filt, Lm, Lp, L1)) {
      return rc;
    }
  }
  ECK(cudaEventRecord(e->ev1, e->st));
  std::vector<StepOut> outs(need);
  ECK(cudaMemcpyAsync(outs.data(), e->d_outs, sizeof(StepOut) * need, cudaMemcpyDeviceToHost, e->st));
  ECK(cudaStreamSynchronize(e->st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e->ev0, e->ev1);
  e->last_ms = ms;
  ens_prof_collect(e);
  int rc = W2_OK, diverged = -1;
  for (int k = 0; k < n; ++k) {
    w2_ctx *c = e->cs[k];
    Sync sy;
    ECK(cudaMemcpy(&sy, c->dev.sync, sizeof(Sync), cudaMemcpyDeviceToHost));
    if (sy.error || sy.halt) {
      Sync z;
      memset(&z, 0, sizeof(z));
      ECK(cudaMemcpy(c->dev.sync, &z, sizeof(Sync), cudaMemcpyHostToDevice));
      if (sy.error && rc == W2_OK)
        rc = efail(e, sy.error, "case %d: device error %d%s", k, sy.error,
                   sy.error == W2_E_TIMEOUT ? " (device wait exceeded its time limit)" : "");
    }
    c->cur = (c->cur + nsteps) & 1;
    for (int s = 0; s < nsteps; ++s) {
      const StepOut &o = outs[(size_t)k * nsteps + s];
      if (stats) {
        w2_stepstat &t = stats[(size_t)k * nsteps + s];
        t.nQLiter = o.nql;
        t.nSorConv = o.nsor;
        for (int q = 0; q < 4; ++q) t.dif[q] = o.dif[q];
        t.divmax = o.divmax;
        t.divmax_int = o.divmax_int;
      }
      const double mx = std::max(std::max(o.dif[0], o.dif[1]), o.dif[2]);
      if (diverged < 0 && mx > 1.0e12) diverged = k;
    }
  }
  if (rc == W2_OK && diverged >= 0)
    return efail(e, W2_E_DIVERGED, "case %d diverged. Please reduce CFL number.", diverged);
  return rc;
}

int wolfd2gpu_ens_info(w2_ens *e, int *blocks_momentum, int *blocks_poisson, double *last_ms,
                       long long *launches) {
  if (!e) return W2_E_ARG;
  if (blocks_momentum) *blocks_momentum = e->blocks_m;
  if (blocks_poisson) *blocks_poisson = e->blocks_p;
  if (last_ms) *last_ms = e->last_ms;
  if (launches) *launches = e->launches;
  return W2_OK;
}

int wolfd2gpu_ens_profile(w2_ens *e, int enable) {
  if (!e) return W2_E_ARG;
  e->prof_on = enable != 0;
  for (int k = 0; k < W2_ENS_NSTAGES; ++k) {
    e->prof_ms[k] = 0.0;
    e->prof_n[k] = 0;
  }
  return W2_OK;
}

int wolfd2gpu_ens_profile_read(w2_ens *e, int stage, double *total_ms, long long *count) {
  if (!e || stage < 0 || stage >= W2_ENS_NSTAGES) return W2_E_ARG;
  if (total_ms) *total_ms = e->prof_ms[stage];
  if (count) *count = e->prof_n[stage];
  return W2_OK;
}

const char *wolfd2gpu_ens_error(w2_ens *e) { return e ? e->err : "null ensemble"; }

int wolfd2gpu_ens_destroy(w2_ens *e) {
  if (!e) return W2_OK;
  if (e->st) cudaStreamSynchronize(e->st);
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  for (void *p : e->allocs) cudaFree(p);
  for (auto &r : e->prof_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t v : e->ev_pool) cudaEventDestroy(v);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
  return W2_OK;
}

}  // extern "C"

// ============================================================================
// Adjoint of the plain FP64 step (kernels in w2_adjoint.cuh)
// ============================================================================

namespace {

// A boundary program as a list of assignments (see AdjBCList).
struct BCProg {
  std::vector<int> stage{0}, tgt, src, nsrc, prof;
  std::vector<double> coef, pcoef;
  size_t nf = 0;
  int ld = 0;
  int code(int f, int i, int j) const { return (int)((size_t)f * nf + (size_t)i + (size_t)j * ld); }
  void op(int t, std::initializer_list<std::pair<int, double>> srcs, int pf = -1, double pc = 0.0) {
    tgt.push_back(t);
    int q = 0;
    for (auto &sc : srcs) {
      src.push_back(sc.first);
      coef.push_back(sc.second);
      ++q;
    }
    for (; q < kAdjSrc; ++q) {
      src.push_back(0);
      coef.push_back(0.0);
    }
    nsrc.push_back((int)srcs.size());
    prof.push_back(pf);
    pcoef.push_back(pc);
  }
  void end_stage() {
    if ((int)tgt.size() > stage.back()) stage.push_back((int)tgt.size());
  }
};

enum { FU = 0, FV = 1, FP = 2 };

// Index into the face-value table of (region, face, var) at pos, or -1.
int prof_slot(const w2_ctx *c, int ir, int jr, int face, int var, int pos) {
  if (c->prof_host.empty()) return -1;
  const int key = ((ir - 1) + (jr - 1) * c->mgri + (face - 1) * c->mgri * c->mgrj) * 2 + (var - 1);
  const int off = c->prof_host[key];
  return off < 0 ? -1 : off + pos;
}

// VelBoundCond (bound_cond.f:511-847) replayed as assignments, in the order
// of w2_bc.cuh vel_bound_cond_block.
void emit_vel_bc(const w2_ctx *c, BCProg &g) {
  const int mgri = c->mgri, mgrj = c->mgrj;
  auto B = [&](int ir, int jr, int s) { return c->tab_brd[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto BT = [&](int ir, int jr, int s) { return c->tab_btype[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto U = [&](int i, int j) { return g.code(FU, i, j); };
  auto V = [&](int i, int j) { return g.code(FV, i, j); };
  for (int jr = 1; jr <= c->nrj; ++jr)
    for (int ir = 1; ir <= c->nri; ++ir) {
      const int iW = B(ir, jr, 1), iE = B(ir, jr, 2), jS = B(ir, jr, 3), jN = B(ir, jr, 4);
      switch (BT(ir, jr, 1)) {
        case W2_BM_WALL1:
          for (int j = jS; j <= jN; ++j) g.op(U(iW, j), {});
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iW, j), {{V(iW + 1, j), -1.0}}, prof_slot(c, ir, jr, 1, 2, j), 2.0);
          g.end_stage();
          break;
        case W2_BM_WALL2:
          for (int j = jS; j <= jN; ++j) g.op(U(iW, j), {});
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iW, j), {{V(iW + 1, j), 1.0}});
          g.end_stage();
          break;
        case W2_BM_INLET:
          for (int j = jS; j <= jN; ++j) g.op(U(iW, j), {}, prof_slot(c, ir, jr, 1, 1, j), 1.0);
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iW, j), {{V(iW + 1, j), -1.0}}, prof_slot(c, ir, jr, 1, 2, j), 2.0);
          g.end_stage();
          break;
        case W2_BM_OUTLT1:
          for (int j = jS; j <= jN; ++j) g.op(U(iW - 1, j), {{U(iW, j), 1.0}});
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iW, j), {{V(iW + 1, j), -1.0}});
          g.end_stage();
          break;
        case W2_BM_OUTLT2:
          for (int j = jS + 1; j <= jN; ++j)
            g.op(U(iW, j), {{U(iW + 1, j), 1.0}, {V(iW + 1, j), 1.0}, {V(iW + 1, j - 1), -1.0}});
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) {
            g.op(V(iW, j), {{V(iW, j - 1), -1.0}, {V(iW + 1, j), 5.0}, {V(iW + 1, j - 1), -5.0},
                            {U(iW + 1, j), 8.0}, {U(iW, j), -8.0}});
            g.end_stage();
          }
          break;
        default: break;
      }
      switch (BT(ir, jr, 2)) {
        case W2_BM_WALL1:
          for (int j = jS; j <= jN; ++j) g.op(U(iE, j), {});
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iE + 1, j), {{V(iE, j), -1.0}}, prof_slot(c, ir, jr, 2, 2, j), 2.0);
          g.end_stage();
          break;
        case W2_BM_WALL2:
          for (int j = jS; j <= jN; ++j) g.op(U(iE, j), {});
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iE + 1, j), {{V(iE, j), 1.0}});
          g.end_stage();
          break;
        case W2_BM_INLET:
          for (int j = jS; j <= jN; ++j) g.op(U(iE, j), {}, prof_slot(c, ir, jr, 2, 1, j), 1.0);
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iE + 1, j), {{V(iE, j), -1.0}}, prof_slot(c, ir, jr, 2, 2, j), 2.0);
          g.end_stage();
          break;
        case W2_BM_OUTLT1:
          for (int j = jS; j <= jN; ++j) g.op(U(iE + 1, j), {{U(iE, j), 1.0}});
          g.end_stage();
          for (int j = jS + 1; j <= jN; ++j) g.op(V(iE + 1, j), {{V(iE, j), -1.0}});
          g.end_stage();
          break;
        case W2_BM_OUTLT2:
          for (int j = jS + 1; j <= jN; ++j)
            g.op(U(iE, j), {{U(iE - 1, j), 1.0}, {V(iE, j), -1.0}, {V(iE, j - 1), 1.0}});
          g.end_stage();
          for (int j = jS + 1; j <= jN - 1; ++j) {
            g.op(V(iE + 1, j), {{V(iE + 1, j - 1), 1.0}, {V(iE, j - 1), 3.0}, {V(iE, j), -3.0},
                                {U(iE, j), -4.0}, {U(iE - 1, j), 4.0}});
            g.end_stage();
          }
          break;
        default: break;
      }
      switch (BT(ir, jr, 3)) {
        case W2_BM_WALL1:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jS), {{U(i, jS + 1), -1.0}}, prof_slot(c, ir, jr, 3, 1, i), 2.0);
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jS), {});
          g.end_stage();
          break;
        case W2_BM_WALL2:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jS), {{U(i, jS + 1), 1.0}});
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jS), {});
          g.end_stage();
          break;
        case W2_BM_INLET:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jS), {{U(i, jS + 1), -1.0}}, prof_slot(c, ir, jr, 3, 1, i), 2.0);
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jS), {}, prof_slot(c, ir, jr, 3, 2, i), 1.0);
          g.end_stage();
          break;
        case W2_BM_OUTLT1:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jS), {{U(i, jS + 1), -1.0}});
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jS), {{V(i, jS), 1.0}});
          g.end_stage();
          break;
        case W2_BM_OUTLT2:
          for (int i = iW + 1; i <= iE; ++i)
            g.op(V(i, jS), {{V(i, jS + 1), 1.0}, {U(i, jS + 1), 1.0}, {U(i - 1, jS + 1), -1.0}});
          g.end_stage();
          for (int i = iW + 1; i <= iE - 1; ++i) {
            g.op(U(i, jS), {{U(i - 1, jS), 1.0}, {U(i - 1, jS + 1), 3.0}, {U(i, jS + 1), -3.0},
                            {V(i, jS + 1), -4.0}, {V(i, jS), 4.0}});
            g.end_stage();
          }
          break;
        default: break;
      }
      switch (BT(ir, jr, 4)) {
        case W2_BM_WALL1:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jN + 1), {{U(i, jN), -1.0}}, prof_slot(c, ir, jr, 4, 1, i), 2.0);
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jN), {});
          g.end_stage();
          break;
        case W2_BM_WALL2:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jN + 1), {{U(i, jN), 1.0}});
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jN), {});
          g.end_stage();
          break;
        case W2_BM_INLET:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jN + 1), {{U(i, jN), -1.0}}, prof_slot(c, ir, jr, 4, 1, i), 2.0);
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jN), {}, prof_slot(c, ir, jr, 4, 2, i), 1.0);
          g.end_stage();
          break;
        case W2_BM_OUTLT1:
          for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jN + 1), {{U(i, jN), -1.0}});
          g.end_stage();
          for (int i = iW; i <= iE; ++i) g.op(V(i, jN + 1), {{V(i, jN), 1.0}});
          g.end_stage();
          break;
        case W2_BM_OUTLT2:
          for (int i = iW; i <= iE; ++i)
            g.op(V(i, jN), {{V(i, jN - 1), 1.0}, {U(i, jN), -1.0}, {U(i - 1, jN), 1.0}});
          g.end_stage();
          for (int i = iW + 1; i <= iE - 1; ++i) {
            g.op(U(i, jN + 1), {{U(i - 1, jN + 1), 1.0}, {U(i - 1, jN), 3.0}, {U(i, jN), -3.0},
                                {V(i, jN), -4.0}, {V(i, jN - 1), 4.0}});
            g.end_stage();
          }
          break;
        default: break;
      }
    }
}

// VelOutflowBCs (bound_cond.f:1656-1874), in the order of
// vel_outflow_bcs_block: outlet faces only.
void emit_outflow_bc(const w2_ctx *c, BCProg &g) {
  const int mgri = c->mgri, mgrj = c->mgrj;
  auto B = [&](int ir, int jr, int s) { return c->tab_brd[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto BT = [&](int ir, int jr, int s) { return c->tab_btype[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto U = [&](int i, int j) { return g.code(FU, i, j); };
  auto V = [&](int i, int j) { return g.code(FV, i, j); };
  for (int jr = 1; jr <= c->nrj; ++jr)
    for (int ir = 1; ir <= c->nri; ++ir) {
      const int iW = B(ir, jr, 1), iE = B(ir, jr, 2), jS = B(ir, jr, 3), jN = B(ir, jr, 4);
      int t = BT(ir, jr, 1);
      if (t == W2_BM_OUTLT1) {
        for (int j = jS; j <= jN; ++j) g.op(U(iW - 1, j), {{U(iW, j), 1.0}});
        g.end_stage();
        for (int j = jS + 1; j <= jN; ++j) g.op(V(iW, j), {{V(iW + 1, j), -1.0}});
        g.end_stage();
      } else if (t == W2_BM_OUTLT2) {
        for (int j = jS + 1; j <= jN; ++j)
          g.op(U(iW, j), {{U(iW + 1, j), 1.0}, {V(iW + 1, j), -1.0}, {V(iW + 1, j - 1), 1.0}});
        g.end_stage();
        for (int j = jS + 1; j <= jN; ++j) {
          g.op(V(iW, j), {{V(iW, j - 1), -1.0}, {V(iW + 1, j), 5.0}, {V(iW + 1, j - 1), -5.0},
                          {U(iW + 1, j), 8.0}, {U(iW, j), -8.0}});
          g.end_stage();
        }
      }
      t = BT(ir, jr, 2);
      if (t == W2_BM_OUTLT1) {
        for (int j = jS; j <= jN; ++j) g.op(U(iE + 1, j), {{U(iE, j), 1.0}});
        g.end_stage();
        for (int j = jS + 1; j <= jN; ++j) g.op(V(iE + 1, j), {{V(iE, j), -1.0}});
        g.end_stage();
      } else if (t == W2_BM_OUTLT2) {
        for (int j = jS + 1; j <= jN; ++j)
          g.op(U(iE, j), {{U(iE - 1, j), 1.0}, {V(iE, j), -1.0}, {V(iE, j - 1), 1.0}});
        g.end_stage();
        for (int j = jS + 1; j <= jN - 1; ++j) {
          g.op(V(iE + 1, j), {{V(iE + 1, j - 1), 1.0}, {V(iE, j - 1), 3.0}, {V(iE, j), -3.0},
                              {U(iE, j), -4.0}, {U(iE - 1, j), 4.0}});
          g.end_stage();
        }
      }
      t = BT(ir, jr, 3);
      if (t == W2_BM_OUTLT1) {
        for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jS), {{U(i, jS + 1), -1.0}});
        g.end_stage();
        for (int i = iW; i <= iE; ++i) g.op(V(i, jS), {{V(i, jS), 1.0}});
        g.end_stage();
      } else if (t == W2_BM_OUTLT2) {
        for (int i = iW + 1; i <= iE; ++i)
          g.op(V(i, jS), {{V(i, jS + 1), 1.0}, {U(i, jS + 1), 1.0}, {U(i - 1, jS + 1), -1.0}});
        g.end_stage();
        for (int i = iW + 1; i <= iE - 1; ++i) {
          g.op(U(i, jS), {{U(i - 1, jS), 1.0}, {U(i - 1, jS + 1), 3.0}, {U(i, jS + 1), -3.0},
                          {V(i, jS + 1), -4.0}, {V(i, jS), 4.0}});
          g.end_stage();
        }
      }
      t = BT(ir, jr, 4);
      if (t == W2_BM_OUTLT1) {
        for (int i = iW + 1; i <= iE; ++i) g.op(U(i, jN + 1), {{U(i, jN), -1.0}});
        g.end_stage();
        for (int i = iW; i <= iE; ++i) g.op(V(i, jN + 1), {{V(i, jN), 1.0}});
        g.end_stage();
      } else if (t == W2_BM_OUTLT2) {
        for (int i = iW; i <= iE; ++i)
          g.op(V(i, jN), {{V(i, jN - 1), 1.0}, {U(i, jN), -1.0}, {U(i - 1, jN), 1.0}});
        g.end_stage();
        for (int i = iW + 1; i <= iE - 1; ++i) {
          g.op(U(i, jN + 1), {{U(i - 1, jN + 1), 1.0}, {U(i - 1, jN), 3.0}, {U(i, jN), -3.0},
                              {V(i, jN), -4.0}, {V(i, jN - 1), 4.0}});
          g.end_stage();
        }
      }
    }
}

// PresBoundCond (bound_cond.f:853-1024), in the order of pres_bound_cond_block.
void emit_pres_bc(const w2_ctx *c, BCProg &g) {
  const int mgri = c->mgri, mgrj = c->mgrj;
  auto B = [&](int ir, int jr, int s) { return c->tab_brd[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto RT = [&](int ir, int jr) { return c->tab_rtype[(ir - 1) + (jr - 1) * mgri]; };
  auto BT = [&](int ir, int jr, int s) { return c->tab_btype[(ir - 1) + (jr - 1) * mgri + (s - 1) * mgri * mgrj]; };
  auto P = [&](int i, int j) { return g.code(FP, i, j); };
  auto wall = [](int t) { return t == W2_BM_WALL1 || t == W2_BM_WALL2 || t == W2_BM_INLET; };
  auto outl = [](int t) { return t == W2_BM_OUTLT1 || t == W2_BM_OUTLT2; };
  for (int jr = 1; jr <= c->nrj; ++jr)
    for (int ir = 1; ir <= c->nri; ++ir) {
      const int iW = B(ir, jr, 1), iE = B(ir, jr, 2), jS = B(ir, jr, 3), jN = B(ir, jr, 4);
      if (RT(ir, jr) == W2_RM_BLOCKG) {
        for (int j = jS + 1; j <= jN; ++j)
          for (int i = iW + 1; i <= iE; ++i) g.op(P(i, j), {});
        g.end_stage();
        for (int j = jS + 1; j <= jN; ++j) g.op(P(iW + 1, j), {{P(iW, j), 1.0}});
        g.end_stage();
        for (int j = jS + 1; j <= jN; ++j) g.op(P(iE, j), {{P(iE + 1, j), 1.0}});
        g.end_stage();
        for (int i = iW + 1; i <= iE; ++i) g.op(P(i, jS + 1), {{P(i, jS), 1.0}});
        g.end_stage();
        for (int i = iW + 1; i <= iE; ++i) g.op(P(i, jN), {{P(i, jN + 1), 1.0}});
        g.end_stage();
        continue;
      }
      int t = BT(ir, jr, 1);
      if (wall(t) || outl(t)) {
        for (int j = jS + 1; j <= jN; ++j) g.op(P(iW, j), {{P(iW + 1, j), wall(t) ? 1.0 : -1.0}});
        g.end_stage();
      }
      t = BT(ir, jr, 2);
      if (wall(t) || outl(t)) {
        for (int j = jS + 1; j <= jN; ++j) g.op(P(iE + 1, j), {{P(iE, j), wall(t) ? 1.0 : -1.0}});
        g.end_stage();
      }
      t = BT(ir, jr, 3);
      if (wall(t) || outl(t)) {
        for (int i = iW + 1; i <= iE; ++i) g.op(P(i, jS), {{P(i, jS + 1), wall(t) ? 1.0 : -1.0}});
        g.end_stage();
      }
      t = BT(ir, jr, 4);
      if (wall(t) || outl(t)) {
        for (int i = iW + 1; i <= iE; ++i) g.op(P(i, jN + 1), {{P(i, jN), wall(t) ? 1.0 : -1.0}});
        g.end_stage();
      }
    }
}

// A BCProg on the device for k_adj_bc; buffers recorded in `mem`.
int upload_bc(w2_ctx *c, const BCProg &g, AdjBCList &L, std::vector<void *> &mem) {
  auto up = [&](const void *h, size_t bytes) -> void * {
    void *p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 8)) != cudaSuccess) return nullptr;
    mem.push_back(p);
    if (h && bytes && cudaMemcpy(p, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return p;
  };
  const size_t n = g.tgt.size();
  L.nstages = (int)g.stage.size() - 1;
  L.nf = g.nf;
  L.stage = (const int *)up(g.stage.data(), g.stage.size() * sizeof(int));
  L.tgt = (const int *)up(g.tgt.data(), n * sizeof(int));
  L.src = (const int *)up(g.src.data(), g.src.size() * sizeof(int));
  L.nsrc = (const int *)up(g.nsrc.data(), n * sizeof(int));
  L.prof = (const int *)up(g.prof.data(), n * sizeof(int));
  L.coef = (const double *)up(g.coef.data(), g.coef.size() * sizeof(double));
  L.pcoef = (const double *)up(g.pcoef.data(), n * sizeof(double));
  L.tmp = (double *)up(nullptr, n * sizeof(double));
  if (!L.stage || !L.tgt || !L.src || !L.nsrc || !L.prof || !L.coef || !L.pcoef || !L.tmp)
    return fail(c, W2_E_CUDA, "out of device memory (boundary adjoint)");
  return W2_OK;
}

// Parameters of step s with its counts frozen: exactly m Q-L iterations and
// n sweeps (no convergence test can stop them earlier).
w2_params frozen(const w2_params *prm, int m, int n) {
  w2_params q = *prm;
  q.mqiter = m;
  q.qtol = -1.0;
  q.msorit = n;
  q.sortol = -1.0;
  return q;
}

int adj_check(w2_ctx *c, const w2_params *prm) {
  int rc = ready(c);
  if (rc) return rc;
  if ((rc = check_params(c, prm))) return rc;
  if (prm->precision != W2_PREC_FP64) return fail(c, W2_E_UNSUPPORTED, "the adjoint runs the plain FP64 step");
  if (prm->npsolver != 5 || !prm->lcartes)
    return fail(c, W2_E_UNSUPPORTED, "the adjoint supports ppe_solver rb_sor (5) on Cartesian grids");
  if (prm->nfiltu == 1 || prm->nfiltv == 1) return fail(c, W2_E_UNSUPPORTED, "the adjoint does not cover Filter");
  if (c->therm_on) return fail(c, W2_E_UNSUPPORTED, "the adjoint does not cover the energy equation");
  if (c->porous) return fail(c, W2_E_UNSUPPORTED, "the adjoint does not cover porous regions");
  return W2_OK;
}

int adj_alloc(w2_ctx *c) {
  if (c->adj_alloc) return W2_OK;
  const int nX = c->nx * (c->ny - 1), nY = (c->nx - 1) * c->ny;
  int rc;
  if ((rc = make_chain(c, c->adj_tx, nX, true)) || (rc = make_chain(c, c->adj_ty, nY, true))) return rc;
  for (int k = 0; k < 8; ++k)
    if (!(c->adj_rows[k] = dalloc<double>(c, (size_t)(k < 4 ? nX : nY) + kMaxSeg)))
      return fail(c, W2_E_CUDA, "out of device memory (adjoint rows)");
  const int wmax = (int)walk_stage_bytes(sizeof(double), kMaxThreads);
  if (cudaFuncSetAttribute((const void *)k_adj_iter, cudaFuncAttributeMaxDynamicSharedMemorySize, wmax) !=
      cudaSuccess)
    return fail(c, W2_E_CUDA, "shared memory attribute (adjoint)");
  c->adj_alloc = true;
  return W2_OK;
}

}  // namespace

extern "C" {

int wolfd2gpu_step_counts(w2_ctx *c, const w2_params *prm, int nsteps, const int *counts, w2_stepstat *stats) {
  int rc = ready(c);
  if (rc) return rc;
  if ((rc = check_params(c, prm))) return rc;
  if (nsteps < 0 || (nsteps > 0 && !counts)) return fail(c, W2_E_ARG, "counts: 2 per step");
  const bool g = c->graph_on;
  c->graph_on = false;
  for (int s = 0; s < nsteps && rc == W2_OK; ++s) {
    const w2_params q = frozen(prm, counts[2 * s], counts[2 * s + 1]);
    w2_stepstat st;
    rc = wolfd2gpu_step(c, &q, 1, &st);
    if (stats) stats[s] = st;
  }
  c->graph_on = g;
  return rc;
}

int wolfd2gpu_adjoint(w2_ctx *c, const w2_params *prm, int nsteps, int every, double weight, double *J,
                      double *gu, double *gv, double *gp, int ireg, int jreg, int face, int var,
                      double *gprof, int nprof, int *counts) {
  NvtxRange nv("wolfd2gpu_adjoint");
  int rc = adj_check(c, prm);
  if (rc) return rc;
  if (nsteps < 1 || every < 1) return fail(c, W2_E_ARG, "nsteps and checkpoint interval must be >= 1");
  if ((rc = adj_alloc(c))) return rc;
  snap_fence(c);
  std::vector<void *> mem;
  struct Free {
    std::vector<void *> &m;
    ~Free() {
      for (void *p : m) cudaFree(p);
    }
  } free_mem{mem};
  auto field = [&]() -> double * {
    void *p = nullptr;
    if (cudaMalloc(&p, c->nf * sizeof(double)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, c->nf * sizeof(double));
    mem.push_back(p);
    return (double *)p;
  };
  const size_t fb = c->nf * sizeof(double);
  const int nck = (nsteps + every - 1) / every, mq = prm->mqiter;
  std::vector<double *> ck(3 * nck), seg(3 * every), tape(2 * (mq + 1));
  double *lu = field(), *lv = field(), *lp = field(), *lb = field(), *lun = field(), *lvn = field();
  double *fin[3] = {field(), field(), field()};
  for (auto &x : ck) x = field();
  for (auto &x : seg) x = field();
  for (auto &x : tape) x = field();
  double *dJ = nullptr, *lprof = nullptr;
  const size_t nprof_all = c->prof_host.empty() ? 1 : (size_t)16 * c->prof_len;
  if (cudaMalloc(&dJ, sizeof(double)) != cudaSuccess) return fail(c, W2_E_CUDA, "out of device memory");
  mem.push_back(dJ);
  if (cudaMalloc(&lprof, nprof_all * sizeof(double)) != cudaSuccess) return fail(c, W2_E_CUDA, "out of device memory");
  mem.push_back(lprof);
  for (double *x : {lu, lv, lp, lb, lun, lvn, fin[0], fin[1], fin[2]})
    if (!x) return fail(c, W2_E_CUDA, "out of device memory (adjoint fields)");
  for (auto *v : {&ck, &seg, &tape})
    for (double *x : *v)
      if (!x) return fail(c, W2_E_CUDA, "out of device memory (adjoint checkpoints)");
  // boundary programs as assignment lists
  BCProg gv_, gp_, go_;
  gv_.nf = gp_.nf = go_.nf = c->nf;
  gv_.ld = gp_.ld = go_.ld = c->ld;
  emit_vel_bc(c, gv_);
  emit_pres_bc(c, gp_);
  emit_outflow_bc(c, go_);
  AdjBCList Lv{}, Lp{}, Lo{};
  if ((rc = upload_bc(c, gv_, Lv, mem)) || (rc = upload_bc(c, gp_, Lp, mem)) || (rc = upload_bc(c, go_, Lo, mem)))
    return rc;
  const bool outflow = c->dev.has_outflow != 0;
  double *wu = field(), *wv = field();
  if (!wu || !wv) return fail(c, W2_E_CUDA, "out of device memory (adjoint fields)");
  CK(cudaDeviceSynchronize());
  const bool graph0 = c->graph_on;
  c->graph_on = false;
  struct Restore {
    w2_ctx *c;
    bool g;
    ~Restore() { c->graph_on = g; }
  } restore{c, graph0};
  StepOut so;
  std::vector<int> cnt(2 * nsteps);
  auto copy3 = [&](double *du, double *dv, double *dp, const double *su, const double *sv, const double *sp) -> int {
    CK(cudaMemcpyAsync(du, su, fb, cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(dv, sv, fb, cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(dp, sp, fb, cudaMemcpyDeviceToDevice, c->st));
    return W2_OK;
  };
  // ---- forward: checkpoints and the iteration counts of every step
  if (nsteps > c->outs_cap) {
    if (c->d_outs) {
      cudaFree(c->d_outs);
      c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void *)c->d_outs), c->allocs.end());
      for (auto &gr : c->graphs) cudaGraphExecDestroy(gr.second.exec);
      c->graphs.clear();
    }
    if (!(c->d_outs = dalloc<StepOut>(c, nsteps))) return fail(c, W2_E_CUDA, "out of device memory (step records)");
    c->outs_cap = nsteps;
  }
  for (int s = 0; s < nsteps; ++s) {
    if (s % every == 0) {
      const int k = s / every;
      if ((rc = copy3(ck[3 * k], ck[3 * k + 1], ck[3 * k + 2], c->U[c->cur], c->V[c->cur], c->P[c->cur]))) return rc;
    }
    if ((rc = issue_steps(c, prm, 1, c->d_outs))) return rc;
    CK(cudaMemcpyAsync(&so, c->d_outs, sizeof(StepOut), cudaMemcpyDeviceToHost, c->st));
    if ((rc = check_sync(c))) return rc;
    cnt[2 * s] = so.nql > 0 ? so.nql : prm->mqiter;
    cnt[2 * s + 1] = so.nsor;
    const double mx = std::max(std::max(so.dif[0], so.dif[1]), so.dif[2]);
    if (!(mx <= 1.0e12)) return fail(c, W2_E_DIVERGED, "forward run diverged at step %d", s + 1);
  }
  if ((rc = copy3(fin[0], fin[1], fin[2], c->U[c->cur], c->V[c->cur], c->P[c->cur]))) return rc;
  // ---- objective and its gradient at the final step
  Dev d = c->dev;
  const int gb = grid_blocks(c);
  CK(cudaMemsetAsync(dJ, 0, sizeof(double), c->st));
  CK(cudaMemsetAsync(lp, 0, fb, c->st));
  CK(cudaMemsetAsync(lprof, 0, nprof_all * sizeof(double), c->st));
  k_adj_objective<<<gb, c->threads, 0, c->st>>>(d, weight, fin[0], fin[1], lu, lv, dJ);
  CK(cudaGetLastError());
  // transposed SOR coefficients, fixed for the call
  AdjPpeCoef pq{field(), field(), field(), field(), field()};
  for (double *x : {pq.q1, pq.q2, pq.q3, pq.q4, pq.q5})
    if (!x) return fail(c, W2_E_CUDA, "out of device memory (adjoint fields)");
  c->launches += 2;
  k_adj_ppe_coef<<<gb, c->threads, 0, c->st>>>(d, prm->sorrel, pq);
  CK(cudaGetLastError());
  // ---- backward, segment by segment
  const int nX = c->nx * (c->ny - 1);
  (void)nX;
  Chain tx = c->adj_tx, ty = c->adj_ty;
  tx.L = ty.L = d.seg;
  tx.nseg = d.f64.x1.nseg;
  ty.nseg = d.f64.y1.nseg;
  const int bl_iter = pick_blocks(c, (const void *)k_adj_iter, (long)c->nx * c->ny, naux_smem(c));
  const int bl_ppe = pick_blocks(c, (const void *)k_adj_ppe, (long)c->nx * c->ny);
  const int bl_naux = pick_blocks(c, (const void *)k_naux, (long)c->nx * c->ny, naux_smem(c));
  double *lprof_arg = c->prof_host.empty() ? nullptr : lprof;
  auto adj_bc = [&](AdjBCList &L) -> int {
    c->launches++;
    k_adj_bc<<<1, 512, 0, c->st>>>(L, lu, lv, lp, lprof_arg);
    CK(cudaGetLastError());
    return W2_OK;
  };
  for (int k = nck - 1; k >= 0; --k) {
    const int s0 = k * every, s1 = std::min(nsteps, s0 + every);
    // recompute the segment's step inputs
    if ((rc = copy3(c->U[c->cur], c->V[c->cur], c->P[c->cur], ck[3 * k], ck[3 * k + 1], ck[3 * k + 2]))) return rc;
    for (int s = s0; s < s1; ++s) {
      const int q = s - s0;
      if ((rc = copy3(seg[3 * q], seg[3 * q + 1], seg[3 * q + 2], c->U[c->cur], c->V[c->cur], c->P[c->cur]))) return rc;
      if (s + 1 < s1) {
        const w2_params f = frozen(prm, cnt[2 * s], cnt[2 * s + 1]);
        if ((rc = issue_steps(c, &f, 1, c->d_outs))) return rc;
      }
    }
    for (int s = s1 - 1; s >= s0; --s) {
      const int q = s - s0, m = cnt[2 * s], ns = cnt[2 * s + 1];
      double *un = seg[3 * q], *vn = seg[3 * q + 1];
      double dk = prm->dk;
      // tail: PresBC, Project, VelBC, PresBC, VelBC, PresBC reversed
      if ((rc = adj_bc(Lp)) || (rc = adj_bc(Lv)) || (rc = adj_bc(Lp)) || (rc = adj_bc(Lv))) return rc;
      c->launches++;
      k_adj_project<<<gb, c->threads, 0, c->st>>>(d, dk, lu, lv, lp);
      CK(cudaGetLastError());
      if ((rc = adj_bc(Lp))) return rc;
      // Ppe (fixed sweep count) and Divergence
      {
        double sr = prm->sorrel;
        int nsv = ns;
        void *args[] = {&d, &nsv, &sr, &dk, &pq, &lp, &lb, &lu, &lv};
        if ((rc = coop(c, (const void *)k_adj_ppe, bl_ppe, args))) return rc;
      }
      // the boundary rows before Ppe: VelBC then PresBC, reversed
      if ((rc = adj_bc(Lp)) || (rc = adj_bc(Lv))) return rc;
      // Q-L iterations: tape the iterates, then transpose them in reverse
      CK(cudaMemcpyAsync(tape[0], un, fb, cudaMemcpyDeviceToDevice, c->st));
      CK(cudaMemcpyAsync(tape[1], vn, fb, cudaMemcpyDeviceToDevice, c->st));
      for (int it = 1; it <= m; ++it) {
        double *us = tape[2 * it], *vs = tape[2 * it + 1];
        CK(cudaMemcpyAsync(us, tape[2 * it - 2], fb, cudaMemcpyDeviceToDevice, c->st));
        CK(cudaMemcpyAsync(vs, tape[2 * it - 1], fb, cudaMemcpyDeviceToDevice, c->st));
        int one = 1;
        double re = prm->re, qt = -1.0;
        StepOut *o = c->d_out;
        void *args[] = {&d, &one, &dk, &re, &qt, &un, &vn, &us, &vs, &o};
        if ((rc = coop(c, (const void *)k_naux, bl_naux, args, naux_smem(c)))) return rc;
      }
      CK(cudaMemsetAsync(lun, 0, fb, c->st));
      CK(cudaMemsetAsync(lvn, 0, fb, c->st));
      for (int it = m; it >= 1; --it) {
        // the iteration starts by VelOutflowBCs on the iterate (outlets)
        const double *us_it = tape[2 * it - 2], *vs_it = tape[2 * it - 1];
        if (outflow) {
          CK(cudaMemcpyAsync(wu, us_it, fb, cudaMemcpyDeviceToDevice, c->st));
          CK(cudaMemcpyAsync(wv, vs_it, fb, cudaMemcpyDeviceToDevice, c->st));
          if ((rc = launch_bc(c, BC_OUTFLOW, wu, wv, c->P[c->cur]))) return rc;
          us_it = wu;
          vs_it = wv;
        }
        AdjIter A{};
        A.us = us_it;
        A.vs = vs_it;
        A.un = un;
        A.vn = vn;
        A.lus = lu;
        A.lvs = lv;
        A.lun = lun;
        A.lvn = lvn;
        A.sa1x = c->adj_rows[0]; A.sa2x = c->adj_rows[1]; A.sa3x = c->adj_rows[2]; A.sx1 = c->adj_rows[3];
        A.sa1y = c->adj_rows[4]; A.sa2y = c->adj_rows[5]; A.sa3y = c->adj_rows[6]; A.sy1 = c->adj_rows[7];
        A.tx = tx;
        A.ty = ty;
        A.dk = dk;
        A.re = prm->re;
        void *args[] = {&d, &A};
        if ((rc = coop(c, (const void *)k_adj_iter, bl_iter, args, naux_smem(c)))) return rc;
        if (outflow && (rc = adj_bc(Lo))) return rc;
      }
      // us = un, vs = vn at the start of the step: the level-n adjoint
      k_axpy2<<<gb, c->threads, 0, c->st>>>(d, lu, lun, lv, lvn);
      c->launches++;
      CK(cudaGetLastError());
    }
  }
  if ((rc = check_sync(c))) return rc;
  // outputs
  CK(cudaMemcpy(J, dJ, sizeof(double), cudaMemcpyDeviceToHost));
  if (gu && (rc = copy_out(c, gu, lu))) return rc;
  if (gv && (rc = copy_out(c, gv, lv))) return rc;
  if (gp && (rc = copy_out(c, gp, lp))) return rc;
  if (gprof && nprof > 0) {
    const int slot = prof_slot(c, ireg, jreg, face, var, 0);
    std::vector<double> h(nprof, 0.0);
    if (slot >= 0) {
      const int n = std::min(nprof, c->prof_len);
      CK(cudaMemcpy(h.data(), lprof + slot, n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    memcpy(gprof, h.data(), nprof * sizeof(double));
  }
  if (counts) memcpy(counts, cnt.data(), cnt.size() * sizeof(int));
  // leave the context at the final state of the run
  if ((rc = copy3(c->U[c->cur], c->V[c->cur], c->P[c->cur], fin[0], fin[1], fin[2]))) return rc;
  CK(cudaStreamSynchronize(c->st));
  return W2_OK;
}

}  // extern "C"
