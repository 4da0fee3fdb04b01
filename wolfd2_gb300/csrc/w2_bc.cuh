// w2_bc.cuh -- boundary-condition rows (bound_cond.f) executed by ONE block.
//
// The reference applies its boundary loops region by region and face by face,
// and later loops read values written by earlier ones (corner ghosts, the
// mass-conservation outlet recurrences).  These routines keep that order: each
// face loop is spread over the block's threads, a __syncthreads separates
// consecutive loops, and the loops that are recurrences (a value depends on
// the one written just before it in the same loop) run on one thread.
#pragma once
#include "w2_common.cuh"

namespace w2 {

enum { BM_INTERN = 0, BM_WALL1 = 1, BM_WALL2 = 2, BM_INLET = 3, BM_OUTLT1 = 4,
       BM_OUTLT2 = 5 };
enum { RM_BLOCKG = 0, RM_INTERN = 1, RM_POROUS = 2 };
enum { WEST = 1, EAST = 2, SOUTH = 3, NORTH = 4 };
enum { VAR_U = 1, VAR_V = 2, VAR_P = 3 };

#define W2_PFOR(var, lo, hi) for (int var = (lo) + (int)threadIdx.x; var <= (hi); var += (int)blockDim.x)
#define W2_SFOR(var, lo, hi) if (threadIdx.x == 0) for (int var = (lo); var <= (hi); ++var)
#define W2_SYNC() __syncthreads()

// Value of a face's boundary variable (VAR_U, VAR_V) at position pos along
// the face (j on west/east faces, i on south/north faces): the values set by
// wolfd2gpu_set_face_profile when there are any (an extension for inflow and
// lid profiles), else the region constant dBCVal.
__device__ __forceinline__ double bcv_at(const Dev &d, int ir, int jr, int face, int var, int pos) {
  if (d.prof_idx) {
    const int k = d.prof_idx[((ir - 1) + (jr - 1) * d.r.mgri + (face - 1) * d.r.mgri * d.r.mgrj) * 2 +
                             (var - 1)];
    if (k >= 0) return d.prof[k + pos];
  }
  return d.r.BV(ir, jr, face, var);
}

// VelBoundCond, bound_cond.f:511-847.  Returns false on an invalid flag.
__device__ bool vel_bound_cond_block(const Dev &d, double *u, double *v) {
  const Regions &r = d.r;
#define UF(i, j) u[IX(d, i, j)]
#define VF(i, j) v[IX(d, i, j)]
  for (int jreg = 1; jreg <= r.nrj; jreg++)
    for (int ireg = 1; ireg <= r.nri; ireg++) {
      const int iW = r.B(ireg, jreg, WEST), iE = r.B(ireg, jreg, EAST);
      const int jS = r.B(ireg, jreg, SOUTH), jN = r.B(ireg, jreg, NORTH);
      switch (r.BT(ireg, jreg, WEST)) {
        case BM_INTERN: break;
        case BM_WALL1: {
          W2_PFOR(j, jS, jN) UF(iW, j) = 0.0;
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iW, j) = 2.0 * bcv_at(d, ireg, jreg, WEST, VAR_V, j) - VF(iW + 1, j);
          W2_SYNC();
        } break;
        case BM_WALL2:
          W2_PFOR(j, jS, jN) UF(iW, j) = 0.0;
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iW, j) = VF(iW + 1, j);
          W2_SYNC();
          break;
        case BM_INLET: {
          W2_PFOR(j, jS, jN) UF(iW, j) = bcv_at(d, ireg, jreg, WEST, VAR_U, j);
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iW, j) = 2.0 * bcv_at(d, ireg, jreg, WEST, VAR_V, j) - VF(iW + 1, j);
          W2_SYNC();
        } break;
        case BM_OUTLT1: {
          const double uw = r.BV(ireg, jreg, WEST, VAR_U);
          W2_PFOR(j, jS, jN) UF(iW - 1, j) = uw + UF(iW, j);
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iW, j) = -VF(iW + 1, j);
          W2_SYNC();
        } break;
        case BM_OUTLT2:
          W2_PFOR(j, jS + 1, jN) UF(iW, j) = UF(iW + 1, j) + VF(iW + 1, j) - VF(iW + 1, j - 1);
          W2_SYNC();
          W2_SFOR(j, jS + 1, jN)
          VF(iW, j) = -VF(iW, j - 1) + 5.0 * (VF(iW + 1, j) - VF(iW + 1, j - 1)) +
                     8.0 * (UF(iW + 1, j) - UF(iW, j));
          W2_SYNC();
          break;
        default: return false;
      }
      switch (r.BT(ireg, jreg, EAST)) {
        case BM_INTERN: break;
        case BM_WALL1: {
          W2_PFOR(j, jS, jN) UF(iE, j) = 0.0;
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iE + 1, j) = 2.0 * bcv_at(d, ireg, jreg, EAST, VAR_V, j) - VF(iE, j);
          W2_SYNC();
        } break;
        case BM_WALL2:
          W2_PFOR(j, jS, jN) UF(iE, j) = 0.0;
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iE + 1, j) = VF(iE, j);
          W2_SYNC();
          break;
        case BM_INLET: {
          W2_PFOR(j, jS, jN) UF(iE, j) = bcv_at(d, ireg, jreg, EAST, VAR_U, j);
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iE + 1, j) = 2.0 * bcv_at(d, ireg, jreg, EAST, VAR_V, j) - VF(iE, j);
          W2_SYNC();
        } break;
        case BM_OUTLT1: {
          const double ue = r.BV(ireg, jreg, EAST, VAR_U);
          W2_PFOR(j, jS, jN) UF(iE + 1, j) = ue + UF(iE, j);
          W2_SYNC();
          W2_PFOR(j, jS + 1, jN) VF(iE + 1, j) = -VF(iE, j);
          W2_SYNC();
        } break;
        case BM_OUTLT2:
          W2_PFOR(j, jS + 1, jN) UF(iE, j) = UF(iE - 1, j) - (VF(iE, j) - VF(iE, j - 1));
          W2_SYNC();
          W2_SFOR(j, jS + 1, jN - 1)
          VF(iE + 1, j) = VF(iE + 1, j - 1) + 3.0 * (VF(iE, j - 1) - VF(iE, j)) -
                         4.0 * (UF(iE, j) - UF(iE - 1, j));
          W2_SYNC();
          break;
        default: return false;
      }
      switch (r.BT(ireg, jreg, SOUTH)) {
        case BM_INTERN: break;
        case BM_WALL1: {
          W2_PFOR(i, iW + 1, iE) UF(i, jS) = 2.0 * bcv_at(d, ireg, jreg, SOUTH, VAR_U, i) - UF(i, jS + 1);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jS) = 0.0;
          W2_SYNC();
        } break;
        case BM_WALL2:
          W2_PFOR(i, iW + 1, iE) UF(i, jS) = UF(i, jS + 1);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jS) = 0.0;
          W2_SYNC();
          break;
        case BM_INLET: {
          W2_PFOR(i, iW + 1, iE) UF(i, jS) = 2.0 * bcv_at(d, ireg, jreg, SOUTH, VAR_U, i) - UF(i, jS + 1);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jS) = bcv_at(d, ireg, jreg, SOUTH, VAR_V, i);
          W2_SYNC();
        } break;
        case BM_OUTLT1: {
          const double vs_ = r.BV(ireg, jreg, SOUTH, VAR_V);
          W2_PFOR(i, iW + 1, iE) UF(i, jS) = -UF(i, jS + 1);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jS) = vs_ + VF(i, jS);
          W2_SYNC();
        } break;
        case BM_OUTLT2:
          W2_PFOR(i, iW + 1, iE) VF(i, jS) = VF(i, jS + 1) + (UF(i, jS + 1) - UF(i - 1, jS + 1));
          W2_SYNC();
          W2_SFOR(i, iW + 1, iE - 1)
          UF(i, jS) = UF(i - 1, jS) + 3.0 * (UF(i - 1, jS + 1) - UF(i, jS + 1)) -
                     4.0 * (VF(i, jS + 1) - VF(i, jS));
          W2_SYNC();
          break;
        default: return false;
      }
      switch (r.BT(ireg, jreg, NORTH)) {
        case BM_INTERN: break;
        case BM_WALL1: {
          W2_PFOR(i, iW + 1, iE) UF(i, jN + 1) = 2.0 * bcv_at(d, ireg, jreg, NORTH, VAR_U, i) - UF(i, jN);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jN) = 0.0;
          W2_SYNC();
        } break;
        case BM_WALL2:
          W2_PFOR(i, iW + 1, iE) UF(i, jN + 1) = UF(i, jN);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jN) = 0.0;
          W2_SYNC();
          break;
        case BM_INLET: {
          W2_PFOR(i, iW + 1, iE) UF(i, jN + 1) = 2.0 * bcv_at(d, ireg, jreg, NORTH, VAR_U, i) - UF(i, jN);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jN) = bcv_at(d, ireg, jreg, NORTH, VAR_V, i);
          W2_SYNC();
        } break;
        case BM_OUTLT1: {
          const double vn_ = r.BV(ireg, jreg, NORTH, VAR_V);
          W2_PFOR(i, iW + 1, iE) UF(i, jN + 1) = -UF(i, jN);
          W2_SYNC();
          W2_PFOR(i, iW, iE) VF(i, jN + 1) = vn_ + VF(i, jN);
          W2_SYNC();
        } break;
        case BM_OUTLT2:
          W2_PFOR(i, iW, iE) VF(i, jN) = VF(i, jN - 1) - (UF(i, jN) - UF(i - 1, jN));
          W2_SYNC();
          W2_SFOR(i, iW + 1, iE - 1)
          UF(i, jN + 1) = UF(i - 1, jN + 1) + 3.0 * (UF(i - 1, jN) - UF(i, jN)) -
                         4.0 * (VF(i, jN) - VF(i, jN - 1));
          W2_SYNC();
          break;
        default: return false;
      }
    }
  return true;
}

// VelOutflowBCs, bound_cond.f:1656-1874 (outlet faces only; note the west
// mass-conservation u row has the opposite v signs to VelBoundCond's).
// T is double on the plain path and float on the mixed one.
template <class T>
__device__ bool vel_outflow_bcs_block(const Dev &d, T *u, T *v) {
  const Regions &r = d.r;
  for (int jreg = 1; jreg <= r.nrj; jreg++)
    for (int ireg = 1; ireg <= r.nri; ireg++) {
      const int iW = r.B(ireg, jreg, WEST), iE = r.B(ireg, jreg, EAST);
      const int jS = r.B(ireg, jreg, SOUTH), jN = r.B(ireg, jreg, NORTH);
      int t = r.BT(ireg, jreg, WEST);
      if (t == BM_OUTLT1) {
        const T uw = T(r.BV(ireg, jreg, WEST, VAR_U));
        W2_PFOR(j, jS, jN) UF(iW - 1, j) = uw + UF(iW, j);
        W2_SYNC();
        W2_PFOR(j, jS + 1, jN) VF(iW, j) = -VF(iW + 1, j);
        W2_SYNC();
      } else if (t == BM_OUTLT2) {
        W2_PFOR(j, jS + 1, jN) UF(iW, j) = UF(iW + 1, j) - VF(iW + 1, j) + VF(iW + 1, j - 1);
        W2_SYNC();
        W2_SFOR(j, jS + 1, jN)
        VF(iW, j) = -VF(iW, j - 1) + T(5.0) * (VF(iW + 1, j) - VF(iW + 1, j - 1)) +
                   T(8.0) * (UF(iW + 1, j) - UF(iW, j));
        W2_SYNC();
      } else if (t < BM_INTERN || t > BM_OUTLT2) {
        return false;
      }
      t = r.BT(ireg, jreg, EAST);
      if (t == BM_OUTLT1) {
        const T ue = T(r.BV(ireg, jreg, EAST, VAR_U));
        W2_PFOR(j, jS, jN) UF(iE + 1, j) = ue + UF(iE, j);
        W2_SYNC();
        W2_PFOR(j, jS + 1, jN) VF(iE + 1, j) = -VF(iE, j);
        W2_SYNC();
      } else if (t == BM_OUTLT2) {
        W2_PFOR(j, jS + 1, jN) UF(iE, j) = UF(iE - 1, j) - (VF(iE, j) - VF(iE, j - 1));
        W2_SYNC();
        W2_SFOR(j, jS + 1, jN - 1)
        VF(iE + 1, j) = VF(iE + 1, j - 1) + T(3.0) * (VF(iE, j - 1) - VF(iE, j)) -
                       T(4.0) * (UF(iE, j) - UF(iE - 1, j));
        W2_SYNC();
      } else if (t < BM_INTERN || t > BM_OUTLT2) {
        return false;
      }
      t = r.BT(ireg, jreg, SOUTH);
      if (t == BM_OUTLT1) {
        const T vs_ = T(r.BV(ireg, jreg, SOUTH, VAR_V));
        W2_PFOR(i, iW + 1, iE) UF(i, jS) = -UF(i, jS + 1);
        W2_SYNC();
        W2_PFOR(i, iW, iE) VF(i, jS) = vs_ + VF(i, jS);
        W2_SYNC();
      } else if (t == BM_OUTLT2) {
        W2_PFOR(i, iW + 1, iE) VF(i, jS) = VF(i, jS + 1) + (UF(i, jS + 1) - UF(i - 1, jS + 1));
        W2_SYNC();
        W2_SFOR(i, iW + 1, iE - 1)
        UF(i, jS) = UF(i - 1, jS) + T(3.0) * (UF(i - 1, jS + 1) - UF(i, jS + 1)) -
                   T(4.0) * (VF(i, jS + 1) - VF(i, jS));
        W2_SYNC();
      } else if (t < BM_INTERN || t > BM_OUTLT2) {
        return false;
      }
      t = r.BT(ireg, jreg, NORTH);
      if (t == BM_OUTLT1) {
        const T vn_ = T(r.BV(ireg, jreg, NORTH, VAR_V));
        W2_PFOR(i, iW + 1, iE) UF(i, jN + 1) = -UF(i, jN);
        W2_SYNC();
        W2_PFOR(i, iW, iE) VF(i, jN + 1) = vn_ + VF(i, jN);
        W2_SYNC();
      } else if (t == BM_OUTLT2) {
        W2_PFOR(i, iW, iE) VF(i, jN) = VF(i, jN - 1) - (UF(i, jN) - UF(i - 1, jN));
        W2_SYNC();
        W2_SFOR(i, iW + 1, iE - 1)
        UF(i, jN + 1) = UF(i - 1, jN + 1) + T(3.0) * (UF(i - 1, jN) - UF(i, jN)) -
                       T(4.0) * (VF(i, jN) - VF(i, jN - 1));
        W2_SYNC();
      } else if (t < BM_INTERN || t > BM_OUTLT2) {
        return false;
      }
    }
  return true;
#undef UF
#undef VF
}

// PresBoundCond, bound_cond.f:853-1024.
__device__ bool pres_bound_cond_block(const Dev &d, double *p) {
  const Regions &r = d.r;
#define PF(i, j) p[IX(d, i, j)]
  for (int jreg = 1; jreg <= r.nrj; jreg++)
    for (int ireg = 1; ireg <= r.nri; ireg++) {
      const int iW = r.B(ireg, jreg, WEST), iE = r.B(ireg, jreg, EAST);
      const int jS = r.B(ireg, jreg, SOUTH), jN = r.B(ireg, jreg, NORTH);
      if (r.RT(ireg, jreg) == RM_BLOCKG) {
        const int w = (iE - iW);
        for (int k = threadIdx.x; k < (jN - jS) * w; k += blockDim.x) {
          int j = jS + 1 + k / w, i = iW + 1 + k % w;
          PF(i, j) = 0.0;
        }
        W2_SYNC();
        const double pw = r.BV(ireg, jreg, WEST, VAR_P), pe = r.BV(ireg, jreg, EAST, VAR_P);
        const double ps = r.BV(ireg, jreg, SOUTH, VAR_P), pnv = r.BV(ireg, jreg, NORTH, VAR_P);
        W2_PFOR(j, jS + 1, jN) PF(iW + 1, j) = pw + PF(iW, j);
        W2_SYNC();
        W2_PFOR(j, jS + 1, jN) PF(iE, j) = pe + PF(iE + 1, j);
        W2_SYNC();
        W2_PFOR(i, iW + 1, iE) PF(i, jS + 1) = ps + PF(i, jS);
        W2_SYNC();
        W2_PFOR(i, iW + 1, iE) PF(i, jN) = pnv + PF(i, jN + 1);
        W2_SYNC();
        continue;
      }
      int t = r.BT(ireg, jreg, WEST);
      double val = r.BV(ireg, jreg, WEST, VAR_P);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        W2_PFOR(j, jS + 1, jN) PF(iW, j) = val + PF(iW + 1, j);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        W2_PFOR(j, jS + 1, jN) PF(iW, j) = 2.0 * val - PF(iW + 1, j);
      } else if (t != BM_INTERN) {
        return false;
      }
      W2_SYNC();
      t = r.BT(ireg, jreg, EAST);
      val = r.BV(ireg, jreg, EAST, VAR_P);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        W2_PFOR(j, jS + 1, jN) PF(iE + 1, j) = val + PF(iE, j);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        W2_PFOR(j, jS + 1, jN) PF(iE + 1, j) = 2.0 * val - PF(iE, j);
      } else if (t != BM_INTERN) {
        return false;
      }
      W2_SYNC();
      t = r.BT(ireg, jreg, SOUTH);
      val = r.BV(ireg, jreg, SOUTH, VAR_P);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        W2_PFOR(i, iW + 1, iE) PF(i, jS) = val + PF(i, jS + 1);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        W2_PFOR(i, iW + 1, iE) PF(i, jS) = 2.0 * val - PF(i, jS + 1);
      } else if (t != BM_INTERN) {
        return false;
      }
      W2_SYNC();
      t = r.BT(ireg, jreg, NORTH);
      val = r.BV(ireg, jreg, NORTH, VAR_P);
      if (t == BM_WALL1 || t == BM_WALL2 || t == BM_INLET) {
        W2_PFOR(i, iW + 1, iE) PF(i, jN + 1) = val + PF(i, jN);
      } else if (t == BM_OUTLT1 || t == BM_OUTLT2) {
        W2_PFOR(i, iW + 1, iE) PF(i, jN + 1) = 2.0 * val - PF(i, jN);
      } else if (t != BM_INTERN) {
        return false;
      }
      W2_SYNC();
    }
  return true;
#undef PF
}

}  // namespace w2
