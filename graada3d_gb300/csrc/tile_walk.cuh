// Walk of one assembly tile by one observation point: the cells of up to
// TL_COLS z-runs (nx = 1 or 2 runs across x times ny runs along y), level by
// level, with the faces shared with the cell above (z, shared memory per run),
// the cell before in y and the cell before in x taken over by
// prism_terms_tiled.  Used by every kernel that evaluates the prism terms of
// all cells for one point (assembly of G, matrix-free G x and G^T y, FP64
// refinement).
#pragma once

#include "kernels.h"
#include "prism.cuh"

namespace grada {

constexpr int TL_THREADS = 128;  // points per block
constexpr int TL_COLS = 8;       // runs per tile
constexpr int TL_LCH = 8;        // levels staged per pass
constexpr int ZC_N = 9;          // doubles of a ZCarry
constexpr int YC_N = 9;          // doubles of a YCarry
constexpr int TL_MAXLEV = 64;    // levels per tile (longer runs continue in the next tile)
constexpr int TL_MAXNX = 2;      // runs across x in a tile

// Bytes of the dynamic shared memory a tile walk needs: the z carries of the
// tile's runs and, for the walk that shares x faces, the y carries of the
// tile's columns across x.
constexpr int tile_walk_dyn_smem(bool share_x) {
  return (int)sizeof(double) * TL_THREADS *
         (TL_COLS * ZC_N + (share_x ? TL_MAXNX * YC_N : 0));
}

struct TileSmem {
  double sc[TL_LCH][TL_COLS][6];
  int64_t ci[TL_LCH][TL_COLS];
};

// All threads of the block call it for the same tile (it synchronises);
// threads without a point pass active = false.  Run a of a tile (td = {first
// cell, runs, levels, nx}) sits at x = a % nx, y = a / nx; its cell at level k
// is cells[td.x + a * levels + k].  f(cell, q, terms) is called for every cell,
// q = k * runs + a.
//  * SHARE_X: within a level the runs are walked y-major, x-minor; the x carry
//    stays in registers and the y carries of the nx columns in shared memory
//    (dyn points to tile_walk_dyn_smem(true) bytes).
//  * otherwise: x-major, y-minor with the y carry in registers and no x
//    sharing (tile_walk_dyn_smem(false) bytes), for kernels whose registers
//    or shared memory are needed elsewhere.
template <bool SHARE_X, class F>
__device__ __forceinline__ void tile_walk(const int4 td, const int64_t *__restrict__ cells,
                                          const double *__restrict__ prisms, TileSmem &ws,
                                          double *__restrict__ dyn, bool active, double px,
                                          double py, double pz, uint32_t fam,
                                          const double *__restrict__ tab, F &&f) {
  const int ncols = td.y, nlev = td.z;
  const int nx = td.w > 1 ? TL_MAXNX : 1;
  const int ny = ncols / nx;
  auto zslot = [&](int a, int q) -> double & {
    return dyn[((int64_t)a * ZC_N + q) * TL_THREADS + threadIdx.x];
  };
  auto yslot = [&](int x, int q) -> double & {
    return dyn[((int64_t)TL_COLS * ZC_N + x * YC_N + q) * TL_THREADS + threadIdx.x];
  };
  for (int k0 = 0; k0 < nlev; k0 += TL_LCH) {
    const int nl = min(TL_LCH, nlev - k0);
    __syncthreads();  // the previous chunk's (or tile's) readers are done with ws
    for (int t = threadIdx.x; t < nl * ncols * 6; t += TL_THREADS) {
      const int k = t / (ncols * 6), a = (t / 6) % ncols, q = t % 6;
      const int64_t cell = cells[td.x + (int64_t)a * nlev + k0 + k];
      ws.sc[k][a][q] = prisms[cell * 6 + q];
      if (q == 0) ws.ci[k][a] = cell;
    }
    __syncthreads();
    if (!active) continue;
    for (int kk = 0; kk < nl; kk++) {
      const int k = k0 + kk;
      const bool top = k > 0;
      // one cell: z carry from/to its run's slot, y and x carries as given
      auto cell_terms = [&](int a, bool yprev, const YCarry &yin, bool xprev, const XCarry &xin,
                            YCarry &yout, XCarry &xout) {
        const double *p = ws.sc[kk][a];
        ZCarry zin, zout;
        if (top) {
          zin.r[0][0] = zslot(a, 0); zin.r[0][1] = zslot(a, 1);
          zin.r[1][0] = zslot(a, 2); zin.r[1][1] = zslot(a, 3);
          zin.qx[0] = zslot(a, 4); zin.qx[1] = zslot(a, 5);
          zin.qy[0] = zslot(a, 6); zin.qy[1] = zslot(a, 7);
          zin.tz = zslot(a, 8);
        }
        PrismTerms t;
        prism_terms_tiled(px, py, pz, p[0], p[1], p[2], p[3], p[4], p[5], fam, tab, top, zin,
                          yprev, yin, xprev, xin, zout, yout, xout, t);
        zslot(a, 0) = zout.r[0][0]; zslot(a, 1) = zout.r[0][1];
        zslot(a, 2) = zout.r[1][0]; zslot(a, 3) = zout.r[1][1];
        zslot(a, 4) = zout.qx[0]; zslot(a, 5) = zout.qx[1];
        zslot(a, 6) = zout.qy[0]; zslot(a, 7) = zout.qy[1];
        zslot(a, 8) = zout.tz;
        f(ws.ci[kk][a], k * ncols + a, t);
      };
      if constexpr (SHARE_X) {
        for (int y = 0; y < ny; y++) {
          XCarry xc;
          for (int x = 0; x < nx; x++) {
            YCarry yin, yout;
            if (y > 0) {
              yin.r[0][0] = yslot(x, 0); yin.r[0][1] = yslot(x, 1);
              yin.r[1][0] = yslot(x, 2); yin.r[1][1] = yslot(x, 3);
              yin.qx[0] = yslot(x, 4); yin.qx[1] = yslot(x, 5);
              yin.qz[0] = yslot(x, 6); yin.qz[1] = yslot(x, 7);
              yin.ty = yslot(x, 8);
            }
            XCarry xout;
            cell_terms(y * nx + x, y > 0, yin, x > 0, xc, yout, xout);
            yslot(x, 0) = yout.r[0][0]; yslot(x, 1) = yout.r[0][1];
            yslot(x, 2) = yout.r[1][0]; yslot(x, 3) = yout.r[1][1];
            yslot(x, 4) = yout.qx[0]; yslot(x, 5) = yout.qx[1];
            yslot(x, 6) = yout.qz[0]; yslot(x, 7) = yout.qz[1];
            yslot(x, 8) = yout.ty;
            xc = xout;
          }
        }
      } else {
        for (int x = 0; x < nx; x++) {
          YCarry yc;
          XCarry xnone, xout;
          for (int y = 0; y < ny; y++) {
            YCarry yout;
            cell_terms(y * nx + x, y > 0, yc, false, xnone, yout, xout);
            yc = yout;
          }
        }
      }
    }
  }
}

}  // namespace grada
