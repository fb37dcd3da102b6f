// Walk of one assembly tile by one observation point: the cells of up to
// TL_COLS y-adjacent z-runs, level by level and run by run, with the faces
// shared in z (shared memory, per run) and in y (registers) taken over by
// prism_terms_tiled.  Used by every kernel that evaluates the prism terms of
// all cells for one point (assembly of G, matrix-free G x, FP64 refinement).
#pragma once

#include "kernels.h"
#include "prism.cuh"

namespace grada {

constexpr int TL_THREADS = 128;  // points per block
#ifndef GRADA_TILE_COLS
#define GRADA_TILE_COLS 8
#endif
constexpr int TL_COLS = GRADA_TILE_COLS;  // runs per tile
constexpr int TL_LCH = 8;        // levels staged per pass
constexpr int ZC_N = 9;          // doubles of a ZCarry
constexpr int TL_MAXLEV = 64;    // levels per tile (longer runs continue in the next tile)

// Bytes of the dynamic shared memory a tile walk needs (the z carries).
constexpr int tile_walk_dyn_smem() { return (int)sizeof(double) * TL_COLS * ZC_N * TL_THREADS; }

struct TileSmem {
  double sc[TL_LCH][TL_COLS][6];
  int64_t ci[TL_LCH][TL_COLS];
};

// All threads of the block call it for the same tile (it synchronises);
// threads without a point pass active = false.  f(cell, terms) is called for
// every cell of the tile in walk order.
template <class F>
__device__ __forceinline__ void tile_walk(const int4 td, const int64_t *__restrict__ cells,
                                          const double *__restrict__ prisms, TileSmem &ws,
                                          double *__restrict__ zsm, bool active, double px,
                                          double py, double pz, uint32_t fam,
                                          const double *__restrict__ tab, F &&f) {
  const int ncols = td.y, nlev = td.z;
  auto zslot = [&](int a, int q) -> double & {
    return zsm[((int64_t)a * ZC_N + q) * TL_THREADS + threadIdx.x];
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
      YCarry yc;
      for (int a = 0; a < ncols; a++) {
        const double *p = ws.sc[kk][a];
        ZCarry zin, zout;
        if (top) {
          zin.r[0][0] = zslot(a, 0); zin.r[0][1] = zslot(a, 1);
          zin.r[1][0] = zslot(a, 2); zin.r[1][1] = zslot(a, 3);
          zin.qx[0] = zslot(a, 4); zin.qx[1] = zslot(a, 5);
          zin.qy[0] = zslot(a, 6); zin.qy[1] = zslot(a, 7);
          zin.tz = zslot(a, 8);
        }
        YCarry yout;
        PrismTerms t;
        prism_terms_tiled(px, py, pz, p[0], p[1], p[2], p[3], p[4], p[5], fam, tab, top, zin,
                          a > 0, yc, zout, yout, t);
        zslot(a, 0) = zout.r[0][0]; zslot(a, 1) = zout.r[0][1];
        zslot(a, 2) = zout.r[1][0]; zslot(a, 3) = zout.r[1][1];
        zslot(a, 4) = zout.qx[0]; zslot(a, 5) = zout.qx[1];
        zslot(a, 6) = zout.qy[0]; zslot(a, 7) = zout.qy[1];
        zslot(a, 8) = zout.tz;
        yc = yout;
        f(ws.ci[kk][a], t);
      }
    }
  }
}

}  // namespace grada
