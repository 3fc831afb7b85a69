/*
 * CFS-PML region kernel.
 *
 * The points inside the CFS-PML faces (about a fifth of a 400 x 400 x 200
 * model with 12-layer faces) take their whole stage update here: interior
 * RHS, free-surface overwrites, the PML corrections of every face containing
 * the point in the reference order x1, x2, y1, y2, z1, z2, sources and the
 * RK combine -- the per-point function of cgfd_stage.cuh, i.e. exactly the
 * reference's sequence (forward/sv_curv_col_el_iso.c:22-1146,
 * forward/drv_rk_curv_col.c:292-446).  The TMA interior kernel skips these
 * points, so both kernels write disjoint points and run concurrently on two
 * streams.
 *
 * The union of the face boxes is split on the host into disjoint boxes
 * (x faces; y faces without the x columns; z faces without both), one
 * thread per point, i fastest.
 */
#ifndef CGFD_PML_CUH
#define CGFD_PML_CUH

#include "cgfd_common.h"
#include "cgfd_stage.cuh"

template <int BX, int BY, int BZ, int KIND>
__global__ void __launch_bounds__(128)
    k_pml_region(const __grid_constant__ StageArgs a, long long total)
{
  long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (n >= total) return;
  int r = 0;
  while (r + 1 < a.nreg && n >= a.reg[r + 1].start) r++;
  const DevBox &B = a.reg[r];
  long long m = n - B.start;
  int bx = B.i2 - B.i1 + 1, by = B.j2 - B.j1 + 1;
  int i = B.i1 + (int)(m % bx);
  int j = B.j1 + (int)((m / bx) % by);
  int k = B.k1 + (int)(m / ((long long)bx * by));
  stage_point<BX, BY, BZ, KIND>(a, i, j, k);
}

#endif
