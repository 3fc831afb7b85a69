/*
 * Launchers of the per-stage kernels, one set per medium.  Each medium's
 * kernels live in their own translation unit (cgfd_launch_{iso,vti,vis,ani}.cu,
 * all expanding cgfd_launch.cuh) so that the library's build compiles them
 * in parallel; cgfd_solver.cu only sees these declarations.
 */
#ifndef CGFD_LAUNCH_H
#define CGFD_LAUNCH_H

#include <cuda.h>
#include <cuda_runtime.h>

#include "cgfd_common.h"

namespace s3 {
struct ShotGeo;
}

/* tensor maps of one solver (cgfd_stage3.cuh) */
struct StageMaps {
  CUtensorMap wav;   /* 5-D (x, y, z, component, level), 9-component planes */
  CUtensorMap met;   /* 4-D metrics, TX x TY tiles */
  CUtensorMap med;   /* 4-D media, TX x TY tiles */
  CUtensorMap pt;    /* 5-D wavefield, TX x TY x 9 tiles (pre / end) */
  CUtensorMap j;     /* 5-D wavefield, TX x TY x 6 nmw tiles (memory variables) */
};

/* fused interior stage kernel: bias code bx*4 + by*2 + bz, kind 0/1/2 */
void cgfd_launch_stage_iso(int code, int kind, dim3 grid, cudaStream_t st,
                           const StageArgs &a, const StageMaps &m);
void cgfd_launch_stage_vti(int code, int kind, dim3 grid, cudaStream_t st,
                           const StageArgs &a, const StageMaps &m);
void cgfd_launch_stage_vis(int code, int kind, dim3 grid, cudaStream_t st,
                           const StageArgs &a, const StageMaps &m);
void cgfd_launch_stage_ani(int code, int kind, dim3 grid, cudaStream_t st,
                           const StageArgs &a, const StageMaps &m);

/* work items of a batched stage launch: nitems (shot, tile, k chunk)
 * items; next == null: one CTA per item; otherwise persistent CTAs take
 * items in the order of order[] from the counter *next (zeroed before the
 * launch) */
struct BatchSched {
  const int *order;
  int nitems;
  int *next;
};

/* the stage of a batch of shots in one launch of `grid` CTAs (per-shot
 * arguments and tensor maps in device memory); isotropic and VTI media.
 * grid <= 0 only sets the kernel's shared-memory attribute (done for every
 * form before a CUDA graph is captured). */
void cgfd_launch_stage_batch_iso(int code, int kind, int grid, cudaStream_t st,
                                 const StageArgs *args, const s3::ShotGeo *geo,
                                 int nshot, const BatchSched &w);
void cgfd_launch_stage_batch_vti(int code, int kind, int grid, cudaStream_t st,
                                 const StageArgs *args, const s3::ShotGeo *geo,
                                 int nshot, const BatchSched &w);

/* CFS-PML face kernel of face f (normal dim, operator bias b), n points */
void cgfd_launch_pml_iso(int dim, int b, int kind, int f, long long n,
                         cudaStream_t st, const StageArgs &a);
void cgfd_launch_pml_vti(int dim, int b, int kind, int f, long long n,
                         cudaStream_t st, const StageArgs &a);
void cgfd_launch_pml_vis(int dim, int b, int kind, int f, long long n,
                         cudaStream_t st, const StageArgs &a);
void cgfd_launch_pml_ani(int dim, int b, int kind, int f, long long n,
                         cudaStream_t st, const StageArgs &a);

/* tile rows (consumer warps) and dynamic shared memory of each medium's
 * stage kernel */
int cgfd_stage_rows_iso(void);
int cgfd_stage_rows_vti(void);
int cgfd_stage_rows_vis(void);
int cgfd_stage_rows_ani(void);
int cgfd_stage_rows_batch_iso(void);
int cgfd_stage_rows_batch_vti(void);
int cgfd_stage_smem_iso(void);
int cgfd_stage_smem_vti(void);
int cgfd_stage_smem_vis(void);
int cgfd_stage_smem_ani(void);

#endif
