/*
 * Launch glue of the stage and CFS-PML kernels for one medium; expanded by
 * cgfd_launch_{iso,vti,vis}.cu with CGFD_MED and CGFD_MED_NAME set.
 */
#ifndef CGFD_LAUNCH_CUH
#define CGFD_LAUNCH_CUH

/* CGFD_SINGLE: the single-problem stage/PML launchers; CGFD_BATCH: the
 * batched stage launchers.  A translation unit may hold either or both. */
#ifndef CGFD_SINGLE
#define CGFD_SINGLE 1
#endif

#include "cgfd_launch.h"
#include "cgfd_media.cuh"
#include "cgfd_pml.cuh"
#include "cgfd_stage3.cuh"

#if CGFD_SINGLE
template <int BX, int BY, int BZ, int KIND, int MED>
static void launch_stage_t(dim3 grid, cudaStream_t st, const StageArgs &a,
                           const StageMaps &m)
{
  static bool attr_set = false;
  constexpr int smem = s3::Slot<MED>::SMEM_BYTES;
  if (!attr_set) {
    cudaFuncSetAttribute(s3::k_stage3<BX, BY, BZ, KIND, MED>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr_set = true;
  }
  s3::k_stage3<BX, BY, BZ, KIND, MED><<<grid, s3::NTHREADS, smem, st>>>(
      a, m.wav, m.met, m.med, m.pt, m.j);
}

template <int BX, int BY, int BZ, int MED>
static void launch_stage_k(int kind, dim3 grid, cudaStream_t st,
                           const StageArgs &a, const StageMaps &m)
{
  if (kind == 0) launch_stage_t<BX, BY, BZ, 0, MED>(grid, st, a, m);
  else if (kind == 1) launch_stage_t<BX, BY, BZ, 1, MED>(grid, st, a, m);
  else launch_stage_t<BX, BY, BZ, 2, MED>(grid, st, a, m);
}

template <int MED>
static void launch_stage_med(int code, int kind, dim3 grid, cudaStream_t st,
                             const StageArgs &a, const StageMaps &m)
{
  switch (code) {
    case 0: launch_stage_k<0, 0, 0, MED>(kind, grid, st, a, m); break;
    case 1: launch_stage_k<0, 0, 1, MED>(kind, grid, st, a, m); break;
    case 2: launch_stage_k<0, 1, 0, MED>(kind, grid, st, a, m); break;
    case 3: launch_stage_k<0, 1, 1, MED>(kind, grid, st, a, m); break;
    case 4: launch_stage_k<1, 0, 0, MED>(kind, grid, st, a, m); break;
    case 5: launch_stage_k<1, 0, 1, MED>(kind, grid, st, a, m); break;
    case 6: launch_stage_k<1, 1, 0, MED>(kind, grid, st, a, m); break;
    default: launch_stage_k<1, 1, 1, MED>(kind, grid, st, a, m); break;
  }
}

#endif

#if CGFD_BATCH
template <int BX, int BY, int BZ, int KIND, int MED>
static void launch_batch_t(int grid, cudaStream_t st, const StageArgs *args,
                           const s3::ShotGeo *geo, int nshot, const BatchSched &w)
{
  constexpr int smem = s3::Slot<MED>::SMEM_BYTES;
  if (grid <= 0) {   /* preparation only: set the shared-memory attribute */
    cudaFuncSetAttribute(s3::k_stage3_batch<BX, BY, BZ, KIND, MED>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return;
  }
  s3::k_stage3_batch<BX, BY, BZ, KIND, MED><<<grid, s3::NTHREADS, smem, st>>>(
      args, geo, nshot, w.order, w.nitems, w.next);
}

template <int BX, int BY, int BZ, int MED>
static void launch_batch_k(int kind, int grid, cudaStream_t st, const StageArgs *args,
                           const s3::ShotGeo *geo, int nshot, const BatchSched &w)
{
  if (kind == 0) launch_batch_t<BX, BY, BZ, 0, MED>(grid, st, args, geo, nshot, w);
  else if (kind == 1) launch_batch_t<BX, BY, BZ, 1, MED>(grid, st, args, geo, nshot, w);
  else launch_batch_t<BX, BY, BZ, 2, MED>(grid, st, args, geo, nshot, w);
}

template <int MED>
static void launch_batch_med(int code, int kind, int grid, cudaStream_t st,
                             const StageArgs *args, const s3::ShotGeo *geo, int nshot,
                             const BatchSched &w)
{
  switch (code) {
    case 0: launch_batch_k<0, 0, 0, MED>(kind, grid, st, args, geo, nshot, w); break;
    case 1: launch_batch_k<0, 0, 1, MED>(kind, grid, st, args, geo, nshot, w); break;
    case 2: launch_batch_k<0, 1, 0, MED>(kind, grid, st, args, geo, nshot, w); break;
    case 3: launch_batch_k<0, 1, 1, MED>(kind, grid, st, args, geo, nshot, w); break;
    case 4: launch_batch_k<1, 0, 0, MED>(kind, grid, st, args, geo, nshot, w); break;
    case 5: launch_batch_k<1, 0, 1, MED>(kind, grid, st, args, geo, nshot, w); break;
    case 6: launch_batch_k<1, 1, 0, MED>(kind, grid, st, args, geo, nshot, w); break;
    default: launch_batch_k<1, 1, 1, MED>(kind, grid, st, args, geo, nshot, w); break;
  }
}
#endif

#if CGFD_SINGLE
template <int DIM, int B, int MED>
static void launch_pml_t(int kind, int f, long long n, cudaStream_t st,
                         const StageArgs &a)
{
  dim3 b(256), gr((unsigned)((n + 255) / 256));
  if (kind == 0) k_pml_face<DIM, B, 0, MED><<<gr, b, 0, st>>>(a, f);
  else if (kind == 1) k_pml_face<DIM, B, 1, MED><<<gr, b, 0, st>>>(a, f);
  else k_pml_face<DIM, B, 2, MED><<<gr, b, 0, st>>>(a, f);
}

template <int MED>
static void launch_pml_med(int dim, int b, int kind, int f, long long n,
                           cudaStream_t st, const StageArgs &a)
{
  if (dim == 0) { if (b) launch_pml_t<0, 1, MED>(kind, f, n, st, a); else launch_pml_t<0, 0, MED>(kind, f, n, st, a); }
  else if (dim == 1) { if (b) launch_pml_t<1, 1, MED>(kind, f, n, st, a); else launch_pml_t<1, 0, MED>(kind, f, n, st, a); }
  else { if (b) launch_pml_t<2, 1, MED>(kind, f, n, st, a); else launch_pml_t<2, 0, MED>(kind, f, n, st, a); }
}

#endif

#define CGFD_CAT2(a, b) a##b
#define CGFD_CAT(a, b) CGFD_CAT2(a, b)

#if CGFD_SINGLE
void CGFD_CAT(cgfd_launch_stage_, CGFD_MED_NAME)(int code, int kind, dim3 grid,
                                                 cudaStream_t st, const StageArgs &a,
                                                 const StageMaps &m)
{
  launch_stage_med<CGFD_MED>(code, kind, grid, st, a, m);
}

#endif

#if CGFD_BATCH
void CGFD_CAT(cgfd_launch_stage_batch_, CGFD_MED_NAME)(int code, int kind, int grid,
                                                       cudaStream_t st,
                                                       const StageArgs *args,
                                                       const s3::ShotGeo *geo, int nshot,
                                                       const BatchSched &w)
{
  launch_batch_med<CGFD_MED>(code, kind, grid, st, args, geo, nshot, w);
}

/* tile rows the batched kernel was compiled with: must equal the single
 * kernel's, whose tensor maps the batch reuses */
int CGFD_CAT(cgfd_stage_rows_batch_, CGFD_MED_NAME)(void) { return s2::TY; }
#endif

#if CGFD_SINGLE
int CGFD_CAT(cgfd_stage_rows_, CGFD_MED_NAME)(void) { return s2::TY; }

int CGFD_CAT(cgfd_stage_smem_, CGFD_MED_NAME)(void)
{
  return s3::Slot<CGFD_MED>::SMEM_BYTES;
}

void CGFD_CAT(cgfd_launch_pml_, CGFD_MED_NAME)(int dim, int b, int kind, int f,
                                               long long n, cudaStream_t st,
                                               const StageArgs &a)
{
  launch_pml_med<CGFD_MED>(dim, b, kind, f, n, st, a);
}
#endif

#endif
