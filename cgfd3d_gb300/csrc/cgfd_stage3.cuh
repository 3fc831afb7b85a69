/*
 * Stage kernel: warp-specialised, TMA-fed, z-marching (sm_103a).
 *
 * Work split.  A CTA owns a 32 x 8 column tile of the (i, j) plane and a run
 * of `kchunk` k planes.  Warp 8 is the producer: its lane 0 issues every
 * load of the CTA as bulk tensor copies (cp.async.bulk.tensor) into shared
 * memory; warps 0-7 are consumers, one tile row each, and never touch global
 * memory for the regular stencil path.
 *
 * Shared memory (167 KB, one CTA per SM):
 *   wavefield ring  NB = 6 plane tiles (9 components with x/y halo, see
 *                   cgfd_stage2.cuh) -- the 5 planes of the z operator's
 *                   window plus one in flight;
 *   stream ring     NS = 2 slots of the per-point streams of one plane:
 *                   the 9 metrics, media (slw, lambda, mu) and, as the
 *                   stage needs them, the `pre` and `end` levels.
 *
 * Synchronisation uses only mbarriers: `full` barriers complete when a
 * copy's bytes land (expect_tx / complete_tx), `empty` barriers complete
 * when all eight consumer warps have released a buffer.  With no CTA-wide
 * barrier in the loop, consumer warps drift freely and the producer runs
 * as far ahead as the rings allow.  Every wait is bounded: on timeout the
 * waiting thread records device error 1 (a.err) and goes on, so the kernel
 * always terminates and the host reports the failure.
 *
 * Per point the consumer computes the interior RHS, the traction image and
 * vlow overwrites at the top layers, the CFS-PML terms of every face that
 * contains the point (in the reference's face order, with the face's
 * auxiliary variables advanced in the same pass), the sources and the RK
 * combine (reference: forward/sv_curv_col_el_iso.c:208-1146,
 * forward/sv_curv_col_el.c:30-479, forward/drv_rk_curv_col.c:292-446).
 * The auxiliary variables are the only operands read straight from global
 * memory: they are pointwise (no stencil), and each consumer thread
 * prefetches its next plane's auxiliaries into L2 one plane ahead so that
 * the loads of the PML points hit L2.  With a.pml_fused = 0 the PML terms
 * are left to the face kernels of cgfd_pml.cuh instead.
 *
 * MED selects the medium (cgfd_media.cuh).  VTI changes Hooke's law only
 * (forward/sv_curv_col_el_vti.c:200-590).  The GMB visco-elastic medium
 * (forward/sv_curv_col_vis_iso.c:165-347) adds, per point, the memory
 * variables J (6 per Maxwell body): their current values and the
 * coefficients Ylam/Ymu arrive through the stream slot, and the stage
 *   hJ_n = wl_n (EV(hT) - J_n),  hT -= lam sum Ylam_n tr(J_n) + 2 mu sum Ymu_n J_n
 * is applied before the sources, as in the reference (EV: strain rates
 * implied by hT).  J's RK combine reads pre/end directly (coalesced rows).
 */
#ifndef CGFD_STAGE3_CUH
#define CGFD_STAGE3_CUH

#include "cgfd_media.cuh"
#include "cgfd_stage2.cuh"

namespace s3 {

using namespace s2;

constexpr int NB = 6;                 /* wavefield ring */
constexpr int NS = 2;                 /* stream ring */
constexpr int NCW = TY;               /* consumer warps (one per tile row) */
constexpr int NTHREADS = (NCW + 1) * 32;
constexpr int PTS = TX * TY;

/* stream-slot layout (floats) for a medium: metrics (the 9 of xi, eta,
 * zeta; jac is read from global memory at the top layers only), media,
 * current memory variables (visco), pre, end */
template <int MED>
struct Slot {
  static constexpr int NMED = MED == MED_VTI ? 6
                            : MED == MED_VIS ? 3 + 2 * CGFD_VIS_NMW_MAX
                            : MED == MED_ANI ? 22 : 3;
  static constexpr int NJ = MED == MED_VIS ? 6 * CGFD_VIS_NMW_MAX : 0;
  static constexpr int S_MET = 0;
  static constexpr int S_MED = 9 * PTS;
  static constexpr int S_JC = S_MED + NMED * PTS;
  static constexpr int S_PRE = S_JC + NJ * PTS;
  static constexpr int S_END = S_PRE + 9 * PTS;
  static constexpr int SLOT = S_END + 9 * PTS;
  static constexpr int SMEM_BYTES = (NB * PLANE + NS * SLOT) * 4;
  /* every bulk tensor copy lands on a 128-byte aligned shared address */
  static_assert(PTS % 32 == 0 && (NB * PLANE) % 32 == 0 && SLOT % 32 == 0,
                "stream-slot regions must stay 128-byte aligned");
  static_assert(SMEM_BYTES <= 232448, "more shared memory than one CTA gets");
};

/* bounded wait; `err` records a timeout, and false is returned */
__device__ __forceinline__ bool wait_full(uint64_t *bar, uint32_t parity, int *err, int limit)
{
  return mbar_wait(bar, parity, err, limit);
}

/* L2 prefetch of one global address (no register, no completion) */
__device__ __forceinline__ void prefetch_l2(const float *p)
{
  asm volatile("prefetch.global.L2::evict_last [%0];" ::"l"(p));
}

__device__ __forceinline__ bool in_face(const DevFace &F, int i, int j, int k)
{
  return F.on && i >= F.i1 && i <= F.i2 && j >= F.j1 && j <= F.j2 &&
         k >= F.k1 && k <= F.k2;
}

/* L2 prefetch of the auxiliary variables a stage reads at (i, j, k) of the
 * faces in `mask` (bit f: face f holds the point) */
template <int KIND>
__device__ __forceinline__ void prefetch_aux(const StageArgs &a, int i, int j, int k,
                                             int mask)
{
#pragma unroll
  for (int f = 0; f < CGFD_NFACE; f++) {
    if (!(mask & (1 << f))) continue;
    const DevFace &F = a.face[f];
    const long long av = F.avol;
    const long long ai = (long long)(i - F.i1) + (long long)(j - F.j1) * F.bx +
                         (long long)(k - F.k1) * F.bx * F.by;
#pragma unroll
    for (int c = 0; c < 9; c++) {
      prefetch_l2(a.acur[f] + c * av + ai);
      if (KIND == 1) prefetch_l2(a.apre[f] + c * av + ai);
      if (KIND >= 1) prefetch_l2(a.aend[f] + c * av + ai);
    }
  }
}

/* CFS-PML terms of face f at one point (forward/sv_curv_col_el_iso.c:
 * 708-1143, VTI forward/sv_curv_col_el_vti.c:592-1075): corrections added
 * to r, the face's auxiliary variables advanced by the RK stage.  d holds
 * the nine derivatives along the face normal, e1..e3 that direction's
 * metric. */
template <int KIND>
struct AuxPt {
  float ac[9], ap[KIND == 1 ? 9 : 1], ae[KIND >= 1 ? 9 : 1];
};

template <int KIND>
__device__ __forceinline__ long long aux_index(const DevFace &F, int i, int j, int k)
{
  return (long long)(i - F.i1) + (long long)(j - F.j1) * F.bx +
         (long long)(k - F.k1) * F.bx * F.by;
}

/* the auxiliary values one stage reads at a face point */
template <int KIND>
__device__ __forceinline__ void load_aux(const StageArgs &a, int f, long long ai,
                                         AuxPt<KIND> &x)
{
  const long long av = a.face[f].avol;
#pragma unroll
  for (int c = 0; c < 9; c++) {
    x.ac[c] = __ldg(a.acur[f] + c * av + ai);
    if (KIND == 1) x.ap[c] = __ldg(a.apre[f] + c * av + ai);
    if (KIND >= 1) x.ae[c] = a.aend[f][c * av + ai];
  }
}

template <int KIND, int MED>
__device__ __forceinline__ void spml_face(const StageArgs &a, int f, int i,
                                          int j, int k, long long q,
                                          const float *d, float e1, float e2,
                                          float e3, float ztx, float zty,
                                          float ztz, const MedPt &m,
                                          const AuxPt<KIND> &x, float *r)
{
  const DevFace &F = a.face[f];
  const long long av = F.avol;
  const long long ai = aux_index<KIND>(F, i, j, k);
  const float *ac = x.ac, *ap = x.ap, *ae = x.ae;
  const int n = F.dim == 0 ? i - F.i1 : (F.dim == 1 ? j - F.j1 : k - F.k1);
  const float cD = __ldg(F.D + n), cA = __ldg(F.A + n), cB = __ldg(F.B + n);
  const float cB1 = cB - 1.0f;
  float sv[9];
  sv[C_VX] = m.slw * (e1 * d[C_TXX] + e2 * d[C_TXY] + e3 * d[C_TXZ]);
  sv[C_VY] = m.slw * (e1 * d[C_TXY] + e2 * d[C_TYY] + e3 * d[C_TYZ]);
  sv[C_VZ] = m.slw * (e1 * d[C_TXZ] + e2 * d[C_TYZ] + e3 * d[C_TZZ]);
  hooke1<MED>(m, e1, e2, e3, d[C_VX], d[C_VY], d[C_VZ], sv);
  float arhs[9];
#pragma unroll
  for (int c = 0; c < 9; c++) {
    r[c] += cB1 * sv[c] - cB * ac[c];
    arhs[c] = cD * sv[c] - cA * ac[c];
  }
  if (F.dim < 2 && a.free_top && k == a.g.nk2) {
    /* free-surface part: the z gradients converted from this direction's
     * (forward/sv_curv_col_el_iso.c:841-901) */
    const long long ij = ((long long)i + (long long)j * a.g.nx) * 9;
    const float *M = (F.dim == 0 ? a.mVx : a.mVy) + ij;
    float DzVx = __ldg(M + 0) * d[C_VX] + __ldg(M + 1) * d[C_VY] + __ldg(M + 2) * d[C_VZ];
    float DzVy = __ldg(M + 3) * d[C_VX] + __ldg(M + 4) * d[C_VY] + __ldg(M + 5) * d[C_VZ];
    float DzVz = __ldg(M + 6) * d[C_VX] + __ldg(M + 7) * d[C_VY] + __ldg(M + 8) * d[C_VZ];
    float t[9];
    hooke1<MED>(m, ztx, zty, ztz, DzVx, DzVy, DzVz, t);
#pragma unroll
    for (int c = C_TXX; c <= C_TXY; c++) {
      r[c] += cB1 * t[c];
      arhs[c] += cD * t[c];
    }
  }
#pragma unroll
  for (int c = 0; c < 9; c++) {
    const long long x = c * av + ai;
    if (KIND == 0) {
      a.atmp_out[f][x] = ac[c] + a.ca * arhs[c];
      a.aend[f][x] = ac[c] + a.cb * arhs[c];
    } else if (KIND == 1) {
      a.atmp_out[f][x] = ap[c] + a.ca * arhs[c];
      a.aend[f][x] = ae[c] + a.cb * arhs[c];
    } else {
      a.aend[f][x] = ae[c] + a.cb * arhs[c];
    }
  }
}

/* tensor maps and CTA grid of one shot of a batch (global memory; the
 * tensor maps keep their 64-byte alignment) */
struct ShotGeo {
  CUtensorMap wav, met, med, pt, j;
  int tiles_x, tiles_y, nchunk, cta0;   /* CTA grid of the shot, first CTA */
  int pad[12];
};

/* One CTA of the stage: tile (bx, by) of the (i, j) plane, k chunk bz. */
template <int BX, int BY, int BZ, int KIND, int MED>
__device__ __forceinline__ void stage3_body(const StageArgs &a,
                                            const CUtensorMap &tmap,
                                            const CUtensorMap &tmap_met,
                                            const CUtensorMap &tmap_med,
                                            const CUtensorMap &tmap_pt,
                                            const CUtensorMap &tmap_j,
                                            int bx, int by, int bz, bool gmem_maps,
                                            bool again = false)
{
  using L = Slot<MED>;
  constexpr int S_MET = L::S_MET, S_MED = L::S_MED, S_JC = L::S_JC,
                S_PRE = L::S_PRE, S_END = L::S_END, SLOT = L::SLOT;
  extern __shared__ __align__(128) float sm[];
  __shared__ __align__(8) uint64_t full_w[NB], empty_w[NB], full_s[NS], empty_s[NS];
  /* set by the first wait that runs out: every warp of the CTA then leaves
   * its loop, and the producer waits for the copies it issued */
  __shared__ int abort_s;
  float *ring = sm;
  float *slots = sm + NB * PLANE;
  const int lim = a.wait_limit > 0 ? a.wait_limit : (1 << 22);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const DevGrid &g = a.g;
  const int i0 = g.ni1 + bx * TX;
  const int j0 = g.nj1 + by * TY;
  const int kbeg = g.nk1 + bz * a.kchunk;
  const int kend = min(kbeg + a.kchunk - 1, g.nk2);
  const int niter = kend - kbeg + 1;
  constexpr int ZS0 = BZ == 0 ? -1 : -3;
  constexpr int YL = BY == 0 ? 1 : 3;
  constexpr int ZC = BZ == 0 ? 1 : 3;
  const int pbase = kbeg + ZS0;       /* plane of ring index 0 */

  if (threadIdx.x == 0) {
    if (again) {
      /* a persistent CTA's next item: the previous one's barriers have no
       * operation left (the caller synchronised after it) */
      for (int b = 0; b < NB; b++) { mbar_inval(&full_w[b]); mbar_inval(&empty_w[b]); }
      for (int b = 0; b < NS; b++) { mbar_inval(&full_s[b]); mbar_inval(&empty_s[b]); }
    }
    for (int b = 0; b < NB; b++) { mbar_init(&full_w[b], 1); mbar_init(&empty_w[b], NCW); }
    for (int b = 0; b < NS; b++) { mbar_init(&full_s[b], 1); mbar_init(&empty_s[b], NCW); }
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  /* ------------------------------------------------------------------ */
  /* producer                                                             */
  /* ------------------------------------------------------------------ */
  if (warp == NCW) {
    if (lane != 0) return;
    if (gmem_maps) {
      /* tensor maps read from global memory: order the writes that put them
       * there before the bulk copies read them */
      const CUtensorMap *maps[5] = {&tmap, &tmap_met, &tmap_med, &tmap_pt, &tmap_j};
#pragma unroll
      for (int m = 0; m < 5; m++)
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                         reinterpret_cast<uint64_t>(maps[m]))
                     : "memory");
    }
    const int bx0 = i0 + g.xoff - XL;  /* 16-byte aligned box origin */
    const int by0 = j0 - YL;
    const int xs = i0 + g.xoff;        /* stream tiles: no halo */
    const int nmed = med_ncomp(MED, a.nmw);
    const uint32_t slot_bytes =
        (9 + nmed + (MED == MED_VIS ? 6 * a.nmw : 0) + (KIND == 1 ? 9 : 0) +
         (KIND >= 1 ? 9 : 0)) * PTS * 4;
    /* the latest copy issued into each buffer (ring position), for the
     * drain after an abort; -1: none */
    int last_w[NB], last_s[NS];
#pragma unroll
    for (int b = 0; b < NB; b++) last_w[b] = -1;
#pragma unroll
    for (int b = 0; b < NS; b++) last_s[b] = -1;
    const bool test_cta = a.test_skip_plane >= 0 && bx == 0 && by == 0 && bz == 0;
    /* false once the CTA has aborted (a wait ran out here or elsewhere) */
    auto live = [&]() { return *(volatile int *)&abort_s == 0; };
    auto issue_wav = [&](int rel) {
      if (!live()) return;
      int b = rel % NB;
      if (rel >= NB) {
        if (!mbar_wait(&empty_w[b], ((rel / NB) - 1) & 1, a.err, lim)) {
          abort_s = 1;
          return;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      }
      if (test_cta && rel == a.test_skip_plane) return;   /* never arrives */
      mbar_expect_tx(&full_w[b], PLANE_DATA * 4);
      tma_load_5d(ring + b * PLANE, &tmap, bx0, by0, pbase + rel, 0, a.cur_level,
                  &full_w[b]);
      last_w[b] = rel;
    };
    auto issue_slot = [&](int it) {
      if (!live()) return;
      int b = it % NS;
      if (it >= NS) {
        if (!mbar_wait(&empty_s[b], ((it / NS) - 1) & 1, a.err, lim)) {
          abort_s = 1;
          return;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      }
      last_s[b] = it;
      float *dst = slots + b * SLOT;
      int k = kbeg + it;
      mbar_expect_tx(&full_s[b], slot_bytes);
      tma_load_4d(dst + S_MET, &tmap_met, xs, j0, k, 1, &full_s[b]);
      tma_load_4d(dst + S_MED, &tmap_med, xs, j0, k, 0, &full_s[b]);
      if (MED == MED_VIS) {
        tma_load_5d(dst + S_JC, &tmap_j, xs, j0, k, 9, a.cur_level, &full_s[b]);
        /* the memory variables' pre/end values are read directly by the
         * consumers (no shared memory left): bring them into L2 now */
        if (KIND == 1) tma_prefetch_5d(&tmap_j, xs, j0, k, 9, a.pre_level);
        if (KIND >= 1) tma_prefetch_5d(&tmap_j, xs, j0, k, 9, a.end_level);
      }
      if (KIND == 1) tma_load_5d(dst + S_PRE, &tmap_pt, xs, j0, k, 0, a.pre_level, &full_s[b]);
      if (KIND >= 1) tma_load_5d(dst + S_END, &tmap_pt, xs, j0, k, 0, a.end_level, &full_s[b]);
    };
    /* L2 prefetch of the tiles a.l2_ahead planes beyond what the rings
     * hold: more bytes in flight per SM than the shared memory allows */
    const int L2_AHEAD = a.l2_ahead;
    auto prefetch_ahead = [&](int it) {
      const int ip = it + L2_AHEAD;
      if (ip < niter) {
        const int k = kbeg + ip;
        tma_prefetch_4d(&tmap_met, xs, j0, k, 1);
        tma_prefetch_4d(&tmap_med, xs, j0, k, 0);
        if (MED == MED_VIS) tma_prefetch_5d(&tmap_j, xs, j0, k, 9, a.cur_level);
        if (KIND == 1) tma_prefetch_5d(&tmap_pt, xs, j0, k, 0, a.pre_level);
        if (KIND >= 1) tma_prefetch_5d(&tmap_pt, xs, j0, k, 0, a.end_level);
      }
      const int rp = it + 5 + L2_AHEAD;
      if (rp < niter + 4) tma_prefetch_5d(&tmap, bx0, by0, pbase + rp, 0, a.cur_level);
    };
    for (int rel = 0; rel < 5; rel++) issue_wav(rel);
    for (int it = 0; it < niter && live(); it++) {
      if (L2_AHEAD > 0) prefetch_ahead(it);
      issue_slot(it);
      if (it + 5 < niter + 4) issue_wav(it + 5);
    }
    if (!live()) {
      /* aborted: the CTA leaves only after the copies it issued have
       * landed in its shared memory (each wait bounded again) */
#pragma unroll
      for (int b = 0; b < NB; b++)
        if (last_w[b] >= 0) mbar_wait(&full_w[b], (last_w[b] / NB) & 1, a.err, lim);
#pragma unroll
      for (int b = 0; b < NS; b++)
        if (last_s[b] >= 0) mbar_wait(&full_s[b], (last_s[b] / NS) & 1, a.err, lim);
    }
    return;
  }

  /* ------------------------------------------------------------------ */
  /* consumers                                                            */
  /* ------------------------------------------------------------------ */
  const int tx = lane, ty = warp;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = (i <= g.ni2) && (j <= g.nj2);
  const int row = ty + YL, col = tx + XL;
  const long long px = g.px, sl = g.sl, vol = g.vol;
  const int sp = ty * TX + tx;        /* point index inside a stream slot */

  /* per-thread constants of the k loop */
  int src_e0 = 0, src_e1 = 0, dd_e0 = 0, dd_e1 = 0;
  if (a.src_n > 0 && valid) {
    long long colidx = (long long)(i - g.ni1) + (long long)(j - g.nj1) * g.ni;
    src_e0 = a.src_col[colidx];
    src_e1 = a.src_col[colidx + 1];
  }
  if (a.dd_n > 0 && valid) {
    long long colidx = (long long)(i - g.ni1) + (long long)(j - g.nj1) * g.ni;
    dd_e0 = a.dd_col[colidx];
    dd_e1 = a.dd_col[colidx + 1];
  }

  /* faces whose (i, j) range holds this column (x/y faces), and the k
   * ranges of the z faces, so that points outside every face skip the PML
   * logic with register tests only */
  int fmask_xy = 0, kz1_top = -1, kz2_bot = 1 << 30;
  if (a.pml_fused && valid) {
#pragma unroll
    for (int f = 0; f < 4; f++) {
      const DevFace &F = a.face[f];
      if (F.on && i >= F.i1 && i <= F.i2 && j >= F.j1 && j <= F.j2) fmask_xy |= 1 << f;
    }
    if (a.face[4].on) kz1_top = a.face[4].k2;
    if (a.face[5].on) kz2_bot = a.face[5].k1;
  }
  /* faces holding the point at plane kk: x/y faces span every k, z faces
   * every (i, j) (forward/bdry_t.c:168-186) */
  auto pml_mask = [&](int kk) {
    return fmask_xy | (kk <= kz1_top ? 16 : 0) | (kk >= kz2_bot ? 32 : 0);
  };
  if (a.pml_fused && valid && pml_mask(kbeg))
    prefetch_aux<KIND>(a, i, j, kbeg, pml_mask(kbeg));

  for (int it = 0; it < niter; it++) {
    const int k = kbeg + it;
    const int rtop = it + 4;
    const int pmask = (a.pml_fused && valid) ? pml_mask(k) : 0;
    if (a.pml_fused && valid && it + 1 < niter && pml_mask(k + 1))
      prefetch_aux<KIND>(a, i, j, k + 1, pml_mask(k + 1));
    /* every lane waits; the warp leaves together when any wait of the CTA
     * has run out */
    bool ok = *(volatile int *)&abort_s == 0;
#pragma unroll
    for (int n = 0; n < 5; n++) {
      /* the window's older planes were waited for in earlier iterations:
       * only the first iteration waits for all five */
      int rel = rtop - 4 + n;
      if (ok && (it == 0 || n == 4)) ok = wait_full(&full_w[rel % NB], (rel / NB) & 1, a.err, lim);
    }
    if (ok) ok = wait_full(&full_s[it % NS], (it / NS) & 1, a.err, lim);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) abort_s = 1;
      break;
    }
    Win w;
    {
      int b = (rtop - 4) % NB;
      w.p0 = ring + b * PLANE; b = b + 1 == NB ? 0 : b + 1;
      w.p1 = ring + b * PLANE; b = b + 1 == NB ? 0 : b + 1;
      w.p2 = ring + b * PLANE; b = b + 1 == NB ? 0 : b + 1;
      w.p3 = ring + b * PLANE; b = b + 1 == NB ? 0 : b + 1;
      w.p4 = ring + b * PLANE;
    }
    const float *cen = w.at(ZC);
    const float *st = slots + (it % NS) * SLOT;

    if (valid) {
      const long long q = (long long)(i + g.xoff) + (long long)j * px +
                          (long long)k * sl;
      const float *ms = st + S_MET + sp;
      float xix = ms[0 * PTS], xiy = ms[1 * PTS], xiz = ms[2 * PTS];
      float etx = ms[3 * PTS], ety = ms[4 * PTS], etz = ms[5 * PTS];
      float ztx = ms[6 * PTS], zty = ms[7 * PTS], ztz = ms[8 * PTS];
      const MedPt m = med_from<MED, false>(st + S_MED + sp, PTS);
      const float slw = m.slw;
      float r[9];
#define DX(c) sdop<BX>(cen + soff(c, row, col), 1)
#define DY(c) sdop<BY>(cen + soff(c, row, col), BW)
#define DZ(c) zdop<BZ>(w, soff(c, row, col))
      {
        float DxTxx = DX(C_TXX), DyTxx = DY(C_TXX), DzTxx = DZ(C_TXX);
        float DxTxy = DX(C_TXY), DyTxy = DY(C_TXY), DzTxy = DZ(C_TXY);
        float DxTxz = DX(C_TXZ), DyTxz = DY(C_TXZ), DzTxz = DZ(C_TXZ);
        r[C_VX] = slw * (xix * DxTxx + xiy * DxTxy + xiz * DxTxz +
                         etx * DyTxx + ety * DyTxy + etz * DyTxz +
                         ztx * DzTxx + zty * DzTxy + ztz * DzTxz);
        float DxTyy = DX(C_TYY), DyTyy = DY(C_TYY), DzTyy = DZ(C_TYY);
        float DxTyz = DX(C_TYZ), DyTyz = DY(C_TYZ), DzTyz = DZ(C_TYZ);
        r[C_VY] = slw * (xix * DxTxy + xiy * DxTyy + xiz * DxTyz +
                         etx * DyTxy + ety * DyTyy + etz * DyTyz +
                         ztx * DzTxy + zty * DzTyy + ztz * DzTyz);
        float DxTzz = DX(C_TZZ), DyTzz = DY(C_TZZ), DzTzz = DZ(C_TZZ);
        r[C_VZ] = slw * (xix * DxTxz + xiy * DxTyz + xiz * DxTzz +
                         etx * DyTxz + ety * DyTyz + etz * DyTzz +
                         ztx * DzTxz + zty * DzTyz + ztz * DzTzz);
      }
      {
        float DxVx = DX(C_VX), DyVx = DY(C_VX);
        float DxVy = DX(C_VY), DyVy = DY(C_VY);
        float DxVz = DX(C_VZ), DyVz = DY(C_VZ);
        float DzVx, DzVy, DzVz;
        const int nk2 = g.nk2;
        if (a.free_top && k >= nk2 - 2) {
          if (k == nk2) {
            long long ij = ((long long)i + (long long)j * g.nx) * 9;
            const float *A = a.mVx + ij, *Bm = a.mVy + ij;
            DzVx = LDG(A + 0) * DxVx + LDG(A + 1) * DxVy + LDG(A + 2) * DxVz +
                   LDG(Bm + 0) * DyVx + LDG(Bm + 1) * DyVy + LDG(Bm + 2) * DyVz;
            DzVy = LDG(A + 3) * DxVx + LDG(A + 4) * DxVy + LDG(A + 5) * DxVz +
                   LDG(Bm + 3) * DyVx + LDG(Bm + 4) * DyVy + LDG(Bm + 5) * DyVz;
            DzVz = LDG(A + 6) * DxVx + LDG(A + 7) * DxVy + LDG(A + 8) * DxVz +
                   LDG(Bm + 6) * DyVx + LDG(Bm + 7) * DyVy + LDG(Bm + 8) * DyVz;
            if (MED != MED_VTI && MED != MED_ANI && a.VS) {
              /* surface force: matF2Vz (VxSrc, VySrc, VzSrc)
               * (forward/sv_curv_col_el_iso.c:583-592) */
              const long long n2 = (long long)g.nx * g.ny, i2 = i + (long long)j * g.nx;
              const float vx = a.VS[i2], vy = a.VS[n2 + i2], vz = a.VS[2 * n2 + i2];
              const float *F = a.mF + ij;
              DzVx += LDG(F + 0) * vx + LDG(F + 1) * vy + LDG(F + 2) * vz;
              DzVy += LDG(F + 3) * vx + LDG(F + 4) * vy + LDG(F + 5) * vz;
              DzVz += LDG(F + 6) * vx + LDG(F + 7) * vy + LDG(F + 8) * vz;
            }
          } else if (k == nk2 - 1) {
            const float *lo = BZ == 0 ? w.at(ZC) : w.at(ZC - 1);
            const float *hi = BZ == 0 ? w.at(ZC + 1) : w.at(ZC);
            int ox = soff(C_VX, row, col), oy = soff(C_VY, row, col),
                oz = soff(C_VZ, row, col);
            DzVx = -lo[ox] + hi[ox];
            DzVy = -lo[oy] + hi[oy];
            DzVz = -lo[oz] + hi[oz];
          } else {
            const float c0 = BZ == 0 ? (float)(-7.0 / 6.0) : (float)(1.0 / 6.0);
            const float c1 = BZ == 0 ? (float)(8.0 / 6.0) : (float)(-8.0 / 6.0);
            const float c2 = BZ == 0 ? (float)(-1.0 / 6.0) : (float)(7.0 / 6.0);
            const float *p0 = BZ == 0 ? w.at(ZC) : w.at(ZC - 2);
            const float *p1 = BZ == 0 ? w.at(ZC + 1) : w.at(ZC - 1);
            const float *p2 = BZ == 0 ? w.at(ZC + 2) : w.at(ZC);
            int ox = soff(C_VX, row, col), oy = soff(C_VY, row, col),
                oz = soff(C_VZ, row, col);
            DzVx = c0 * p0[ox] + c1 * p1[ox] + c2 * p2[ox];
            DzVy = c0 * p0[oy] + c1 * p1[oy] + c2 * p2[oy];
            DzVz = c0 * p0[oz] + c1 * p1[oz] + c2 * p2[oz];
          }
        } else {
          DzVx = DZ(C_VX);
          DzVy = DZ(C_VY);
          DzVz = DZ(C_VZ);
        }
        hooke9<MED>(m, xix, xiy, xiz, etx, ety, etz, ztx, zty, ztz, DxVx, DxVy,
                    DxVz, DyVx, DyVy, DyVz, DzVx, DzVy, DzVz, r);
      }
      if (a.free_top && k >= g.nk2 - (BZ == 0 ? 3 : 1)) {
        float tx = 0.f, ty = 0.f, tz = 0.f;
        if (a.TS) {
          const long long n2 = (long long)g.nx * g.ny, i2 = i + (long long)j * g.nx;
          tx = a.TS[i2]; ty = a.TS[n2 + i2]; tz = a.TS[2 * n2 + i2];
        }
        r[C_VX] = stimg_row<BX, BY, BZ>(a, w, cen, row, col, q, k, 0, tx);
        r[C_VY] = stimg_row<BX, BY, BZ>(a, w, cen, row, col, q, k, 1, ty);
        r[C_VZ] = stimg_row<BX, BY, BZ>(a, w, cen, row, col, q, k, 2, tz);
      }

      /* CFS-PML, faces in the reference order x1, x2, y1, y2, z1, z2 */
      if (pmask) {
        /* unrolled over the faces: every face parameter is a static
         * operand of the kernel's parameter space */
#pragma unroll
        for (int f = 0; f < CGFD_NFACE; f++) {
          if (!(pmask & (1 << f))) continue;
          const DevFace &F = a.face[f];
          AuxPt<KIND> pax;
          load_aux<KIND>(a, f, aux_index<KIND>(F, i, j, k), pax);
          float d[9];
          if (f < 2) {
#pragma unroll
            for (int c = 0; c < 9; c++) d[c] = DX(c);
            spml_face<KIND, MED>(a, f, i, j, k, q, d, xix, xiy, xiz, ztx, zty, ztz, m, pax, r);
          } else if (f < 4) {
#pragma unroll
            for (int c = 0; c < 9; c++) d[c] = DY(c);
            spml_face<KIND, MED>(a, f, i, j, k, q, d, etx, ety, etz, ztx, zty, ztz, m, pax, r);
          } else {
#pragma unroll
            for (int c = 0; c < 9; c++) d[c] = DZ(c);
            spml_face<KIND, MED>(a, f, i, j, k, q, d, ztx, zty, ztz, ztx, zty, ztz, m, pax, r);
          }
        }
      }
#undef DX
#undef DY
#undef DZ

      /* GMB attenuation (forward/sv_curv_col_vis_iso.c:250-347) */
      float hJ[MED == MED_VIS ? 6 * CGFD_VIS_NMW_MAX : 1];
      if (MED == MED_VIS) {
        float ev[6];
        vis_strain_rate(m.lam, m.mu, r, ev);
        float sl_ = 0.f, sm_[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const int nyl = 3, nym = 3 + a.nmw;
#pragma unroll
        for (int n = 0; n < CGFD_VIS_NMW_MAX; n++) {
          if (n < a.nmw) {
            const float *jc = st + S_JC + 6 * n * PTS + sp;
            const float yl = st[S_MED + (nyl + n) * PTS + sp];
            const float ym = st[S_MED + (nym + n) * PTS + sp];
            float J[6];
#pragma unroll
            for (int c = 0; c < 6; c++) {
              J[c] = jc[c * PTS];
              hJ[6 * n + c] = a.wl[n] * (ev[c] - J[c]);
              sm_[c] += ym * J[c];
            }
            sl_ += yl * (J[0] + J[1] + J[2]);
          }
        }
        const float lsl = m.lam * sl_, mu2 = 2.0f * m.mu;
        r[C_TXX] -= lsl + mu2 * sm_[0];
        r[C_TYY] -= lsl + mu2 * sm_[1];
        r[C_TZZ] -= lsl + mu2 * sm_[2];
        r[C_TYZ] -= mu2 * sm_[3];
        r[C_TXZ] -= mu2 * sm_[4];
        r[C_TXY] -= mu2 * sm_[5];
      }

      if (src_e0 < src_e1) {
        int itg = *a.d_it;
        for (int e = src_e0; e < src_e1; e++) {
          SrcEntry s = a.src_ent[e];
          if (s.k != k) continue;
          if (itg < a.src_it_begin[s.is] || itg > a.src_it_end[s.is]) continue;
          long long t = ((long long)s.is * a.src_max_nt +
                         (itg - a.src_it_begin[s.is])) * a.src_max_stage + a.istage;
          if (a.src_force && s.force_on) {
            r[C_VX] += a.Fx[t] * s.vf;
            r[C_VY] += a.Fy[t] * s.vf;
            r[C_VZ] += a.Fz[t] * s.vf;
          }
          if (a.src_moment) {
            r[C_TXX] -= a.Mxx[t] * s.rjac;
            r[C_TYY] -= a.Myy[t] * s.rjac;
            r[C_TZZ] -= a.Mzz[t] * s.rjac;
            r[C_TXZ] -= a.Mxz[t] * s.rjac;
            r[C_TYZ] -= a.Myz[t] * s.rjac;
            r[C_TXY] -= a.Mxy[t] * s.rjac;
          }
        }
      }
      if (dd_e0 < dd_e1) {
        /* distributed sources after the others (forward/sv_curv_col_el.c:
         * 487-590), while the step is below dd_max_nt */
        const int itg = *a.d_it;
        if (itg < a.dd_max_nt) {
          const long long t0 = ((long long)itg * 4 + a.istage) * a.dd_n;
          for (int e = dd_e0; e < dd_e1; e++) {
            SrcEntry s = a.dd_ent[e];
            if (s.k != k) continue;
            const long long t = t0 + s.is;
            if (a.dd_vi) {
              r[C_VX] += a.dd_vi[3 * t + 0] * s.vf;
              r[C_VY] += a.dd_vi[3 * t + 1] * s.vf;
              r[C_VZ] += a.dd_vi[3 * t + 2] * s.vf;
            }
            if (a.dd_mij) {
              r[C_TXX] -= a.dd_mij[6 * t + 0] * s.rjac;
              r[C_TYY] -= a.dd_mij[6 * t + 1] * s.rjac;
              r[C_TZZ] -= a.dd_mij[6 * t + 2] * s.rjac;
              r[C_TYZ] -= a.dd_mij[6 * t + 3] * s.rjac;
              r[C_TXZ] -= a.dd_mij[6 * t + 4] * s.rjac;
              r[C_TXY] -= a.dd_mij[6 * t + 5] * s.rjac;
            }
          }
        }
      }

      /* RK combine; the last stage also applies the Graves Q factor
       * (forward/drv_rk_curv_col.c:408-416: end += b dt rhs, then end *= Qatt) */
      float qa = 1.0f;
      const bool graves = KIND == 2 && a.qatt != nullptr;
      if (graves) qa = __ldg(a.qatt + q);
#pragma unroll
      for (int c = 0; c < 9; c++) {
        long long x = c * vol + q;
        if (KIND == 0) {
          float p = cen[soff(c, row, col)];
          a.tmp_out[x] = p + a.ca * r[c];
          a.end[x] = p + a.cb * r[c];
        } else if (KIND == 1) {
          a.tmp_out[x] = st[S_PRE + c * PTS + sp] + a.ca * r[c];
          a.end[x] = st[S_END + c * PTS + sp] + a.cb * r[c];
        } else {
          float v = st[S_END + c * PTS + sp] + a.cb * r[c];
          a.end[x] = graves ? v * qa : v;
        }
      }
      if (MED == MED_VIS) {
        /* memory variables: RK combine (pre/end read directly) */
#pragma unroll
        for (int n = 0; n < CGFD_VIS_NMW_MAX; n++) {
          if (n < a.nmw) {
            float pv[6], ev[6];
#pragma unroll
            for (int c = 0; c < 6; c++) {
              long long x = (long long)(9 + 6 * n + c) * vol + q;
              if (KIND == 0) pv[c] = st[S_JC + (6 * n + c) * PTS + sp];
              else if (KIND == 1) pv[c] = __ldg(a.pre + x);
              if (KIND >= 1) ev[c] = a.end[x];
            }
#pragma unroll
            for (int c = 0; c < 6; c++) {
              long long x = (long long)(9 + 6 * n + c) * vol + q;
              float h = hJ[6 * n + c];
              if (KIND == 0) {
                a.tmp_out[x] = pv[c] + a.ca * h;
                a.end[x] = pv[c] + a.cb * h;
              } else if (KIND == 1) {
                a.tmp_out[x] = pv[c] + a.ca * h;
                a.end[x] = ev[c] + a.cb * h;
              } else {
                a.end[x] = ev[c] + a.cb * h;
              }
            }
          }
        }
      }
    }

    /* release the oldest window plane and this plane's stream slot */
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&empty_w[(rtop - 4) % NB]);
      mbar_arrive(&empty_s[it % NS]);
    }
  }
}

/* the stage of one problem: grid (tiles_x, tiles_y, k chunks) */
template <int BX, int BY, int BZ, int KIND, int MED>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_stage3(const __grid_constant__ StageArgs a,
             const __grid_constant__ CUtensorMap tmap,
             const __grid_constant__ CUtensorMap tmap_met,
             const __grid_constant__ CUtensorMap tmap_med,
             const __grid_constant__ CUtensorMap tmap_pt,
             const __grid_constant__ CUtensorMap tmap_j)
{
  stage3_body<BX, BY, BZ, KIND, MED>(a, tmap, tmap_met, tmap_med, tmap_pt, tmap_j,
                                     blockIdx.x, blockIdx.y, blockIdx.z, false);
}

/* The same stage for a batch of independent shots in one launch: a 1-D
 * index space over every shot's CTAs, shot s owning [geo[s].cta0,
 * geo[s+1].cta0); each item reads its shot's arguments and tensor maps from
 * global memory.  All shots share the step's operator biases and RK stage.
 *
 * Two schedules.  next == null: one CTA per item (grid = nitems), item =
 * blockIdx.x.  next != null: persistent -- a CTA per SM takes items from
 * the global counter *next (zeroed before the launch) in the order of
 * order[] (largest first), runs the stage body on each, re-initialising its
 * barriers between items, and stops after its shot's error word is set. */
template <int BX, int BY, int BZ, int KIND, int MED>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_stage3_batch(const StageArgs *__restrict__ args,
                   const ShotGeo *__restrict__ geo, int nshot,
                   const int *__restrict__ order, int nitems, int *next)
{
  /* the shot's arguments in shared memory where the CTA's 227 KB allow
   * it: the stage reads them all through its loops, and shared loads are
   * cheaper than re-reading global memory.  The body reads the tile
   * geometry from them before its own first barrier, so the copy
   * completes first. */
  constexpr bool kArgsInSmem =
      Slot<MED>::SMEM_BYTES + (int)sizeof(StageArgs) + 256 <= 232448;
  __shared__ int item_s;
  int shot_cur = -1;
  for (int round = 0;; round++) {
    if (next) {
      if (threadIdx.x == 0) {
        const bool stop = round > 0 && *(volatile const int *)args[shot_cur].err != 0;
        item_s = stop ? nitems : atomicAdd(next, 1);
      }
      __syncthreads();
    } else if (round > 0) {
      break;
    }
    const int w = next ? item_s : (int)blockIdx.x;
    if (w >= nitems) break;
    const int cta = order ? order[w] : w;
    int lo = 0, hi = nshot - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (geo[mid].cta0 <= cta) lo = mid; else hi = mid - 1;
    }
    const ShotGeo &G = geo[lo];
    int c = cta - G.cta0;
    const int bx = c % G.tiles_x;
    c /= G.tiles_x;
    const int by = c % G.tiles_y;
    const int bz = c / G.tiles_y;
    if constexpr (kArgsInSmem) {
      __shared__ __align__(16) StageArgs sa;
      if (lo != shot_cur) {
        const int n4 = (int)(sizeof(StageArgs) / 4);
        const uint32_t *src = reinterpret_cast<const uint32_t *>(args + lo);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sa);
        for (int t = threadIdx.x; t < n4; t += blockDim.x) dst[t] = src[t];
      }
      __syncthreads();
      stage3_body<BX, BY, BZ, KIND, MED>(sa, G.wav, G.met, G.med, G.pt, G.j, bx, by,
                                         bz, true, round > 0);
    } else {
      stage3_body<BX, BY, BZ, KIND, MED>(args[lo], G.wav, G.met, G.med, G.pt, G.j,
                                         bx, by, bz, true, round > 0);
    }
    shot_cur = lo;
    /* every thread is done with the item, its barriers and its arguments */
    __syncthreads();
  }
}

}  // namespace s3

#endif
