// tile2d.cuh - persistent, asynchronously pipelined fused step kernel for
// 2D batches.
//
// Every CTA (256 threads) walks tiles of 64 (z) x 32 (x) outputs across all
// shots of the batch.  While it computes tile k from one shared-memory stage,
// the next tile's inputs are already in flight into the other stage through
// cp.async (16-byte global->shared copies that hold no registers):
//   u2 (and vel for the adjoint) with a 4-cell halo, 72 x 40 floats;
//   u1, u0, u_1 (and vel for the forward stencil), 64 x 32 floats each.
// The CTA's tile list and the batch's compact shot descriptors are copied
// to shared memory once, so the loop issues no dependent global loads.  Each
// thread computes 4 consecutive z rows in two columns from shared memory
// with 128-bit reads, packed FP32 pair arithmetic (f32x2.cuh) and 128-bit
// stores of u3.  Work only a few tiles have (injection boxes, snapshot and
// imaging steps) is decided once per tile.  The floating-point operation
// order is the reference's (see batch.cu).
#pragma once

#include "batch.cuh"
#include "f32x2.cuh"

namespace swave {

constexpr int T2_Z = 64, T2_X = 32;
constexpr int T2_SZ = T2_Z + 8;          // staged column length (with halo)
constexpr int T2_SX = T2_X + 8;          // staged columns (with halo)
constexpr int T2_HALO = T2_SX * T2_SZ;   // 2880 floats
constexpr int T2_CORE = T2_X * T2_Z;     // 2048 floats
constexpr int T2_MAX_TILES_PER_CTA = 320;

// Floats of one pipeline stage.
template <bool ADJ>
__host__ __device__ constexpr int t2_stage_floats() {
  return ADJ ? 2 * T2_HALO + 3 * T2_CORE : T2_HALO + 4 * T2_CORE;
}
// Per-step scalars of one shot, computed once per CTA and launch.
struct T2Step {
  int it;              // time sample of the step
  int live;            // the shot steps in this launch with this stencil variant
  int snap;            // snapshot step with snapshot or imaging work
  int extract;         // save the snapshot this step
  int img;             // RTM (1), LSRTM (2) or AFWI (3) imaging this step, else 0
  float dt2snap;       // AFWI: (dt snapi)^2
  float *wsave;        // snapshot slot written this step
  const float *wimg;   // snapshot slot read by the imaging
  float *image, *illum;
  const float *taperx; // null: no taper
  float tapery0;
};

// One thread's imaging inputs for a tile (2 columns x 4 rows), loaded before
// the tile's stage is waited for so that their latency overlaps the wait.
struct T2Img {
  float w[2][4], im[2][4], il[2][4];
};

// Dynamic shared memory: two stages, the shot table, the per-step scalars,
// the tile list and two mbarriers.
template <bool ADJ>
__host__ __device__ constexpr size_t t2_smem_bytes() {
  return 2 * sizeof(float) * t2_stage_floats<ADJ>() + sizeof(T2Shot) * T2_MAX_SHOTS +
         sizeof(T2Step) * T2_MAX_SHOTS + sizeof(int) * (T2_MAX_TILES_PER_CTA + 8) + 64;
}

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
// Programmatic dependent launch: wait for the grids this one depends on to
// complete (and their writes to be visible); allow the next grid in the
// stream to start its own prologue.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Orders this thread's generic-proxy shared-memory writes before later
// tensor copies (async proxy) into the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for a phase of an mbarrier: false after T2_WAIT_LIMIT polls
// (each poll may suspend the thread for a while), so a copy that never
// completes ends the kernel with an error status instead of a hang.
constexpr int T2_WAIT_LIMIT = 1 << 22;
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
  for (int q = 0; q < T2_WAIT_LIMIT; ++q)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// 2D tensor copy global -> shared memory, completing on an mbarrier.
__device__ __forceinline__ void tma_2d(float *dst, const CUtensorMap *map, int x, int y,
                                       unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ int t2_b(int e) { return e >> 24; }
__device__ __forceinline__ int t2_tzi(int e) { return (e >> 12) & 0xfff; }
__device__ __forceinline__ int t2_txi(int e) { return e & 0xfff; }
// First row / column of a tile.
__device__ __forceinline__ int t2_z0(const T2Shot &h, int e) {
  return h.nmin1 - h.off1 + t2_tzi(e) * T2_Z;
}
__device__ __forceinline__ int t2_x0(const T2Shot &h, int e) {
  return h.nmin2 - h.off2 + t2_txi(e) * T2_X;
}

// Issues the tensor copies of one tile into a stage (one thread).  Tensor
// map 2*buf+0 has the 72 x 40 halo box, 2*buf+1 the 64 x 32 core box; buf
// 0..4 are the shot's time-level buffers, 5 its velocity.  Halo coordinates
// are row z0-4 and column x0-4 relative to the padded array's origin (4
// cells before the compute domain), so they may be negative for the first
// tiles; elements outside the array read 0 and only feed outputs that are
// never stored.  The row coordinate is a multiple of 4 (16 bytes).
// The copies split in two: t2_issue_old (the whole stage's byte count,
// then every input that older launches wrote: u1, u0, u_1 and the
// velocity) and t2_issue_u2 (u2, the level the previous launch writes).
template <bool ADJ>
__device__ __forceinline__ void t2_issue_old(const T2Maps &M, const T2Shot &h, int s, int e,
                                             float *st, unsigned long long *bar) {
  constexpr unsigned bytes = 4u * (unsigned)t2_stage_floats<ADJ>();
  const int zi = t2_tzi(e) * T2_Z - h.off1, xi = t2_txi(e) * T2_X - h.off2;
  mbar_expect_tx(bar, bytes);
  if (ADJ) tma_2d(st + T2_HALO, &M.m[10], zi, xi, bar);
  float *cst = st + (ADJ ? 2 : 1) * T2_HALO;
  tma_2d(cst, &M.m[2 * ((s + 2) % 5) + 1], zi + 4, xi + 4, bar);
  tma_2d(cst + T2_CORE, &M.m[2 * ((s + 1) % 5) + 1], zi + 4, xi + 4, bar);
  tma_2d(cst + 2 * T2_CORE, &M.m[2 * (s % 5) + 1], zi + 4, xi + 4, bar);
  if (!ADJ) tma_2d(cst + 3 * T2_CORE, &M.m[11], zi + 4, xi + 4, bar);
}
template <bool ADJ>
__device__ __forceinline__ void t2_issue_u2(const T2Maps &M, const T2Shot &h, int s, int e,
                                            float *st, unsigned long long *bar) {
  const int zi = t2_tzi(e) * T2_Z - h.off1, xi = t2_txi(e) * T2_X - h.off2;
  tma_2d(st, &M.m[2 * ((s + 3) % 5)], zi, xi, bar);
}
template <bool ADJ>
__device__ __forceinline__ void t2_issue(const T2Maps &M, const T2Shot &h, int s, int e,
                                         float *st, unsigned long long *bar) {
  t2_issue_old<ADJ>(M, h, s, e, st, bar);
  t2_issue_u2<ADJ>(M, h, s, e, st, bar);
}

__device__ __forceinline__ float f4get(const float4 &a, int e) {
  return e == 0 ? a.x : e == 1 ? a.y : e == 2 ? a.z : a.w;
}

// Born source and AFWI imaging of one element on a snapshot step (the
// imaging modes the vectorised t2_snap_col path does not cover).
__device__ __noinline__ float t2_snap_generic(const ShotDev &S, int it, int i, int j, float se,
                                              float u2c, float vc) {
  const Geom &g = S.g;
  if (i < 1 || i > g.nz || j < 1 || j > g.nx) return se;
  const long long nphys = (long long)g.nz * g.nx;
  const long long pp = (long long)(i - 1) + (long long)g.nz * (j - 1);
  const float taper = S.taperx ? S.taperx[j - 1] * S.tapery[0] : 1.f;
  const int cnt = S.tstep > 0 ? it / S.snapi - (S.tcnt - 1) / S.snapi
                              : S.tcnt / S.snapi - (it - 1) / S.snapi;
  // Rows above a free surface: stored as zero, no Born source or imaging.
  const bool below = i >= S.irow0;
  // Injection_Born (Imaging.f90:747-788).
  if (S.imaging == 4 && S.tstep > 0 && below && cnt <= S.ntsnap)
    se = se + (((2.0f * taper) * S.ref[pp]) * S.wave[(long long)(cnt - 1) * nphys + pp]) / vc;
  // Extraction_wavefield (Extraction.f90:562-601).
  if (S.extract_wave && cnt <= S.ntsnap)
    S.wave[(long long)(cnt - 1) * nphys + pp] = below ? u2c : 0.f;
  if (S.imaging == 3 && S.tstep < 0 && below) {
    const int index = S.ntsnap - cnt + 1;
    if (index >= 1) {
      const float wsn = S.wave[(long long)(index - 1) * nphys + pp];
      const int ip1 = min(index + 1, S.ntsnap), im1 = max(index - 1, 1);
      const float tt = ((S.wave[(long long)(im1 - 1) * nphys + pp] - 2.0f * wsn) +
                        S.wave[(long long)(ip1 - 1) * nphys + pp]) /
                       (S.dt2snap * ((vc * vc) * vc));
      S.image[pp] = S.image[pp] + (u2c * tt) * taper;             // Imaging.f90:410-411
      S.illum[pp] = S.illum[pp] + (wsn * wsn) * taper;
    }
  }
  return se;
}

__device__ __forceinline__ float4 lds4(const float *p) {
  return *reinterpret_cast<const float4 *>(p);
}

// Constants of a shot used by the packed arithmetic.
struct T2Pairs {
  float cz[5], cx[5], k12;
  P2 div11;
};

__device__ __forceinline__ T2Pairs t2_pairs(const T2Shot &h) {
  T2Pairs c;
  c.cz[0] = h.c0z; c.cz[1] = h.c1z; c.cz[2] = h.c2z; c.cz[3] = h.c3z; c.cz[4] = h.c4z;
  c.cx[0] = h.c0x; c.cx[1] = h.c1x; c.cx[2] = h.c2x; c.cx[3] = h.c3x; c.cx[4] = h.c4x;
  c.k12 = h.k12;
  c.div11 = p2s(h.div11);
  return c;
}

// Whether a tile overlaps the physical domain.
__device__ __forceinline__ bool t2_phys_tile(const T2Shot &h, int e) {
  const int z0 = t2_z0(h, e), x0 = t2_x0(h, e);
  return !(z0 + T2_Z - 1 < 1 || z0 > h.nz || x0 + T2_X - 1 < 1 || x0 > h.nx);
}

// Physical-domain tests of one thread's rows and columns.
__device__ __forceinline__ bool t2_row_ok(const T2Shot &h, int i) { return i >= 1 && i <= h.nz; }
__device__ __forceinline__ bool t2_col_ok(const T2Shot &h, int j) { return j >= 1 && j <= h.nx; }

// Snapshot and imaging work use a row mapping of their own: thread (tz, tx)
// handles rows z0+tz+16m (m = 0..3) of columns x0+tx and x0+tx+16, so that
// every global load and store of a warp covers 16 consecutive floats of a
// column.  Their inputs (u2 and the velocity) are read from the staged tile.

// Loads the snapshot, image and illumination values of a thread's elements
// for an imaging step (zeros outside the physical domain).
__device__ __forceinline__ void t2_img_load(const T2Shot &h, const T2Step &stp, int e, T2Img &P,
                                            int tid) {
  const int z0 = t2_z0(h, e), x0 = t2_x0(h, e);
  const int tz = tid & 15, tx = tid >> 4;
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int j = x0 + tx + 16 * hh;
    const long long pc = (long long)h.nz * (j - 1) - 1;   // pp = pc + i
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int i = z0 + tz + 16 * m;
      const bool ok = t2_col_ok(h, j) && t2_row_ok(h, i);
      P.w[hh][m] = ok ? stp.wimg[pc + i] : 0.f;
      P.im[hh][m] = ok ? stp.image[pc + i] : 0.f;
      P.il[hh][m] = ok ? stp.illum[pc + i] : 0.f;
    }
  }
}

// Snapshot saving (Extraction.f90:562-601) and RTM / LSRTM / AFWI imaging
// (Imaging.f90:265 and 735) of a thread's elements; su is the staged u2 halo
// tile and svel the staged velocity: the halo tile for the adjoint stencil,
// the core tile (column stride T2_Z) for the forward one (the backward pass
// of CHEAP_LSRTM images on the forward grid).  The operations are those of
// the element-by-element path.
template <bool ADJ>
__device__ __forceinline__ void t2_snap_tile(const T2Shot &h, const T2Step &stp, const T2Img &P,
                                             int e, const float *su, const float *svel, int tid) {
  const int z0 = t2_z0(h, e), x0 = t2_x0(h, e);
  const int tz = tid & 15, tx = tid >> 4;
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int jl = tx + 16 * hh, j = x0 + jl;
    if (!t2_col_ok(h, j)) continue;
    const long long pc = (long long)h.nz * (j - 1) - 1;
    const float taper = stp.taperx ? stp.taperx[j - 1] * stp.tapery0 : 1.f;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int r = tz + 16 * m, i = z0 + r;
      if (!t2_row_ok(h, i)) continue;
      // Under a free surface the rows above it are stored as zero and take
      // no imaging (Extraction.f90:580-592, Imaging.f90:248-258).
      const bool below = i >= h.irow0;
      const float u = su[(jl + 4) * T2_SZ + 4 + r];
      if (stp.extract) stp.wsave[pc + i] = below ? u : 0.f;
      if (stp.img && below) {
        const float wsn = P.w[hh][m];
        float im = P.im[hh][m];
        if (stp.img == 1) {
          im = im + (u * wsn) * taper;
        } else if (stp.img == 2) {
          const float v = ADJ ? svel[(jl + 4) * T2_SZ + 4 + r] : svel[jl * T2_Z + r];
          im = im + (((2.0f * taper) * u) * wsn) / v;
        } else {
          // AFWI (Imaging.f90:410-411): second time difference of the
          // snapshots over v^3.
          const float v = ADJ ? svel[(jl + 4) * T2_SZ + 4 + r] : svel[jl * T2_Z + r];
          const long long np = (long long)h.nz * h.nx;
          const float *wm = stp.wimg - ((stp.img & 16) ? np : 0);
          const float *wp = stp.wimg + ((stp.img & 32) ? np : 0);
          const float tt = ((wm[pc + i] - 2.0f * wsn) + wp[pc + i]) / (stp.dt2snap * ((v * v) * v));
          im = im + (u * tt) * taper;
        }
        stp.image[pc + i] = im;
        stp.illum[pc + i] = P.il[hh][m] + (wsn * wsn) * taper;
      }
    }
  }
}

// Laplacian part of rows i0..i0+3 of two adjacent columns jl0, jl0+1 of a
// tile, away from the edges of the compute domain, as row pairs.  The ten
// columns jl0-4..jl0+5 at rows i0..i0+3 are read once and serve the x
// derivatives of both columns.  col0 points at row i0 of column jl0 of the
// staged u2 tile, vcol0 at the same place of the staged velocity halo
// (adjoint), vcore0 at row i0 of column jl0 of the staged core velocity
// (forward).  u2c receives the raw u2 values of the two columns.  Per lane
// the operations are those of the scalar loops (FDderivatives.f90:715-743
// forward, 847-891 adjoint).
template <bool ADJ, bool PRE = false>
__device__ __forceinline__ void t2_pair_fast(const T2Pairs &c, const float *col0,
                                             const float *vcol0, const float *vcore0,
                                             P2 sv[2][2], float4 u2c[2]) {
  float4 N[10];
  if (PRE) {
    // vcol0 points at the staged w = (v*v)*u of the tile (t2_premul).
    u2c[0] = lds4(col0);
    u2c[1] = lds4(col0 + T2_SZ);
#pragma unroll
    for (int m = 0; m < 10; ++m) N[m] = lds4(vcol0 + (m - 4) * T2_SZ);
  } else {
#pragma unroll
    for (int m = 0; m < 10; ++m) N[m] = lds4(col0 + (m - 4) * T2_SZ);
    u2c[0] = N[4];
    u2c[1] = N[5];
  }
  if (ADJ && !PRE) {
    // w = (v*v)*u at every stencil point (FDderivatives.f90:847-891).
#pragma unroll
    for (int m = 0; m < 10; ++m) {
      const float4 v = lds4(vcol0 + (m - 4) * T2_SZ);
      const P2 a = s_mul(p_mul(lo2(v), lo2(v)), lo2(N[m]));
      const P2 b = s_mul(p_mul(hi2(v), hi2(v)), hi2(N[m]));
      N[m] = make_float4(a.x, a.y, b.x, b.y);
    }
  }
#pragma unroll
  for (int cc = 0; cc < 2; ++cc) {
    const float *col = col0 + cc * T2_SZ;
    float4 za, zc;
    if (PRE) {
      const float *wcol = vcol0 + cc * T2_SZ;
      za = lds4(wcol - 4);
      zc = lds4(wcol + 4);
    } else {
      za = lds4(col - 4);
      zc = lds4(col + 4);
    }
    if (ADJ && !PRE) {
      const float *vcol = vcol0 + cc * T2_SZ;
      const float4 va = lds4(vcol - 4), vc = lds4(vcol + 4);
      const P2 a0 = s_mul(p_mul(lo2(va), lo2(va)), lo2(za));
      const P2 a1 = s_mul(p_mul(hi2(va), hi2(va)), hi2(za));
      const P2 c0 = s_mul(p_mul(lo2(vc), lo2(vc)), lo2(zc));
      const P2 c1 = s_mul(p_mul(hi2(vc), hi2(vc)), hi2(zc));
      za = make_float4(a0.x, a0.y, a1.x, a1.y);
      zc = make_float4(c0.x, c0.y, c1.x, c1.y);
    }
    const float4 zb = N[4 + cc];
    const P2 P[6] = {lo2(za), hi2(za), lo2(zb), hi2(zb), lo2(zc), hi2(zc)};
    // Pairs of rows (2k+1, 2k+2) for the odd z offsets.
    P2 Q[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) Q[k] = p2(P[k].y, P[k + 1].x);
    P2 tzz[2], txx[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      P2 a = s_mul(c.cz[0], P[2 + p]);
      a = p_add(a, s_mul(c.cz[1], p_add(Q[2 + p], Q[1 + p])));
      a = p_add(a, s_mul(c.cz[2], p_add(P[3 + p], P[1 + p])));
      a = p_add(a, s_mul(c.cz[3], p_add(Q[3 + p], Q[p])));
      a = p_add(a, s_mul(c.cz[4], p_add(P[4 + p], P[p])));
      tzz[p] = a;
      txx[p] = s_mul(c.cx[0], P[2 + p]);
    }
#pragma unroll
    for (int l = 1; l <= 4; ++l) {
      const float4 rp = N[4 + cc + l], rm = N[4 + cc - l];
      txx[0] = p_add(txx[0], s_mul(c.cx[l], p_add(lo2(rp), lo2(rm))));
      txx[1] = p_add(txx[1], s_mul(c.cx[l], p_add(hi2(rp), hi2(rm))));
    }
    if (ADJ) {
      sv[cc][0] = p_add(txx[0], tzz[0]);
      sv[cc][1] = p_add(txx[1], tzz[1]);
    } else {
      const float4 vv = lds4(vcore0 + cc * T2_Z);
      sv[cc][0] = p_mul(p_mul(lo2(vv), lo2(vv)), p_add(txx[0], tzz[0]));
      sv[cc][1] = p_mul(p_mul(hi2(vv), hi2(vv)), p_add(txx[1], tzz[1]));
    }
  }
}

// The adjoint stencil's w = (v*v)*u (FDderivatives.f90:847-891) over the
// whole staged u2 halo tile, written over the staged velocity halo: every
// staged value is squared and multiplied once per tile instead of once per
// stencil point that reads it.  Same operations, same roundings.  The
// caller synchronises before the tile is computed.
__device__ __forceinline__ void t2_premul(float *st, int tid, int nthreads) {
  const float4 *u = reinterpret_cast<const float4 *>(st);
  float4 *vw = reinterpret_cast<float4 *>(st + T2_HALO);
  for (int q = tid; q < T2_HALO / 4; q += nthreads) {
    const float4 v = vw[q], x = u[q];
    const P2 a = s_mul(p_mul(lo2(v), lo2(v)), lo2(x));
    const P2 b = s_mul(p_mul(hi2(v), hi2(v)), hi2(x));
    vw[q] = make_float4(a.x, a.y, b.x, b.y);
  }
}

// Whether an adjoint tile reads the staged velocity itself (LSRTM imaging,
// and the element-by-element snapshot work: AFWI imaging and the Born
// source); the others take the pre-multiplied w (t2_premul).
__device__ __forceinline__ bool t2_needs_vel(const T2Shot &h, const T2Step &stp, int e) {
  return stp.img == 2 || (stp.snap && h.imaging > 2 && t2_phys_tile(h, e));
}

// Computes one tile from a completed stage.  Thread (tz, tx) owns rows
// i0..i0+3 of the adjacent columns x0+2tx and x0+2tx+1.
template <bool ADJ>
__device__ __forceinline__ void t2_compute(const BatchTables &t, const T2Shot &h,
                                           const T2Step &stp, int b, int s, int e,
                                           const float *st, int tid, bool pre) {
  const int z0 = t2_z0(h, e), x0 = t2_x0(h, e);
  const int tz = tid & 15, tx = tid >> 4;
  const int i0 = z0 + 4 * tz;
  // Row groups outside the compute domain (the first tile starts off1, a
  // multiple of 4, rows early) compute nothing.
  if (i0 > h.nmax1 || i0 < h.nmin1) return;
  const int it = stp.it;
  // Tile-level decisions.
  const int zl = z0 + T2_Z - 1, xl = x0 + T2_X - 1;
  const bool inj_tile = h.inj_on && !(zl < h.bi0 || z0 > h.bi1 || xl < h.bj0 || x0 > h.bj1);
  const bool snap_tile = stp.snap && t2_phys_tile(h, e);
  // Snapshot saving and RTM / LSRTM / AFWI imaging take the vectorised path
  // after the update; injection and the Born source go element by element.
  const bool snap_fast = snap_tile && h.imaging <= 3;
  const bool snap_slow = snap_tile && !snap_fast;
  const bool slow_extras = inj_tile || snap_slow;
  const float *su = st;
  const float *svel = st + T2_HALO;                       // adjoint only
  const float *core = st + (ADJ ? 2 : 1) * T2_HALO;
  const T2Pairs c = t2_pairs(h);
  P2 sv[2][2];
  float4 u2c[2];
  // The adjoint reads v at every stencil point with indices clamped to the
  // compute domain (FDderivatives.f90:863-878).  The padded velocity
  // replicates the physical model's edge values outwards (k_pad_velocity)
  // and the compute domain contains the physical one, so the padded value at
  // any index equals the clamped lookup; no tile needs a special case.
  {
    const int o = (2 * tx + 4) * T2_SZ + 4 * tz + 4;
    if (ADJ && pre)
      t2_pair_fast<ADJ, true>(c, su + o, svel + o, nullptr, sv, u2c);
    else
      t2_pair_fast<ADJ, false>(c, su + o, svel + o, core + 3 * T2_CORE + 2 * tx * T2_Z + 4 * tz,
                               sv, u2c);
  }
  if (slow_extras) {
    const ShotDev &S = t.shots[b];
    const bool rows_inj = inj_tile && i0 + 3 >= h.bi0 && i0 <= h.bi1;
    if (rows_inj) {
      // Injection (Injection.f90:151-456,561-591): every cell adds the
      // step's terms of its entries (k_bterms) in entry order.  The offsets
      // and the first 4 terms of all 8 cells are loaded before any sum.
      int beg[2][4], end[2][4];
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int j = x0 + 2 * tx + hh;
        const bool cin = j >= h.bj0 && j <= h.bj1 && j >= h.nmin2 && j <= h.nmax2;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = i0 + q;
          beg[hh][q] = end[hh][q] = 0;
          if (cin && i >= h.bi0 && i <= h.bi1) {
            const int bx = (i - h.bi0) + (h.bi1 - h.bi0 + 1) * (j - h.bj0);
            beg[hh][q] = S.inj_off[bx];
            end[hh][q] = S.inj_off[bx + 1];
          }
        }
      }
      // Term of entry k: precomputed, or formed here for a shot with few
      // entries (its source), the same operations as k_bterms.
      auto term = [&](int k) {
        if (!h.inj_direct) return S.inj_term[k];
        const InjEntry E = S.inj_ent[k];
        const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
        return (((E.v2r * tr) * E.wz) * E.wx) * E.wy;
      };
      float tv[2][4][4];
#pragma unroll
      for (int hh = 0; hh < 2; ++hh)
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int m = 0; m < 4; ++m)
            tv[hh][q][m] = beg[hh][q] + m < end[hh][q] ? term(beg[hh][q] + m) : 0.f;
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        float r[4] = {sv[hh][0].x, sv[hh][0].y, sv[hh][1].x, sv[hh][1].y};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
          for (int m = 0; m < 4; ++m)
            if (beg[hh][q] + m < end[hh][q]) r[q] = r[q] + tv[hh][q][m];
          for (int k = beg[hh][q] + 4; k < end[hh][q]; ++k) r[q] = r[q] + term(k);
        }
        sv[hh][0] = p2(r[0], r[1]);
        sv[hh][1] = p2(r[2], r[3]);
      }
    }
    if (snap_slow) {
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int jl = 2 * tx + hh, j = x0 + jl;
        if (j > h.nmax2 || j < h.nmin2) continue;
        float r[4] = {sv[hh][0].x, sv[hh][0].y, sv[hh][1].x, sv[hh][1].y};
        const float *cc = core + jl * T2_Z + 4 * tz;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float vc = ADJ ? svel[(jl + 4) * T2_SZ + 4 * tz + 4 + q] : cc[3 * T2_CORE + q];
          r[q] = t2_snap_generic(S, it, i0 + q, j, r[q], f4get(u2c[hh], q), vc);
        }
        sv[hh][0] = p2(r[0], r[1]);
        sv[hh][1] = p2(r[2], r[3]);
      }
    }
  }
  // FD_2nd_time_derivative_grid (FDderivatives.f90:960-982).
  float *__restrict__ u3 = const_cast<float *>(h.f[(s + 4) % 5]);
  const int rbase = t2_tzi(e) * T2_Z - h.off1;   // row z0-4 relative to the padded origin
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int jl = 2 * tx + hh, j = x0 + jl;
    const float *cc = core + jl * T2_Z + 4 * tz;
    const float4 a1 = lds4(cc), a0 = lds4(cc + T2_CORE), am = lds4(cc + 2 * T2_CORE);
    P2 o[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      const P2 u = p ? hi2(u2c[hh]) : lo2(u2c[hh]);
      P2 a = s_mul(20.0f, u);
      a = p_sub(a, s_mul(6.0f, p ? hi2(a1) : lo2(a1)));
      a = p_sub(a, s_mul(4.0f, p ? hi2(a0) : lo2(a0)));
      a = p_add(a, p ? hi2(am) : lo2(am));
      a = p_add(a, s_mul(c.k12, sv[hh][p]));
      o[p] = p_mul(a, c.div11);
    }
    if (j > h.nmax2 || j < h.nmin2) continue;
    const int off = (rbase + 4 + 4 * tz) + h.ld1 * (j - h.lo2);
    if (i0 + 3 <= h.nmax1) {
      *reinterpret_cast<float4 *>(u3 + off) = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
    } else {
      const float ov[4] = {o[0].x, o[0].y, o[1].x, o[1].y};
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (i0 + q <= h.nmax1) u3[off + q] = ov[q];
    }
  }
}

// Barrier of the threads that compute a tile: the whole CTA (bar 0) or one
// 256-thread consumer group (named barrier bar).
__device__ __forceinline__ void t2_bar(int bar) {
  if (bar == 0) __syncthreads();
  else asm volatile("bar.sync %0, 256;" ::"r"(bar) : "memory");
}

// Higdon recurrence of one edge half line (Boundary_3d, Boundary.f90:89-184)
// from gathered values: U2[m], U1[m] (m = 0..9) run from 2 cells inside the
// innermost output to the outermost one; a and bq are u3 one and two cells
// inside it.  out[k] (k = 0..7) from the innermost cell outwards.
__device__ __forceinline__ void t2_higdon8(const float c[8], const float U2[10],
                                           const float U1[10], float a, float bq,
                                           float out[8]) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    float r = c[0] * a;
    r = r + c[1] * bq;
    r = r + c[2] * U2[k + 2];
    r = r + c[3] * U2[k + 1];
    r = r + c[4] * U2[k];
    r = r + c[5] * U1[k + 2];
    r = r + c[6] * U1[k + 1];
    r = r + c[7] * U1[k];
    out[k] = -r;
    bq = a;
    a = out[k];
  }
}

// Higdon edges of a tile at the boundary of the compute domain, after its
// interior values are stored: the z lines of its columns (top and / or
// bottom), then the x lines of its rows (left and / or right), the order of
// the reference (z before x).  Every value a line reads lies in this tile:
// u2 in the staged halo, u1 in the staged core, u3 just stored by this CTA.
template <bool ADJ>
__device__ __forceinline__ void t2_edges(const T2Shot &h, int s, int e, const float *st, int tid,
                                         int bar) {
  if (h.rigid) return;   // exact-adjoint mode: no absorbing boundary
  const int tzi = t2_tzi(e), txi = t2_txi(e);
  // A free surface does not absorb at the top (Boundary.f90:104-108).
  const bool top = tzi == 0 && !h.surf, bottom = tzi == h.ntz - 1;
  const bool left = txi == 0, right = txi == h.ntx - 1;
  if (!(top || bottom || left || right)) return;
  const int z0 = t2_z0(h, e), x0 = t2_x0(h, e);
  const float *su = st;                                   // u2, rows z0-4.., columns x0-4..
  const float *cu1 = st + (ADJ ? 2 : 1) * T2_HALO;        // u1, rows z0.., columns x0..
  float *u3 = const_cast<float *>(h.f[(s + 4) % 5]);
  const long long L = h.ld1;
  auto gidx = [&](int i, int j) {
    return (long long)(i - (h.nmin1 - 4)) + L * (long long)(j - h.lo2);
  };
  const int warp = tid >> 5, lane = tid & 31;
  const int n1 = h.nmax1 - h.nmin1 + 1, n2 = h.nmax2 - h.nmin2 + 1;
  t2_bar(bar);   // interior values of the tile are stored
  if (top || bottom) {
    // Warp 0: top z lines, warp 1: bottom z lines; lane = column.
    const bool mine = (warp == 0 && top) || (warp == 1 && bottom);
    const int j = x0 + lane;
    if (mine && j >= h.nmin2 && j <= h.nmax2) {
      const bool bot = warp == 1;
      const int dir = bot ? -1 : 1;                       // towards the interior
      const int p = bot ? h.nmax1 - 3 : h.nmin1 + 3;      // innermost output row
      float c[8], U2[10], U1[10], out[8];
      const float *gc = h.gz + (j - h.nmin2) + (bot ? 8 * n2 : 0);
#pragma unroll
      for (int q = 0; q < 8; ++q) c[q] = gc[q * n2];
#pragma unroll
      for (int m = 0; m < 10; ++m) {
        const int i = p - (m - 2) * dir;
        U2[m] = su[(lane + 4) * T2_SZ + (i - (z0 - 4))];
        U1[m] = cu1[lane * T2_Z + (i - z0)];
      }
      t2_higdon8(c, U2, U1, u3[gidx(p + dir, j)], u3[gidx(p + 2 * dir, j)], out);
#pragma unroll
      for (int k = 0; k < 8; ++k) u3[gidx(p - k * dir, j)] = out[k];
    }
  }
  t2_bar(bar);   // z lines done before the x lines read the corners
  if (left || right) {
    // Threads 0..63: left x lines, 64..127: right x lines; one row each.
    const bool rgt = tid >= 64;
    const bool mine = tid < 128 && ((!rgt && left) || (rgt && right));
    const int r = tid & 63, i = z0 + r;
    // Under a free surface the side lines start at row 1.
    if (mine && i >= (h.surf ? 1 : h.nmin1) && i <= h.nmax1) {
      const int dir = rgt ? -1 : 1;
      const int p = rgt ? h.nmax2 - 3 : h.nmin2 + 3;      // innermost output column
      float c[8], U2[10], U1[10], out[8];
      const float *gc = h.gx + (i - h.nmin1) + (rgt ? 8 * n1 : 0);
#pragma unroll
      for (int q = 0; q < 8; ++q) c[q] = gc[q * n1];
#pragma unroll
      for (int m = 0; m < 10; ++m) {
        const int j = p - (m - 2) * dir;
        U2[m] = su[(j - (x0 - 4)) * T2_SZ + (r + 4)];
        U1[m] = cu1[(j - x0) * T2_Z + r];
      }
      t2_higdon8(c, U2, U1, u3[gidx(i, p + dir)], u3[gidx(i, p + 2 * dir)], out);
#pragma unroll
      for (int k = 0; k < 8; ++k) u3[gidx(i, p - k * dir)] = out[k];
    }
  }
}

// Per-step scalars of shot b for step s of this launch.
template <bool ADJ>
__device__ __forceinline__ T2Step t2_step_of(const BatchTables &t, const T2Shot &h, int b, int s) {
  const ShotDev &S = t.shots[b];
  T2Step st;
  st.live = s < h.nsteps && (h.adj2d != 0) == ADJ;
  st.it = h.tmin + s * h.tstep;
  st.snap = (st.it % h.snapi) == 0 && (h.extract_wave || h.imaging != 0);
  const int cnt = h.tstep > 0 ? st.it / h.snapi - (h.tcnt - 1) / h.snapi
                              : h.tcnt / h.snapi - (st.it - 1) / h.snapi;
  const long long nphys = (long long)h.nz * h.nx;
  st.extract = st.snap && h.extract_wave && cnt <= S.ntsnap && h.imaging <= 2;
  st.wsave = st.extract ? S.wave + (long long)(cnt - 1) * nphys : nullptr;
  const int index = S.ntsnap - cnt + 1;
  st.img = (st.snap && h.imaging >= 1 && h.imaging <= 3 && h.tstep < 0 && index >= 1)
               ? h.imaging : 0;
  st.wimg = st.img ? S.wave + (long long)(index - 1) * nphys : nullptr;
  // AFWI reads the slots before and after (clamped to the first and last):
  // bit 4 of img when index - 1 >= 1, bit 5 when index + 1 <= ntsnap.
  if (st.img == 3) st.img |= (index > 1 ? 16 : 0) | (index < S.ntsnap ? 32 : 0);
  st.dt2snap = S.dt2snap;
  st.image = S.image;
  st.illum = S.illum;
  st.taperx = S.taperx;
  st.tapery0 = S.taperx ? S.tapery[0] : 1.f;
  return st;
}

template <bool ADJ>
__device__ __forceinline__ void tile2d_persistent(const BatchTables &t, int s_off, int n_tiles) {
  extern __shared__ __align__(128) float t2_smem[];
  constexpr int SF = t2_stage_floats<ADJ>();
  T2Shot *shots = reinterpret_cast<T2Shot *>(t2_smem + 2 * t2_stage_floats<ADJ>());
  T2Step *steps = reinterpret_cast<T2Step *>(shots + T2_MAX_SHOTS);
  int *list = reinterpret_cast<int *>(steps + T2_MAX_SHOTS);
  int *nlist = list + T2_MAX_TILES_PER_CTA;
  int *abort_flag = nlist + 1;
  unsigned long long *full = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<char *>(t2_smem) + t2_smem_bytes<ADJ>() - 64);
  const int tid = threadIdx.x;
  // Shot table and this CTA's tile list into shared memory: constant over
  // the run, so this overlaps the end of the previous step's kernel (the
  // launch allows programmatic dependent launch).
  {
    const int *src = reinterpret_cast<const int *>(t.t2shots);
    int *dst = reinterpret_cast<int *>(shots);
    const int nw = t.nshots * (int)(sizeof(T2Shot) / sizeof(int));
    for (int q = tid; q < nw; q += 256) dst[q] = src[q];
    for (int k = tid; blockIdx.x + k * gridDim.x < n_tiles && k < T2_MAX_TILES_PER_CTA; k += 256)
      list[k] = t.tile_tab[blockIdx.x + k * gridDim.x];
    if (tid == 0) {
      mbar_init(&full[0], 1);
      mbar_init(&full[1], 1);
      mbar_fence_init();
      *abort_flag = 0;
    }
  }
  // Before the wait on the previous kernel: the step counter (changed only
  // between replays of a chunk of steps), the per-shot step scalars, this
  // step's tile list and the first tile's copies of the levels that older
  // launches wrote; this overlaps the tail of the previous step's kernel.
  const int s = *t.counter + s_off;
  __syncthreads();
  if (tid < t.nshots) steps[tid] = t2_step_of<ADJ>(t, shots[tid], tid, s);
  __syncthreads();
  if (tid == 0) {
    // Keep the tiles of shots that are live this step and use this variant.
    int n = 0;
    for (int k = 0; blockIdx.x + k * gridDim.x < n_tiles && k < T2_MAX_TILES_PER_CTA; ++k) {
      const int e = list[k];
      if (steps[t2_b(e)].live) list[n++] = e;
    }
    *nlist = n;
    if (n > 0)
      t2_issue_old<ADJ>(t.t2maps[t2_b(list[0])], shots[t2_b(list[0])], s, list[0], t2_smem,
                        &full[0]);
  }
  // Everything after this reads what the previous kernels of the step
  // sequence wrote (u2, injection terms, the image of the last step).
  pdl_wait();
  pdl_launch_dependents();
  if (tid == 0 && *nlist > 0)
    t2_issue_u2<ADJ>(t.t2maps[t2_b(list[0])], shots[t2_b(list[0])], s, list[0], t2_smem,
                     &full[0]);
  __syncthreads();
  const int n = *nlist;
  for (int k = 0; k < n; ++k) {
    const int cur = k & 1;
    // The other stage was released by the barrier that ended tile k-1.
    if (tid == 0 && k + 1 < n)
      t2_issue<ADJ>(t.t2maps[t2_b(list[k + 1])], shots[t2_b(list[k + 1])], s, list[k + 1],
                    t2_smem + (cur ^ 1) * SF, &full[cur ^ 1]);
    const int e = list[k];
    const T2Shot &h = shots[t2_b(e)];
    const T2Step &stp = steps[t2_b(e)];
    T2Img P;
    if (stp.img && t2_phys_tile(h, e)) t2_img_load(h, stp, e, P, tid);
    // A wait that gives up records the error; the tile is still computed (on
    // whatever the stage holds) so that every thread reaches the same
    // barriers, and the loop ends after it.
    if (!mbar_wait(&full[cur], (unsigned)((k >> 1) & 1))) {
      atomicOr(t.err, 1);
      *abort_flag = 1;
    }
    {
      float *st = t2_smem + cur * SF;
      const bool pre = ADJ && !t2_needs_vel(h, stp, e);
      if (pre) {
        t2_premul(st, tid, 256);
        __syncthreads();
      }
      t2_compute<ADJ>(t, h, stp, t2_b(e), s, e, st, tid, pre);
      if ((stp.extract || stp.img) && t2_phys_tile(h, e))
        t2_snap_tile<ADJ>(h, stp, P, e, st, ADJ ? st + T2_HALO : st + T2_HALO + 3 * T2_CORE,
                          tid);
      t2_edges<ADJ>(h, s, e, st, tid, 0);
      // The stage was written (t2_premul): order that before the tensor
      // copies of tile k+2 overwrite it.
      if (pre) fence_proxy_async_smem();
    }
    __syncthreads();   // the stage is free for tile k+2
    if (*abort_flag) {
      // Wait (bounded) for the copies still in flight so that no tensor
      // copy lands in the shared memory of a finished CTA.
      if (tid == 0) {
        mbar_wait(&full[cur], (unsigned)((k >> 1) & 1));
        if (k + 1 < n) mbar_wait(&full[cur ^ 1], (unsigned)(((k + 1) >> 1) & 1));
      }
      break;
    }
  }
}

// ---------------------------------------------------------------------------
// Warp-specialised variant: one CTA per SM with a producer warp and two
// consumer groups of 8 warps.  Four stages; tile k of the CTA's list goes
// to stage k % 4 and consumer group k % 2, so each group computes while the
// producer keeps up to three further tiles in flight.  Stages are handed
// back through "empty" mbarriers (one arrival per consumer warp) instead of
// CTA-wide barriers; the groups synchronise internally with named barriers.
// ---------------------------------------------------------------------------
constexpr int T2W_STAGES = 4;
constexpr int T2W_THREADS = 544;   // 2 x 256 consumers + 1 producer warp

template <bool ADJ>
__host__ __device__ constexpr size_t t2w_smem_bytes() {
  return T2W_STAGES * sizeof(float) * t2_stage_floats<ADJ>() + sizeof(T2Shot) * T2_MAX_SHOTS +
         sizeof(T2Step) * T2_MAX_SHOTS + sizeof(int) * (T2_MAX_TILES_PER_CTA + 8) +
         2 * T2W_STAGES * 8;
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <bool ADJ>
__device__ __forceinline__ void tile2d_ws(const BatchTables &t, int s_off, int n_tiles) {
  extern __shared__ __align__(128) float t2_smem[];
  constexpr int SF = t2_stage_floats<ADJ>();
  T2Shot *shots = reinterpret_cast<T2Shot *>(t2_smem + T2W_STAGES * SF);
  T2Step *steps = reinterpret_cast<T2Step *>(shots + T2_MAX_SHOTS);
  int *list = reinterpret_cast<int *>(steps + T2_MAX_SHOTS);
  int *nlist = list + T2_MAX_TILES_PER_CTA;
  volatile int *abort_flag = nlist + 1;
  unsigned long long *full = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<char *>(t2_smem) + t2w_smem_bytes<ADJ>() - 2 * T2W_STAGES * 8);
  unsigned long long *empty = full + T2W_STAGES;
  const int tid = threadIdx.x;
  const int s = *t.counter + s_off;
  {
    const int *src = reinterpret_cast<const int *>(t.t2shots);
    int *dst = reinterpret_cast<int *>(shots);
    const int nw = t.nshots * (int)(sizeof(T2Shot) / sizeof(int));
    for (int q = tid; q < nw; q += T2W_THREADS) dst[q] = src[q];
    for (int k = tid; blockIdx.x + k * gridDim.x < n_tiles && k < T2_MAX_TILES_PER_CTA;
         k += T2W_THREADS)
      list[k] = t.tile_tab[blockIdx.x + k * gridDim.x];
    if (tid == 0) {
      for (int q = 0; q < T2W_STAGES; ++q) {
        mbar_init(&full[q], 1);
        mbar_init(&empty[q], 8);
      }
      mbar_fence_init();
      *abort_flag = 0;
    }
  }
  __syncthreads();
  if (tid < t.nshots) steps[tid] = t2_step_of<ADJ>(t, shots[tid], tid, s);
  __syncthreads();
  if (tid == 0) {
    int n = 0;
    for (int k = 0; blockIdx.x + k * gridDim.x < n_tiles && k < T2_MAX_TILES_PER_CTA; ++k) {
      const int e = list[k];
      if (steps[t2_b(e)].live) list[n++] = e;
    }
    *nlist = n;
  }
  __syncthreads();
  const int n = *nlist;
  const int warp = tid >> 5;
  if (warp == 16) {
    // Producer: one thread issues every tile once its stage is free.
    if ((tid & 31) == 0) {
      int k = 0;
      for (; k < n && !*abort_flag; ++k) {
        const int st = k % T2W_STAGES, use = k / T2W_STAGES;
        if (use > 0 && !mbar_wait(&empty[st], (unsigned)((use - 1) & 1))) {
          atomicOr(t.err, 1);
          *abort_flag = 1;
          break;
        }
        const int e = list[k];
        t2_issue<ADJ>(t.t2maps[t2_b(e)], shots[t2_b(e)], s, e, t2_smem + st * SF, &full[st]);
      }
      // After an abort, wait (bounded) for the latest copy issued into each
      // stage, so that none lands after the CTA has finished.
      if (*abort_flag) {
        for (int q = (k > T2W_STAGES ? k - T2W_STAGES : 0); q < k; ++q)
          mbar_wait(&full[q % T2W_STAGES], (unsigned)((q / T2W_STAGES) & 1));
      }
    }
    return;
  }
  // Consumers never leave the loop early, so every thread of a group reaches
  // the group's named barriers; after an abort the waits are skipped and
  // the remaining tiles are run through (their results are discarded with
  // the error status).
  const int g = warp >> 3, gtid = tid & 255;
  for (int k = g; k < n; k += 2) {
    const int st = k % T2W_STAGES;
    const int e = list[k];
    const T2Shot &h = shots[t2_b(e)];
    const T2Step &stp = steps[t2_b(e)];
    T2Img P;
    if (stp.img && t2_phys_tile(h, e)) t2_img_load(h, stp, e, P, gtid);
    if (!*abort_flag && !mbar_wait(&full[st], (unsigned)((k / T2W_STAGES) & 1))) {
      atomicOr(t.err, 1);
      *abort_flag = 1;
    }
    float *stg = t2_smem + st * SF;
    const bool pre = ADJ && !t2_needs_vel(h, stp, e);
    if (pre) {
      t2_premul(stg, gtid, 256);
      t2_bar(1 + g);
    }
    t2_compute<ADJ>(t, h, stp, t2_b(e), s, e, stg, gtid, pre);
    if ((stp.extract || stp.img) && t2_phys_tile(h, e))
      t2_snap_tile<ADJ>(h, stp, P, e, stg,
                        ADJ ? stg + T2_HALO : stg + T2_HALO + 3 * T2_CORE, gtid);
    t2_edges<ADJ>(h, s, e, stg, gtid, 1 + g);
    if (pre) fence_proxy_async_smem();
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(&empty[st]);
  }
}

}  // namespace swave
