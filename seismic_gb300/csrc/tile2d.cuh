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
// with 128-bit reads and writes u3 with 128-bit stores.  Work only a few
// tiles have (injection boxes, snapshot / imaging steps, clamped adjoint
// edges) is decided once per tile.  The floating-point operation order is
// the reference's (see batch.cu).
#pragma once

#include "batch.cuh"

namespace swave {

constexpr int T2_Z = 64, T2_X = 32;
constexpr int T2_SZ = T2_Z + 8;          // staged column length (with halo)
constexpr int T2_SX = T2_X + 8;          // staged columns (with halo)
constexpr int T2_HALO = T2_SX * T2_SZ;   // 2880 floats
constexpr int T2_CORE = T2_X * T2_Z;     // 2048 floats
constexpr int T2_MAX_TILES_PER_CTA = 512;

// Floats of one pipeline stage.
template <bool ADJ>
__host__ __device__ constexpr int t2_stage_floats() {
  return ADJ ? 2 * T2_HALO + 3 * T2_CORE : T2_HALO + 4 * T2_CORE;
}
// Dynamic shared memory: two stages, the shot table and the tile list.
template <bool ADJ>
__host__ __device__ constexpr size_t t2_smem_bytes() {
  return 2 * sizeof(float) * t2_stage_floats<ADJ>() + sizeof(T2Shot) * T2_MAX_SHOTS +
         sizeof(int) * (T2_MAX_TILES_PER_CTA + 4);
}

__device__ __forceinline__ void cp_async16(float *smem, const float *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ int t2_b(int e) { return e >> 24; }
__device__ __forceinline__ int t2_tzi(int e) { return (e >> 12) & 0xfff; }
__device__ __forceinline__ int t2_txi(int e) { return e & 0xfff; }

// Issues the cp.async copies of one tile into a stage.
template <bool ADJ>
__device__ __forceinline__ void t2_issue(const T2Shot &h, int s, int e, float *st) {
  const float *u2 = h.f[(s + 3) % 5];
  const int L = h.ld1;
  const int jmaxp = h.lo2 + h.n2p - 1;
  const int rbase = t2_tzi(e) * T2_Z;   // row offset of z0-4 inside a column
  const int x0 = h.nmin2 + t2_txi(e) * T2_X;
  const int tid = threadIdx.x;
  // Halo tiles: 40 columns x 18 float4.
  for (int q = tid; q < T2_SX * (T2_SZ / 4); q += 256) {
    const int col = q / (T2_SZ / 4), grp = q - col * (T2_SZ / 4);
    const int j = min(x0 - 4 + col, jmaxp);
    const int off = min(rbase + 4 * grp, L - 4) + L * (j - h.lo2);
    cp_async16(st + col * T2_SZ + 4 * grp, u2 + off);
    if (ADJ) cp_async16(st + T2_HALO + col * T2_SZ + 4 * grp, h.vel + off);
  }
  // Core tiles: 32 columns x 16 float4, rows z0..z0+63.
  const float *c0 = h.f[(s + 2) % 5], *c1 = h.f[(s + 1) % 5], *c2 = h.f[s % 5];
  float *cst = st + (ADJ ? 2 : 1) * T2_HALO;
  for (int q = tid; q < T2_X * (T2_Z / 4); q += 256) {
    const int col = q / (T2_Z / 4), grp = q - col * (T2_Z / 4);
    const int j = min(x0 + col, jmaxp);
    const int off = min(rbase + 4 + 4 * grp, L - 4) + L * (j - h.lo2);
    float *d = cst + col * T2_Z + 4 * grp;
    cp_async16(d, c0 + off);
    cp_async16(d + T2_CORE, c1 + off);
    cp_async16(d + 2 * T2_CORE, c2 + off);
    if (!ADJ) cp_async16(d + 3 * T2_CORE, h.vel + off);
  }
}

__device__ __forceinline__ float f4get(const float4 &a, int e) {
  return e == 0 ? a.x : e == 1 ? a.y : e == 2 ? a.z : a.w;
}

// Injection, Born source, snapshot and imaging of one element (rare tiles;
// reads the full shot descriptor from global memory).
__device__ __noinline__ float t2_extras(const ShotDev &S, int it, bool snapstep, int i, int j,
                                        float se, float u2c, float vc) {
  const Geom &g = S.g;
  if (S.inj_on && i >= S.bi0 && i <= S.bi1 && j >= S.bj0 && j <= S.bj1) {
    const int bx = (i - S.bi0) + (S.bi1 - S.bi0 + 1) * (j - S.bj0);
    const int e1 = S.inj_off[bx + 1];
    for (int q = S.inj_off[bx]; q < e1; ++q) {
      const InjEntry E = S.inj_ent[q];
      const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
      se = se + (((E.v2r * tr) * E.wz) * E.wx) * E.wy;   // Injection.f90:151-456,561-591
    }
  }
  if (snapstep && i >= 1 && i <= g.nz && j >= 1 && j <= g.nx) {
    const long long nphys = (long long)g.nz * g.nx;
    const long long pp = (long long)(i - 1) + (long long)g.nz * (j - 1);
    const float taper = S.taperx ? S.taperx[j - 1] * S.tapery[0] : 1.f;
    const int cnt = S.tstep > 0 ? it / S.snapi - (S.tmin - 1) / S.snapi
                                : S.tmin / S.snapi - (it - 1) / S.snapi;
    // Injection_Born (Imaging.f90:747-788).
    if (S.imaging == 4 && S.tstep > 0 && cnt <= S.ntsnap)
      se = se + (((2.0f * taper) * S.ref[pp]) * S.wave[(long long)(cnt - 1) * nphys + pp]) / vc;
    // Extraction_wavefield (Extraction.f90:562-601).
    if (S.extract_wave && cnt <= S.ntsnap) S.wave[(long long)(cnt - 1) * nphys + pp] = u2c;
    if (S.imaging >= 1 && S.imaging <= 3 && S.tstep < 0) {
      const int index = S.ntsnap - cnt + 1;
      if (index >= 1) {
        const float wsn = S.wave[(long long)(index - 1) * nphys + pp];
        float im = S.image[pp];
        if (S.imaging == 1) {
          im = im + (u2c * wsn) * taper;                          // Imaging.f90:265
        } else if (S.imaging == 2) {
          im = im + (((2.0f * taper) * u2c) * wsn) / vc;          // Imaging.f90:735
        } else {
          const int ip1 = min(index + 1, S.ntsnap), im1 = max(index - 1, 1);
          const float tt = ((S.wave[(long long)(im1 - 1) * nphys + pp] - 2.0f * wsn) +
                            S.wave[(long long)(ip1 - 1) * nphys + pp]) /
                           (S.dt2snap * ((vc * vc) * vc));
          im = im + (u2c * tt) * taper;                           // Imaging.f90:410-411
        }
        S.image[pp] = im;
        S.illum[pp] = S.illum[pp] + (wsn * wsn) * taper;
      }
    }
  }
  return se;
}

// Computes one tile from a completed stage.
template <bool ADJ>
__device__ __forceinline__ void t2_compute(const BatchTables &t, const T2Shot &h, int b, int s,
                                           int e, const float *st) {
  const int z0 = h.nmin1 + t2_tzi(e) * T2_Z, x0 = h.nmin2 + t2_txi(e) * T2_X;
  const int tid = threadIdx.x;
  const int tz = tid & 15, tx = tid >> 4;
  const int i0 = z0 + 4 * tz;
  if (i0 > h.nmax1) return;
  const int it = h.tmin + s * h.tstep;
  const bool snapstep = (it % h.snapi) == 0;
  // Tile-level decisions.
  const int zl = z0 + T2_Z - 1, xl = x0 + T2_X - 1;
  const bool inj_tile = h.inj_on && !(zl < h.bi0 || z0 > h.bi1 || xl < h.bj0 || x0 > h.bj1);
  const bool snap_tile = snapstep && (h.extract_wave || h.imaging != 0) &&
                         !(zl < 1 || z0 > h.nz || xl < 1 || x0 > h.nx);
  const bool clamp_free = !ADJ || (z0 - 4 >= h.nmin1 && zl + 4 <= h.nmax1 &&
                                   x0 - 4 >= h.nmin2 && xl + 4 <= h.nmax2);
  const float *su = st;
  const float *svel = st + T2_HALO;                       // adjoint only
  const float *core = st + (ADJ ? 2 : 1) * T2_HALO;
  float *__restrict__ u3 = const_cast<float *>(h.f[(s + 4) % 5]);
  const int L = h.ld1;
  const int rbase = t2_tzi(e) * T2_Z;
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int jl = tx + 16 * hh;
    const int j = x0 + jl;
    if (j > h.nmax2) break;
    const int sc = jl + 4;                        // staged halo column
    const float *col = su + sc * T2_SZ + 4 * tz;  // rows i0-4 .. i0+7 start here
    float sv[4];
    if (clamp_free) {
      const float4 za = *reinterpret_cast<const float4 *>(col);
      const float4 zb = *reinterpret_cast<const float4 *>(col + 4);
      const float4 zc = *reinterpret_cast<const float4 *>(col + 8);
      float zr[12] = {za.x, za.y, za.z, za.w, zb.x, zb.y, zb.z, zb.w, zc.x, zc.y, zc.z, zc.w};
      if (ADJ) {
        const float *vcol = svel + sc * T2_SZ + 4 * tz;
        const float4 va = *reinterpret_cast<const float4 *>(vcol);
        const float4 vb = *reinterpret_cast<const float4 *>(vcol + 4);
        const float4 vc4 = *reinterpret_cast<const float4 *>(vcol + 8);
        const float vr[12] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w,
                              vc4.x, vc4.y, vc4.z, vc4.w};
        // w = (v*v)*u at every stencil point (FDderivatives.f90:847-891).
#pragma unroll
        for (int q = 0; q < 12; ++q) zr[q] = (vr[q] * vr[q]) * zr[q];
      }
      // FD_2nd_2D_derivatives_scalar_forward_grid (FDderivatives.f90:715-743).
      float tzz[4], txx[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int m = 4 + q;
        float a = h.c0z * zr[m];
        a = a + h.c1z * (zr[m + 1] + zr[m - 1]);
        a = a + h.c2z * (zr[m + 2] + zr[m - 2]);
        a = a + h.c3z * (zr[m + 3] + zr[m - 3]);
        a = a + h.c4z * (zr[m + 4] + zr[m - 4]);
        tzz[q] = a;
        txx[q] = h.c0x * zr[m];
      }
      const float cx[5] = {h.c0x, h.c1x, h.c2x, h.c3x, h.c4x};
#pragma unroll
      for (int l = 1; l <= 4; ++l) {
        float4 rp = *reinterpret_cast<const float4 *>(col + l * T2_SZ + 4);
        float4 rm = *reinterpret_cast<const float4 *>(col - l * T2_SZ + 4);
        if (ADJ) {
          const float *vcol = svel + sc * T2_SZ + 4 * tz + 4;
          const float4 vp = *reinterpret_cast<const float4 *>(vcol + l * T2_SZ);
          const float4 vm = *reinterpret_cast<const float4 *>(vcol - l * T2_SZ);
          rp = make_float4((vp.x * vp.x) * rp.x, (vp.y * vp.y) * rp.y, (vp.z * vp.z) * rp.z,
                           (vp.w * vp.w) * rp.w);
          rm = make_float4((vm.x * vm.x) * rm.x, (vm.y * vm.y) * rm.y, (vm.z * vm.z) * rm.z,
                           (vm.w * vm.w) * rm.w);
        }
        txx[0] = txx[0] + cx[l] * (rp.x + rm.x);
        txx[1] = txx[1] + cx[l] * (rp.y + rm.y);
        txx[2] = txx[2] + cx[l] * (rp.z + rm.z);
        txx[3] = txx[3] + cx[l] * (rp.w + rm.w);
      }
      if (ADJ) {
#pragma unroll
        for (int q = 0; q < 4; ++q) sv[q] = txx[q] + tzz[q];
      } else {
        const float4 vv = *reinterpret_cast<const float4 *>(core + 3 * T2_CORE + jl * T2_Z + 4 * tz);
        sv[0] = (vv.x * vv.x) * (txx[0] + tzz[0]);
        sv[1] = (vv.y * vv.y) * (txx[1] + tzz[1]);
        sv[2] = (vv.z * vv.z) * (txx[2] + tzz[2]);
        sv[3] = (vv.w * vv.w) * (txx[3] + tzz[3]);
      }
    } else {
      // Adjoint tile at an edge of the compute domain: vel indices clamped
      // element by element (FDderivatives.f90:863-878).
      auto U = [&](int zi, int xi) { return su[(xi - x0 + 4) * T2_SZ + (zi - z0 + 4)]; };
      auto W = [&](int zi, int xi) {
        const int zc = min(max(zi, h.nmin1), h.nmax1), xc = min(max(xi, h.nmin2), h.nmax2);
        const float v = svel[(xc - x0 + 4) * T2_SZ + (zc - z0 + 4)];
        return (v * v) * U(zi, xi);
      };
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = i0 + q;
        float a = h.c0z * W(i, j);
        a = a + h.c1z * (W(i + 1, j) + W(i - 1, j));
        a = a + h.c2z * (W(i + 2, j) + W(i - 2, j));
        a = a + h.c3z * (W(i + 3, j) + W(i - 3, j));
        a = a + h.c4z * (W(i + 4, j) + W(i - 4, j));
        float bx = h.c0x * W(i, j);
        bx = bx + h.c1x * (W(i, j + 1) + W(i, j - 1));
        bx = bx + h.c2x * (W(i, j + 2) + W(i, j - 2));
        bx = bx + h.c3x * (W(i, j + 3) + W(i, j - 3));
        bx = bx + h.c4x * (W(i, j + 4) + W(i, j - 4));
        sv[q] = bx + a;
      }
    }
    const float4 u2c = *reinterpret_cast<const float4 *>(col + 4);
    const float *cc = core + jl * T2_Z + 4 * tz;
    if (inj_tile || snap_tile) {
      const ShotDev &S = t.shots[b];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float vc = ADJ ? svel[(jl + 4) * T2_SZ + 4 * tz + 4 + q] : cc[3 * T2_CORE + q];
        sv[q] = t2_extras(S, it, snap_tile, i0 + q, j, sv[q], f4get(u2c, q), vc);
      }
    }
    // FD_2nd_time_derivative_grid (FDderivatives.f90:960-982).
    const float4 a1 = *reinterpret_cast<const float4 *>(cc);
    const float4 a0 = *reinterpret_cast<const float4 *>(cc + T2_CORE);
    const float4 am = *reinterpret_cast<const float4 *>(cc + 2 * T2_CORE);
    float o[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float a = 20.0f * f4get(u2c, q);
      a = a - 6.0f * f4get(a1, q);
      a = a - 4.0f * f4get(a0, q);
      a = a + f4get(am, q);
      a = a + h.k12 * sv[q];
      o[q] = a * h.div11;
    }
    const int off = (rbase + 4 + 4 * tz) + L * (j - h.lo2);
    if (i0 + 3 <= h.nmax1) {
      *reinterpret_cast<float4 *>(u3 + off) = make_float4(o[0], o[1], o[2], o[3]);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (i0 + q <= h.nmax1) u3[off + q] = o[q];
    }
  }
}

template <bool ADJ>
__device__ __forceinline__ void tile2d_persistent(const BatchTables &t, int s_off, int n_tiles) {
  extern __shared__ __align__(16) float t2_smem[];
  float *stage0 = t2_smem;
  float *stage1 = t2_smem + t2_stage_floats<ADJ>();
  T2Shot *shots = reinterpret_cast<T2Shot *>(t2_smem + 2 * t2_stage_floats<ADJ>());
  int *list = reinterpret_cast<int *>(shots + T2_MAX_SHOTS);
  int *nlist = list + T2_MAX_TILES_PER_CTA;
  const int tid = threadIdx.x;
  const int s = *t.counter + s_off;
  // Shot table and this CTA's tile list into shared memory.
  {
    const int *src = reinterpret_cast<const int *>(t.t2shots);
    int *dst = reinterpret_cast<int *>(shots);
    const int nw = t.nshots * (int)(sizeof(T2Shot) / sizeof(int));
    for (int q = tid; q < nw; q += 256) dst[q] = src[q];
    for (int k = tid; blockIdx.x + k * gridDim.x < n_tiles && k < T2_MAX_TILES_PER_CTA; k += 256)
      list[k] = t.tile_tab[blockIdx.x + k * gridDim.x];
  }
  __syncthreads();
  if (tid == 0) {
    // Keep the tiles of shots that are live this step and use this variant.
    int n = 0;
    for (int k = 0; blockIdx.x + k * gridDim.x < n_tiles && k < T2_MAX_TILES_PER_CTA; ++k) {
      const int e = list[k];
      const T2Shot &h = shots[t2_b(e)];
      if (s < h.nsteps && (h.adj2d != 0) == ADJ) list[n++] = e;
    }
    *nlist = n;
  }
  __syncthreads();
  const int n = *nlist;
  if (n == 0) return;
  t2_issue<ADJ>(shots[t2_b(list[0])], s, list[0], stage0);
  cp_async_commit();
  for (int k = 0; k < n; ++k) {
    float *cur = (k & 1) ? stage1 : stage0;
    float *nxt = (k & 1) ? stage0 : stage1;
    if (k + 1 < n) t2_issue<ADJ>(shots[t2_b(list[k + 1])], s, list[k + 1], nxt);
    cp_async_commit();
    cp_async_wait<1>();    // the current tile's group has landed
    __syncthreads();
    const int e = list[k];
    t2_compute<ADJ>(t, shots[t2_b(e)], t2_b(e), s, e, cur);
    __syncthreads();       // the stage is free for the tile after next
  }
  cp_async_wait<0>();
}

}  // namespace swave
