// tile3d.cuh - persistent, TMA-pipelined fused step kernel for 3D batches.
//
// A work unit is a 32 (z) x 32 (x) column block of one shot over TY planes
// of y.  A CTA of 256 threads marches the unit's planes: for every plane k,
// one thread issues the tensor copies of plane k + S - 1 (the u2 plane tile
// with a 4-cell z/x halo, 40 x 40, the adjoint's velocity halo tile, and the
// 32 x 32 core tiles of u1, u0, u_1 and, forward, the velocity) into a ring
// of S shared-memory stages on mbarriers, while the CTA computes plane k.
// Thread (tz, tx) owns rows i0..i0+3 of column x0 + tx: the z and x
// derivatives come from the staged plane, the y derivative from a register
// queue of the column's values at planes k-4..k+4 (read from global memory
// one plane ahead; for the adjoint the queue holds v^2 u2).  The floating-
// point operation order is the reference's (FDderivatives.f90:97-131
// forward, 780-819 adjoint, 960-982 time update), as in stream3d.cuh.
#pragma once

#include "batch.cuh"
#include "tile2d.cuh"

namespace swave {

constexpr int T3_Z = 32, T3_X = 32;
constexpr int T3_SZ = T3_Z + 8, T3_SX = T3_X + 8;
constexpr int T3_HALO = T3_SZ * T3_SX;   // 1600 floats
constexpr int T3_CORE = T3_Z * T3_X;     // 1024 floats
constexpr int T3_STAGES = 4;
constexpr int T3_MAX_UNITS_PER_CTA = 512;

template <bool ADJ>
__host__ __device__ constexpr int t3_stage_floats() {
  return ADJ ? 2 * T3_HALO + 3 * T3_CORE : T3_HALO + 4 * T3_CORE;
}
template <bool ADJ>
__host__ __device__ constexpr size_t t3_smem_bytes() {
  return T3_STAGES * sizeof(float) * t3_stage_floats<ADJ>() + sizeof(int) * (T3_MAX_UNITS_PER_CTA + 8) +
         T3_STAGES * 8;
}

// 3D tensor copy global -> shared memory, completing on an mbarrier.
__device__ __forceinline__ void tma_3d(float *dst, const CUtensorMap *map, int x, int y, int z,
                                       unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Unit entry: (shot << 24) | (tzi << 16) | (txi << 8) | kyi, decoded with the
// shot's tile counts.
__device__ __forceinline__ int t3_b(int e) { return e >> 24; }
__device__ __forceinline__ int t3_tzi(int e) { return (e >> 16) & 0xff; }
__device__ __forceinline__ int t3_txi(int e) { return (e >> 8) & 0xff; }
__device__ __forceinline__ int t3_kyi(int e) { return e & 0xff; }

template <bool ADJ>
__device__ __forceinline__ void t3_issue(const T3Maps &M, int s, int zi, int xi, int kp,
                                         float *st, unsigned long long *bar) {
  constexpr unsigned bytes = 4u * (unsigned)t3_stage_floats<ADJ>();
  mbar_expect_tx(bar, bytes);
  tma_3d(st, &M.m[2 * ((s + 3) % 5)], zi, xi, kp, bar);
  if (ADJ) tma_3d(st + T3_HALO, &M.m[10], zi, xi, kp, bar);
  float *cst = st + (ADJ ? 2 : 1) * T3_HALO;
  tma_3d(cst, &M.m[2 * ((s + 2) % 5) + 1], zi + 4, xi + 4, kp, bar);
  tma_3d(cst + T3_CORE, &M.m[2 * ((s + 1) % 5) + 1], zi + 4, xi + 4, kp, bar);
  tma_3d(cst + 2 * T3_CORE, &M.m[2 * (s % 5) + 1], zi + 4, xi + 4, kp, bar);
  if (!ADJ) tma_3d(cst + 3 * T3_CORE, &M.m[11], zi + 4, xi + 4, kp, bar);
}

// Injection, Born source, snapshot and imaging of one element (3D); the
// operations of stream3d.cuh.  se is the Laplacian part; returns it with
// the sources added.  The snapshot / imaging part runs after the update
// (post = true) with u2c the element's u2.
__device__ __noinline__ float t3_extras(const ShotDev &S, int it, int i, int j, int k, float se,
                                        float vc, bool post, float u2c, bool inj = true) {
  const Geom &g = S.g;
  if (!post && inj) {
    if (S.inj_on && i >= S.bi0 && i <= S.bi1 && j >= S.bj0 && j <= S.bj1 && k >= S.bk0 &&
        k <= S.bk1) {
      const int bx =
          (i - S.bi0) + (S.bi1 - S.bi0 + 1) * ((j - S.bj0) + (S.bj1 - S.bj0 + 1) * (k - S.bk0));
      const int e1 = S.inj_off[bx + 1];
      for (int e = S.inj_off[bx]; e < e1; ++e) {
        const InjEntry E = S.inj_ent[e];
        const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
        se = se + (((E.v2r * tr) * E.wz) * E.wx) * E.wy;
      }
    }
  }
  const bool phys = i >= 1 && i <= g.nz && j >= 1 && j <= g.nx && k >= 1 && k <= g.ny;
  if (!phys || (it % S.snapi) != 0) return se;
  const long long nphys = (long long)g.nz * g.nx * g.ny;
  const long long pp = g.pidx(i, j, k);
  const float taper = S.taperx ? S.taperx[j - 1] * S.tapery[k - 1] : 1.f;
  const int cnt = S.tstep > 0 ? it / S.snapi - (S.tcnt - 1) / S.snapi
                              : S.tcnt / S.snapi - (it - 1) / S.snapi;
  if (!post) {
    if (S.imaging == 4 && S.tstep > 0 && cnt <= S.ntsnap)
      se = se + (((2.0f * taper) * S.ref[pp]) * S.wave[(long long)(cnt - 1) * nphys + pp]) / vc;
    return se;
  }
  if (S.extract_wave && cnt <= S.ntsnap) S.wave[(long long)(cnt - 1) * nphys + pp] = u2c;
  if (S.imaging >= 1 && S.imaging <= 3 && S.tstep < 0) {
    const int index = S.ntsnap - cnt + 1;
    if (index >= 1) {
      const float wsn = S.wave[(long long)(index - 1) * nphys + pp];
      float im = S.image[pp];
      if (S.imaging == 1) {
        im = im + (u2c * wsn) * taper;
      } else if (S.imaging == 2) {
        im = im + (((2.0f * taper) * u2c) * wsn) / vc;
      } else {
        const int ip1 = min(index + 1, S.ntsnap), im1 = max(index - 1, 1);
        const float tt = ((S.wave[(long long)(im1 - 1) * nphys + pp] - 2.0f * wsn) +
                          S.wave[(long long)(ip1 - 1) * nphys + pp]) /
                         (S.dt2snap * ((vc * vc) * vc));
        im = im + (u2c * tt) * taper;
      }
      S.image[pp] = im;
      S.illum[pp] = S.illum[pp] + (wsn * wsn) * taper;
    }
  }
  return se;
}

template <bool ADJ>
__device__ __forceinline__ float4 t3_col4(const float *u2, const float *vel, long long off) {
  float4 u = *reinterpret_cast<const float4 *>(u2 + off);
  if (ADJ) {
    const float4 v = *reinterpret_cast<const float4 *>(vel + off);
    u = make_float4((v.x * v.x) * u.x, (v.y * v.y) * u.y, (v.z * v.z) * u.z, (v.w * v.w) * u.w);
  }
  return u;
}

template <bool ADJ>
__device__ __forceinline__ void tile3d_persistent(const BatchTables &t, int s_off, int n_units) {
  extern __shared__ __align__(128) float t3_smem[];
  constexpr int SF = t3_stage_floats<ADJ>();
  int *list = reinterpret_cast<int *>(t3_smem + T3_STAGES * SF);
  int *nlist = list + T3_MAX_UNITS_PER_CTA;
  volatile int *abort_flag = nlist + 1;
  unsigned long long *full = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<char *>(t3_smem) + t3_smem_bytes<ADJ>() - T3_STAGES * 8);
  const int tid = threadIdx.x;
  const int tz = tid & 7, tx = tid >> 3;
  const int s = *t.counter + s_off;
  if (tid == 0) {
    for (int q = 0; q < T3_STAGES; ++q) mbar_init(&full[q], 1);
    mbar_fence_init();
    *abort_flag = 0;
    int n = 0;
    for (int k = 0; blockIdx.x + k * gridDim.x < n_units && k < T3_MAX_UNITS_PER_CTA; ++k) {
      const int e = t.tile_tab[blockIdx.x + k * gridDim.x];
      const ShotDev &S = t.shots[t3_b(e)];
      if (s < S.nsteps && (S.adj3d != 0) == ADJ) list[n++] = e;
    }
    *nlist = n;
  }
  __syncthreads();
  const int n = *nlist;
  int pc = 0;   // planes processed by this CTA (stage ring position)
  for (int u = 0; u < n; ++u) {
    const int e = list[u];
    const ShotDev &S = t.shots[t3_b(e)];
    const T3Maps &M = t.t3maps[t3_b(e)];
    const Geom &g = S.g;
    const int z0 = g.nmin1 + t3_tzi(e) * T3_Z, x0 = g.nmin2 + t3_txi(e) * T3_X;
    const int k0 = g.nmin3 + t3_kyi(e) * S.t3_ty;
    const int k1 = min(k0 + S.t3_ty, g.nmax3 + 1);
    const int np = k1 - k0;
    const int zi = z0 - 4 - g.lo1, xi = x0 - 4 - g.lo2;
    // Prologue: the first S-1 planes of the unit.
    if (tid == 0) {
      for (int p = 0; p < T3_STAGES - 1 && p < np; ++p) {
        const int q = (pc + p) % T3_STAGES;
        t3_issue<ADJ>(M, s, zi, xi, k0 + p - g.lo3, t3_smem + q * SF, &full[q]);
      }
    }
    const int i0 = z0 + 4 * tz, j = x0 + tx;
    const bool colok = j <= g.nmax2 && i0 <= g.nmax1;
    // Column of the y queue (clamped inside the padded array; values of
    // columns or rows that are not computed are never used).
    const int ic = min(i0, g.lo1 + g.ld1 - 4), jc = min(j, g.lo2 + g.n2p - 1);
    const float *u2 = S.f[(s + 3) % 5];
    const long long colbase = (long long)(ic - g.lo1) + (long long)g.ld1 * (jc - g.lo2);
    const long long P = g.plane();
    float4 q[9];
#pragma unroll
    for (int l = 0; l < 8; ++l) q[l] = t3_col4<ADJ>(u2, S.vel, colbase + P * (k0 - 4 + l - g.lo3));
    float4 nxt = t3_col4<ADJ>(u2, S.vel, colbase + P * (k0 + 4 - g.lo3));
    const int it = S.tmin + s * S.tstep;
    const bool snapstep = (it % S.snapi) == 0 && (S.extract_wave || S.imaging != 0);
    const Coefs c = S.c;
    float *u3 = S.f[(s + 4) % 5];
    for (int p = 0; p < np; ++p) {
      const int k = k0 + p;
      const int qs = (pc + p) % T3_STAGES;
      // Plane p + S - 1 into the stage the barrier of plane p - 1 released.
      if (tid == 0 && p + T3_STAGES - 1 < np) {
        const int qn = (pc + p + T3_STAGES - 1) % T3_STAGES;
        t3_issue<ADJ>(M, s, zi, xi, k + T3_STAGES - 1 - g.lo3, t3_smem + qn * SF, &full[qn]);
      }
      q[8] = nxt;
      if (p + 1 < np) nxt = t3_col4<ADJ>(u2, S.vel, colbase + P * (k + 5 - g.lo3));
      if (!*abort_flag && !mbar_wait(&full[qs], (unsigned)(((pc + p) / T3_STAGES) & 1))) {
        atomicOr(t.err, 1);
        *abort_flag = 1;
      }
      const float *st = t3_smem + qs * SF;
      const float *su = st;                                   // u2 (or v^2 u2 below)
      const float *sv2 = st + T3_HALO;                        // adjoint velocity halo
      const float *core = st + (ADJ ? 2 : 1) * T3_HALO;
      if (colok) {
        const float *col = su + (tx + 4) * T3_SZ + 4 * tz;    // row i0-4
        float zr[12];
        {
          const float4 a = *reinterpret_cast<const float4 *>(col);
          const float4 b = *reinterpret_cast<const float4 *>(col + 4);
          const float4 cc = *reinterpret_cast<const float4 *>(col + 8);
          const float r[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, cc.x, cc.y, cc.z, cc.w};
#pragma unroll
          for (int m = 0; m < 12; ++m) zr[m] = r[m];
          if (ADJ) {
            const float *vcol = sv2 + (tx + 4) * T3_SZ + 4 * tz;
#pragma unroll
            for (int m = 0; m < 12; ++m) zr[m] = (vcol[m] * vcol[m]) * zr[m];
          }
        }
        float tzz[4], txx[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int m = 4 + r;
          float a = c.c0z * zr[m];
          a = a + c.c1z * (zr[m + 1] + zr[m - 1]);
          a = a + c.c2z * (zr[m + 2] + zr[m - 2]);
          a = a + c.c3z * (zr[m + 3] + zr[m - 3]);
          a = a + c.c4z * (zr[m + 4] + zr[m - 4]);
          tzz[r] = a;
          txx[r] = c.c0x * zr[m];
        }
        const float cx[5] = {c.c0x, c.c1x, c.c2x, c.c3x, c.c4x};
#pragma unroll
        for (int l = 1; l <= 4; ++l) {
          float4 rp = *reinterpret_cast<const float4 *>(col + l * T3_SZ + 4);
          float4 rm = *reinterpret_cast<const float4 *>(col - l * T3_SZ + 4);
          if (ADJ) {
            const float *vcol = sv2 + (tx + 4) * T3_SZ + 4 * tz + 4;
            const float4 vp = *reinterpret_cast<const float4 *>(vcol + l * T3_SZ);
            const float4 vm = *reinterpret_cast<const float4 *>(vcol - l * T3_SZ);
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
        float sv[4];
        const float cy[5] = {c.c0y, c.c1y, c.c2y, c.c3y, c.c4y};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          auto Y = [&](int l) {
            const float4 &v = q[l];
            return r == 0 ? v.x : r == 1 ? v.y : r == 2 ? v.z : v.w;
          };
          float tyy = cy[0] * Y(4);
          tyy = tyy + cy[1] * (Y(5) + Y(3));
          tyy = tyy + cy[2] * (Y(6) + Y(2));
          tyy = tyy + cy[3] * (Y(7) + Y(1));
          tyy = tyy + cy[4] * (Y(8) + Y(0));
          sv[r] = (txx[r] + tzz[r]) + tyy;
        }
        const float *cc = core + tx * T3_Z + 4 * tz;
        float vcen[4];
        if (ADJ) {
          const float *vc = sv2 + (tx + 4) * T3_SZ + 4 * tz + 4;
#pragma unroll
          for (int r = 0; r < 4; ++r) vcen[r] = vc[r];
        } else {
          const float4 vv = *reinterpret_cast<const float4 *>(cc + 3 * T3_CORE);
          vcen[0] = vv.x; vcen[1] = vv.y; vcen[2] = vv.z; vcen[3] = vv.w;
#pragma unroll
          for (int r = 0; r < 4; ++r) sv[r] = (vcen[r] * vcen[r]) * sv[r];
        }
        const float4 u2c4 = *reinterpret_cast<const float4 *>(col + 4);
        const float u2c[4] = {u2c4.x, u2c4.y, u2c4.z, u2c4.w};
        // Injection (Injection.f90:151-456): each cell's entries in order,
        // their terms precomputed for this step by k_bterms, or formed here
        // (the same operations) for a shot with few entries.
        const bool inj = S.inj_on && k >= S.bk0 && k <= S.bk1 && j >= S.bj0 && j <= S.bj1 &&
                         i0 + 3 >= S.bi0 && i0 <= S.bi1;
        if (inj) {
          const int nbi = S.bi1 - S.bi0 + 1;
          const int cb = nbi * ((j - S.bj0) + (S.bj1 - S.bj0 + 1) * (k - S.bk0));
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int i = i0 + r;
            if (i > g.nmax1 || i < S.bi0 || i > S.bi1) continue;
            const int e1 = S.inj_off[cb + (i - S.bi0) + 1];
            for (int e = S.inj_off[cb + (i - S.bi0)]; e < e1; ++e) {
              float tv;
              if (S.inj_pre) {
                tv = S.inj_term[e];
              } else {
                const InjEntry E = S.inj_ent[e];
                const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
                tv = (((E.v2r * tr) * E.wz) * E.wx) * E.wy;
              }
              sv[r] = sv[r] + tv;
            }
          }
        }
        // The Born source (imaging 4): element by element.
        if (snapstep && S.imaging == 4) {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (i0 + r <= g.nmax1)
              sv[r] = t3_extras(S, it, i0 + r, j, k, sv[r], vcen[r], false, 0.f, false);
        }
        // FD_2nd_time_derivative_grid (FDderivatives.f90:960-982).
        const float4 a1 = *reinterpret_cast<const float4 *>(cc);
        const float4 a0 = *reinterpret_cast<const float4 *>(cc + T3_CORE);
        const float4 am = *reinterpret_cast<const float4 *>(cc + 2 * T3_CORE);
        const float A1[4] = {a1.x, a1.y, a1.z, a1.w}, A0[4] = {a0.x, a0.y, a0.z, a0.w},
                    AM[4] = {am.x, am.y, am.z, am.w};
        float o[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          float a = 20.0f * u2c[r];
          a = a - 6.0f * A1[r];
          a = a - 4.0f * A0[r];
          a = a + AM[r];
          a = a + S.k12 * sv[r];
          o[r] = a * S.div11;
        }
        const long long off = g.idx(i0, j, k);
        if (i0 + 3 <= g.nmax1) {
          *reinterpret_cast<float4 *>(u3 + off) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (i0 + r <= g.nmax1) u3[off + r] = o[r];
        }
        // Snapshot saves and imaging of this step: k_bsnap3d, after the
        // launch.
      }
      __syncthreads();   // the stage is free for plane p + S
#pragma unroll
      for (int l = 0; l < 8; ++l) q[l] = q[l + 1];
    }
    pc += np;
  }
}

}  // namespace swave
