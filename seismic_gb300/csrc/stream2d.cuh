// stream2d.cuh - streaming fused step kernel for 2D batches.
//
// A CTA of TZ threads owns rows [z0, z0+TZ) of one shot and walks TX
// columns in x (TX is a launch parameter, TZ a compile-time one).  Each thread keeps u2 at its row for columns j-4..j+4 in
// registers (the x-derivative) and stages column j in shared memory (the
// z-derivative), so every u2 value is read from memory once per sweep.  The
// next column's loads are issued before the barrier of the current one so
// that two columns are in flight per warp.  The arithmetic is the same
// sequence of IEEE operations as the reference loops (see batch.cu).
#pragma once

#include "batch.cuh"

namespace swave {

template <int TZ>
struct Stream2dSmem {
  float u[2][TZ + 8];
  float v2[2][TZ + 8];
};

template <int TZ, bool ADJ>
__device__ __forceinline__ void stream2d_body(const BatchTables &t, int s_off, int b,
                                              int local, int TX) {
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;   // uniform over the CTA
  __shared__ Stream2dSmem<TZ> sm;
  const Geom g = S.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
  const int ntz = (n1 + TZ - 1) / TZ;
  const int tz = local % ntz, tx = local / ntz;
  (void)n2;
  const int tid = threadIdx.x;
  const int z0 = g.nmin1 + tz * TZ;
  const int i = z0 + tid;
  const bool row_ok = i <= g.nmax1;
  const int ir = min(i, g.nmax1 + 4);           // rows beyond nmax1+4 are never read
  const int j0 = g.nmin2 + tx * TX;
  const int j1 = min(j0 + TX, g.nmax2 + 1);
  const int it = S.tmin + s * S.tstep;
  const float *__restrict__ um1 = S.f[s % 5];
  const float *__restrict__ u0 = S.f[(s + 1) % 5];
  const float *__restrict__ u1 = S.f[(s + 2) % 5];
  const float *__restrict__ u2 = S.f[(s + 3) % 5];
  float *__restrict__ u3 = S.f[(s + 4) % 5];
  const float *__restrict__ vel = S.vel;
  const int L = g.ld1;
  const Coefs c = S.c;
  const float k12 = S.k12, div11 = S.div11;
  // Halo rows of the shared column: threads 0..3 load z0-4+tid, threads
  // TZ-4..TZ-1 load z0+TZ+(tid-TZ+4) (clamped to the last padded row).
  const bool top = tid < 4, bot = tid >= TZ - 4;
  const int hrow = top ? z0 - 4 + tid : min(z0 + TZ + (tid - (TZ - 4)), g.nmax1 + 4);
  const int hslot = top ? tid : tid + 8;
  // Clamped row offsets for the adjoint's v^2 in shared memory.
  int zp[5], zm[5];
#pragma unroll
  for (int l = 1; l <= 4; ++l) {
    zp[l] = tid + 4 + (min(g.nmax1, i + l) - i);
    zm[l] = tid + 4 - (i - max(g.nmin1, i - l));
  }
  // 32-bit element offsets: the runner keeps every padded array below 2^31.
  const int rowbase = (int)g.idx(ir, 0, 1);     // idx(ir, j, 1) = rowbase + j*L
  const int hbase = (int)g.idx(hrow, 0, 1);
  const int pbase = (int)g.idx(min(i, g.nmax1), 0, 1);
  // Register window: w[l] = u2(ir, j-4+l); for the adjoint wv[l] = v^2(ir, j-4+l).
  float w[9], wv[9];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    w[l] = u2[rowbase + (j0 - 4 + l) * L];
    if (ADJ) {
      const float vv = vel[rowbase + (j0 - 4 + l) * L];
      wv[l] = vv * vv;
    }
  }
  w[8] = 0.f;
  wv[8] = 0.f;
  // Prefetch registers for column j.
  float n_u2 = u2[rowbase + (j0 + 4) * L];
  float n_v = ADJ ? vel[rowbase + (j0 + 4) * L] : vel[pbase + j0 * L];
  float n_u1 = 0.f, n_u0 = 0.f, n_um1 = 0.f;
  if (row_ok) {
    n_u1 = u1[pbase + j0 * L];
    n_u0 = u0[pbase + j0 * L];
    n_um1 = um1[pbase + j0 * L];
  }
  float n_h = (top || bot) ? u2[hbase + j0 * L] : 0.f;
  float n_hv = (ADJ && (top || bot)) ? vel[hbase + j0 * L] : 0.f;
  const bool snapstep = (it % S.snapi) == 0;
  const long long nphys = (long long)g.nz * g.nx * g.ny;
  int buf = 0;
  for (int j = j0; j < j1; ++j, buf ^= 1) {
    const float c_u2 = n_u2, c_v = n_v, c_u1 = n_u1, c_u0 = n_u0, c_um1 = n_um1, c_h = n_h,
                c_hv = n_hv;
    if (j + 1 < j1) {
      const int jn = (j + 1) * L;
      n_u2 = u2[rowbase + jn + 4 * L];
      n_v = ADJ ? vel[rowbase + jn + 4 * L] : vel[pbase + jn];
      if (row_ok) {
        n_u1 = u1[pbase + jn];
        n_u0 = u0[pbase + jn];
        n_um1 = um1[pbase + jn];
      }
      if (top || bot) {
        n_h = u2[hbase + jn];
        if (ADJ) n_hv = vel[hbase + jn];
      }
    }
    w[8] = c_u2;
    if (ADJ) wv[8] = c_v * c_v;
    sm.u[buf][tid + 4] = w[4];
    if (ADJ) sm.v2[buf][tid + 4] = wv[4];
    if (top || bot) {
      sm.u[buf][hslot] = c_h;
      if (ADJ) sm.v2[buf][hslot] = c_hv * c_hv;
    }
    __syncthreads();
    if (row_ok) {
      const float *su = sm.u[buf];
      float sv;
      if (!ADJ) {
        // FD_2nd_2D_derivatives_scalar_forward_grid (FDderivatives.f90:715-743).
        float tzz = c.c0z * su[tid + 4];
        tzz = tzz + c.c1z * (su[tid + 5] + su[tid + 3]);
        tzz = tzz + c.c2z * (su[tid + 6] + su[tid + 2]);
        tzz = tzz + c.c3z * (su[tid + 7] + su[tid + 1]);
        tzz = tzz + c.c4z * (su[tid + 8] + su[tid + 0]);
        float txx = c.c0x * w[4];
        txx = txx + c.c1x * (w[5] + w[3]);
        txx = txx + c.c2x * (w[6] + w[2]);
        txx = txx + c.c3x * (w[7] + w[1]);
        txx = txx + c.c4x * (w[8] + w[0]);
        sv = (c_v * c_v) * (txx + tzz);
      } else {
        // FD_2nd_2D_derivatives_scalar_adjoint_grid (FDderivatives.f90:847-891):
        // v^2 taken at indices clamped to the compute domain.
        const float *sv2 = sm.v2[buf];
        float tzz = c.c0z * (sv2[tid + 4] * su[tid + 4]);
        tzz = tzz + c.c1z * (sv2[zp[1]] * su[tid + 5] + sv2[zm[1]] * su[tid + 3]);
        tzz = tzz + c.c2z * (sv2[zp[2]] * su[tid + 6] + sv2[zm[2]] * su[tid + 2]);
        tzz = tzz + c.c3z * (sv2[zp[3]] * su[tid + 7] + sv2[zm[3]] * su[tid + 1]);
        tzz = tzz + c.c4z * (sv2[zp[4]] * su[tid + 8] + sv2[zm[4]] * su[tid + 0]);
        float vp[5], vm[5];
        if (j - 4 >= g.nmin2 && j + 4 <= g.nmax2) {
#pragma unroll
          for (int l = 1; l <= 4; ++l) {
            vp[l] = wv[4 + l];
            vm[l] = wv[4 - l];
          }
        } else {
          const int rp = g.nmax2 - j, rm = j - g.nmin2;   // >= 0
#pragma unroll
          for (int l = 1; l <= 4; ++l) {
            const int ap = min(l, rp), am = min(l, rm);
            vp[l] = ap == 0 ? wv[4] : ap == 1 ? wv[5] : ap == 2 ? wv[6] : ap == 3 ? wv[7] : wv[8];
            vm[l] = am == 0 ? wv[4] : am == 1 ? wv[3] : am == 2 ? wv[2] : am == 3 ? wv[1] : wv[0];
          }
        }
        float txx = c.c0x * (wv[4] * w[4]);
        txx = txx + c.c1x * (vp[1] * w[5] + vm[1] * w[3]);
        txx = txx + c.c2x * (vp[2] * w[6] + vm[2] * w[2]);
        txx = txx + c.c3x * (vp[3] * w[7] + vm[3] * w[1]);
        txx = txx + c.c4x * (vp[4] * w[8] + vm[4] * w[0]);
        sv = txx + tzz;
      }
      // Injection (Injection.f90:151-456, 561-591), sources in order.
      if (S.inj_on && i >= S.bi0 && i <= S.bi1 && j >= S.bj0 && j <= S.bj1) {
        const int bx = (i - S.bi0) + (S.bi1 - S.bi0 + 1) * (j - S.bj0);
        const int e1 = S.inj_off[bx + 1];
        for (int e = S.inj_off[bx]; e < e1; ++e) {
          const InjEntry E = S.inj_ent[e];
          const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
          sv = sv + (((E.v2r * tr) * E.wz) * E.wx) * E.wy;
        }
      }
      const int p = pbase + j * L;
      const bool phys = i >= 1 && i <= g.nz && j >= 1 && j <= g.nx;
      int cnt = 0;
      long long pp = 0;
      float taper = 1.f;
      if (phys && snapstep) {
        pp = (long long)(i - 1) + (long long)g.nz * (j - 1);
        if (S.taperx) taper = S.taperx[j - 1] * S.tapery[0];
        cnt = S.tstep > 0 ? it / S.snapi - (S.tcnt - 1) / S.snapi
                          : S.tcnt / S.snapi - (it - 1) / S.snapi;
        // Injection_Born (Imaging.f90:747-788).
        if (S.imaging == 4 && S.tstep > 0 && cnt <= S.ntsnap) {
          const float vc = ADJ ? vel[p] : c_v;
          sv = sv + (((2.0f * taper) * S.ref[pp]) * S.wave[(long long)(cnt - 1) * nphys + pp]) / vc;
        }
      }
      // FD_2nd_time_derivative_grid (FDderivatives.f90:960-982).
      const float u2c = w[4];
      float a = 20.0f * u2c;
      a = a - 6.0f * c_u1;
      a = a - 4.0f * c_u0;
      a = a + c_um1;
      a = a + k12 * sv;
      u3[p] = a * div11;
      if (phys && snapstep) {
        if (S.extract_wave && cnt <= S.ntsnap) S.wave[(long long)(cnt - 1) * nphys + pp] = u2c;
        if (S.imaging >= 1 && S.imaging <= 3 && S.tstep < 0) {
          const int index = S.ntsnap - cnt + 1;
          if (index >= 1) {
            const float wsn = S.wave[(long long)(index - 1) * nphys + pp];
            const float vc = ADJ ? vel[p] : c_v;
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
      }
    }
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      w[l] = w[l + 1];
      if (ADJ) wv[l] = wv[l + 1];
    }
  }
}

}  // namespace swave
