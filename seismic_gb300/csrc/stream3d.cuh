// stream3d.cuh - 2.5D streaming fused step kernel for 3D batches.
//
// A CTA of 32x8 threads owns a 32 (z) x 16 (x) column tile of one shot and
// marches along y over TY planes.  Each thread owns two x positions (j and
// j+8) and keeps, for each, the nine values at planes k-4..k+4 in
// registers (the y derivative).  Plane k of the tile plus a 4-cell halo is
// staged in shared memory for the z and x derivatives.  For the 3D adjoint
// (FDderivatives.f90:780-819) the staged and windowed values are v^2*u2,
// formed as they are loaded, so no separate pass over the grid is needed.
// The arithmetic order is the reference's (see batch.cu).
#pragma once

#include "batch.cuh"

namespace swave {

constexpr int S3_BZ = 32;   // z extent of the tile (threadIdx.x)
constexpr int S3_BY = 8;    // threadIdx.y
constexpr int S3_BX = 16;   // x extent of the tile (two points per thread)

struct Stream3dSmem {
  float t[S3_BX + 8][S3_BZ + 8];   // [x][z] plane tile with halo
};

template <bool ADJ>
__device__ __forceinline__ float s3_load(const float *__restrict__ u2,
                                         const float *__restrict__ vel, int p) {
  if (ADJ) {
    const float v = vel[p];
    return (v * v) * u2[p];
  }
  return u2[p];
}

template <bool ADJ>
__device__ __forceinline__ void stream3d_body(const BatchTables &t, int s_off, int b, int local,
                                              int TY) {
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;
  __shared__ Stream3dSmem sm;
  const Geom g = S.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
  const int ntz = (n1 + S3_BZ - 1) / S3_BZ, ntx = (n2 + S3_BX - 1) / S3_BX;
  const int tz = local % ntz;
  local /= ntz;
  const int tx = local % ntx;
  const int ty = local / ntx;
  const int lx = threadIdx.x, ly = threadIdx.y;
  const int z0 = g.nmin1 + tz * S3_BZ, x0 = g.nmin2 + tx * S3_BX;
  const int k0 = g.nmin3 + ty * TY;
  const int k1 = min(k0 + TY, g.nmax3 + 1);
  const int i = z0 + lx;
  const int ja = x0 + ly, jb = x0 + ly + 8;
  const bool okz = i <= g.nmax1;
  const bool oka = okz && ja <= g.nmax2, okb = okz && jb <= g.nmax2;
  // Clamped coordinates for loads (values outside the padded array are
  // never used by points that are computed).
  const int ic = min(i, g.nmax1 + 4);
  const int jac = min(ja, g.nmax2 + 4), jbc = min(jb, g.nmax2 + 4);
  const int it = S.tmin + s * S.tstep;
  const float *__restrict__ um1 = S.f[s % 5];
  const float *__restrict__ u0 = S.f[(s + 1) % 5];
  const float *__restrict__ u1 = S.f[(s + 2) % 5];
  const float *__restrict__ u2 = S.f[(s + 3) % 5];
  float *__restrict__ u3 = S.f[(s + 4) % 5];
  const float *__restrict__ vel = S.vel;
  const int P = (int)g.plane();
  const Coefs c = S.c;
  const float k12 = S.k12, div11 = S.div11;
  const int pa0 = (int)g.idx(ic, jac, 0), pb0 = (int)g.idx(ic, jbc, 0);   // + k*P
  float wa[9], wb[9];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    wa[l] = s3_load<ADJ>(u2, vel, pa0 + (k0 - 4 + l) * P);
    wb[l] = s3_load<ADJ>(u2, vel, pb0 + (k0 - 4 + l) * P);
  }
  wa[8] = wb[8] = 0.f;
  // Halo loads of the plane tile: z halo (8 rows x 16 columns) by threads
  // with ly < 4 (two columns each... ) and x halo (32 rows x 8 columns).
  const bool snapstep = (it % S.snapi) == 0;
  const long long nphys = (long long)g.nz * g.nx * g.ny;
  for (int k = k0; k < k1; ++k) {
    wa[8] = s3_load<ADJ>(u2, vel, pa0 + (k + 4) * P);
    wb[8] = s3_load<ADJ>(u2, vel, pb0 + (k + 4) * P);
    __syncthreads();   // previous plane's readers are done with the tile
    sm.t[ly + 4][lx + 4] = wa[4];
    sm.t[ly + 12][lx + 4] = wb[4];
    const int kP = k * P;
    // z halo: rows z0-4..z0-1 and z0+32..z0+35 for the 16 tile columns.
    if (lx < 8) {
      const int zr = lx < 4 ? z0 - 4 + lx : min(z0 + S3_BZ + (lx - 4), g.nmax1 + 4);
      const int slot = lx < 4 ? lx : S3_BZ + 4 + (lx - 4);
      sm.t[ly + 4][slot] = s3_load<ADJ>(u2, vel, (int)g.idx(zr, jac, 0) + kP);
      sm.t[ly + 12][slot] = s3_load<ADJ>(u2, vel, (int)g.idx(zr, jbc, 0) + kP);
    }
    // x halo: columns x0-4..x0-1 and x0+16..x0+19 for the 32 tile rows.
    {
      const int hx = ly;   // 0..7
      const int xc = hx < 4 ? x0 - 4 + hx : min(x0 + S3_BX + (hx - 4), g.nmax2 + 4);
      const int slot = hx < 4 ? hx : S3_BX + 4 + (hx - 4);
      sm.t[slot][lx + 4] = s3_load<ADJ>(u2, vel, (int)g.idx(ic, xc, 0) + kP);
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const bool ok = h == 0 ? oka : okb;
      if (!ok) continue;
      const float *w = h == 0 ? wa : wb;
      const int sx = (h == 0 ? ly : ly + 8) + 4, sz = lx + 4;
      const int j = h == 0 ? ja : jb;
      float tzz = c.c0z * sm.t[sx][sz];
      tzz = tzz + c.c1z * (sm.t[sx][sz + 1] + sm.t[sx][sz - 1]);
      tzz = tzz + c.c2z * (sm.t[sx][sz + 2] + sm.t[sx][sz - 2]);
      tzz = tzz + c.c3z * (sm.t[sx][sz + 3] + sm.t[sx][sz - 3]);
      tzz = tzz + c.c4z * (sm.t[sx][sz + 4] + sm.t[sx][sz - 4]);
      float txx = c.c0x * sm.t[sx][sz];
      txx = txx + c.c1x * (sm.t[sx + 1][sz] + sm.t[sx - 1][sz]);
      txx = txx + c.c2x * (sm.t[sx + 2][sz] + sm.t[sx - 2][sz]);
      txx = txx + c.c3x * (sm.t[sx + 3][sz] + sm.t[sx - 3][sz]);
      txx = txx + c.c4x * (sm.t[sx + 4][sz] + sm.t[sx - 4][sz]);
      float tyy = c.c0y * w[4];
      tyy = tyy + c.c1y * (w[5] + w[3]);
      tyy = tyy + c.c2y * (w[6] + w[2]);
      tyy = tyy + c.c3y * (w[7] + w[1]);
      tyy = tyy + c.c4y * (w[8] + w[0]);
      const int p = (int)g.idx(i, j, k);
      float sv;
      if (ADJ) {
        sv = (txx + tzz) + tyy;
      } else {
        const float vv = vel[p];
        sv = (vv * vv) * ((txx + tzz) + tyy);
      }
      if (S.inj_on && i >= S.bi0 && i <= S.bi1 && j >= S.bj0 && j <= S.bj1 && k >= S.bk0 &&
          k <= S.bk1) {
        const int bx = (i - S.bi0) + (S.bi1 - S.bi0 + 1) * ((j - S.bj0) + (S.bj1 - S.bj0 + 1) * (k - S.bk0));
        const int e1 = S.inj_off[bx + 1];
        for (int e = S.inj_off[bx]; e < e1; ++e) {
          const InjEntry E = S.inj_ent[e];
          const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
          sv = sv + (((E.v2r * tr) * E.wz) * E.wx) * E.wy;
        }
      }
      const bool phys = i >= 1 && i <= g.nz && j >= 1 && j <= g.nx && k >= 1 && k <= g.ny;
      int cnt = 0;
      long long pp = 0;
      float taper = 1.f;
      if (phys && snapstep) {
        pp = g.pidx(i, j, k);
        if (S.taperx) taper = S.taperx[j - 1] * S.tapery[k - 1];
        cnt = S.tstep > 0 ? it / S.snapi - (S.tcnt - 1) / S.snapi
                          : S.tcnt / S.snapi - (it - 1) / S.snapi;
        if (S.imaging == 4 && S.tstep > 0 && cnt <= S.ntsnap)
          sv = sv + (((2.0f * taper) * S.ref[pp]) * S.wave[(long long)(cnt - 1) * nphys + pp]) / vel[p];
      }
      const float u2c = u2[p];
      float a = 20.0f * u2c;
      a = a - 6.0f * u1[p];
      a = a - 4.0f * u0[p];
      a = a + um1[p];
      a = a + k12 * sv;
      u3[p] = a * div11;
      if (phys && snapstep) {
        if (S.extract_wave && cnt <= S.ntsnap) S.wave[(long long)(cnt - 1) * nphys + pp] = u2c;
        if (S.imaging >= 1 && S.imaging <= 3 && S.tstep < 0) {
          const int index = S.ntsnap - cnt + 1;
          if (index >= 1) {
            const float wsn = S.wave[(long long)(index - 1) * nphys + pp];
            const float vc = vel[p];
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
      wa[l] = wa[l + 1];
      wb[l] = wb[l + 1];
    }
  }
}

}  // namespace swave
