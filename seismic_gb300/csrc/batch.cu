// batch.cu - multi-shot time-step kernels (compiled with --fmad=false).
//
// One launch of each kernel covers every shot of a batch; the time step s
// comes from a device counter so that the launches of all steps are
// identical and graph-capturable.  The arithmetic restates the reference
// loops in their evaluation order (file:line cited at each kernel).
#include <algorithm>

#include "batch.cuh"
#include "higdon.cuh"
#include "stream2d.cuh"
#include "stream3d.cuh"
#include "tile2d.cuh"
#include "tile2d2.cuh"
#include "tile3d.cuh"

namespace swave {

__device__ __forceinline__ int find_shot(const int *start, int n, int idx) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= idx) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Number of snapshot steps (it multiple of snapi) met so far in this phase,
// counting the current one: the value of wfld%counter / model%counter in
// Extraction_wavefield (Extraction.f90:574-575) and the imaging conditions
// (Imaging.f90:242-244, 760-762).
__device__ __forceinline__ int snap_count(const ShotDev &S, int it) {
  if (S.tstep > 0) return it / S.snapi - (S.tcnt - 1) / S.snapi;
  return S.tcnt / S.snapi - (it - 1) / S.snapi;
}

__device__ __forceinline__ float lap_axis(const float *__restrict__ u, long long p, long long s,
                                          float c0, float c1, float c2, float c3, float c4) {
  float t = c0 * u[p];
  t = t + c1 * (u[p + s] + u[p - s]);
  t = t + c2 * (u[p + 2 * s] + u[p - 2 * s]);
  t = t + c3 * (u[p + 3 * s] + u[p - 3 * s]);
  t = t + c4 * (u[p + 4 * s] + u[p - 4 * s]);
  return t;
}

__device__ __forceinline__ void step_tail(const ShotDev &S, const Geom &g, int i, int j, int k,
                                          long long p, int it, float sv, float u2c, float u1c,
                                          float u0c, float um1c, const float *__restrict__ u2,
                                          float *__restrict__ u3, bool snapstep, bool maybe_inj);

// ---------------------------------------------------------------------------
// Fused step: stencil -> injection -> Born source -> 5-level time update,
// with the snapshot and imaging reads of u2 (Propagator.f90:182-218).
// ---------------------------------------------------------------------------
template <bool TWO_D>
__global__ void __launch_bounds__(256) k_bstep(BatchTables t, int s_off) {
  const int b = find_shot(t.step_tiles, t.nshots, blockIdx.x);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;
  const Geom &g = S.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
  const int ntz = (n1 + 31) >> 5, ntx = (n2 + 7) >> 3;
  int local = blockIdx.x - t.step_tiles[b];
  const int tz = local % ntz;
  local /= ntz;
  const int tx = local % ntx;
  const int kk = local / ntx;
  const int i = g.nmin1 + tz * 32 + threadIdx.x;
  const int j = g.nmin2 + tx * 8 + threadIdx.y;
  const int k = TWO_D ? 1 : g.nmin3 + kk;
  if (i > g.nmax1 || j > g.nmax2) return;
  const int it = S.tmin + s * S.tstep;
  const float *__restrict__ um1 = S.f[s % 5];
  const float *__restrict__ u0 = S.f[(s + 1) % 5];
  const float *__restrict__ u1 = S.f[(s + 2) % 5];
  const float *__restrict__ u2 = S.f[(s + 3) % 5];
  float *__restrict__ u3 = S.f[(s + 4) % 5];
  const long long p = g.idx(i, j, k);
  const long long L = g.ld1;
  const Coefs &c = S.c;
  float sv;
  if (S.rho_on) {
    // Divergence of the staggered gradient times v^2*rho
    // (FDderivatives.f90:371-380 3D, 642-655 2D).
    const Coefs &r = S.cr;
    const float *__restrict__ sz = S.sz;
    const float *__restrict__ sx = S.sx;
    float tz = r.c1z * (sz[p] - sz[p - 1]);
    tz = tz + r.c2z * (sz[p + 1] - sz[p - 2]);
    tz = tz + r.c3z * (sz[p + 2] - sz[p - 3]);
    tz = tz + r.c4z * (sz[p + 3] - sz[p - 4]);
    float tx = r.c1x * (sx[p] - sx[p - L]);
    tx = tx + r.c2x * (sx[p + L] - sx[p - 2 * L]);
    tx = tx + r.c3x * (sx[p + 2 * L] - sx[p - 3 * L]);
    tx = tx + r.c4x * (sx[p + 3 * L] - sx[p - 4 * L]);
    const float vv = S.vel[p];
    const float vr = (vv * vv) * S.rho[p];
    if (TWO_D) {
      sv = vr * (tx + tz);
    } else {
      const long long P = g.plane();
      const float *__restrict__ sy = S.sy;
      float ty = r.c1y * (sy[p] - sy[p - P]);
      ty = ty + r.c2y * (sy[p + P] - sy[p - 2 * P]);
      ty = ty + r.c3y * (sy[p + 2 * P] - sy[p - 3 * P]);
      ty = ty + r.c4y * (sy[p + 3 * P] - sy[p - 4 * P]);
      sv = vr * ((tx + ty) + tz);
    }
  } else if (TWO_D && S.adj2d) {
    // FD_2nd_2D_derivatives_scalar_adjoint_grid (FDderivatives.f90:847-891):
    // vel indices clamped to the compute domain.
    const float *__restrict__ v = S.vel;
    auto w = [&](long long pu, long long pv) -> float {
      const float vv = v[pv];
      return (vv * vv) * u2[pu];
    };
    long long pz[5], mz[5], px[5], mx[5];
#pragma unroll
    for (int l = 1; l <= 4; ++l) {
      pz[l] = p + (min(g.nmax1, i + l) - i);
      mz[l] = p - (i - max(g.nmin1, i - l));
      px[l] = p + L * (min(g.nmax2, j + l) - j);
      mx[l] = p - L * (j - max(g.nmin2, j - l));
    }
    float tzz = c.c0z * w(p, p);
    tzz = tzz + c.c1z * (w(p + 1, pz[1]) + w(p - 1, mz[1]));
    tzz = tzz + c.c2z * (w(p + 2, pz[2]) + w(p - 2, mz[2]));
    tzz = tzz + c.c3z * (w(p + 3, pz[3]) + w(p - 3, mz[3]));
    tzz = tzz + c.c4z * (w(p + 4, pz[4]) + w(p - 4, mz[4]));
    float txx = c.c0x * w(p, p);
    txx = txx + c.c1x * (w(p + L, px[1]) + w(p - L, mx[1]));
    txx = txx + c.c2x * (w(p + 2 * L, px[2]) + w(p - 2 * L, mx[2]));
    txx = txx + c.c3x * (w(p + 3 * L, px[3]) + w(p - 3 * L, mx[3]));
    txx = txx + c.c4x * (w(p + 4 * L, px[4]) + w(p - 4 * L, mx[4]));
    sv = txx + tzz;
  } else {
    // FD_2nd_{2D,3D}_derivatives_scalar_forward_grid (FDderivatives.f90:
    // 715-743, 97-131).  For the 3D adjoint (FDderivatives.f90:780-819)
    // the Laplacian acts on v^2*u2 and the v^2 factor is skipped.
    const float *__restrict__ u = (!TWO_D && S.adj3d) ? S.v2u : u2;
    const float tzz = lap_axis(u, p, 1, c.c0z, c.c1z, c.c2z, c.c3z, c.c4z);
    const float txx = lap_axis(u, p, L, c.c0x, c.c1x, c.c2x, c.c3x, c.c4x);
    if (TWO_D) {
      const float vv = S.vel[p];
      sv = (vv * vv) * (txx + tzz);
    } else {
      const float tyy = lap_axis(u, p, g.plane(), c.c0y, c.c1y, c.c2y, c.c3y, c.c4y);
      if (S.adj3d) {
        sv = (txx + tzz) + tyy;
      } else {
        const float vv = S.vel[p];
        sv = (vv * vv) * ((txx + tzz) + tyy);
      }
    }
  }
  step_tail(S, g, i, j, k, p, it, sv, u2[p], u1[p], u0[p], um1[p], u2, u3, (it % S.snapi) == 0,
            true);
}

// The part of a point update after the spatial operator sv: injection, the
// Born source, the 5-level time update of u3, the snapshot save and the
// imaging conditions on u2, for the point (i, j, k) at padded offset p of
// step it.  u2c, u1c, u0c, um1c are the point's values of u2, u1, u0 and
// u_1; snapstep says whether it is a multiple of snapi; maybe_inj false
// says the point lies outside the shot's injection box.
__device__ __forceinline__ void step_tail(const ShotDev &S, const Geom &g, int i, int j, int k,
                                          long long p, int it, float sv, float u2c, float u1c,
                                          float u0c, float um1c, const float *__restrict__ u2,
                                          float *__restrict__ u3, bool snapstep, bool maybe_inj) {
  // Injection (Injection.f90:151-456, 561-591): contributions in source order.
  if (maybe_inj && S.inj_on && i >= S.bi0 && i <= S.bi1 && j >= S.bj0 && j <= S.bj1 && k >= S.bk0 &&
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
  // Under a free surface the rows above it are stored as zero and take no
  // imaging or Born source (Extraction.f90:580-592, Imaging.f90:248-258).
  const bool below = i >= S.irow0;
  int cnt = 0;
  long long pp = 0;
  float taper = 1.f;
  if (phys) {
    pp = g.pidx(i, j, k);
    if (S.taperx) taper = S.taperx[j - 1] * S.tapery[k - 1];
    if (snapstep) cnt = snap_count(S, it);
  }
  const long long nphys = (long long)g.nz * g.nx * g.ny;
  // Injection_Born (Imaging.f90:747-788), tstep = +1 only.
  if (S.imaging == 4 && S.tstep > 0 && phys && below && snapstep && cnt <= S.ntsnap) {
    const float *w0 = S.wave + (long long)(cnt - 1) * nphys;
    sv = sv + (((2.0f * taper) * S.ref[pp]) * w0[pp]) / S.vel[p];
  }
  // FD_2nd_time_derivative_grid (FDderivatives.f90:960-982).
  float a = 20.0f * u2c;
  a = a - 6.0f * u1c;
  a = a - 4.0f * u0c;
  a = a + um1c;
  a = a + S.k12 * sv;
  u3[p] = a * S.div11;
  if (phys && snapstep) {
    // Extraction_wavefield (Extraction.f90:562-601).
    if (S.extract_wave && cnt <= S.ntsnap)
      S.wave[(long long)(cnt - 1) * nphys + pp] = below ? u2c : 0.f;
    // Imaging conditions on u2 before the step, tstep = -1 (Propagator.f90:192-194).
    if (S.imaging >= 1 && S.imaging <= 3 && S.tstep < 0 && below) {
      const int index = S.ntsnap - cnt + 1;
      if (index >= 1) {
        const float w = S.wave[(long long)(index - 1) * nphys + pp];
        float im = S.image[pp];
        if (S.imaging == 1) {
          im = im + (u2c * w) * taper;                            // Imaging.f90:265
        } else if (S.imaging == 2) {
          im = im + (((2.0f * taper) * u2c) * w) / S.vel[p];      // Imaging.f90:735
        } else {
          const int ip1 = min(index + 1, S.ntsnap), im1 = max(index - 1, 1);
          const float vv = S.vel[p];
          const float tt = ((S.wave[(long long)(im1 - 1) * nphys + pp] - 2.0f * w) +
                            S.wave[(long long)(ip1 - 1) * nphys + pp]) /
                           (S.dt2snap * ((vv * vv) * vv));
          im = im + (u2c * tt) * taper;                           // Imaging.f90:410-411
        }
        S.image[pp] = im;
        S.illum[pp] = S.illum[pp] + (w * w) * taper;
      }
    }
    // Imaging_condition_AFWI_RHOVP_from_memory (Imaging.f90:424-511): forward
    // differences of u2 and of the snapshot (backward ones on the last row
    // and column; none along y in 2D), the second time difference of the
    // snapshots, and the velocity and density gradients.
    if (S.imaging == 5 && S.tstep < 0 && below) {   // SW_IMG_AFWI_RHO
      const int index = S.ntsnap - cnt + 1;
      if (index >= 1) {
        const int ip1 = min(index + 1, S.ntsnap), im1 = max(index - 1, 1);
        const float *wi = S.wave + (long long)(index - 1) * nphys;
        const int dk = g.ny == 1 ? 0 : 1;
        const int ip = min(g.nz, i + 1), jp = min(j + 1, g.nx), kp = min(k + dk, g.ny);
        const int im = ip - 1, jm = jp - 1, km = kp - dk;
        const float dzi = S.dzi, dxi = S.dxi, dyi = S.dyi;   // 1/delta (rho setup)
        const float dti2 = 1.0f / S.dt2snap;
        auto U = [&](int a, int b2, int c2) { return u2[g.idx(a, b2, c2)]; };
        auto Wv = [&](int a, int b2, int c2) { return wi[g.pidx(a, b2, c2)]; };
        float tmp = dzi * (U(ip, jm, km) - U(im, jm, km)) * dzi * (Wv(ip, jm, km) - Wv(im, jm, km));
        tmp = tmp + dxi * (U(im, jp, km) - U(im, jm, km)) * dxi * (Wv(im, jp, km) - Wv(im, jm, km));
        tmp = tmp + dyi * (U(im, jm, kp) - U(im, jm, km)) * dyi * (Wv(im, jm, kp) - Wv(im, jm, km));
        const float w = wi[pp];
        const float tmp1 = u2c * dti2 *
                           ((S.wave[(long long)(im1 - 1) * nphys + pp] - 2.0f * w) +
                            S.wave[(long long)(ip1 - 1) * nphys + pp]);
        const float vv = S.vel[p], rr = S.rho[p];
        S.image[pp] = S.image[pp] + ((2.0f * tmp1) * taper) / (((vv * vv) * vv) * rr);
        S.image2[pp] = S.image2[pp] + (tmp * taper) / (rr * rr) +
                       (tmp1 * taper) / ((rr * rr) * (vv * vv));
        S.illum[pp] = S.illum[pp] + (w * w) * taper;
      }
    }
  }
}

// v^2*u2 over the padded array (FDderivatives.f90:789-790), 3D adjoint only.
__global__ void k_bv2u(BatchTables t, int s_off) {
  const int b = find_shot(t.v2u_blocks, t.nshots, blockIdx.x);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (!S.adj3d || s >= S.nsteps) return;
  const float *__restrict__ u2 = S.f[(s + 3) % 5];
  const long long n = S.g.total();
  const int nb = t.v2u_blocks[b + 1] - t.v2u_blocks[b];
  for (long long q = (long long)(blockIdx.x - t.v2u_blocks[b]) * blockDim.x + threadIdx.x; q < n;
       q += (long long)nb * blockDim.x) {
    const float v = S.vel[q];
    S.v2u[q] = (v * v) * u2[q];
  }
}

// Snapshot save and RTM / LSRTM / AFWI imaging of step s for the 3D shots
// of the pipelined kernel (the post-update part of t3_extras, which that
// kernel leaves to this one): one thread per physical point, z fastest, on
// u2 of the step (the level the step kernel read, unchanged by it).  Per
// element the operations of Propagator.f90:182-218 and Imaging.f90 as in
// t3_extras.
__global__ void k_bsnap3d(BatchTables t, int s_off) {
  const int b = find_shot(t.snap_blocks, t.nshots, blockIdx.x);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;
  const int it = S.tmin + s * S.tstep;
  if ((it % S.snapi) != 0) return;
  const Geom &g = S.g;
  const int cnt = S.tstep > 0 ? it / S.snapi - (S.tcnt - 1) / S.snapi
                              : S.tcnt / S.snapi - (it - 1) / S.snapi;
  const bool save = S.extract_wave && cnt <= S.ntsnap;
  const int index = S.ntsnap - cnt + 1;
  const bool img = S.imaging >= 1 && S.imaging <= 3 && S.tstep < 0 && index >= 1;
  if (!save && !img) return;
  const float *__restrict__ u2 = S.f[(s + 3) % S.nbuf];
  const long long nphys = (long long)g.nz * g.nx * g.ny;
  float *ws = save ? S.wave + (long long)(cnt - 1) * nphys : nullptr;
  const float *wr = img ? S.wave + (long long)(index - 1) * nphys : nullptr;
  const float *wrm = nullptr, *wrp = nullptr;
  if (img && S.imaging == 3) {
    wrm = S.wave + (long long)(max(index - 1, 1) - 1) * nphys;
    wrp = S.wave + (long long)(min(index + 1, S.ntsnap) - 1) * nphys;
  }
  // One element: its u2 (and velocity), the saved snapshot, the image and
  // illumination update.
  auto point = [&](long long q, int i, int j, int k) {
    const long long p = g.idx(i, j, k);
    const float u2c = u2[p];
    if (ws) ws[q] = u2c;
    if (!wr) return;
    const float taper = S.taperx ? S.taperx[j - 1] * S.tapery[k - 1] : 1.f;
    const float wsn = wr[q];
    float im = S.image[q];
    if (S.imaging == 1) {
      im = im + (u2c * wsn) * taper;
    } else if (S.imaging == 2) {
      im = im + (((2.0f * taper) * u2c) * wsn) / S.vel[p];
    } else {
      const float vc = S.vel[p];
      const float tt = ((wrm[q] - 2.0f * wsn) + wrp[q]) / (S.dt2snap * ((vc * vc) * vc));
      im = im + (u2c * tt) * taper;
    }
    S.image[q] = im;
    S.illum[q] = S.illum[q] + (wsn * wsn) * taper;
  };
  const int nb = t.snap_blocks[b + 1] - t.snap_blocks[b];
  const long long first = (long long)(blockIdx.x - t.snap_blocks[b]) * blockDim.x + threadIdx.x;
  const long long stride = (long long)nb * blockDim.x;
  if ((g.nz & 3) == 0 && nphys < (1LL << 31)) {
    // 4 consecutive rows of a column per thread, 32-bit index arithmetic.
    const unsigned nz = (unsigned)g.nz, nx = (unsigned)g.nx;
    const bool al = ((reinterpret_cast<uintptr_t>(ws) | reinterpret_cast<uintptr_t>(wr) |
                      reinterpret_cast<uintptr_t>(wrm) | reinterpret_cast<uintptr_t>(wrp) |
                      reinterpret_cast<uintptr_t>(S.image) | reinterpret_cast<uintptr_t>(S.illum)) &
                     15) == 0;
    for (long long w = first; w < nphys / 4; w += stride) {
      const unsigned q = 4u * (unsigned)w;
      const unsigned col = q / nz;
      const int i0 = (int)(q - col * nz) + 1, j = (int)(col % nx) + 1, k = (int)(col / nx) + 1;
      if (!al || S.imaging == 3) {
#pragma unroll
        for (int r = 0; r < 4; ++r) point((long long)q + r, i0 + r, j, k);
        continue;
      }
      // 16-byte snapshot, image and illumination accesses; per element the
      // operations of point().
      const long long p = g.idx(i0, j, k);
      const float u[4] = {u2[p], u2[p + 1], u2[p + 2], u2[p + 3]};
      if (ws) *reinterpret_cast<float4 *>(ws + q) = make_float4(u[0], u[1], u[2], u[3]);
      if (!wr) continue;
      const float taper = S.taperx ? S.taperx[j - 1] * S.tapery[k - 1] : 1.f;
      const float4 w4 = *reinterpret_cast<const float4 *>(wr + q);
      const float4 m4 = *reinterpret_cast<const float4 *>(S.image + q);
      const float4 l4 = *reinterpret_cast<const float4 *>(S.illum + q);
      const float wsn[4] = {w4.x, w4.y, w4.z, w4.w};
      float im[4] = {m4.x, m4.y, m4.z, m4.w}, il[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if (S.imaging == 1) im[r] = im[r] + (u[r] * wsn[r]) * taper;
        else im[r] = im[r] + (((2.0f * taper) * u[r]) * wsn[r]) / S.vel[p + r];
        il[r] = il[r] + (wsn[r] * wsn[r]) * taper;
      }
      *reinterpret_cast<float4 *>(S.image + q) = make_float4(im[0], im[1], im[2], im[3]);
      *reinterpret_cast<float4 *>(S.illum + q) = make_float4(il[0], il[1], il[2], il[3]);
    }
  } else {
    for (long long q = first; q < nphys; q += stride) {
      const int i = (int)(q % g.nz) + 1;
      const long long r = q / g.nz;
      point(q, i, (int)(r % g.nx) + 1, (int)(r / g.nx) + 1);
    }
  }
}

// Staggered gradient of u2 scaled by delp = 1/rho2 for the variable-density
// operator (FDderivatives.f90:277-336 3D, 601-640 2D): the 8th-order
// difference at half cells inside the compute domain, a first-order
// difference scaled by delp of the adjacent face in the three padding cells
// beyond each face.  Only the cells the divergence reads are written; the
// fourth padding cell, which the reference reads but never writes, stays at
// its initial zero.
__global__ void k_brho_grad(BatchTables t, int s_off) {
  const int b = find_shot(t.v2u_blocks, t.nshots, blockIdx.x);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (!S.rho_on || s >= S.nsteps) return;
  const Geom &g = S.g;
  const float *__restrict__ u = S.f[(s + 3) % 5];
  const float *__restrict__ dp = S.delp;
  const Coefs &c = S.cr;
  const long long n = (long long)g.n1p * g.n2p * g.n3p;
  const long long L = g.ld1, P = g.plane();
  const int nb = t.v2u_blocks[b + 1] - t.v2u_blocks[b];
  // 32-bit index arithmetic (the padded grid of one shot has fewer than
  // 2^31 points, checked when the batch is set up).
  const unsigned n1p = (unsigned)g.n1p, n2p = (unsigned)g.n2p;
  for (long long q = (long long)(blockIdx.x - t.v2u_blocks[b]) * blockDim.x + threadIdx.x; q < n;
       q += (long long)nb * blockDim.x) {
    const unsigned uq = (unsigned)q, rr = uq / n1p;
    const int i = g.lo1 + (int)(uq - rr * n1p);
    const int j = g.lo2 + (int)(rr % n2p), k = g.lo3 + (int)(rr / n2p);
    const bool iin = i >= g.nmin1 && i <= g.nmax1, jin = j >= g.nmin2 && j <= g.nmax2;
    const bool kin = g.twoD || (k >= g.nmin3 && k <= g.nmax3);
    const long long p = g.idx(i, j, k);
    if (jin && kin) {
      if (iin) {
        float a = c.c1z * (u[p + 1] - u[p]);
        a = a + c.c2z * (u[p + 2] - u[p - 1]);
        a = a + c.c3z * (u[p + 3] - u[p - 2]);
        a = a + c.c4z * (u[p + 4] - u[p - 3]);
        S.sz[p] = a * dp[p];
      } else if (i >= g.nmin1 - 3 && i <= g.nmax1 + 3) {
        const int ie = i < g.nmin1 ? g.nmin1 : g.nmax1;
        S.sz[p] = (S.dzi * (u[p + 1] - u[p])) * dp[g.idx(ie, j, k)];
      }
    }
    if (iin && kin) {
      if (jin) {
        float a = c.c1x * (u[p + L] - u[p]);
        a = a + c.c2x * (u[p + 2 * L] - u[p - L]);
        a = a + c.c3x * (u[p + 3 * L] - u[p - 2 * L]);
        a = a + c.c4x * (u[p + 4 * L] - u[p - 3 * L]);
        S.sx[p] = a * dp[p];
      } else if (j >= g.nmin2 - 3 && j <= g.nmax2 + 3) {
        const int je = j < g.nmin2 ? g.nmin2 : g.nmax2;
        S.sx[p] = (S.dxi * (u[p + L] - u[p])) * dp[g.idx(i, je, k)];
      }
    }
    if (!g.twoD && iin && jin) {
      if (kin) {
        float a = c.c1y * (u[p + P] - u[p]);
        a = a + c.c2y * (u[p + 2 * P] - u[p - P]);
        a = a + c.c3y * (u[p + 3 * P] - u[p - 2 * P]);
        a = a + c.c4y * (u[p + 4 * P] - u[p - 3 * P]);
        S.sy[p] = a * dp[p];
      } else if (k >= g.nmin3 - 3 && k <= g.nmax3 + 3) {
        const int ke = k < g.nmin3 ? g.nmin3 : g.nmax3;
        S.sy[p] = (S.dyi * (u[p + P] - u[p])) * dp[g.idx(i, j, ke)];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The 2D variable-density step in one pass (FDderivatives.f90:601-657 and
// the time update): each block owns a tile of 64 (z) x 32 (x) outputs.  At
// its start it issues asynchronous 16-byte copies (cp.async, zero-filled
// outside the padded array) of every input into shared memory: u2 with an
// 8-cell halo (80 x 48), delp with a 4-cell halo (72 x 40), and the tile's
// v, rho, u1, u0 and u_1 (64 x 32 each).  It then forms the staggered
// gradients the tile's divergence reads - sz on rows z0-4..z0+67 of the
// tile's columns, sx on columns x0-4..x0+35 of its rows - with the
// operations and padding-cell rules of k_brho_grad, and finally the
// divergence times v^2*rho and the rest of the point update (step_tail).
// sz and sx never go through HBM: 32 bytes per point (u2, delp, v, rho, u1,
// u0, u_1 read, u3 written) instead of the two passes' 52.
// ---------------------------------------------------------------------------
constexpr int R2_Z = 64, R2_X = 32;
constexpr int R2_UZ = R2_Z + 16, R2_UX = R2_X + 16;   // staged u2: rows z0-8.., columns x0-8..
constexpr int R2_GZ = R2_Z + 8, R2_GX = R2_X + 8;     // delp and sz rows z0-4.., sx columns x0-4..
constexpr int R2_CORE = R2_Z * R2_X;
// Shared-memory layout in floats, every array [column][row].
constexpr int R2_SU = 0;                                // u2, R2_UX x R2_UZ
constexpr int R2_SDP = R2_SU + R2_UX * R2_UZ;           // delp, R2_GX x R2_GZ
constexpr int R2_SC = R2_SDP + R2_GX * R2_GZ;           // v, rho, u1, u0, u_1: 5 x R2_CORE
constexpr int R2_SSZ = R2_SC + 5 * R2_CORE;             // sz, R2_X x R2_GZ
constexpr int R2_SSX = R2_SSZ + R2_X * R2_GZ;           // sx, R2_GX x R2_Z
constexpr int R2_FLOATS = R2_SSX + R2_GX * R2_Z;
constexpr size_t R2_SMEM = sizeof(float) * R2_FLOATS;   // 87 296 bytes: two blocks per SM
// 16-byte chunks of the staged arrays.
constexpr int R2_QU = R2_UX * (R2_UZ / 4), R2_QD = R2_GX * (R2_GZ / 4), R2_QC = R2_X * (R2_Z / 4);

// 16-byte asynchronous global -> shared copy; with in false nothing is read
// and the destination is zero-filled.
__device__ __forceinline__ void cp_async16(float *dst, const float *src, bool in) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(in ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
// Waits until at most N of this thread's committed groups are in flight.
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// step_tail of one point of k_brho2d's tiles that carry injection or
// snapshot work, kept out of line so that the common path stays small.
__device__ __noinline__ void rho_tail(const ShotDev &S, int i, int j, int p, int it, float sv,
                                      float u2c, float u1c, float u0c, float um1c,
                                      const float *u2, float *u3, bool snapstep, bool inj) {
  step_tail(S, S.g, i, j, 1, p, it, sv, u2c, u1c, u0c, um1c, u2, u3, snapstep, inj);
}

// Four consecutive shared-memory floats (16-byte aligned) into r[0..3].
__device__ __forceinline__ void lds4_to(float *r, const float *p) {
  const float4 v = *reinterpret_cast<const float4 *>(p);
  r[0] = v.x;
  r[1] = v.y;
  r[2] = v.z;
  r[3] = v.w;
}

__global__ void __launch_bounds__(256, 2) k_brho2d(BatchTables t, int s_off) {
  extern __shared__ __align__(16) float r2s[];
  float *su = r2s + R2_SU, *sdp = r2s + R2_SDP, *sc = r2s + R2_SC;
  float *ssz = r2s + R2_SSZ, *ssx = r2s + R2_SSX;
  const int b = find_shot(t.step_tiles, t.nshots, blockIdx.x);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;   // the whole block
  const Geom &g = S.g;
  const int nmin1 = g.nmin1, nmax1 = g.nmax1, nmin2 = g.nmin2, nmax2 = g.nmax2;
  const int lo1 = g.lo1, lo2 = g.lo2, ld = g.ld1, n2p = g.n2p;
  const int ntz = (nmax1 - nmin1 + R2_Z) / R2_Z;
  const int local = blockIdx.x - t.step_tiles[b];
  const int z0 = nmin1 + (local % ntz) * R2_Z, x0 = nmin2 + (local / ntz) * R2_X;
  const int tid = threadIdx.x;
  const float *__restrict__ u2 = S.f[(s + 3) % 5];
  float *__restrict__ u3 = S.f[(s + 4) % 5];
  // 32-bit offsets in the padded array (fewer than 2^31 points per shot,
  // checked when the batch is set up).
  auto off = [&](int i, int j) { return (i - lo1) + ld * (j - lo2); };
  // Every chunk starts 4k rows after the padded array's first row (z0 - lo1
  // = 64 t + 4), so a chunk lies wholly inside a column's ld1 rows or wholly
  // outside them; the arrays are 256-byte aligned and ld1 is a multiple of
  // 32, so every source address is 16-byte aligned.  Cells beyond the
  // padded array (zero-filled, or rows n1p..ld1-1 of a column) feed no value
  // that a stored output depends on: the gradients read rows
  // nmin1-3..nmax1+4 and columns nmin2-3..nmax2+4 of u2.
  auto stage = [&](float *dst, const float *src, int i0, int j) {
    const bool in = i0 >= lo1 && i0 < lo1 + ld && j >= lo2 && j < lo2 + n2p;
    cp_async16(dst, in ? src + off(i0, j) : src, in);
  };
  for (int q = tid; q < R2_QU; q += 256) {
    const int cc = q / (R2_UZ / 4), k = q - cc * (R2_UZ / 4);
    stage(su + cc * R2_UZ + 4 * k, u2, z0 - 8 + 4 * k, x0 - 8 + cc);
  }
  for (int q = tid; q < R2_QD; q += 256) {
    const int cc = q / (R2_GZ / 4), k = q - cc * (R2_GZ / 4);
    stage(sdp + cc * R2_GZ + 4 * k, S.delp, z0 - 4 + 4 * k, x0 - 4 + cc);
  }
  cp_async_commit();   // group 1: what the gradients read
  {
    // v, rho, then u1, u0, u_1 (levels s+2, s+1, s of the 5-level ring):
    // two chunks of each per thread.
    static_assert(R2_QC == 2 * 256, "core chunks per thread");
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      const float *src = a == 0 ? S.vel : a == 1 ? S.rho : S.f[(s + 4 - a) % 5];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = tid + 256 * h, cc = q >> 4, k = q & 15;
        stage(sc + a * R2_CORE + cc * R2_Z + 4 * k, src, z0 + 4 * k, x0 + cc);
      }
    }
  }
  cp_async_commit();   // group 2: the point update's inputs
  // The shot's scalars, loaded while the copies are in flight.
  const Coefs &cf = S.cr;
  const float c1z = cf.c1z, c2z = cf.c2z, c3z = cf.c3z, c4z = cf.c4z;
  const float c1x = cf.c1x, c2x = cf.c2x, c3x = cf.c3x, c4x = cf.c4x;
  const float dzi = S.dzi, dxi = S.dxi;
  const int it = S.tmin + s * S.tstep;
  const bool snapstep = (it % S.snapi) == 0;
  const bool inj_tile = S.inj_on && !(z0 + R2_Z - 1 < S.bi0 || z0 > S.bi1 ||
                                      x0 + R2_X - 1 < S.bj0 || x0 > S.bj1);
  // Without injection in the tile and without snapshot or imaging work in
  // the step, step_tail reduces to the time update (FDderivatives.f90:
  // 960-982), done below on four rows at once.
  const bool heavy = inj_tile || (snapstep && (S.imaging != 0 || S.extract_wave));
  const float k12 = S.k12, div11 = S.div11;
  cp_async_wait<1>();
  __syncthreads();
  // sz at rows z0-4+rr..+3 of column x0+cc, four rows per item: the
  // 8th-order difference times delp inside the compute domain, the
  // first-order one times delp of the face in the three padding cells, 0
  // beyond (the fourth padding cell, which the reference reads and never
  // writes) and off the compute columns.  delp at (i, j) is
  // sdp[(j - x0 + 4) * R2_GZ + i - z0 + 4]; a face row or column that a
  // padding cell of the tile needs lies inside the staged 72 x 40 block
  // (z0 >= nmin1, x0 >= nmin2).
  // A tile whose gradient cells all lie inside the compute domain (most of
  // them) takes the 8th-order difference everywhere, without the per-cell
  // domain and padding tests.
  const bool interior = z0 - 4 >= nmin1 && z0 + R2_Z + 3 <= nmax1 && x0 - 4 >= nmin2 &&
                        x0 + R2_X + 3 <= nmax2;
  if (interior) {
    for (int q = tid; q < R2_X * (R2_GZ / 4); q += 256) {
      const int cc = q / (R2_GZ / 4), rr = 4 * (q - cc * (R2_GZ / 4));
      float U[12], D[4], v[4];
      const float *col = su + (cc + 8) * R2_UZ + rr;
      lds4_to(U, col);
      lds4_to(U + 4, col + 4);
      lds4_to(U + 8, col + 8);
      lds4_to(D, sdp + (cc + 4) * R2_GZ + rr);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float a = c1z * (U[e + 5] - U[e + 4]);
        a = a + c2z * (U[e + 6] - U[e + 3]);
        a = a + c3z * (U[e + 7] - U[e + 2]);
        a = a + c4z * (U[e + 8] - U[e + 1]);
        v[e] = a * D[e];
      }
      *reinterpret_cast<float4 *>(ssz + cc * R2_GZ + rr) = make_float4(v[0], v[1], v[2], v[3]);
    }
    for (int q = tid; q < R2_GX * (R2_Z / 4); q += 256) {
      const int cc = q >> 4, rr = 4 * (q & 15);
      float V[8][4], D[4], v[4];
#pragma unroll
      for (int m = 0; m < 8; ++m) lds4_to(V[m], su + (cc + 1 + m) * R2_UZ + rr + 8);
      lds4_to(D, sdp + cc * R2_GZ + rr + 4);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float a = c1x * (V[4][e] - V[3][e]);
        a = a + c2x * (V[5][e] - V[2][e]);
        a = a + c3x * (V[6][e] - V[1][e]);
        a = a + c4x * (V[7][e] - V[0][e]);
        v[e] = a * D[e];
      }
      *reinterpret_cast<float4 *>(ssx + cc * R2_Z + rr) = make_float4(v[0], v[1], v[2], v[3]);
    }
  } else {
    for (int q = tid; q < R2_X * (R2_GZ / 4); q += 256) {
      const int cc = q / (R2_GZ / 4), rr = 4 * (q - cc * (R2_GZ / 4));
      const int i0 = z0 - 4 + rr, j = x0 + cc;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (j <= nmax2) {
        // u2 at rows i0-3..i0+7 of column j: staged rows rr+1..rr+11.
        float U[12], D[4];
        const float *col = su + (cc + 8) * R2_UZ + rr;
        lds4_to(U, col);
        lds4_to(U + 4, col + 4);
        lds4_to(U + 8, col + 8);
        const float *dcol = sdp + (cc + 4) * R2_GZ;
        lds4_to(D, dcol + rr);
  #pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          if (i >= nmin1 && i <= nmax1) {
            float a = c1z * (U[e + 5] - U[e + 4]);
            a = a + c2z * (U[e + 6] - U[e + 3]);
            a = a + c3z * (U[e + 7] - U[e + 2]);
            a = a + c4z * (U[e + 8] - U[e + 1]);
            v[e] = a * D[e];
          } else if (i >= nmin1 - 3 && i <= nmax1 + 3) {
            const int ie = i < nmin1 ? nmin1 : nmax1;
            v[e] = (dzi * (U[e + 5] - U[e + 4])) * dcol[ie - z0 + 4];
          }
        }
      }
      *reinterpret_cast<float4 *>(ssz + cc * R2_GZ + rr) = make_float4(v[0], v[1], v[2], v[3]);
    }
    // sx at rows z0+rr..+3 of column x0-4+cc, by the same rules along x.
    for (int q = tid; q < R2_GX * (R2_Z / 4); q += 256) {
      const int cc = q >> 4, rr = 4 * (q & 15);
      const int i0 = z0 + rr, j = x0 - 4 + cc;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      const bool jin = j >= nmin2 && j <= nmax2;
      if (i0 <= nmax1 && (jin || (j >= nmin2 - 3 && j <= nmax2 + 3))) {
        // u2 at columns j-3..j+4 of rows i0..i0+3: V[m] is column j-3+m.
        float V[8][4], D[4];
  #pragma unroll
        for (int m = 0; m < 8; ++m) lds4_to(V[m], su + (cc + 1 + m) * R2_UZ + rr + 8);
        const int je = jin ? j : (j < nmin2 ? nmin2 : nmax2);
        lds4_to(D, sdp + (je - x0 + 4) * R2_GZ + rr + 4);
  #pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (i0 + e > nmax1) continue;
          if (jin) {
            float a = c1x * (V[4][e] - V[3][e]);
            a = a + c2x * (V[5][e] - V[2][e]);
            a = a + c3x * (V[6][e] - V[1][e]);
            a = a + c4x * (V[7][e] - V[0][e]);
            v[e] = a * D[e];
          } else {
            v[e] = (dxi * (V[4][e] - V[3][e])) * D[e];
          }
        }
      }
      *reinterpret_cast<float4 *>(ssx + cc * R2_Z + rr) = make_float4(v[0], v[1], v[2], v[3]);
    }
  }
  cp_async_wait<0>();
  __syncthreads();
  // Divergence times v^2*rho (FDderivatives.f90:642-655) and the point
  // update, four rows per item: lanes 0-15 of a warp take the 16 row
  // groups of one column, lanes 16-31 those of the next.
  const int rr = 4 * (tid & 15);
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    const int cc = (tid >> 4) + 16 * h, j = x0 + cc, i0 = z0 + rr;
    if (j > nmax2 || i0 > nmax1) continue;
    // sz at rows i0-4..i0+7: Z[m] is row i0-4+m.
    float Z[12];
    const float *zc = ssz + cc * R2_GZ + rr;
    lds4_to(Z, zc);
    lds4_to(Z + 4, zc + 4);
    lds4_to(Z + 8, zc + 8);
    // sx at columns j-4..j+3: X[m] is column j-4+m.
    float X[8][4];
#pragma unroll
    for (int m = 0; m < 8; ++m) lds4_to(X[m], ssx + (cc + m) * R2_Z + rr);
    float VV[4], RH[4], A1[4], A0[4], AM[4], U2[4];
    const float *cv = sc + cc * R2_Z + rr;
    lds4_to(VV, cv);
    lds4_to(RH, cv + R2_CORE);
    lds4_to(A1, cv + 2 * R2_CORE);
    lds4_to(A0, cv + 3 * R2_CORE);
    lds4_to(AM, cv + 4 * R2_CORE);
    lds4_to(U2, su + (cc + 8) * R2_UZ + rr + 8);
    float sv[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      float tz = c1z * (Z[e + 4] - Z[e + 3]);
      tz = tz + c2z * (Z[e + 5] - Z[e + 2]);
      tz = tz + c3z * (Z[e + 6] - Z[e + 1]);
      tz = tz + c4z * (Z[e + 7] - Z[e + 0]);
      float tx = c1x * (X[4][e] - X[3][e]);
      tx = tx + c2x * (X[5][e] - X[2][e]);
      tx = tx + c3x * (X[6][e] - X[1][e]);
      tx = tx + c4x * (X[7][e] - X[0][e]);
      const float vr = (VV[e] * VV[e]) * RH[e];
      sv[e] = vr * (tx + tz);
    }
    const int p0 = off(i0, j);
    if (heavy) {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (i0 + e <= nmax1)
          rho_tail(S, i0 + e, j, p0 + e, it, sv[e], U2[e], A1[e], A0[e], AM[e], u2, u3, snapstep,
                   inj_tile);
      continue;
    }
    float o[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      float a = 20.0f * U2[e];
      a = a - 6.0f * A1[e];
      a = a - 4.0f * A0[e];
      a = a + AM[e];
      a = a + k12 * sv[e];
      o[e] = a * div11;
    }
    if (i0 + 3 <= nmax1) {
      *reinterpret_cast<float4 *>(u3 + p0) = make_float4(o[0], o[1], o[2], o[3]);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (i0 + e <= nmax1) u3[p0 + e] = o[e];
    }
  }
}

static cudaError_t launch_rho2d(const BatchTables &t, int s_off, int n_tiles, cudaStream_t s) {
  // The shared-memory opt-in is a per-device function attribute.
  static unsigned long long attr_set = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !(attr_set & (1ull << dev))) {
    e = cudaFuncSetAttribute(k_brho2d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)R2_SMEM);
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_set |= 1ull << dev;
  }
  k_brho2d<<<n_tiles, 256, R2_SMEM, s>>>(t, s_off);
  return cudaGetLastError();
}

// Sinc gather of one receiver in the loop order of Extraction_1trace_sinc_xy
// (Extraction.f90:511-560) / _xyz (Extraction.f90:276-337).  H is the
// half-width when known at compile time (lsinc = 7), else -1.
// ---------------------------------------------------------------------------
// Receiver extraction (Extraction.f90:71-135, 217-247, 276-337, 511-560):
// one warp per receiver.  The lanes form the lsinc^2 (3D: lsinc^3) products
// of a sinc gather 32 at a time, and lane 0 adds them to the trace sample
// one by one in the reference's loop order (z fastest, then x, then y).
// ---------------------------------------------------------------------------
__global__ void k_bextract(BatchTables t, int s_off) {
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int ntot = t.rec_start[t.nshots];
  if (q >= ntot) return;   // uniform per warp
  const int b = find_shot(t.rec_start, t.nshots, q);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps || S.ext_mode == 0) return;
  const int r = q - t.rec_start[b];
  const int it = S.tmin + s * S.tstep;
  const Geom &g = S.g;
  const float *__restrict__ u2 = S.f[(s + 3) % S.nbuf];
  const int i0 = S.ric[3 * r], j0 = S.ric[3 * r + 1], k0 = g.twoD ? 1 : S.ric[3 * r + 2];
  float *trp = S.rec_tr + (long long)r * S.nt + (it - 1);
  if (S.ext_mode == 2) {  // Extraction_array_simple_afwi_noomp
    if (lane == 0) {
      if (S.ext_mirror) *trp = *trp + (u2[g.idx(i0, j0, k0)] - u2[g.idx(-i0, j0, k0)]);
      else *trp = *trp + u2[g.idx(i0, j0, k0)];
    }
    return;
  }
  float v;
  if (S.ext_mode == 1) {  // Extraction_array_sinc: v**2 in 2D, v in 3D
    const float vv = S.vel[g.idx(i0, j0, k0)];
    v = g.twoD ? vv * vv : vv;
  } else {
    v = S.vconst;
  }
  const int h = S.ext_half, ls = 2 * h + 1;
  const int ntap = g.twoD ? ls * ls : ls * ls * ls;
  const float *wz = S.wz + (long long)r * ls, *wx = S.wx + (long long)r * ls;
  float tr = lane == 0 ? *trp : 0.f;
  for (int c0 = 0; c0 < ntap; c0 += 32) {
    const int tp = c0 + lane;
    float prod = 0.f;
    if (tp < ntap) {
      const int ii = tp % ls, rest = tp / ls;
      const int jj = rest % ls, kq = rest / ls;
      const int kc = g.twoD ? 1 : k0 - h + kq;
      const long long p = g.idx(i0 - h + ii, j0 - h + jj, kc);
      // A mirror receiver takes u minus u at the row reflected through row 0
      // (Extraction.f90:549-555, 324-333).
      const float uv = S.ext_mirror ? u2[p] - u2[g.idx(h - ii - i0, j0 - h + jj, kc)] : u2[p];
      prod = ((v * uv) * wz[ii]) * wx[jj];
      if (!g.twoD) prod = prod * wx[kq];     // the y weights are the x column
    }
    const int nlane = min(32, ntap - c0);
    for (int l = 0; l < nlane; ++l) {
      const float pl = __shfl_sync(0xffffffffu, prod, l);
      tr = tr + pl;
    }
  }
  if (lane == 0) *trp = tr;
}

// ---------------------------------------------------------------------------
// Higdon recurrences (Boundary_3d, Boundary.f90:89-184; Higdon_factor,
// Boundary.f90:366-447) for the kernels that do not apply them in the tile.
// ---------------------------------------------------------------------------


// Fused 2D edges: the z (top, bottom) and x (left, right) Higdon
// recurrences of one step in one launch.  Each half line loads its 10 u2 and
// u1 values, two u3 values and 8 coefficients first and then runs the 8-cell
// recurrence in registers.  The reference applies all z lines and then all x
// lines; only the x half lines of the 4 rows next to a z edge read or
// overwrite cells the z half lines write (columns within 6 of an x edge),
// so each corner is one warp that runs those 6 z half lines, synchronises
// and then runs the 4 x half lines.  Every other half line is independent.
__global__ void __launch_bounds__(128) k_bedges2d(BatchTables t, int s_off) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= t.edge_start[t.nshots]) return;
  const int b = find_shot(t.edge_start, t.nshots, q);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;   // uniform over the shot's warps
  const Geom &g = S.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
  const float *u1 = S.f[(s + 2) % 5], *u2 = S.f[(s + 3) % 5];
  float *u3 = S.f[(s + 4) % 5];
  const long long L = g.ld1;
  const long long csz = n2, csx = n1;
  // z half line of column j (bottom: the 8 coefficients after the top's).
  auto zhalf = [&](int j, int bottom) {
    const float *gc = S.gz + (j - g.nmin2) + (bottom ? 8 * csz : 0);
    if (!bottom) higdon_half(gc, csz, u1, u2, u3, g.idx(g.nmin1 + 3, j, g.nmin3), 1);
    else higdon_half(gc, csz, u1, u2, u3, g.idx(g.nmax1 - 3, j, g.nmin3), -1);
  };
  auto xhalf = [&](int i, int right) {
    const float *gc = S.gx + (i - g.nmin1) + (right ? 8 * csx : 0);
    if (!right) higdon_half(gc, csx, u1, u2, u3, g.idx(i, g.nmin2 + 3, g.nmin3), L);
    else higdon_half(gc, csx, u1, u2, u3, g.idx(i, g.nmax2 - 3, g.nmin3), -L);
  };
  const int local = q - t.edge_start[b];
  if (local < 128) {
    const int w = local >> 5, lane = local & 31;
    const int bottom = w & 1, right = w >> 1;
    if (lane < 6) zhalf(right ? g.nmax2 - lane : g.nmin2 + lane, bottom);
    __syncwarp();
    if (lane < 4) xhalf(bottom ? g.nmax1 - lane : g.nmin1 + lane, right);
    return;
  }
  int r = local - 128;
  const int nz_rest = n2 - 12, nx_rest = n1 - 8;
  if (r < 2 * nz_rest) {
    const int bottom = r >= nz_rest;
    zhalf(g.nmin2 + 6 + (bottom ? r - nz_rest : r), bottom);
    return;
  }
  r -= 2 * nz_rest;
  if (r < 2 * nx_rest) {
    const int right = r >= nx_rest;
    xhalf(g.nmin1 + 4 + (right ? r - nx_rest : r), right);
  }
}

// One thread per half line (line = q / 2, half = q % 2: the near and the far
// edge are independent); z lines (n2*n3 per shot), x lines (n1*n3), y lines
// (n1*n2, 3D only), launched in that order like the reference's loops.
// Boundary_set_free_surface_grid (Boundary.f90:1609-1658) on u2 of the
// step, one thread per (x, y) column of a shot with a free surface: zero the
// rows above the surface row ielev, then write the mirror image of the rows
// below it with the opposite sign, on the grid (the surface on a row) or
// through the sinc weights fs_sinc (the surface between rows).
__global__ void k_bfree(BatchTables t, int s_off) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= t.hz_start[t.nshots]) return;
  const int b = find_shot(t.hz_start, t.nshots, q);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (!S.surf || s >= S.nsteps) return;
  const Geom &g = S.g;
  const int n2 = g.nmax2 - g.nmin2 + 1;
  const long long l = q - t.hz_start[b];
  const int j = g.nmin2 + (int)(l % n2), k = g.nmin3 + (int)(l / n2);
  float *u2 = S.f[(s + 3) % 5];
  const int ie = S.ielev;
  for (int i = g.nmin1; i <= ie - 1; ++i) u2[g.idx(i, j, k)] = 0.f;
  if (S.fs_grid) {
    for (int i = 0; i <= 2; ++i) u2[g.idx(ie - 2 - i, j, k)] = -u2[g.idx(ie + i, j, k)];
    return;
  }
  const int h = S.ext_half;
  float ui[15];
  for (int i = -h; i <= h; ++i) {
    float f = 0.f;
    for (int l2 = -h; l2 <= h; ++l2) f = f + u2[g.idx(ie + l2 + i, j, k)] * S.fs_sinc[h + l2];
    ui[h + i] = f;
  }
  for (int i = 2; i <= h + 1; ++i)
    for (int l2 = -h; l2 <= i - 1; ++l2) {
      const long long p = g.idx(ie - i + l2, j, k);
      u2[p] = u2[p] - ui[h + i - 1] * S.fs_sinc[h + l2];
    }
}

__global__ void k_bhiggz(BatchTables t, int s_off) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if ((q >> 1) >= t.hz_start[t.nshots]) return;
  const int b = find_shot(t.hz_start, t.nshots, q >> 1);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;
  const Geom &g = S.g;
  const int n2 = g.nmax2 - g.nmin2 + 1;
  const long long l = (q >> 1) - t.hz_start[b];
  const int j = g.nmin2 + (int)(l % n2), k = g.nmin3 + (int)(l / n2);
  if ((q & 1) == 0 && S.surf) return;   // a free surface: the top does not absorb
  higdon_zline(S, j, k, (q & 1) != 0, S.f[(s + 2) % 5], S.f[(s + 3) % 5], S.f[(s + 4) % 5]);
}

__global__ void k_bhiggx(BatchTables t, int s_off) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if ((q >> 1) >= t.hx_start[t.nshots]) return;
  const int b = find_shot(t.hx_start, t.nshots, q >> 1);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;
  const Geom &g = S.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  const long long l = (q >> 1) - t.hx_start[b];
  const long long cs = (long long)n1 * n3;
  const int i = g.nmin1 + (int)(l % n1), k = g.nmin3 + (int)(l / n1);
  if (S.surf && i < 1) return;   // side lines from row 1 under a free surface
  const float *u1 = S.f[(s + 2) % 5], *u2 = S.f[(s + 3) % 5];
  float *u3 = S.f[(s + 4) % 5];
  const long long L = g.ld1;
  if ((q & 1) == 0) higdon_half(S.gx + l, cs, u1, u2, u3, g.idx(i, g.nmin2 + 3, k), L);
  else higdon_half(S.gx + l + 8 * cs, cs, u1, u2, u3, g.idx(i, g.nmax2 - 3, k), -L);
}

__global__ void k_bhiggy(BatchTables t, int s_off) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if ((q >> 1) >= t.hy_start[t.nshots]) return;
  const int b = find_shot(t.hy_start, t.nshots, q >> 1);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps || S.g.nbound == 0) return;
  const Geom &g = S.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
  const long long l = (q >> 1) - t.hy_start[b];
  const long long cs = (long long)n1 * n2;
  const int i = g.nmin1 + (int)(l % n1), j = g.nmin2 + (int)(l / n1);
  if (S.surf && i < 1) return;   // side lines from row 1 under a free surface
  const float *u1 = S.f[(s + 2) % 5], *u2 = S.f[(s + 3) % 5];
  float *u3 = S.f[(s + 4) % 5];
  const long long P = g.plane();
  if ((q & 1) == 0) higdon_half(S.gy + l, cs, u1, u2, u3, g.idx(i, j, g.nmin3 + 3), P);
  else higdon_half(S.gy + l + 8 * cs, cs, u1, u2, u3, g.idx(i, j, g.nmax3 - 3), -P);
}

// Streaming 2D step (stream2d.cuh); the shot's stencil variant is uniform
// over the CTA.
// Streaming 2D step (stream2d.cuh): one kernel per stencil variant; a CTA
// whose shot uses the other variant exits at once.
template <int TZ, bool ADJ>
__global__ void __launch_bounds__(TZ, 1024 / TZ) k_bstep2d_s(BatchTables t, int s_off, int tx) {
  const int b = find_shot(t.step_tiles, t.nshots, blockIdx.x);
  if ((t.shots[b].adj2d != 0) != ADJ) return;
  stream2d_body<TZ, ADJ>(t, s_off, b, blockIdx.x - t.step_tiles[b], tx);
}

template <int TZ>
static void launch_stream2d(const BatchTables &t, int s_off, int n, const StepTile &tile,
                            int has_fwd, int has_adj, cudaStream_t s, int *nl) {
  if (has_fwd) {
    k_bstep2d_s<TZ, false><<<n, TZ, 0, s>>>(t, s_off, tile.tx);
    ++*nl;
  }
  if (has_adj) {
    k_bstep2d_s<TZ, true><<<n, TZ, 0, s>>>(t, s_off, tile.tx);
    ++*nl;
  }
}

// Persistent pipelined 2D step (tile2d.cuh), one kernel per stencil variant.
template <bool ADJ>
__global__ void __launch_bounds__(256, 2) k_bstep2d_t(BatchTables t, int s_off, int n_tiles) {
  tile2d_persistent<ADJ>(t, s_off, n_tiles);
}

// Two CTAs per SM: 228 KB of shared memory per SM, 1 KB reserved per CTA.
static_assert(2 * (t2_smem_bytes<false>() + 1024) <= 228 * 1024, "tile kernel smem (fwd)");
static_assert(2 * (t2_smem_bytes<true>() + 1024) <= 228 * 1024, "tile kernel smem (adj)");

template <bool ADJ>
static cudaError_t launch_tile2d(const BatchTables &t, int s_off, int n_tiles, int nsm,
                                 cudaStream_t s) {
  // The shared-memory opt-in is a per-device function attribute.
  static unsigned long long attr_set = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !(attr_set & (1ull << dev))) {
    e = cudaFuncSetAttribute(k_bstep2d_t<ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)t2_smem_bytes<ADJ>());
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_set |= 1ull << dev;
  }
  // Two resident CTAs per SM; more CTAs only when a CTA's tile list would
  // overflow its shared-memory copy.
  const int grid = std::max({1, std::min(n_tiles, 2 * nsm),
                             (n_tiles + T2_MAX_TILES_PER_CTA - 1) / T2_MAX_TILES_PER_CTA});
  // Programmatic dependent launch: the CTAs of this step start (shot tables
  // into shared memory, barriers) as the previous kernel's CTAs retire, and
  // wait in the kernel before touching its results.
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = t2_smem_bytes<ADJ>();
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, k_bstep2d_t<ADJ>, t, s_off, n_tiles);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Two-step persistent 2D kernel (tile2d2.cuh): one CTA of 512 threads per SM.
template <bool ADJ>
__global__ void __launch_bounds__(TF_THREADS, 1) k_bstep2d_f(BatchTables t, int s_off,
                                                            int n_tiles) {
  tile2d_fused<ADJ>(t, s_off, n_tiles);
}

static_assert(tf_smem_bytes<false>() + 1024 <= 228 * 1024, "two-step kernel smem (fwd)");
static_assert(tf_smem_bytes<true>() + 1024 <= 228 * 1024, "two-step kernel smem (adj)");

template <bool ADJ>
static cudaError_t launch_tile2d_f(const BatchTables &t, int s_off, int n_tiles, int nsm,
                                   cudaStream_t s) {
  static unsigned long long attr_set = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !(attr_set & (1ull << dev))) {
    e = cudaFuncSetAttribute(k_bstep2d_f<ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tf_smem_bytes<ADJ>());
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_set |= 1ull << dev;
  }
  const int grid = std::max({1, std::min(n_tiles, nsm),
                             (n_tiles + TF_MAX_TILES_PER_CTA - 1) / TF_MAX_TILES_PER_CTA});
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(TF_THREADS);
  cfg.dynamicSmemBytes = tf_smem_bytes<ADJ>();
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, k_bstep2d_f<ADJ>, t, s_off, n_tiles);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Warp-specialised persistent 2D step (tile2d.cuh): one CTA per SM.
static_assert(t2w_smem_bytes<false>() <= 227 * 1024, "ws tile kernel smem (fwd)");
static_assert(t2w_smem_bytes<true>() <= 227 * 1024, "ws tile kernel smem (adj)");

template <bool ADJ>
__global__ void __launch_bounds__(T2W_THREADS, 1) k_bstep2d_w(BatchTables t, int s_off,
                                                              int n_tiles) {
  tile2d_ws<ADJ>(t, s_off, n_tiles);
}

template <bool ADJ>
static cudaError_t launch_tile2d_ws(const BatchTables &t, int s_off, int n_tiles, int nsm,
                                    cudaStream_t s) {
  static unsigned long long attr_set = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !(attr_set & (1ull << dev))) {
    e = cudaFuncSetAttribute(k_bstep2d_w<ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)t2w_smem_bytes<ADJ>());
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_set |= 1ull << dev;
  }
  const int grid = std::max({1, std::min(n_tiles, nsm),
                             (n_tiles + T2_MAX_TILES_PER_CTA - 1) / T2_MAX_TILES_PER_CTA});
  k_bstep2d_w<ADJ><<<grid, T2W_THREADS, t2w_smem_bytes<ADJ>(), s>>>(t, s_off, n_tiles);
  return cudaGetLastError();
}

// TMA-pipelined persistent 3D step (tile3d.cuh), one kernel per variant.
static_assert(2 * (t3_smem_bytes<false>() + 1024) <= 228 * 1024, "3D tile kernel smem (fwd)");
static_assert(2 * (t3_smem_bytes<true>() + 1024) <= 228 * 1024, "3D tile kernel smem (adj)");

template <bool ADJ>
__global__ void __launch_bounds__(256, 2) k_bstep3d_t(BatchTables t, int s_off, int n_units) {
  tile3d_persistent<ADJ>(t, s_off, n_units);
}

template <bool ADJ>
static cudaError_t launch_tile3d(const BatchTables &t, int s_off, int n_units, int nsm,
                                 cudaStream_t s) {
  static unsigned long long attr_set = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !(attr_set & (1ull << dev))) {
    e = cudaFuncSetAttribute(k_bstep3d_t<ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)t3_smem_bytes<ADJ>());
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_set |= 1ull << dev;
  }
  const int grid = std::max({1, std::min(n_units, 2 * nsm),
                             (n_units + T3_MAX_UNITS_PER_CTA - 1) / T3_MAX_UNITS_PER_CTA});
  k_bstep3d_t<ADJ><<<grid, 256, t3_smem_bytes<ADJ>(), s>>>(t, s_off, n_units);
  return cudaGetLastError();
}

// Streaming 3D step (stream3d.cuh), one kernel per stencil variant.
template <bool ADJ>
__global__ void __launch_bounds__(256, 4) k_bstep3d_s(BatchTables t, int s_off, int ty) {
  const int b = find_shot(t.step_tiles, t.nshots, blockIdx.x);
  if ((t.shots[b].adj3d != 0) != ADJ) return;
  stream3d_body<ADJ>(t, s_off, b, blockIdx.x - t.step_tiles[b], ty);
}

__global__ void k_counter_add(int *counter, int add) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *counter += add;
}

// Injection terms of the step, one thread per (shot, entry):
// term = (((v2r * trace(it)) * wz) * wx) * wy (Injection.f90:151-456,
// 561-591); the step kernel adds a cell's terms in entry order.
// sub = 1 forms the terms of the second step of a two-step launch (step
// s_off - 1 + 1 of the counter) into the second block of inj_term.
__global__ void k_bterms(BatchTables t, int s_off, int sub) {
  // The next (step) kernel may start at once: it reads nothing this kernel
  // or the previous step writes before its own wait, which returns only
  // after this kernel completes - and this kernel completes only after the
  // previous step kernel, which still reads the terms overwritten here.
  pdl_launch_dependents();
  pdl_wait();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= t.term_start[t.nshots]) return;
  const int b = find_shot(t.term_start, t.nshots, q);
  const ShotDev &S = t.shots[b];
  const int s = *t.counter + s_off;
  if (s >= S.nsteps) return;
  const int k = q - t.term_start[b];
  const int it = S.tmin + s * S.tstep;
  const InjEntry E = S.inj_ent[k];
  const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
  S.inj_term[(long long)sub * S.inj_nterm + k] = (((E.v2r * tr) * E.wz) * E.wx) * E.wy;
}

cudaError_t launch_batch_step(const BatchTables &t, int s_off, int n_step_tiles, int n_rec,
                              int n_hz, int n_hx, int n_hy, int n_v2u, int has_ext, int has_3d,
                              int has_adj3d, const StepTile &tile, cudaStream_t s,
                              int *nlaunch, cudaEvent_t ev_before, cudaEvent_t ev_after,
                              int n_term) {
  int nl = 0;
  // Every kernel of the step reads s = *counter + s_off; the counter is
  // advanced once per chunk of steps.
  if (has_ext && n_rec > 0) {
    k_bextract<<<(n_rec + 3) / 4, 128, 0, s>>>(t, s_off);
    ++nl;
  }
  if (n_term > 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((n_term + 255) / 256);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_bterms, t, s_off, 0);
    if (e != cudaSuccess) return e;
    ++nl;
  }
  if (has_adj3d && n_v2u > 0 && !tile.stream3d) {
    k_bv2u<<<n_v2u, 256, 0, s>>>(t, s_off);
    ++nl;
  }
  if (tile.has_surf && n_hz > 0) {
    k_bfree<<<(n_hz + 127) / 128, 128, 0, s>>>(t, s_off);
    ++nl;
  }
  if (tile.has_rho && n_v2u > 0 && !tile.rho2d) {
    k_brho_grad<<<n_v2u, 256, 0, s>>>(t, s_off);
    ++nl;
  }
  dim3 bs(32, 8, 1);
  // Inside stream capture the records must be external nodes (a plain
  // record only adds a dependency and would never timestamp the event at
  // graph replay); outside capture a plain record is required.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (ev_before || ev_after) {
    cudaError_t ec = cudaStreamIsCapturing(s, &cap);
    if (ec != cudaSuccess) return ec;
  }
  auto record = [&](cudaEvent_t ev) {
    return cap == cudaStreamCaptureStatusActive
               ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
               : cudaEventRecord(ev, s);
  };
  if (ev_before) {
    cudaError_t ec = record(ev_before);
    if (ec != cudaSuccess) return ec;
  }
  if (has_3d && tile.stream3d == 2) {
    cudaError_t e = cudaSuccess;
    if (tile.has_fwd3d) {
      e = launch_tile3d<false>(t, s_off, n_step_tiles, tile.nsm, s);
      ++nl;
    }
    if (e == cudaSuccess && tile.has_adj3d) {
      e = launch_tile3d<true>(t, s_off, n_step_tiles, tile.nsm, s);
      ++nl;
    }
    if (e != cudaSuccess) return e;
  } else if (has_3d && tile.stream3d) {
    dim3 b3(S3_BZ, S3_BY, 1);
    if (tile.has_fwd3d) {
      k_bstep3d_s<false><<<n_step_tiles, b3, 0, s>>>(t, s_off, tile.ty);
      ++nl;
    }
    if (tile.has_adj3d) {
      k_bstep3d_s<true><<<n_step_tiles, b3, 0, s>>>(t, s_off, tile.ty);
      ++nl;
    }
  } else if (has_3d) {
    k_bstep<false><<<n_step_tiles, bs, 0, s>>>(t, s_off);
    ++nl;
  } else if (tile.stream2d == 3) {
    cudaError_t e = cudaSuccess;
    if (tile.has_fwd2d) {
      e = launch_tile2d_ws<false>(t, s_off, n_step_tiles, tile.nsm, s);
      ++nl;
    }
    if (e == cudaSuccess && tile.has_adj2d) {
      e = launch_tile2d_ws<true>(t, s_off, n_step_tiles, tile.nsm, s);
      ++nl;
    }
    if (e != cudaSuccess) return e;
  } else if (tile.stream2d == 2) {
    cudaError_t e = cudaSuccess;
    if (tile.has_fwd2d) {
      e = launch_tile2d<false>(t, s_off, n_step_tiles, tile.nsm, s);
      ++nl;
    }
    if (e == cudaSuccess && tile.has_adj2d) {
      e = launch_tile2d<true>(t, s_off, n_step_tiles, tile.nsm, s);
      ++nl;
    }
    if (e != cudaSuccess) return e;
  } else if (tile.stream2d) {
    const int hf = tile.has_fwd2d, ha = tile.has_adj2d;
    if (tile.tz == 128) launch_stream2d<128>(t, s_off, n_step_tiles, tile, hf, ha, s, &nl);
    else if (tile.tz == 32) launch_stream2d<32>(t, s_off, n_step_tiles, tile, hf, ha, s, &nl);
    else launch_stream2d<64>(t, s_off, n_step_tiles, tile, hf, ha, s, &nl);
  } else if (tile.rho2d) {
    cudaError_t e = launch_rho2d(t, s_off, n_step_tiles, s);
    if (e != cudaSuccess) return e;
    ++nl;
  } else {
    k_bstep<true><<<n_step_tiles, bs, 0, s>>>(t, s_off);
    ++nl;
  }
  if (ev_after) {
    cudaError_t ec = record(ev_after);
    if (ec != cudaSuccess) return ec;
  }
  // Snapshot saves and imaging of the pipelined 3D kernel's shots.
  if (has_3d && tile.stream3d == 2 && tile.n_snap3d > 0) {
    k_bsnap3d<<<tile.n_snap3d, 256, 0, s>>>(t, s_off);
    ++nl;
  }
  if (tile.rigid) {
    // Exact-adjoint mode: no absorbing boundary, the halo stays zero.
  } else if (!has_3d && (tile.stream2d == 2 || tile.stream2d == 3)) {
    // The pipelined 2D kernel applies the Higdon edges itself.
  } else if (!has_3d && tile.fused_edges) {
    k_bedges2d<<<(tile.n_edge + 127) / 128, 128, 0, s>>>(t, s_off);
    ++nl;
  } else {
    k_bhiggz<<<(2 * n_hz + 127) / 128, 128, 0, s>>>(t, s_off);
    k_bhiggx<<<(2 * n_hx + 127) / 128, 128, 0, s>>>(t, s_off);
    nl += 2;
  }
  if (has_3d && n_hy > 0 && !tile.rigid) {
    k_bhiggy<<<(2 * n_hy + 127) / 128, 128, 0, s>>>(t, s_off);
    ++nl;
  }
  if (nlaunch) *nlaunch = nl;
  return cudaGetLastError();
}

// Two time steps s = *counter + s_off and s + 1 of a 2D batch in one
// launch of the two-step tile kernel: receiver extraction of step s, the
// injection terms of both steps, the fused kernel (stencils, time updates,
// injection, snapshots, imaging and Higdon edges of both steps), then the
// extraction of step s + 1 from the level the launch wrote.
cudaError_t launch_batch_step2(const BatchTables &t, int s_off, int n_step_tiles, int n_rec,
                               int has_ext, const StepTile &tile, cudaStream_t s, int *nlaunch,
                               cudaEvent_t ev_before, cudaEvent_t ev_after, int n_term) {
  int nl = 0;
  if (has_ext && n_rec > 0) {
    k_bextract<<<(n_rec + 3) / 4, 128, 0, s>>>(t, s_off);
    ++nl;
  }
  for (int sub = 0; sub < 2 && n_term > 0; ++sub) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((n_term + 255) / 256);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_bterms, t, s_off + sub, sub);
    if (e != cudaSuccess) return e;
    ++nl;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (ev_before || ev_after) {
    cudaError_t ec = cudaStreamIsCapturing(s, &cap);
    if (ec != cudaSuccess) return ec;
  }
  auto record = [&](cudaEvent_t ev) {
    return cap == cudaStreamCaptureStatusActive
               ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
               : cudaEventRecord(ev, s);
  };
  if (ev_before) {
    cudaError_t ec = record(ev_before);
    if (ec != cudaSuccess) return ec;
  }
  cudaError_t e = cudaSuccess;
  if (tile.has_fwd2d) {
    e = launch_tile2d_f<false>(t, s_off, n_step_tiles, tile.nsm, s);
    ++nl;
  }
  if (e == cudaSuccess && tile.has_adj2d) {
    e = launch_tile2d_f<true>(t, s_off, n_step_tiles, tile.nsm, s);
    ++nl;
  }
  if (e != cudaSuccess) return e;
  if (ev_after) {
    cudaError_t ec = record(ev_after);
    if (ec != cudaSuccess) return ec;
  }
  if (has_ext && n_rec > 0) {
    k_bextract<<<(n_rec + 3) / 4, 128, 0, s>>>(t, s_off + 1);
    ++nl;
  }
  if (nlaunch) *nlaunch = nl;
  return cudaGetLastError();
}

cudaError_t launch_counter_add(int *counter, int add, cudaStream_t s) {
  k_counter_add<<<1, 32, 0, s>>>(counter, add);
  return cudaGetLastError();
}

}  // namespace swave
