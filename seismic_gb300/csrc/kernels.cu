// kernels.cu - sm_103a kernels of libswave (compiled with --fmad=false).
//
// Each kernel restates one reference loop nest with the same floating-point
// operation order; the comments give the reference file:line.  Paths are
// relative to the reference project root.
#include "swave_dev.cuh"

namespace swave {

// ---------------------------------------------------------------------------
// Padding and coefficients
// ---------------------------------------------------------------------------

// model_pad (libs/libwave/ReadSouVelRho.f90:545-596): edge replication is
// a clamp of every padded index onto the physical window.
__global__ void k_pad_velocity(Geom g, const float *__restrict__ vp, float *__restrict__ out) {
  const long long n = (long long)g.n1p * g.n2p * g.n3p;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(q % g.n1p);
    const long long r = q / g.n1p;
    const int b = (int)(r % g.n2p);
    const int c = (int)(r / g.n2p);
    const int i = g.lo1 + a, j = g.lo2 + b, k = g.lo3 + c;
    const int ii = min(max(i, 1), g.nz), jj = min(max(j, 1), g.nx), kk = min(max(k, 1), g.ny);
    out[g.idx(i, j, k)] = vp[g.pidx(ii, jj, kk)];
  }
}

// Higdon_coeff (libs/libwave/Boundary.f90:66-87).
__device__ __forceinline__ void higdon_coeff(float nu, float *c, int stride) {
  const float beta1 = 1.0f, beta2 = 0.7f, weight = 0.5f;
  float fdum = (beta1 + nu) * (1.0f - weight);
  const float qx = (weight * (beta1 + nu) - nu) / fdum;
  const float qt = (weight * (beta1 + nu) - beta1) / fdum;
  const float qxt = weight / (weight - 1.0f);
  fdum = (beta2 + nu) * (1.0f - weight);
  const float rx = (weight * (beta2 + nu) - nu) / fdum;
  const float rt = (weight * (beta2 + nu) - beta2) / fdum;
  const float rxt = weight / (weight - 1.0f);
  c[0 * stride] = qx + rx;
  c[1 * stride] = qx * rx;
  c[2 * stride] = qt + rt;
  c[3 * stride] = ((qx * rt + qt * rx) + qxt) + rxt;
  c[4 * stride] = qx * rxt + rx * qxt;
  c[5 * stride] = qt * rt;
  c[6 * stride] = qt * rxt + rt * qxt;
  c[7 * stride] = qxt * rxt;
}

// Higdon (libs/libwave/Boundary.f90:17-63).  Layouts: gz[c][k][j],
// gx[c][k][i], gy[c][j][i].
__global__ void k_higdon_coeffs(Geom g, const float *__restrict__ vel, float dt, float dxi,
                                float dyi, float dzi, float *gz, float *gx, float *gy) {
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  const long long nzc = (long long)n2 * n3, nxc = (long long)n1 * n3;
  const long long nyc = (g.nmax3 > 1) ? (long long)n1 * n2 : 0;
  const long long tot = nzc + nxc + nyc;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < tot;
       q += (long long)gridDim.x * blockDim.x) {
    if (q < nzc) {
      const int j = g.nmin2 + (int)(q % n2), k = g.nmin3 + (int)(q / n2);
      higdon_coeff((vel[g.idx(g.nmin1, j, k)] * dt) * dzi, gz + q, (int)nzc);
      higdon_coeff((vel[g.idx(g.nmax1, j, k)] * dt) * dzi, gz + q + 8 * nzc, (int)nzc);
    } else if (q < nzc + nxc) {
      const long long r = q - nzc;
      const int i = g.nmin1 + (int)(r % n1), k = g.nmin3 + (int)(r / n1);
      higdon_coeff((vel[g.idx(i, g.nmin2, k)] * dt) * dxi, gx + r, (int)nxc);
      higdon_coeff((vel[g.idx(i, g.nmax2, k)] * dt) * dxi, gx + r + 8 * nxc, (int)nxc);
    } else {
      const long long r = q - nzc - nxc;
      const int i = g.nmin1 + (int)(r % n1), j = g.nmin2 + (int)(r / n1);
      higdon_coeff((vel[g.idx(i, j, g.nmin3)] * dt) * dyi, gy + r, (int)nyc);
      higdon_coeff((vel[g.idx(i, j, g.nmax3)] * dt) * dyi, gy + r + 8 * nyc, (int)nyc);
    }
  }
}

// ---------------------------------------------------------------------------
// Fused step: stencil -> injection -> Born source -> time update, plus the
// snapshot and imaging reads of u2 (Propagator.f90:182-218).
// ---------------------------------------------------------------------------

__device__ __forceinline__ float lap_axis(const float *__restrict__ u, long long p, long long s,
                                          float c0, float c1, float c2, float c3, float c4) {
  float t = c0 * u[p];
  t = t + c1 * (u[p + s] + u[p - s]);
  t = t + c2 * (u[p + 2 * s] + u[p - 2 * s]);
  t = t + c3 * (u[p + 3 * s] + u[p - 3 * s]);
  t = t + c4 * (u[p + 4 * s] + u[p - 4 * s]);
  return t;
}

template <bool TWO_D, bool ADJ2D>
__global__ void __launch_bounds__(256) k_step(StepArgs a) {
  const Geom &g = a.g;
  const int i = g.nmin1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.nmin2 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = TWO_D ? 1 : g.nmin3 + (int)blockIdx.z;
  if (i > g.nmax1 || j > g.nmax2) return;
  const long long p = g.idx(i, j, k);
  const long long L = g.ld1;
  const Coefs &c = a.c;
  float s;
  if (ADJ2D) {
    // FD_2nd_2D_derivatives_scalar_adjoint_grid (FDderivatives.f90:847-891).
    const float *__restrict__ u = a.u2;
    const float *__restrict__ v = a.vel;
    auto w = [&](long long pu, long long pv) -> float {
      const float vv = v[pv];
      return (vv * vv) * u[pu];
    };
    long long pz[5], mz[5], px[5], mx[5];
#pragma unroll
    for (int l = 1; l <= 4; ++l) {
      pz[l] = p + (min(g.nmax1, i + l) - i);
      mz[l] = p - (i - max(g.nmin1, i - l));
      px[l] = p + L * (min(g.nmax2, j + l) - j);
      mx[l] = p - L * (j - max(g.nmin2, j - l));
    }
    float tz = c.c0z * w(p, p);
    tz = tz + c.c1z * (w(p + 1, pz[1]) + w(p - 1, mz[1]));
    tz = tz + c.c2z * (w(p + 2, pz[2]) + w(p - 2, mz[2]));
    tz = tz + c.c3z * (w(p + 3, pz[3]) + w(p - 3, mz[3]));
    tz = tz + c.c4z * (w(p + 4, pz[4]) + w(p - 4, mz[4]));
    float tx = c.c0x * w(p, p);
    tx = tx + c.c1x * (w(p + L, px[1]) + w(p - L, mx[1]));
    tx = tx + c.c2x * (w(p + 2 * L, px[2]) + w(p - 2 * L, mx[2]));
    tx = tx + c.c3x * (w(p + 3 * L, px[3]) + w(p - 3 * L, mx[3]));
    tx = tx + c.c4x * (w(p + 4 * L, px[4]) + w(p - 4 * L, mx[4]));
    s = tx + tz;
  } else {
    // FD_2nd_{2D,3D}_derivatives_scalar_forward_grid (FDderivatives.f90:
    // 715-743, 97-131); for the 3D adjoint lap_src holds v^2*u2
    // (FDderivatives.f90:780-819) and the v^2 factor is skipped.
    const float *__restrict__ u = a.lap_src;
    const float tz = lap_axis(u, p, 1, c.c0z, c.c1z, c.c2z, c.c3z, c.c4z);
    const float tx = lap_axis(u, p, L, c.c0x, c.c1x, c.c2x, c.c3x, c.c4x);
    if (TWO_D) {
      const float vv = a.vel[p];
      s = (vv * vv) * (tx + tz);
    } else {
      const float ty = lap_axis(u, p, g.plane(), c.c0y, c.c1y, c.c2y, c.c3y, c.c4y);
      if (a.lap_src != a.u2) {
        s = (tx + tz) + ty;
      } else {
        const float vv = a.vel[p];
        s = (vv * vv) * ((tx + tz) + ty);
      }
    }
  }
  // Injection (Injection.f90:151-456,561-591): contributions in source order.
  if (a.inj_on && i >= a.bi0 && i <= a.bi1 && j >= a.bj0 && j <= a.bj1 && k >= a.bk0 &&
      k <= a.bk1) {
    const int b = (i - a.bi0) + (a.bi1 - a.bi0 + 1) * ((j - a.bj0) + (a.bj1 - a.bj0 + 1) * (k - a.bk0));
    const int e1 = a.inj_off[b + 1];
    for (int e = a.inj_off[b]; e < e1; ++e) {
      const InjEntry E = a.inj_ent[e];
      const float t = a.src_tr[(long long)E.tr * a.nt + (a.it - 1)];
      s = s + (((E.v2r * t) * E.wz) * E.wx) * E.wy;
    }
  }
  const bool phys = i >= 1 && i <= g.nz && j >= 1 && j <= g.nx && k >= 1 && k <= g.ny;
  long long pp = 0;
  float taper = 0.f;
  if (phys) {
    pp = g.pidx(i, j, k);
    taper = a.taperx ? a.taperx[j - 1] * a.tapery[k - 1] : 1.f;
  }
  // Injection_Born (Imaging.f90:747-788).
  if (a.born_on && phys) s = s + (((2.0f * taper) * a.ref[pp]) * a.w0[pp]) / a.vel[p];
  // FD_2nd_time_derivative_grid (FDderivatives.f90:960-982).
  const float u2c = a.u2[p];
  float t = 20.0f * u2c;
  t = t - 6.0f * a.u1[p];
  t = t - 4.0f * a.u0[p];
  t = t + a.um1[p];
  t = t + a.k12 * s;
  a.u3[p] = t * a.div11;
  if (phys) {
    // Extraction_wavefield (Extraction.f90:562-601).
    if (a.snap_on) a.snap_out[pp] = u2c;
    if (a.img) {
      const float w = a.w0[pp];
      float im = a.image[pp];
      if (a.img == 1) {
        im = im + (u2c * w) * taper;                              // Imaging.f90:265
      } else if (a.img == 2) {
        im = im + (((2.0f * taper) * u2c) * w) / a.vel[p];        // Imaging.f90:735
      } else {
        const float vv = a.vel[p];
        const float tt = ((a.wm1[pp] - 2.0f * w) + a.wp1[pp]) / (a.dt2snap * ((vv * vv) * vv));
        im = im + (u2c * tt) * taper;                             // Imaging.f90:410-411
      }
      a.image[pp] = im;
      a.illum[pp] = a.illum[pp] + (w * w) * taper;
    }
  }
}

// v^2*u2 over the padded array (FDderivatives.f90:790).
__global__ void k_v2u(long long n, const float *__restrict__ vel, const float *__restrict__ u2,
                      float *__restrict__ out) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float v = vel[q];
    out[q] = (v * v) * u2[q];
  }
}

// ---------------------------------------------------------------------------
// Higdon recurrences (Boundary_3d, Boundary.f90:89-184; Higdon_factor
// Boundary.f90:366-447).  Each thread owns one line along the edge normal
// and runs its eight-cell recurrence in order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float hsum(const float *__restrict__ gc, long long cs, float a, float b,
                                      float cc, float d, float e, float f, float gg, float h) {
  float r = gc[0] * a;
  r = r + gc[cs] * b;
  r = r + gc[2 * cs] * cc;
  r = r + gc[3 * cs] * d;
  r = r + gc[4 * cs] * e;
  r = r + gc[5 * cs] * f;
  r = r + gc[6 * cs] * gg;
  r = r + gc[7 * cs] * h;
  return -r;
}

// Axis 1 (top and bottom), one thread per (j, k).
__global__ void k_higdon_z(HigArgs a) {
  const Geom &g = a.g;
  const int n2 = g.nmax2 - g.nmin2 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)n2 * n3) return;
  const long long cs = (long long)n2 * n3;
  const int j = g.nmin2 + (int)(q % n2), k = g.nmin3 + (int)(q / n2);
  const float *gc = a.gz + q;
  float *u3 = a.u3;
  const float *u2 = a.u2, *u1 = a.u1;
  long long p0 = g.idx(0, j, k);  // row offset base: idx(i) = p0 + i
  for (int i = g.nmin1 + 3; i >= g.nmin1 - 4; --i) {
    const long long p = p0 + i;
    u3[p] = hsum(gc, cs, u3[p + 1], u3[p + 2], u2[p], u2[p + 1], u2[p + 2], u1[p], u1[p + 1],
                 u1[p + 2]);
  }
  gc += 8 * cs;
  for (int i = g.nmax1 - 3; i <= g.nmax1 + 4; ++i) {
    const long long p = p0 + i;
    u3[p] = hsum(gc, cs, u3[p - 1], u3[p - 2], u2[p], u2[p - 1], u2[p - 2], u1[p], u1[p - 1],
                 u1[p - 2]);
  }
}

// Axis 2 (left and right), one thread per (i, k), i = nz0..nmax1.
__global__ void k_higdon_x(HigArgs a) {
  const Geom &g = a.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)n1 * n3) return;
  const long long cs = (long long)n1 * n3;
  const int i = g.nmin1 + (int)(q % n1), k = g.nmin3 + (int)(q / n1);
  const long long L = g.ld1;
  const float *gc = a.gx + q;
  float *u3 = a.u3;
  const float *u2 = a.u2, *u1 = a.u1;
  for (int j = g.nmin2 + 3; j >= g.nmin2 - 4; --j) {
    const long long p = g.idx(i, j, k);
    u3[p] = hsum(gc, cs, u3[p + L], u3[p + 2 * L], u2[p], u2[p + L], u2[p + 2 * L], u1[p],
                 u1[p + L], u1[p + 2 * L]);
  }
  gc += 8 * cs;
  for (int j = g.nmax2 - 3; j <= g.nmax2 + 4; ++j) {
    const long long p = g.idx(i, j, k);
    u3[p] = hsum(gc, cs, u3[p - L], u3[p - 2 * L], u2[p], u2[p - L], u2[p - 2 * L], u1[p],
                 u1[p - L], u1[p - 2 * L]);
  }
}

// Axis 3 (front and back, 3D only), one thread per (i, j).
__global__ void k_higdon_y(HigArgs a) {
  const Geom &g = a.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)n1 * n2) return;
  const long long cs = (long long)n1 * n2;
  const int i = g.nmin1 + (int)(q % n1), j = g.nmin2 + (int)(q / n1);
  const long long P = g.plane();
  const float *gc = a.gy + q;
  float *u3 = a.u3;
  const float *u2 = a.u2, *u1 = a.u1;
  for (int k = g.nmin3 + 3; k >= g.nmin3 - 4; --k) {
    const long long p = g.idx(i, j, k);
    u3[p] = hsum(gc, cs, u3[p + P], u3[p + 2 * P], u2[p], u2[p + P], u2[p + 2 * P], u1[p],
                 u1[p + P], u1[p + 2 * P]);
  }
  gc += 8 * cs;
  for (int k = g.nmax3 - 3; k <= g.nmax3 + 4; ++k) {
    const long long p = g.idx(i, j, k);
    u3[p] = hsum(gc, cs, u3[p - P], u3[p - 2 * P], u2[p], u2[p - P], u2[p - 2 * P], u1[p],
                 u1[p - P], u1[p - 2 * P]);
  }
}

// ---------------------------------------------------------------------------
// Receiver extraction (Extraction.f90:71-135,217-247,276-337,511-560):
// one thread per receiver, the sinc sum in the reference loop order.
// ---------------------------------------------------------------------------
__global__ void k_extract(ExtArgs a) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nrec) return;
  const Geom &g = a.g;
  const int i0 = a.ic[3 * r], j0 = a.ic[3 * r + 1], k0 = g.twoD ? 1 : a.ic[3 * r + 2];
  float *trp = a.tr + (long long)r * a.nt + (a.it - 1);
  float tr = *trp;
  if (a.mode == 2) {  // SW_EXT_SIMPLE_AFWI
    tr = tr + a.u2[g.idx(i0, j0, k0)];
    *trp = tr;
    return;
  }
  float v;
  if (a.mode == 1) {  // SW_EXT_SINC: v**2 in 2D, v in 3D
    const float vv = a.vel[g.idx(i0, j0, k0)];
    v = g.twoD ? vv * vv : vv;
  } else {
    v = a.vconst;
  }
  const int h = a.half, ls = 2 * h + 1;
  const float *wz = a.wz + (long long)r * ls, *wx = a.wx + (long long)r * ls;
  if (g.twoD) {
    for (int jj = -h; jj <= h; ++jj) {
      const long long pj = g.idx(i0, j0 + jj, 1);
      for (int ii = -h; ii <= h; ++ii)
        tr = tr + ((v * a.u2[pj + ii]) * wz[h + ii]) * wx[h + jj];
    }
  } else {
    for (int kk = -h; kk <= h; ++kk)
      for (int jj = -h; jj <= h; ++jj) {
        const long long pj = g.idx(i0, j0 + jj, k0 + kk);
        for (int ii = -h; ii <= h; ++ii)
          tr = tr + (((v * a.u2[pj + ii]) * wz[h + ii]) * wx[h + jj]) * wx[h + kk];
      }
  }
  *trp = tr;
}

// ---------------------------------------------------------------------------
// FWI helpers
// ---------------------------------------------------------------------------

// mod_window_pad(adj=.true.) (ExtractPadModel.f90:509-549).
__global__ void k_window_vel(int nz, int nx, int ny, float ox, float oy, float dx, float dy,
                             int nxw, int nyw, float oxw, float oyw, const float *__restrict__ big,
                             float *__restrict__ small) {
  const long long n = (long long)nz * nxw * nyw;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(q % nz);
    const long long r = q / nz;
    const int i = 1 + (int)(r % nxw), j = 1 + (int)(r / nxw);
    const float cy = (float)(j - 1) * dy + oyw;
    const int iy = (int)lroundf((cy - oy) / dy) + 1;
    const int iy1 = min(ny, max(1, iy));
    const float cx = (float)(i - 1) * dx + oxw;
    const int ix = (int)lroundf((cx - ox) / dx) + 1;
    const int ix1 = min(nx, max(1, ix));
    small[q] = 0.f + big[(long long)l + (long long)nz * ((ix1 - 1) + (long long)nx * (iy1 - 1))];
  }
}

// mod_copy_image (ExtractPadModel.f90:662-697); the window-to-model column
// map is injective, so threads never collide.
__global__ void k_copy_image(int nz, int nx, int ny, float ox, float oy, float dx, float dy,
                             int nxw, int nyw, float oxw, float oyw, const float *__restrict__ ims,
                             const float *__restrict__ ils, float *image, float *illum) {
  const long long n = (long long)nz * nxw * nyw;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(q % nz);
    const long long r = q / nz;
    const int i = 1 + (int)(r % nxw), j = 1 + (int)(r / nxw);
    const float cy = (float)(j - 1) * dy + oyw;
    const int iy = (int)lroundf((cy - oy) / dy) + 1;
    if (iy < 1 || iy > ny) continue;
    const float cx = (float)(i - 1) * dx + oxw;
    const int ix = (int)lroundf((cx - ox) / dx) + 1;
    if (ix < 1 || ix > nx) continue;
    const long long o = (long long)l + (long long)nz * ((ix - 1) + (long long)nx * (iy - 1));
    image[o] = image[o] + ims[q];
    illum[o] = illum[o] + ils[q];
  }
}

// Compute_OF_RES_ADJ (Objective_Function_Residual_Adjsource.f90:17-40) with
// the L2 norm (Norm.f90:26-28): one thread per trace, sequential FP64 sum.
__global__ void k_residual(int nrec, int nt, const float *__restrict__ dobs,
                           const float *__restrict__ mute, float *dmod, float *resid,
                           double *partial) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  const long long o = (long long)r * nt;
  double ssum = 0.0;
  for (int t = 0; t < nt; ++t) {
    const float m = mute ? mute[o + t] : 1.0f;
    const float d = m * (dobs[o + t] - dmod[o + t]);
    ssum = ssum + (double)d * (double)d;
    if (resid) resid[o + t] = d;
    dmod[o + t] = m * d;
  }
  partial[r] = ssum / 2;
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
static inline int nblocks(long long n, int bs, int cap = 152 * 16) {
  long long b = (n + bs - 1) / bs;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

cudaError_t launch_pad_velocity(const Geom &g, const float *vel_phys, float *vel_pad,
                                cudaStream_t s) {
  const long long n = (long long)g.n1p * g.n2p * g.n3p;
  k_pad_velocity<<<nblocks(n, 256), 256, 0, s>>>(g, vel_phys, vel_pad);
  return cudaGetLastError();
}

cudaError_t launch_higdon_coeffs(const Geom &g, const float *vel_pad, float dt, float dxi,
                                 float dyi, float dzi, float *gz, float *gx, float *gy,
                                 cudaStream_t s) {
  const long long n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1,
                  n3 = g.nmax3 - g.nmin3 + 1;
  const long long tot = n2 * n3 + n1 * n3 + (g.nmax3 > 1 ? n1 * n2 : 0);
  k_higdon_coeffs<<<nblocks(tot, 256), 256, 0, s>>>(g, vel_pad, dt, dxi, dyi, dzi, gz, gx, gy);
  return cudaGetLastError();
}

cudaError_t launch_step(const StepArgs &a, int adjoint2d, cudaStream_t s) {
  const Geom &g = a.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  dim3 bs(32, 8, 1);
  dim3 gs((n1 + 31) / 32, (n2 + 7) / 8, g.twoD ? 1 : n3);
  if (g.twoD) {
    if (adjoint2d) k_step<true, true><<<gs, bs, 0, s>>>(a);
    else k_step<true, false><<<gs, bs, 0, s>>>(a);
  } else {
    k_step<false, false><<<gs, bs, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_v2u(const Geom &g, const float *vel, const float *u2, float *out,
                       cudaStream_t s) {
  const long long n = g.total();
  k_v2u<<<nblocks(n, 256), 256, 0, s>>>(n, vel, u2, out);
  return cudaGetLastError();
}

cudaError_t launch_higdon(const HigArgs &a, cudaStream_t s, int *nlaunch) {
  const Geom &g = a.g;
  const long long n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1,
                  n3 = g.nmax3 - g.nmin3 + 1;
  k_higdon_z<<<(int)((n2 * n3 + 127) / 128), 128, 0, s>>>(a);
  k_higdon_x<<<(int)((n1 * n3 + 127) / 128), 128, 0, s>>>(a);
  int nl = 2;
  if (g.nbound > 0) {
    k_higdon_y<<<(int)((n1 * n2 + 127) / 128), 128, 0, s>>>(a);
    ++nl;
  }
  if (nlaunch) *nlaunch = nl;
  return cudaGetLastError();
}

cudaError_t launch_extract(const ExtArgs &a, cudaStream_t s) {
  k_extract<<<(a.nrec + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_window_vel(int nz, int nx, int ny, float ox, float oy, float dx, float dy,
                              int nxw, int nyw, float oxw, float oyw, const float *big,
                              float *small, cudaStream_t s) {
  const long long n = (long long)nz * nxw * nyw;
  k_window_vel<<<nblocks(n, 256), 256, 0, s>>>(nz, nx, ny, ox, oy, dx, dy, nxw, nyw, oxw, oyw,
                                                big, small);
  return cudaGetLastError();
}

cudaError_t launch_copy_image(int nz, int nx, int ny, float ox, float oy, float dx, float dy,
                              int nxw, int nyw, float oxw, float oyw, const float *ims,
                              const float *ils, float *image, float *illum, cudaStream_t s) {
  const long long n = (long long)nz * nxw * nyw;
  k_copy_image<<<nblocks(n, 256), 256, 0, s>>>(nz, nx, ny, ox, oy, dx, dy, nxw, nyw, oxw, oyw,
                                                ims, ils, image, illum);
  return cudaGetLastError();
}

cudaError_t launch_residual(int nrec, int nt, const float *dobs, const float *mute, float *dmod,
                            float *resid, double *partial, cudaStream_t s) {
  k_residual<<<(nrec + 127) / 128, 128, 0, s>>>(nrec, nt, dobs, mute, dmod, resid, partial);
  return cudaGetLastError();
}

}  // namespace swave
