// kernels.cu - sm_103a kernels of libswave (compiled with --fmad=false).
//
// Each kernel restates one reference loop nest with the same floating-point
// operation order; the comments give the reference file:line.  Paths are
// relative to the reference project root.
#include "../../include/swave.h"
#include "norms.cuh"
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

// max|m*(dobs - dmod)| of every trace: the threshold fct_compute takes when
// data_threshold is 0 (Norm.f90:37-40).
__global__ void k_trace_maxabs(int nrec, int nt, const float *__restrict__ dobs,
                               const float *__restrict__ mute, const float *__restrict__ dmod,
                               float *maxabs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  const long long o = (long long)r * nt;
  float mx = 0.0f;
  for (int t = 0; t < nt; ++t) {
    const float m = mute ? mute[o + t] : 1.0f;
    mx = fmaxf(mx, fabsf(m * (dobs[o + t] - dmod[o + t])));
  }
  maxabs[r] = mx;
}

// Compute_OF_RES_ADJ for the L1, Huber, Cauchy and hyperbolic norms
// (Objective_Function_Residual_Adjsource.f90:32-38 with fct_compute and
// gdt_compute, libs/libinv/Norm.f90:12-141): one thread per trace, the
// trace's misfit summed in FP32 in sample order like the reference's
// sum() of a real array.  Trace r's threshold is thresh0, or, when that is
// 0, max|r| of the first trace k <= r whose maximum is not 0 (the caller's
// threshold is reset by the first such trace and kept by the following
// ones); with no such trace it stays 0, as in the reference.
__global__ void k_residual_nrm(int ntype, int nrec, int nt, const float *__restrict__ dobs,
                               const float *__restrict__ mute, float *dmod, float *resid,
                               double *partial, float thresh0, const float *__restrict__ maxabs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  float g = thresh0;
  if (g == 0.0f && maxabs) {
    for (int k = 0; k <= r; ++k)
      if (maxabs[k] != 0.0f) {
        g = maxabs[k];
        break;
      }
  }
  const long long o = (long long)r * nt;
  float fs = 0.0f;
  for (int t = 0; t < nt; ++t) {
    const float m = mute ? mute[o + t] : 1.0f;
    const float d = m * (dobs[o + t] - dmod[o + t]);
    if (resid) resid[o + t] = d;
    fs = fs + nrm_term(ntype, d, g);
    dmod[o + t] = nrm_gdt(ntype, m * d, g);
  }
  partial[r] = (double)fs;
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

// One pass of Interpolate (Interpolate.f90:63-126) along `axis` (0 z, 1 x,
// 2 y): every line of the padded array is filtered by the 9-point half-cell
// sinc, its end values extended past both ends; one thread per line, taps
// added in order from -4 to +4.  recip stores 1/f (delp = 1/rho2,
// FDderivatives.f90:393,581) instead of f.
struct Sinc9 {
  float s[9];
};

__global__ void k_sinc9_lines(Geom g, int axis, Sinc9 w, const float *__restrict__ src,
                              float *__restrict__ dst, int recip) {
  const long long nl = axis == 0 ? (long long)g.n2p * g.n3p
                                 : axis == 1 ? (long long)g.n1p * g.n3p
                                             : (long long)g.n1p * g.n2p;
  for (long long L = blockIdx.x * (long long)blockDim.x + threadIdx.x; L < nl;
       L += (long long)gridDim.x * blockDim.x) {
    long long base, stride;
    int len;
    if (axis == 0) {
      base = g.idx(g.lo1, g.lo2 + (int)(L % g.n2p), g.lo3 + (int)(L / g.n2p));
      len = g.n1p;
      stride = 1;
    } else if (axis == 1) {
      base = g.idx(g.lo1 + (int)(L % g.n1p), g.lo2, g.lo3 + (int)(L / g.n1p));
      len = g.n2p;
      stride = g.ld1;
    } else {
      base = g.idx(g.lo1 + (int)(L % g.n1p), g.lo2 + (int)(L / g.n1p), g.lo3);
      len = g.n3p;
      stride = g.plane();
    }
    for (int q = 0; q < len; ++q) {
      float f = 0.f;
#pragma unroll
      for (int l = -4; l <= 4; ++l) {
        const int qq = min(max(q + l, 0), len - 1);
        f = f + w.s[4 + l] * src[base + (long long)qq * stride];
      }
      dst[base + (long long)q * stride] = recip ? 1.f / f : f;
    }
  }
}

cudaError_t launch_rho_delp(const Geom &g, const float *rho_pad, float *delp, float *tmp,
                            const float *sinc9, cudaStream_t s, int *nlaunch) {
  Sinc9 w;
  for (int q = 0; q < 9; ++q) w.s[q] = sinc9[q];
  auto go = [&](int axis, const float *a, float *b, int recip) {
    const long long nl = axis == 0 ? (long long)g.n2p * g.n3p
                                   : axis == 1 ? (long long)g.n1p * g.n3p
                                               : (long long)g.n1p * g.n2p;
    k_sinc9_lines<<<nblocks(nl, 128), 128, 0, s>>>(g, axis, w, a, b, recip);
    ++*nlaunch;
  };
  if (g.n3p > 1) {
    go(0, rho_pad, delp, 0);
    go(1, delp, tmp, 0);
    go(2, tmp, delp, 1);
  } else {
    go(0, rho_pad, tmp, 0);
    go(1, tmp, delp, 1);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Band-pass of traces (Bandpass.f90:89-149 with the filters of bandpass.c):
// one thread per trace.  The trace is padded by npad samples at each end with
// cosine-squared ramps from its end values, run through the low-cut and then
// the high-cut cascade of second-order sections (forward, and for a
// zero-phase filter again over the reversed samples 2..n-2), and its middle
// nt samples are returned.  The work arrays are sample-major (sample i of
// trace t at i*ntr + t) so that a warp's accesses coalesce.  Each section is
// run in place: the old input samples and the new output samples it still
// needs are carried in registers.  The first two outputs of every section
// stay zero, as the reference's never-written work samples do.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bp_sections(float *X, int n, int ntr, int t, int ns,
                                            const float *__restrict__ c) {
  for (int q = 0; q < ns; ++q) {
    const float c0 = c[5 * q], c1 = c[5 * q + 1], c2 = c[5 * q + 2], c3 = c[5 * q + 3],
                c4 = c[5 * q + 4];
    float xm2 = X[t], xm1 = X[(size_t)ntr + t], nm2 = 0.f, nm1 = 0.f;
    for (int i = 2; i < n; ++i) {
      const float xc = X[(size_t)i * ntr + t];
      const float v = (((c0 * xc + c1 * xm1) + c2 * xm2) - c3 * nm1) - c4 * nm2;
      X[(size_t)i * ntr + t] = v;
      xm2 = xm1;
      xm1 = xc;
      nm2 = nm1;
      nm1 = v;
    }
    X[t] = 0.f;
    X[(size_t)ntr + t] = 0.f;
  }
}

__device__ __forceinline__ void bp_filter(float *D, float *T, int n, int ntr, int t, int ns,
                                          const float *__restrict__ c, int phase) {
  bp_sections(D, n, ntr, t, ns, c);
  if (phase == 0) {
    T[t] = 0.f;
    T[(size_t)ntr + t] = 0.f;
    for (int i = 2; i < n; ++i) T[(size_t)i * ntr + t] = D[(size_t)(n + 1 - i) * ntr + t];
    bp_sections(T, n, ntr, t, ns, c);
    for (int i = 2; i < n; ++i) D[(size_t)i * ntr + t] = T[(size_t)(n + 1 - i) * ntr + t];
  }
}

__global__ void k_bandpass(int ntr, int nt, int npad, int phase, int nlo, const float *clo,
                           int nhi, const float *chi, const float *lead, const float *trail,
                           const float *__restrict__ in, float *__restrict__ out, float *D,
                           float *T) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntr) return;
  const int n = nt + 2 * npad;
  const float *tr = in + (size_t)t * nt;
  for (int i = 0; i < nt; ++i) D[(size_t)(npad + i) * ntr + t] = tr[i];
  for (int j = 0; j < npad; ++j) {
    D[(size_t)j * ntr + t] = tr[0] * lead[j];
    D[(size_t)(n - npad + j) * ntr + t] = tr[nt - 1] * trail[j];
  }
  if (nlo > 0) bp_filter(D, T, n, ntr, t, nlo, clo, phase);
  if (nhi > 0) bp_filter(D, T, n, ntr, t, nhi, chi, phase);
  float *o = out + (size_t)t * nt;
  for (int i = 0; i < nt; ++i) o[i] = D[(size_t)(npad + i) * ntr + t];
}

cudaError_t launch_bandpass(int ntr, int nt, int npad, int phase, int nlo, const float *clo,
                            int nhi, const float *chi, const float *lead, const float *trail,
                            const float *in, float *out, float *D, float *T, cudaStream_t s) {
  k_bandpass<<<(ntr + 127) / 128, 128, 0, s>>>(ntr, nt, npad, phase, nlo, clo, nhi, chi, lead,
                                                trail, in, out, D, T);
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

cudaError_t launch_residual_nrm(int ntype, float thresh, int nrec, int nt, const float *dobs,
                                const float *mute, float *dmod, float *resid, double *partial,
                                float *maxabs, cudaStream_t s) {
  const bool need_max = ntype != SW_NRM_L1 && thresh == 0.0f;
  if (need_max)
    k_trace_maxabs<<<(nrec + 127) / 128, 128, 0, s>>>(nrec, nt, dobs, mute, dmod, maxabs);
  k_residual_nrm<<<(nrec + 127) / 128, 128, 0, s>>>(ntype, nrec, nt, dobs, mute, dmod, resid,
                                                    partial, thresh, need_max ? maxabs : nullptr);
  return cudaGetLastError();
}

}  // namespace swave
