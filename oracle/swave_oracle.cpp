// swave_oracle.cpp - CPU restatement of the reference acoustic path.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h): what the CUDA engine is compared with
// and the timed CPU baseline.  Parity status: UNPINNED (no compilable
// reference, no golden vectors in the reference tree).
//
// Every routine cites the Fortran it restates (paths relative to the
// reference project root).  Arithmetic is written in the Fortran evaluation
// order and must be compiled with -ffp-contract=off.  The template parameter
// T is float for the parity build and double for the FP64 twin.

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Bounds and padded arrays
// ---------------------------------------------------------------------------

// FDbounds as set by readvel / copy_window_vel_gath for
// shot_type = surf_type = 0 (libs/libwave/ReadSouVelRho.f90:456-470,
// libs/libwave/ExtractPadModel.f90:483-498).
struct Bounds {
  int nmin1, nmax1, nmin2, nmax2, nmin3, nmax3, nbound;
};

static Bounds make_bounds(const sw_genpar &g) {
  Bounds b;
  // Mirror sources extend the top padding to hold the mirrored footprint;
  // a free surface replaces the top taper by lsinc cells
  // (ExtractPadModel.f90:228-234).
  if (g.shot_type > 0 || g.surf_type > 0) {
    if (g.shot_type > 0) b.nmin1 = -(g.ntaper + g.lsinc / 2 + 2) + 1;
    if (g.surf_type > 0) b.nmin1 = -g.lsinc + 1;
  } else {
    b.nmin1 = -g.ntaper + 1;
  }
  b.nmax1 = g.nz + g.ntaper;
  b.nmin2 = -g.ntaper + 1;
  b.nmax2 = g.nx + g.ntaper;
  if (!g.twoD) {
    b.nmin3 = -g.ntaper + 1;
    b.nmax3 = g.ny + g.ntaper;
    b.nbound = 4;
  } else {
    b.nmin3 = 1;
    b.nmax3 = 1;
    b.nbound = 0;
  }
  return b;
}

// A Fortran array u(nmin1-4:nmax1+4, nmin2-4:nmax2+4,
// nmin3-nbound:nmax3+nbound), column major.
template <class T> struct F3 {
  std::vector<T> v;
  int lo1 = 0, lo2 = 0, lo3 = 0, n1 = 0, n2 = 0, n3 = 0;
  void init(const Bounds &b) {
    lo1 = b.nmin1 - 4;
    lo2 = b.nmin2 - 4;
    lo3 = b.nmin3 - b.nbound;
    n1 = b.nmax1 + 4 - lo1 + 1;
    n2 = b.nmax2 + 4 - lo2 + 1;
    n3 = b.nmax3 + b.nbound - lo3 + 1;
    v.assign((size_t)n1 * n2 * n3, T(0));
  }
  inline T &operator()(int i, int j, int k) {
    return v[(size_t)(i - lo1) +
             (size_t)n1 * ((size_t)(j - lo2) + (size_t)n2 * (size_t)(k - lo3))];
  }
  inline T operator()(int i, int j, int k) const {
    return v[(size_t)(i - lo1) +
             (size_t)n1 * ((size_t)(j - lo2) + (size_t)n2 * (size_t)(k - lo3))];
  }
};

// model_pad (libs/libwave/ReadSouVelRho.f90:545-596): copy the nz*nx*ny
// window into (1:nz,1:nx,1:ny) and replicate the edges outwards.
template <class T, class S>
static void model_pad(const S *tmp, F3<T> &f, const Bounds &b, int nz, int nx,
                      int ny, bool twoD) {
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= nz; ++i)
        f(i, j, k) = (T)tmp[(size_t)(i - 1) + (size_t)nz * ((j - 1) + (size_t)nx * (k - 1))];
  for (int k = 1; k <= ny; ++k)
    for (int j = 1; j <= nx; ++j) {
      for (int i = b.nmin1 - 4; i <= 0; ++i) f(i, j, k) = f(1, j, k);
      for (int i = nz + 1; i <= b.nmax1 + 4; ++i) f(i, j, k) = f(nz, j, k);
    }
  for (int k = 1; k <= ny; ++k) {
    for (int j = b.nmin2 - 4; j <= 0; ++j)
      for (int i = b.nmin1 - 4; i <= b.nmax1 + 4; ++i) f(i, j, k) = f(i, 1, k);
    for (int j = nx + 1; j <= b.nmax2 + 4; ++j)
      for (int i = b.nmin1 - 4; i <= b.nmax1 + 4; ++i) f(i, j, k) = f(i, nx, k);
  }
  if (!twoD) {
    for (int k = b.nmin3 - b.nbound; k <= 0; ++k)
      for (int j = b.nmin2 - 4; j <= b.nmax2 + 4; ++j)
        for (int i = b.nmin1 - 4; i <= b.nmax1 + 4; ++i) f(i, j, k) = f(i, j, 1);
    for (int k = ny + 1; k <= b.nmax3 + b.nbound; ++k)
      for (int j = b.nmin2 - 4; j <= b.nmax2 + 4; ++j)
        for (int i = b.nmin1 - 4; i <= b.nmax1 + 4; ++i) f(i, j, k) = f(i, j, ny);
  }
}

// ---------------------------------------------------------------------------
// Coefficients (libs/libwave/FDcoefs.f90:25-36, FDtypes.f90:50-80)
// ---------------------------------------------------------------------------
template <class T> struct Coefs {
  T c0x, c1x, c2x, c3x, c4x, c0y, c1y, c2y, c3y, c4y, c0z, c1z, c2z, c3z, c4z;
};

template <class T> static Coefs<T> make_coefs(const sw_genpar &g) {
  // FD_acoustic_init_coefs: -205/72, 8/5, -1/5, 8/315, -1/560.
  const T c0 = T(-205.) / T(72.), c1 = T(8.) / T(5), c2 = T(-1.) / T(5.),
          c3 = T(8.) / T(315.), c4 = T(-1.) / T(560.);
  // FD_types_assign_scaled_coefs, coefpower = 2 (scalar wave equation).
  const T dxi = T(1.) / (T)g.dx, dyi = T(1.) / (T)g.dy, dzi = T(1.) / (T)g.dz;
  const T px = dxi * dxi, py = dyi * dyi, pz = dzi * dzi;
  Coefs<T> c;
  c.c0x = c0 * px; c.c1x = c1 * px; c.c2x = c2 * px; c.c3x = c3 * px; c.c4x = c4 * px;
  c.c0y = c0 * py; c.c1y = c1 * py; c.c2y = c2 * py; c.c3y = c3 * py; c.c4y = c4 * py;
  c.c0z = c0 * pz; c.c1z = c1 * pz; c.c2z = c2 * pz; c.c3z = c3 * pz; c.c4z = c4 * pz;
  return c;
}

// ---------------------------------------------------------------------------
// Stencils (libs/libwave/FDderivatives.f90)
// ---------------------------------------------------------------------------

// FD_2nd_2D_derivatives_scalar_forward_grid (FDderivatives.f90:715-743).
// Column pointers keep the inner z loop vectorisable; the per-point
// operation order is the Fortran one.
template <class T>
static void stencil2d_fwd(const Coefs<T> &c, const Bounds &b, const F3<T> &u2,
                          F3<T> &u3, const F3<T> &vel) {
  const long L = u2.n1;
#pragma omp parallel for schedule(static)
  for (int j = b.nmin2; j <= b.nmax2; ++j) {
    const T *u = &u2.v[(size_t)(b.nmin1 - u2.lo1) + (size_t)u2.n1 * (size_t)(j - u2.lo2)];
    const T *v = &vel.v[(size_t)(b.nmin1 - vel.lo1) + (size_t)vel.n1 * (size_t)(j - vel.lo2)];
    T *o = &u3.v[(size_t)(b.nmin1 - u3.lo1) + (size_t)u3.n1 * (size_t)(j - u3.lo2)];
    const int n = b.nmax1 - b.nmin1 + 1;
#pragma omp simd
    for (int q = 0; q < n; ++q) {
      T tz = c.c0z * u[q];
      tz = tz + c.c1z * (u[q + 1] + u[q - 1]);
      tz = tz + c.c2z * (u[q + 2] + u[q - 2]);
      tz = tz + c.c3z * (u[q + 3] + u[q - 3]);
      tz = tz + c.c4z * (u[q + 4] + u[q - 4]);
      T tx = c.c0x * u[q];
      tx = tx + c.c1x * (u[q + L] + u[q - L]);
      tx = tx + c.c2x * (u[q + 2 * L] + u[q - 2 * L]);
      tx = tx + c.c3x * (u[q + 3 * L] + u[q - 3 * L]);
      tx = tx + c.c4x * (u[q + 4 * L] + u[q - 4 * L]);
      const T vv = v[q];
      o[q] = (vv * vv) * (tx + tz);
    }
  }
}

// FD_2nd_3D_derivatives_scalar_forward_grid (FDderivatives.f90:97-131).
template <class T>
static void stencil3d_fwd(const Coefs<T> &c, const Bounds &b, const F3<T> &u2,
                          F3<T> &u3, const F3<T> &vel) {
  const long L = u2.n1, P = (long)u2.n1 * u2.n2;
#pragma omp parallel for schedule(static) collapse(2)
  for (int k = b.nmin3; k <= b.nmax3; ++k)
    for (int j = b.nmin2; j <= b.nmax2; ++j) {
      const size_t off = (size_t)(b.nmin1 - u2.lo1) +
                         (size_t)u2.n1 * ((size_t)(j - u2.lo2) + (size_t)u2.n2 * (size_t)(k - u2.lo3));
      const T *u = &u2.v[off];
      const T *v = &vel.v[off];
      T *o = &u3.v[off];
      const int n = b.nmax1 - b.nmin1 + 1;
#pragma omp simd
      for (int q = 0; q < n; ++q) {
        T tz = c.c0z * u[q];
        tz = tz + c.c1z * (u[q + 1] + u[q - 1]);
        tz = tz + c.c2z * (u[q + 2] + u[q - 2]);
        tz = tz + c.c3z * (u[q + 3] + u[q - 3]);
        tz = tz + c.c4z * (u[q + 4] + u[q - 4]);
        T tx = c.c0x * u[q];
        tx = tx + c.c1x * (u[q + L] + u[q - L]);
        tx = tx + c.c2x * (u[q + 2 * L] + u[q - 2 * L]);
        tx = tx + c.c3x * (u[q + 3 * L] + u[q - 3 * L]);
        tx = tx + c.c4x * (u[q + 4 * L] + u[q - 4 * L]);
        T ty = c.c0y * u[q];
        ty = ty + c.c1y * (u[q + P] + u[q - P]);
        ty = ty + c.c2y * (u[q + 2 * P] + u[q - 2 * P]);
        ty = ty + c.c3y * (u[q + 3 * P] + u[q - 3 * P]);
        ty = ty + c.c4y * (u[q + 4 * P] + u[q - 4 * P]);
        const T vv = v[q];
        o[q] = (vv * vv) * ((tx + tz) + ty);
      }
    }
}

// FD_2nd_2D_derivatives_scalar_adjoint_grid (FDderivatives.f90:847-891):
// u3 = Laplacian(v^2 u2) with the vel index clamped to the compute domain.
template <class T>
static void stencil2d_adj(const Coefs<T> &c, const Bounds &b, const F3<T> &u2,
                          F3<T> &u3, const F3<T> &vel) {
#pragma omp parallel for schedule(static)
  for (int j = b.nmin2; j <= b.nmax2; ++j) {
    int jp[5], jm[5];
    for (int l = 1; l <= 4; ++l) {
      jp[l] = std::min(b.nmax2, j + l);
      jm[l] = std::max(b.nmin2, j - l);
    }
    for (int i = b.nmin1; i <= b.nmax1; ++i) {
      int ip[5], im[5];
      for (int l = 1; l <= 4; ++l) {
        ip[l] = std::min(b.nmax1, i + l);
        im[l] = std::max(b.nmin1, i - l);
      }
      auto w = [&](int ii, int jj, int vi, int vj) -> T {
        const T v = vel(vi, vj, 1);
        return (v * v) * u2(ii, jj, 1);
      };
      T tz = c.c0z * w(i, j, i, j);
      tz = tz + c.c1z * (w(i + 1, j, ip[1], j) + w(i - 1, j, im[1], j));
      tz = tz + c.c2z * (w(i + 2, j, ip[2], j) + w(i - 2, j, im[2], j));
      tz = tz + c.c3z * (w(i + 3, j, ip[3], j) + w(i - 3, j, im[3], j));
      tz = tz + c.c4z * (w(i + 4, j, ip[4], j) + w(i - 4, j, im[4], j));
      T tx = c.c0x * w(i, j, i, j);
      tx = tx + c.c1x * (w(i, j + 1, i, jp[1]) + w(i, j - 1, i, jm[1]));
      tx = tx + c.c2x * (w(i, j + 2, i, jp[2]) + w(i, j - 2, i, jm[2]));
      tx = tx + c.c3x * (w(i, j + 3, i, jp[3]) + w(i, j - 3, i, jm[3]));
      tx = tx + c.c4x * (w(i, j + 4, i, jp[4]) + w(i, j - 4, i, jm[4]));
      u3(i, j, 1) = tx + tz;
    }
  }
}

// FD_2nd_3D_derivatives_scalar_adjoint_grid (FDderivatives.f90:780-819):
// tmp = vel**2 * u2 over the whole padded array, then the Laplacian.
template <class T>
static void stencil3d_adj(const Coefs<T> &c, const Bounds &b, const F3<T> &u2,
                          F3<T> &u3, const F3<T> &vel, F3<T> &tmp) {
  const size_t n = u2.v.size();
#pragma omp parallel for schedule(static)
  for (size_t q = 0; q < n; ++q) {
    const T v = vel.v[q];
    tmp.v[q] = (v * v) * u2.v[q];
  }
#pragma omp parallel for schedule(static)
  for (int k = b.nmin3; k <= b.nmax3; ++k)
    for (int j = b.nmin2; j <= b.nmax2; ++j)
      for (int i = b.nmin1; i <= b.nmax1; ++i) {
        T tz = c.c0z * tmp(i, j, k);
        tz = tz + c.c1z * (tmp(i + 1, j, k) + tmp(i - 1, j, k));
        tz = tz + c.c2z * (tmp(i + 2, j, k) + tmp(i - 2, j, k));
        tz = tz + c.c3z * (tmp(i + 3, j, k) + tmp(i - 3, j, k));
        tz = tz + c.c4z * (tmp(i + 4, j, k) + tmp(i - 4, j, k));
        T tx = c.c0x * tmp(i, j, k);
        tx = tx + c.c1x * (tmp(i, j + 1, k) + tmp(i, j - 1, k));
        tx = tx + c.c2x * (tmp(i, j + 2, k) + tmp(i, j - 2, k));
        tx = tx + c.c3x * (tmp(i, j + 3, k) + tmp(i, j - 3, k));
        tx = tx + c.c4x * (tmp(i, j + 4, k) + tmp(i, j - 4, k));
        T ty = c.c0y * tmp(i, j, k);
        ty = ty + c.c1y * (tmp(i, j, k + 1) + tmp(i, j, k - 1));
        ty = ty + c.c2y * (tmp(i, j, k + 2) + tmp(i, j, k - 2));
        ty = ty + c.c3y * (tmp(i, j, k + 3) + tmp(i, j, k - 3));
        ty = ty + c.c4y * (tmp(i, j, k + 4) + tmp(i, j, k - 4));
        u3(i, j, k) = (tx + tz) + ty;
      }
}

// FD_2nd_time_derivative_grid (FDderivatives.f90:960-982):
// u3 = (20 u2 - 6 u1 - 4 u0 + u_1 + 12 dt^2 u3) / 11 on the compute domain.
template <class T>
static void time_update(const Bounds &b, T dt, const F3<T> &u2, const F3<T> &u1,
                        const F3<T> &u0, const F3<T> &um1, F3<T> &u3) {
  const T div11 = T(1.) / T(11);
  const T dt2 = dt * dt;
  const T k12 = T(12.) * dt2;
#pragma omp parallel for schedule(static) collapse(2)
  for (int k = b.nmin3; k <= b.nmax3; ++k)
    for (int j = b.nmin2; j <= b.nmax2; ++j) {
      const size_t off = (size_t)(b.nmin1 - u2.lo1) +
                         (size_t)u2.n1 * ((size_t)(j - u2.lo2) + (size_t)u2.n2 * (size_t)(k - u2.lo3));
      const T *a2 = &u2.v[off], *a1 = &u1.v[off], *a0 = &u0.v[off], *am = &um1.v[off];
      T *o = &u3.v[off];
      const int n = b.nmax1 - b.nmin1 + 1;
#pragma omp simd
      for (int q = 0; q < n; ++q) {
        T a = T(20.) * a2[q];
        a = a - T(6.) * a1[q];
        a = a - T(4.) * a0[q];
        a = a + am[q];
        a = a + k12 * o[q];
        o[q] = a * div11;
      }
    }
}

// ---------------------------------------------------------------------------
// Higdon absorbing boundary (libs/libwave/Boundary.f90)
// ---------------------------------------------------------------------------

// Higdon_coeff (Boundary.f90:66-87), beta1 = 1, beta2 = 0.7, weight = 0.5.
template <class T> static void higdon_coeff(T nu, T *coeff) {
  const T beta1 = T(1.0), beta2 = T(0.7), weight = T(0.5);
  T fdum = (beta1 + nu) * (T(1) - weight);
  const T qx = (weight * (beta1 + nu) - nu) / fdum;
  const T qt = (weight * (beta1 + nu) - beta1) / fdum;
  const T qxt = weight / (weight - T(1));
  fdum = (beta2 + nu) * (T(1) - weight);
  const T rx = (weight * (beta2 + nu) - nu) / fdum;
  const T rt = (weight * (beta2 + nu) - beta2) / fdum;
  const T rxt = weight / (weight - T(1));
  coeff[0] = qx + rx;
  coeff[1] = qx * rx;
  coeff[2] = qt + rt;
  coeff[3] = ((qx * rt + qt * rx) + qxt) + rxt;
  coeff[4] = qx * rxt + rx * qxt;
  coeff[5] = qt * rt;
  coeff[6] = qt * rxt + rt * qxt;
  coeff[7] = qxt * rxt;
}

template <class T> struct Higdon {
  // gz(16, nmin2:nmax2, nmin3:nmax3), gx(16, nmin1:nmax1, nmin3:nmax3),
  // gy(16, nmin1:nmax1, nmin2:nmax2) (Propagator.f90:152-154).
  std::vector<T> gz, gx, gy;
  int n1, n2, n3;
  Bounds b;
  T *Gz(int j, int k) { return &gz[16 * ((size_t)(j - b.nmin2) + (size_t)n2 * (k - b.nmin3))]; }
  T *Gx(int i, int k) { return &gx[16 * ((size_t)(i - b.nmin1) + (size_t)n1 * (k - b.nmin3))]; }
  T *Gy(int i, int j) { return &gy[16 * ((size_t)(i - b.nmin1) + (size_t)n1 * (j - b.nmin2))]; }
};

// Higdon (Boundary.f90:17-63).
template <class T>
static void higdon_init(Higdon<T> &h, const Bounds &b, const F3<T> &vel, T dt,
                        const sw_genpar &g) {
  h.b = b;
  h.n1 = b.nmax1 - b.nmin1 + 1;
  h.n2 = b.nmax2 - b.nmin2 + 1;
  h.n3 = b.nmax3 - b.nmin3 + 1;
  h.gz.assign(16 * (size_t)h.n2 * h.n3, T(0));
  h.gx.assign(16 * (size_t)h.n1 * h.n3, T(0));
  h.gy.assign(16 * (size_t)h.n1 * h.n2, T(0));
  const T dxi = T(1.) / (T)g.dx, dyi = T(1.) / (T)g.dy, dzi = T(1.) / (T)g.dz;
  for (int k = b.nmin3; k <= b.nmax3; ++k)
    for (int j = b.nmin2; j <= b.nmax2; ++j) {
      higdon_coeff<T>((vel(b.nmin1, j, k) * dt) * dzi, h.Gz(j, k));
      higdon_coeff<T>((vel(b.nmax1, j, k) * dt) * dzi, h.Gz(j, k) + 8);
    }
  for (int k = b.nmin3; k <= b.nmax3; ++k)
    for (int i = b.nmin1; i <= b.nmax1; ++i) {
      higdon_coeff<T>((vel(i, b.nmin2, k) * dt) * dxi, h.Gx(i, k));
      higdon_coeff<T>((vel(i, b.nmax2, k) * dt) * dxi, h.Gx(i, k) + 8);
    }
  if (b.nmax3 > 1)
    for (int j = b.nmin2; j <= b.nmax2; ++j)
      for (int i = b.nmin1; i <= b.nmax1; ++i) {
        higdon_coeff<T>((vel(i, j, b.nmin3) * dt) * dyi, h.Gy(i, j));
        higdon_coeff<T>((vel(i, j, b.nmax3) * dt) * dyi, h.Gy(i, j) + 8);
      }
}

// Higdon_factor (Boundary.f90:366-447) called from Boundary_3d as
// (u0, u1, u2) = (grid%u1, grid%u2, grid%u3).  a/b/c are the three time
// levels along the line at offsets 0, s, 2s.
template <class T>
static inline T higdon_sum(const T *g, T u3p1, T u3p2, T u2p0, T u2p1, T u2p2,
                           T u1p0, T u1p1, T u1p2) {
  T f = g[0] * u3p1;
  f = f + g[1] * u3p2;
  f = f + g[2] * u2p0;
  f = f + g[3] * u2p1;
  f = f + g[4] * u2p2;
  f = f + g[5] * u1p0;
  f = f + g[6] * u1p1;
  f = f + g[7] * u1p2;
  return -f;
}

// Boundary_3d (Boundary.f90:89-184) for surf_type = 0 (nz0 = nmin1).
template <class T>
static void boundary(Higdon<T> &h, const Bounds &b, const F3<T> &u1,
                     const F3<T> &u2, F3<T> &u3, bool surf = false) {
  const int nst = 3;
  // With a free surface the top is not absorbing and the side lines start
  // at row 1 (Boundary.f90:104-108,123-128).
  const int nz0 = surf ? 1 : b.nmin1;
#pragma omp parallel for schedule(static)
  for (int k = b.nmin3; k <= b.nmax3; ++k) {
    for (int j = b.nmin2; j <= b.nmax2; ++j) {
      const T *g = h.Gz(j, k);
      if (!surf)
        for (int i = nz0 + nst; i >= b.nmin1 - 4; --i)
          u3(i, j, k) = higdon_sum(g, u3(i + 1, j, k), u3(i + 2, j, k), u2(i, j, k),
                                   u2(i + 1, j, k), u2(i + 2, j, k), u1(i, j, k),
                                   u1(i + 1, j, k), u1(i + 2, j, k));
      for (int i = b.nmax1 - nst; i <= b.nmax1 + 4; ++i)
        u3(i, j, k) = higdon_sum(g + 8, u3(i - 1, j, k), u3(i - 2, j, k), u2(i, j, k),
                                 u2(i - 1, j, k), u2(i - 2, j, k), u1(i, j, k),
                                 u1(i - 1, j, k), u1(i - 2, j, k));
    }
    for (int j = b.nmin2 + nst; j >= b.nmin2 - 4; --j)
      for (int i = nz0; i <= b.nmax1; ++i) {
        const T *g = h.Gx(i, k);
        u3(i, j, k) = higdon_sum(g, u3(i, j + 1, k), u3(i, j + 2, k), u2(i, j, k),
                                 u2(i, j + 1, k), u2(i, j + 2, k), u1(i, j, k),
                                 u1(i, j + 1, k), u1(i, j + 2, k));
      }
    for (int j = b.nmax2 - nst; j <= b.nmax2 + 4; ++j)
      for (int i = nz0; i <= b.nmax1; ++i) {
        const T *g = h.Gx(i, k) + 8;
        u3(i, j, k) = higdon_sum(g, u3(i, j - 1, k), u3(i, j - 2, k), u2(i, j, k),
                                 u2(i, j - 1, k), u2(i, j - 2, k), u1(i, j, k),
                                 u1(i, j - 1, k), u1(i, j - 2, k));
      }
  }
  if (b.nbound > 0) {
#pragma omp parallel for schedule(static)
    for (int j = b.nmin2; j <= b.nmax2; ++j) {
      for (int k = b.nmin3 + nst; k >= b.nmin3 - 4; --k)
        for (int i = nz0; i <= b.nmax1; ++i) {
          const T *g = h.Gy(i, j);
          u3(i, j, k) = higdon_sum(g, u3(i, j, k + 1), u3(i, j, k + 2), u2(i, j, k),
                                   u2(i, j, k + 1), u2(i, j, k + 2), u1(i, j, k),
                                   u1(i, j, k + 1), u1(i, j, k + 2));
        }
      for (int k = b.nmax3 - nst; k <= b.nmax3 + 4; ++k)
        for (int i = nz0; i <= b.nmax1; ++i) {
          const T *g = h.Gy(i, j) + 8;
          u3(i, j, k) = higdon_sum(g, u3(i, j, k - 1), u3(i, j, k - 2), u2(i, j, k),
                                   u2(i, j, k - 1), u2(i, j, k - 2), u1(i, j, k),
                                   u1(i, j, k - 1), u1(i, j, k - 2));
        }
    }
  }
}

// ---------------------------------------------------------------------------
// Sinc weights and positions
// ---------------------------------------------------------------------------
static inline float t_sin(float x) { return sinf(x); }
static inline double t_sin(double x) { return sin(x); }
static inline float t_cos(float x) { return cosf(x); }
static inline double t_cos(double x) { return cos(x); }
static inline long t_nint(float x) { return lroundf(x); }
static inline long t_nint(double x) { return lround(x); }

// mksinc (libs/libwave/Interpolate.f90:15-42).
template <class T> static void mksinc(T *sinc, int lsinc, T shift) {
  const T pi = T(3.141592654);
  T fsum = T(0.);
  for (int n = 1; n <= lsinc; ++n) {
    T fact;
    if (n <= (int)((T)(lsinc / 2 + 1) + shift))
      fact = ((T)(n - 1) - shift) / (T)(lsinc / 2);
    else
      fact = ((T)(lsinc - n) + shift) / (T)(lsinc / 2);
    if (fact <= T(0.)) fact = T(0.);
    const T pos = pi * ((T)(n - (lsinc / 2 + 1)) - shift);
    if (std::fabs(pos) > T(0.005f))
      sinc[n - 1] = (fact * t_sin(pos)) / pos;
    else
      sinc[n - 1] = fact * (T(1.) - (pos * pos) / T(6.));
    fsum = fsum + sinc[n - 1];
  }
  for (int n = 1; n <= lsinc; ++n) sinc[n - 1] = sinc[n - 1] / fsum;
}

// ---------------------------------------------------------------------------
// Variable density (genpar%withRho)
// ---------------------------------------------------------------------------

// FD_acoustic_rho_init_coefs (FDcoefs.f90:12-23) scaled by
// FD_types_assign_scaled_coefs with coefpower = 1 (FDtypes.f90:50-80).
template <class T> static Coefs<T> make_rho_coefs(const sw_genpar &g) {
  const T c0 = T(0.), c1 = T(1225.) / T(1024.), c2 = T(-1225.) / (T(1024.) * T(15.)),
          c3 = T(1225.) / (T(1024.) * T(125.)), c4 = T(-1225.) / (T(1024.) * T(1715.));
  const T dxi = T(1.) / (T)g.dx, dyi = T(1.) / (T)g.dy, dzi = T(1.) / (T)g.dz;
  Coefs<T> c;
  c.c0x = c0 * dxi; c.c1x = c1 * dxi; c.c2x = c2 * dxi; c.c3x = c3 * dxi; c.c4x = c4 * dxi;
  c.c0y = c0 * dyi; c.c1y = c1 * dyi; c.c2y = c2 * dyi; c.c3y = c3 * dyi; c.c4y = c4 * dyi;
  c.c0z = c0 * dzi; c.c1z = c1 * dzi; c.c2z = c2 * dzi; c.c3z = c3 * dzi; c.c4z = c4 * dzi;
  return c;
}

// Interpolate (Interpolate.f90:44-130): rho2 = rho shifted half a cell along
// z, then x, then (3D) y by a 9-point sinc, each line extended by its end
// values.
template <class T>
static void rho_interpolate(const Bounds &b, const F3<T> &rho, F3<T> &rho2) {
  const int lsinc = 9, h = lsinc / 2;
  T sinc[9];
  mksinc<T>(sinc, lsinc, T(0.5));
  rho2 = rho;
  const int lo1 = b.nmin1 - 4, hi1 = b.nmax1 + 4, lo2 = b.nmin2 - 4, hi2 = b.nmax2 + 4;
  const int lo3 = b.nmin3 - b.nbound, hi3 = b.nmax3 + b.nbound;
  std::vector<T> tr;
  // One line: tr[q - lo + lsinc] holds sample q, q in lo-lsinc..hi+lsinc.
  auto filter = [&](int lo, int hi, auto get, auto put) {
    tr.assign((size_t)(hi - lo + 1 + 2 * lsinc), T(0));
    for (int q = lo; q <= hi; ++q) tr[(size_t)(q - lo + lsinc)] = get(q);
    for (int q = lo - lsinc; q <= lo - 1; ++q) tr[(size_t)(q - lo + lsinc)] = get(lo);
    for (int q = hi + 1; q <= hi + lsinc; ++q) tr[(size_t)(q - lo + lsinc)] = get(hi);
    for (int q = lo; q <= hi; ++q) {
      T f = T(0.);
      for (int l = -h; l <= h; ++l) f = f + sinc[h + l] * tr[(size_t)(q + l - lo + lsinc)];
      put(q, f);
    }
  };
  for (int k = lo3; k <= hi3; ++k)
    for (int j = lo2; j <= hi2; ++j)
      filter(lo1, hi1, [&](int i) { return rho(i, j, k); },
             [&](int i, T f) { rho2(i, j, k) = f; });
  for (int k = lo3; k <= hi3; ++k)
    for (int i = lo1; i <= hi1; ++i)
      filter(lo2, hi2, [&](int j) { return rho2(i, j, k); },
             [&](int j, T f) { rho2(i, j, k) = f; });
  if (hi3 > 1)
    for (int j = lo2; j <= hi2; ++j)
      for (int i = lo1; i <= hi1; ++i)
        filter(lo3, hi3, [&](int k) { return rho2(i, j, k); },
               [&](int k, T f) { rho2(i, j, k) = f; });
}

// FD_2D_derivatives_acoustic_forward_grid (FDderivatives.f90:588-657) and
// FD_3D_derivatives_acoustic_forward_grid (FDderivatives.f90:263-382): the
// staggered gradient of u2 scaled by delp = 1/rho2 (with first-order
// differences in the three padding cells beyond each face), then its
// staggered divergence times v^2*rho.  The gradient arrays persist over the
// steps of a propagation; the cells the reference never writes (the fourth
// padding cell, read by the divergence at the domain's first cell) stay zero.
template <class T> struct RhoState {
  F3<T> rho, delp, sz, sx, sy;
  Coefs<T> c;
  T dzi, dxi, dyi;
};

template <class T>
static void rho_state_init(RhoState<T> &r, const sw_genpar &g, const Bounds &b, const T *rho_in) {
  r.rho.init(b);
  model_pad(rho_in, r.rho, b, g.nz, g.nx, g.ny, g.twoD != 0);
  F3<T> rho2;
  rho_interpolate(b, r.rho, rho2);
  r.delp = rho2;
  for (auto &v : r.delp.v) v = T(1.) / v;
  r.sz.init(b);
  r.sx.init(b);
  if (!g.twoD) r.sy.init(b);
  r.c = make_rho_coefs<T>(g);
  r.dzi = T(1.) / (T)g.dz;
  r.dxi = T(1.) / (T)g.dx;
  r.dyi = T(1.) / (T)g.dy;
}

template <class T>
static void stencil_rho(RhoState<T> &r, const Bounds &b, bool twoD, const F3<T> &u2, F3<T> &u3,
                        const F3<T> &vel) {
  const Coefs<T> &c = r.c;
  F3<T> &sz = r.sz, &sx = r.sx, &sy = r.sy;
  const F3<T> &dp = r.delp;
  const int k0 = twoD ? 1 : b.nmin3, k1 = twoD ? 1 : b.nmax3;
  for (int k = k0; k <= k1; ++k)
    for (int j = b.nmin2; j <= b.nmax2; ++j)
      for (int i = b.nmin1; i <= b.nmax1; ++i) {
        const T d = dp(i, j, k);
        T a = c.c1z * (u2(i + 1, j, k) - u2(i, j, k));
        a = a + c.c2z * (u2(i + 2, j, k) - u2(i - 1, j, k));
        a = a + c.c3z * (u2(i + 3, j, k) - u2(i - 2, j, k));
        a = a + c.c4z * (u2(i + 4, j, k) - u2(i - 3, j, k));
        sz(i, j, k) = a * d;
        a = c.c1x * (u2(i, j + 1, k) - u2(i, j, k));
        a = a + c.c2x * (u2(i, j + 2, k) - u2(i, j - 1, k));
        a = a + c.c3x * (u2(i, j + 3, k) - u2(i, j - 2, k));
        a = a + c.c4x * (u2(i, j + 4, k) - u2(i, j - 3, k));
        sx(i, j, k) = a * d;
        if (!twoD) {
          a = c.c1y * (u2(i, j, k + 1) - u2(i, j, k));
          a = a + c.c2y * (u2(i, j, k + 2) - u2(i, j, k - 1));
          a = a + c.c3y * (u2(i, j, k + 3) - u2(i, j, k - 2));
          a = a + c.c4y * (u2(i, j, k + 4) - u2(i, j, k - 3));
          sy(i, j, k) = a * d;
        }
      }
  // First-order gradient in the padding cells, scaled by delp of the
  // adjacent domain face.
  auto pad = [&](int i, int j, int k, T d) {
    sz(i, j, k) = (r.dzi * (u2(i + 1, j, k) - u2(i, j, k))) * d;
    sx(i, j, k) = (r.dxi * (u2(i, j + 1, k) - u2(i, j, k))) * d;
    if (!twoD) sy(i, j, k) = (r.dyi * (u2(i, j, k + 1) - u2(i, j, k))) * d;
  };
  for (int k = k0; k <= k1; ++k) {
    for (int j = b.nmin2; j <= b.nmax2; ++j) {
      for (int i = b.nmin1 - 1; i >= b.nmin1 - 3; --i) pad(i, j, k, dp(b.nmin1, j, k));
      for (int i = b.nmax1 + 1; i <= b.nmax1 + 3; ++i) pad(i, j, k, dp(b.nmax1, j, k));
    }
    for (int j = b.nmin2 - 1; j >= b.nmin2 - 3; --j)
      for (int i = b.nmin1; i <= b.nmax1; ++i) pad(i, j, k, dp(i, b.nmin2, k));
    for (int j = b.nmax2 + 1; j <= b.nmax2 + 3; ++j)
      for (int i = b.nmin1; i <= b.nmax1; ++i) pad(i, j, k, dp(i, b.nmax2, k));
  }
  if (!twoD) {
    for (int k = b.nmin3 - 1; k >= b.nmin3 - 3; --k)
      for (int j = b.nmin2; j <= b.nmax2; ++j)
        for (int i = b.nmin1; i <= b.nmax1; ++i) pad(i, j, k, dp(i, j, b.nmin3));
    for (int k = b.nmax3 + 1; k <= b.nmax3 + 3; ++k)
      for (int j = b.nmin2; j <= b.nmax2; ++j)
        for (int i = b.nmin1; i <= b.nmax1; ++i) pad(i, j, k, dp(i, j, b.nmax3));
  }
  for (int k = k0; k <= k1; ++k)
    for (int j = b.nmin2; j <= b.nmax2; ++j)
      for (int i = b.nmin1; i <= b.nmax1; ++i) {
        T tz = c.c1z * (sz(i, j, k) - sz(i - 1, j, k));
        tz = tz + c.c2z * (sz(i + 1, j, k) - sz(i - 2, j, k));
        tz = tz + c.c3z * (sz(i + 2, j, k) - sz(i - 3, j, k));
        tz = tz + c.c4z * (sz(i + 3, j, k) - sz(i - 4, j, k));
        T tx = c.c1x * (sx(i, j, k) - sx(i, j - 1, k));
        tx = tx + c.c2x * (sx(i, j + 1, k) - sx(i, j - 2, k));
        tx = tx + c.c3x * (sx(i, j + 2, k) - sx(i, j - 3, k));
        tx = tx + c.c4x * (sx(i, j + 3, k) - sx(i, j - 4, k));
        const T v = vel(i, j, k);
        if (twoD) {
          u3(i, j, k) = ((v * v) * r.rho(i, j, k)) * (tx + tz);
        } else {
          T ty = c.c1y * (sy(i, j, k) - sy(i, j, k - 1));
          ty = ty + c.c2y * (sy(i, j, k + 1) - sy(i, j, k - 2));
          ty = ty + c.c3y * (sy(i, j, k + 2) - sy(i, j, k - 3));
          ty = ty + c.c4y * (sy(i, j, k + 3) - sy(i, j, k - 4));
          u3(i, j, k) = ((v * v) * r.rho(i, j, k)) * ((tx + ty) + tz);
        }
      }
}

// find_i_d (libs/libwave/ModelSpaceTypes.f90:144-151).
template <class T>
static void find_i_d(int &ielev, T &delev, T elev, T orig, T delta) {
  ielev = (int)t_nint((elev - orig) / delta) + 1;
  delev = elev - (orig + (T)(ielev - 1) * delta);
}

template <class T> struct Pos {
  int ic[3];
  T dc[3];
  std::vector<T> sz, sx, sy;   // sinc weights per axis
};

// ModelSpace_compute_xyz_positions (ModelSpaceTypes.f90:112-124) plus the
// per-trace sinc weights of Injection_source_sinc_* / Extraction_1trace_*
// (computed once: they do not depend on the time step).
template <class T>
static bool make_positions(const sw_genpar &g, const Bounds &b, int n,
                           const T *coord, std::vector<Pos<T>> &out,
                           bool need_sinc, bool mirror = false, bool mirror_in_domain = false) {
  out.resize(n);
  const T om[3] = {(T)g.oz, (T)g.ox, (T)(g.twoD ? 0.f : g.oy)};
  const T de[3] = {(T)g.dz, (T)g.dx, (T)(g.twoD ? 1.f : g.dy)};
  const int half = g.lsinc / 2;
  for (int r = 0; r < n; ++r) {
    Pos<T> &p = out[r];
    for (int a = 0; a < 3; ++a) find_i_d<T>(p.ic[a], p.dc[a], coord[3 * r + a], om[a], de[a]);
    if (g.twoD && p.ic[2] != 1) return false;
    const int hw = need_sinc ? half : 0;
    if (p.ic[0] - hw < b.nmin1 - 4 || p.ic[0] + hw > b.nmax1 + 4) return false;
    // The mirrored footprint (rows -ic-hw..-ic+hw) must lie in the array too.
    // A mirror source must also lie in the compute domain (an injection
    // into the padding cells would be overwritten by the boundary update).
    const int mlo = mirror_in_domain ? b.nmin1 : b.nmin1 - 4;
    const int mhi = mirror_in_domain ? b.nmax1 : b.nmax1 + 4;
    if (mirror && (-p.ic[0] - hw < mlo || -p.ic[0] + hw > mhi)) return false;
    if (p.ic[1] - hw < b.nmin2 - 4 || p.ic[1] + hw > b.nmax2 + 4) return false;
    if (!g.twoD && (p.ic[2] - hw < b.nmin3 - 4 || p.ic[2] + hw > b.nmax3 + 4)) return false;
    if (need_sinc) {
      p.sz.resize(g.lsinc);
      p.sx.resize(g.lsinc);
      p.sy.resize(g.lsinc);
      mksinc<T>(p.sz.data(), g.lsinc, p.dc[0] / de[0]);
      mksinc<T>(p.sx.data(), g.lsinc, p.dc[1] / de[1]);
      mksinc<T>(p.sy.data(), g.lsinc, p.dc[2] / de[2]);
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// Tapers (libs/libwave/Taper.f90:14-44)
// ---------------------------------------------------------------------------
template <class T> static void cos_sin_taper(std::vector<T> &a, int ntaper, int n) {
  const T pi = T(3.14159265359);
  const int m = std::min(ntaper, n);
  for (int i = 1; i <= m; ++i) {
    const T s = t_sin((pi * (T)(i - 1)) / (T)(2 * (m - 1)));
    a[i - 1] = s * s;
  }
  const int i0 = std::max(1, n - ntaper);
  for (int i = i0; i <= n; ++i) {
    const T c = t_cos((pi * (T)(i - i0)) / (T)(2 * ntaper));
    a[i - 1] = c * c;
  }
}

template <class T>
static void compute_taper(int nxw, int nyw, std::vector<T> &tx, std::vector<T> &ty) {
  tx.assign(nxw, T(1.));
  ty.assign(nyw, T(1.));
  cos_sin_taper(tx, std::min(nxw / 2, 10), nxw);
  if (nyw > 1) cos_sin_taper(ty, std::min(nyw / 2, 10), nyw);
}

// ---------------------------------------------------------------------------
// Rigid-boundary switch (no counterpart in the reference): the Higdon
// recurrence is skipped, so the halo stays zero.  With it the Born / LSRTM
// pair is an exact adjoint pair (the Higdon boundary is not self-adjoint).
static int g_rigid = 0;

// propagator_acoustic (libs/libwave/Propagator.f90:27-270)
// ---------------------------------------------------------------------------
template <class T> struct IO {
  const T *vel;
  int nsou;
  const T *sou_coord;
  const T *sou_trace;
  int nrec;
  const T *rec_coord;
  T *rec_trace;
  T *wave;
  T *image;
  T *illum;
  const T *ref;
  T *final_u2;
  const T *rho;   // unpadded density (withRho), or null
  T *image2;      // SW_IMG_AFWI_RHO: the density gradient
};

static int check_genpar(const sw_genpar &g) {
  if (g.surf_type < 0 || g.shot_type < 0 || g.rec_type < 0) return SW_BAD_PARAM;
  if (g.nz < 1 || g.nx < 1 || g.ny < 1 || g.nt < 1 || g.ntaper < 1 || g.snapi < 1)
    return SW_BAD_PARAM;
  if (g.lsinc < 3 || (g.lsinc % 2) == 0) return SW_BAD_PARAM;
  if (g.twoD && g.ny != 1) return SW_BAD_PARAM;
  if (!(g.dz > 0.f) || !(g.dx > 0.f) || (!g.twoD && !(g.dy > 0.f)) || !(g.dt > 0.f))
    return SW_BAD_PARAM;
  return SW_OK;
}

template <class T> static int propagate(const sw_prop_desc &d, const IO<T> &io) {
  const sw_genpar &g = d.g;
  int st = check_genpar(g);
  if (st) return st;
  if (d.tstep != 1 && d.tstep != -1) return SW_BAD_PARAM;
  if (d.imaging < SW_IMG_NONE || d.imaging > SW_IMG_AFWI_RHO) return SW_BAD_PARAM;
  if (d.imaging == SW_IMG_AFWI_RHO && (!io.rho || !io.image2)) return SW_BAD_PARAM;
  const Bounds b = make_bounds(g);
  const int nt = g.nt;
  const int ntsnap = nt / g.snapi;
  const int nz = g.nz, nx = g.nx, ny = g.ny;

  F3<T> vel, ua, ub, uc, ud, ue, tmp;
  vel.init(b);
  model_pad(io.vel, vel, b, nz, nx, ny, g.twoD != 0);
  // allocateUSpace + zeroUSpace (Propagator.f90:144-145).
  ua.init(b); ub.init(b); uc.init(b); ud.init(b); ue.init(b);
  if (!g.twoD && d.fd_scheme == SW_FD_ADJOINT) tmp.init(b);
  F3<T> *um1 = &ua, *u0 = &ub, *u1 = &uc, *u2 = &ud, *u3 = &ue;

  const Coefs<T> c = make_coefs<T>(g);
  RhoState<T> rs;
  if (io.rho) {
    // The variable-density drivers run the forward-grid operator in both
    // directions (to_disk_to_memory_RTM.f90:388-398,455-465).
    if (d.fd_scheme != SW_FD_FORWARD) return SW_UNSUPPORTED;
    rho_state_init(rs, g, b, io.rho);
  }
  Higdon<T> hig;
  higdon_init(hig, b, vel, (T)g.dt, g);

  std::vector<Pos<T>> spos, rpos;
  const bool inj_sinc = d.injection == SW_INJ_SINC || d.injection == SW_INJ_LSRTM_SINC;
  const bool ext_sinc = d.extraction == SW_EXT_SINC || d.extraction == SW_EXT_LSRTM_SINC ||
                        d.extraction == SW_EXT_SINC_AFWI;
  // Mirror sources / receivers (Injection.f90:160-164, Extraction.f90:38-50):
  // the injected side of a backward propagation (tmax = 1) follows rec_type.
  const bool inj_mirror = (d.tmax == 1 ? g.rec_type : g.shot_type) != 0;
  const bool ext_mirror = g.rec_type != 0;
  const bool surf = g.surf_type != 0;
  if (d.injection != SW_INJ_NONE && io.nsou > 0)
    if (!make_positions<T>(g, b, io.nsou, io.sou_coord, spos, inj_sinc, inj_mirror, true))
      return SW_BAD_PARAM;
  if (d.extraction != SW_EXT_NONE && io.nrec > 0)
    if (!make_positions<T>(g, b, io.nrec, io.rec_coord, rpos, ext_sinc, ext_mirror))
      return SW_BAD_PARAM;
  // Flat surface at elevation 0 (drivers allocate elev%elev = 0):
  // find_i_d (ModelSpaceTypes.f90:144-151) gives its row and offset.
  int ielev = 1;
  T delev = T(0);
  if (surf) find_i_d<T>(ielev, delev, T(0), (T)g.oz, (T)g.dz);
  const int irow0 = surf ? std::max(ielev, 1) : 1;   // first row kept in snapshots and images
  if (surf && (ielev - 2 * (g.lsinc / 2) - 1 < b.nmin1 - 4 || ielev + 2 * (g.lsinc / 2) > b.nmax1 + 4))
    return SW_BAD_PARAM;
  std::vector<T> fs_sinc(g.lsinc), fs_interp(g.lsinc);
  if (surf && delev != T(0)) mksinc<T>(fs_sinc.data(), g.lsinc, delev / (T)g.dz);

  std::vector<T> taperx, tapery;
  if (d.imaging != SW_IMG_NONE) compute_taper<T>(nx, ny, taperx, tapery);

  const int half = g.lsinc / 2;
  const T dprod2 = (T)g.dz * (T)g.dx;
  const T inv_d2 = T(1) / dprod2;
  const T inv_d3 = T(1) / (dprod2 * (T)g.dy);
  const T xsnap = (T)g.dt * (T)g.snapi;
  const T dt2snap = xsnap * xsnap;   // genpar%dt2 (compute_function_gradient.f90:237)
  int wcounter = 0, mcounter = 0;

  const size_t n3w = (size_t)nz * nx * ny;
  auto W = [&](int i, int j, int k, int s) -> T & {
    return io.wave[(size_t)(i - 1) + (size_t)nz * ((j - 1) + (size_t)nx * ((k - 1) + (size_t)ny * (s - 1)))];
  };
  auto M = [&](T *a, int i, int j, int k) -> T & {
    return a[(size_t)(i - 1) + (size_t)nz * ((j - 1) + (size_t)nx * (k - 1))];
  };
  (void)n3w;

  const int nsteps = (d.tmax - d.tmin + d.tstep) / d.tstep;
  int it = d.tmin;
  for (int s = 0; s < nsteps; ++s, it += d.tstep) {
    // ExtractData(u2) (Propagator.f90:176-178).
    if (d.extraction != SW_EXT_NONE && io.nrec > 0) {
      for (int r = 0; r < io.nrec; ++r) {
        const Pos<T> &p = rpos[r];
        T &tr = io.rec_trace[(size_t)r * nt + (it - 1)];
        if (d.extraction == SW_EXT_SIMPLE_AFWI) {
          // Extraction_array_simple_afwi_noomp (Extraction.f90:71-107).
          const int k1 = g.twoD ? 1 : p.ic[2];
          if (ext_mirror) tr = tr + ((*u2)(p.ic[0], p.ic[1], k1) - (*u2)(-p.ic[0], p.ic[1], k1));
          else tr = tr + (*u2)(p.ic[0], p.ic[1], k1);
          continue;
        }
        T v;
        if (d.extraction == SW_EXT_SINC) {
          // Extraction_array_sinc: v**2 in 2D, v in 3D (Extraction.f90:120-131).
          if (g.twoD) {
            const T vv = vel(p.ic[0], p.ic[1], 1);
            v = vv * vv;
          } else {
            v = vel(p.ic[0], p.ic[1], p.ic[2]);
          }
        } else if (d.extraction == SW_EXT_LSRTM_SINC) {
          v = g.twoD ? inv_d2 : inv_d3;   // Extraction.f90:232-243
        } else {
          v = T(1.);                       // Extraction.f90:137-162
        }
        // The mirror receiver takes u at the cell reflected through row 0
        // (Extraction.f90:549-555, 324-333).
        auto uval = [&](int i, int j, int k) -> T {
          return ext_mirror ? (*u2)(i, j, k) - (*u2)(-i, j, k) : (*u2)(i, j, k);
        };
        if (g.twoD) {
          // Extraction_1trace_sinc_xy (Extraction.f90:511-560).
          for (int j = -half; j <= half; ++j)
            for (int i = -half; i <= half; ++i)
              tr = tr + ((v * uval(i + p.ic[0], j + p.ic[1], 1)) * p.sz[half + i]) * p.sx[half + j];
        } else {
          // Extraction_1trace_sinc_xyz (Extraction.f90:276-337); the y
          // weight is the x sinc column (sinc(maxy+1+k,2)).
          for (int k = -half; k <= half; ++k)
            for (int j = -half; j <= half; ++j)
              for (int i = -half; i <= half; ++i)
                tr = tr + (((v * uval(i + p.ic[0], j + p.ic[1], k + p.ic[2])) * p.sz[half + i]) *
                           p.sx[half + j]) * p.sx[half + k];
        }
      }
    }
    // ExtractWave(u2) = Extraction_wavefield (Extraction.f90:562-601).
    if (d.extract_wave && (it % g.snapi) == 0) {
      ++wcounter;
      if (wcounter <= ntsnap) {
        // With a free surface the rows above it are stored as zero
        // (Extraction.f90:580-592).
        for (int k = 1; k <= ny; ++k)
          for (int j = 1; j <= nx; ++j)
            for (int i = 1; i <= nz; ++i) W(i, j, k, wcounter) = i >= irow0 ? (*u2)(i, j, k) : T(0);
      }
    }
    // ImagingCondition(u2) for tstep = -1 (Propagator.f90:192-194).
    if (d.imaging != SW_IMG_NONE && d.imaging != SW_IMG_BORN && d.tstep == -1 &&
        (it % g.snapi) == 0) {
      ++mcounter;
      const int index = ntsnap - mcounter + 1;
      if (index >= 1) {
        const int ip1 = std::min(index + 1, ntsnap);
        const int im1 = std::max(index - 1, 1);
        for (int k = 1; k <= ny; ++k)
          for (int j = 1; j <= nx; ++j) {
            const T taper = taperx[j - 1] * tapery[k - 1];
            for (int i = irow0; i <= nz; ++i) {
              const T u = (*u2)(i, j, k);
              const T w = W(i, j, k, index);
              T &im = M(io.image, i, j, k);
              T &il = M(io.illum, i, j, k);
              if (d.imaging == SW_IMG_AFWI_RHO) {
                // Imaging_condition_AFWI_RHOVP_from_memory (Imaging.f90:424-511).
                const int dk = ny == 1 ? 0 : 1;
                const int ip = std::min(nz, i + 1), jp = std::min(j + 1, nx), kp = std::min(k + dk, ny);
                const int im_ = ip - 1, jm = jp - 1, km = kp - dk;
                const T dzi = T(1) / (T)g.dz, dxi = T(1) / (T)g.dx, dyi = T(1) / (T)g.dy;
                const T dti2 = T(1) / dt2snap;
                T tmp = dzi * ((*u2)(ip, jm, km) - (*u2)(im_, jm, km)) * dzi *
                        (W(ip, jm, km, index) - W(im_, jm, km, index));
                tmp = tmp + dxi * ((*u2)(im_, jp, km) - (*u2)(im_, jm, km)) * dxi *
                                (W(im_, jp, km, index) - W(im_, jm, km, index));
                tmp = tmp + dyi * ((*u2)(im_, jm, kp) - (*u2)(im_, jm, km)) * dyi *
                                (W(im_, jm, kp, index) - W(im_, jm, km, index));
                const T tmp1 = u * dti2 * ((W(i, j, k, im1) - T(2) * w) + W(i, j, k, ip1));
                const T v = vel(i, j, k);
                const T r = io.rho[(size_t)(i - 1) + (size_t)nz * ((j - 1) + (size_t)nx * (k - 1))];
                im = im + ((T(2) * tmp1) * taper) / (((v * v) * v) * r);
                T &im2 = M(io.image2, i, j, k);
                im2 = im2 + (tmp * taper) / (r * r) + (tmp1 * taper) / ((r * r) * (v * v));
              } else if (d.imaging == SW_IMG_RTM) {
                // Imaging.f90:265-266
                im = im + (u * w) * taper;
              } else if (d.imaging == SW_IMG_LSRTM) {
                // Imaging.f90:735-736
                im = im + (((T(2) * taper) * u) * w) / vel(i, j, k);
              } else {
                // Imaging.f90:410-412
                const T v = vel(i, j, k);
                const T t = ((W(i, j, k, im1) - T(2) * w) + W(i, j, k, ip1)) /
                            (dt2snap * ((v * v) * v));
                im = im + (u * t) * taper;
              }
              il = il + (w * w) * taper;
            }
          }
      }
    }
    // Boundary_set_free_surface_grid (Boundary.f90:1609-1658, called at
    // Propagator.f90:198): zero above the surface, then the mirror image of
    // the rows below it with the opposite sign (on the grid, or through a
    // sinc when the surface lies between rows).
    if (surf) {
      const int h = g.lsinc / 2;
      for (int k = b.nmin3; k <= b.nmax3; ++k)
        for (int j = b.nmin2; j <= b.nmax2; ++j) {
          for (int i = b.nmin1; i <= ielev - 1; ++i) (*u2)(i, j, k) = T(0);
          if (delev == T(0)) {
            for (int i = 0; i <= 2; ++i) (*u2)(ielev - 2 - i, j, k) = -(*u2)(ielev + i, j, k);
          } else {
            for (int i = -h; i <= h; ++i) {
              T f = T(0);
              for (int l = -h; l <= h; ++l) f = f + (*u2)(ielev + l + i, j, k) * fs_sinc[h + l];
              fs_interp[h + i] = f;
            }
            for (int i = 2; i <= h + 1; ++i)
              for (int l = -h; l <= i - 1; ++l)
                (*u2)(ielev - i + l, j, k) =
                    (*u2)(ielev - i + l, j, k) - fs_interp[h + i - 1] * fs_sinc[h + l];
          }
        }
    }
    // FD_scheme(u2 -> u3) (Propagator.f90:202).
    if (io.rho) {
      stencil_rho(rs, b, g.twoD != 0, *u2, *u3, vel);
    } else if (d.fd_scheme == SW_FD_FORWARD) {
      if (g.twoD) stencil2d_fwd(c, b, *u2, *u3, vel);
      else stencil3d_fwd(c, b, *u2, *u3, vel);
    } else {
      if (g.twoD) stencil2d_adj(c, b, *u2, *u3, vel);
      else stencil3d_adj(c, b, *u2, *u3, vel, tmp);
    }
    // Injection(u3) (Propagator.f90:208-209).
    if (d.injection != SW_INJ_NONE) {
      for (int r = 0; r < io.nsou; ++r) {
        const Pos<T> &p = spos[r];
        const T tr = io.sou_trace[(size_t)r * nt + (it - 1)];
        const int k1 = g.twoD ? 1 : p.ic[2];
        if (d.injection == SW_INJ_SIMPLE) {
          // Injection_simple_noomp + Injection_source_simple_xyz
          // (Injection.f90:63-104,561-591); v^2*rho with density.
          const T vv = vel(p.ic[0], p.ic[1], k1);
          const T v2r = io.rho ? (vv * vv) * rs.rho(p.ic[0], p.ic[1], k1) : vv * vv;
          (*u3)(p.ic[0], p.ic[1], k1) = (*u3)(p.ic[0], p.ic[1], k1) + v2r * tr;
          if (inj_mirror) (*u3)(-p.ic[0], p.ic[1], k1) = (*u3)(-p.ic[0], p.ic[1], k1) - v2r * tr;
          continue;
        }
        T v2r;
        if (d.injection == SW_INJ_SINC) {
          // Injection_sinc (Injection.f90:170-190): v^2, times rho with density.
          const T vv = vel(p.ic[0], p.ic[1], k1);
          v2r = io.rho ? (vv * vv) * rs.rho(p.ic[0], p.ic[1], k1) : vv * vv;
        } else {
          v2r = g.twoD ? inv_d2 : inv_d3;   // Injection.f90:258-270
        }
        const T a = v2r * tr;
        if (g.twoD) {
          // Injection_source_sinc_xz (Injection.f90:402-456).
          for (int j = -half; j <= half; ++j)
            for (int i = -half; i <= half; ++i) {
              T &u = (*u3)(i + p.ic[0], j + p.ic[1], 1);
              u = u + (a * p.sz[half + i]) * p.sx[half + j];
              if (inj_mirror) {
                // The mirror source: reflected row, reflected z weight
                // (Injection.f90:440-449).
                T &m = (*u3)(i - p.ic[0], j + p.ic[1], 1);
                m = m - (a * p.sz[half - i]) * p.sx[half + j];
              }
            }
        } else {
          // Injection_source_sinc_xyz (Injection.f90:274-338), x sinc on y.
          for (int k = -half; k <= half; ++k)
            for (int j = -half; j <= half; ++j)
              for (int i = -half; i <= half; ++i) {
                T &u = (*u3)(i + p.ic[0], j + p.ic[1], k + p.ic[2]);
                u = u + ((a * p.sz[half + i]) * p.sx[half + j]) * p.sx[half + k];
                if (inj_mirror) {
                  T &m = (*u3)(i - p.ic[0], j + p.ic[1], k + p.ic[2]);
                  m = m - ((a * p.sz[half - i]) * p.sx[half + j]) * p.sx[half + k];
                }
              }
        }
      }
    }
    // Born secondary source on u3 for tstep = +1 (Propagator.f90:212-214,
    // Injection_Born Imaging.f90:747-788).
    if (d.imaging == SW_IMG_BORN && d.tstep == 1 && (it % g.snapi) == 0) {
      ++mcounter;
      if (mcounter <= ntsnap) {
        for (int k = 1; k <= ny; ++k)
          for (int j = 1; j <= nx; ++j) {
            const T taper = taperx[j - 1] * tapery[k - 1];
            for (int i = irow0; i <= nz; ++i) {
              T &u = (*u3)(i, j, k);
              const T rf = io.ref[(size_t)(i - 1) + (size_t)nz * ((j - 1) + (size_t)nx * (k - 1))];
              u = u + (((T(2) * taper) * rf) * W(i, j, k, mcounter)) / vel(i, j, k);
            }
          }
      }
    }
    // TimeDer (Propagator.f90:218), Higdon (Propagator.f90:222-228).
    time_update(b, (T)g.dt, *u2, *u1, *u0, *um1, *u3);
    if (!g_rigid) boundary(hig, b, *u1, *u2, *u3, surf);
    // FDswaptime_pointer (FDswaptimes.f90:14-24).
    F3<T> *t = um1;
    um1 = u0; u0 = u1; u1 = u2; u2 = u3; u3 = t;
  }
  if (io.final_u2) std::memcpy(io.final_u2, u2->v.data(), u2->v.size() * sizeof(T));
  return SW_OK;
}

// ---------------------------------------------------------------------------
// Drivers
// ---------------------------------------------------------------------------
template <class T>
static sw_prop_desc base_desc(const sw_genpar &g, int fwd) {
  sw_prop_desc d;
  std::memset(&d, 0, sizeof(d));
  d.g = g;
  if (fwd) { d.tmin = 1; d.tmax = g.nt; d.tstep = 1; }
  else { d.tmin = g.nt; d.tmax = 1; d.tstep = -1; }
  return d;
}

template <class T>
static int modeling(const sw_genpar &g, const T *vel, const T *sou_coord,
                    const T *wavelet, int nrec, const T *rec_coord, T *data,
                    T *final_u2) {
  // progs/modeling/Acoustic_modeling.f90:115-123.
  sw_prop_desc d = base_desc<T>(g, 1);
  d.fd_scheme = SW_FD_FORWARD;
  d.injection = SW_INJ_SINC;
  d.extraction = SW_EXT_SINC;
  IO<T> io{};
  io.vel = vel;
  io.nsou = 1; io.sou_coord = sou_coord; io.sou_trace = wavelet;
  io.nrec = nrec; io.rec_coord = rec_coord; io.rec_trace = data;
  io.final_u2 = final_u2;
  std::fill(data, data + (size_t)nrec * g.nt, T(0));
  return propagate<T>(d, io);
}

template <class T>
static int rtm_like(const sw_genpar &g, const T *vel, const T *sou_coord,
                    const T *wavelet, int nrec, const T *rec_coord, const T *data,
                    T *image, T *illum, bool lsrtm) {
  // RTM_to_memory / LSRTM_to_memory (progs/rtm/to_disk_to_memory_RTM.f90:358-580).
  const int ntsnap = g.nt / g.snapi;
  const size_t n3 = (size_t)g.nz * g.nx * g.ny;
  std::vector<T> wave(n3 * (size_t)std::max(ntsnap, 1), T(0));
  sw_prop_desc d = base_desc<T>(g, 1);
  d.fd_scheme = SW_FD_FORWARD;
  d.injection = SW_INJ_SINC;
  d.extract_wave = 1;
  IO<T> io{};
  io.vel = vel;
  io.nsou = 1; io.sou_coord = sou_coord; io.sou_trace = wavelet;
  io.wave = wave.data();
  int st = propagate<T>(d, io);
  if (st) return st;
  std::fill(image, image + n3, T(0));
  std::fill(illum, illum + n3, T(0));
  sw_prop_desc b = base_desc<T>(g, 0);
  if (lsrtm) {
    b.fd_scheme = SW_FD_ADJOINT;
    b.injection = SW_INJ_LSRTM_SINC;
    b.imaging = SW_IMG_LSRTM;
  } else {
    b.fd_scheme = g.twoD ? SW_FD_ADJOINT : SW_FD_FORWARD;
    b.injection = SW_INJ_SINC;
    b.imaging = SW_IMG_RTM;
  }
  IO<T> jo{};
  jo.vel = vel;
  jo.nsou = nrec; jo.sou_coord = rec_coord; jo.sou_trace = data;
  jo.wave = wave.data();
  jo.image = image; jo.illum = illum;
  return propagate<T>(b, jo);
}

template <class T>
static int born(const sw_genpar &g, const T *vel, const T *ref, const T *sou_coord,
                const T *wavelet, int nrec, const T *rec_coord, T *data) {
  // BORN_to_memory (progs/modeling/to_disk_to_memory_BORN.f90:123-220).
  const int ntsnap = g.nt / g.snapi;
  const size_t n3 = (size_t)g.nz * g.nx * g.ny;
  std::vector<T> wave(n3 * (size_t)std::max(ntsnap, 1), T(0));
  sw_prop_desc d = base_desc<T>(g, 1);
  d.fd_scheme = SW_FD_FORWARD;
  d.injection = SW_INJ_SINC;
  d.extract_wave = 1;
  IO<T> io{};
  io.vel = vel;
  io.nsou = 1; io.sou_coord = sou_coord; io.sou_trace = wavelet;
  io.wave = wave.data();
  int st = propagate<T>(d, io);
  if (st) return st;
  std::fill(data, data + (size_t)nrec * g.nt, T(0));
  sw_prop_desc b = base_desc<T>(g, 1);
  b.fd_scheme = SW_FD_FORWARD;
  b.injection = SW_INJ_NONE;     // no sou: Injection is never called
  b.extraction = SW_EXT_LSRTM_SINC;
  b.imaging = SW_IMG_BORN;
  IO<T> jo{};
  jo.vel = vel;
  jo.nrec = nrec; jo.rec_coord = rec_coord; jo.rec_trace = data;
  jo.wave = wave.data();
  jo.ref = ref;
  return propagate<T>(b, jo);
}

// ---------------------------------------------------------------------------
// FWI objective / gradient
// ---------------------------------------------------------------------------

// triangle / boxconv (libs/libwave/Smoothing.f90:140-229).
static void boxconv(int nb, int nx, const float *xx, float *yy) {
  const int ny = nx + nb - 1;
  std::vector<float> bb(nx + nb, 0.f);
  bb[0] = xx[0];
  for (int i = 2; i <= nx; ++i) bb[i - 1] = bb[i - 2] + xx[i - 1];
  for (int i = nx + 1; i <= ny; ++i) bb[i - 1] = bb[i - 2];
  for (int i = 1; i <= nb; ++i) yy[i - 1] = bb[i - 1];
  for (int i = nb + 1; i <= ny; ++i) yy[i - 1] = bb[i - 1] - bb[i - nb - 1];
  for (int i = 1; i <= ny; ++i) yy[i - 1] = yy[i - 1] / (float)nb;
}

static void triangle(int nr, int n12, const float *uu, float *vv) {
  std::vector<float> pp(n12 + nr - 1), qq(n12 + 2 * nr - 1), tt(n12);
  for (int i = 0; i < n12; ++i) qq[i] = uu[i];
  if (n12 == 1) {
    tt[0] = qq[0];
  } else {
    boxconv(nr, n12, qq.data(), pp.data());
    const int np = nr + n12 - 1;
    boxconv(nr, np, pp.data(), qq.data());
    for (int i = 1; i <= n12; ++i) tt[i - 1] = qq[i + nr - 2];
    for (int i = 1; i <= nr - 1; ++i) tt[i - 1] = tt[i - 1] + qq[nr - i - 1];
    for (int i = 1; i <= nr - 1; ++i)
      tt[n12 - i] = tt[n12 - i] + qq[n12 + (nr - 1) + i - 1];
  }
  for (int i = 0; i < n12; ++i) vv[i] = tt[i];
}

// triangle2 (Smoothing.f90:87-138).  The reference's y pass uses rect1/n1
// and its x pass copies uu=ss inside the i3 loop; both only matter in 3D and
// read unset memory there, so the 3D passes use the intended rect3/n3 and a
// single copy after the loop.
static int triangle2(float *uu, int n1, int n2, int n3, int rect1, int rect2,
                     int rect3, bool doz, bool dox, bool doy) {
  auto U = [&](int i1, int i2, int i3) -> float & {
    return uu[(size_t)i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)];
  };
  if ((dox && (rect2 < 1 || rect2 > n2)) || (doz && (rect1 < 1 || rect1 > n1)) ||
      (doy && (rect3 < 1 || rect3 > n3)))
    return SW_BAD_PARAM;
  std::vector<float> ss((size_t)n1 * n2 * n3);
  std::vector<float> a, bq;
  if (dox) {
    a.resize(n2); bq.resize(n2);
    for (int i3 = 0; i3 < n3; ++i3)
      for (int i1 = 0; i1 < n1; ++i1) {
        for (int i2 = 0; i2 < n2; ++i2) a[i2] = U(i1, i2, i3);
        triangle(rect2, n2, a.data(), bq.data());
        for (int i2 = 0; i2 < n2; ++i2) ss[(size_t)i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)] = bq[i2];
      }
    std::memcpy(uu, ss.data(), ss.size() * sizeof(float));
  }
  if (doz) {
    a.resize(n1); bq.resize(n1);
    for (int i3 = 0; i3 < n3; ++i3)
      for (int i2 = 0; i2 < n2; ++i2) {
        triangle(rect1, n1, &U(0, i2, i3), bq.data());
        for (int i1 = 0; i1 < n1; ++i1) ss[(size_t)i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)] = bq[i1];
      }
    std::memcpy(uu, ss.data(), ss.size() * sizeof(float));
  }
  if (doy) {
    a.resize(n3); bq.resize(n3);
    for (int i2 = 0; i2 < n2; ++i2)
      for (int i1 = 0; i1 < n1; ++i1) {
        for (int i3 = 0; i3 < n3; ++i3) a[i3] = U(i1, i2, i3);
        triangle(rect3, n3, a.data(), bq.data());
        for (int i3 = 0; i3 < n3; ++i3) ss[(size_t)i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)] = bq[i3];
      }
    std::memcpy(uu, ss.data(), ss.size() * sizeof(float));
  }
  return SW_OK;
}

// Shot window: extract_coord_source_receiver_patch
// (ExtractPadModel.f90:19-85) and copy_window_vel_gath (ExtractPadModel.f90:
// 395-507) with mod_window_pad(adj=.true.) (ExtractPadModel.f90:509-549).
struct Window {
  float oxw, oyw, endx, endy;
  int nxw, nyw;
};

static int shot_window(const sw_fwi_desc &d, const sw_fwi_shot &s, Window &w) {
  const sw_genpar &g = d.g;
  const float sx = s.sou_coord[1], sy = s.sou_coord[2];
  if (s.nrec < 1) return SW_BAD_PARAM;
  float gx1 = s.rec_coord[1], gy1 = s.rec_coord[2], gxn = gx1, gyn = gy1;
  for (int i = 1; i < s.nrec; ++i) {
    gx1 = std::min(gx1, s.rec_coord[3 * i + 1]);
    gxn = std::max(gxn, s.rec_coord[3 * i + 1]);
    gy1 = std::min(gy1, s.rec_coord[3 * i + 2]);
    gyn = std::max(gyn, s.rec_coord[3 * i + 2]);
  }
  const float minx = std::min(sx, gx1), miny = std::min(sy, gy1);
  const float maxx = std::max(sx, gxn), maxy = std::max(sy, gyn);
  const float mx1 = (gx1 + sx) / 2, mxn = (gxn + sx) / 2;
  const float my1 = (gy1 + sy) / 2, myn = (gyn + sy) / 2;
  const float cx = mx1 + std::fabs(mxn - mx1) / 2;
  const float cy = my1 + std::fabs(myn - my1) / 2;
  w.oxw = std::min(minx, cx - d.aperture_x / 2);
  w.endx = std::max(maxx, cx + d.aperture_x / 2);
  w.oyw = std::min(miny, cy - d.aperture_y / 2);
  w.endy = std::max(maxy, cy + d.aperture_y / 2);
  w.nxw = (int)lroundf((w.endx - w.oxw) / g.dx) + 1;
  w.nyw = (int)lroundf((w.endy - w.oyw) / g.dy) + 1;
  if (g.twoD) { w.nyw = 1; w.oyw = g.oy; }
  return SW_OK;
}

static void window_vel(const sw_genpar &g, const Window &w, const float *big, float *small) {
  for (int j = 1; j <= w.nyw; ++j) {
    const float cy = (float)(j - 1) * g.dy + w.oyw;
    const int iy = (int)lroundf((cy - g.oy) / g.dy) + 1;
    const int iy1 = std::min(g.ny, std::max(1, iy));
    for (int i = 1; i <= w.nxw; ++i) {
      const float cx = (float)(i - 1) * g.dx + w.oxw;
      const int ix = (int)lroundf((cx - g.ox) / g.dx) + 1;
      const int ix1 = std::min(g.nx, std::max(1, ix));
      for (int l = 0; l < g.nz; ++l)
        small[(size_t)l + (size_t)g.nz * ((i - 1) + (size_t)w.nxw * (j - 1))] =
            0.f + big[(size_t)l + (size_t)g.nz * ((ix1 - 1) + (size_t)g.nx * (iy1 - 1))];
    }
  }
}

// mod_copy_image (ExtractPadModel.f90:662-697).
static void copy_image(const sw_genpar &g, const Window &w, const float *ims,
                       const float *ils, float *image, float *illum) {
  for (int j = 1; j <= w.nyw; ++j) {
    const float cy = (float)(j - 1) * g.dy + w.oyw;
    const int iy = (int)lroundf((cy - g.oy) / g.dy) + 1;
    if (iy < 1 || iy > g.ny) continue;
    for (int i = 1; i <= w.nxw; ++i) {
      const float cx = (float)(i - 1) * g.dx + w.oxw;
      const int ix = (int)lroundf((cx - g.ox) / g.dx) + 1;
      if (ix < 1 || ix > g.nx) continue;
      for (int l = 0; l < g.nz; ++l) {
        const size_t o = (size_t)l + (size_t)g.nz * ((ix - 1) + (size_t)g.nx * (iy - 1));
        const size_t s = (size_t)l + (size_t)g.nz * ((i - 1) + (size_t)w.nxw * (j - 1));
        image[o] = image[o] + ims[s];
        illum[o] = illum[o] + ils[s];
      }
    }
  }
}

// compute_mig-style stacking of RTM_to_memory images
// (compute_function_gradient.f90:352-470, to_disk_to_memory_RTM.f90:358-492).
static int rtm_job(const sw_genpar &M, float apx, float apy, const float *vel,
                   const float *wavelet, int nshot, const sw_shot *shots, float *image,
                   float *illum, float *image_norm) {
  const size_t nfull = (size_t)M.nz * M.nx * M.ny;
  std::vector<float> im(nfull, 0.f), il(nfull, 0.f);
  sw_fwi_desc d;
  std::memset(&d, 0, sizeof(d));
  d.g = M;
  d.aperture_x = apx;
  d.aperture_y = apy;
  for (int is = 0; is < nshot; ++is) {
    const sw_shot &s = shots[is];
    sw_fwi_shot fs;
    std::memset(&fs, 0, sizeof(fs));
    std::memcpy(fs.sou_coord, s.sou_coord, sizeof(fs.sou_coord));
    fs.nrec = s.nrec;
    fs.rec_coord = s.rec_coord;
    Window w;
    int st = shot_window(d, fs, w);
    if (st) return st;
    sw_genpar g = M;
    g.nx = w.nxw; g.ny = w.nyw; g.ox = w.oxw; g.oy = w.oyw; g.nt = s.nt;
    const size_t nw = (size_t)g.nz * g.nx * g.ny;
    std::vector<float> vs(nw), ims(nw), ils(nw);
    window_vel(M, w, vel, vs.data());
    st = rtm_like<float>(g, vs.data(), s.sou_coord, wavelet, s.nrec, s.rec_coord, s.data,
                         ims.data(), ils.data(), false);
    if (st) return st;
    copy_image(M, w, ims.data(), ils.data(), im.data(), il.data());
  }
  if (image) std::memcpy(image, im.data(), nfull * sizeof(float));
  if (illum) std::memcpy(illum, il.data(), nfull * sizeof(float));
  if (image_norm) {
    float m = il[0];
    double ss = 0.;
    for (size_t q = 0; q < nfull; ++q) {
      m = std::max(m, il[q]);
      ss = ss + (double)il[q] * (double)il[q];
    }
    const double r = std::sqrt(ss / (double)nfull);
    for (size_t q = 0; q < nfull; ++q)
      image_norm[q] = im[q] / (float)((double)(il[q] + m / 10000.f) / r);
  }
  return SW_OK;
}

// fct_compute (libs/libinv/Norm.f90:12-81) of one trace rd[0..n): L2 as an
// FP64 sum of FP64 products, the other norms as FP32 sums in sample order
// (sum() of a real array).  thresh is the caller's threshold: when it is 0
// the thresholded norms set it to max|rd| (Norm.f90:37-40), and the caller
// keeps that value for its next traces.
static double norm_fct(int ntype, const float *rd, int n, float &thresh) {
  if (ntype == SW_NRM_L2) {
    double s = 0.;
    for (int t = 0; t < n; ++t) s = s + (double)rd[t] * (double)rd[t];
    return s / 2;
  }
  if (ntype == SW_NRM_L1) {
    float s = 0.f;
    for (int t = 0; t < n; ++t) s = s + std::fabs(rd[t]);
    return (double)s;
  }
  if (thresh == 0.f) {
    float mx = 0.f;
    for (int t = 0; t < n; ++t) mx = std::fmax(mx, std::fabs(rd[t]));
    thresh = mx;
  }
  const float g = thresh;
  float s = 0.f;
  for (int t = 0; t < n; ++t) {
    float v;
    if (ntype == SW_NRM_HUBER) {
      const float a = std::fabs(rd[t]);
      v = a > g ? a - g / 2.0f : rd[t] * rd[t] / (2.0f * g);
    } else if (ntype == SW_NRM_CAUCHY) {
      const float q = rd[t] / g;
      v = std::log(1.0f + q * q) / 2.0f;
    } else {
      v = std::sqrt(g * g + rd[t] * rd[t]) - g;
    }
    s = s + v;
  }
  return (double)s;
}

// gdt_compute (libs/libinv/Norm.f90:83-141): the adjoint source of one
// trace, in place, with the threshold fct_compute left.
static void norm_gdt(int ntype, float *rd, int n, float g) {
  for (int t = 0; t < n; ++t) {
    const float e = rd[t];
    switch (ntype) {
      case SW_NRM_L2: break;
      case SW_NRM_L1: rd[t] = e < 0.f ? -1.f : (e > 0.f ? 1.f : 0.f); break;
      case SW_NRM_HUBER: rd[t] = std::fmax(-1.0f, std::fmin(1.0f, e / g)); break;
      case SW_NRM_CAUCHY: rd[t] = e / (g * g + e * e); break;
      default: rd[t] = (e / g) / std::sqrt(1.0f + e * e / (g * g)); break;
    }
  }
}

// Compute_OF_RES_ADJ (Objective_Function_Residual_Adjsource.f90:17-40) of
// one gather: dmod (modelled traces in, adjoint source out), the residual
// m*(dobs - dmod) into resid when given; every trace's misfit is added to
// the running total f in trace order.  The threshold starts from
// data_threshold for every gather.
static void residual_gather(int ntype, float thresh0, int nrec, int nt, const float *dobs,
                            const float *mute, float *dmod, float *resid, double &f) {
  float thresh = thresh0;
  for (int r = 0; r < nrec; ++r) {
    float *dm = &dmod[(size_t)r * nt];
    const float *dob = &dobs[(size_t)r * nt];
    const float *mu = mute ? &mute[(size_t)r * nt] : nullptr;
    for (int t = 0; t < nt; ++t) {
      const float m = mu ? mu[t] : 1.f;
      dm[t] = m * (dob[t] - dm[t]);
    }
    f = f + norm_fct(ntype, dm, nt, thresh);
    if (resid) std::memcpy(&resid[(size_t)r * nt], dm, sizeof(float) * nt);
    for (int t = 0; t < nt; ++t) {
      const float m = mu ? mu[t] : 1.f;
      dm[t] = m * dm[t];
    }
    norm_gdt(ntype, dm, nt, thresh);
  }
}

static bool known_norm(int ntype) {
  return ntype == SW_NRM_L1 || ntype == SW_NRM_L2 || ntype == SW_NRM_HUBER ||
         ntype == SW_NRM_CAUCHY || ntype == SW_NRM_HYPERBOLIC;
}

static int fwi_fct_gdt(const sw_fwi_desc &d, const float *vel, const float *wavelet,
                       int nshot, const sw_fwi_shot *shots, const float *vpmask,
                       double *f, float *grad, float *illum_out) {
  const sw_genpar &G = d.g;
  const size_t nfull = (size_t)G.nz * G.nx * G.ny;
  const int nt = G.nt;
  const int ntype = d.dat_nrm_type == 0 ? SW_NRM_L2 : d.dat_nrm_type;
  if (!known_norm(ntype)) return SW_BAD_PARAM;
  std::vector<float> gradacc(nfull, 0.f), illacc(nfull, 0.f);
  double fsum = 0.;
  long ntotaltraces = 0;
  for (int is = 0; is < nshot; ++is) {
    const sw_fwi_shot &s = shots[is];
    Window w;
    int st = shot_window(d, s, w);
    if (st) return st;
    sw_genpar g = G;
    g.nx = w.nxw;
    g.ny = w.nyw;
    g.ox = w.oxw;
    g.oy = w.oyw;
    const size_t nw = (size_t)g.nz * g.nx * g.ny;
    std::vector<float> vsmall(nw);
    window_vel(G, w, vel, vsmall.data());
    const int ntsnap = nt / g.snapi;
    std::vector<float> wave(nw * (size_t)std::max(ntsnap, 1), 0.f);
    std::vector<float> dmod((size_t)s.nrec * nt, 0.f);
    // AMOD_to_memory (progs/afwi/to_disk_to_memory_AMOD.f90:27-82).
    sw_prop_desc a = base_desc<float>(g, 1);
    a.fd_scheme = SW_FD_FORWARD;
    a.injection = SW_INJ_SINC;
    a.extraction = SW_EXT_SIMPLE_AFWI;
    a.extract_wave = 1;
    IO<float> io{};
    io.vel = vsmall.data();
    io.nsou = 1; io.sou_coord = s.sou_coord; io.sou_trace = wavelet;
    io.nrec = s.nrec; io.rec_coord = s.rec_coord; io.rec_trace = dmod.data();
    io.wave = wave.data();
    st = propagate<float>(a, io);
    if (st) return st;
    residual_gather(ntype, d.dat_thresh, s.nrec, nt, s.dobs, s.mute, dmod.data(), s.resid, fsum);
    ntotaltraces += s.nrec;
    // AGRAD_to_memory (progs/afwi/to_disk_to_memory_AGRAD.f90:27-79).
    std::vector<float> ims(nw, 0.f), ils(nw, 0.f);
    sw_prop_desc b = base_desc<float>(g, 0);
    b.fd_scheme = SW_FD_FORWARD;
    b.injection = SW_INJ_SIMPLE;
    b.imaging = SW_IMG_AFWI;
    IO<float> jo{};
    jo.vel = vsmall.data();
    jo.nsou = s.nrec; jo.sou_coord = s.rec_coord; jo.sou_trace = dmod.data();
    jo.wave = wave.data();
    jo.image = ims.data(); jo.illum = ils.data();
    st = propagate<float>(b, jo);
    if (st) return st;
    copy_image(G, w, ims.data(), ils.data(), gradacc.data(), illacc.data());
  }
  // Post-processing (compute_function_gradient.f90:314-343).
  for (size_t q = 0; q < nfull; ++q) {
    if (d.illu_pow != 1.f) illacc[q] = powf(illacc[q], d.illu_pow);
  }
  const double scaling = (double)(2 * (long)nt * ntotaltraces);
  fsum = fsum / scaling;
  const float sscal = (float)scaling;
  float maxil = illacc[0];
  double ss = 0.;
  for (size_t q = 0; q < nfull; ++q) {
    gradacc[q] = (2.f * gradacc[q]) / sscal;
    maxil = std::max(maxil, illacc[q]);
    ss = ss + (double)illacc[q] * (double)illacc[q];
  }
  const double rmsil = std::sqrt(ss / (double)nfull);
  for (size_t q = 0; q < nfull; ++q) {
    illacc[q] = (float)((double)(illacc[q] + maxil / 10000.f) / rmsil);
    gradacc[q] = gradacc[q] / illacc[q];
    gradacc[q] = gradacc[q] * (vpmask ? vpmask[q] : 1.f);
  }
  int st = triangle2(gradacc.data(), G.nz, G.nx, G.ny, d.smooth_rect1, d.smooth_rect2,
                     d.smooth_rect3, d.smooth_doz != 0, d.smooth_dox != 0,
                     d.smooth_doy != 0);
  if (st) return st;
  for (size_t q = 0; q < nfull; ++q) gradacc[q] = gradacc[q] * (vpmask ? vpmask[q] : 1.f);
  *f = fsum;
  std::memcpy(grad, gradacc.data(), nfull * sizeof(float));
  if (illum_out) std::memcpy(illum_out, illacc.data(), nfull * sizeof(float));
  return SW_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// L-BFGS (libs/libinv/lbfgs.f)
// ---------------------------------------------------------------------------
struct or_lbfgs {
  int n, m;
  double xmin, xmax;
  std::vector<float> mask;
  int boundt;
  bool type;
  std::vector<double> xinit;
  std::vector<double> w;     // 1-based, N*(2M+1)+2M
  std::vector<double> diag;  // 1-based
  // libs/libnlinv's variant (LBFGSOC / LBFGSOLD): per-parameter bounds, the
  // first-step options and its line-search constants.
  bool oc = false;
  int nparam = 1;
  std::vector<double> pmin, pmax;
  int stp1_opt = 1;
  double step_init = 999999.0;
  // LBFGS SAVE state
  int iter = 0, nfun = 0, point = 0, ispt = 0, iypt = 0, npt = 0, bound = 0, info = 0,
      nfev = 0, maxfev = 20, cp = 0;
  double stp = 0, stp1 = 0, ftol = 1e-4, gnorm = 0, xnorm = 0, ys = 0, yy = 0;
  bool finish = false;
  // MCSRCH SAVE state
  int infoc = 0;
  bool brackt = false, stage1 = true;
  double dg = 0, dgm = 0, dginit = 0, dgtest = 0, dgx = 0, dgxm = 0, dgy = 0, dgym = 0,
         finit = 0, ftest1 = 0, fm = 0, fx = 0, fxm = 0, fy = 0, fym = 0, stx = 0, sty = 0,
         stmin = 0, stmax = 0, width = 0, width1 = 0;
};

namespace {
// COMMON /LB3/ from BLOCK DATA LB2 (lbfgs.f:636-641).
const double kGTOL = 0.9, kSTPMIN = 1.0e-20, kSTPMAX = 1.0e+20;

// ddot with the reference's unroll-by-5 summation order (blas.f:58-90).
double ddot(int n, const double *dx, const double *dy) {
  double dtemp = 0.0;
  if (n <= 0) return 0.0;
  const int m = n % 5;
  for (int i = 0; i < m; ++i) dtemp = dtemp + dx[i] * dy[i];
  if (n < 5) return dtemp;
  for (int i = m; i < n; i += 5)
    dtemp = dtemp + dx[i] * dy[i] + dx[i + 1] * dy[i + 1] + dx[i + 2] * dy[i + 2] +
            dx[i + 3] * dy[i + 3] + dx[i + 4] * dy[i + 4];
  return dtemp;
}

// FREEZE_XOC (nlinv_lbfgs.f:1-22): block j of n / nparam values clipped to
// [xmin(j), xmax(j)].
void freeze_xoc(const or_lbfgs &s, double *x) {
  const int m = s.n / s.nparam;
  for (int j = 0; j < s.nparam; ++j)
    for (int i = j * m; i < j * m + m; ++i) {
      x[i] = std::max(s.pmin[j], x[i]);
      x[i] = std::min(s.pmax[j], x[i]);
    }
}

// FREEZE_X (lbfgs.f:1-43).
void freeze_x(const or_lbfgs &s, double *x) {
  if (s.oc) {
    freeze_xoc(s, x);
    return;
  }
  if (s.type) {
    for (int i = 0; i < s.n; ++i) {
      x[i] = std::max(s.xmin, x[i]);
      x[i] = std::min(s.xmax, x[i]);
    }
  } else {
    for (int i = 0; i < s.n; ++i)
      if (s.mask[i] != 0.f && s.mask[i] != 2.f) {
        x[i] = std::max(s.xmin, x[i]);
        x[i] = std::min(s.xmax, x[i]);
      }
    for (int i = 0; i < s.n; ++i)
      if (s.mask[i] == 0.f || s.mask[i] == 2.f) x[i] = s.xinit[i];
  }
}

// MCSTEP (lbfgs.f:985-1210).
void mcstep(double &stx, double &fx, double &dx, double &sty, double &fy, double &dy,
            double &stp, double fp, double dp, bool &brackt, double stpmin,
            double stpmax, int &info) {
  info = 0;
  if ((brackt && (stp <= std::min(stx, sty) || stp >= std::max(stx, sty))) ||
      dx * (stp - stx) >= 0.0 || stpmax < stpmin)
    return;
  const double sgnd = dp * (dx / std::fabs(dx));
  bool bound;
  double theta, s, gamma, p, q, r, stpc, stpq, stpf;
  if (fp > fx) {
    info = 1;
    bound = true;
    theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
    s = std::max(std::max(std::fabs(theta), std::fabs(dx)), std::fabs(dp));
    gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp < stx) gamma = -gamma;
    p = (gamma - dx) + theta;
    q = ((gamma - dx) + gamma) + dp;
    r = p / q;
    stpc = stx + r * (stp - stx);
    stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2) * (stp - stx);
    if (std::fabs(stpc - stx) < std::fabs(stpq - stx))
      stpf = stpc;
    else
      stpf = stpc + (stpq - stpc) / 2;
    brackt = true;
  } else if (sgnd < 0.0) {
    info = 2;
    bound = false;
    theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
    s = std::max(std::max(std::fabs(theta), std::fabs(dx)), std::fabs(dp));
    gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp > stx) gamma = -gamma;
    p = (gamma - dp) + theta;
    q = ((gamma - dp) + gamma) + dx;
    r = p / q;
    stpc = stp + r * (stx - stp);
    stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (std::fabs(stpc - stp) > std::fabs(stpq - stp))
      stpf = stpc;
    else
      stpf = stpq;
    brackt = true;
  } else if (std::fabs(dp) < std::fabs(dx)) {
    info = 3;
    bound = true;
    theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
    s = std::max(std::max(std::fabs(theta), std::fabs(dx)), std::fabs(dp));
    gamma = s * std::sqrt(std::max(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
    if (stp > stx) gamma = -gamma;
    p = (gamma - dp) + theta;
    q = (gamma + (dx - dp)) + gamma;
    r = p / q;
    if (r < 0.0 && gamma != 0.0)
      stpc = stp + r * (stx - stp);
    else if (stp > stx)
      stpc = stpmax;
    else
      stpc = stpmin;
    stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (brackt) {
      if (std::fabs(stp - stpc) < std::fabs(stp - stpq))
        stpf = stpc;
      else
        stpf = stpq;
    } else {
      if (std::fabs(stp - stpc) > std::fabs(stp - stpq))
        stpf = stpc;
      else
        stpf = stpq;
    }
  } else {
    info = 4;
    bound = false;
    if (brackt) {
      theta = 3 * (fp - fy) / (sty - stp) + dy + dp;
      s = std::max(std::max(std::fabs(theta), std::fabs(dy)), std::fabs(dp));
      gamma = s * std::sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
      if (stp > sty) gamma = -gamma;
      p = (gamma - dp) + theta;
      q = ((gamma - dp) + gamma) + dy;
      r = p / q;
      stpc = stp + r * (sty - stp);
      stpf = stpc;
    } else if (stp > stx) {
      stpf = stpmax;
    } else {
      stpf = stpmin;
    }
  }
  if (fp > fx) {
    sty = stp; fy = fp; dy = dp;
  } else {
    if (sgnd < 0.0) { sty = stx; fy = fx; dy = dx; }
    stx = stp; fx = fp; dx = dp;
  }
  stpf = std::min(stpmax, stpf);
  stpf = std::max(stpmin, stpf);
  stp = stpf;
  // The literal 0.66 is a REAL constant in the F77 source.
  const double p66s = (double)0.66f;
  if (brackt && bound) {
    if (sty > stx)
      stp = std::min(stx + p66s * (sty - stx), stp);
    else
      stp = std::max(stx + p66s * (sty - stx), stp);
  }
}

// MCSRCH (lbfgs.f:652-982).  s = search direction, wa = work (DIAG).
void mcsrch(or_lbfgs &S, double *x, double f, const double *g, const double *s,
            double &stp, double ftol, double xtol, int maxfev, int &info, int &nfev,
            double *wa) {
  const int n = S.n;
  // XTRAPF is 4.0D1 in libinv's MCSRCH (lbfgs.f:792) and 4.0D0 in libnlinv's
  // MCSRCHOC / MCSRCHOLD (nlinv_lbfgs.f:752,1773).
  const double p5 = 0.5, p66 = 0.66, xtrapf = S.oc ? 4.0 : 40.0, zero = 0.0;
  if (info == -1) goto L45;
  S.infoc = 1;
  if (n <= 0 || stp <= zero || ftol < zero || kGTOL < zero || xtol < zero ||
      kSTPMIN < zero || kSTPMAX < kSTPMIN || maxfev <= 0)
    return;
  S.dginit = zero;
  for (int j = 0; j < n; ++j) S.dginit = S.dginit + g[j] * s[j];
  if (S.dginit >= zero) return;
  S.brackt = false;
  S.stage1 = true;
  nfev = 0;
  S.finit = f;
  S.dgtest = ftol * S.dginit;
  S.width = kSTPMAX - kSTPMIN;
  S.width1 = S.width / p5;
  for (int j = 0; j < n; ++j) wa[j] = x[j];
  S.stx = zero; S.fx = S.finit; S.dgx = S.dginit;
  S.sty = zero; S.fy = S.finit; S.dgy = S.dginit;
L30:
  if (S.brackt) {
    S.stmin = std::min(S.stx, S.sty);
    S.stmax = std::max(S.stx, S.sty);
  } else {
    S.stmin = S.stx;
    S.stmax = stp + xtrapf * (stp - S.stx);
  }
  stp = std::max(stp, kSTPMIN);
  stp = std::min(stp, kSTPMAX);
  if ((S.brackt && (stp <= S.stmin || stp >= S.stmax)) || nfev >= maxfev - 1 ||
      S.infoc == 0 || (S.brackt && S.stmax - S.stmin <= xtol * S.stmax))
    stp = S.stx;
  for (int j = 0; j < n; ++j) x[j] = wa[j] + stp * s[j];
  if (S.boundt == 1) freeze_x(S, x);
  info = -1;
  return;
L45:
  info = 0;
  nfev = nfev + 1;
  S.dg = zero;
  for (int j = 0; j < n; ++j) S.dg = S.dg + g[j] * s[j];
  S.ftest1 = S.finit + stp * S.dgtest;
  if ((S.brackt && (stp <= S.stmin || stp >= S.stmax)) || S.infoc == 0) info = 6;
  if (stp == kSTPMAX && f <= S.ftest1 && S.dg <= S.dgtest) info = 5;
  if (stp == kSTPMIN && (f > S.ftest1 || S.dg >= S.dgtest)) info = 4;
  if (nfev >= maxfev) info = 3;
  if (S.brackt && S.stmax - S.stmin <= xtol * S.stmax) info = 2;
  if (f <= S.ftest1 && std::fabs(S.dg) <= kGTOL * (-S.dginit)) info = 1;
  if (info != 0) return;
  if (S.stage1 && f <= S.ftest1 && S.dg >= std::min(ftol, kGTOL) * S.dginit) S.stage1 = false;
  if (S.stage1 && f <= S.fx && f > S.ftest1) {
    S.fm = f - stp * S.dgtest;
    S.fxm = S.fx - S.stx * S.dgtest;
    S.fym = S.fy - S.sty * S.dgtest;
    S.dgm = S.dg - S.dgtest;
    S.dgxm = S.dgx - S.dgtest;
    S.dgym = S.dgy - S.dgtest;
    mcstep(S.stx, S.fxm, S.dgxm, S.sty, S.fym, S.dgym, stp, S.fm, S.dgm, S.brackt,
           S.stmin, S.stmax, S.infoc);
    S.fx = S.fxm + S.stx * S.dgtest;
    S.fy = S.fym + S.sty * S.dgtest;
    S.dgx = S.dgxm + S.dgtest;
    S.dgy = S.dgym + S.dgtest;
  } else {
    mcstep(S.stx, S.fx, S.dgx, S.sty, S.fy, S.dgy, stp, f, S.dg, S.brackt, S.stmin,
           S.stmax, S.infoc);
  }
  if (S.brackt) {
    if (std::fabs(S.sty - S.stx) >= p66 * S.width1) stp = S.stx + p5 * (S.sty - S.stx);
    S.width1 = S.width;
    S.width = std::fabs(S.sty - S.stx);
  }
  goto L30;
}

// LBFGS (lbfgs.f:49-558), DIAGCO = .false.
int lbfgs(or_lbfgs &S, double *x, double f, const double *g, double eps, double xtol,
          int &iflag, int &myinfo) {
  const int n = S.n, m = S.m;
  double *W = S.w.data();      // W[1..]
  double *DIAG = S.diag.data(); // DIAG[1..]
  if (iflag == 0) goto L10;
  if (iflag == 1) goto L172;
  if (iflag == 2) goto L100;
  return SW_BAD_PARAM;
L10:
  S.iter = 0;
  if (n <= 0 || m <= 0) { iflag = -3; return SW_OK; }
  S.nfun = 1;
  S.point = 0;
  S.finish = false;
  for (int i = 1; i <= n; ++i) DIAG[i] = 1.0;
  S.ispt = n + 2 * m;
  S.iypt = S.ispt + n * m;
  for (int i = 1; i <= n; ++i) W[S.ispt + i] = -g[i - 1] * DIAG[i];
  S.gnorm = std::sqrt(ddot(n, g, g));
  if (S.oc) {
    // nlinv_lbfgs.f:333-341 (LBFGSOLD, :1366-1370: step_init or 1/|g|).
    if (S.stp1_opt == 1) S.stp1 = std::sqrt(ddot(n, x, x)) / S.gnorm / 100;
    else S.stp1 = 1.0 / S.gnorm;
    if (S.step_init != 999999.0) S.stp1 = S.step_init;
  } else {
    const double xnorm2 = std::sqrt(ddot(n, x, x));
    if (S.boundt == 0) S.stp1 = 1.0 / S.gnorm;
    else S.stp1 = xnorm2 / S.gnorm / 100;
  }
  S.ftol = 1.0e-4;
  S.maxfev = 20;
L80:
  S.iter = S.iter + 1;
  S.info = 0;
  S.bound = S.iter - 1;
  if (S.iter == 1) goto L165;
  if (S.iter > m) S.bound = m;
  S.ys = 0.0;
  for (int j = 1; j <= n; ++j) S.ys = S.ys + W[S.iypt + S.npt + j] * W[S.ispt + S.npt + j];
  S.yy = 0.0;
  for (int j = 1; j <= n; ++j) S.yy = S.yy + W[S.iypt + S.npt + j] * W[S.iypt + S.npt + j];
  for (int i = 1; i <= n; ++i) DIAG[i] = S.ys / S.yy;
L100:
  S.cp = S.point;
  if (S.point == 0) S.cp = m;
  W[n + S.cp] = 1.0 / S.ys;
  for (int i = 1; i <= n; ++i) W[i] = -g[i - 1];
  S.cp = S.point;
  for (int i = 1; i <= S.bound; ++i) {
    S.cp = S.cp - 1;
    if (S.cp == -1) S.cp = m - 1;
    double sq = 0.0;
    for (int j = 1; j <= n; ++j) sq = sq + W[S.ispt + S.cp * n + j] * W[j];
    const int inmc = n + m + S.cp + 1;
    const int iycn = S.iypt + S.cp * n;
    W[inmc] = W[n + S.cp + 1] * sq;
    for (int j = 1; j <= n; ++j) W[j] = W[j] - W[inmc] * W[iycn + j];
  }
  for (int i = 1; i <= n; ++i) W[i] = DIAG[i] * W[i];
  for (int i = 1; i <= S.bound; ++i) {
    double yr = 0.0;
    for (int j = 1; j <= n; ++j) yr = yr + W[S.iypt + S.cp * n + j] * W[j];
    double beta = W[n + S.cp + 1] * yr;
    const int inmc = n + m + S.cp + 1;
    beta = W[inmc] - beta;
    const int iscn = S.ispt + S.cp * n;
    for (int j = 1; j <= n; ++j) W[j] = W[j] + beta * W[iscn + j];
    S.cp = S.cp + 1;
    if (S.cp == m) S.cp = 0;
  }
  for (int i = 1; i <= n; ++i) W[S.ispt + S.point * n + i] = W[i];
L165:
  S.nfev = 0;
  S.stp = 1.0;
  if (S.iter == 1) S.stp = S.stp1;
  for (int i = 1; i <= n; ++i) W[i] = g[i - 1];
L172:
  mcsrch(S, x, f, g, &W[S.ispt + S.point * n + 1], S.stp, S.ftol, xtol, S.maxfev, S.info,
         S.nfev, &DIAG[1]);
  if (S.info == -1) { iflag = 1; return SW_OK; }
  if (S.info != 1) { iflag = -1; return SW_OK; }
  S.nfun = S.nfun + S.nfev;
  myinfo = S.info;
  if (S.boundt == 2 && S.info == 1) freeze_x(S, x);
  S.npt = S.point * n;
  for (int i = 1; i <= n; ++i) {
    W[S.ispt + S.npt + i] = S.stp * W[S.ispt + S.npt + i];
    W[S.iypt + S.npt + i] = g[i - 1] - W[i];
  }
  S.point = S.point + 1;
  if (S.point == m) S.point = 0;
  S.gnorm = std::sqrt(ddot(n, g, g));
  S.xnorm = std::sqrt(ddot(n, x, x));
  S.xnorm = std::max(1.0, S.xnorm);
  if (S.gnorm / S.xnorm <= eps) S.finish = true;
  if (S.finish) { iflag = 0; return SW_OK; }
  goto L80;
}

}  // namespace

// ---------------------------------------------------------------------------
// C entry points
// ---------------------------------------------------------------------------
extern "C" {

void oracle_set_rigid(int on) { g_rigid = on != 0; }

int oracle_propagate_f32(const sw_prop_desc *d, const sw_prop_io *io) {
  IO<float> o{io->vel, io->nsou, io->sou_coord, io->sou_trace, io->nrec, io->rec_coord,
              io->rec_trace, io->wave, io->image, io->illum, io->ref, io->final_u2, io->rho,
              io->image2};
  return propagate<float>(*d, o);
}

int oracle_propagate_f64(const sw_prop_desc *d, const or_prop_io64 *io) {
  IO<double> o{io->vel, io->nsou, io->sou_coord, io->sou_trace, io->nrec, io->rec_coord,
               io->rec_trace, io->wave, io->image, io->illum, io->ref, io->final_u2, io->rho,
               io->image2};
  return propagate<double>(*d, o);
}

int oracle_modeling_f32(const sw_genpar *g, const float *vel, const float *sou_coord,
                        const float *wavelet, int nrec, const float *rec_coord,
                        float *data, float *final_u2) {
  return modeling<float>(*g, vel, sou_coord, wavelet, nrec, rec_coord, data, final_u2);
}
int oracle_modeling_f64(const sw_genpar *g, const double *vel, const double *sou_coord,
                        const double *wavelet, int nrec, const double *rec_coord,
                        double *data, double *final_u2) {
  return modeling<double>(*g, vel, sou_coord, wavelet, nrec, rec_coord, data, final_u2);
}
int oracle_rtm_f32(const sw_genpar *g, const float *vel, const float *sou_coord,
                   const float *wavelet, int nrec, const float *rec_coord,
                   const float *data, float *image, float *illum) {
  return rtm_like<float>(*g, vel, sou_coord, wavelet, nrec, rec_coord, data, image,
                         illum, false);
}
int oracle_rtm_f64(const sw_genpar *g, const double *vel, const double *sou_coord,
                   const double *wavelet, int nrec, const double *rec_coord,
                   const double *data, double *image, double *illum) {
  return rtm_like<double>(*g, vel, sou_coord, wavelet, nrec, rec_coord, data, image,
                          illum, false);
}
int oracle_born_f32(const sw_genpar *g, const float *vel, const float *ref,
                    const float *sou_coord, const float *wavelet, int nrec,
                    const float *rec_coord, float *data) {
  return born<float>(*g, vel, ref, sou_coord, wavelet, nrec, rec_coord, data);
}
int oracle_born_f64(const sw_genpar *g, const double *vel, const double *ref,
                    const double *sou_coord, const double *wavelet, int nrec,
                    const double *rec_coord, double *data) {
  return born<double>(*g, vel, ref, sou_coord, wavelet, nrec, rec_coord, data);
}
int oracle_lsrtm_f32(const sw_genpar *g, const float *vel, const float *sou_coord,
                     const float *wavelet, int nrec, const float *rec_coord,
                     const float *data, float *image, float *illum) {
  return rtm_like<float>(*g, vel, sou_coord, wavelet, nrec, rec_coord, data, image,
                         illum, true);
}
int oracle_lsrtm_f64(const sw_genpar *g, const double *vel, const double *sou_coord,
                     const double *wavelet, int nrec, const double *rec_coord,
                     const double *data, double *image, double *illum) {
  return rtm_like<double>(*g, vel, sou_coord, wavelet, nrec, rec_coord, data, image,
                          illum, true);
}

// readsou Born/LSRTM branch (ReadSouVelRho.f90:318-326).
// ---------------------------------------------------------------------------
// Band-pass (libs/libwave/Bandpass.f90:89-149 and the Butterworth filters of
// libs/libwave/bandpass.c), restated with the reference's work arrays: data,
// newdata and tempdata zeroed per trace, the filters writing samples 2..n-1,
// every section copying newdata back in full.  The float/double mix of the C
// coefficient formulas is kept.  The Fortran copies data(npad+1:nt) into an
// nt-sample trace, a non-conforming assignment; it is taken as the nt samples
// from npad+1 on (the unpadded trace).
// ---------------------------------------------------------------------------
namespace {
const double kPiD = 3.1415926535897932384626433832795028841971693;

struct BpCoef {
  int ns;
  std::vector<float> c;   // 5 per section
};

BpCoef bp_highcut(float fhi, int nphi, int phase) {
  int nodd = nphi % 2;
  if (phase == 0) {
    if (nodd != 0) nphi = (nphi + 1) / 2;
    else nphi = nphi / 2;
    nodd = nphi % 2;
  }
  BpCoef r;
  r.ns = (nphi + 1) / 2;
  r.c.assign(5 * r.ns, 0.f);
  float a = (float)(2.0 * tan(kPiD * fhi));
  float aa = a * a;
  float aap4 = (float)(aa + 4.0);
  float dtheta = (float)(kPiD / nphi);
  float theta0 = nodd != 0 ? 0.0f : (float)(dtheta / 2.0);
  if (nodd != 0) {
    r.c[0] = (float)(a / (a + 2.0));
    r.c[1] = r.c[0];
    r.c[2] = 0.0f;
    r.c[3] = (float)((a - 2.0) / (a + 2.0));
    r.c[4] = 0.0f;
  }
  for (int j = nodd; j < r.ns; ++j) {
    double c = 4.0 * a * cos((double)(theta0 + j * dtheta));
    r.c[5 * j + 0] = (float)(aa / (aap4 + c));
    r.c[5 * j + 1] = (float)(2.0 * r.c[5 * j + 0]);
    r.c[5 * j + 2] = r.c[5 * j + 0];
    r.c[5 * j + 3] = (float)((2.0 * aa - 8.0) / (aap4 + c));
    r.c[5 * j + 4] = (float)((aap4 - c) / (aap4 + c));
  }
  return r;
}

BpCoef bp_lowcut(float flo, int nplo, int phase) {
  int nodd = nplo % 2;
  if (phase == 0) {
    if (nodd != 0) nplo = (nplo + 1) / 2;
    else nplo = nplo / 2;
    nodd = nplo % 2;
  }
  BpCoef r;
  r.ns = (nplo + 1) / 2;
  r.c.assign(5 * r.ns, 0.f);
  float fno2 = 0.25f;
  float a = (float)(2. * sin(kPiD * fno2) / cos(kPiD * fno2));
  float aa = a * a;
  float aap4 = aa + 4;
  float e = (float)(-cos(kPiD * (flo + fno2)) / cos(kPiD * (flo - fno2)));
  float ee = e * e;
  float dtheta = (float)(kPiD / nplo);
  float theta0 = nodd != 0 ? 0.0f : dtheta / 2;
  if (nodd != 0) {
    float b1 = a / (a + 2);
    float b2 = (a - 2) / (a + 2);
    float den = (float)(1.0 - b2 * e);
    r.c[0] = (float)(b1 * (1. - e) / den);
    r.c[1] = -r.c[0];
    r.c[2] = 0.f;
    r.c[3] = (e - b2) / den;
    r.c[4] = 0.f;
  }
  for (int j = nodd; j < r.ns; ++j) {
    double c = 4. * a * cos((double)(theta0 + j * dtheta));
    float b1 = (float)(aa / (aap4 + c));
    float b2 = (float)((2. * aa - 8.) / (aap4 + c));
    float b3 = (float)((aap4 - c) / (aap4 + c));
    float den = (float)(1. - b2 * e + b3 * ee);
    r.c[5 * j + 0] = (float)(b1 * (1. - e) * (1. - e) / den);
    r.c[5 * j + 1] = (float)(-2. * r.c[5 * j + 0]);
    r.c[5 * j + 2] = r.c[5 * j + 0];
    r.c[5 * j + 3] = (float)((2. * e * (1. + b3) - b2 * (1. + ee)) / den);
    r.c[5 * j + 4] = (ee - b2 * e + b3) / den;
  }
  return r;
}

void bp_run(const BpCoef &k, int phase, int n1, float *data, float *newdata, float *tempdata) {
  for (int s = 0; s < k.ns; ++s) {
    const float *b = &k.c[5 * s];
    for (int i1 = 2; i1 < n1; ++i1)
      newdata[i1] = b[0] * data[i1] + b[1] * data[i1 - 1] + b[2] * data[i1 - 2] -
                    b[3] * newdata[i1 - 1] - b[4] * newdata[i1 - 2];
    for (int i1 = 0; i1 < n1; ++i1) data[i1] = newdata[i1];
  }
  if (phase == 0) {
    for (int i1 = 2; i1 < n1; ++i1) tempdata[i1] = data[n1 + 1 - i1];
    for (int s = 0; s < k.ns; ++s) {
      const float *b = &k.c[5 * s];
      for (int i1 = 2; i1 < n1; ++i1)
        newdata[i1] = b[0] * tempdata[i1] + b[1] * tempdata[i1 - 1] + b[2] * tempdata[i1 - 2] -
                      b[3] * newdata[i1 - 1] - b[4] * newdata[i1 - 2];
      for (int i1 = 0; i1 < n1; ++i1) tempdata[i1] = newdata[i1];
    }
    for (int i1 = 2; i1 < n1; ++i1) data[i1] = tempdata[n1 + 1 - i1];
  }
}
}  // namespace

int oracle_bandpass(float *traces, int ntr, int nt, float dt, float flo, float fhi, int nplo,
                    int nphi, int phase) {
  const float pi = 3.1415926535f;
  const float flo_tmp = flo * dt, fhi_tmp = fhi * dt;
  const int npad = 10, n1pad = nt + 2 * npad;
  if (flo_tmp < 0.0001f && fhi_tmp > 0.4999f) return SW_BAD_PARAM;
  std::vector<float> data(n1pad), newdata(n1pad), tempdata(n1pad);
  for (int i = 0; i < ntr; ++i) {
    float *in = traces + (size_t)i * nt;
    std::fill(data.begin(), data.end(), 0.f);
    std::fill(newdata.begin(), newdata.end(), 0.f);
    std::fill(tempdata.begin(), tempdata.end(), 0.f);
    for (int q = 0; q < nt; ++q) data[npad + q] = in[q];
    for (int j = 1; j <= npad; ++j) {
      const float s1 = sinf((j - 1) * pi / (2 * (npad - 1)));
      const float s2 = sinf((npad - j) * pi / (2 * (npad - 1)));
      data[j - 1] = in[0] * (s1 * s1);
      data[n1pad - npad + j - 1] = in[nt - 1] * (s2 * s2);
    }
    if (flo_tmp > 0.000001f) bp_run(bp_lowcut(flo_tmp, nplo, phase), phase, n1pad, data.data(),
                                     newdata.data(), tempdata.data());
    if (fhi_tmp < 4.999999f) bp_run(bp_highcut(fhi_tmp, nphi, phase), phase, n1pad, data.data(),
                                    newdata.data(), tempdata.data());
    for (int q = 0; q < nt; ++q) in[q] = data[npad + q];
  }
  return SW_OK;
}

// compute_top_mute / compute_bottom_mute (libs/libwave/Mute.f90:172-219) and
// their product (MuteParam_compute_mask, Mute.f90:50-95).  Array sections
// that would start before sample 1 start at sample 1.
int oracle_mute_mask(int nrec, int nt, float dt, float ot, const float *sou,
                     const float *rec, float v0, float v1, float t0, float t1, float tramp,
                     float *mask) {
  const float pi = 3.1415926535f;
  std::vector<float> top(nt + 1), bot(nt + 1);
  for (int r = 0; r < nrec; ++r) {
    const float hx = rec[3 * r + 1] - sou[1], hy = rec[3 * r + 2] - sou[2];
    int nramp = (int)(tramp / dt + 1.5f);
    float tmute = sqrtf(t0 * t0 + ((hx + hy) / v0) * ((hx + hy) / v0));
    int it = (int)((tmute - ot) / dt + 1.5f);
    for (int i = 1; i <= nt; ++i) top[i] = 0.f;
    for (int i = std::max(1, it - nramp); i <= std::min(nt, it); ++i) {
      const float sv = sinf((i - it + nramp) * pi / (2 * nramp));
      top[i] = sv * sv;
    }
    for (int i = std::max(1, it + 1); i <= nt; ++i) top[i] = 1.f;
    tmute = sqrtf(t1 * t1 + ((hx + hy) / v1) * ((hx + hy) / v1));
    it = (int)((tmute - ot) / dt + 1.5f);
    for (int i = 1; i <= nt; ++i) bot[i] = 1.f;
    for (int i = std::max(1, it + 1); i <= std::min(nt, it + 1 + nramp); ++i) {
      const float cv = cosf((i - it - 1) * pi / (2 * nramp));
      bot[i] = cv * cv;
    }
    for (int i = std::max(1, it + 1 + nramp); i <= nt; ++i) bot[i] = 0.f;
    for (int i = 1; i <= nt; ++i) mask[(size_t)r * nt + i - 1] = top[i] * bot[i];
  }
  return SW_OK;
}

// readsou withRho branch (ReadSouVelRho.f90:328-343).
int oracle_rho_wavelet(float *w, int nt, int lsinc) {
  std::vector<float> sinc(lsinc), tr(w, w + nt);
  mksinc<float>(sinc.data(), lsinc, 0.5f);
  const int h = lsinc / 2;
  for (int it = 1; it <= nt; ++it) {
    float fscale = 1.f, fdum = 0.f;
    for (int l = -h; l <= h; ++l) {
      if (it + l >= 1 && it + l <= nt) fdum = fdum + sinc[h + l] * tr[it + l - 1];
      else fscale = fscale - sinc[h + l];
    }
    w[it - 1] = fdum / fscale;
  }
  return SW_OK;
}

int oracle_born_wavelet(float *w, int nt, float dt) {
  if (nt < 1) return SW_BAD_PARAM;
  std::vector<float> tr(w, w + nt);
  for (int i = 0; i < nt; ++i) w[i] = 0.f;
  for (int it = 2; it <= nt - 1; ++it)
    w[it - 1] = w[it - 1] + ((-2 * tr[it - 1] + tr[it - 2]) + tr[it]) / (dt * dt);
  return SW_OK;
}

// vel_check (ReadSouVelRho.f90:603-756).
int oracle_vel_check(const sw_genpar *g, const float *vel, float *courant, float *samplerate) {
  const size_t n = (size_t)g->nz * g->nx * g->ny;
  float vmax = vel[0], vmin = vel[0];
  for (size_t q = 1; q < n; ++q) { vmax = std::max(vmax, vel[q]); vmin = std::min(vmin, vel[q]); }
  const float stab_cond = g->twoD ? 0.45f : 0.35f;
  float stab;
  if (g->twoD) stab = vmax * g->dt / std::min(g->dz, g->dx);
  else stab = vmax * g->dt / std::min(std::min(g->dz, g->dx), g->dy);
  const float lambdamin = vmin / g->fmax;
  float sr;
  if (g->twoD) sr = lambdamin / std::max(g->dz, g->dx);
  else sr = lambdamin / std::max(std::max(g->dz, g->dx), g->dy);
  if (courant) *courant = stab;
  if (samplerate) *samplerate = sr;
  if (stab > stab_cond) return SW_BAD_PARAM;
  if (sr < 2.0f) return SW_BAD_PARAM;
  return SW_OK;
}

int oracle_fwi_fct_gdt(const sw_fwi_desc *d, const float *vel, const float *wavelet,
                       int nshot, const sw_fwi_shot *shots, const float *vpmask,
                       double *f, float *grad, float *illum) {
  return fwi_fct_gdt(*d, vel, wavelet, nshot, shots, vpmask, f, grad, illum);
}

// ---------------------------------------------------------------------------
// Model regularisation of 2DAFWI (compute_fct_gdt_reg,
// progs/afwi/compute_function_gradient.f90:98-206).
// ---------------------------------------------------------------------------
struct RegGrid {
  int nz, nx, ny, tz, tx, ty;
  size_t nzt() const { return (size_t)nz + 2 * tz; }
  size_t nxt() const { return (size_t)nx + 2 * tx; }
  size_t nyt() const { return (size_t)ny + 2 * ty; }
  size_t ntap() const { return nzt() * nxt() * nyt(); }
  size_t n() const { return (size_t)nz * nx * ny; }
  // Index of model sample (iz, ix, iy) in the padded array.
  size_t tap(int iz, int ix, int iy) const {
    return (size_t)(iz + tz) + nzt() * ((size_t)(ix + tx) + nxt() * (size_t)(iy + ty));
  }
};

// SparseRegularization_add_taper, forw (Sparse_regularization.f90:399-437):
// the interior is the model, the pads repeat the edge samples (z first, then
// x, then y, which is the clamped index on every axis).
static void reg_pad(const RegGrid &R, const float *a, float *tap) {
  for (size_t k = 0; k < R.nyt(); ++k)
    for (size_t j = 0; j < R.nxt(); ++j)
      for (size_t i = 0; i < R.nzt(); ++i) {
        const int iz = std::min(std::max((int)i - R.tz, 0), R.nz - 1);
        const int ix = std::min(std::max((int)j - R.tx, 0), R.nx - 1);
        const int iy = std::min(std::max((int)k - R.ty, 0), R.ny - 1);
        tap[i + R.nzt() * (j + R.nxt() * k)] = a[iz + (size_t)R.nz * (ix + (size_t)R.nx * iy)];
      }
}

// helicon_mod_lop (libs/libflt/helicon.f90:25-60) with the filters that
// SparseRegularization_filter_init builds (Sparse_regularization.f90:
// 166-213): createhelix of the GEE helix library (not in the reference
// tree) gives, for a 2-point box along one axis with the "1" at its first
// point, a single lag (1 along z, nzt along x, nzt*nxt along y), and flt is
// set to -1.  The output is cleared (adjnull), the zero lag added, then the
// lag term, over the whole padded array as one line (the helix).
static void helix_fwd(const float *xx, float *yy, size_t n, size_t lag) {
  for (size_t i = 0; i < n; ++i) yy[i] = 0.f + xx[i];
  for (size_t iy = lag; iy < n; ++iy) yy[iy] = yy[iy] + xx[iy - lag] * -1.f;
}
static void helix_adj(float *xx, const float *yy, size_t n, size_t lag) {
  for (size_t i = 0; i < n; ++i) xx[i] = 0.f + yy[i];
  for (size_t iy = lag; iy < n; ++iy) xx[iy - lag] = xx[iy - lag] + yy[iy] * -1.f;
}

// SparseRegularization_Compute_f_g (Sparse_regularization.f90:258-327) and,
// with logistic set, LogisticRegularization_Compute_f_g (:329-397).
static void reg_compute_f_g(const RegGrid &R, const float *zweight, const float *vel,
                            size_t lag, bool hinge, bool logistic, int ntype, float &thresh,
                            double &f, float *g) {
  const size_t nt = R.ntap(), n = R.n();
  std::vector<float> zwt(nt, 1.f), mask(nt, logistic ? 0.f : 1.f), rm(nt), rt(nt), gtmp(n, 0.f);
  if (zweight) reg_pad(R, zweight, zwt.data());
  reg_pad(R, vel, rt.data());
  helix_fwd(rt.data(), rm.data(), nt, lag);
  if (logistic) {
    for (size_t i = 0; i < nt; ++i) mask[i] = rm[i] <= 0.f ? 1.f : 0.f;
    for (size_t i = 0; i < nt; ++i) rm[i] = rm[i] * mask[i] * zwt[i];
  } else {
    if (hinge)
      for (size_t i = 0; i < nt; ++i) mask[i] = rm[i] <= 0.f ? 0.f : 1.f;
    for (size_t i = 0; i < nt; ++i) rm[i] = rm[i] * zwt[i] * mask[i];
  }
  for (int iy = 0; iy < R.ny; ++iy)
    for (int ix = 0; ix < R.nx; ++ix)
      for (int iz = 0; iz < R.nz; ++iz) {
        const size_t k = iz + (size_t)R.nz * (ix + (size_t)R.nx * iy);
        gtmp[k] = gtmp[k] + rm[R.tap(iz, ix, iy)];
      }
  f = f + norm_fct(ntype, gtmp.data(), R.nz * R.nx, thresh);
  norm_gdt(ntype, rm.data(), (int)(R.nzt() * R.nxt()), thresh);
  for (size_t i = 0; i < nt; ++i)
    rm[i] = logistic ? mask[i] * rm[i] * zwt[i] : rm[i] * zwt[i] * mask[i];
  helix_adj(rt.data(), rm.data(), nt, lag);
  for (int iy = 0; iy < R.ny; ++iy)
    for (int ix = 0; ix < R.nx; ++ix)
      for (int iz = 0; iz < R.nz; ++iz) {
        const size_t k = iz + (size_t)R.nz * (ix + (size_t)R.nx * iy);
        g[k] = g[k] + (0.f + rt[R.tap(iz, ix, iy)]);
      }
}

static int fwi_regularize(const sw_reg_desc &d, sw_reg_state &st, int eval, const float *vel,
                          const float *vpmask, double &f, float *grad) {
  if (d.nz < 1 || d.nx < 1 || d.ny < 1 || d.ntaperz < 0 || d.ntaperx < 0 || d.ntapery < 0)
    return SW_BAD_PARAM;
  const int mtype = d.mod_nrm_type == 0 ? SW_NRM_L2 : d.mod_nrm_type;
  const int htype = d.hin_nrm_type == 0 ? SW_NRM_L2 : d.hin_nrm_type;
  if ((d.wantreg && !known_norm(mtype)) || (d.wantlog && !known_norm(htype))) return SW_BAD_PARAM;
  // Init_SparseRegularization (Sparse_regularization.f90:81-93): no y pad in 2D.
  const RegGrid R{d.nz, d.nx, d.ny, d.ntaperz, d.ntaperx, d.ny != 1 ? d.ntapery : 0};
  const size_t n = R.n();
  const double scaling = (double)d.nx * d.ny * d.nz;
  double ftmp = 0., ftmp1 = 0.;
  std::vector<float> gtmp(n);
  if (d.compute_eps && eval == 0) st.eps = 0.f;
  if (d.compute_eps_log && eval == 0) st.eps_log = 0.f;
  if (d.wantreg) {
    // SparseRegularization_apply (:238-256): x, then z, then y (the x filter).
    std::fill(gtmp.begin(), gtmp.end(), 0.f);
    const size_t lx = R.nzt();
    if (d.derivdx)
      reg_compute_f_g(R, d.zweight, vel, lx, false, false, mtype, st.mod_thresh, ftmp, gtmp.data());
    if (d.derivdz)
      reg_compute_f_g(R, d.zweight, vel, 1, d.log_z_plus != 0, false, mtype, st.mod_thresh, ftmp,
                      gtmp.data());
    if (d.ny != 1 && d.derivdy)
      reg_compute_f_g(R, d.zweight, vel, lx, false, false, mtype, st.mod_thresh, ftmp, gtmp.data());
    ftmp = ftmp / scaling;
    for (size_t i = 0; i < n; ++i) gtmp[i] = gtmp[i] / (float)scaling;
    if (d.compute_eps && eval == 0) {
      if (d.ratio == 0.f)
        st.eps = 0.f;
      else if (ftmp != 0.)
        st.eps = (float)std::fabs(f / ((double)d.ratio * ftmp));
      else
        return SW_NUMERIC;
    }
    for (size_t i = 0; i < n; ++i) grad[i] = grad[i] - gtmp[i] * st.eps;
  } else {
    st.eps = 0.f;
  }
  if (d.wantlog) {
    std::fill(gtmp.begin(), gtmp.end(), 0.f);
    reg_compute_f_g(R, d.zweight, vel, 1, false, true, htype, st.hin_thresh, ftmp1, gtmp.data());
    ftmp1 = ftmp1 / scaling;
    for (size_t i = 0; i < n; ++i) gtmp[i] = gtmp[i] / (float)scaling;
    if (d.compute_eps_log && eval == 0) {
      if (d.ratio_log == 0.f)
        st.eps_log = 0.f;
      else if (ftmp1 == 0.)
        st.eps_log = (float)std::fabs(f / ((double)d.ratio_log * ftmp));
      else
        st.eps_log = (float)std::fabs(f / ((double)d.ratio_log * ftmp1));
    }
    for (size_t i = 0; i < n; ++i) grad[i] = grad[i] - gtmp[i] * st.eps_log;
  } else {
    st.eps_log = 0.f;
  }
  if (vpmask)
    for (size_t i = 0; i < n; ++i) grad[i] = grad[i] * vpmask[i];
  f = f + ftmp * (double)st.eps + ftmp1 * (double)st.eps_log;
  return SW_OK;
}

int oracle_fwi_regularize(const sw_reg_desc *d, sw_reg_state *state, int eval, const float *vel,
                          const float *vpmask, double *f, float *grad) {
  if (!d || !state || !vel || !f || !grad) return SW_BAD_PARAM;
  return fwi_regularize(*d, *state, eval, vel, vpmask, *f, grad);
}

int oracle_data_norm(int ntype, float thresh, int nrec, int nt, const float *dobs,
                     const float *mute, float *dmod, float *resid, double *f) {
  if (ntype == 0) ntype = SW_NRM_L2;
  if (!known_norm(ntype) || nrec < 0 || nt < 0 || !f) return SW_BAD_PARAM;
  *f = 0.;
  residual_gather(ntype, thresh, nrec, nt, dobs, mute, dmod, resid, *f);
  return SW_OK;
}

int oracle_rtm_job(const sw_genpar *model, float apx, float apy, const float *vel,
                   const float *wavelet, int nshot, const sw_shot *shots, float *image,
                   float *illum, float *image_norm) {
  return rtm_job(*model, apx, apy, vel, wavelet, nshot, shots, image, illum, image_norm);
}

// One application of the scalar stencil (forward: v^2 Lap u; adjoint:
// Lap(v^2 u)) on a padded field; the compute domain of out is overwritten.
int oracle_stencil_f64(const sw_genpar *g, int adjoint, const double *vel,
                       const double *u2, double *u3) {
  int st = check_genpar(*g);
  if (st) return st;
  const Bounds b = make_bounds(*g);
  F3<double> v, a, o, t;
  v.init(b); a.init(b); o.init(b);
  model_pad(vel, v, b, g->nz, g->nx, g->ny, g->twoD != 0);
  std::memcpy(a.v.data(), u2, a.v.size() * sizeof(double));
  std::memcpy(o.v.data(), u3, o.v.size() * sizeof(double));
  const Coefs<double> c = make_coefs<double>(*g);
  if (!adjoint) {
    if (g->twoD) stencil2d_fwd(c, b, a, o, v);
    else stencil3d_fwd(c, b, a, o, v);
  } else {
    if (g->twoD) stencil2d_adj(c, b, a, o, v);
    else { t.init(b); stencil3d_adj(c, b, a, o, v, t); }
  }
  std::memcpy(u3, o.v.data(), o.v.size() * sizeof(double));
  return SW_OK;
}

int oracle_stencil_rho_f64(const sw_genpar *g, const double *vel, const double *rho,
                           const double *u2, double *u3) {
  int st = check_genpar(*g);
  if (st) return st;
  const Bounds b = make_bounds(*g);
  F3<double> v, a, o;
  v.init(b); a.init(b); o.init(b);
  model_pad(vel, v, b, g->nz, g->nx, g->ny, g->twoD != 0);
  std::memcpy(a.v.data(), u2, a.v.size() * sizeof(double));
  std::memcpy(o.v.data(), u3, o.v.size() * sizeof(double));
  RhoState<double> rs;
  rho_state_init(rs, *g, b, rho);
  stencil_rho(rs, b, g->twoD != 0, a, o, v);
  std::memcpy(u3, o.v.data(), o.v.size() * sizeof(double));
  return SW_OK;
}

int oracle_triangle2(float *uu, int n1, int n2, int n3, int rect1, int rect2, int rect3,
                     int doz, int dox, int doy) {
  return triangle2(uu, n1, n2, n3, rect1, rect2, rect3, doz != 0, dox != 0, doy != 0);
}

void oracle_mksinc(float *sinc, int lsinc, float shift) { mksinc<float>(sinc, lsinc, shift); }

or_lbfgs *oracle_lbfgs_create(int n, int m, double xmin, double xmax, const float *mask,
                              int bound_type, int freeze_soft, const double *xinit) {
  or_lbfgs *s = new or_lbfgs();
  s->n = n; s->m = m; s->xmin = xmin; s->xmax = xmax;
  s->mask.assign(mask, mask + n);
  s->boundt = bound_type;
  s->type = freeze_soft != 0;
  s->xinit.assign(xinit, xinit + n);
  s->w.assign((size_t)n * (2 * m + 1) + 2 * m + 1, 0.0);
  s->diag.assign((size_t)n + 1, 0.0);
  return s;
}
void oracle_lbfgs_destroy(or_lbfgs *s) { delete s; }
int oracle_lbfgs_step(or_lbfgs *s, double *x, double f, const double *g, double eps,
                      double xtol, int *iflag, int *myinfo) {
  return lbfgs(*s, x, f, g, eps, xtol, *iflag, *myinfo);
}
// One LBFGSOC / LBFGSOLD call (nlinv_lbfgs.f:31-613,1066-1636) with the
// saved state passed in and out, as L_BFGS.f90 keeps it in files.
int oracle_lbfgs_oc_step(const sw_lbfgs_oc_desc *d, double *x, double f, const double *g,
                         double *w, double *diag, sw_lbfgs_oc_state *st, int *iflag,
                         int *myinfo) {
  if (!d || d->n <= 0 || d->m <= 0 || d->nparam <= 0 || d->n % d->nparam) return SW_BAD_PARAM;
  const int n = d->n, m = d->m;
  or_lbfgs S;
  S.n = n; S.m = m;
  S.oc = true;
  S.nparam = d->nparam;
  S.type = false;
  if (d->lbfgs_type == 1) {
    if (!d->xmin || !d->xmax) return SW_BAD_PARAM;
    S.pmin.assign(d->xmin, d->xmin + d->nparam);
    S.pmax.assign(d->xmax, d->xmax + d->nparam);
    S.boundt = d->bound_type;
    S.stp1_opt = d->stp1_opt;
  } else {
    S.boundt = 0;
    S.stp1_opt = 0;
  }
  S.step_init = d->step_init;
  const size_t nw = (size_t)n * (2 * m + 1) + 2 * m;
  S.w.assign(nw + 1, 0.0);
  S.diag.assign((size_t)n + 1, 0.0);
  if (*iflag != 0) {
    std::copy(w, w + nw, S.w.begin() + 1);
    std::copy(diag, diag + n, S.diag.begin() + 1);
    S.gnorm = st->gnorm; S.stp1 = st->stp1; S.ftol = st->ftol; S.stp = st->stp;
    S.ys = st->ys; S.yy = st->yy; S.xnorm = st->xnorm;
    S.iter = st->iter; S.nfun = st->nfun; S.point = st->point; S.ispt = st->ispt;
    S.iypt = st->iypt; S.maxfev = st->maxfev; S.info = st->info; S.bound = st->bound;
    S.npt = st->npt; S.cp = st->cp; S.nfev = st->nfev; S.finish = st->finish != 0;
    S.infoc = st->infoc; S.brackt = st->brackt != 0; S.stage1 = st->stage1 != 0;
    S.dg = st->dg; S.dgm = st->dgm; S.dginit = st->dginit; S.dgtest = st->dgtest;
    S.dgx = st->dgx; S.dgxm = st->dgxm; S.dgy = st->dgy; S.dgym = st->dgym;
    S.finit = st->finit; S.ftest1 = st->ftest1; S.fm = st->fm; S.fx = st->fx;
    S.fxm = st->fxm; S.fy = st->fy; S.fym = st->fym; S.stx = st->stx; S.sty = st->sty;
    S.stmin = st->stmin; S.stmax = st->stmax; S.width = st->width; S.width1 = st->width1;
  }
  const int rc = lbfgs(S, x, f, g, d->eps, d->xtol, *iflag, *myinfo);
  std::copy(S.w.begin() + 1, S.w.end(), w);
  std::copy(S.diag.begin() + 1, S.diag.end(), diag);
  std::memset(st, 0, sizeof(*st));
  st->gtol = kGTOL; st->one = 1.0; st->zero = 0.0; st->gnorm = S.gnorm; st->stp1 = S.stp1;
  st->ftol = S.ftol; st->stpmin = kSTPMIN; st->stpmax = kSTPMAX; st->stp = S.stp;
  st->ys = S.ys; st->yy = S.yy; st->xnorm = S.xnorm;
  st->mp = 6; st->lp = 6; st->iter = S.iter; st->nfun = S.nfun; st->point = S.point;
  st->ispt = n + 2 * m; st->iypt = n + 2 * m + n * m; st->maxfev = S.maxfev;
  st->info = S.info; st->bound = S.bound; st->npt = S.npt; st->cp = S.cp; st->nfev = S.nfev;
  st->finish = S.finish ? 1 : 0;
  st->infoc = S.infoc; st->brackt = S.brackt ? 1 : 0; st->stage1 = S.stage1 ? 1 : 0;
  st->dg = S.dg; st->dgm = S.dgm; st->dginit = S.dginit; st->dgtest = S.dgtest;
  st->dgx = S.dgx; st->dgxm = S.dgxm; st->dgy = S.dgy; st->dgym = S.dgym;
  st->finit = S.finit; st->ftest1 = S.ftest1; st->fm = S.fm; st->fx = S.fx; st->fxm = S.fxm;
  st->fy = S.fy; st->fym = S.fym; st->stx = S.stx; st->sty = S.sty;
  st->stmin = S.stmin; st->stmax = S.stmax; st->width = S.width; st->width1 = S.width1;
  return rc;
}

void oracle_lbfgs_diag(const or_lbfgs *s, double *o) {
  o[0] = s->iter; o[1] = s->nfun; o[2] = s->stp; o[3] = s->gnorm;
  o[4] = s->ys; o[5] = s->yy; o[6] = s->dginit; o[7] = s->dg;
}

}  // extern "C"
