// swave_dev.cuh - device-side layout and kernel interfaces of libswave.
//
// Wavefields live in HBM in the reference's padded Fortran layout
// u(nmin1-4:nmax1+4, nmin2-4:nmax2+4, nmin3-nbound:nmax3+nbound), z fastest,
// with the z extent rounded up to a multiple of 32 floats so that every
// (x, y) column starts on a 128-byte boundary.
//
// All kernels that reproduce reference arithmetic are compiled with
// --fmad=false and spell out the Fortran evaluation order, so they produce
// the same IEEE-754 results as the CPU restatement.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace swave {

// Padded-grid geometry (FDbounds + padded extents).
struct Geom {
  int nmin1, nmax1, nmin2, nmax2, nmin3, nmax3, nbound;
  int lo1, lo2, lo3;      // lower bounds of the padded array
  int n1p, n2p, n3p;      // padded extents
  int ld1;                // leading dimension (>= n1p, multiple of 32)
  int nz, nx, ny;         // physical window
  int twoD;
  __host__ __device__ inline long long idx(int i, int j, int k) const {
    return (long long)(i - lo1) +
           (long long)ld1 * ((long long)(j - lo2) + (long long)n2p * (long long)(k - lo3));
  }
  __host__ __device__ inline long long plane() const { return (long long)ld1 * n2p; }
  __host__ __device__ inline long long total() const { return plane() * n3p; }
  // physical (1..nz, 1..nx, 1..ny) -> dense nz*nx*ny offset
  __host__ __device__ inline long long pidx(int i, int j, int k) const {
    return (long long)(i - 1) + (long long)nz * ((long long)(j - 1) + (long long)nx * (k - 1));
  }
};

struct Coefs {
  float c0x, c1x, c2x, c3x, c4x, c0y, c1y, c2y, c3y, c4y, c0z, c1z, c2z, c3z, c4z;
};

// One injection contribution: u3 += (((v2r*trace[tr][it])*wz)*wx)*wy.
// Unused weights are 1.0f, which leaves the product unchanged.
struct InjEntry {
  int tr;
  float v2r, wz, wx, wy;
};

// Launchers (kernels.cu).
cudaError_t launch_pad_velocity(const Geom &g, const float *vel_phys, float *vel_pad,
                                cudaStream_t s);
cudaError_t launch_higdon_coeffs(const Geom &g, const float *vel_pad, float dt, float dxi,
                                 float dyi, float dzi, float *gz, float *gx, float *gy,
                                 cudaStream_t s);
// Band-pass of ntr traces of nt samples (in/out trace-major, D and T work
// arrays of (nt + 2*npad)*ntr floats); clo/chi: nlo/nhi sections of 5
// coefficients (device).
cudaError_t launch_bandpass(int ntr, int nt, int npad, int phase, int nlo, const float *clo,
                            int nhi, const float *chi, const float *lead, const float *trail,
                            const float *in, float *out, float *D, float *T, cudaStream_t s);
// delp = 1/rho2 from the padded rho (Interpolate.f90:44-130); tmp is a
// scratch array of the same size; sinc9 = mksinc(9, 0.5).
cudaError_t launch_rho_delp(const Geom &g, const float *rho_pad, float *delp, float *tmp,
                            const float *sinc9, cudaStream_t s, int *nlaunch);

// FWI helpers (kernels.cu).
cudaError_t launch_window_vel(int nz, int nx, int ny, float ox, float oy, float dx, float dy,
                              int nxw, int nyw, float oxw, float oyw, const float *big,
                              float *small, cudaStream_t s);
cudaError_t launch_copy_image(int nz, int nx, int ny, float ox, float oy, float dx, float dy,
                              int nxw, int nyw, float oxw, float oyw, const float *ims,
                              const float *ils, float *image, float *illum, cudaStream_t s);
cudaError_t launch_residual(int nrec, int nt, const float *dobs, const float *mute,
                            float *dmod, float *resid, double *partial, cudaStream_t s);
// The L1 / Huber / Cauchy / hyperbolic residual (SW_NRM_*); maxabs holds
// nrec floats of scratch.  Launches 2 kernels when a threshold is searched
// for, else 1.
cudaError_t launch_residual_nrm(int ntype, float thresh, int nrec, int nt, const float *dobs,
                                const float *mute, float *dmod, float *resid, double *partial,
                                float *maxabs, cudaStream_t s);

}  // namespace swave
