// batch.cuh - multi-shot step kernels of libswave.
//
// Many shots of different window size and record length advance together:
// every launch covers all shots of a batch, and everything that changes
// from one time step to the next (time index, rotating time levels,
// snapshot slot, imaging index) is derived inside the kernels from a step
// counter held in device memory.  All launches of a step are therefore
// identical, which lets the time loop be captured once as a CUDA graph and
// replayed.
#pragma once

#include "swave_dev.cuh"

namespace swave {

// Per-shot state of one propagation phase (device resident).
struct ShotDev {
  Geom g;
  Coefs c;
  float *f[5];            // five time levels, rotated by the step counter
  const float *vel;       // padded velocity
  float *v2u;             // 3D adjoint: v^2*u2 scratch (else null)
  const float *gz, *gx, *gy;
  // injection
  int inj_on;
  int bi0, bi1, bj0, bj1, bk0, bk1;
  const int *inj_off;
  const InjEntry *inj_ent;
  const float *src_tr;    // nsrc*nt
  // extraction
  int ext_mode, nrec, ext_half;
  const int *ric;
  const float *wz, *wx;
  float vconst;
  float *rec_tr;          // nrec*nt
  // time axis of this phase
  int tmin, tstep, nsteps, nt, snapi, ntsnap;
  int extract_wave, imaging, adj2d, adj3d;
  float *wave;            // ntsnap*nz*nx*ny snapshots
  float *image, *illum;
  const float *ref;
  const float *taperx, *tapery;
  float k12, div11, dt2snap;
  long long npts;         // compute-domain points
};

// Prefix tables of a batch (device resident).
struct BatchTables {
  int nshots;
  const ShotDev *shots;
  const int *step_tiles;  // nshots+1: fused-step tiles
  const int *rec_start;   // nshots+1: receivers
  const int *hz_start;    // nshots+1: z-edge lines (n2*n3)
  const int *hx_start;    // nshots+1: x-edge lines (n1*n3)
  const int *hy_start;    // nshots+1: y-edge lines (n1*n2, 3D)
  const int *v2u_blocks;  // nshots+1: blocks of the v^2*u2 pass
  int *counter;           // step counter s (0-based)
};

// Launches one full time step of the batch (extract, [v2u], fused step,
// Higdon z/x/[y]) for step s = *counter + s_off.
// ev_before / ev_after (may be null) bracket the fused step kernel.
cudaError_t launch_batch_step(const BatchTables &t, int s_off, int n_step_tiles, int n_rec,
                              int n_hz, int n_hx, int n_hy, int n_v2u, int has_ext, int has_3d,
                              int has_adj3d, cudaStream_t s, int *nlaunch,
                              cudaEvent_t ev_before, cudaEvent_t ev_after);
cudaError_t launch_counter_add(int *counter, int add, cudaStream_t s);

}  // namespace swave
