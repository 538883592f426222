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

#include <cuda.h>

#include "swave_dev.cuh"

namespace swave {

// Per-shot state of one propagation phase (device resident).
struct ShotDev {
  Geom g;
  Coefs c;
  float *f[6];            // time levels, rotated by the step counter: level L of
                          // step s in f[(s + L) % nbuf]
  int nbuf;               // 5, or 6 when two steps run per launch (the second
                          // step's output must not overwrite the first's input)
  const float *vel;       // padded velocity
  float *v2u;             // 3D adjoint: v^2*u2 scratch (else null)
  const float *gz, *gx, *gy;
  // injection
  int inj_on;
  int bi0, bi1, bj0, bj1, bk0, bk1;
  const int *inj_off;
  const InjEntry *inj_ent;
  float *inj_term;        // per entry: its contribution at the current step
                          // (two-step launches: a second block of inj_nterm
                          // entries for the step after it)
  int inj_nterm;
  int inj_pre;            // the terms of this step are in inj_term (k_bterms ran)
  const float *src_tr;    // nsrc*nt
  // extraction
  int ext_mode, nrec, ext_half;
  const int *ric;
  const float *wz, *wx;
  float vconst;
  float *rec_tr;          // nrec*nt
  // time axis of this phase
  int tmin, tstep, nsteps, nt, snapi, ntsnap;
  int tcnt;               // first time sample of the whole phase (snapshot counting)
  int t3_ty;              // planes per work unit of the pipelined 3D kernel
  int extract_wave, imaging, adj2d, adj3d;
  float *wave;            // ntsnap*nz*nx*ny snapshots
  float *image, *illum;
  float *image2;          // SW_IMG_AFWI_RHO: the density gradient
  const float *ref;
  const float *taperx, *tapery;
  float k12, div11, dt2snap;
  long long npts;         // compute-domain points
  // Variable density (withRho): padded rho, delp = 1/rho2 and the staggered
  // gradient arrays (sy in 3D), with the rho-operator coefficients.
  int rho_on;
  const float *rho, *delp;
  float *sz, *sx, *sy;
  Coefs cr;
  float dzi, dxi, dyi;
  // Mirror receivers (rec_type > 0) and the free surface (surf_type > 0):
  // the surface row ielev, its grid (1) or sinc (0) mirror with the weights
  // fs_sinc, and irow0, the first row kept in snapshots and images.
  int ext_mirror, surf, ielev, fs_grid, irow0;
  float fs_sinc[15];
};

// Compact per-shot view used by the pipelined 2D kernel; the kernel keeps the
// whole array in shared memory.
struct T2Shot {
  const float *f[5];      // (the two-step kernel reads all six levels and their
                          // count from the ShotDev)
  const float *vel;
  const float *gz, *gx;   // Higdon coefficients (z and x edges)
  float c0z, c1z, c2z, c3z, c4z, c0x, c1x, c2x, c3x, c4x, k12, div11;
  int ld1, lo2, n2p, nmin1, nmax1, nmin2, nmax2, nz, nx;
  int nsteps, tmin, tstep, snapi, adj2d, inj_on, bi0, bi1, bj0, bj1, extract_wave, imaging;
  int tcnt;
  unsigned char inj_direct;  // 1: form injection terms in the tile (few entries)
  unsigned char rigid;       // 1: no Higdon edges (exact-adjoint mode)
  unsigned char surf;        // 1: free surface (no Higdon top edge, side lines from row 1)
  unsigned char pad_;
  int irow0;              // first row kept in snapshots and images (row 1, or the
                          // surface row under a free surface)
  int off1, off2;         // tile origin: nmin1 - off1, nmin2 - off2
  int ntz, ntx;           // tiles along z and x
};

// Tile origin of the pipelined 2D kernel.  Tiles of 64 rows x 32 columns
// start off1 rows before nmin1 and off2 columns before nmin2, chosen so that
// the first and last tile along each axis own at least 6 rows (columns) of
// the compute domain and stage the 4 padding cells beyond it: then every
// Higdon edge line lies inside one tile and the tile can apply it.  off1 is
// a multiple of 4 (tensor-copy row coordinates must be 16-byte aligned).
// Returns false when the domain is too small (n1 or n2 below 16).
inline bool t2_origin(int n1, int n2, int *off1, int *off2, int *ntz, int *ntx) {
  if (n1 < 16 || n2 < 16) return false;
  int a = -1, b = -1;
  for (int o = 4; o <= 56 && a < 0; o += 4) {
    const int nt = (n1 + o + 63) / 64, r = n1 + o - 64 * (nt - 1);
    if (r >= 6 && r <= 60) a = o;
  }
  for (int o = 4; o <= 26 && b < 0; ++o) {
    const int nt = (n2 + o + 31) / 32, r = n2 + o - 32 * (nt - 1);
    if (r >= 6 && r <= 28) b = o;
  }
  if (a < 0 || b < 0) return false;
  *off1 = a;
  *off2 = b;
  *ntz = (n1 + a + 63) / 64;
  *ntx = (n2 + b + 31) / 32;
  return true;
}

// Largest batch the pipelined 2D kernel accepts (its shot table is shared).
constexpr int T2_MAX_SHOTS = 64;
// Largest batch of the two-step 2D kernel (tile2d2.cuh).
constexpr int TF_MAX_SHOTS = 32;

// Tensor maps of one shot for the pipelined 2D kernel: [2*buf + box] with
// buf 0..4 the time-level buffers and 5 the padded velocity, box 0 the
// 72 x 40 halo tile and 1 the 64 x 32 core tile.
struct T2Maps {
  CUtensorMap m[12];
};

// Tensor maps of one shot for the two-step 2D kernel (tile2d2.cuh):
// [2*buf + box] for the six time-level buffers, box 0 the 80 x 80 tile with
// an 8-cell halo, box 1 the 72 x 72 tile with a 4-cell halo; [12] the
// velocity's 72 x 72 box, [13] its 80 x 80 box.
struct T2FMaps {
  CUtensorMap m[14];
};

// Tile origin of the two-step 2D kernel: 64 x 64 tiles starting off1 rows /
// off2 columns before the compute domain (off1 a multiple of 4).  The first
// and last tile along each axis own 8..60 rows (columns) of the compute
// domain, so that each holds its 8-cell Higdon edge zone and the 4 padding
// cells beyond in its core, and no other tile's 4-cell extended region
// reaches an edge zone.  A single tile along an axis holds both.
inline bool tf_origin_axis(int n, bool aligned, int *off, int *nt) {
  for (int o = 4; o <= 56; o += aligned ? 4 : 1) {
    const int k = (n + o + 4 + 63) / 64;
    if (k == 1) {
      *off = o;
      *nt = 1;
      return true;
    }
    const int first = 64 - o, last = n - (64 * (k - 1) - o);
    if (first >= 8 && last >= 8 && last <= 60) {
      *off = o;
      *nt = k;
      return true;
    }
  }
  return false;
}
inline bool tf_origin(int n1, int n2, int *off1, int *off2, int *ntz, int *ntx) {
  if (n1 < 16 || n2 < 16) return false;
  return tf_origin_axis(n1, true, off1, ntz) && tf_origin_axis(n2, false, off2, ntx);
}

// Tensor maps of one shot for the pipelined 3D kernel (rank 3, one plane per
// box): [2*buf + box], box 0 the 40 x 40 plane tile with halo, 1 the
// 32 x 32 core tile.
struct T3Maps {
  CUtensorMap m[12];
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
  const T2Shot *t2shots;  // nshots compact views (pipelined 2D kernel)
  const int *tile_tab;    // pipelined 2D kernel: (shot << 24) | (tzi << 12) | txi per tile
  const int *edge_start;  // nshots+1: threads of the fused 2D edge kernel
  const int *term_start;  // nshots+1: injection entries (per-step term kernel)
  const int *snap_blocks; // nshots+1: blocks of the 3D snapshot / imaging kernel
  const T2Maps *t2maps;   // nshots tensor-map sets (pipelined 2D kernel)
  const T2FMaps *tfmaps;  // nshots tensor-map sets (two-step 2D kernel)
  const T3Maps *t3maps;   // nshots tensor-map sets (pipelined 3D kernel)
  int *err;               // device error flags (bit 0: a bounded wait gave up)
  int *counter;           // step counter s (0-based)
};

// Launches one full time step of the batch (extract, [v2u], fused step,
// Higdon z/x/[y]) for step s = *counter + s_off.
// Tile shape of the fused step kernel.  2D: stream2d = 1 selects the
// streaming kernel with TZ = tz rows per CTA (32, 64 or 128) walking tx
// columns; otherwise 32x8 point tiles.  3D: 32x8 point tiles per plane.
struct StepTile {
  int stream2d = 2;    // 2D: 0 point tiles, 1 streaming (stream2d.cuh), 2 tiled, 3 tiled and
                       // warp-specialised (tile2d.cuh), 4 two steps per launch where the
                       // batch allows it (tile2d2.cuh), else 2
  int tz = 64;
  int tx = 64;
  int stream3d = 2;    // 3D: 1 2.5D streaming kernel (stream3d.cuh), 2 TMA-pipelined (tile3d.cuh)
  int ty = 32;         // 3D: y planes marched per CTA
  int has_fwd2d = 1;   // set by the runner from the batch's stencil variants
  int has_adj2d = 1;
  int has_fwd3d = 1;
  int has_adj3d = 1;
  int nsm = 152;       // SMs of the device (persistent grids)
  int fused_edges = 0; // 2D: one launch for the z and x Higdon edges (set by the runner)
  int n_edge = 0;      // threads of that launch
  int n_snap3d = 0;    // blocks of k_bsnap3d (pipelined 3D kernel with snapshots / imaging)
  int rigid = 0;       // skip the Higdon boundary (exact-adjoint mode)
  int has_rho = 0;     // some shot runs the variable-density operator
  int rho2d = 0;       // every shot is 2D with a density: the one-pass k_brho2d
  int has_surf = 0;    // some shot has a free surface (point tiles, k_bfree)
  int fuse2 = 0;       // 2D tiles: two time steps per launch (tile2d2.cuh)
};

// Threads of the fused 2D edge kernel for one shot: four corner warps and
// one thread per remaining half line, rounded to whole warps.  0 when the
// compute domain is too small for the corner scheme (n1 or n2 below 16).
inline int edge_threads_2d(const Geom &g) {
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
  if (n1 < 16 || n2 < 16) return 0;
  return 128 + (2 * (n2 - 12) + 2 * (n1 - 8) + 31) / 32 * 32;
}

// Number of fused-step CTAs a shot needs with this tile shape.
inline int step_ctas(const Geom &g, const StepTile &tile) {
  const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  if (g.twoD && tile.rho2d) return ((n1 + 63) / 64) * ((n2 + 31) / 32);
  if (g.twoD && tile.fuse2) {
    int o1, o2, nz, nx;
    return tf_origin(n1, n2, &o1, &o2, &nz, &nx) ? nz * nx : 0;
  }
  if (g.twoD && (tile.stream2d == 2 || tile.stream2d == 3)) {
    int o1, o2, nz, nx;
    return t2_origin(n1, n2, &o1, &o2, &nz, &nx) ? nz * nx : 0;
  }
  if (g.twoD && tile.stream2d) return ((n1 + tile.tz - 1) / tile.tz) * ((n2 + tile.tx - 1) / tile.tx);
  if (!g.twoD && tile.stream3d == 2)
    return ((n1 + 31) / 32) * ((n2 + 31) / 32) * ((n3 + tile.ty - 1) / tile.ty);
  if (!g.twoD && tile.stream3d)
    return ((n1 + 31) / 32) * ((n2 + 15) / 16) * ((n3 + tile.ty - 1) / tile.ty);
  return ((n1 + 31) / 32) * ((n2 + 7) / 8) * n3;
}

// ev_before / ev_after (may be null) bracket the fused step kernel.
cudaError_t launch_batch_step(const BatchTables &t, int s_off, int n_step_tiles, int n_rec,
                              int n_hz, int n_hx, int n_hy, int n_v2u, int has_ext, int has_3d,
                              int has_adj3d, const StepTile &tile, cudaStream_t s,
                              int *nlaunch, cudaEvent_t ev_before, cudaEvent_t ev_after,
                              int n_term = 0);
// Two steps per launch (StepTile::fuse2): steps s = *counter + s_off and s + 1.
cudaError_t launch_batch_step2(const BatchTables &t, int s_off, int n_step_tiles, int n_rec,
                               int has_ext, const StepTile &tile, cudaStream_t s, int *nlaunch,
                               cudaEvent_t ev_before, cudaEvent_t ev_after, int n_term);
cudaError_t launch_counter_add(int *counter, int add, cudaStream_t s);

}  // namespace swave
