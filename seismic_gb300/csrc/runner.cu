// runner.cu - runs one propagation phase for a batch of shots.
//
// Every shot of the batch gets its own five time levels, Higdon
// coefficients, injection and extraction plans; the device descriptor
// array (ShotDev) and prefix tables let one launch of each kernel cover the
// whole batch.  The time loop is a CUDA graph of `chunk` steps captured
// once and replayed; the step counter lives in device memory.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "batch.cuh"
#include "engine.h"

namespace swave {

// cuTensorMapEncodeTiled from the driver, looked up once.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

namespace {

// 2D FP32 tensor map over a padded field (ld1 rows x n2p columns) with a
// box of bz rows x bx columns; out-of-range elements read as zero.
bool encode_field_map(CUtensorMap *m, const float *base, const Geom &g, int bz, int bx) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)g.ld1, (cuuint64_t)g.n2p};
  const cuuint64_t strides[1] = {(cuuint64_t)g.ld1 * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)bz, (cuuint32_t)bx};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <class T>
T *carve(char *&cur, size_t n) {
  T *p = reinterpret_cast<T *>(cur);
  cur += (n * sizeof(T) + 255) / 256 * 256;
  return p;
}

size_t rup(size_t b) { return (b + 255) / 256 * 256; }

// Injection entries from which a shot's terms are formed by k_bterms.
constexpr size_t kTermKernelMin = 2048;

// 3D FP32 tensor map over a padded field (ld1 x n2p x n3p) with a box of
// bz rows x bx columns x 1 plane.
bool encode_field_map3(CUtensorMap *m, const float *base, const Geom &g, int bz, int bx) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)g.ld1, (cuuint64_t)g.n2p, (cuuint64_t)g.n3p};
  const cuuint64_t strides[2] = {(cuuint64_t)g.ld1 * sizeof(float),
                                 (cuuint64_t)g.ld1 * g.n2p * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)bx, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int run_phases(sw_ctx *c, std::vector<PhaseShot> &shots, const RunOpts &opt) {
  const int nb = (int)shots.size();
  if (nb == 0) return SW_OK;
  cudaStream_t s = c->stream;
  cudaError_t e;
  int st = SW_OK;
  std::vector<Geom> G(nb);
  std::vector<InjPlan> inj(nb);
  std::vector<ExtPlan> ext(nb);
  std::vector<std::vector<float>> tx(nb), ty(nb);
  bool has_3d = false, has_adj3d = false, has_ext = false;
  // The pipelined 2D kernel keeps the batch's shot table in shared memory
  // and packs tile coordinates into 12 bits each; larger batches, grids
  // beyond that or domains below 16 cells use the streaming kernel.
  StepTile tile = opt.tile;
  // The variable-density operator: in 2D one pass per step (k_brho2d) when
  // every shot of the batch has a density, else the point-tile step kernel
  // after a gradient pass (k_brho_grad).  A free surface and mirror sources
  // or receivers run on the single-step 2D tile kernel (k_bfree before it;
  // the mirror terms are injection and extraction entries); in 3D on the
  // point tiles.
  tile.has_rho = 0;
  tile.rho2d = 0;
  tile.has_surf = 0;
  bool special = false, all_rho2d = true;
  for (int b = 0; b < nb; ++b) {
    const sw_genpar &g = shots[b].d.g;
    if (shots[b].io.rho_pad) tile.has_rho = 1;
    // k_brho2d copies 16-byte chunks of v, rho and delp (and of the level
    // buffers, carved at 256-byte boundaries).
    const uintptr_t al = reinterpret_cast<uintptr_t>(shots[b].io.rho_pad) |
                         reinterpret_cast<uintptr_t>(shots[b].io.delp) |
                         reinterpret_cast<uintptr_t>(shots[b].io.vel_pad);
    if (!shots[b].io.rho_pad || !g.twoD || (al & 15) != 0) all_rho2d = false;
    if (g.surf_type != 0) tile.has_surf = 1;
    if (g.surf_type != 0 || g.shot_type != 0 || g.rec_type != 0) special = true;
  }
  if (tile.has_rho) {
    tile.stream2d = 0;
    tile.stream3d = 0;
    tile.rho2d = all_rho2d ? 1 : 0;
  }
  if (special) {
    if (tile.stream2d != 0) tile.stream2d = 2;
    tile.stream3d = 0;
  }
  // Two time steps per launch (tile2d2.cuh) for 2D batches of up to
  // TF_MAX_SHOTS shots whose imaging reads only the staged fields (none,
  // RTM, LSRTM); other batches take the single-step tile kernel.
  tile.fuse2 = 0;
  if (tile.stream2d == 4) {
    bool ok = shots[0].d.g.twoD && nb <= TF_MAX_SHOTS;
    for (int b = 0; b < nb && ok; ++b) {
      const sw_prop_desc &d = shots[b].d;
      const Geom g = make_geom(d.g);
      int o1, o2, ntz, ntx;
      ok = d.g.twoD &&
           (d.imaging == SW_IMG_NONE || d.imaging == SW_IMG_RTM || d.imaging == SW_IMG_LSRTM) &&
           g.nmax1 - g.nmin1 + 1 <= 64 * 4000 && g.nmax2 - g.nmin2 + 1 <= 64 * 4000 &&
           tf_origin(g.nmax1 - g.nmin1 + 1, g.nmax2 - g.nmin2 + 1, &o1, &o2, &ntz, &ntx);
    }
    tile.stream2d = 2;
    tile.fuse2 = ok ? 1 : 0;
  }
  if ((tile.stream2d == 2 || tile.stream2d == 3) && !tile.fuse2) {
    bool fits = nb <= T2_MAX_SHOTS;
    for (int b = 0; b < nb && fits; ++b) {
      const Geom g = make_geom(shots[b].d.g);
      const int n1 = g.nmax1 - g.nmin1 + 1, n2 = g.nmax2 - g.nmin2 + 1;
      int o1, o2, ntz, ntx;
      fits = !g.twoD || (n1 <= 64 * 4000 && n2 <= 32 * 4000 &&
                         t2_origin(n1, n2, &o1, &o2, &ntz, &ntx));
    }
    if (!fits) tile.stream2d = 1;
  }
  const bool t2 = (tile.stream2d == 2 || tile.stream2d == 3) && shots[0].d.g.twoD;
  // The pipelined 3D kernel packs (shot, z tile, x tile, y unit) into 7/8/8/8
  // bits; larger batches or grids use the streaming kernel.
  if (!shots[0].d.g.twoD && tile.stream3d == 2) {
    bool fits = nb < 128 && tile.ty >= 1;
    for (int b = 0; b < nb && fits; ++b) {
      const Geom g = make_geom(shots[b].d.g);
      fits = (g.nmax1 - g.nmin1 + 32) / 32 <= 256 && (g.nmax2 - g.nmin2 + 32) / 32 <= 256 &&
             (g.nmax3 - g.nmin3 + tile.ty) / tile.ty <= 256;
    }
    if (!fits) tile.stream3d = 1;
  }
  const bool t3 = !shots[0].d.g.twoD && tile.stream3d == 2;
  // ---- host-side plans and arena sizes ----
  size_t bytes = 0;
  for (int b = 0; b < nb; ++b) {
    const sw_prop_desc &d = shots[b].d;
    const DevIO &io = shots[b].io;
    if ((st = check_genpar(c, d.g))) return st;
    if (d.tstep != 1 && d.tstep != -1) return fail(c, SW_BAD_PARAM, "tstep must be +-1");
    if (make_geom(d.g).total() >= (1LL << 31))
      return fail(c, SW_BAD_PARAM, "padded grid of shot %d exceeds 2^31 points", b);
    if (b > 0 && (d.g.twoD != shots[0].d.g.twoD))
      return fail(c, SW_BAD_PARAM, "a batch mixes 2D and 3D shots");
    G[b] = make_geom(d.g);
    has_3d = has_3d || !d.g.twoD;
    has_adj3d = has_adj3d || (!d.g.twoD && d.fd_scheme == SW_FD_ADJOINT);
    if (io.rho_pad && d.fd_scheme != SW_FD_FORWARD)
      return fail(c, SW_UNSUPPORTED, "the variable-density operator has no adjoint-grid form");
    // The injected side of a backward propagation (tmax = 1) follows
    // rec_type, a forward one shot_type (Injection.f90:160-164).
    const bool inj_mirror = (d.tmax == 1 ? d.g.rec_type : d.g.shot_type) != 0;
    if ((st = build_injection(c, d.g, G[b], d.injection, io.nsou, io.sou_coord, io.vel_phys_host,
                              inj[b], io.rho_pad ? io.rho_phys_host : nullptr, inj_mirror)))
      return st;
    if ((st = build_extraction(c, d.g, G[b], d.extraction, io.nrec, io.rec_coord, ext[b],
                               d.g.rec_type != 0)))
      return st;
    has_ext = has_ext || ext[b].on;
    if (d.imaging != SW_IMG_NONE) compute_taper(d.g.nx, d.g.ny, tx[b], ty[b]);
    const size_t fb = (size_t)G[b].total() * sizeof(float);
    const long long n1 = G[b].nmax1 - G[b].nmin1 + 1, n2 = G[b].nmax2 - G[b].nmin2 + 1,
                    n3 = G[b].nmax3 - G[b].nmin3 + 1;
    bytes += (tile.fuse2 ? 6 : 5) * rup(fb);
    if (!d.g.twoD && d.fd_scheme == SW_FD_ADJOINT && !tile.stream3d) bytes += rup(fb);
    // The staggered gradient arrays of the two-pass density operator.
    if (io.rho_pad && !tile.rho2d) bytes += (d.g.twoD ? 2 : 3) * rup(fb);
    bytes += rup(16 * n2 * n3 * 4) + rup(16 * n1 * n3 * 4) + rup(16 * n1 * n2 * 4);
    bytes += rup(inj[b].off.size() * 4) + rup(inj[b].ent.size() * sizeof(InjEntry)) +
             rup((tile.fuse2 ? 2 : 1) * inj[b].ent.size() * sizeof(float));
    bytes += rup(ext[b].ic.size() * 4) + 2 * rup(ext[b].wz.size() * 4);
    bytes += 2 * rup(std::max<size_t>(tx[b].size(), ty[b].size()) * 4 + 4);
  }
  bytes += rup(nb * sizeof(ShotDev)) + 9 * rup((nb + 1) * sizeof(int)) + rup(sizeof(int));
  if (t2) {
    size_t ntile = 0;
    for (int b = 0; b < nb; ++b) ntile += (size_t)step_ctas(G[b], tile);
    bytes += rup(nb * sizeof(T2Shot)) + rup(ntile * sizeof(int)) +
             (tile.fuse2 ? rup(nb * sizeof(T2FMaps)) : rup(nb * sizeof(T2Maps)));
  }
  if (t3) {
    size_t ntile = 0;
    for (int b = 0; b < nb; ++b) ntile += (size_t)step_ctas(G[b], tile);
    bytes += rup(ntile * sizeof(int)) + rup(nb * sizeof(T3Maps));
  }
  bytes += rup(sizeof(int));   // error flags
  // A quarter of headroom when the arena grows: batches of slightly larger
  // windows then reuse it instead of reallocating.
  char *arena = (char *)dbuf(c, "batch_arena", bytes, &st, bytes / 4);
  if (!arena) return st;
  char *cur = arena;
  // ---- carve and fill ----
  std::vector<ShotDev> hs(nb);
  std::vector<int> step_tiles(nb + 1, 0), rec_start(nb + 1, 0), hz(nb + 1, 0), hx(nb + 1, 0),
      hy(nb + 1, 0), v2b(nb + 1, 0), edge(nb + 1, 0), term(nb + 1, 0), snapb(nb + 1, 0);
  // The fused 2D edge kernel needs n1, n2 >= 16 in every shot.
  bool fused_edges = !has_3d && !tile.has_surf;
  for (int b = 0; b < nb && fused_edges; ++b) fused_edges = edge_threads_2d(G[b]) > 0;
  int max_steps = 0;
  for (int b = 0; b < nb; ++b) {
    const sw_prop_desc &d = shots[b].d;
    const DevIO &io = shots[b].io;
    const sw_genpar &g = d.g;
    ShotDev &S = hs[b];
    std::memset(&S, 0, sizeof(S));
    S.g = G[b];
    S.c = make_coefs(g);
    const size_t nf = (size_t)G[b].total();
    S.nbuf = tile.fuse2 ? 6 : 5;
    for (int q = 0; q < S.nbuf; ++q) {
      S.f[q] = carve<float>(cur, nf);
      // Level L at step 0 is buffer L: a checkpointed phase resumes from the
      // saved u_1, u0, u1, u2; u3 (and every level otherwise) starts at 0.
      if (io.init_state && q < 4)
        e = cudaMemcpyAsync(S.f[q], io.init_state + (size_t)q * nf, nf * sizeof(float),
                            cudaMemcpyDeviceToDevice, s);
      else
        e = cudaMemsetAsync(S.f[q], 0, nf * sizeof(float), s);
      if (e != cudaSuccess) return cuda_fail(c, e, "initial fields");
    }
    S.adj2d = g.twoD && d.fd_scheme == SW_FD_ADJOINT;
    S.adj3d = !g.twoD && d.fd_scheme == SW_FD_ADJOINT;
    if (S.adj3d && !tile.stream3d) {
      S.v2u = carve<float>(cur, nf);
      SW_CK(cudaMemsetAsync(S.v2u, 0, nf * sizeof(float), s));
    }
    S.vel = io.vel_pad;
    if (io.rho_pad) {
      if (!io.delp || !io.rho_phys_host) return fail(c, SW_BAD_PARAM, "density arrays missing");
      S.rho_on = 1;
      S.rho = io.rho_pad;
      S.delp = io.delp;
      S.cr = make_rho_coefs(g);
      S.dzi = 1.f / g.dz;
      S.dxi = 1.f / g.dx;
      S.dyi = 1.f / g.dy;
      // k_brho2d forms sz and sx in shared memory; the two-pass operator
      // (k_brho_grad, then the point tiles) keeps them in HBM.
      if (!tile.rho2d) {
        S.sz = carve<float>(cur, nf);
        S.sx = carve<float>(cur, nf);
        SW_CK(cudaMemsetAsync(S.sz, 0, nf * sizeof(float), s));
        SW_CK(cudaMemsetAsync(S.sx, 0, nf * sizeof(float), s));
        if (!g.twoD) {
          S.sy = carve<float>(cur, nf);
          SW_CK(cudaMemsetAsync(S.sy, 0, nf * sizeof(float), s));
        }
      }
    }
    const long long n1 = G[b].nmax1 - G[b].nmin1 + 1, n2 = G[b].nmax2 - G[b].nmin2 + 1,
                    n3 = G[b].nmax3 - G[b].nmin3 + 1;
    float *gz = carve<float>(cur, 16 * n2 * n3), *gx = carve<float>(cur, 16 * n1 * n3),
          *gy = carve<float>(cur, 16 * n1 * n2);
    if ((e = launch_higdon_coeffs(G[b], io.vel_pad, g.dt, 1.f / g.dx, 1.f / g.dy, 1.f / g.dz, gz,
                                  gx, gy, s)) != cudaSuccess)
      return cuda_fail(c, e, "higdon coeffs");
    c->stats.launches_total++;
    S.gz = gz; S.gx = gx; S.gy = gy;
    S.inj_on = inj[b].on;
    if (inj[b].on) {
      S.bi0 = inj[b].bi0; S.bi1 = inj[b].bi1; S.bj0 = inj[b].bj0; S.bj1 = inj[b].bj1;
      S.bk0 = inj[b].bk0; S.bk1 = inj[b].bk1;
      int *off = carve<int>(cur, inj[b].off.size());
      InjEntry *ent = carve<InjEntry>(cur, inj[b].ent.size());
      SW_CK(cudaMemcpyAsync(off, inj[b].off.data(), inj[b].off.size() * 4, cudaMemcpyHostToDevice, s));
      SW_CK(cudaMemcpyAsync(ent, inj[b].ent.data(), inj[b].ent.size() * sizeof(InjEntry),
                      cudaMemcpyHostToDevice, s));
      S.inj_off = off;
      S.inj_ent = ent;
      S.inj_nterm = (int)inj[b].ent.size();
      S.inj_term = carve<float>(cur, (tile.fuse2 ? 2 : 1) * inj[b].ent.size());
      S.src_tr = io.sou_trace_dev;
    }
    S.ext_mode = ext[b].on ? ext[b].mode : 0;
    S.ext_mirror = ext[b].on ? ext[b].mirror : 0;
    S.irow0 = 1;
    if (g.surf_type != 0) {
      // Flat surface at elevation 0 (the drivers' elev%elev = 0): find_i_d
      // (ModelSpaceTypes.f90:144-151) gives its row and offset.
      S.surf = 1;
      S.ielev = (int)lroundf((0.f - g.oz) / g.dz) + 1;
      const float delev = 0.f - (g.oz + (float)(S.ielev - 1) * g.dz);
      S.fs_grid = delev == 0.f;
      if (!S.fs_grid) mksinc(S.fs_sinc, g.lsinc, delev / g.dz);
      S.irow0 = std::max(S.ielev, 1);
      const int h = g.lsinc / 2;
      if (S.ielev - 2 * h - 1 < G[b].lo1 || S.ielev + 2 * h > G[b].nmax1 + 4)
        return fail(c, SW_BAD_PARAM, "free surface row %d leaves the padded grid", S.ielev);
    }
    S.nrec = ext[b].on ? ext[b].nrec : 0;
    S.ext_half = g.lsinc / 2;
    if (ext[b].on) {
      int *ric = carve<int>(cur, ext[b].ic.size());
      float *wz = carve<float>(cur, ext[b].wz.size()), *wx = carve<float>(cur, ext[b].wx.size());
      SW_CK(cudaMemcpyAsync(ric, ext[b].ic.data(), ext[b].ic.size() * 4, cudaMemcpyHostToDevice, s));
      SW_CK(cudaMemcpyAsync(wz, ext[b].wz.data(), ext[b].wz.size() * 4, cudaMemcpyHostToDevice, s));
      SW_CK(cudaMemcpyAsync(wx, ext[b].wx.data(), ext[b].wx.size() * 4, cudaMemcpyHostToDevice, s));
      S.ric = ric; S.wz = wz; S.wx = wx;
      S.rec_tr = io.rec_trace_dev;
      S.vconst = 1.f;
      if (d.extraction == SW_EXT_LSRTM_SINC)
        S.vconst = g.twoD ? 1.f / (g.dz * g.dx) : 1.f / ((g.dz * g.dx) * g.dy);
    }
    S.tmin = d.tmin;
    S.tcnt = io.tcnt ? io.tcnt : d.tmin;
    S.t3_ty = tile.ty;

    S.tstep = d.tstep;
    S.nsteps = (d.tmax - d.tmin + d.tstep) / d.tstep;
    S.nt = g.nt;
    S.snapi = g.snapi;
    S.ntsnap = g.nt / g.snapi;
    S.extract_wave = d.extract_wave;
    S.imaging = d.imaging;
    S.wave = io.wave_dev;
    S.image = io.image_dev;
    S.illum = io.illum_dev;
    S.image2 = io.image2_dev;
    S.ref = io.ref_dev;
    if (d.imaging != SW_IMG_NONE) {
      float *a = carve<float>(cur, tx[b].size() + 1), *bq = carve<float>(cur, ty[b].size() + 1);
      SW_CK(cudaMemcpyAsync(a, tx[b].data(), tx[b].size() * 4, cudaMemcpyHostToDevice, s));
      SW_CK(cudaMemcpyAsync(bq, ty[b].data(), ty[b].size() * 4, cudaMemcpyHostToDevice, s));
      S.taperx = a;
      S.tapery = bq;
    }
    S.k12 = 12.f * (g.dt * g.dt);
    S.div11 = 1.f / 11.f;
    {
      const float xs = g.dt * (float)g.snapi;
      S.dt2snap = xs * xs;  // genpar%dt2 (compute_function_gradient.f90:237)
    }
    S.npts = n1 * n2 * n3;
    if ((S.extract_wave || (S.imaging != SW_IMG_NONE)) && !S.wave)
      return fail(c, SW_BAD_PARAM, "snapshot buffer missing");
    if (S.imaging < SW_IMG_NONE || S.imaging > SW_IMG_AFWI_RHO)
      return fail(c, SW_BAD_PARAM, "imaging %d", S.imaging);
    if (((S.imaging >= 1 && S.imaging <= 3) || S.imaging == SW_IMG_AFWI_RHO) &&
        (!S.image || !S.illum))
      return fail(c, SW_BAD_PARAM, "image buffers missing");
    if (S.imaging == SW_IMG_AFWI_RHO && (!S.image2 || !S.rho_on))
      return fail(c, SW_BAD_PARAM, "SW_IMG_AFWI_RHO needs rho and image2");
    if (S.imaging == SW_IMG_BORN && !S.ref) return fail(c, SW_BAD_PARAM, "reflectivity missing");
    max_steps = std::max(max_steps, S.nsteps);
    step_tiles[b + 1] = step_tiles[b] + step_ctas(G[b], tile);
    rec_start[b + 1] = rec_start[b] + S.nrec;
    hz[b + 1] = hz[b] + (int)(n2 * n3);
    hx[b + 1] = hx[b] + (int)(n1 * n3);
    hy[b + 1] = hy[b] + (g.twoD ? 0 : (int)(n1 * n2));
    edge[b + 1] = edge[b] + (fused_edges ? edge_threads_2d(G[b]) : 0);
    // The pipelined 2D kernel adds injection terms computed per step by
    // k_bterms when a shot has many entries (receiver-side injection);
    // a few source entries are formed in the tile.
    term[b + 1] = term[b] + ((t2 || t3) && inj[b].on && inj[b].ent.size() >= kTermKernelMin
                                 ? (int)inj[b].ent.size() : 0);
    // The pipelined 3D kernel leaves a shot's snapshot saves and imaging to
    // k_bsnap3d (one thread per physical point).
    S.inj_pre = term[b + 1] > term[b];
    snapb[b + 1] = snapb[b] + ((t3 && (S.extract_wave || S.imaging != 0))
                                   ? (int)std::min<long long>(
                                         8192, ((long long)g.nz * g.nx * g.ny + 255) / 256)
                                   : 0);
    v2b[b + 1] = v2b[b] + (((S.adj3d && !tile.stream3d) || S.rho_on)
                               ? (int)std::min<long long>(4096, (G[b].total() + 255) / 256)
                               : 0);
  }
  ShotDev *dshots = carve<ShotDev>(cur, nb);
  int *dtab[9];
  std::vector<int> *htab[9] = {&step_tiles, &rec_start, &hz, &hx, &hy, &v2b, &edge, &term,
                               &snapb};
  for (int q = 0; q < 9; ++q) {
    dtab[q] = carve<int>(cur, nb + 1);
    SW_CK(cudaMemcpyAsync(dtab[q], htab[q]->data(), (nb + 1) * 4, cudaMemcpyHostToDevice, s));
  }
  int *counter = carve<int>(cur, 1);
  SW_CK(cudaMemcpyAsync(dshots, hs.data(), nb * sizeof(ShotDev), cudaMemcpyHostToDevice, s));
  // Compact shot views and the shot-major tile table of the pipelined 2D
  // kernel.
  std::vector<T2Shot> h2(t2 ? nb : 0);
  std::vector<int> htile;
  std::vector<T2Maps> hmaps;
  std::vector<T2FMaps> hfmaps;
  T2Shot *d2 = nullptr;
  int *dtile = nullptr;
  T2Maps *dmaps = nullptr;
  T2FMaps *dfmaps = nullptr;
  if (t2) {
    for (int b = 0; b < nb; ++b) {
      const ShotDev &S = hs[b];
      T2Shot &h = h2[b];
      std::memset(&h, 0, sizeof(h));
      for (int q = 0; q < 5; ++q) h.f[q] = S.f[q];
      h.vel = S.vel;
      h.c0z = S.c.c0z; h.c1z = S.c.c1z; h.c2z = S.c.c2z; h.c3z = S.c.c3z; h.c4z = S.c.c4z;
      h.c0x = S.c.c0x; h.c1x = S.c.c1x; h.c2x = S.c.c2x; h.c3x = S.c.c3x; h.c4x = S.c.c4x;
      h.k12 = S.k12; h.div11 = S.div11;
      h.ld1 = S.g.ld1; h.lo2 = S.g.lo2; h.n2p = S.g.n2p;
      h.nmin1 = S.g.nmin1; h.nmax1 = S.g.nmax1; h.nmin2 = S.g.nmin2; h.nmax2 = S.g.nmax2;
      h.nz = S.g.nz; h.nx = S.g.nx;
      h.nsteps = S.nsteps; h.tmin = S.tmin; h.tstep = S.tstep; h.snapi = S.snapi;
      h.tcnt = S.tcnt;
      h.adj2d = S.adj2d; h.inj_on = S.inj_on;
      h.inj_direct = S.inj_on && inj[b].ent.size() < kTermKernelMin;
      h.rigid = opt.rigid ? 1 : 0;
      h.surf = S.surf ? 1 : 0;
      h.irow0 = S.irow0;
      h.bi0 = S.bi0; h.bi1 = S.bi1; h.bj0 = S.bj0; h.bj1 = S.bj1;
      h.extract_wave = S.extract_wave; h.imaging = S.imaging;
      h.gz = S.gz; h.gx = S.gx;
      const bool org = tile.fuse2 ? tf_origin(S.g.nmax1 - S.g.nmin1 + 1, S.g.nmax2 - S.g.nmin2 + 1,
                                              &h.off1, &h.off2, &h.ntz, &h.ntx)
                                  : t2_origin(S.g.nmax1 - S.g.nmin1 + 1, S.g.nmax2 - S.g.nmin2 + 1,
                                              &h.off1, &h.off2, &h.ntz, &h.ntx);
      if (!org) return fail(c, SW_CUDA_ERR, "tile origin");
      const int n1t = h.ntz, n2t = h.ntx;
      for (int xi = 0; xi < n2t; ++xi)
        for (int zi = 0; zi < n1t; ++zi) htile.push_back((b << 24) | (zi << 12) | xi);
    }
    if ((int)htile.size() != step_tiles[nb]) return fail(c, SW_CUDA_ERR, "tile table size");
    if (tile.fuse2) {
      // Six level buffers with the 80 x 80 and 72 x 72 boxes, then the
      // velocity's 72 x 72 and 80 x 80 boxes.
      hfmaps.resize(nb);
      for (int b = 0; b < nb; ++b) {
        const ShotDev &S = hs[b];
        bool ok = true;
        for (int q = 0; q < 6 && ok; ++q)
          ok = encode_field_map(&hfmaps[b].m[2 * q], S.f[q], S.g, 80, 80) &&
               encode_field_map(&hfmaps[b].m[2 * q + 1], S.f[q], S.g, 72, 72);
        ok = ok && encode_field_map(&hfmaps[b].m[12], S.vel, S.g, 72, 72) &&
             encode_field_map(&hfmaps[b].m[13], S.vel, S.g, 80, 80);
        if (!ok) return fail(c, SW_CUDA_ERR, "tensor map encoding failed (shot %d)", b);
      }
    } else {
      hmaps.resize(nb);
      for (int b = 0; b < nb; ++b) {
        const ShotDev &S = hs[b];
        for (int q = 0; q < 6; ++q) {
          const float *base = q < 5 ? S.f[q] : S.vel;
          if (!encode_field_map(&hmaps[b].m[2 * q], base, S.g, 72, 40) ||
              !encode_field_map(&hmaps[b].m[2 * q + 1], base, S.g, 64, 32))
            return fail(c, SW_CUDA_ERR, "tensor map encoding failed (shot %d)", b);
        }
      }
    }
    d2 = carve<T2Shot>(cur, nb);
    dtile = carve<int>(cur, htile.size());
    if (tile.fuse2) {
      dfmaps = carve<T2FMaps>(cur, nb);
      SW_CK(cudaMemcpyAsync(dfmaps, hfmaps.data(), nb * sizeof(T2FMaps), cudaMemcpyHostToDevice,
                            s));
    } else {
      dmaps = carve<T2Maps>(cur, nb);
      SW_CK(cudaMemcpyAsync(dmaps, hmaps.data(), nb * sizeof(T2Maps), cudaMemcpyHostToDevice, s));
    }
    SW_CK(cudaMemcpyAsync(d2, h2.data(), nb * sizeof(T2Shot), cudaMemcpyHostToDevice, s));
    SW_CK(cudaMemcpyAsync(dtile, htile.data(), htile.size() * sizeof(int), cudaMemcpyHostToDevice,
                          s));
  }
  std::vector<T3Maps> hmaps3;
  T3Maps *dmaps3 = nullptr;
  if (t3) {
    // Units that meet a shot's injection box (the receiver layer of a
    // backward pass: several times the work of the others) come first, so
    // that the round-robin assignment gives every CTA at most its share of
    // them; the rest follow in the same z-fastest order.
    std::vector<int> light;
    for (int b = 0; b < nb; ++b) {
      const Geom &g = G[b];
      const int n1t = (g.nmax1 - g.nmin1 + 32) / 32, n2t = (g.nmax2 - g.nmin2 + 32) / 32;
      const int n3t = (g.nmax3 - g.nmin3 + tile.ty) / tile.ty;
      const InjPlan &P = inj[b];
      for (int ky = 0; ky < n3t; ++ky)
        for (int xi = 0; xi < n2t; ++xi)
          for (int zi = 0; zi < n1t; ++zi) {
            const int e = (b << 24) | (zi << 16) | (xi << 8) | ky;
            const int z0 = g.nmin1 + 32 * zi, x0 = g.nmin2 + 32 * xi, y0 = g.nmin3 + ky * tile.ty;
            const bool heavy = P.on && z0 <= P.bi1 && z0 + 31 >= P.bi0 && x0 <= P.bj1 &&
                               x0 + 31 >= P.bj0 && y0 <= P.bk1 && y0 + tile.ty - 1 >= P.bk0;
            (heavy ? htile : light).push_back(e);
          }
    }
    htile.insert(htile.end(), light.begin(), light.end());
    if ((int)htile.size() != step_tiles[nb]) return fail(c, SW_CUDA_ERR, "unit table size");
    hmaps3.resize(nb);
    for (int b = 0; b < nb; ++b) {
      const ShotDev &S = hs[b];
      for (int q = 0; q < 6; ++q) {
        const float *base = q < 5 ? S.f[q] : S.vel;
        if (!encode_field_map3(&hmaps3[b].m[2 * q], base, S.g, 40, 40) ||
            !encode_field_map3(&hmaps3[b].m[2 * q + 1], base, S.g, 32, 32))
          return fail(c, SW_CUDA_ERR, "tensor map encoding failed (shot %d)", b);
      }
    }
    dtile = carve<int>(cur, htile.size());
    dmaps3 = carve<T3Maps>(cur, nb);
    SW_CK(cudaMemcpyAsync(dmaps3, hmaps3.data(), nb * sizeof(T3Maps), cudaMemcpyHostToDevice, s));
    SW_CK(cudaMemcpyAsync(dtile, htile.data(), htile.size() * sizeof(int), cudaMemcpyHostToDevice,
                          s));
  }
  SW_CK(cudaMemsetAsync(counter, 0, sizeof(int), s));
  // A queued (asynchronous) phase records its errors in the context's
  // run_err flag, which outlives it; a synchronous one in the arena.
  bool async = opt.async_end && !c->profiling;
  for (int b = 0; b < nb && async; ++b)
    if (shots[b].io.final_u2_host || shots[b].io.save_state) async = false;
  int *derr = carve<int>(cur, 1);
  if (async) {
    derr = (int *)dbuf(c, "run_err", sizeof(int), &st);
    if (!derr) return st;
  } else {
    SW_CK(cudaMemsetAsync(derr, 0, sizeof(int), s));
  }
  if ((size_t)(cur - arena) > bytes) return fail(c, SW_CUDA_ERR, "arena overflow");
  BatchTables t;
  t.nshots = nb;
  t.shots = dshots;
  t.step_tiles = dtab[0];
  t.rec_start = dtab[1];
  t.hz_start = dtab[2];
  t.hx_start = dtab[3];
  t.hy_start = dtab[4];
  t.v2u_blocks = dtab[5];
  t.edge_start = dtab[6];
  t.term_start = dtab[7];
  t.snap_blocks = dtab[8];
  t.t2shots = d2;
  t.tile_tab = dtile;
  t.t2maps = dmaps;
  t.tfmaps = dfmaps;
  t.t3maps = dmaps3;
  t.err = derr;
  t.counter = counter;
  // The host plans above must stay alive until the uploads complete.  Copies
  // from pageable memory are staged before cudaMemcpyAsync returns, so a
  // queued phase need not wait here (the previous phase keeps running).
  if (!async && (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_fail(c, e, "batch setup");

  const int n_term = term[nb];
  const int n_tiles = step_tiles[nb], n_rec = rec_start[nb], n_hz = hz[nb], n_hx = hx[nb],
            n_hy = hy[nb], n_v2u = v2b[nb];
  tile.n_snap3d = snapb[nb];
  {
    int dev = 0, nsm = 0;
    SW_CK(cudaGetDevice(&dev));
    SW_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    tile.nsm = nsm;
  }
  tile.has_fwd2d = tile.has_adj2d = tile.has_fwd3d = tile.has_adj3d = 0;
  tile.fused_edges = fused_edges ? 1 : 0;
  tile.rigid = opt.rigid ? 1 : 0;
  tile.n_edge = edge[nb];

  for (auto &S : hs) {
    if (S.g.twoD) {
      if (S.adj2d) tile.has_adj2d = 1;
      else tile.has_fwd2d = 1;
    } else {
      if (S.adj3d) tile.has_adj3d = 1;
      else tile.has_fwd3d = 1;
    }
  }
  long long npts_total = 0;
  for (auto &S : hs) npts_total += S.npts;
  // ---- time loop ----
  // Two-step launches cover steps q and q + 1 of a chunk: chunks of an even
  // number of steps (steps past a shot's last one are skipped by the kernels).
  const int stride = tile.fuse2 ? 2 : 1;
  int chunk = std::max(1, std::min(opt.chunk, max_steps));
  if (chunk % stride) chunk += stride - chunk % stride;
  const int nchunks = (max_steps + chunk - 1) / chunk;
  const bool prof = c->profiling;
  // Algorithmic bytes of the fused step kernel at step sidx: 24 B per point
  // update (u2, u1, u0, u_1, vel read, u3 written) plus, on a shot's
  // snapshot steps, per physical point 4 B for a saved snapshot and the
  // imaging traffic (RTM/LSRTM: snapshot read + image and illumination
  // read-modify-write = 20 B; AFWI: two more snapshot reads = 28 B; Born
  // source: snapshot + reflectivity = 8 B).
  auto step_bytes_at = [&](int sidx) -> uint64_t {
    uint64_t by = 0;
    for (auto &S : hs) {
      if (sidx >= S.nsteps) continue;
      // 24 B per point (u2, u1, u0, u_1, v read, u3 written); with a density
      // also rho and delp read (one pass, k_brho2d), or on the point tiles
      // the gradient arrays instead of delp (sz, sx and in 3D sy).
      uint64_t per_pt = 24;
      if (S.rho_on) per_pt = tile.rho2d ? 32 : (S.g.twoD ? 36 : 40);
      by += (uint64_t)S.npts * per_pt;
      if (t3) continue;   // snapshots and imaging: k_bsnap3d
      const int it = S.tmin + sidx * S.tstep;
      if (it % S.snapi != 0) continue;
      const int cnt = S.tstep > 0 ? it / S.snapi - (S.tcnt - 1) / S.snapi
                                  : S.tcnt / S.snapi - (it - 1) / S.snapi;
      const bool slot = S.tstep > 0 ? cnt <= S.ntsnap : S.ntsnap - cnt + 1 >= 1;
      if (!slot) continue;
      uint64_t per = S.extract_wave ? 4 : 0;
      if (S.imaging == SW_IMG_RTM || S.imaging == SW_IMG_LSRTM) per += 20;
      if (S.imaging == SW_IMG_AFWI) per += 28;
      if (S.imaging == SW_IMG_AFWI_RHO) per += 36;
      if (S.imaging == SW_IMG_BORN) per += 8;
      by += (uint64_t)S.g.nz * S.g.nx * S.g.ny * per;
    }
    return by;
  };
  // Two-step launch at steps sidx, sidx + 1: 28 B per point that takes both
  // steps (u2, u1, u0, u_1, vel read, two levels written), 24 B for one,
  // plus each step's snapshot and imaging traffic.
  auto step_bytes2_at = [&](int sidx) -> uint64_t {
    uint64_t by = step_bytes_at(sidx) + step_bytes_at(sidx + 1);
    for (auto &S : hs)
      if (sidx + 1 < S.nsteps) by -= (uint64_t)S.npts * 20ull;
    return by;
  };
  // Profiling: events around the fused step kernel of every
  // kProfileEvery-th chunk of steps.  Those chunks replay a second graph
  // that contains the event records; the host reads a profiled chunk's
  // times after the next chunk is queued, so the device never waits.
  constexpr int kProfileEvery = 8;
  if (prof && (int)c->ev.size() < 2 * chunk) {
    const size_t old = c->ev.size();
    c->ev.resize(2 * chunk);
    for (size_t q = old; q < c->ev.size(); ++q) SW_CK(cudaEventCreate(&c->ev[q]));
  }
  auto record_chunk = [&](int nsteps_here, bool with_events) -> int {
    int launched = 0;
    for (int q = 0; q < nsteps_here; q += stride) {
      int nl = 0;
      const int k = q / stride;   // launch of the chunk
      // In profiling mode events bracket the fused step kernel only.
      cudaEvent_t e0 = with_events ? c->ev[2 * k] : nullptr;
      cudaEvent_t e1 = with_events ? c->ev[2 * k + 1] : nullptr;
      if (tile.fuse2)
        e = launch_batch_step2(t, q, n_tiles, n_rec, has_ext, tile, s, &nl, e0, e1, n_term);
      else
        e = launch_batch_step(t, q, n_tiles, n_rec, n_hz, n_hx, n_hy, n_v2u, has_ext, has_3d,
                              has_adj3d, tile, s, &nl, e0, e1, n_term);
      if (e != cudaSuccess) return -1;
      launched += nl;
    }
    if ((e = launch_counter_add(counter, nsteps_here, s)) != cudaSuccess) return -1;
    return launched + 1;
  };
  auto read_chunk = [&](int q) -> int {
    const int live = (std::min(chunk, max_steps - q * chunk) + stride - 1) / stride;
    SW_CK(cudaEventSynchronize(c->ev[2 * live - 1]));
    for (int k = 0; k < live; ++k) {
      float ms = 0.f;
      SW_CK(cudaEventElapsedTime(&ms, c->ev[2 * k], c->ev[2 * k + 1]));
      c->stats.step_kernel_ms += ms;
      c->stats.step_kernel_timed++;
      c->stats.step_bytes += tile.fuse2 ? step_bytes2_at(q * chunk + 2 * k)
                                        : step_bytes_at(q * chunk + k);
    }
    return SW_OK;
  };
  uint64_t launches = 0;
  if (opt.use_graph && nchunks > 1) {
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    const int ngraph = prof ? 2 : 1;   // [0] plain, [1] with event records
    int per = 0;
    auto cleanup = [&]() {
      for (int k = 0; k < 2; ++k) {
        if (exec[k]) cudaGraphExecDestroy(exec[k]);
        if (graph[k]) cudaGraphDestroy(graph[k]);
      }
    };
    for (int k = 0; k < ngraph; ++k) {
      if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        cleanup();
        return cuda_fail(c, e, "begin capture");
      }
      per = record_chunk(chunk, k == 1);
      cudaError_t ec = cudaStreamEndCapture(s, &graph[k]);
      if (per < 0 || ec != cudaSuccess) {
        cleanup();
        return cuda_fail(c, per < 0 ? e : ec, "capture step graph");
      }
      if ((e = cudaGraphInstantiate(&exec[k], graph[k], 0)) != cudaSuccess) {
        cleanup();
        return cuda_fail(c, e, "instantiate step graph");
      }
    }
    int rs = SW_OK, pending = -1;
    for (int q = 0; q < nchunks; ++q) {
      const bool timed = prof && q % kProfileEvery == 0;
      if ((e = cudaGraphLaunch(exec[timed ? 1 : 0], s)) != cudaSuccess) break;
      launches += per;
      if (pending >= 0) {
        rs = read_chunk(pending);
        pending = -1;
        if (rs != SW_OK) break;
      }
      if (timed) pending = q;
    }
    if (e == cudaSuccess && rs == SW_OK && pending >= 0) rs = read_chunk(pending);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
    if (rs != SW_OK) return rs;
  } else {
    for (int q = 0; q < max_steps; q += stride) {
      const int per = record_chunk(stride, prof);
      if (per < 0) return cuda_fail(c, e, "step launch");
      launches += per;
      if (prof) {
        SW_CK(cudaEventSynchronize(c->ev[1]));
        float ms = 0.f;
        SW_CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        c->stats.step_kernel_ms += ms;
        c->stats.step_kernel_timed++;
        c->stats.step_bytes += tile.fuse2 ? step_bytes2_at(q) : step_bytes_at(q);
      }
    }
  }
  // Point updates actually performed (inactive shots skip their tiles).
  uint64_t upd = 0;
  for (auto &S : hs) upd += (uint64_t)S.npts * (uint64_t)S.nsteps;
  c->stats.points_updated += upd;
  for (auto &S : hs) (S.tstep > 0 ? c->stats.steps_forward : c->stats.steps_backward) += S.nsteps;
  c->stats.launches_total += launches;
  c->stats.launches_step += (uint64_t)max_steps;
  // ---- outputs ----
  for (int b = 0; b < nb; ++b) {
    if (!shots[b].io.save_state) continue;
    // Level L after the last step is buffer (L + nsteps) mod nbuf.
    const size_t nf = (size_t)G[b].total();
    for (int q = 0; q < 4; ++q) {
      e = cudaMemcpyAsync(shots[b].io.save_state + (size_t)q * nf,
                          hs[b].f[(q + hs[b].nsteps) % hs[b].nbuf],
                          nf * sizeof(float), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_fail(c, e, "save state");
    }
  }
  for (int b = 0; b < nb; ++b) {
    if (!shots[b].io.final_u2_host) continue;
    const int last = hs[b].nsteps;   // u2 after the last step = f[(last+3)%nbuf]
    const float *u2 = hs[b].f[(last + 3) % hs[b].nbuf];
    e = cudaMemcpy2DAsync(shots[b].io.final_u2_host, (size_t)G[b].n1p * sizeof(float), u2,
                          (size_t)G[b].ld1 * sizeof(float), (size_t)G[b].n1p * sizeof(float),
                          (size_t)G[b].n2p * G[b].n3p, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "download u2");
  }
  if (async) return SW_OK;
  int herr = 0;
  SW_CK(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s));
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(c, e, "batch run");
  if (herr)
    return fail(c, SW_TIMEOUT, "step kernel gave up waiting for a tile copy (error flags %d)",
                herr);
  return SW_OK;
}

}  // namespace swave
