// engine.cu - host side of libswave: context, device buffers, the
// propagation driver (propagator_acoustic) and the operator drivers.
//
// Host arithmetic that feeds the kernels (sinc weights, tapers, positions)
// restates the reference in float, compiled with -ffp-contract=off, so the
// weights are bit-identical to the reference formulas evaluated in IEEE
// single precision.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/swave.h"
#include "butterworth.h"
#include "engine.h"
#include "batch.cuh"
#include "swave_dev.cuh"

using namespace swave;

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------

int sw_ctx_create(int device, sw_ctx **out) {
  if (!out) return SW_BAD_PARAM;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return SW_CUDA_ERR;
  if (device < 0 || device >= ndev) return SW_BAD_PARAM;
  if (cudaSetDevice(device) != cudaSuccess) return SW_CUDA_ERR;
  sw_ctx *c = new sw_ctx();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return SW_CUDA_ERR;
  }
  *out = c;
  return SW_OK;
}

int sw_ctx_destroy(sw_ctx *c) {
  if (!c) return SW_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto &kv : c->bufs) cudaFree(kv.second.p);
  for (auto &e : c->ev) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
  return SW_OK;
}

const char *sw_last_error(const sw_ctx *c) { return c ? c->err.c_str() : "null context"; }

const char *sw_version(void) { return "swave 0.1 (sm_103a, FP32 wavefields, FP64 reductions)"; }

int sw_ctx_get_stats(const sw_ctx *c, sw_stats *o) {
  if (!c || !o) return SW_BAD_PARAM;
  *o = c->stats;
  return SW_OK;
}
int sw_ctx_reset_stats(sw_ctx *c) {
  if (!c) return SW_BAD_PARAM;
  std::memset(&c->stats, 0, sizeof(c->stats));
  return SW_OK;
}
int sw_ctx_set_tuning(sw_ctx *c, const sw_tuning *t) {
  if (!c || !t) return SW_BAD_PARAM;
  if (t->step_kernel < 0 || t->step_kernel > 4 || t->graph_chunk < 1 || t->tile_x < 1 ||
      t->tile_y < 1 ||
      (t->tile_z != 32 && t->tile_z != 64 && t->tile_z != 128))
    return swave::fail(c, SW_BAD_PARAM, "invalid tuning");
  c->run_opts.tile.stream2d = t->step_kernel;
  c->run_opts.tile.stream3d = t->step_kernel == 0 ? 0 : t->step_kernel == 1 ? 1 : 2;
  c->run_opts.tile.ty = t->tile_y;
  c->run_opts.tile.tz = t->tile_z;
  c->run_opts.tile.tx = t->tile_x;
  c->run_opts.chunk = t->graph_chunk;
  c->run_opts.use_graph = t->use_graph != 0;
  return SW_OK;
}

int sw_ctx_get_tuning(const sw_ctx *c, sw_tuning *t) {
  if (!c || !t) return SW_BAD_PARAM;
  t->step_kernel = c->run_opts.tile.stream2d;
  t->tile_z = c->run_opts.tile.tz;
  t->tile_x = c->run_opts.tile.tx;
  t->tile_y = c->run_opts.tile.ty;
  t->graph_chunk = c->run_opts.chunk;
  t->use_graph = c->run_opts.use_graph ? 1 : 0;
  return SW_OK;
}

int sw_ctx_set_boundary(sw_ctx *c, int mode) {
  if (!c || mode < 0 || mode > 1) return SW_BAD_PARAM;
  c->run_opts.rigid = mode == 1;
  return SW_OK;
}

int sw_ctx_set_profiling(sw_ctx *c, int on) {
  if (!c) return SW_BAD_PARAM;
  c->profiling = on != 0;
  return SW_OK;
}

namespace swave {

int fail(sw_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int cuda_fail(sw_ctx *c, cudaError_t e, const char *what) {
  return fail(c, SW_CUDA_ERR, "%s: %s", what, cudaGetErrorString(e));
}

// Grow-only named device buffers owned by the context.
void *dbuf(sw_ctx *c, const std::string &name, size_t bytes, int *st, size_t slack) {
  if (bytes == 0) bytes = 16;
  DBuf &b = c->bufs[name];
  if (b.cap < bytes) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes + slack);
    if (e == cudaErrorMemoryAllocation && slack > 0) {
      cudaGetLastError();
      slack = 0;
      e = cudaMalloc(&b.p, bytes);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      *st = fail(c, e == cudaErrorMemoryAllocation ? SW_OOM_ADMISSION : SW_CUDA_ERR,
                 "cudaMalloc(%s, %zu bytes): %s", name.c_str(), bytes, cudaGetErrorString(e));
      return nullptr;
    }
    b.cap = bytes + slack;
  }
  return b.p;
}

int check_genpar(sw_ctx *c, const sw_genpar &g) {
  if (g.surf_type < 0 || g.shot_type < 0 || g.rec_type < 0)
    return fail(c, SW_BAD_PARAM, "negative surf_type/shot_type/rec_type");
  if (g.nz < 1 || g.nx < 1 || g.ny < 1 || g.nt < 1 || g.ntaper < 4 || g.snapi < 1)
    return fail(c, SW_BAD_PARAM, "bad sizes nz=%d nx=%d ny=%d nt=%d ntaper=%d snapi=%d", g.nz,
                g.nx, g.ny, g.nt, g.ntaper, g.snapi);
  if (g.lsinc < 3 || (g.lsinc % 2) == 0 || g.lsinc > 15)
    return fail(c, SW_BAD_PARAM, "lsinc must be odd in [3,15], got %d", g.lsinc);
  if (g.twoD && g.ny != 1) return fail(c, SW_BAD_PARAM, "twoD requires ny = 1");
  if (!(g.dz > 0.f) || !(g.dx > 0.f) || (!g.twoD && !(g.dy > 0.f)) || !(g.dt > 0.f))
    return fail(c, SW_BAD_PARAM, "non-positive spacing or dt");
  return SW_OK;
}

// FDbounds for shot_type = surf_type = 0 (ReadSouVelRho.f90:456-470).
Geom make_geom(const sw_genpar &g) {
  Geom G;
  // Mirror sources extend the top padding; a free surface replaces the top
  // taper by lsinc cells (ExtractPadModel.f90:228-234).
  if (g.shot_type > 0 || g.surf_type > 0) {
    if (g.shot_type > 0) G.nmin1 = -(g.ntaper + g.lsinc / 2 + 2) + 1;
    if (g.surf_type > 0) G.nmin1 = -g.lsinc + 1;
  } else {
    G.nmin1 = -g.ntaper + 1;
  }
  G.nmax1 = g.nz + g.ntaper;
  G.nmin2 = -g.ntaper + 1;
  G.nmax2 = g.nx + g.ntaper;
  if (!g.twoD) {
    G.nmin3 = -g.ntaper + 1;
    G.nmax3 = g.ny + g.ntaper;
    G.nbound = 4;
  } else {
    G.nmin3 = 1;
    G.nmax3 = 1;
    G.nbound = 0;
  }
  G.lo1 = G.nmin1 - 4;
  G.lo2 = G.nmin2 - 4;
  G.lo3 = G.nmin3 - G.nbound;
  G.n1p = G.nmax1 + 4 - G.lo1 + 1;
  G.n2p = G.nmax2 + 4 - G.lo2 + 1;
  G.n3p = G.nmax3 + G.nbound - G.lo3 + 1;
  G.ld1 = (G.n1p + 31) / 32 * 32;
  G.nz = g.nz;
  G.nx = g.nx;
  G.ny = g.ny;
  G.twoD = g.twoD;
  return G;
}

// FD_acoustic_init_coefs + FD_types_assign_scaled_coefs (FDcoefs.f90:25-36,
// FDtypes.f90:50-80), coefpower = 2.
Coefs make_coefs(const sw_genpar &g) {
  const float c0 = -205.f / 72.f, c1 = 8.f / 5.f, c2 = -1.f / 5.f, c3 = 8.f / 315.f,
              c4 = -1.f / 560.f;
  const float dxi = 1.f / g.dx, dyi = 1.f / g.dy, dzi = 1.f / g.dz;
  const float px = dxi * dxi, py = dyi * dyi, pz = dzi * dzi;
  Coefs c;
  c.c0x = c0 * px; c.c1x = c1 * px; c.c2x = c2 * px; c.c3x = c3 * px; c.c4x = c4 * px;
  c.c0y = c0 * py; c.c1y = c1 * py; c.c2y = c2 * py; c.c3y = c3 * py; c.c4y = c4 * py;
  c.c0z = c0 * pz; c.c1z = c1 * pz; c.c2z = c2 * pz; c.c3z = c3 * pz; c.c4z = c4 * pz;
  return c;
}

Coefs make_rho_coefs(const sw_genpar &g) {
  const float c0 = 0.f, c1 = 1225.f / 1024.f, c2 = -1225.f / (1024.f * 15.f),
              c3 = 1225.f / (1024.f * 125.f), c4 = -1225.f / (1024.f * 1715.f);
  const float dxi = 1.f / g.dx, dyi = 1.f / g.dy, dzi = 1.f / g.dz;
  Coefs c;
  c.c0x = c0 * dxi; c.c1x = c1 * dxi; c.c2x = c2 * dxi; c.c3x = c3 * dxi; c.c4x = c4 * dxi;
  c.c0y = c0 * dyi; c.c1y = c1 * dyi; c.c2y = c2 * dyi; c.c3y = c3 * dyi; c.c4y = c4 * dyi;
  c.c0z = c0 * dzi; c.c1z = c1 * dzi; c.c2z = c2 * dzi; c.c3z = c3 * dzi; c.c4z = c4 * dzi;
  return c;
}

// mksinc (Interpolate.f90:15-42), evaluated once per trace.
void mksinc(float *sinc, int lsinc, float shift) {
  const float pi = 3.141592654f;
  float fsum = 0.f;
  for (int n = 1; n <= lsinc; ++n) {
    float fact;
    if (n <= (int)((float)(lsinc / 2 + 1) + shift))
      fact = ((float)(n - 1) - shift) / (float)(lsinc / 2);
    else
      fact = ((float)(lsinc - n) + shift) / (float)(lsinc / 2);
    if (fact <= 0.f) fact = 0.f;
    const float pos = pi * ((float)(n - (lsinc / 2 + 1)) - shift);
    if (std::fabs(pos) > 0.005f)
      sinc[n - 1] = (fact * sinf(pos)) / pos;
    else
      sinc[n - 1] = fact * (1.f - (pos * pos) / 6.f);
    fsum = fsum + sinc[n - 1];
  }
  for (int n = 1; n <= lsinc; ++n) sinc[n - 1] = sinc[n - 1] / fsum;
}

// find_i_d (ModelSpaceTypes.f90:144-151) for the three axes.
void positions(const sw_genpar &g, int n, const float *coord, std::vector<int> &ic,
               std::vector<float> &dc) {
  ic.resize(3 * (size_t)n);
  dc.resize(3 * (size_t)n);
  const float om[3] = {g.oz, g.ox, g.twoD ? 0.f : g.oy};
  const float de[3] = {g.dz, g.dx, g.twoD ? 1.f : g.dy};
  for (int r = 0; r < n; ++r)
    for (int a = 0; a < 3; ++a) {
      const float e = coord[3 * r + a];
      const int ie = (int)lroundf((e - om[a]) / de[a]) + 1;
      ic[3 * r + a] = ie;
      dc[3 * r + a] = e - (om[a] + (float)(ie - 1) * de[a]);
    }
}

// compute_taper / cos_sin_taper (Taper.f90:14-44).
static void cos_sin_taper(std::vector<float> &a, int ntaper, int n) {
  const float pi = 3.14159265359f;
  const int m = std::min(ntaper, n);
  for (int i = 1; i <= m; ++i) {
    const float s = sinf((pi * (float)(i - 1)) / (float)(2 * (m - 1)));
    a[i - 1] = s * s;
  }
  const int i0 = std::max(1, n - ntaper);
  for (int i = i0; i <= n; ++i) {
    const float cc = cosf((pi * (float)(i - i0)) / (float)(2 * ntaper));
    a[i - 1] = cc * cc;
  }
}
void compute_taper(int nxw, int nyw, std::vector<float> &tx, std::vector<float> &ty) {
  tx.assign(nxw, 1.f);
  ty.assign(nyw, 1.f);
  cos_sin_taper(tx, std::min(nxw / 2, 10), nxw);
  if (nyw > 1) cos_sin_taper(ty, std::min(nyw / 2, 10), nyw);
}

static inline float host_vel(const sw_genpar &g, const float *vp, int i, int j, int k) {
  const int ii = std::min(std::max(i, 1), g.nz), jj = std::min(std::max(j, 1), g.nx),
            kk = std::min(std::max(k, 1), g.ny);
  return vp[(size_t)(ii - 1) + (size_t)g.nz * ((jj - 1) + (size_t)g.nx * (kk - 1))];
}

// Builds the injection plan: a box covering every contribution and, per box
// cell, the contributions in source order.
int build_injection(sw_ctx *c, const sw_genpar &g, const Geom &G, int mode, int nsou,
                    const float *sou_coord, const float *vel_phys, InjPlan &plan,
                    const float *rho_phys, bool mirror) {
  plan.on = 0;
  if (mode == SW_INJ_NONE || nsou <= 0) return SW_OK;
  std::vector<int> ic;
  std::vector<float> dc;
  positions(g, nsou, sou_coord, ic, dc);
  const bool sinc = mode == SW_INJ_SINC || mode == SW_INJ_LSRTM_SINC;
  const int h = sinc ? g.lsinc / 2 : 0;
  const int ls = g.lsinc;
  const float de[3] = {g.dz, g.dx, g.twoD ? 1.f : g.dy};
  int bi0 = 1 << 30, bi1 = -(1 << 30), bj0 = bi0, bj1 = bi1, bk0 = bi0, bk1 = bi1;
  for (int r = 0; r < nsou; ++r) {
    const int i = ic[3 * r], j = ic[3 * r + 1], k = g.twoD ? 1 : ic[3 * r + 2];
    if (g.twoD && ic[3 * r + 2] != 1)
      return fail(c, SW_BAD_PARAM, "2D source %d has a non-zero y coordinate", r);
    const int hk = g.twoD ? 0 : h;
    if (i - h < G.nmin1 || i + h > G.nmax1 || j - h < G.nmin2 || j + h > G.nmax2 ||
        k - hk < G.nmin3 || k + hk > G.nmax3)
      return fail(c, SW_BAD_PARAM, "source %d footprint leaves the compute domain", r);
    if (mirror) {
      // The mirror source sits at row -i (Injection.f90:440-449).
      if (-i - h < G.nmin1 || -i + h > G.nmax1)
        return fail(c, SW_BAD_PARAM, "mirror of source %d leaves the compute domain", r);
      bi0 = std::min(bi0, -i - h); bi1 = std::max(bi1, -i + h);
    }
    bi0 = std::min(bi0, i - h); bi1 = std::max(bi1, i + h);
    bj0 = std::min(bj0, j - h); bj1 = std::max(bj1, j + h);
    bk0 = std::min(bk0, k - hk); bk1 = std::max(bk1, k + hk);
  }
  const long long nb = (long long)(bi1 - bi0 + 1) * (bj1 - bj0 + 1) * (bk1 - bk0 + 1);
  struct Tmp { int cell; InjEntry e; };
  std::vector<Tmp> all;
  const long long per = (sinc ? (long long)ls * ls * (g.twoD ? 1 : ls) : 1) * (mirror ? 2 : 1);
  all.reserve((size_t)(per * nsou));
  std::vector<float> sz(ls), sx(ls), sy(ls);
  const float inv_d2 = 1.f / (g.dz * g.dx);
  const float inv_d3 = 1.f / ((g.dz * g.dx) * g.dy);
  for (int r = 0; r < nsou; ++r) {
    const int i0 = ic[3 * r], j0 = ic[3 * r + 1], k0 = g.twoD ? 1 : ic[3 * r + 2];
    float v2r;
    if (mode == SW_INJ_LSRTM_SINC) {
      v2r = g.twoD ? inv_d2 : inv_d3;
    } else {
      // Injection_sinc / Injection_simple: v**2, times rho with density
      // (Injection.f90:170-190).
      const float vv = host_vel(g, vel_phys, i0, j0, k0);
      v2r = rho_phys ? (vv * vv) * host_vel(g, rho_phys, i0, j0, k0) : vv * vv;
    }
    auto cell = [&](int i, int j, int k) {
      return (int)((i - bi0) + (long long)(bi1 - bi0 + 1) * ((j - bj0) + (long long)(bj1 - bj0 + 1) * (k - bk0)));
    };
    // A mirror entry subtracts the term of the reflected row with the
    // reflected z weight; it carries -v2r, which negates the product exactly.
    if (!sinc) {
      all.push_back({cell(i0, j0, k0), {r, v2r, 1.f, 1.f, 1.f}});
      if (mirror) all.push_back({cell(-i0, j0, k0), {r, -v2r, 1.f, 1.f, 1.f}});
      continue;
    }
    mksinc(sz.data(), ls, dc[3 * r] / de[0]);
    mksinc(sx.data(), ls, dc[3 * r + 1] / de[1]);
    if (g.twoD) {
      for (int j = -h; j <= h; ++j)
        for (int i = -h; i <= h; ++i) {
          all.push_back({cell(i0 + i, j0 + j, 1), {r, v2r, sz[h + i], sx[h + j], 1.f}});
          if (mirror)
            all.push_back({cell(i - i0, j0 + j, 1), {r, -v2r, sz[h - i], sx[h + j], 1.f}});
        }
    } else {
      // Injection_source_sinc_xyz weights y with the x sinc column
      // (Injection.f90:314).
      for (int k = -h; k <= h; ++k)
        for (int j = -h; j <= h; ++j)
          for (int i = -h; i <= h; ++i) {
            all.push_back({cell(i0 + i, j0 + j, k0 + k), {r, v2r, sz[h + i], sx[h + j], sx[h + k]}});
            if (mirror)
              all.push_back(
                  {cell(i - i0, j0 + j, k0 + k), {r, -v2r, sz[h - i], sx[h + j], sx[h + k]}});
          }
    }
  }
  // Stable counting sort by cell keeps source order inside a cell.
  std::vector<int> off((size_t)nb + 1, 0);
  for (auto &t : all) off[(size_t)t.cell + 1]++;
  for (long long b = 0; b < nb; ++b) off[(size_t)b + 1] += off[(size_t)b];
  std::vector<int> pos(off.begin(), off.end() - 1);
  std::vector<InjEntry> ent(all.size());
  for (auto &t : all) ent[(size_t)pos[(size_t)t.cell]++] = t.e;
  plan.on = 1;
  plan.bi0 = bi0; plan.bi1 = bi1; plan.bj0 = bj0; plan.bj1 = bj1; plan.bk0 = bk0; plan.bk1 = bk1;
  plan.off = std::move(off);
  plan.ent = std::move(ent);
  return SW_OK;
}

int build_extraction(sw_ctx *c, const sw_genpar &g, const Geom &G, int mode, int nrec,
                     const float *rec_coord, ExtPlan &plan, bool mirror) {
  plan.on = 0;
  if (mode == SW_EXT_NONE || nrec <= 0) return SW_OK;
  std::vector<float> dc;
  positions(g, nrec, rec_coord, plan.ic, dc);
  const int h = g.lsinc / 2, ls = g.lsinc;
  const bool sinc = mode != SW_EXT_SIMPLE_AFWI;
  const float de[3] = {g.dz, g.dx, g.twoD ? 1.f : g.dy};
  plan.wz.assign((size_t)nrec * ls, 0.f);
  plan.wx.assign((size_t)nrec * ls, 0.f);
  for (int r = 0; r < nrec; ++r) {
    const int i = plan.ic[3 * r], j = plan.ic[3 * r + 1], k = plan.ic[3 * r + 2];
    if (g.twoD && k != 1) return fail(c, SW_BAD_PARAM, "2D receiver %d has non-zero y", r);
    const int hh = sinc ? h : 0;
    const int kk = g.twoD ? 1 : k;
    const int hk = g.twoD ? 0 : hh;
    if (i - hh < G.lo1 || i + hh > G.nmax1 + 4 || j - hh < G.lo2 || j + hh > G.nmax2 + 4 ||
        kk - hk < G.lo3 || kk + hk > G.nmax3 + G.nbound)
      return fail(c, SW_BAD_PARAM, "receiver %d footprint leaves the padded grid", r);
    if (mirror && (-i - hh < G.lo1 || -i + hh > G.nmax1 + 4))
      return fail(c, SW_BAD_PARAM, "mirror of receiver %d leaves the padded grid", r);
    if (sinc) {
      mksinc(&plan.wz[(size_t)r * ls], ls, dc[3 * r] / de[0]);
      mksinc(&plan.wx[(size_t)r * ls], ls, dc[3 * r + 1] / de[1]);
    }
  }
  plan.on = 1;
  plan.mode = mode;
  plan.nrec = nrec;
  plan.mirror = mirror ? 1 : 0;
  return SW_OK;
}

// ---------------------------------------------------------------------------
// One propagation on device-resident fields (propagator_acoustic)
// ---------------------------------------------------------------------------

int propagate_dev(sw_ctx *c, const sw_prop_desc &d, const DevIO &io) {
  std::vector<PhaseShot> one(1);
  one[0].d = d;
  one[0].io = io;
  return run_phases(c, one, c->run_opts);
}

// Uploads the physical velocity and pads it on the device.
int upload_velocity(sw_ctx *c, const sw_genpar &g, const float *vel, const char *slot,
                    float **vel_pad) {
  int st = SW_OK;
  const Geom G = make_geom(g);
  const size_t nphys = (size_t)g.nz * g.nx * g.ny;
  float *vp = (float *)dbuf(c, std::string(slot) + "_phys", nphys * sizeof(float), &st);
  float *pad = (float *)dbuf(c, slot, (size_t)G.total() * sizeof(float), &st);
  if (!vp || !pad) return st;
  cudaError_t e = cudaMemcpyAsync(vp, vel, nphys * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "upload vel");
  if ((e = launch_pad_velocity(G, vp, pad, c->stream)) != cudaSuccess) return cuda_fail(c, e, "pad");
  c->stats.launches_total++;
  *vel_pad = pad;
  return SW_OK;
}

int prepare_rho(sw_ctx *c, const sw_genpar &g, const float *rho_host, const char *slot,
                const float **rho_pad, const float **delp) {
  int st = SW_OK;
  float *pad = nullptr;
  if ((st = upload_velocity(c, g, rho_host, slot, &pad))) return st;
  const Geom G = make_geom(g);
  const size_t nf = (size_t)G.total();
  float *a = (float *)dbuf(c, std::string(slot) + "_delp", nf * sizeof(float), &st);
  float *b = (float *)dbuf(c, std::string(slot) + "_tmp", nf * sizeof(float), &st);
  if (!a || !b) return st;
  float sinc[9];
  mksinc(sinc, 9, 0.5f);
  int nl = 0;
  cudaError_t e = launch_rho_delp(G, pad, a, b, sinc, c->stream, &nl);
  if (e != cudaSuccess) return cuda_fail(c, e, "rho interpolation");
  c->stats.launches_total += nl;
  *rho_pad = pad;
  *delp = a;
  return SW_OK;
}

int upload(sw_ctx *c, const char *slot, const void *h, size_t bytes, void **d) {
  int st = SW_OK;
  void *p = dbuf(c, slot, bytes, &st);
  if (!p) return st;
  if (h) {
    cudaError_t e = cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "upload");
  } else {
    cudaError_t e = cudaMemsetAsync(p, 0, bytes, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "memset");
  }
  *d = p;
  return SW_OK;
}

int download(sw_ctx *c, void *h, const void *d, size_t bytes) {
  cudaError_t e = cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "download");
  return SW_OK;
}

}  // namespace swave

// ---------------------------------------------------------------------------
// Public entry points
// ---------------------------------------------------------------------------

int sw_vel_check(const sw_genpar *g, const float *vel, float *courant, float *samplerate) {
  if (!g || !vel) return SW_BAD_PARAM;
  const size_t n = (size_t)g->nz * g->nx * g->ny;
  float vmax = vel[0], vmin = vel[0];
  for (size_t q = 1; q < n; ++q) {
    vmax = std::max(vmax, vel[q]);
    vmin = std::min(vmin, vel[q]);
  }
  // vel_check (ReadSouVelRho.f90:629-656, 669-753).
  const float stab_cond = g->twoD ? 0.45f : 0.35f;
  const float stab = g->twoD ? vmax * g->dt / std::min(g->dz, g->dx)
                             : vmax * g->dt / std::min(std::min(g->dz, g->dx), g->dy);
  const float lambdamin = vmin / g->fmax;
  const float sr = g->twoD ? lambdamin / std::max(g->dz, g->dx)
                           : lambdamin / std::max(std::max(g->dz, g->dx), g->dy);
  if (courant) *courant = stab;
  if (samplerate) *samplerate = sr;
  if (stab > stab_cond || sr < 2.0f) return SW_BAD_PARAM;
  return SW_OK;
}

int sw_propagate(sw_ctx *c, const sw_prop_desc *d, const sw_prop_io *io) {
  if (!c || !d || !io || !io->vel) return SW_BAD_PARAM;
  cudaSetDevice(c->device);
  const sw_genpar &g = d->g;
  int st = check_genpar(c, g);
  if (st) return st;
  const int nt = g.nt, ntsnap = nt / g.snapi;
  const size_t nphys = (size_t)g.nz * g.nx * g.ny;
  DevIO dio;
  if ((st = upload_velocity(c, g, io->vel, "vel", &dio.vel_pad))) return st;
  dio.vel_phys_host = io->vel;
  if (io->rho) {
    // The variable-density drivers use the forward-grid operator in both
    // directions (to_disk_to_memory_RTM.f90:388-398,455-465).
    if (d->fd_scheme != SW_FD_FORWARD)
      return fail(c, SW_UNSUPPORTED, "the variable-density operator has no adjoint-grid form");
    if ((st = prepare_rho(c, g, io->rho, "rho", &dio.rho_pad, &dio.delp))) return st;
    dio.rho_phys_host = io->rho;
  }
  dio.nsou = d->injection != SW_INJ_NONE ? io->nsou : 0;
  dio.sou_coord = io->sou_coord;
  void *p = nullptr;
  if (dio.nsou > 0) {
    if (!io->sou_coord || !io->sou_trace) return fail(c, SW_BAD_PARAM, "missing source arrays");
    if ((st = upload(c, "sou_tr", io->sou_trace, (size_t)dio.nsou * nt * sizeof(float), &p))) return st;
    dio.sou_trace_dev = (float *)p;
  }
  dio.nrec = d->extraction != SW_EXT_NONE ? io->nrec : 0;
  dio.rec_coord = io->rec_coord;
  if (dio.nrec > 0) {
    if (!io->rec_coord || !io->rec_trace) return fail(c, SW_BAD_PARAM, "missing receiver arrays");
    if ((st = upload(c, "rec_tr", io->rec_trace, (size_t)dio.nrec * nt * sizeof(float), &p))) return st;
    dio.rec_trace_dev = (float *)p;
  }
  const bool need_wave = d->extract_wave || d->imaging != SW_IMG_NONE;
  if (need_wave) {
    if (!io->wave) return fail(c, SW_BAD_PARAM, "wave array required");
    if ((st = upload(c, "wave", io->wave, nphys * std::max(ntsnap, 1) * sizeof(float), &p))) return st;
    dio.wave_dev = (float *)p;
  }
  const bool img = d->imaging != SW_IMG_NONE && d->imaging != SW_IMG_BORN;
  if (img) {
    if (!io->image || !io->illum) return fail(c, SW_BAD_PARAM, "image/illum required");
    if ((st = upload(c, "image", io->image, nphys * sizeof(float), &p))) return st;
    dio.image_dev = (float *)p;
    if ((st = upload(c, "illum", io->illum, nphys * sizeof(float), &p))) return st;
    dio.illum_dev = (float *)p;
  }
  if (d->imaging == SW_IMG_AFWI_RHO) {
    // Only the variable-density AFWI driver calls it (to_disk_to_memory_AFWI.f90:
    // 375-381,397-403).
    if (!io->rho || !io->image2)
      return fail(c, SW_BAD_PARAM, "SW_IMG_AFWI_RHO needs rho and image2");
    if ((st = upload(c, "image2", io->image2, nphys * sizeof(float), &p))) return st;
    dio.image2_dev = (float *)p;
  }
  if (d->imaging == SW_IMG_BORN) {
    if (!io->ref) return fail(c, SW_BAD_PARAM, "ref required");
    if ((st = upload(c, "ref", io->ref, nphys * sizeof(float), &p))) return st;
    dio.ref_dev = (float *)p;
  }
  dio.final_u2_host = io->final_u2;
  if ((st = propagate_dev(c, *d, dio))) return st;
  if (dio.nrec > 0 && (st = download(c, io->rec_trace, dio.rec_trace_dev, (size_t)dio.nrec * nt * sizeof(float))))
    return st;
  if (d->extract_wave &&
      (st = download(c, io->wave, dio.wave_dev, nphys * std::max(ntsnap, 1) * sizeof(float))))
    return st;
  if (img) {
    if ((st = download(c, io->image, dio.image_dev, nphys * sizeof(float)))) return st;
    if ((st = download(c, io->illum, dio.illum_dev, nphys * sizeof(float)))) return st;
  }
  if (dio.image2_dev &&
      (st = download(c, io->image2, dio.image2_dev, nphys * sizeof(float))))
    return st;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "sw_propagate");
  return SW_OK;
}

static sw_prop_desc base_desc(const sw_genpar &g, bool fwd) {
  sw_prop_desc d;
  std::memset(&d, 0, sizeof(d));
  d.g = g;
  if (fwd) { d.tmin = 1; d.tmax = g.nt; d.tstep = 1; }
  else { d.tmin = g.nt; d.tmax = 1; d.tstep = -1; }
  return d;
}

int sw_modeling(sw_ctx *c, const sw_genpar *g, const float *vel, const float *sou_coord,
                const float *wavelet, int nrec, const float *rec_coord, float *data,
                float *final_u2) {
  if (!c || !g || !vel || !sou_coord || !wavelet || !data || (nrec > 0 && !rec_coord))
    return SW_BAD_PARAM;
  std::fill(data, data + (size_t)nrec * g->nt, 0.f);
  sw_prop_desc d = base_desc(*g, true);
  d.fd_scheme = SW_FD_FORWARD;
  d.injection = SW_INJ_SINC;
  d.extraction = SW_EXT_SINC;
  sw_prop_io io;
  std::memset(&io, 0, sizeof(io));
  io.vel = vel;
  io.nsou = 1; io.sou_coord = sou_coord; io.sou_trace = wavelet;
  io.nrec = nrec; io.rec_coord = rec_coord; io.rec_trace = data;
  io.final_u2 = final_u2;
  return sw_propagate(c, &d, &io);
}

// Forward with device snapshots, then a backward or Born propagation that
// reads them (RTM_to_memory, LSRTM_to_memory, BORN_to_memory).
static int two_pass(sw_ctx *c, const sw_genpar &g, const float *vel, const float *ref,
                    const float *sou_coord, const float *wavelet, int nrec,
                    const float *rec_coord, const float *data_in, float *data_out,
                    float *image, float *illum, int kind) {
  cudaSetDevice(c->device);
  int st = check_genpar(c, g);
  if (st) return st;
  const int nt = g.nt, ntsnap = nt / g.snapi;
  const size_t nphys = (size_t)g.nz * g.nx * g.ny;
  DevIO f;
  if ((st = upload_velocity(c, g, vel, "vel", &f.vel_pad))) return st;
  f.vel_phys_host = vel;
  void *p = nullptr;
  if ((st = upload(c, "sou_tr", wavelet, (size_t)nt * sizeof(float), &p))) return st;
  f.sou_trace_dev = (float *)p;
  f.nsou = 1;
  f.sou_coord = sou_coord;
  if ((st = upload(c, "wave", nullptr, nphys * std::max(ntsnap, 1) * sizeof(float), &p))) return st;
  f.wave_dev = (float *)p;
  sw_prop_desc d = base_desc(g, true);
  d.fd_scheme = SW_FD_FORWARD;
  d.injection = SW_INJ_SINC;
  d.extract_wave = 1;
  if ((st = propagate_dev(c, d, f))) return st;

  DevIO b;
  b.vel_pad = f.vel_pad;
  b.vel_phys_host = vel;
  b.wave_dev = f.wave_dev;
  sw_prop_desc e2;
  if (kind == 2) {  // Born
    e2 = base_desc(g, true);
    e2.fd_scheme = SW_FD_FORWARD;
    e2.injection = SW_INJ_NONE;
    e2.extraction = SW_EXT_LSRTM_SINC;
    e2.imaging = SW_IMG_BORN;
    if ((st = upload(c, "ref", ref, nphys * sizeof(float), &p))) return st;
    b.ref_dev = (float *)p;
    b.nrec = nrec;
    b.rec_coord = rec_coord;
    if ((st = upload(c, "rec_tr", nullptr, (size_t)nrec * nt * sizeof(float), &p))) return st;
    b.rec_trace_dev = (float *)p;
  } else {
    e2 = base_desc(g, false);
    if (kind == 0) {  // RTM
      e2.fd_scheme = g.twoD ? SW_FD_ADJOINT : SW_FD_FORWARD;
      e2.injection = SW_INJ_SINC;
      e2.imaging = SW_IMG_RTM;
    } else {          // LSRTM
      e2.fd_scheme = SW_FD_ADJOINT;
      e2.injection = SW_INJ_LSRTM_SINC;
      e2.imaging = SW_IMG_LSRTM;
    }
    b.nsou = nrec;
    b.sou_coord = rec_coord;
    if ((st = upload(c, "dat_tr", data_in, (size_t)nrec * nt * sizeof(float), &p))) return st;
    b.sou_trace_dev = (float *)p;
    if ((st = upload(c, "image", nullptr, nphys * sizeof(float), &p))) return st;
    b.image_dev = (float *)p;
    if ((st = upload(c, "illum", nullptr, nphys * sizeof(float), &p))) return st;
    b.illum_dev = (float *)p;
  }
  if ((st = propagate_dev(c, e2, b))) return st;
  if (kind == 2) {
    if ((st = download(c, data_out, b.rec_trace_dev, (size_t)nrec * nt * sizeof(float)))) return st;
  } else {
    if ((st = download(c, image, b.image_dev, nphys * sizeof(float)))) return st;
    if ((st = download(c, illum, b.illum_dev, nphys * sizeof(float)))) return st;
  }
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "two_pass");
  return SW_OK;
}

int sw_rtm(sw_ctx *c, const sw_genpar *g, const float *vel, const float *sou_coord,
           const float *wavelet, int nrec, const float *rec_coord, const float *data,
           float *image, float *illum) {
  if (!c || !g || !vel || !sou_coord || !wavelet || !rec_coord || !data || !image || !illum)
    return SW_BAD_PARAM;
  return two_pass(c, *g, vel, nullptr, sou_coord, wavelet, nrec, rec_coord, data, nullptr, image,
                  illum, 0);
}

int sw_lsrtm(sw_ctx *c, const sw_genpar *g, const float *vel, const float *sou_coord,
             const float *wavelet, int nrec, const float *rec_coord, const float *data,
             float *image, float *illum) {
  if (!c || !g || !vel || !sou_coord || !wavelet || !rec_coord || !data || !image || !illum)
    return SW_BAD_PARAM;
  return two_pass(c, *g, vel, nullptr, sou_coord, wavelet, nrec, rec_coord, data, nullptr, image,
                  illum, 1);
}

int sw_born(sw_ctx *c, const sw_genpar *g, const float *vel, const float *ref,
            const float *sou_coord, const float *wavelet, int nrec, const float *rec_coord,
            float *data) {
  if (!c || !g || !vel || !ref || !sou_coord || !wavelet || !rec_coord || !data)
    return SW_BAD_PARAM;
  return two_pass(c, *g, vel, ref, sou_coord, wavelet, nrec, rec_coord, nullptr, data, nullptr,
                  nullptr, 2);
}

int sw_bandpass(sw_ctx *c, int ntr, int nt, float dt, float flo, float fhi, int nplo,
                int nphi, int phase, float *traces) {
  if (!c || !traces || ntr < 1 || nt < 2 || !(dt > 0.f) || nplo < 1 || nphi < 1 ||
      nplo > 2 * swave_bp::kMaxSections || nphi > 2 * swave_bp::kMaxSections)
    return SW_BAD_PARAM;
  cudaSetDevice(c->device);
  // bandpass (Bandpass.f90:89-149): cutoffs in cycles per sample; a
  // low-cut below 1e-6 or a high-cut at or above 4.999999 is skipped, and a
  // filter that passes everything is refused.
  const float flo_t = flo * dt, fhi_t = fhi * dt;
  if (flo_t < 0.0001f && fhi_t > 0.4999f)
    return fail(c, SW_BAD_PARAM, "band-pass needs flo or fhi inside the band");
  swave_bp::Sections lo, hi;
  if (flo_t > 0.000001f) lo = swave_bp::lowcut_sections(flo_t, nplo, phase);
  if (fhi_t < 4.999999f) hi = swave_bp::highcut_sections(fhi_t, nphi, phase);
  const int npad = 10, n = nt + 2 * npad;
  std::vector<float> hostc(5 * (lo.n + hi.n) + 2 * npad);
  std::memcpy(hostc.data(), lo.c, sizeof(float) * 5 * lo.n);
  std::memcpy(hostc.data() + 5 * lo.n, hi.c, sizeof(float) * 5 * hi.n);
  swave_bp::end_tapers(npad, hostc.data() + 5 * (lo.n + hi.n),
                       hostc.data() + 5 * (lo.n + hi.n) + npad);
  int st = SW_OK;
  void *p = nullptr;
  if ((st = upload(c, "bp_coef", hostc.data(), hostc.size() * sizeof(float), &p))) return st;
  const float *dc = (const float *)p;
  const size_t nb = (size_t)ntr * nt * sizeof(float);
  if ((st = upload(c, "bp_in", traces, nb, &p))) return st;
  const float *din = (const float *)p;
  float *dout = (float *)dbuf(c, "bp_out", nb, &st);
  float *D = (float *)dbuf(c, "bp_d", (size_t)n * ntr * sizeof(float), &st);
  float *T = (float *)dbuf(c, "bp_t", (size_t)n * ntr * sizeof(float), &st);
  if (!dout || !D || !T) return st;
  cudaError_t e = launch_bandpass(ntr, nt, npad, phase, lo.n, dc, hi.n, dc + 5 * lo.n,
                                  dc + 5 * (lo.n + hi.n), dc + 5 * (lo.n + hi.n) + npad, din,
                                  dout, D, T, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "band-pass");
  c->stats.launches_total++;
  if ((st = download(c, traces, dout, nb))) return st;
  if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cuda_fail(c, e, "band-pass");
  return SW_OK;
}

int sw_mute_mask(int nrec, int nt, float dt, float ot, const float *sou_coord,
                 const float *rec_coord, float v0, float v1, float t0, float t1, float tramp,
                 float *mask) {
  if (nrec < 0 || nt < 1 || !(dt > 0.f) || !sou_coord || (nrec > 0 && (!rec_coord || !mask)))
    return SW_BAD_PARAM;
  // MuteParam_compute_mask (Mute.f90:50-95) with compute_top_mute and
  // compute_bottom_mute (Mute.f90:172-219): a sin^2 ramp up to the top mute
  // time, a cos^2 ramp down after the bottom one, both at the offset
  // (hx + hy) over their velocity; the mask is their product.
  const float pi = 3.1415926535f;
  const int nramp = (int)(tramp / dt + 1.5f);
  for (int r = 0; r < nrec; ++r) {
    const float hx = rec_coord[3 * r + 1] - sou_coord[1];
    const float hy = rec_coord[3 * r + 2] - sou_coord[2];
    float *m = mask + (size_t)r * nt;
    // top: 0, ramp over samples it-nramp..it, then 1
    const float ht = (hx + hy) / v0;
    const float tt = std::sqrt(t0 * t0 + ht * ht);
    const int it = (int)((tt - ot) / dt + 1.5f);
    // bottom: 1, ramp over samples ib+1..ib+1+nramp, then 0
    const float hb = (hx + hy) / v1;
    const float tb = std::sqrt(t1 * t1 + hb * hb);
    const int ib = (int)((tb - ot) / dt + 1.5f);
    for (int i = 1; i <= nt; ++i) {
      float top = i > it ? 1.f : 0.f;
      if (i >= std::max(1, it - nramp) && i <= std::min(nt, it)) {
        const float sv = std::sin((float)(i - it + nramp) * pi / (float)(2 * nramp));
        top = sv * sv;
      }
      float bot = 1.f;
      if (i >= std::max(1, ib + 1) && i <= std::min(nt, ib + 1 + nramp)) {
        const float cv = std::cos((float)(i - ib - 1) * pi / (float)(2 * nramp));
        bot = cv * cv;
      }
      if (i >= ib + 1 + nramp) bot = 0.f;   // mute(it+1+nramp:) = 0 comes last
      m[i - 1] = top * bot;
    }
  }
  return SW_OK;
}

int sw_rho_wavelet(float *w, int nt, int lsinc) {
  if (!w || nt < 1 || lsinc < 3 || (lsinc % 2) == 0) return SW_BAD_PARAM;
  // readsou, withRho branch (ReadSouVelRho.f90:328-343): w'(t) = w(t + dt/2)
  // by an lsinc-point sinc; taps outside the trace are dropped and the
  // remaining weights renormalised.
  std::vector<float> sinc(lsinc), tr(w, w + nt);
  mksinc(sinc.data(), lsinc, 0.5f);
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

int sw_born_wavelet(float *w, int nt, float dt) {
  if (!w || nt < 1) return SW_BAD_PARAM;
  // readsou, Born/LSRTM branch (ReadSouVelRho.f90:318-326).
  std::vector<float> tr(w, w + nt);
  for (int i = 0; i < nt; ++i) w[i] = 0.f;
  for (int it = 2; it <= nt - 1; ++it)
    w[it - 1] = w[it - 1] + ((-2 * tr[it - 1] + tr[it - 2]) + tr[it]) / (dt * dt);
  return SW_OK;
}
