// noalloc.cu - 2D shot modelling that allocates no device memory.
//
// sw_modeling_noalloc runs the same propagation as sw_modeling (2D forward
// stencil, sinc source injection, sinc receiver extraction) for callers that
// cannot allocate device memory while they call it: a process whose device
// memory is already committed to its own pool (an RTM job holding its
// snapshot arena, say) or a caller that must not let cudaMalloc / cudaFree
// synchronise the device in the middle of other work.  Every device array of
// the run - velocity, the five time levels, Higdon coefficients, injection
// and extraction plans, traces and the batch descriptor - is carved from one
// file-scope __device__ array of kNoallocScratchBytes, which every GPU that
// loads the library holds until the process exits.
//
// The first call on a device looks up the array's device address there with
// cudaGetSymbolAddress (a host-side name is not a device address); make
// that first call before any stream capture.  The lookup is guarded by a
// mutex, so first calls from several host threads are safe.  The cached
// address belongs to the device's primary context: after cudaDeviceReset
// the module is loaded again, possibly elsewhere, so do not reset a device
// on which this entry point has run.  Only the reference's default
// geometry is built: surf_type, shot_type and rec_type must be 0 (the free
// surface and mirror modes return SW_UNSUPPORTED).  All calls share the array and
// it keeps the last call's contents: the time levels, the receiver traces,
// the step counter and the error flags are cleared at the start of each
// call.  Calls that overlap on the GPU (from several host threads, or
// while an earlier call's work is still running) race on the array.
// Work runs on the legacy default stream of the current device; the call
// returns after the traces are copied back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/swave.h"
#include "batch.cuh"
#include "engine.h"

namespace swave {
namespace {

constexpr size_t kNoallocScratchBytes = 32u << 20;   // 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of the scratch array on each device (set up once, under
// g_scratch_mu).
unsigned char *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

size_t rup256(size_t b) { return (b + 255) / 256 * 256; }

struct Carver {
  unsigned char *base;
  size_t used = 0;
  template <class T>
  T *take(size_t n) {
    T *p = reinterpret_cast<T *>(base + used);
    used += rup256(std::max<size_t>(n, 1) * sizeof(T));
    return p;
  }
};

}  // namespace
}  // namespace swave

using namespace swave;

extern "C" int sw_modeling_noalloc(const sw_genpar *g, const float *vel, const float *sou_coord,
                                   const float *wavelet, int nrec, const float *rec_coord,
                                   float *data) {
  if (!g || !vel || !sou_coord || !wavelet || !data || nrec < 0 || (nrec > 0 && !rec_coord))
    return SW_BAD_PARAM;
  if (!g->twoD || g->ny != 1) return SW_UNSUPPORTED;
  // The free surface and the mirror sources / receivers need the surface
  // plan and the mirror injection entries; this entry point builds neither.
  if (g->surf_type != 0 || g->shot_type != 0 || g->rec_type != 0) return SW_UNSUPPORTED;
  int st = check_genpar(nullptr, *g);
  if (st) return st;
  const Geom G = make_geom(*g);
  const int nt = g->nt;
  const long long n1 = G.nmax1 - G.nmin1 + 1, n2 = G.nmax2 - G.nmin2 + 1;
  const size_t nf = (size_t)G.total();
  const size_t nphys = (size_t)g->nz * g->nx;

  // Host plans (no device memory involved).
  InjPlan inj;
  if ((st = build_injection(nullptr, *g, G, SW_INJ_SINC, 1, sou_coord, vel, inj))) return st;
  ExtPlan ext;
  if ((st = build_extraction(nullptr, *g, G, SW_EXT_SINC, nrec, rec_coord, ext))) return st;

  // Scratch layout and the size limit.
  const size_t need =
      rup256(nphys * 4) + 6 * rup256(nf * 4) + rup256(16 * n2 * 4) + rup256(16 * n1 * 4) +
      rup256(std::max<size_t>(inj.off.size(), 1) * 4) +
      rup256(std::max<size_t>(inj.ent.size(), 1) * sizeof(InjEntry)) +
      rup256(std::max<size_t>(ext.ic.size(), 1) * 4) +
      2 * rup256(std::max<size_t>(ext.wz.size(), 1) * 4) + rup256((size_t)nt * 4) +
      rup256(std::max<size_t>((size_t)nrec * nt, 1) * 4) + rup256(sizeof(ShotDev)) +
      7 * rup256(2 * sizeof(int)) + 2 * rup256(sizeof(int));
  if (need > kNoallocScratchBytes) return SW_OOM_ADMISSION;

  // Once per device: the scratch array's device address.
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SW_CUDA_ERR;
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SW_CUDA_ERR;
      g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    base = g_scratch_ptr[dev];
  }
  cudaStream_t s = 0;   // legacy default stream
  Carver cv{base};
  float *vphys = cv.take<float>(nphys);
  float *vpad = cv.take<float>(nf);
  ShotDev S;
  std::memset(&S, 0, sizeof(S));
  S.nbuf = 5;   // one step per launch: five rotating time levels
  for (int q = 0; q < 5; ++q) S.f[q] = cv.take<float>(nf);
  float *gz = cv.take<float>(16 * n2), *gx = cv.take<float>(16 * n1);
  int *ioff = cv.take<int>(inj.off.size());
  InjEntry *ient = cv.take<InjEntry>(inj.ent.size());
  int *ric = cv.take<int>(ext.ic.size());
  float *wz = cv.take<float>(ext.wz.size()), *wx = cv.take<float>(ext.wx.size());
  float *src = cv.take<float>((size_t)nt);
  float *rec = cv.take<float>((size_t)nrec * nt);
  ShotDev *dshot = cv.take<ShotDev>(1);
  int *dtab[7];
  for (int q = 0; q < 7; ++q) dtab[q] = cv.take<int>(2);
  int *counter = cv.take<int>(1), *err = cv.take<int>(1);
  if (cv.used > kNoallocScratchBytes) return SW_OOM_ADMISSION;

  auto ck = [](cudaError_t e) { return e == cudaSuccess; };
  // Inputs; the time levels, traces, counter and flags start at zero.
  bool ok = ck(cudaMemcpyAsync(vphys, vel, nphys * 4, cudaMemcpyHostToDevice, s)) &&
            ck(launch_pad_velocity(G, vphys, vpad, s)) &&
            ck(cudaMemcpyAsync(src, wavelet, (size_t)nt * 4, cudaMemcpyHostToDevice, s));
  for (int q = 0; q < 5 && ok; ++q) ok = ck(cudaMemsetAsync(S.f[q], 0, nf * 4, s));
  ok = ok && ck(cudaMemsetAsync(rec, 0, std::max<size_t>((size_t)nrec * nt, 1) * 4, s)) &&
       ck(cudaMemsetAsync(counter, 0, sizeof(int), s)) &&
       ck(cudaMemsetAsync(err, 0, sizeof(int), s)) &&
       ck(launch_higdon_coeffs(G, vpad, g->dt, 1.f / g->dx, 1.f / g->dy, 1.f / g->dz, gz, gx, gz,
                               s));
  if (ok && inj.on)
    ok = ck(cudaMemcpyAsync(ioff, inj.off.data(), inj.off.size() * 4, cudaMemcpyHostToDevice,
                            s)) &&
         ck(cudaMemcpyAsync(ient, inj.ent.data(), inj.ent.size() * sizeof(InjEntry),
                            cudaMemcpyHostToDevice, s));
  if (ok && ext.on)
    ok = ck(cudaMemcpyAsync(ric, ext.ic.data(), ext.ic.size() * 4, cudaMemcpyHostToDevice, s)) &&
         ck(cudaMemcpyAsync(wz, ext.wz.data(), ext.wz.size() * 4, cudaMemcpyHostToDevice, s)) &&
         ck(cudaMemcpyAsync(wx, ext.wx.data(), ext.wx.size() * 4, cudaMemcpyHostToDevice, s));
  if (!ok) return SW_CUDA_ERR;

  // The shot descriptor (the fields a forward modelling run reads).
  S.g = G;
  S.c = make_coefs(*g);
  S.vel = vpad;
  S.gz = gz; S.gx = gx; S.gy = gz;
  S.inj_on = inj.on;
  S.bi0 = inj.bi0; S.bi1 = inj.bi1; S.bj0 = inj.bj0; S.bj1 = inj.bj1;
  S.bk0 = inj.bk0; S.bk1 = inj.bk1;
  S.inj_off = ioff;
  S.inj_ent = ient;
  S.src_tr = src;
  S.ext_mode = ext.on ? ext.mode : 0;
  S.nrec = ext.on ? ext.nrec : 0;
  S.ext_half = g->lsinc / 2;
  S.ric = ric; S.wz = wz; S.wx = wx;
  S.rec_tr = rec;
  S.vconst = 1.f;
  S.tmin = 1;
  S.tcnt = 1;
  S.tstep = 1;
  S.nsteps = nt;
  S.nt = nt;
  S.snapi = g->snapi;
  S.ntsnap = nt / g->snapi;
  S.k12 = 12.f * (g->dt * g->dt);
  S.div11 = 1.f / 11.f;
  {
    const float xs = g->dt * (float)g->snapi;
    S.dt2snap = xs * xs;
  }
  S.npts = n1 * n2;
  // Prefix tables of a one-shot batch: {0, count}.
  StepTile tile;
  tile.stream2d = 0;   // 32x8 point tiles, Higdon edges in their own kernels
  tile.has_fwd2d = 1;
  tile.has_adj2d = tile.has_fwd3d = tile.has_adj3d = 0;
  tile.fused_edges = 0;
  const int counts[7] = {step_ctas(G, tile), S.nrec, (int)n2, (int)n1, 0, 0, 0};
  for (int q = 0; q < 7 && ok; ++q) {
    const int h[2] = {0, counts[q]};
    ok = ck(cudaMemcpyAsync(dtab[q], h, sizeof(h), cudaMemcpyHostToDevice, s));
    // Pageable copies are staged before the call returns, so h may go.
  }
  ok = ok && ck(cudaMemcpyAsync(dshot, &S, sizeof(S), cudaMemcpyHostToDevice, s));
  if (!ok) return SW_CUDA_ERR;
  BatchTables t;
  std::memset(&t, 0, sizeof(t));
  t.nshots = 1;
  t.shots = dshot;
  t.step_tiles = dtab[0];
  t.rec_start = dtab[1];
  t.hz_start = dtab[2];
  t.hx_start = dtab[3];
  t.hy_start = dtab[4];
  t.v2u_blocks = dtab[5];
  t.edge_start = dtab[6];
  t.counter = counter;
  t.err = err;
  // Time loop: step q reads s = *counter + q with the counter left at 0.
  for (int q = 0; q < nt; ++q) {
    if (launch_batch_step(t, q, counts[0], counts[1], counts[2], counts[3], 0, 0, ext.on ? 1 : 0,
                          0, 0, tile, s, nullptr, nullptr, nullptr) != cudaSuccess)
      return SW_CUDA_ERR;
  }
  if (nrec > 0 &&
      !ck(cudaMemcpyAsync(data, rec, (size_t)nrec * nt * 4, cudaMemcpyDeviceToHost, s)))
    return SW_CUDA_ERR;
  // The step kernels record a bounded wait that gave up in the error flag.
  int herr = 0;
  if (!ck(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
      !ck(cudaStreamSynchronize(s)))
    return SW_CUDA_ERR;
  return herr ? SW_TIMEOUT : SW_OK;
}
