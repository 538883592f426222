// rtmjob.cu - multi-shot RTM: windows, batches admitted by HBM footprint,
// forward + backward phases of a whole batch in the same launches, image
// stacking and illumination normalisation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swave.h"
#include "batch.cuh"
#include "engine.h"

using namespace swave;

namespace swave {

// extract_coord_source_receiver_patch (ExtractPadModel.f90:19-85) and the
// window size of copy_window_vel_gath (ExtractPadModel.f90:446-451).
int compute_window(sw_ctx *c, const sw_genpar &g, float apx, float apy, const float *sou,
                   int nrec, const float *rec, Window &w) {
  if (nrec < 1 || !rec) return fail(c, SW_BAD_PARAM, "shot without receivers");
  const float sx = sou[1], sy = sou[2];
  float gx1 = rec[1], gy1 = rec[2], gxn = gx1, gyn = gy1;
  for (int i = 1; i < nrec; ++i) {
    gx1 = std::min(gx1, rec[3 * i + 1]);
    gxn = std::max(gxn, rec[3 * i + 1]);
    gy1 = std::min(gy1, rec[3 * i + 2]);
    gyn = std::max(gyn, rec[3 * i + 2]);
  }
  const float minx = std::min(sx, gx1), miny = std::min(sy, gy1);
  const float maxx = std::max(sx, gxn), maxy = std::max(sy, gyn);
  const float mx1 = (gx1 + sx) / 2, mxn = (gxn + sx) / 2;
  const float my1 = (gy1 + sy) / 2, myn = (gyn + sy) / 2;
  const float cx = mx1 + std::fabs(mxn - mx1) / 2;
  const float cy = my1 + std::fabs(myn - my1) / 2;
  w.oxw = std::min(minx, cx - apx / 2);
  w.endx = std::max(maxx, cx + apx / 2);
  w.oyw = std::min(miny, cy - apy / 2);
  w.endy = std::max(maxy, cy + apy / 2);
  w.nxw = (int)lroundf((w.endx - w.oxw) / g.dx) + 1;
  w.nyw = (int)lroundf((w.endy - w.oyw) / g.dy) + 1;
  if (g.twoD) {
    w.nyw = 1;
    w.oyw = g.oy;
  }
  if (w.nxw < 4 || w.nyw < 1) return fail(c, SW_BAD_PARAM, "degenerate shot window");
  return SW_OK;
}

// mod_window_pad(adj=.true.) on the host copy of the model (the injection
// plan needs v at the source nodes).
void window_host(const sw_genpar &g, const Window &w, const float *big, std::vector<float> &small) {
  small.resize((size_t)g.nz * w.nxw * w.nyw);
  for (int j = 1; j <= w.nyw; ++j) {
    const float cy = (float)(j - 1) * g.dy + w.oyw;
    const int iy1 = std::min(g.ny, std::max(1, (int)lroundf((cy - g.oy) / g.dy) + 1));
    for (int i = 1; i <= w.nxw; ++i) {
      const float cx = (float)(i - 1) * g.dx + w.oxw;
      const int ix1 = std::min(g.nx, std::max(1, (int)lroundf((cx - g.ox) / g.dx) + 1));
      std::memcpy(&small[(size_t)g.nz * ((i - 1) + (size_t)w.nxw * (j - 1))],
                  &big[(size_t)g.nz * ((ix1 - 1) + (size_t)g.nx * (iy1 - 1))],
                  (size_t)g.nz * sizeof(float));
    }
  }
}

// mod_window_pad(adj=.false.) / mod_copy_image_to_disk
// (ExtractPadModel.f90:532-546,551-590): window columns that fall inside the
// model are added to the model column of the nearest node.
void window_scatter_add_host(const sw_genpar &g, const Window &w, const float *small, float *big) {
  for (int j = 1; j <= w.nyw; ++j) {
    const float cy = (float)(j - 1) * g.dy + w.oyw;
    const int iy = (int)lroundf((cy - g.oy) / g.dy) + 1;
    if (iy < 1 || iy > g.ny) continue;
    for (int i = 1; i <= w.nxw; ++i) {
      const float cx = (float)(i - 1) * g.dx + w.oxw;
      const int ix = (int)lroundf((cx - g.ox) / g.dx) + 1;
      if (ix < 1 || ix > g.nx) continue;
      float *dst = &big[(size_t)g.nz * ((ix - 1) + (size_t)g.nx * (iy - 1))];
      const float *src = &small[(size_t)g.nz * ((i - 1) + (size_t)w.nxw * (j - 1))];
      for (int k = 0; k < g.nz; ++k) dst[k] = dst[k] + src[k];
    }
  }
}

}  // namespace swave

// ---- C-ABI window helpers (host only) --------------------------------------
int sw_shot_window(const sw_genpar *model, float aperture_x, float aperture_y,
                   const float *sou_coord, int nrec, const float *rec_coord, sw_window *out) {
  if (!model || !sou_coord || !rec_coord || !out) return SW_BAD_PARAM;
  Window w;
  const int st = compute_window(nullptr, *model, aperture_x, aperture_y, sou_coord, nrec,
                                rec_coord, w);
  if (st) return st;
  out->oxw = w.oxw;
  out->oyw = w.oyw;
  out->endx = w.endx;
  out->endy = w.endy;
  out->nxw = w.nxw;
  out->nyw = w.nyw;
  return SW_OK;
}

static Window to_window(const sw_window *w) {
  Window v;
  v.oxw = w->oxw;
  v.oyw = w->oyw;
  v.endx = w->endx;
  v.endy = w->endy;
  v.nxw = w->nxw;
  v.nyw = w->nyw;
  return v;
}

int sw_window_extract(const sw_genpar *model, const sw_window *w, const float *big, float *small) {
  if (!model || !w || !big || !small || w->nxw < 1 || w->nyw < 1) return SW_BAD_PARAM;
  std::vector<float> tmp;
  window_host(*model, to_window(w), big, tmp);
  std::memcpy(small, tmp.data(), tmp.size() * sizeof(float));
  return SW_OK;
}

int sw_window_scatter_add(const sw_genpar *model, const sw_window *w, const float *small,
                          float *big) {
  if (!model || !w || !big || !small || w->nxw < 1 || w->nyw < 1) return SW_BAD_PARAM;
  window_scatter_add_host(*model, to_window(w), small, big);
  return SW_OK;
}

namespace {

__global__ void k_illum_stats(long long n, const float *il, float *pmax, double *psum) {
  __shared__ float smax[256];
  __shared__ double ssum[256];
  float m = -INFINITY;
  double s = 0.0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float v = il[q];
    m = fmaxf(m, v);
    s = s + (double)v * (double)v;
  }
  smax[threadIdx.x] = m;
  ssum[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      smax[threadIdx.x] = fmaxf(smax[threadIdx.x], smax[threadIdx.x + w]);
      ssum[threadIdx.x] = ssum[threadIdx.x] + ssum[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    pmax[blockIdx.x] = smax[0];
    psum[blockIdx.x] = ssum[0];
  }
}

// illu = (illu + maxval(illu)/10000)/sqrt(sum(dprod(illu,illu))/size(illu));
// imag = imag/illu (compute_function_gradient.f90:452-453).
__global__ void k_illum_normalise(long long n, int nb, const float *pmax, const double *psum,
                                  const float *im, const float *il, float *out) {
  __shared__ float m;
  __shared__ double r;
  if (threadIdx.x == 0) {
    float mm = pmax[0];
    double ss = 0.0;
    for (int b = 0; b < nb; ++b) {
      mm = fmaxf(mm, pmax[b]);
      ss = ss + psum[b];
    }
    m = mm;
    r = sqrt(ss / (double)n);
  }
  __syncthreads();
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float v = (float)((double)(il[q] + m / 10000.f) / r);
    out[q] = im[q] / v;
  }
}

}  // namespace

struct sw_rtm_job {
  sw_ctx *c;
  sw_genpar g;
  float apx, apy;
  std::vector<float> vel_host;
  float *vel = nullptr;       // full model (device)
  float *wavelet = nullptr;   // g.nt (device)
  float *image = nullptr, *illum = nullptr;
  struct Shot {
    sw_shot s;
    Window w;
    std::vector<float> rec;   // host copy of coordinates
    float *data = nullptr;    // device nrec*nt
  };
  std::vector<Shot> shots;
  int max_batch = 64;
  double mem_fraction = 0.85;
  int last_batch = 0;
  uint64_t points = 0;
};

static void job_free(sw_rtm_job *j) {
  for (auto &s : j->shots)
    if (s.data) cudaFree(s.data);
  for (void *p : {(void *)j->vel, (void *)j->wavelet, (void *)j->image, (void *)j->illum})
    if (p) cudaFree(p);
}

int sw_rtm_job_create(sw_ctx *c, const sw_genpar *model, float apx, float apy, const float *vel,
                      const float *wavelet, int nshot, const sw_shot *shots, sw_rtm_job **out) {
  if (!c || !model || !vel || !wavelet || nshot < 1 || !shots || !out) return SW_BAD_PARAM;
  cudaSetDevice(c->device);
  int st = check_genpar(c, *model);
  if (st) return st;
  sw_rtm_job *j = new sw_rtm_job();
  j->c = c;
  j->g = *model;
  j->apx = apx;
  j->apy = apy;
  const size_t n = (size_t)model->nz * model->nx * model->ny;
  j->vel_host.assign(vel, vel + n);
  auto bail = [&](int code) {
    job_free(j);
    delete j;
    return code;
  };
  cudaStream_t s = c->stream;
  if (cudaMalloc(&j->vel, n * 4) != cudaSuccess || cudaMalloc(&j->image, n * 4) != cudaSuccess ||
      cudaMalloc(&j->illum, n * 4) != cudaSuccess ||
      cudaMalloc(&j->wavelet, (size_t)model->nt * 4) != cudaSuccess) {
    cudaGetLastError();
    return bail(fail(c, SW_OOM_ADMISSION, "RTM job model buffers do not fit"));
  }
  SW_CK(cudaMemcpyAsync(j->vel, vel, n * 4, cudaMemcpyHostToDevice, s));
  SW_CK(cudaMemcpyAsync(j->wavelet, wavelet, (size_t)model->nt * 4, cudaMemcpyHostToDevice, s));
  SW_CK(cudaMemsetAsync(j->image, 0, n * 4, s));
  SW_CK(cudaMemsetAsync(j->illum, 0, n * 4, s));
  j->shots.resize(nshot);
  for (int i = 0; i < nshot; ++i) {
    auto &S = j->shots[i];
    S.s = shots[i];
    if (S.s.nt < 1 || S.s.nt > model->nt)
      return bail(fail(c, SW_BAD_PARAM, "shot %d: bad record length", i));
    if ((st = compute_window(c, *model, apx, apy, S.s.sou_coord, S.s.nrec, S.s.rec_coord, S.w)))
      return bail(st);
    S.rec.assign(S.s.rec_coord, S.s.rec_coord + 3 * (size_t)S.s.nrec);
    S.s.rec_coord = S.rec.data();
    const size_t db = (size_t)S.s.nrec * S.s.nt * 4;
    if (S.s.data) {
      if (cudaMalloc(&S.data, db) != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(c, SW_OOM_ADMISSION, "RTM job data of shot %d does not fit", i));
      }
      if (cudaMemcpyAsync(S.data, S.s.data, db, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return bail(fail(c, SW_CUDA_ERR, "upload of shot %d data failed", i));
    }
    S.s.data = nullptr;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return bail(fail(c, SW_CUDA_ERR, "job upload"));
  *out = j;
  return SW_OK;
}

int sw_rtm_job_set_batch(sw_rtm_job *j, int max_shots, double frac) {
  if (!j || max_shots < 1 || !(frac > 0.0 && frac <= 1.0)) return SW_BAD_PARAM;
  j->max_batch = max_shots;
  j->mem_fraction = frac;
  return SW_OK;
}

int sw_rtm_job_info(const sw_rtm_job *j, int *last_batch, uint64_t *points) {
  if (!j) return SW_BAD_PARAM;
  if (last_batch) *last_batch = j->last_batch;
  if (points) *points = j->points;
  return SW_OK;
}

int sw_rtm_job_reset(sw_rtm_job *j) {
  if (!j) return SW_BAD_PARAM;
  sw_ctx *c = j->c;
  const size_t n = (size_t)j->g.nz * j->g.nx * j->g.ny;
  SW_CK(cudaMemsetAsync(j->image, 0, n * 4, j->c->stream));
  SW_CK(cudaMemsetAsync(j->illum, 0, n * 4, j->c->stream));
  j->points = 0;
  return cudaStreamSynchronize(j->c->stream) == cudaSuccess ? SW_OK : SW_CUDA_ERR;
}

int sw_rtm_job_destroy(sw_rtm_job *j) {
  if (!j) return SW_OK;
  cudaSetDevice(j->c->device);
  cudaStreamSynchronize(j->c->stream);
  job_free(j);
  delete j;
  return SW_OK;
}

namespace {

sw_genpar shot_genpar(const sw_genpar &m, const Window &w, int nt) {
  sw_genpar g = m;
  g.nx = w.nxw;
  g.ny = w.nyw;
  g.ox = w.oxw;
  g.oy = w.oyw;
  g.nt = nt;
  return g;
}

}  // namespace

namespace {

// Device buffers of one shot while its batch runs.
struct ShotBufs {
  float *vpad, *vsmall, *image, *illum, *wave, *traces;
};

// Arena bytes of one shot of a batch: padded velocity, windowed velocity,
// image, illumination, snapshots (RTM) or traces (modelling).
size_t shot_arena_bytes(const sw_genpar &g, int nrec, bool modeling) {
  const Geom G = make_geom(g);
  const size_t nw = (size_t)g.nz * g.nx * g.ny;
  const size_t ntsnap = modeling ? 0 : (size_t)std::max(1, g.nt / g.snapi);
  size_t t = ((size_t)G.total() * 4 + 255) / 256 * 256;        // vel_pad
  t += (nw * 4 + 255) / 256 * 256 * 3;                          // vsmall, image, illum
  t += (nw * ntsnap * 4 + 255) / 256 * 256;                     // snapshots
  t += ((size_t)nrec * g.nt * 4 + 255) / 256 * 256;             // traces
  return t;
}

// The admission budget: mem_fraction of the free device memory, the job
// arena already held counted as free.
int admission_budget(sw_rtm_job *j, double *budget) {
  sw_ctx *c = j->c;
  size_t freeb = 0, totalb = 0;
  SW_CK(cudaMemGetInfo(&freeb, &totalb));
  size_t held = 0;
  auto it = c->bufs.find("rtm_arena");
  if (it != c->bufs.end()) held = it->second.cap;
  *budget = (double)(freeb + held) * j->mem_fraction;
  return SW_OK;
}

// Shots [next, end) admitted into one batch: at most max_batch, and within
// the budget once the first is in.  Each shot also needs the fields and
// plans of run_phases (7 padded grids).  Returns the count; *first_bytes
// is the first shot's need (the caller fails when it alone exceeds the
// budget).
int admit_shots(const sw_rtm_job *j, int next, int end, bool modeling, double budget,
                size_t *first_bytes) {
  const sw_genpar &M = j->g;
  size_t need = 0;
  int n = 0;
  *first_bytes = 0;
  while (next + n < end && n < j->max_batch) {
    const auto &S = j->shots[next + n];
    const sw_genpar g = shot_genpar(M, S.w, S.s.nt);
    const size_t bsz = shot_arena_bytes(g, modeling ? S.s.nrec : 0, modeling) +
                       (size_t)make_geom(g).total() * 4 * 7;
    if (n == 0) *first_bytes = bsz;
    if ((double)(need + bsz) > budget) {
      if (n == 0) return 0;
      break;
    }
    need += bsz;
    ++n;
  }
  return n;
}

// Admits shots [next, end) into a batch by HBM footprint, carves their
// buffers from one arena, windows and pads their velocity.  `modeling`
// batches need trace buffers and no snapshots.
int prepare_batch(sw_rtm_job *j, int &next, int end, bool modeling, std::vector<int> &batch,
                  std::vector<ShotBufs> &bufs, std::vector<std::vector<float>> &vhost) {
  sw_ctx *c = j->c;
  cudaStream_t s = c->stream;
  cudaError_t e;
  int st = SW_OK;
  const sw_genpar &M = j->g;
  auto need_of = [&](const sw_genpar &g, int nrec) -> size_t {
    return shot_arena_bytes(g, nrec, modeling);
  };
  size_t held = 0;
  auto it = c->bufs.find("rtm_arena");
  if (it != c->bufs.end()) held = it->second.cap;
  double budget = 0.0;
  if ((st = admission_budget(j, &budget))) return st;
  batch.clear();
  size_t first_bytes = 0;
  const int nadm = admit_shots(j, next, end, modeling, budget, &first_bytes);
  if (next < end && nadm == 0)
    return fail(c, SW_OOM_ADMISSION, "shot %d needs %zu bytes, budget %.0f", next, first_bytes,
                budget);
  for (int q = 0; q < nadm; ++q) batch.push_back(next++);
  j->last_batch = (int)batch.size();
  std::vector<size_t> offs;
  size_t total = 0;
  for (int id : batch) {
    const auto &S = j->shots[id];
    offs.push_back(total);
    total += need_of(shot_genpar(M, S.w, S.s.nt), modeling ? S.s.nrec : 0);
  }
  // Growing the arena frees and reallocates it (tens of milliseconds at
  // these sizes); when it must grow, size it for the largest batch of
  // max_batch consecutive shots of the job (within the budget), so that it
  // grows at most once per job.
  size_t reserve = total;
  if (held < total) {
    const int ns = (int)j->shots.size();
    std::vector<size_t> need_i(ns);
    for (int q = 0; q < ns; ++q) {
      const auto &S = j->shots[q];
      need_i[q] = need_of(shot_genpar(M, S.w, S.s.nt), modeling ? S.s.nrec : 0);
    }
    size_t window = 0;
    for (int q = 0; q < ns; ++q) {
      window += need_i[q];
      if (q >= j->max_batch) window -= need_i[q - j->max_batch];
      reserve = std::max(reserve, std::min(window, (size_t)budget));
    }
  }
  char *arena = (char *)dbuf(c, "rtm_arena", reserve, &st);
  if (!arena) return st;
  bufs.assign(batch.size(), ShotBufs{});
  vhost.assign(batch.size(), {});
  for (size_t q = 0; q < batch.size(); ++q) {
    const auto &S = j->shots[batch[q]];
    const sw_genpar g = shot_genpar(M, S.w, S.s.nt);
    const Geom G = make_geom(g);
    const size_t nw = (size_t)g.nz * g.nx * g.ny;
    const size_t ntsnap = modeling ? 0 : (size_t)std::max(1, g.nt / g.snapi);
    char *cur = arena + offs[q];
    ShotBufs &B = bufs[q];
    B.vpad = (float *)cur; cur += ((size_t)G.total() * 4 + 255) / 256 * 256;
    B.vsmall = (float *)cur; cur += (nw * 4 + 255) / 256 * 256;
    B.image = (float *)cur; cur += (nw * 4 + 255) / 256 * 256;
    B.illum = (float *)cur; cur += (nw * 4 + 255) / 256 * 256;
    B.wave = (float *)cur; cur += (nw * ntsnap * 4 + 255) / 256 * 256;
    B.traces = (float *)cur;
    // copy_window_vel_gath: window on the device, then model_pad.
    if ((e = launch_window_vel(M.nz, M.nx, M.ny, M.ox, M.oy, M.dx, M.dy, S.w.nxw, S.w.nyw,
                               S.w.oxw, S.w.oyw, j->vel, B.vsmall, s)) != cudaSuccess)
      return cuda_fail(c, e, "window vel");
    if ((e = launch_pad_velocity(G, B.vsmall, B.vpad, s)) != cudaSuccess)
      return cuda_fail(c, e, "pad vel");
    c->stats.launches_total += 2;
    if (modeling) {
      SW_CK(cudaMemsetAsync(B.traces, 0, (size_t)S.s.nrec * g.nt * 4, s));
    } else {
      SW_CK(cudaMemsetAsync(B.image, 0, nw * 4, s));
      SW_CK(cudaMemsetAsync(B.illum, 0, nw * 4, s));
    }
    window_host(M, S.w, j->vel_host.data(), vhost[q]);
  }
  return SW_OK;
}

// Forward phase of one shot: Injection_sinc of the wavelet; snapshots for
// RTM, Extraction_array_sinc for modelling.
PhaseShot forward_phase(sw_rtm_job *j, const sw_rtm_job::Shot &S, const ShotBufs &B,
                        const std::vector<float> &vh, bool modeling) {
  const sw_genpar g = shot_genpar(j->g, S.w, S.s.nt);
  PhaseShot F;
  std::memset(&F.d, 0, sizeof(F.d));
  F.d.g = g;
  F.d.tmin = 1; F.d.tmax = g.nt; F.d.tstep = 1;
  F.d.fd_scheme = SW_FD_FORWARD;
  F.d.injection = SW_INJ_SINC;
  F.io.vel_pad = B.vpad;
  F.io.vel_phys_host = vh.data();
  F.io.nsou = 1;
  F.io.sou_coord = S.s.sou_coord;
  F.io.sou_trace_dev = j->wavelet;
  if (modeling) {
    F.d.extraction = SW_EXT_SINC;
    F.io.nrec = S.s.nrec;
    F.io.rec_coord = S.rec.data();
    F.io.rec_trace_dev = B.traces;
  } else {
    F.d.extract_wave = 1;
    F.io.wave_dev = B.wave;
  }
  return F;
}

}  // namespace

int sw_rtm_job_admit(sw_rtm_job *j, int first, int modeling, int *count) {
  if (!j || !count || first < 0 || first >= (int)j->shots.size()) return SW_BAD_PARAM;
  cudaSetDevice(j->c->device);
  double budget = 0.0;
  int st = admission_budget(j, &budget);
  if (st) return st;
  size_t first_bytes = 0;
  *count = admit_shots(j, first, (int)j->shots.size(), modeling != 0, budget, &first_bytes);
  if (*count == 0)
    return fail(j->c, SW_OOM_ADMISSION, "shot %d needs %zu bytes, budget %.0f", first,
                first_bytes, budget);
  return SW_OK;
}

int sw_rtm_job_run(sw_rtm_job *j, int first, int count) {
  if (!j || first < 0 || count < 1 || first + count > (int)j->shots.size()) return SW_BAD_PARAM;
  sw_ctx *c = j->c;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  cudaError_t e;
  int st = SW_OK;
  const sw_genpar &M = j->g;
  for (int q = first; q < first + count; ++q)
    if (!j->shots[q].data) return fail(c, SW_BAD_PARAM, "shot %d has no observed data", q);
  int next = first;
  const int end = first + count;
  std::vector<int> batch;
  std::vector<ShotBufs> bufs;
  std::vector<std::vector<float>> vhost;
  // The phases are queued without waiting for each other: the host builds
  // the next phase's plans (the backward pass's receiver injection plan is
  // the large one) while the device runs the previous phase.  Errors of the
  // step kernels collect in the run_err flag, read once at the end.
  RunOpts opts = c->run_opts;
  opts.async_end = true;
  int *rerr = (int *)dbuf(c, "run_err", sizeof(int), &st);
  if (!rerr) return st;
  SW_CK(cudaMemsetAsync(rerr, 0, sizeof(int), s));
  while (next < end) {
    if ((st = prepare_batch(j, next, end, false, batch, bufs, vhost))) return st;
    std::vector<PhaseShot> fwd(batch.size()), bwd(batch.size());
    for (size_t q = 0; q < batch.size(); ++q) {
      const auto &S = j->shots[batch[q]];
      const ShotBufs &B = bufs[q];
      const sw_genpar g = shot_genpar(M, S.w, S.s.nt);
      fwd[q] = forward_phase(j, S, B, vhost[q], false);
      // Backward: 2D adjoint (3D forward) stencil, Injection_sinc of the data,
      // Imaging_condition_sourceonly_from_memory (to_disk_to_memory_RTM.f90:450-486).
      PhaseShot &R = bwd[q];
      std::memset(&R.d, 0, sizeof(R.d));
      R.d.g = g;
      R.d.tmin = g.nt; R.d.tmax = 1; R.d.tstep = -1;
      R.d.fd_scheme = g.twoD ? SW_FD_ADJOINT : SW_FD_FORWARD;
      R.d.injection = SW_INJ_SINC;
      R.d.imaging = SW_IMG_RTM;
      R.io.vel_pad = B.vpad;
      R.io.vel_phys_host = vhost[q].data();
      R.io.nsou = S.s.nrec;
      R.io.sou_coord = S.rec.data();
      R.io.sou_trace_dev = S.data;
      R.io.wave_dev = B.wave;
      R.io.image_dev = B.image;
      R.io.illum_dev = B.illum;
    }
    const uint64_t p0 = c->stats.points_updated;
    if ((st = run_phases(c, fwd, opts))) return st;
    if ((st = run_phases(c, bwd, opts))) return st;
    j->points += c->stats.points_updated - p0;
    // mod_copy_image, shots in order.
    for (size_t q = 0; q < batch.size(); ++q) {
      const auto &S = j->shots[batch[q]];
      if ((e = launch_copy_image(M.nz, M.nx, M.ny, M.ox, M.oy, M.dx, M.dy, S.w.nxw, S.w.nyw,
                                 S.w.oxw, S.w.oyw, bufs[q].image, bufs[q].illum, j->image,
                                 j->illum, s)) != cudaSuccess)
        return cuda_fail(c, e, "copy image");
      c->stats.launches_total++;
    }
  }
  int herr = 0;
  SW_CK(cudaMemcpyAsync(&herr, rerr, sizeof(int), cudaMemcpyDeviceToHost, s));
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(c, e, "rtm job");
  if (herr)
    return fail(c, SW_TIMEOUT, "step kernel gave up waiting for a tile copy (error flags %d)",
                herr);
  return SW_OK;
}

int sw_rtm_job_model(sw_rtm_job *j, int first, int count, float *const *data) {
  if (!j || !data || first < 0 || count < 1 || first + count > (int)j->shots.size())
    return SW_BAD_PARAM;
  sw_ctx *c = j->c;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  int st = SW_OK;
  int next = first;
  const int end = first + count;
  std::vector<int> batch;
  std::vector<ShotBufs> bufs;
  std::vector<std::vector<float>> vhost;
  while (next < end) {
    if ((st = prepare_batch(j, next, end, true, batch, bufs, vhost))) return st;
    std::vector<PhaseShot> fwd(batch.size());
    for (size_t q = 0; q < batch.size(); ++q)
      fwd[q] = forward_phase(j, j->shots[batch[q]], bufs[q], vhost[q], true);
    const uint64_t p0 = c->stats.points_updated;
    if ((st = run_phases(c, fwd, c->run_opts))) return st;
    j->points += c->stats.points_updated - p0;
    for (size_t q = 0; q < batch.size(); ++q) {
      const auto &S = j->shots[batch[q]];
      float *out = data[batch[q] - first];
      if (!out) return fail(c, SW_BAD_PARAM, "null output for shot %d", batch[q]);
      SW_CK(cudaMemcpyAsync(out, bufs[q].traces, (size_t)S.s.nrec * S.s.nt * 4,
                            cudaMemcpyDeviceToHost, s));
    }
    SW_CK(cudaStreamSynchronize(s));
  }
  return SW_OK;
}

int sw_rtm_job_result(sw_rtm_job *j, float *image, float *illum, float *image_norm) {
  if (!j) return SW_BAD_PARAM;
  sw_ctx *c = j->c;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const long long n = (long long)j->g.nz * j->g.nx * j->g.ny;
  int st = SW_OK;
  if (image) SW_CK(cudaMemcpyAsync(image, j->image, n * 4, cudaMemcpyDeviceToHost, s));
  if (illum) SW_CK(cudaMemcpyAsync(illum, j->illum, n * 4, cudaMemcpyDeviceToHost, s));
  if (image_norm) {
    const int nb = 296;
    float *pmax = (float *)dbuf(c, "red_pmax", nb * sizeof(float), &st);
    double *psum = (double *)dbuf(c, "red_psum", nb * sizeof(double), &st);
    float *out = (float *)dbuf(c, "rtm_norm", n * 4, &st);
    if (!pmax || !psum || !out) return st;
    k_illum_stats<<<nb, 256, 0, s>>>(n, j->illum, pmax, psum);
    k_illum_normalise<<<nb, 256, 0, s>>>(n, nb, pmax, psum, j->image, j->illum, out);
    c->stats.launches_total += 2;
    SW_CK(cudaMemcpyAsync(image_norm, out, n * 4, cudaMemcpyDeviceToHost, s));
  }
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? SW_OK : cuda_fail(c, e, "rtm result");
}
