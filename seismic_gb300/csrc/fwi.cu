// fwi.cu - FWI objective/gradient driver and the FP64 L-BFGS of libswave.
//
// compute_fct_gdt (progs/afwi/compute_function_gradient.f90:208-350) runs
// shot by shot on the device; the misfit is accumulated in FP64 in the
// reference's trace order.  The L-BFGS keeps its correction pairs and
// search vectors in HBM in FP64 (libs/libinv/lbfgs.f:49-558); only the
// scalar line-search logic (MCSRCH/MCSTEP) runs on the host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swave.h"
#include "engine.h"
#include "swave_dev.cuh"

using namespace swave;

namespace {

constexpr int kRedBlocks = 296;  // 2 x 148: fixed partition => deterministic sums
constexpr int kRedThreads = 256;

// ---------------------------------------------------------------------------
// Post-processing kernels (compute_function_gradient.f90:332-343)
// ---------------------------------------------------------------------------
__global__ void k_illu_pow(long long n, float p, float *il) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    il[q] = powf(il[q], p);
}

// Per-block partial max(illum) and sum(dprod(illum, illum)); also scales the
// gradient: grad = 2*grad/sngl(scaling).
__global__ void k_grad_scale_stats(long long n, float sscal, float *grad, const float *il,
                                   float *pmax, double *psum) {
  __shared__ float smax[kRedThreads];
  __shared__ double ssum[kRedThreads];
  float m = -INFINITY;
  double s = 0.0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    grad[q] = (2.0f * grad[q]) / sscal;
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

__global__ void k_final_stats(int nb, long long n, const float *pmax, const double *psum,
                              float *maxil, double *rmsil) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float m = pmax[0];
  double s = 0.0;
  for (int b = 0; b < nb; ++b) {
    m = fmaxf(m, pmax[b]);
    s = s + psum[b];
  }
  *maxil = m;
  *rmsil = sqrt(s / (double)n);
}

// illu = (illu + maxval/10000)/sqrt(sum(dprod)/size); grad = grad/illu*mask.
__global__ void k_normalise(long long n, const float *maxil, const double *rmsil, float *il,
                            float *grad, const float *mask) {
  const float m = *maxil;
  const double r = *rmsil;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float v = (float)((double)(il[q] + m / 10000.f) / r);
    il[q] = v;
    float g = grad[q] / v;
    g = g * (mask ? mask[q] : 1.0f);
    grad[q] = g;
  }
}

__global__ void k_mask(long long n, float *grad, const float *mask) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    grad[q] = grad[q] * (mask ? mask[q] : 1.0f);
}

// triangle (Smoothing.f90:140-181) with boxconv (Smoothing.f90:194-227): one
// thread per line; element e of line l is at base(l) + e*estride.  The
// three work vectors of each line live in `scratch`.
__device__ void d_boxconv(int nb, int nx, const float *xx, float *yy, float *bb) {
  const int ny = nx + nb - 1;
  bb[0] = xx[0];
  for (int i = 2; i <= nx; ++i) bb[i - 1] = bb[i - 2] + xx[i - 1];
  for (int i = nx + 1; i <= ny; ++i) bb[i - 1] = bb[i - 2];
  for (int i = 1; i <= nb; ++i) yy[i - 1] = bb[i - 1];
  for (int i = nb + 1; i <= ny; ++i) yy[i - 1] = bb[i - 1] - bb[i - nb - 1];
  for (int i = 1; i <= ny; ++i) yy[i - 1] = yy[i - 1] / (float)nb;
}

__global__ void k_triangle(int n12, int nr, int nlines, int lines_inner, long long lstride_in,
                           long long lstride_out, long long estride, const float *uu, float *vv,
                           float *scratch) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nlines) return;
  // Line l = (a, b) with a < lines_inner fastest.
  const int la = l % lines_inner, lb = l / lines_inner;
  const long long base = (long long)la * lstride_in + (long long)lb * lstride_out;
  const long long per = 4LL * (n12 + 2 * nr);
  float *qq = scratch + (long long)l * per;
  float *pp = qq + (n12 + 2 * nr);
  float *bb = pp + (n12 + 2 * nr);
  float *tt = bb + (n12 + 2 * nr);
  for (int i = 0; i < n12; ++i) qq[i] = uu[base + i * estride];
  if (n12 == 1) {
    tt[0] = qq[0];
  } else {
    d_boxconv(nr, n12, qq, pp, bb);
    const int np = nr + n12 - 1;
    d_boxconv(nr, np, pp, qq, bb);
    for (int i = 1; i <= n12; ++i) tt[i - 1] = qq[i + nr - 2];
    for (int i = 1; i <= nr - 1; ++i) tt[i - 1] = tt[i - 1] + qq[nr - i - 1];
    for (int i = 1; i <= nr - 1; ++i) tt[n12 - i] = tt[n12 - i] + qq[n12 + (nr - 1) + i - 1];
  }
  for (int i = 0; i < n12; ++i) vv[base + i * estride] = tt[i];
}

// ---------------------------------------------------------------------------
// FP64 vector kernels for the L-BFGS
// ---------------------------------------------------------------------------
__global__ void k_dot_partial(long long n, const double *a, const double *b, double *part) {
  __shared__ double sh[kRedThreads];
  double s = 0.0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    s = s + a[q] * b[q];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_partials(int nb, const double *part, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s = s + part[b];
  *out = s;
}

// y = a*x + y  (a on host)
__global__ void k_axpy(long long n, double a, const double *x, double *y) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    y[q] = y[q] + a * x[q];
}
// y = y - a*x
__global__ void k_aymx(long long n, double a, const double *x, double *y) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    y[q] = y[q] - a * x[q];
}
// y = a*y
__global__ void k_scal(long long n, double a, double *y) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    y[q] = a * y[q];
}
// y = -x*d (d scalar; DIAG is uniform when DIAGCO = .false.)
__global__ void k_negmul(long long n, const double *x, double d, double *y) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    y[q] = -x[q] * d;
}
// z = x - y
__global__ void k_sub(long long n, const double *x, const double *y, double *z) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    z[q] = x[q] - y[q];
}
// x = wa + stp*s
__global__ void k_step_x(long long n, const double *wa, double stp, const double *s, double *x) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    x[q] = wa[q] + stp * s[q];
}
// FREEZE_X (lbfgs.f:1-43)
__global__ void k_freeze(long long n, int type, double xmin, double xmax, const float *mask,
                         const double *xinit, double *x) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    double v = x[q];
    if (type) {
      v = fmax(xmin, v);
      v = fmin(xmax, v);
    } else {
      const float m = mask[q];
      if (m != 0.f && m != 2.f) {
        v = fmax(xmin, v);
        v = fmin(xmax, v);
      }
      if (m == 0.f || m == 2.f) v = xinit[q];
    }
    x[q] = v;
  }
}

// FREEZE_XOC (nlinv_lbfgs.f:1-22): block j of m values clipped to
// [pmin(j), pmax(j)].
__global__ void k_freeze_blocks(long long n, long long m, const double *pmin, const double *pmax,
                                double *x) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const long long j = q / m;
    double v = fmax(pmin[j], x[q]);
    x[q] = fmin(pmax[j], v);
  }
}

inline int gsz(long long n) {
  long long b = (n + 255) / 256;
  return (int)std::max(1LL, std::min(b, 152LL * 8));
}

// ---------------------------------------------------------------------------
// Binomial checkpoint schedule (revolve) over checkpoint segments.
// Reversing l segments whose first state is available, with s free state
// slots, takes at least t(l, s + 1) segment advances (Griewank 1992:
// t(l, c) = r l - beta(c + 1, r - 1) with beta(c, r) = (c + r)! / (c! r!) and
// r the smallest integer with beta(c, r) >= l).  The schedule attains it by
// splitting at the m minimising m + t(l - m, s - 1) + t(m, s): advance m
// segments, keep that state in a slot, reverse the last l - m segments with
// one slot less, release the slot, reverse the first m.  Without a free
// slot every segment is reached from the first state through a work slot.
// ---------------------------------------------------------------------------
double binom_beta(int c, long long r) {
  if (r < 0) return 0.0;
  double b = 1.0;
  for (long long i = 1; i <= r; ++i) b = b * (double)(c + i) / (double)i;
  return b;
}

long long revolve_advances(long long l, int s) {
  if (l <= 1) return 0;
  const int c = s + 1;
  long long r = 0;
  double b = 1.0;   // beta(c, r)
  while (b < (double)l) {
    ++r;
    b = b * (double)(c + r) / (double)r;
  }
  return r * l - (long long)std::llround(binom_beta(c + 1, r - 1));
}

struct CkOp {
  int process;   // 0: advance S_a -> S_b from slot src into slot dst; 1: segment a from src
  int a, b, src, dst;
};

void revolve_schedule(int a, int b, int src, std::vector<int> &freel, int work,
                      std::vector<CkOp> &ops) {
  const int l = b - a;
  if (l == 1) {
    ops.push_back({1, a, a + 1, src, -1});
    return;
  }
  const int s = (int)freel.size();
  if (s == 0) {
    for (int k = b - 1; k > a; --k) {
      ops.push_back({0, a, k, src, work});
      ops.push_back({1, k, k + 1, work, -1});
    }
    ops.push_back({1, a, a + 1, src, -1});
    return;
  }
  long long best = -1;
  int bm = 1;
  for (int m = 1; m < l; ++m) {
    const long long cost = m + revolve_advances(l - m, s - 1) + revolve_advances(m, s);
    if (best < 0 || cost < best) {
      best = cost;
      bm = m;
    }
  }
  const int slot = freel.back();
  freel.pop_back();
  ops.push_back({0, a, a + bm, src, slot});
  revolve_schedule(a + bm, b, slot, freel, work, ops);
  freel.push_back(slot);
  revolve_schedule(a, a + bm, src, freel, work, ops);
}

}  // namespace

long long sw_revolve_advances_internal(long long l, int s) { return revolve_advances(l, s); }

// ---------------------------------------------------------------------------
// compute_fct_gdt
// ---------------------------------------------------------------------------
namespace {

// Compute_OF_RES_ADJ (Objective_Function_Residual_Adjsource.f90:17-40) of
// one shot: the modelled traces dmod become the adjoint source in place,
// part receives the per-receiver FP64 misfit terms, sh.resid (if given) the
// residual.
int shot_residual(sw_ctx *c, const sw_fwi_desc &d, int ntype, const sw_fwi_shot &sh, int nt,
                  float *dmod, std::vector<double> &part) {
  cudaStream_t s = c->stream;
  cudaError_t e;
  int st = SW_OK;
  void *p = nullptr;
  float *ddobs = nullptr, *dmute = nullptr, *dres = nullptr;
  if ((st = upload(c, "dobs", sh.dobs, (size_t)sh.nrec * nt * sizeof(float), &p))) return st;
  ddobs = (float *)p;
  if (sh.mute) {
    if ((st = upload(c, "mute", sh.mute, (size_t)sh.nrec * nt * sizeof(float), &p))) return st;
    dmute = (float *)p;
  }
  if (sh.resid) {
    dres = (float *)dbuf(c, "resid", (size_t)sh.nrec * nt * sizeof(float), &st);
    if (!dres) return st;
  }
  double *dpart = (double *)dbuf(c, "fpart", (size_t)sh.nrec * sizeof(double), &st);
  if (!dpart) return st;
  if (ntype == SW_NRM_L2) {
    if ((e = launch_residual(sh.nrec, nt, ddobs, dmute, dmod, dres, dpart, s)) != cudaSuccess)
      return cuda_fail(c, e, "residual");
    c->stats.launches_total++;
  } else {
    float *dmax = (float *)dbuf(c, "fmaxabs", (size_t)sh.nrec * sizeof(float), &st);
    if (!dmax) return st;
    if ((e = launch_residual_nrm(ntype, d.dat_thresh, sh.nrec, nt, ddobs, dmute, dmod, dres,
                                 dpart, dmax, s)) != cudaSuccess)
      return cuda_fail(c, e, "residual");
    c->stats.launches_total += (ntype != SW_NRM_L1 && d.dat_thresh == 0.f) ? 2 : 1;
  }
  part.resize(sh.nrec);
  if ((st = download(c, part.data(), dpart, (size_t)sh.nrec * sizeof(double)))) return st;
  if (sh.resid && (st = download(c, sh.resid, dres, (size_t)sh.nrec * nt * sizeof(float))))
    return st;
  return SW_OK;
}

constexpr int kFwiBatch = 16;   // shots per batch of the store-all gradient

// The store-all gradient (every snapshot of a shot in HBM) for several
// shots at a time: shots are admitted into a batch by device-memory
// footprint (like the RTM job), the batch's forward passes (AMOD_to_memory)
// run as one multi-shot propagation, then each shot's residual, then the
// backward passes with the AFWI imaging condition (AGRAD_to_memory) as one
// propagation, then the windowed images are added into the full grid in
// shot order (mod_copy_image).  Per shot the operations are those of the
// one-shot loop, so misfit and gradient equal it bit for bit.
int fct_gdt_batched(sw_ctx *c, const sw_fwi_desc &d, int ntype, const float *vel,
                    const float *dvel, const float *dwav, int nshot, const sw_fwi_shot *shots,
                    float *dgrad, float *dill, double &fsum, long long &ntotal) {
  cudaStream_t s = c->stream;
  cudaError_t e;
  int st = SW_OK;
  const sw_genpar &G = d.g;
  const int nt = G.nt;
  struct Info {
    Window w;
    sw_genpar g;
    size_t nw, nf;
    int ntsnap;
  };
  std::vector<Info> info(nshot);
  for (int is = 0; is < nshot; ++is) {
    const sw_fwi_shot &sh = shots[is];
    if (!sh.dobs) return fail(c, SW_BAD_PARAM, "shot %d without observed data", is);
    Info &I = info[is];
    if ((st = compute_window(c, G, d.aperture_x, d.aperture_y, sh.sou_coord, sh.nrec,
                             sh.rec_coord, I.w)))
      return st;
    I.g = G;
    I.g.nx = I.w.nxw;
    I.g.ny = I.w.nyw;
    I.g.ox = I.w.oxw;
    I.g.oy = I.w.oyw;
    I.nw = (size_t)I.g.nz * I.g.nx * I.g.ny;
    I.nf = (size_t)make_geom(I.g).total();
    I.ntsnap = nt / I.g.snapi;
  }
  auto r256 = [](size_t b) { return (b + 255) / 256 * 256; };
  auto arena_of = [&](int is) -> size_t {
    const Info &I = info[is];
    return r256(I.nw * 4) * 3 + r256(I.nf * 4) +
           r256(I.nw * (size_t)std::max(I.ntsnap, 1) * 4) + r256((size_t)shots[is].nrec * nt * 4);
  };
  std::vector<std::vector<float>> hv;
  std::vector<double> part;
  int next = 0;
  while (next < nshot) {
    size_t freeb = 0, totalb = 0;
    SW_CK(cudaMemGetInfo(&freeb, &totalb));
    size_t held = 0;
    auto it = c->bufs.find("fwi_arena");
    if (it != c->bufs.end()) held = it->second.cap;
    const double budget = (double)(freeb + held) * 0.85;
    int end = next;
    size_t need = 0, arena = 0;
    while (end < nshot && end - next < kFwiBatch) {
      const size_t a = arena_of(end), b = a + info[end].nf * 4 * 7;   // + run_phases fields
      if (end > next && (double)(need + b) > budget) break;
      need += b;
      arena += a;
      ++end;
    }
    if ((double)need > budget)
      return fail(c, SW_OOM_ADMISSION, "shot %d needs %zu bytes, budget %.0f", next, need, budget);
    char *cur = (char *)dbuf(c, "fwi_arena", arena, &st);
    if (!cur) return st;
    const int nb = end - next;
    std::vector<PhaseShot> fwd(nb), bwd(nb);
    std::vector<float *> rtr(nb), img(nb), ill(nb);
    hv.assign(nb, {});
    for (int q = 0; q < nb; ++q) {
      const int is = next + q;
      const Info &I = info[is];
      const sw_fwi_shot &sh = shots[is];
      float *vsmall = (float *)cur; cur += r256(I.nw * 4);
      float *vpad = (float *)cur; cur += r256(I.nf * 4);
      img[q] = (float *)cur; cur += r256(I.nw * 4);
      ill[q] = (float *)cur; cur += r256(I.nw * 4);
      float *wave = (float *)cur; cur += r256(I.nw * (size_t)std::max(I.ntsnap, 1) * 4);
      rtr[q] = (float *)cur; cur += r256((size_t)sh.nrec * nt * 4);
      // copy_window_vel_gath: window the model on the device, then pad.
      if ((e = launch_window_vel(G.nz, G.nx, G.ny, G.ox, G.oy, G.dx, G.dy, I.w.nxw, I.w.nyw,
                                 I.w.oxw, I.w.oyw, dvel, vsmall, s)) != cudaSuccess)
        return cuda_fail(c, e, "window vel");
      if ((e = launch_pad_velocity(make_geom(I.g), vsmall, vpad, s)) != cudaSuccess)
        return cuda_fail(c, e, "pad");
      c->stats.launches_total += 2;
      SW_CK(cudaMemsetAsync(rtr[q], 0, (size_t)sh.nrec * nt * 4, s));
      SW_CK(cudaMemsetAsync(wave, 0, I.nw * (size_t)std::max(I.ntsnap, 1) * 4, s));
      SW_CK(cudaMemsetAsync(img[q], 0, I.nw * 4, s));
      SW_CK(cudaMemsetAsync(ill[q], 0, I.nw * 4, s));
      window_host(G, I.w, vel, hv[q]);
      // AMOD_to_memory (to_disk_to_memory_AMOD.f90:27-82).
      PhaseShot &F = fwd[q];
      std::memset(&F.d, 0, sizeof(F.d));
      F.d.g = I.g;
      F.d.tmin = 1; F.d.tmax = nt; F.d.tstep = 1;
      F.d.fd_scheme = SW_FD_FORWARD;
      F.d.injection = SW_INJ_SINC;
      F.d.extraction = SW_EXT_SIMPLE_AFWI;
      F.d.extract_wave = 1;
      F.io.vel_pad = vpad;
      F.io.vel_phys_host = hv[q].data();
      F.io.nsou = 1;
      F.io.sou_coord = sh.sou_coord;
      F.io.sou_trace_dev = dwav;
      F.io.nrec = sh.nrec;
      F.io.rec_coord = sh.rec_coord;
      F.io.rec_trace_dev = rtr[q];
      F.io.wave_dev = wave;
      // AGRAD_to_memory (to_disk_to_memory_AGRAD.f90:27-79).
      PhaseShot &B = bwd[q];
      std::memset(&B.d, 0, sizeof(B.d));
      B.d.g = I.g;
      B.d.tmin = nt; B.d.tmax = 1; B.d.tstep = -1;
      B.d.fd_scheme = SW_FD_FORWARD;
      B.d.injection = SW_INJ_SIMPLE;
      B.d.imaging = SW_IMG_AFWI;
      B.io.vel_pad = vpad;
      B.io.vel_phys_host = hv[q].data();
      B.io.nsou = sh.nrec;
      B.io.sou_coord = sh.rec_coord;
      B.io.sou_trace_dev = rtr[q];
      B.io.wave_dev = wave;
      B.io.image_dev = img[q];
      B.io.illum_dev = ill[q];
    }
    if ((st = run_phases(c, fwd, c->run_opts))) return st;
    std::vector<std::vector<double>> parts(nb);
    for (int q = 0; q < nb; ++q)
      if ((st = shot_residual(c, d, ntype, shots[next + q], nt, rtr[q], parts[q]))) return st;
    if ((st = run_phases(c, bwd, c->run_opts))) return st;
    // mod_copy_image (ExtractPadModel.f90:662-697), shots in order.
    for (int q = 0; q < nb; ++q) {
      const Info &I = info[next + q];
      if ((e = launch_copy_image(G.nz, G.nx, G.ny, G.ox, G.oy, G.dx, G.dy, I.w.nxw, I.w.nyw,
                                 I.w.oxw, I.w.oyw, img[q], ill[q], dgrad, dill, s)) !=
          cudaSuccess)
        return cuda_fail(c, e, "copy image");
      c->stats.launches_total++;
      for (int r = 0; r < shots[next + q].nrec; ++r) fsum = fsum + parts[q][r];
      ntotal += shots[next + q].nrec;
    }
    SW_CK(cudaStreamSynchronize(s));
    next = end;
  }
  return SW_OK;
}

}  // namespace

int sw_fwi_fct_gdt(sw_ctx *c, const sw_fwi_desc *dp, const float *vel, const float *wavelet,
                   int nshot, const sw_fwi_shot *shots, const float *vpmask, double *f,
                   float *grad, float *illum) {
  if (!c || !dp || !vel || !wavelet || nshot < 1 || !shots || !f || !grad) return SW_BAD_PARAM;
  cudaSetDevice(c->device);
  const sw_fwi_desc &d = *dp;
  const sw_genpar &G = d.g;
  int st = check_genpar(c, G);
  if (st) return st;
  const int ntype = d.dat_nrm_type == 0 ? SW_NRM_L2 : d.dat_nrm_type;
  if (ntype != SW_NRM_L1 && ntype != SW_NRM_L2 && ntype != SW_NRM_HUBER &&
      ntype != SW_NRM_CAUCHY && ntype != SW_NRM_HYPERBOLIC)
    return fail(c, SW_BAD_PARAM, "dat_nrm_type %d is not a data norm", d.dat_nrm_type);
  cudaStream_t s = c->stream;
  cudaError_t e;
  const long long nfull = (long long)G.nz * G.nx * G.ny;
  const int nt = G.nt;
  void *p = nullptr;
  if ((st = upload(c, "fwi_vel", vel, nfull * sizeof(float), &p))) return st;
  const float *dvel = (const float *)p;
  if ((st = upload(c, "fwi_grad", nullptr, nfull * sizeof(float), &p))) return st;
  float *dgrad = (float *)p;
  if ((st = upload(c, "fwi_illum", nullptr, nfull * sizeof(float), &p))) return st;
  float *dill = (float *)p;
  if ((st = upload(c, "sou_tr", wavelet, (size_t)nt * sizeof(float), &p))) return st;
  const float *dwav = (const float *)p;

  double fsum = 0.0;
  long long ntotal = 0;
  std::vector<float> hv;
  std::vector<double> part;
  // Every snapshot in HBM: several shots per propagation.
  const bool batched = d.checkpoint_snaps <= 0 && nshot > 1;
  if (batched &&
      (st = fct_gdt_batched(c, d, ntype, vel, dvel, dwav, nshot, shots, dgrad, dill, fsum, ntotal)))
    return st;
  for (int is = 0; is < (batched ? 0 : nshot); ++is) {
    const sw_fwi_shot &sh = shots[is];
    Window w;
    if ((st = compute_window(c, G, d.aperture_x, d.aperture_y, sh.sou_coord, sh.nrec, sh.rec_coord, w)))
      return st;
    if (!sh.dobs) return fail(c, SW_BAD_PARAM, "shot %d without observed data", is);
    sw_genpar g = G;
    g.nx = w.nxw;
    g.ny = w.nyw;
    g.ox = w.oxw;
    g.oy = w.oyw;
    const Geom Gw = make_geom(g);
    const size_t nw = (size_t)g.nz * g.nx * g.ny;
    const int ntsnap = nt / g.snapi;
    // copy_window_vel_gath: window the model on the device, then pad.
    float *vsmall = (float *)dbuf(c, "vel_phys", nw * sizeof(float), &st);
    float *vpad = (float *)dbuf(c, "vel", (size_t)Gw.total() * sizeof(float), &st);
    if (!vsmall || !vpad) return st;
    if ((e = launch_window_vel(G.nz, G.nx, G.ny, G.ox, G.oy, G.dx, G.dy, w.nxw, w.nyw, w.oxw,
                               w.oyw, dvel, vsmall, s)) != cudaSuccess)
      return cuda_fail(c, e, "window vel");
    if ((e = launch_pad_velocity(Gw, vsmall, vpad, s)) != cudaSuccess) return cuda_fail(c, e, "pad");
    c->stats.launches_total += 2;
    // Host copy of the window velocity: the injection weights v^2 at the
    // source and receiver nodes are part of the injection plans.
    window_host(G, w, vel, hv);
    // AMOD_to_memory (to_disk_to_memory_AMOD.f90:27-82).
    DevIO a;
    a.vel_pad = vpad;
    a.vel_phys_host = hv.data();
    a.nsou = 1;
    a.sou_coord = sh.sou_coord;
    a.sou_trace_dev = dwav;
    a.nrec = sh.nrec;
    a.rec_coord = sh.rec_coord;
    if ((st = upload(c, "rec_tr", nullptr, (size_t)sh.nrec * nt * sizeof(float), &p))) return st;
    a.rec_trace_dev = (float *)p;
    sw_prop_desc fd;
    std::memset(&fd, 0, sizeof(fd));
    fd.g = g;
    fd.tmin = 1; fd.tmax = nt; fd.tstep = 1;
    fd.fd_scheme = SW_FD_FORWARD;
    fd.injection = SW_INJ_SINC;
    fd.extraction = SW_EXT_SIMPLE_AFWI;
    // Checkpointed snapshots: K snapshots per segment (K >= 2).
    const int K = d.checkpoint_snaps > 0 ? std::max(d.checkpoint_snaps, 2) : 0;
    const bool ckpt = K > 0 && ntsnap > K;
    const int nseg = ckpt ? (ntsnap + K - 1) / K : 1;
    // Binomial schedule: nslot state slots (+ one work slot) instead of one
    // per segment boundary; the forward runs happen inside the schedule.
    const int nslot = ckpt && d.revolve_slots > 0 ? std::min(d.revolve_slots, nseg - 1) : 0;
    const bool revolve = nslot > 0;
    const size_t nf = (size_t)Gw.total();
    float *dck = nullptr, *dseg = nullptr, *dadj = nullptr;
    if (!ckpt) {
      if ((st = upload(c, "wave", nullptr, nw * std::max(ntsnap, 1) * sizeof(float), &p))) return st;
      a.wave_dev = (float *)p;
      fd.extract_wave = 1;
      if ((st = propagate_dev(c, fd, a))) return st;
    } else if (revolve) {
      dck = (float *)dbuf(c, "fwi_ckpt", (size_t)(nslot + 1) * 4 * nf * sizeof(float), &st);
      dseg = (float *)dbuf(c, "fwi_seg", (size_t)(K + 2) * nw * sizeof(float), &st);
      dadj = (float *)dbuf(c, "fwi_adj_state", 4 * nf * sizeof(float), &st);
      if (!dck || !dseg || !dadj) return st;
    } else {
      // Forward in segments; the state after step (jK-1)*snapi, j = 1..nseg-1,
      // is kept as checkpoint j (4 padded fields).
      dck = (float *)dbuf(c, "fwi_ckpt", (size_t)(nseg - 1) * 4 * nf * sizeof(float), &st);
      dseg = (float *)dbuf(c, "fwi_seg", (size_t)(K + 2) * nw * sizeof(float), &st);
      dadj = (float *)dbuf(c, "fwi_adj_state", 4 * nf * sizeof(float), &st);
      if (!dck || !dseg || !dadj) return st;
      for (int j = 0; j < nseg; ++j) {
        fd.tmin = j == 0 ? 1 : (j * K - 1) * g.snapi + 1;
        fd.tmax = j == nseg - 1 ? nt : ((j + 1) * K - 1) * g.snapi;
        DevIO aj = a;
        aj.tcnt = 1;
        aj.init_state = j > 0 ? dck + (size_t)(j - 1) * 4 * nf : nullptr;
        aj.save_state = j < nseg - 1 ? dck + (size_t)j * 4 * nf : nullptr;
        if ((st = propagate_dev(c, fd, aj))) return st;
      }
      c->stats.ckpt_advances += (uint64_t)(nseg - 1);
    }
    // Compute_OF_RES_ADJ (Objective_Function_Residual_Adjsource.f90:17-40);
    // with the binomial schedule it runs once the first pass has reached
    // the end of the record.
    auto residual = [&]() -> int {
      return shot_residual(c, d, ntype, sh, nt, a.rec_trace_dev, part);
    };
    if (!revolve && (st = residual())) return st;
    // AGRAD_to_memory (to_disk_to_memory_AGRAD.f90:27-79).
    DevIO b;
    b.vel_pad = vpad;
    b.vel_phys_host = hv.data();
    b.nsou = sh.nrec;
    b.sou_coord = sh.rec_coord;
    b.sou_trace_dev = a.rec_trace_dev;
    b.wave_dev = a.wave_dev;
    if ((st = upload(c, "image", nullptr, nw * sizeof(float), &p))) return st;
    b.image_dev = (float *)p;
    if ((st = upload(c, "illum", nullptr, nw * sizeof(float), &p))) return st;
    b.illum_dev = (float *)p;
    sw_prop_desc bd;
    std::memset(&bd, 0, sizeof(bd));
    bd.g = g;
    bd.tmin = nt; bd.tmax = 1; bd.tstep = -1;
    bd.fd_scheme = SW_FD_FORWARD;
    bd.injection = SW_INJ_SIMPLE;
    bd.imaging = SW_IMG_AFWI;
    if (!ckpt) {
      if ((st = propagate_dev(c, bd, b))) return st;
    } else {
      // Segments from the last to the first: recompute snapshots
      // max(jK,1)..min((j+1)K+1, ntsnap) from checkpoint j into the segment
      // buffer (slot = snapshot - jK), then run the backward steps whose
      // imaging reads them; the adjoint state carries over between segments.
      // The wave pointer is offset so that the kernels' global snapshot
      // numbers land in the segment buffer.
      sw_prop_desc rd = fd;
      rd.extract_wave = 1;
      // The forward steps already run (their data are extracted once).
      int frontier = 0;
      // Segment j: recompute its K + 2 snapshots from its first state, then
      // the backward steps whose imaging reads them.
      auto segment = [&](int j, const float *state) -> int {
        float *wbase = dseg - (ptrdiff_t)(j * K - 1) * (ptrdiff_t)nw;
        rd.tmin = j == 0 ? 1 : (j * K - 1) * g.snapi + 1;
        rd.tmax = std::min(((j + 1) * K + 1) * g.snapi, nt);
        const bool first = revolve && rd.tmin == frontier + 1;
        DevIO rj = a;
        rd.extraction = first ? fd.extraction : SW_EXT_NONE;
        if (!first) {
          rj.nrec = 0;
          rj.rec_trace_dev = nullptr;
        }
        rj.wave_dev = wbase;
        rj.tcnt = 1;
        rj.init_state = state;
        int q;
        if ((q = propagate_dev(c, rd, rj))) return q;
        frontier = std::max(frontier, rd.tmax);
        if (first && (q = residual())) return q;
        bd.tmin = j == nseg - 1 ? nt : (j + 1) * K * g.snapi;
        bd.tmax = j == 0 ? 1 : j * K * g.snapi + 1;
        DevIO bj = b;
        bj.wave_dev = wbase;
        bj.tcnt = nt;
        bj.init_state = j == nseg - 1 ? nullptr : dadj;
        bj.save_state = j > 0 ? dadj : nullptr;
        return propagate_dev(c, bd, bj);
      };
      if (!revolve) {
        for (int j = nseg - 1; j >= 0; --j)
          if ((st = segment(j, j > 0 ? dck + (size_t)(j - 1) * 4 * nf : nullptr))) return st;
      } else {
        std::vector<int> freel(nslot);
        for (int q = 0; q < nslot; ++q) freel[q] = q;
        std::vector<CkOp> ops;
        revolve_schedule(0, nseg, -1, freel, nslot, ops);
        auto slot = [&](int q) { return q < 0 ? nullptr : dck + (size_t)q * 4 * nf; };
        for (const CkOp &op : ops) {
          if (op.process) {
            if ((st = segment(op.a, slot(op.src)))) return st;
            continue;
          }
          // Advance S_a -> S_b (the state after step (bK - 1) snapi); the
          // first pass over these steps extracts the data.
          fd.tmin = op.a == 0 ? 1 : (op.a * K - 1) * g.snapi + 1;
          fd.tmax = (op.b * K - 1) * g.snapi;
          const bool first = fd.tmin == frontier + 1;
          if (!first && fd.tmax > frontier)
            return fail(c, SW_BAD_PARAM, "checkpoint schedule runs past the first pass");
          DevIO aj = a;
          sw_prop_desc fa = fd;
          if (!first) {
            fa.extraction = SW_EXT_NONE;
            aj.nrec = 0;
            aj.rec_trace_dev = nullptr;
          }
          aj.tcnt = 1;
          aj.init_state = slot(op.src);
          aj.save_state = slot(op.dst);
          if ((st = propagate_dev(c, fa, aj))) return st;
          frontier = std::max(frontier, fd.tmax);
          c->stats.ckpt_advances += (uint64_t)(op.b - op.a);
        }
      }
    }
    // mod_copy_image (ExtractPadModel.f90:662-697), shots in order.
    if ((e = launch_copy_image(G.nz, G.nx, G.ny, G.ox, G.oy, G.dx, G.dy, w.nxw, w.nyw, w.oxw,
                               w.oyw, b.image_dev, b.illum_dev, dgrad, dill, s)) != cudaSuccess)
      return cuda_fail(c, e, "copy image");
    c->stats.launches_total++;
    cudaStreamSynchronize(s);
    for (int r = 0; r < sh.nrec; ++r) fsum = fsum + part[r];
    ntotal += sh.nrec;
  }
  // Post-processing (compute_function_gradient.f90:314-343).
  if (d.illu_pow != 1.f) {
    k_illu_pow<<<gsz(nfull), 256, 0, s>>>(nfull, d.illu_pow, dill);
    c->stats.launches_total++;
  }
  const double scaling = (double)(2LL * nt * ntotal);
  float *pmax = (float *)dbuf(c, "red_pmax", kRedBlocks * sizeof(float), &st);
  double *psum = (double *)dbuf(c, "red_psum", kRedBlocks * sizeof(double), &st);
  float *maxil = (float *)dbuf(c, "red_maxil", sizeof(float), &st);
  double *rmsil = (double *)dbuf(c, "red_rmsil", sizeof(double), &st);
  if (!pmax || !psum || !maxil || !rmsil) return st;
  k_grad_scale_stats<<<kRedBlocks, kRedThreads, 0, s>>>(nfull, (float)scaling, dgrad, dill, pmax,
                                                       psum);
  k_final_stats<<<1, 32, 0, s>>>(kRedBlocks, nfull, pmax, psum, maxil, rmsil);
  float *dmask = nullptr;
  if (vpmask) {
    if ((st = upload(c, "vpmask", vpmask, nfull * sizeof(float), &p))) return st;
    dmask = (float *)p;
  }
  k_normalise<<<gsz(nfull), 256, 0, s>>>(nfull, maxil, rmsil, dill, dgrad, dmask);
  c->stats.launches_total += 3;
  // triangle2 (Smoothing.f90:87-138); y pass with rect3/n3 (see the oracle).
  const int n1 = G.nz, n2 = G.nx, n3 = G.ny;
  float *tmpb = (float *)dbuf(c, "tri_out", nfull * sizeof(float), &st);
  if (!tmpb) return st;
  auto tri = [&](int n12, int nr, int nlines, int inner, long long ls_in, long long ls_out,
                 long long es) -> int {
    if (nr < 1 || nr > n12) return fail(c, SW_BAD_PARAM, "triangle radius %d out of range", nr);
    const size_t per = 4ull * (size_t)(n12 + 2 * nr);
    float *scr = (float *)dbuf(c, "tri_scr", per * (size_t)nlines * sizeof(float), &st);
    if (!scr) return st;
    k_triangle<<<(nlines + 127) / 128, 128, 0, s>>>(n12, nr, nlines, inner, ls_in, ls_out, es,
                                                    dgrad, tmpb, scr);
    cudaError_t ee = cudaMemcpyAsync(dgrad, tmpb, nfull * sizeof(float), cudaMemcpyDeviceToDevice, s);
    c->stats.launches_total++;
    return ee == cudaSuccess ? SW_OK : cuda_fail(c, ee, "triangle");
  };
  if (d.smooth_dox && (st = tri(n2, d.smooth_rect2, n1 * n3, n1, 1, (long long)n1 * n2, n1))) return st;
  if (d.smooth_doz && (st = tri(n1, d.smooth_rect1, n2 * n3, n2, n1, (long long)n1 * n2, 1))) return st;
  if (d.smooth_doy && n3 > 1 &&
      (st = tri(n3, d.smooth_rect3, n1 * n2, n1, 1, n1, (long long)n1 * n2)))
    return st;
  k_mask<<<gsz(nfull), 256, 0, s>>>(nfull, dgrad, dmask);
  c->stats.launches_total++;
  if ((st = download(c, grad, dgrad, nfull * sizeof(float)))) return st;
  if (illum && (st = download(c, illum, dill, nfull * sizeof(float)))) return st;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(c, e, "fwi");
  *f = fsum / scaling;
  // A NaN or Inf anywhere (data, model, an unstable propagation) reaches
  // the FP64 misfit or the gradient; report it instead of returning it.
  if (!std::isfinite(*f)) return fail(c, SW_NUMERIC, "misfit is not finite (%g)", *f);
  for (long long q = 0; q < nfull; ++q)
    if (!std::isfinite(grad[q]))
      return fail(c, SW_NUMERIC, "gradient is not finite at model index %lld", q);
  return SW_OK;
}

// ---------------------------------------------------------------------------
// L-BFGS (libs/libinv/lbfgs.f) with device-resident FP64 vectors
// ---------------------------------------------------------------------------
struct sw_lbfgs {
  sw_ctx *c;
  int n, m;
  double xmin, xmax;
  int boundt, type;
  float *mask = nullptr;     // device
  double *xinit = nullptr;   // device
  double *S = nullptr;       // m search steps, n each
  double *Y = nullptr;       // m gradient differences
  double *w0 = nullptr;      // W(1..N)
  double *wa = nullptr;      // DIAG used as MCSRCH work array
  double *x = nullptr, *g = nullptr;
  double *part = nullptr, *res = nullptr;
  std::vector<double> rho, alpha;   // W(N+1..N+M), W(N+M+1..N+2M)
  // libs/libnlinv's variant (LBFGSOC / LBFGSOLD): per-parameter bounds
  // (device arrays of nparam values), the first-step options and its
  // line-search constants.
  bool oc = false;
  int nparam = 1;
  double *pmin = nullptr, *pmax = nullptr;
  int stp1_opt = 1;
  double step_init = 999999.0;
  // LBFGS SAVE state
  int iter = 0, nfun = 0, point = 0, npt = 0, bound = 0, info = 0, nfev = 0, maxfev = 20, cp = 0;
  double stp = 0, stp1 = 0, ftol = 1e-4, gnorm = 0, xnorm = 0, ys = 0, yy = 0, diag = 1.0;
  bool finish = false;
  // MCSRCH SAVE state
  int infoc = 0;
  bool brackt = false, stage1 = true;
  double dg = 0, dgm = 0, dginit = 0, dgtest = 0, dgx = 0, dgxm = 0, dgy = 0, dgym = 0, finit = 0,
         ftest1 = 0, fm = 0, fx = 0, fxm = 0, fy = 0, fym = 0, stx = 0, sty = 0, stmin = 0,
         stmax = 0, width = 0, width1 = 0;
};

namespace {
const double kGTOL = 0.9, kSTPMIN = 1.0e-20, kSTPMAX = 1.0e+20;

double ddot(sw_lbfgs &L, const double *a, const double *b) {
  cudaStream_t s = L.c->stream;
  k_dot_partial<<<kRedBlocks, kRedThreads, 0, s>>>(L.n, a, b, L.part);
  k_sum_partials<<<1, 32, 0, s>>>(kRedBlocks, L.part, L.res);
  L.c->stats.launches_total += 2;
  double h = 0.0;
  cudaMemcpyAsync(&h, L.res, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  return h;
}

void freeze(sw_lbfgs &L, double *x) {
  if (L.oc)
    k_freeze_blocks<<<gsz(L.n), 256, 0, L.c->stream>>>(L.n, L.n / L.nparam, L.pmin, L.pmax, x);
  else
    k_freeze<<<gsz(L.n), 256, 0, L.c->stream>>>(L.n, L.type, L.xmin, L.xmax, L.mask, L.xinit, x);
  L.c->stats.launches_total++;
}

// MCSTEP (lbfgs.f:985-1210); identical scalar code to the oracle.
void mcstep(double &stx, double &fx, double &dx, double &sty, double &fy, double &dy, double &stp,
            double fp, double dp, bool &brackt, double stpmin, double stpmax, int &info) {
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
    stpf = (std::fabs(stpc - stx) < std::fabs(stpq - stx)) ? stpc : stpc + (stpq - stpc) / 2;
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
    stpf = (std::fabs(stpc - stp) > std::fabs(stpq - stp)) ? stpc : stpq;
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
    if (r < 0.0 && gamma != 0.0) stpc = stp + r * (stx - stp);
    else if (stp > stx) stpc = stpmax;
    else stpc = stpmin;
    stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (brackt) stpf = (std::fabs(stp - stpc) < std::fabs(stp - stpq)) ? stpc : stpq;
    else stpf = (std::fabs(stp - stpc) > std::fabs(stp - stpq)) ? stpc : stpq;
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
  const double p66s = (double)0.66f;  // REAL literal in the F77 source
  if (brackt && bound) {
    if (sty > stx) stp = std::min(stx + p66s * (sty - stx), stp);
    else stp = std::max(stx + p66s * (sty - stx), stp);
  }
}

// MCSRCH (lbfgs.f:652-982) with device vectors.
void mcsrch(sw_lbfgs &L, double f, const double *s, double xtol) {
  // XTRAPF is 4.0D1 in libinv's MCSRCH (lbfgs.f:792) and 4.0D0 in libnlinv's
  // MCSRCHOC / MCSRCHOLD (nlinv_lbfgs.f:752,1773).
  const double p5 = 0.5, p66 = 0.66, xtrapf = L.oc ? 4.0 : 40.0, zero = 0.0;
  cudaStream_t st = L.c->stream;
  if (L.info == -1) goto L45;
  L.infoc = 1;
  if (L.n <= 0 || L.stp <= zero || L.ftol < zero || xtol < zero || L.maxfev <= 0) return;
  L.dginit = ddot(L, L.g, s);
  if (L.dginit >= zero) return;
  L.brackt = false;
  L.stage1 = true;
  L.nfev = 0;
  L.finit = f;
  L.dgtest = L.ftol * L.dginit;
  L.width = kSTPMAX - kSTPMIN;
  L.width1 = L.width / p5;
  cudaMemcpyAsync(L.wa, L.x, (size_t)L.n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  L.stx = zero; L.fx = L.finit; L.dgx = L.dginit;
  L.sty = zero; L.fy = L.finit; L.dgy = L.dginit;
L30:
  if (L.brackt) {
    L.stmin = std::min(L.stx, L.sty);
    L.stmax = std::max(L.stx, L.sty);
  } else {
    L.stmin = L.stx;
    L.stmax = L.stp + xtrapf * (L.stp - L.stx);
  }
  L.stp = std::max(L.stp, kSTPMIN);
  L.stp = std::min(L.stp, kSTPMAX);
  if ((L.brackt && (L.stp <= L.stmin || L.stp >= L.stmax)) || L.nfev >= L.maxfev - 1 ||
      L.infoc == 0 || (L.brackt && L.stmax - L.stmin <= xtol * L.stmax))
    L.stp = L.stx;
  k_step_x<<<gsz(L.n), 256, 0, st>>>(L.n, L.wa, L.stp, s, L.x);
  L.c->stats.launches_total++;
  if (L.boundt == 1) freeze(L, L.x);
  L.info = -1;
  return;
L45:
  L.info = 0;
  L.nfev = L.nfev + 1;
  L.dg = ddot(L, L.g, s);
  L.ftest1 = L.finit + L.stp * L.dgtest;
  if ((L.brackt && (L.stp <= L.stmin || L.stp >= L.stmax)) || L.infoc == 0) L.info = 6;
  if (L.stp == kSTPMAX && f <= L.ftest1 && L.dg <= L.dgtest) L.info = 5;
  if (L.stp == kSTPMIN && (f > L.ftest1 || L.dg >= L.dgtest)) L.info = 4;
  if (L.nfev >= L.maxfev) L.info = 3;
  if (L.brackt && L.stmax - L.stmin <= xtol * L.stmax) L.info = 2;
  if (f <= L.ftest1 && std::fabs(L.dg) <= kGTOL * (-L.dginit)) L.info = 1;
  if (L.info != 0) return;
  if (L.stage1 && f <= L.ftest1 && L.dg >= std::min(L.ftol, kGTOL) * L.dginit) L.stage1 = false;
  if (L.stage1 && f <= L.fx && f > L.ftest1) {
    L.fm = f - L.stp * L.dgtest;
    L.fxm = L.fx - L.stx * L.dgtest;
    L.fym = L.fy - L.sty * L.dgtest;
    L.dgm = L.dg - L.dgtest;
    L.dgxm = L.dgx - L.dgtest;
    L.dgym = L.dgy - L.dgtest;
    mcstep(L.stx, L.fxm, L.dgxm, L.sty, L.fym, L.dgym, L.stp, L.fm, L.dgm, L.brackt, L.stmin,
           L.stmax, L.infoc);
    L.fx = L.fxm + L.stx * L.dgtest;
    L.fy = L.fym + L.sty * L.dgtest;
    L.dgx = L.dgxm + L.dgtest;
    L.dgy = L.dgym + L.dgtest;
  } else {
    mcstep(L.stx, L.fx, L.dgx, L.sty, L.fy, L.dgy, L.stp, f, L.dg, L.brackt, L.stmin, L.stmax,
           L.infoc);
  }
  if (L.brackt) {
    if (std::fabs(L.sty - L.stx) >= p66 * L.width1) L.stp = L.stx + p5 * (L.sty - L.stx);
    L.width1 = L.width;
    L.width = std::fabs(L.sty - L.stx);
  }
  goto L30;
}

void free_lbfgs(sw_lbfgs *L) {
  for (void *q : {(void *)L->mask, (void *)L->xinit, (void *)L->S, (void *)L->Y, (void *)L->w0,
                  (void *)L->wa, (void *)L->x, (void *)L->g, (void *)L->part, (void *)L->res,
                  (void *)L->pmin, (void *)L->pmax})
    if (q) cudaFree(q);
}

}  // namespace

int sw_lbfgs_create(sw_ctx *c, int n, int m, double xmin, double xmax, const float *mask,
                    int bound_type, int freeze_soft, const double *xinit, sw_lbfgs **out) {
  if (!c || n <= 0 || m <= 0 || !out || !mask || !xinit) return SW_BAD_PARAM;
  cudaSetDevice(c->device);
  sw_lbfgs *L = new sw_lbfgs();
  L->c = c;
  L->n = n;
  L->m = m;
  L->xmin = xmin;
  L->xmax = xmax;
  L->boundt = bound_type;
  L->type = freeze_soft != 0;
  L->rho.assign(m + 1, 0.0);
  L->alpha.assign(m + 1, 0.0);
  const size_t nb = (size_t)n * sizeof(double);
  bool ok = cudaMalloc(&L->mask, (size_t)n * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&L->xinit, nb) == cudaSuccess &&
            cudaMalloc(&L->S, nb * m) == cudaSuccess && cudaMalloc(&L->Y, nb * m) == cudaSuccess &&
            cudaMalloc(&L->w0, nb) == cudaSuccess && cudaMalloc(&L->wa, nb) == cudaSuccess &&
            cudaMalloc(&L->x, nb) == cudaSuccess && cudaMalloc(&L->g, nb) == cudaSuccess &&
            cudaMalloc(&L->part, kRedBlocks * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&L->res, sizeof(double)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    free_lbfgs(L);
    delete L;
    return fail(c, SW_OOM_ADMISSION, "L-BFGS state of n=%d m=%d does not fit", n, m);
  }
  cudaMemcpy(L->mask, mask, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(L->xinit, xinit, nb, cudaMemcpyHostToDevice);
  cudaMemset(L->S, 0, nb * m);
  cudaMemset(L->Y, 0, nb * m);
  *out = L;
  return SW_OK;
}

int sw_lbfgs_destroy(sw_lbfgs *L) {
  if (!L) return SW_OK;
  cudaSetDevice(L->c->device);
  cudaStreamSynchronize(L->c->stream);
  free_lbfgs(L);
  delete L;
  return SW_OK;
}

int sw_lbfgs_diag(const sw_lbfgs *L, double *o) {
  if (!L || !o) return SW_BAD_PARAM;
  o[0] = L->iter; o[1] = L->nfun; o[2] = L->stp; o[3] = L->gnorm;
  o[4] = L->ys; o[5] = L->yy; o[6] = L->dginit; o[7] = L->dg;
  return SW_OK;
}

// LBFGS (lbfgs.f:49-558) with DIAGCO = .false.
int sw_lbfgs_step(sw_lbfgs *Lp, double *xh, double f, const double *gh, double eps, double xtol,
                  int *iflag, int *myinfo) {
  if (!Lp || !xh || !gh || !iflag || !myinfo) return SW_BAD_PARAM;
  sw_lbfgs &L = *Lp;
  sw_ctx *c = L.c;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int n = L.n, m = L.m;
  const size_t nb = (size_t)n * sizeof(double);
  cudaMemcpyAsync(L.x, xh, nb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(L.g, gh, nb, cudaMemcpyHostToDevice, s);
  double *Sv = nullptr;
  if (*iflag == 0) goto L10;
  if (*iflag == 1) goto L172;
  if (*iflag == 2) goto L100;
  return fail(c, SW_BAD_PARAM, "iflag must be 0, 1 or 2");
L10:
  L.iter = 0;
  L.nfun = 1;
  L.point = 0;
  L.finish = false;
  L.diag = 1.0;
  k_negmul<<<gsz(n), 256, 0, s>>>(n, L.g, L.diag, L.S);  // W(ISPT+I) = -G(I)*DIAG(I)
  c->stats.launches_total++;
  L.gnorm = std::sqrt(ddot(L, L.g, L.g));
  if (L.oc) {
    // nlinv_lbfgs.f:333-341 (LBFGSOLD, :1366-1370: step_init or 1/|g|).
    L.stp1 = L.stp1_opt == 1 ? std::sqrt(ddot(L, L.x, L.x)) / L.gnorm / 100 : 1.0 / L.gnorm;
    if (L.step_init != 999999.0) L.stp1 = L.step_init;
  } else {
    const double xnorm2 = std::sqrt(ddot(L, L.x, L.x));
    L.stp1 = (L.boundt == 0) ? 1.0 / L.gnorm : xnorm2 / L.gnorm / 100;
  }
  L.ftol = 1.0e-4;
  L.maxfev = 20;
L80:
  L.iter = L.iter + 1;
  L.info = 0;
  L.bound = L.iter - 1;
  if (L.iter == 1) goto L165;
  if (L.iter > m) L.bound = m;
  L.ys = ddot(L, L.Y + L.npt, L.S + L.npt);
  L.yy = ddot(L, L.Y + L.npt, L.Y + L.npt);
  L.diag = L.ys / L.yy;
L100:
  L.cp = L.point;
  if (L.point == 0) L.cp = m;
  L.rho[L.cp] = 1.0 / L.ys;   // W(N+CP)
  k_negmul<<<gsz(n), 256, 0, s>>>(n, L.g, 1.0, L.w0);   // W(I) = -G(I)
  c->stats.launches_total++;
  L.cp = L.point;
  for (int i = 1; i <= L.bound; ++i) {
    L.cp = L.cp - 1;
    if (L.cp == -1) L.cp = m - 1;
    const double sq = ddot(L, L.S + (size_t)L.cp * n, L.w0);
    L.alpha[L.cp + 1] = L.rho[L.cp + 1] * sq;   // W(INMC) = W(N+CP+1)*SQ
    k_aymx<<<gsz(n), 256, 0, s>>>(n, L.alpha[L.cp + 1], L.Y + (size_t)L.cp * n, L.w0);
    c->stats.launches_total++;
  }
  k_scal<<<gsz(n), 256, 0, s>>>(n, L.diag, L.w0);   // W(I) = DIAG(I)*W(I)
  c->stats.launches_total++;
  for (int i = 1; i <= L.bound; ++i) {
    const double yr = ddot(L, L.Y + (size_t)L.cp * n, L.w0);
    double beta = L.rho[L.cp + 1] * yr;
    beta = L.alpha[L.cp + 1] - beta;
    k_axpy<<<gsz(n), 256, 0, s>>>(n, beta, L.S + (size_t)L.cp * n, L.w0);
    c->stats.launches_total++;
    L.cp = L.cp + 1;
    if (L.cp == m) L.cp = 0;
  }
  cudaMemcpyAsync(L.S + (size_t)L.point * n, L.w0, nb, cudaMemcpyDeviceToDevice, s);
L165:
  L.nfev = 0;
  L.stp = 1.0;
  if (L.iter == 1) L.stp = L.stp1;
  cudaMemcpyAsync(L.w0, L.g, nb, cudaMemcpyDeviceToDevice, s);   // W(I) = G(I)
L172:
  Sv = L.S + (size_t)L.point * n;
  mcsrch(L, f, Sv, xtol);
  if (L.info == -1) {
    *iflag = 1;
    cudaMemcpyAsync(xh, L.x, nb, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return SW_OK;
  }
  if (L.info != 1) {
    *iflag = -1;
    cudaStreamSynchronize(s);
    return SW_OK;
  }
  L.nfun = L.nfun + L.nfev;
  *myinfo = L.info;
  if (L.boundt == 2 && L.info == 1) freeze(L, L.x);
  L.npt = L.point * n;
  k_scal<<<gsz(n), 256, 0, s>>>(n, L.stp, L.S + L.npt);            // S = STP*S
  k_sub<<<gsz(n), 256, 0, s>>>(n, L.g, L.w0, L.Y + L.npt);         // Y = G - W
  c->stats.launches_total += 2;
  L.point = L.point + 1;
  if (L.point == m) L.point = 0;
  L.gnorm = std::sqrt(ddot(L, L.g, L.g));
  L.xnorm = std::sqrt(ddot(L, L.x, L.x));
  L.xnorm = std::max(1.0, L.xnorm);
  if (L.gnorm / L.xnorm <= eps) L.finish = true;
  if (L.finish) {
    *iflag = 0;
    cudaMemcpyAsync(xh, L.x, nb, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return SW_OK;
  }
  goto L80;
}

// One LBFGSOC / LBFGSOLD call (libs/libnlinv/nlinv_lbfgs.f:31-613,
// 1066-1636): the saved state comes in from the caller's arrays, the
// vectors run on the device, and the state goes back out in the
// reference's layout.
int sw_lbfgs_oc_step(sw_ctx *c, const sw_lbfgs_oc_desc *d, double *xh, double f,
                     const double *gh, double *w, double *diag, sw_lbfgs_oc_state *st,
                     int *iflag, int *myinfo) {
  if (!c || !d || !xh || !gh || !w || !diag || !st || !iflag || !myinfo) return SW_BAD_PARAM;
  if (d->n <= 0 || d->m <= 0 || d->nparam <= 0 || d->n % d->nparam != 0)
    return fail(c, SW_BAD_PARAM, "L-BFGS: n=%d m=%d nparam=%d", d->n, d->m, d->nparam);
  if (d->lbfgs_type == 1 && (!d->xmin || !d->xmax))
    return fail(c, SW_BAD_PARAM, "L-BFGS: bounds missing");
  cudaSetDevice(c->device);
  const int n = d->n, m = d->m;
  sw_lbfgs *L = new sw_lbfgs();
  L->c = c;
  L->n = n;
  L->m = m;
  L->oc = true;
  L->nparam = d->nparam;
  L->boundt = d->lbfgs_type == 1 ? d->bound_type : 0;
  L->stp1_opt = d->lbfgs_type == 1 ? d->stp1_opt : 0;
  L->step_init = d->step_init;
  L->rho.assign(m + 1, 0.0);
  L->alpha.assign(m + 1, 0.0);
  const size_t nb = (size_t)n * sizeof(double);
  const int np = d->nparam;
  bool ok = cudaMalloc(&L->S, nb * m) == cudaSuccess && cudaMalloc(&L->Y, nb * m) == cudaSuccess &&
            cudaMalloc(&L->w0, nb) == cudaSuccess && cudaMalloc(&L->wa, nb) == cudaSuccess &&
            cudaMalloc(&L->x, nb) == cudaSuccess && cudaMalloc(&L->g, nb) == cudaSuccess &&
            cudaMalloc(&L->part, kRedBlocks * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&L->res, sizeof(double)) == cudaSuccess &&
            cudaMalloc(&L->pmin, np * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&L->pmax, np * sizeof(double)) == cudaSuccess;
  auto done = [&](int rc) {
    cudaStreamSynchronize(c->stream);
    free_lbfgs(L);
    delete L;
    return rc;
  };
  if (!ok) {
    cudaGetLastError();
    return done(fail(c, SW_OOM_ADMISSION, "L-BFGS state of n=%d m=%d does not fit", n, m));
  }
  cudaStream_t s = c->stream;
  const std::vector<double> zeros(np, 0.0);
  cudaMemcpyAsync(L->pmin, d->lbfgs_type == 1 ? d->xmin : zeros.data(), np * sizeof(double),
                  cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(L->pmax, d->lbfgs_type == 1 ? d->xmax : zeros.data(), np * sizeof(double),
                  cudaMemcpyHostToDevice, s);
  // W: [0, n) the gradient / work vector, [n, n+m) rho, [n+m, n+2m) alpha,
  // then the m search steps and the m gradient differences of n values.
  const size_t ispt = (size_t)n + 2 * m, iypt = ispt + (size_t)n * m;
  if (*iflag != 0) {
    cudaMemcpyAsync(L->w0, w, nb, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(L->S, w + ispt, nb * m, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(L->Y, w + iypt, nb * m, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(L->wa, diag, nb, cudaMemcpyHostToDevice, s);
    for (int q = 1; q <= m; ++q) {
      L->rho[q] = w[n + q - 1];
      L->alpha[q] = w[n + m + q - 1];
    }
    L->gnorm = st->gnorm; L->stp1 = st->stp1; L->ftol = st->ftol; L->stp = st->stp;
    L->ys = st->ys; L->yy = st->yy; L->xnorm = st->xnorm;
    L->iter = st->iter; L->nfun = st->nfun; L->point = st->point; L->maxfev = st->maxfev;
    L->info = st->info; L->bound = st->bound; L->npt = st->npt; L->cp = st->cp;
    L->nfev = st->nfev; L->finish = st->finish != 0;
    L->infoc = st->infoc; L->brackt = st->brackt != 0; L->stage1 = st->stage1 != 0;
    L->dg = st->dg; L->dgm = st->dgm; L->dginit = st->dginit; L->dgtest = st->dgtest;
    L->dgx = st->dgx; L->dgxm = st->dgxm; L->dgy = st->dgy; L->dgym = st->dgym;
    L->finit = st->finit; L->ftest1 = st->ftest1; L->fm = st->fm; L->fx = st->fx;
    L->fxm = st->fxm; L->fy = st->fy; L->fym = st->fym; L->stx = st->stx; L->sty = st->sty;
    L->stmin = st->stmin; L->stmax = st->stmax; L->width = st->width; L->width1 = st->width1;
  } else {
    cudaMemsetAsync(L->S, 0, nb * m, s);
    cudaMemsetAsync(L->Y, 0, nb * m, s);
  }
  int rc = sw_lbfgs_step(L, xh, f, gh, d->eps, d->xtol, iflag, myinfo);
  if (rc != SW_OK) return done(rc);
  cudaMemcpyAsync(w, L->w0, nb, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(w + ispt, L->S, nb * m, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(w + iypt, L->Y, nb * m, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(diag, L->wa, nb, cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return done(cuda_fail(c, e, "L-BFGS state"));
  for (int q = 1; q <= m; ++q) {
    w[n + q - 1] = L->rho[q];
    w[n + m + q - 1] = L->alpha[q];
  }
  std::memset(st, 0, sizeof(*st));
  st->gtol = kGTOL; st->one = 1.0; st->zero = 0.0; st->gnorm = L->gnorm; st->stp1 = L->stp1;
  st->ftol = L->ftol; st->stpmin = kSTPMIN; st->stpmax = kSTPMAX; st->stp = L->stp;
  st->ys = L->ys; st->yy = L->yy; st->xnorm = L->xnorm;
  st->mp = 6; st->lp = 6; st->iter = L->iter; st->nfun = L->nfun; st->point = L->point;
  st->ispt = (int)ispt; st->iypt = (int)iypt; st->maxfev = L->maxfev; st->info = L->info;
  st->bound = L->bound; st->npt = L->npt; st->cp = L->cp; st->nfev = L->nfev;
  st->finish = L->finish ? 1 : 0;
  st->infoc = L->infoc; st->brackt = L->brackt ? 1 : 0; st->stage1 = L->stage1 ? 1 : 0;
  st->dg = L->dg; st->dgm = L->dgm; st->dginit = L->dginit; st->dgtest = L->dgtest;
  st->dgx = L->dgx; st->dgxm = L->dgxm; st->dgy = L->dgy; st->dgym = L->dgym;
  st->finit = L->finit; st->ftest1 = L->ftest1; st->fm = L->fm; st->fx = L->fx;
  st->fxm = L->fxm; st->fy = L->fy; st->fym = L->fym; st->stx = L->stx; st->sty = L->sty;
  st->stmin = L->stmin; st->stmax = L->stmax; st->width = L->width; st->width1 = L->width1;
  return done(SW_OK);
}
