// regularize.cu - the model regularisation of 2DAFWI on the device:
// compute_fct_gdt_reg (progs/afwi/compute_function_gradient.f90:98-206)
// with SparseRegularization_apply / LogisticRegularization_apply
// (libs/libwave/Sparse_regularization.f90:223-397).
//
// Every pass pads the model by edge replication, applies the helix filter
// 1 - Z^lag (helicon_mod_lop, libs/libflt/helicon.f90:25-60, one
// coefficient -1) over the padded array as one line, weights and masks the
// differences, takes the norm of the interior (one block, FP32 or FP64 sum
// in sample order like the reference's sum()), applies gdt_compute,
// weights again, applies the adjoint filter and adds the interior to the
// pass's gradient.  All element-wise steps are one thread per sample with
// the reference's operation order (the library is built with
// --fmad=false), so the result is the reference's to the bit except the
// FP32 log of the Cauchy norm.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/swave.h"
#include "engine.h"
#include "norms.cuh"
#include "swave_dev.cuh"

using namespace swave;

namespace {

struct RegDims {
  int nz, nx, ny, tz, tx, ty;
  long long nzt, nxt, nyt, ntap, n;
};

inline int grid_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}

#define GRID_STRIDE(q, n)                                                      \
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (n); \
       q += (long long)gridDim.x * blockDim.x)

// SparseRegularization_add_taper, forw (Sparse_regularization.f90:399-437):
// the clamped index on every axis.
__global__ void k_reg_pad(RegDims R, const float *__restrict__ a, float *__restrict__ tap) {
  GRID_STRIDE(q, R.ntap) {
    const long long i = q % R.nzt, j = (q / R.nzt) % R.nxt, k = q / (R.nzt * R.nxt);
    const long long iz = min(max(i - R.tz, 0LL), (long long)R.nz - 1);
    const long long ix = min(max(j - R.tx, 0LL), (long long)R.nx - 1);
    const long long iy = min(max(k - R.ty, 0LL), (long long)R.ny - 1);
    tap[q] = a[iz + R.nz * (ix + R.nx * iy)];
  }
}

// helicon_mod_lop forward: y = 0, y += x (zero lag), y[i] += x[i-lag] * -1.
__global__ void k_helix_fwd(long long n, long long lag, const float *__restrict__ x,
                            float *__restrict__ y) {
  GRID_STRIDE(q, n) {
    float v = 0.0f + x[q];
    if (q >= lag) v = v + x[q - lag] * -1.0f;
    y[q] = v;
  }
}

// helicon_mod_lop adjoint: x = 0, x += y (zero lag), x[i] += y[i+lag] * -1.
__global__ void k_helix_adj(long long n, long long lag, const float *__restrict__ y,
                            float *__restrict__ x) {
  GRID_STRIDE(q, n) {
    float v = 0.0f + y[q];
    if (q + lag < n) v = v + y[q + lag] * -1.0f;
    x[q] = v;
  }
}

// The mask and the first weighting of a pass.  mode 0: mask 1; mode 1
// (log_z_plus hinge, :286-292): mask 0 where the difference is <= 0;
// mode 2 (logistic, :361-368): mask 1 where it is <= 0, and the product
// taken as (r*mask)*w instead of (r*w)*mask.
__global__ void k_reg_weight(long long n, int mode, float *__restrict__ rm,
                             const float *__restrict__ zwt, float *__restrict__ mask) {
  GRID_STRIDE(q, n) {
    float r = rm[q];
    const float w = zwt ? zwt[q] : 1.0f;
    float m;
    if (mode == 2) {
      m = r <= 0.0f ? 1.0f : 0.0f;
      r = r * m * w;
    } else {
      m = mode == 1 ? (r <= 0.0f ? 0.0f : 1.0f) : 1.0f;
      r = r * w * m;
    }
    mask[q] = m;
    rm[q] = r;
  }
}

constexpr int kFctThreads = 1024;
constexpr int kFctChunk = 4096;

// fct_compute over the first nz*nx samples of the model-sized copy of the
// differences (the interior of the first y plane): one block.  The
// threshold, when it is 0 for a thresholded norm, becomes the block's exact
// max|.|; the terms are formed in parallel into shared memory and thread 0
// adds them in sample order.
__global__ void __launch_bounds__(kFctThreads)
    k_reg_fct(int ntype, RegDims R, const float *__restrict__ rm, float *thresh, double *fout) {
  __shared__ double sterm[kFctChunk];
  __shared__ float smax[kFctThreads];
  const long long nd = (long long)R.nz * R.nx;
  auto at = [&](long long k) {
    const long long iz = k % R.nz, ix = k / R.nz;
    return rm[(iz + R.tz) + R.nzt * ((ix + R.tx) + R.nxt * R.ty)];
  };
  const bool thr = ntype == SW_NRM_HUBER || ntype == SW_NRM_CAUCHY || ntype == SW_NRM_HYPERBOLIC;
  if (thr && *thresh == 0.0f) {
    float mx = 0.0f;
    for (long long k = threadIdx.x; k < nd; k += blockDim.x) mx = fmaxf(mx, fabsf(at(k)));
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) smax[threadIdx.x] = fmaxf(smax[threadIdx.x], smax[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) *thresh = smax[0];
    __syncthreads();
  }
  const float g = thr ? *thresh : 0.0f;
  double f2 = 0.0;  // L2: FP64 sum of FP64 products
  float f1 = 0.0f;  // the others: FP32 sum of FP32 terms
  for (long long c0 = 0; c0 < nd; c0 += kFctChunk) {
    const int len = (int)min((long long)kFctChunk, nd - c0);
    for (int k = threadIdx.x; k < len; k += blockDim.x) {
      const float d = at(c0 + k);
      sterm[k] = ntype == SW_NRM_L2 ? (double)d * (double)d : (double)nrm_term(ntype, d, g);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (ntype == SW_NRM_L2)
        for (int k = 0; k < len; ++k) f2 = f2 + sterm[k];
      else
        for (int k = 0; k < len; ++k) f1 = f1 + (float)sterm[k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *fout = ntype == SW_NRM_L2 ? f2 / 2 : (double)f1;
}

// gdt_compute over the first nzt*nxt samples, then the second weighting
// (:317 / :388).
__global__ void k_reg_gdt(long long n, long long ngdt, int ntype, int logistic,
                          const float *__restrict__ thresh, float *__restrict__ rm,
                          const float *__restrict__ zwt, const float *__restrict__ mask) {
  const bool thr = ntype == SW_NRM_HUBER || ntype == SW_NRM_CAUCHY || ntype == SW_NRM_HYPERBOLIC;
  const float g = thr ? *thresh : 0.0f;
  GRID_STRIDE(q, n) {
    float r = rm[q];
    if (q < ngdt) r = nrm_gdt(ntype, r, g);
    const float w = zwt ? zwt[q] : 1.0f, m = mask[q];
    rm[q] = logistic ? m * r * w : r * w * m;
  }
}

// g = g + (0 + interior of the adjoint output) (add_taper, forw=.false.,
// into a cleared gtmp, then g=g+gtmp).
__global__ void k_reg_accum(RegDims R, const float *__restrict__ rt, float *__restrict__ g) {
  GRID_STRIDE(q, R.n) {
    const long long iz = q % R.nz, ix = (q / R.nz) % R.nx, iy = q / ((long long)R.nz * R.nx);
    g[q] = g[q] + (0.0f + rt[(iz + R.tz) + R.nzt * ((ix + R.tx) + R.nxt * (iy + R.ty))]);
  }
}

// gtmp = gtmp / sngl(scaling); grad = grad - gtmp * eps.
__global__ void k_reg_update(long long n, float scale, float eps, const float *__restrict__ gt,
                             float *__restrict__ grad) {
  GRID_STRIDE(q, n) grad[q] = grad[q] - (gt[q] / scale) * eps;
}

__global__ void k_mask_mul(long long n, const float *__restrict__ m, float *__restrict__ grad) {
  GRID_STRIDE(q, n) grad[q] = grad[q] * m[q];
}

bool known_norm(int t) {
  return t == SW_NRM_L1 || t == SW_NRM_L2 || t == SW_NRM_HUBER || t == SW_NRM_CAUCHY ||
         t == SW_NRM_HYPERBOLIC;
}

}  // namespace

int sw_fwi_regularize(sw_ctx *c, const sw_reg_desc *dp, sw_reg_state *stp, int eval,
                      const float *vel, const float *vpmask, double *f, float *grad) {
  if (!c || !dp || !stp || !vel || !f || !grad) return SW_BAD_PARAM;
  const sw_reg_desc &d = *dp;
  sw_reg_state &S = *stp;
  if (d.nz < 1 || d.nx < 1 || d.ny < 1 || d.ntaperz < 0 || d.ntaperx < 0 || d.ntapery < 0)
    return fail(c, SW_BAD_PARAM, "regularisation grid %d x %d x %d, tapers %d %d %d", d.nz, d.nx,
                d.ny, d.ntaperz, d.ntaperx, d.ntapery);
  const int mtype = d.mod_nrm_type == 0 ? SW_NRM_L2 : d.mod_nrm_type;
  const int htype = d.hin_nrm_type == 0 ? SW_NRM_L2 : d.hin_nrm_type;
  if ((d.wantreg && !known_norm(mtype)) || (d.wantlog && !known_norm(htype)))
    return fail(c, SW_BAD_PARAM, "model_nrm_type %d / hinge_nrm_type %d is not a norm",
                d.mod_nrm_type, d.hin_nrm_type);
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  RegDims R;
  R.nz = d.nz; R.nx = d.nx; R.ny = d.ny;
  R.tz = d.ntaperz; R.tx = d.ntaperx; R.ty = d.ny != 1 ? d.ntapery : 0;
  R.nzt = R.nz + 2LL * R.tz; R.nxt = R.nx + 2LL * R.tx; R.nyt = R.ny + 2LL * R.ty;
  R.ntap = R.nzt * R.nxt * R.nyt;
  R.n = (long long)R.nz * R.nx * R.ny;
  const long long n = R.n, nt = R.ntap;
  int st = 0;
  void *p = nullptr;
  if ((st = upload(c, "reg_grad", grad, n * sizeof(float), &p))) return st;
  float *dgrad = (float *)p;
  const bool any = d.wantreg || d.wantlog;
  float *dthr = nullptr, *dvt = nullptr, *drm = nullptr, *drt = nullptr, *dmask = nullptr,
        *dzw = nullptr, *dgt = nullptr;
  double *dfct = nullptr;
  if (any) {
    if ((st = upload(c, "reg_vel", vel, n * sizeof(float), &p))) return st;
    const float *dvel = (const float *)p;
    const float thr[2] = {S.mod_thresh, S.hin_thresh};
    if ((st = upload(c, "reg_thr", thr, sizeof(thr), &p))) return st;
    dthr = (float *)p;
    dvt = (float *)dbuf(c, "reg_vtap", nt * sizeof(float), &st);
    drm = (float *)dbuf(c, "reg_rm", nt * sizeof(float), &st);
    drt = (float *)dbuf(c, "reg_rt", nt * sizeof(float), &st);
    dmask = (float *)dbuf(c, "reg_mask", nt * sizeof(float), &st);
    dgt = (float *)dbuf(c, "reg_gtmp", 2 * n * sizeof(float), &st);
    dfct = (double *)dbuf(c, "reg_fct", 4 * sizeof(double), &st);
    if (!dvt || !drm || !drt || !dmask || !dgt || !dfct) return st;
    k_reg_pad<<<grid_for(nt), 256, 0, s>>>(R, dvel, dvt);
    if (d.zweight) {
      if ((st = upload(c, "reg_zw", d.zweight, n * sizeof(float), &p))) return st;
      dzw = (float *)dbuf(c, "reg_zwtap", nt * sizeof(float), &st);
      if (!dzw) return st;
      k_reg_pad<<<grid_for(nt), 256, 0, s>>>(R, (const float *)p, dzw);
    }
    SW_CK(cudaMemsetAsync(dgt, 0, 2 * n * sizeof(float), s));
  }
  // One SparseRegularization_Compute_f_g / LogisticRegularization_Compute_f_g.
  auto pass = [&](long long lag, int mode, int ntype, float *thr, double *fslot, float *g) {
    k_helix_fwd<<<grid_for(nt), 256, 0, s>>>(nt, lag, dvt, drm);
    k_reg_weight<<<grid_for(nt), 256, 0, s>>>(nt, mode, drm, dzw, dmask);
    k_reg_fct<<<1, kFctThreads, 0, s>>>(ntype, R, drm, thr, fslot);
    k_reg_gdt<<<grid_for(nt), 256, 0, s>>>(nt, R.nzt * R.nxt, ntype, mode == 2, thr, drm, dzw,
                                           dmask);
    k_helix_adj<<<grid_for(nt), 256, 0, s>>>(nt, lag, drm, drt);
    k_reg_accum<<<grid_for(n), 256, 0, s>>>(R, drt, g);
    c->stats.launches_total += 6;
  };
  // SparseRegularization_apply (:238-256): x, z, then y with the x filter.
  int nsp = 0;
  if (d.wantreg) {
    if (d.derivdx) pass(R.nzt, 0, mtype, dthr, dfct + nsp++, dgt);
    if (d.derivdz) pass(1, d.log_z_plus ? 1 : 0, mtype, dthr, dfct + nsp++, dgt);
    if (d.ny != 1 && d.derivdy) pass(R.nzt, 0, mtype, dthr, dfct + nsp++, dgt);
  }
  if (d.wantlog) pass(1, 2, htype, dthr + 1, dfct + 3, dgt + n);
  SW_CK(cudaGetLastError());
  double fv[4] = {0., 0., 0., 0.};
  if (any) {
    float thr[2];
    if ((st = download(c, fv, dfct, sizeof(fv)))) return st;
    if ((st = download(c, thr, dthr, sizeof(thr)))) return st;
    S.mod_thresh = thr[0];
    S.hin_thresh = thr[1];
  }
  // compute_fct_gdt_reg (compute_function_gradient.f90:115-203).
  const double scaling = (double)d.nx * d.ny * d.nz;
  double ftmp = 0., ftmp1 = 0.;
  if (d.compute_eps && eval == 0) S.eps = 0.f;
  if (d.compute_eps_log && eval == 0) S.eps_log = 0.f;
  if (d.wantreg) {
    for (int i = 0; i < nsp; ++i) ftmp = ftmp + fv[i];
    ftmp = ftmp / scaling;
    if (d.compute_eps && eval == 0) {
      if (d.ratio == 0.f)
        S.eps = 0.f;
      else if (ftmp != 0.)
        S.eps = (float)std::fabs(*f / ((double)d.ratio * ftmp));
      else
        return fail(c, SW_NUMERIC, "cannot compute eps for regularization: the term is 0");
    }
    k_reg_update<<<grid_for(n), 256, 0, s>>>(n, (float)scaling, S.eps, dgt, dgrad);
    c->stats.launches_total++;
  } else {
    S.eps = 0.f;
  }
  if (d.wantlog) {
    ftmp1 = fv[3] / scaling;
    if (d.compute_eps_log && eval == 0) {
      if (d.ratio_log == 0.f)
        S.eps_log = 0.f;
      else if (ftmp1 == 0.)
        S.eps_log = (float)std::fabs(*f / ((double)d.ratio_log * ftmp));
      else
        S.eps_log = (float)std::fabs(*f / ((double)d.ratio_log * ftmp1));
    }
    k_reg_update<<<grid_for(n), 256, 0, s>>>(n, (float)scaling, S.eps_log, dgt + n, dgrad);
    c->stats.launches_total++;
  } else {
    S.eps_log = 0.f;
  }
  if (vpmask) {
    if ((st = upload(c, "reg_mask_in", vpmask, n * sizeof(float), &p))) return st;
    k_mask_mul<<<grid_for(n), 256, 0, s>>>(n, (const float *)p, dgrad);
    c->stats.launches_total++;
  }
  SW_CK(cudaGetLastError());
  if ((st = download(c, grad, dgrad, n * sizeof(float)))) return st;
  *f = *f + ftmp * (double)S.eps + ftmp1 * (double)S.eps_log;
  return SW_OK;
}
