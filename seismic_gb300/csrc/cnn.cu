// cnn.cu - the convolutional gradient preconditioner (no reference
// counterpart): a small stack of 3x3 convolutions (ReLU between layers)
// that maps the FWI gradient and the source illumination to a search
// direction, with training and inference on the GPU.
//
// Convolutions are implicit GEMMs on the 5th-generation tensor cores
// (umma.cuh): a CTA of 128 threads gathers the 3x3 neighbourhoods of 128
// pixels (BF16, K = 9 * Cin padded to a multiple of 16) and the layer's
// BF16 weights (N = 16 output channels) into shared memory, one thread
// issues the K/16 tcgen05.mma instructions into an FP32 accumulator in
// tensor memory, and the epilogue adds the bias.  The input gradient of a
// layer is the same implicit GEMM with mirrored taps and transposed
// weights; the weight gradient is a per-tap reduction over pixels in FP32
// on the CUDA cores.  Master weights and Adam moments stay in FP32; BF16
// copies in both GEMM layouts are rewritten after every update.
//
// Images are nz x nx with z fastest (pixel p = x * nz + z); activations are
// channels-last.  At most 16 channels per layer.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/swave.h"
#include "engine.h"
#include "umma.cuh"

using namespace swave;

namespace {

constexpr int kMaxC = 16;        // channels per layer (GEMM N)
constexpr int kTile = 128;       // pixels per CTA (GEMM M)
constexpr int kMaxK = 9 * kMaxC; // 144

int kpad(int k) { return (k + 15) / 16 * 16; }

// ---------------------------------------------------------------------------
// Implicit-GEMM 3x3 convolution on tcgen05.
//   out[p][n] = bias[n] + sum_{tap, c} in[p + s * off(tap)][c] * W[n][tap * C + c]
// with s = +1 (forward) or -1 (input gradient, mirrored taps) and zero
// padding outside the image.  W is BF16 [16][KP] K-major (zero padded).
// ---------------------------------------------------------------------------
template <int KP>
__global__ void __launch_bounds__(kTile, 1)
    k_conv_umma(const __nv_bfloat16 *__restrict__ in, int C, int nz, int nx,
                const __nv_bfloat16 *__restrict__ W, const float *__restrict__ bias, int nout,
                int mirror, float *__restrict__ out, int *err) {
  __shared__ __align__(1024) unsigned char sA[kTile * KP * 2];
  __shared__ __align__(1024) unsigned char sB[kMaxC * KP * 2];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ unsigned tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int npix = nz * nx;
  const int p0 = blockIdx.x * kTile;
  if (warp == 0) umma_alloc(&tmem_base, 32);
  if (tid == 0) umma_mbar_init(&mbar);
  // Weights: 16 rows x KP, 16-byte chunks.
  for (int q = tid; q < kMaxC * KP / 8; q += kTile) {
    const int r = q / (KP / 8), k = (q % (KP / 8)) * 8;
    *reinterpret_cast<uint4 *>(sB + umma_off(r, k, kMaxC)) =
        *reinterpret_cast<const uint4 *>(W + (size_t)r * KP + k);
  }
  // Pixel neighbourhoods: thread = pixel row of the tile.
  {
    const int p = p0 + tid;
    const int x = p / nz, z = p - x * nz;
    const int kv = 9 * C;
    for (int k = 0; k < KP; ++k) {
      __nv_bfloat16 v = __float2bfloat16(0.f);
      if (k < kv && p < npix) {
        const int tap = k / C, c = k - tap * C;
        const int dz = (tap % 3 - 1) * (mirror ? -1 : 1), dx = (tap / 3 - 1) * (mirror ? -1 : 1);
        const int zz = z + dz, xx = x + dx;
        if (zz >= 0 && zz < nz && xx >= 0 && xx < nx) v = in[((size_t)xx * nz + zz) * C + c];
      }
      *reinterpret_cast<__nv_bfloat16 *>(sA + umma_off(tid, k, kTile)) = v;
    }
  }
  umma_fence_smem();
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  const unsigned tmem = tmem_base;
  if (tid == 0) {
    constexpr uint32_t idesc = umma_idesc_bf16(kTile, kMaxC);
#pragma unroll
    for (int ks = 0; ks < KP / 16; ++ks) {
      const uint64_t ad =
          umma_smem_desc(umma_su32(sA) + ks * 2 * (kTile / 8) * 128, (kTile / 8) * 128, 128);
      const uint64_t bd =
          umma_smem_desc(umma_su32(sB) + ks * 2 * (kMaxC / 8) * 128, (kMaxC / 8) * 128, 128);
      umma_bf16(tmem, ad, bd, idesc, ks > 0);
    }
    umma_commit(&mbar);
  }
  const bool ok = umma_mbar_wait(&mbar, 0);
  if (!ok && tid == 0) atomicOr(err, 1);
  umma_fence_after();
  float acc[16];
  umma_ld16(tmem + ((unsigned)(warp * 32) << 16), acc);
  const int p = p0 + tid;
  if (p < npix && ok) {
#pragma unroll
    for (int n = 0; n < 16; ++n)
      if (n < nout) out[(size_t)p * nout + n] = acc[n] + (bias ? bias[n] : 0.f);
  }
  umma_fence_before();
  __syncthreads();
  if (warp == 0) umma_dealloc(tmem, 32);
}

// Planar FP32 channels (c, p) -> channels-last BF16.
__global__ void k_pack_input(const float *__restrict__ in, int C, int npix,
                             __nv_bfloat16 *__restrict__ out) {
  const long long n = (long long)C * npix;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(q % C);
    const long long p = q / C;
    out[q] = __float2bfloat16(in[(size_t)c * npix + p]);
  }
}

// ReLU of a pre-activation into BF16 activations.
__global__ void k_relu_bf16(const float *__restrict__ z, long long n, __nv_bfloat16 *__restrict__ a) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    a[q] = __float2bfloat16(z[q] > 0.f ? z[q] : 0.f);
}

// dz = da * [z > 0] (FP32 for the weight gradient, BF16 for the next
// input-gradient GEMM).
__global__ void k_relu_back(const float *__restrict__ da, const float *__restrict__ z, long long n,
                            float *__restrict__ dz, __nv_bfloat16 *__restrict__ dzb) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float v = z[q] > 0.f ? da[q] : 0.f;
    dz[q] = v;
    dzb[q] = __float2bfloat16(v);
  }
}

// Mean-square loss of a one-channel output: d = (out - target) / npix and
// per-block FP64 partial sums of (out - target)^2.
__global__ void k_loss(const float *__restrict__ out, const float *__restrict__ tgt, int npix,
                       float *__restrict__ d, __nv_bfloat16 *__restrict__ db,
                       double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    const float e = out[p] - tgt[p];
    s += (double)e * (double)e;
    d[p] = e / (float)npix;
    db[p] = __float2bfloat16(e / (float)npix);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Weight and bias gradient partials of one layer: block (tap, chunk) sums
// dz[p][co] * a[p + off(tap)][ci] over its pixel chunk; tap 9 is the bias.
__global__ void k_wgrad(const float *__restrict__ dz, int Cout, const __nv_bfloat16 *__restrict__ a,
                        int Cin, int nz, int nx, int chunk, float *__restrict__ part) {
  const int tap = blockIdx.x, cb = blockIdx.y;
  const int npix = nz * nx;
  const int co = threadIdx.x / kMaxC, ci = threadIdx.x % kMaxC;
  const bool active = co < Cout && (tap == 9 ? ci == 0 : ci < Cin);
  float s = 0.f;
  if (active) {
    const int dzo = tap % 3 - 1, dxo = tap / 3 - 1;
    const int pe = min(npix, (cb + 1) * chunk);
    for (int p = cb * chunk; p < pe; ++p) {
      const float g = dz[(size_t)p * Cout + co];
      if (tap == 9) {
        s += g;
      } else {
        const int x = p / nz, z = p - x * nz;
        const int zz = z + dzo, xx = x + dxo;
        if (zz >= 0 && zz < nz && xx >= 0 && xx < nx)
          s += g * __bfloat162float(a[((size_t)xx * nz + zz) * Cin + ci]);
      }
    }
  }
  part[((size_t)cb * 10 + tap) * (kMaxC * kMaxC) + threadIdx.x] = s;
}

// Sums the chunk partials in chunk order into the layer's gradient buffer
// (FP32, [co][tap][ci] then bias[co]) - added to what it holds.
__global__ void k_wgrad_sum(const float *__restrict__ part, int nchunk, int Cout, int Cin,
                            float *__restrict__ gw) {
  const int tap = blockIdx.x, t = threadIdx.x;
  const int co = t / kMaxC, ci = t % kMaxC;
  if (co >= Cout || (tap == 9 ? ci != 0 : ci >= Cin)) return;
  float s = 0.f;
  for (int c = 0; c < nchunk; ++c) s += part[((size_t)c * 10 + tap) * (kMaxC * kMaxC) + t];
  if (tap == 9) gw[(size_t)Cout * 9 * Cin + co] += s;
  else gw[((size_t)co * 9 + tap) * Cin + ci] += s;
}

// Adam on the FP32 master weights, then the BF16 GEMM copies: forward
// [co][tap*Cin + ci] and input-gradient [ci][tap*Cout + co], zero padded.
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2, float gscale) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gg = g[q] * gscale;
  const float mm = b1 * m[q] + (1.f - b1) * gg;
  const float vv = b2 * v[q] + (1.f - b2) * gg * gg;
  m[q] = mm;
  v[q] = vv;
  w[q] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}
__global__ void k_weights_bf16(const float *__restrict__ w, int Cout, int Cin, int KPF, int KPB,
                               __nv_bfloat16 *__restrict__ wf, __nv_bfloat16 *__restrict__ wb) {
  const int t = threadIdx.x;
  for (int q = t; q < kMaxC * KPF; q += blockDim.x) {
    const int co = q / KPF, k = q % KPF;
    float v = 0.f;
    if (co < Cout && k < 9 * Cin) {
      const int tap = k / Cin, ci = k % Cin;
      v = w[((size_t)co * 9 + tap) * Cin + ci];
    }
    wf[q] = __float2bfloat16(v);
  }
  for (int q = t; q < kMaxC * KPB; q += blockDim.x) {
    const int ci = q / KPB, k = q % KPB;
    float v = 0.f;
    if (ci < Cin && k < 9 * Cout) {
      const int tap = k / Cout, co = k % Cout;
      v = w[((size_t)co * 9 + tap) * Cin + ci];
    }
    wb[q] = __float2bfloat16(v);
  }
}

int nblk(long long n) { return (int)std::min<long long>(4096, (n + 255) / 256); }

cudaError_t launch_conv(int KP, const __nv_bfloat16 *in, int C, int nz, int nx,
                        const __nv_bfloat16 *W, const float *bias, int nout, int mirror,
                        float *out, int *err, cudaStream_t s) {
  const int grid = (nz * nx + kTile - 1) / kTile;
  switch (KP) {
    case 16: k_conv_umma<16><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 32: k_conv_umma<32><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 48: k_conv_umma<48><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 64: k_conv_umma<64><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 80: k_conv_umma<80><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 96: k_conv_umma<96><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 112: k_conv_umma<112><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 128: k_conv_umma<128><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    case 144: k_conv_umma<144><<<grid, kTile, 0, s>>>(in, C, nz, nx, W, bias, nout, mirror, out, err); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

struct sw_cnn {
  sw_ctx *ctx = nullptr;
  int nl = 0;
  std::vector<int> ch;                 // nl + 1 channel counts
  std::vector<size_t> woff;            // offset of layer l in the packed weights
  size_t nw = 0;                       // packed FP32 weights (w then b per layer)
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  std::vector<__nv_bfloat16 *> wf, wb; // BF16 GEMM copies per layer
  int step = 0;
  // Per-image buffers (grow-only).
  size_t cap = 0;
  std::vector<float *> z;              // pre-activations per layer [p][Cout]
  std::vector<__nv_bfloat16 *> a;      // activations per layer input [p][Cin]
  float *da = nullptr, *dz = nullptr, *part = nullptr, *in32 = nullptr, *tgt = nullptr;
  __nv_bfloat16 *dzb = nullptr;
  double *lpart = nullptr;
  int *err = nullptr;
};

namespace {

int cnn_fail(sw_cnn *n, cudaError_t e, const char *what) {
  return cuda_fail(n ? n->ctx : nullptr, e, what);
}

void free_images(sw_cnn *n) {
  for (auto p : n->z) cudaFree(p);
  for (auto p : n->a) cudaFree(p);
  n->z.clear();
  n->a.clear();
  cudaFree(n->da); cudaFree(n->dz); cudaFree(n->part); cudaFree(n->in32); cudaFree(n->tgt);
  cudaFree(n->dzb); cudaFree(n->lpart);
  n->da = n->dz = n->part = n->in32 = n->tgt = nullptr;
  n->dzb = nullptr;
  n->lpart = nullptr;
  n->cap = 0;
}

int ensure_images(sw_cnn *n, size_t npix) {
  if (npix <= n->cap) return SW_OK;
  free_images(n);
  auto ck = [&](cudaError_t e) { return e == cudaSuccess; };
  bool ok = true;
  n->z.assign(n->nl, nullptr);
  n->a.assign(n->nl, nullptr);
  for (int l = 0; l < n->nl && ok; ++l) {
    ok = ck(cudaMalloc(&n->z[l], npix * n->ch[l + 1] * sizeof(float))) &&
         ck(cudaMalloc(&n->a[l], npix * n->ch[l] * sizeof(__nv_bfloat16)));
  }
  const int nchunk = (int)((npix + 2047) / 2048);
  ok = ok && ck(cudaMalloc(&n->da, npix * kMaxC * sizeof(float))) &&
       ck(cudaMalloc(&n->dz, npix * kMaxC * sizeof(float))) &&
       ck(cudaMalloc(&n->dzb, npix * kMaxC * sizeof(__nv_bfloat16))) &&
       ck(cudaMalloc(&n->part, (size_t)nchunk * 10 * kMaxC * kMaxC * sizeof(float))) &&
       ck(cudaMalloc(&n->in32, npix * n->ch[0] * sizeof(float))) &&
       ck(cudaMalloc(&n->tgt, npix * sizeof(float))) &&
       ck(cudaMalloc(&n->lpart, 1024 * sizeof(double)));
  if (!ok) {
    cudaGetLastError();
    free_images(n);
    return fail(n->ctx, SW_OOM_ADMISSION, "cnn image buffers");
  }
  n->cap = npix;
  return SW_OK;
}

int refresh_bf16(sw_cnn *n) {
  cudaStream_t s = n->ctx->stream;
  for (int l = 0; l < n->nl; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    k_weights_bf16<<<1, 256, 0, s>>>(n->w + n->woff[l], Cout, Cin, kpad(9 * Cin), kpad(9 * Cout),
                                     n->wf[l], n->wb[l]);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SW_OK : cnn_fail(n, e, "cnn weights");
}

// Forward pass of one image already packed into n->a[0]; output in n->z[nl-1].
int forward(sw_cnn *n, int nz, int nx) {
  cudaStream_t s = n->ctx->stream;
  const long long npix = (long long)nz * nx;
  cudaError_t e;
  for (int l = 0; l < n->nl; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    const float *b = n->w + n->woff[l] + (size_t)Cout * 9 * Cin;
    if ((e = launch_conv(kpad(9 * Cin), n->a[l], Cin, nz, nx, n->wf[l], b, Cout, 0, n->z[l],
                         n->err, s)) != cudaSuccess)
      return cnn_fail(n, e, "cnn conv");
    if (l + 1 < n->nl) {
      k_relu_bf16<<<nblk(npix * Cout), 256, 0, s>>>(n->z[l], npix * Cout, n->a[l + 1]);
      if ((e = cudaGetLastError()) != cudaSuccess) return cnn_fail(n, e, "cnn relu");
    }
  }
  return SW_OK;
}

int check_err(sw_cnn *n) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, n->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(n->ctx->stream);
  if (e != cudaSuccess) return cnn_fail(n, e, "cnn");
  if (h) return fail(n->ctx, SW_TIMEOUT, "cnn: a tensor-core wait gave up");
  return SW_OK;
}

}  // namespace

extern "C" {

int sw_cnn_create(sw_ctx *c, int nlayers, const int *channels, uint64_t seed, sw_cnn **out) {
  if (!c || !channels || !out || nlayers < 1 || nlayers > 16) return SW_BAD_PARAM;
  *out = nullptr;
  for (int l = 0; l <= nlayers; ++l)
    if (channels[l] < 1 || channels[l] > kMaxC) return fail(c, SW_BAD_PARAM, "cnn channels must be 1..16");
  cudaSetDevice(c->device);
  sw_cnn *n = new sw_cnn();
  n->ctx = c;
  n->nl = nlayers;
  n->ch.assign(channels, channels + nlayers + 1);
  for (int l = 0; l < nlayers; ++l) {
    n->woff.push_back(n->nw);
    n->nw += (size_t)n->ch[l + 1] * 9 * n->ch[l] + n->ch[l + 1];
  }
  // He initialisation, zero biases.
  std::vector<float> h(n->nw, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < nlayers; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (9.f * Cin)));
    for (int q = 0; q < Cout * 9 * Cin; ++q) h[n->woff[l] + q] = nd(rng);
  }
  auto ck = [](cudaError_t e) { return e == cudaSuccess; };
  bool ok = ck(cudaMalloc(&n->w, n->nw * 4)) && ck(cudaMalloc(&n->g, n->nw * 4)) &&
            ck(cudaMalloc(&n->m, n->nw * 4)) && ck(cudaMalloc(&n->v, n->nw * 4)) &&
            ck(cudaMalloc(&n->err, sizeof(int)));
  n->wf.assign(nlayers, nullptr);
  n->wb.assign(nlayers, nullptr);
  for (int l = 0; l < nlayers && ok; ++l)
    ok = ck(cudaMalloc(&n->wf[l], kMaxC * kpad(9 * n->ch[l]) * 2)) &&
         ck(cudaMalloc(&n->wb[l], kMaxC * kpad(9 * n->ch[l + 1]) * 2));
  ok = ok && ck(cudaMemcpy(n->w, h.data(), n->nw * 4, cudaMemcpyHostToDevice)) &&
       ck(cudaMemset(n->m, 0, n->nw * 4)) && ck(cudaMemset(n->v, 0, n->nw * 4)) &&
       ck(cudaMemset(n->err, 0, sizeof(int)));
  if (!ok || refresh_bf16(n) != SW_OK) {
    cudaGetLastError();
    sw_cnn_destroy(n);
    return fail(c, SW_CUDA_ERR, "cnn create");
  }
  *out = n;
  return SW_OK;
}

int sw_cnn_destroy(sw_cnn *n) {
  if (!n) return SW_OK;
  cudaSetDevice(n->ctx->device);
  cudaStreamSynchronize(n->ctx->stream);
  free_images(n);
  cudaFree(n->w); cudaFree(n->g); cudaFree(n->m); cudaFree(n->v); cudaFree(n->err);
  for (auto p : n->wf) cudaFree(p);
  for (auto p : n->wb) cudaFree(p);
  delete n;
  return SW_OK;
}

int sw_cnn_num_weights(const sw_cnn *n) { return n ? (int)n->nw : 0; }

int sw_cnn_get_weights(const sw_cnn *n, float *w) {
  if (!n || !w) return SW_BAD_PARAM;
  cudaSetDevice(n->ctx->device);
  if (cudaMemcpy(w, n->w, n->nw * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return SW_CUDA_ERR;
  return SW_OK;
}

int sw_cnn_set_weights(sw_cnn *n, const float *w) {
  if (!n || !w) return SW_BAD_PARAM;
  cudaSetDevice(n->ctx->device);
  if (cudaMemcpy(n->w, w, n->nw * 4, cudaMemcpyHostToDevice) != cudaSuccess) return SW_CUDA_ERR;
  const int st = refresh_bf16(n);
  if (st) return st;
  return cudaStreamSynchronize(n->ctx->stream) == cudaSuccess ? SW_OK : SW_CUDA_ERR;
}

int sw_cnn_forward(sw_cnn *n, int nz, int nx, const float *in, float *out) {
  if (!n || !in || !out || nz < 1 || nx < 1) return SW_BAD_PARAM;
  if (n->ch[n->nl] != 1) return fail(n->ctx, SW_BAD_PARAM, "cnn output must have one channel");
  cudaSetDevice(n->ctx->device);
  cudaStream_t s = n->ctx->stream;
  const size_t npix = (size_t)nz * nx;
  int st = ensure_images(n, npix);
  if (st) return st;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(n->in32, in, npix * n->ch[0] * 4, cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return cnn_fail(n, e, "cnn input");
  k_pack_input<<<nblk((long long)npix * n->ch[0]), 256, 0, s>>>(n->in32, n->ch[0], (int)npix,
                                                                 n->a[0]);
  if ((st = forward(n, nz, nx))) return st;
  if ((e = cudaMemcpyAsync(out, n->z[n->nl - 1], npix * 4, cudaMemcpyDeviceToHost, s)) !=
      cudaSuccess)
    return cnn_fail(n, e, "cnn output");
  return check_err(n);
}

int sw_cnn_train_step(sw_cnn *n, int nbatch, int nz, int nx, const float *in,
                      const float *target, float lr, double *loss) {
  if (!n || !in || !target || nbatch < 1 || nz < 1 || nx < 1) return SW_BAD_PARAM;
  if (n->ch[n->nl] != 1) return fail(n->ctx, SW_BAD_PARAM, "cnn output must have one channel");
  cudaSetDevice(n->ctx->device);
  cudaStream_t s = n->ctx->stream;
  const size_t npix = (size_t)nz * nx;
  int st = ensure_images(n, npix);
  if (st) return st;
  cudaError_t e;
  if ((e = cudaMemsetAsync(n->g, 0, n->nw * 4, s)) != cudaSuccess) return cnn_fail(n, e, "cnn");
  const int chunk = 2048, nchunk = (int)((npix + chunk - 1) / chunk);
  const int lblocks = (int)std::min<size_t>(1024, (npix + 255) / 256);
  double lsum = 0.0;
  std::vector<double> hp(lblocks);
  for (int ib = 0; ib < nbatch; ++ib) {
    const float *xin = in + (size_t)ib * npix * n->ch[0];
    const float *tin = target + (size_t)ib * npix;
    if ((e = cudaMemcpyAsync(n->in32, xin, npix * n->ch[0] * 4, cudaMemcpyHostToDevice, s)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(n->tgt, tin, npix * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return cnn_fail(n, e, "cnn batch");
    k_pack_input<<<nblk((long long)npix * n->ch[0]), 256, 0, s>>>(n->in32, n->ch[0], (int)npix,
                                                                   n->a[0]);
    if ((st = forward(n, nz, nx))) return st;
    // d loss / d output (one channel), FP64 loss partials.
    k_loss<<<lblocks, 256, 0, s>>>(n->z[n->nl - 1], n->tgt, (int)npix, n->dz, n->dzb, n->lpart);
    for (int l = n->nl - 1; l >= 0; --l) {
      const int Cin = n->ch[l], Cout = n->ch[l + 1];
      // Weight / bias gradient from dz (this layer) and the layer input.
      k_wgrad<<<dim3(10, nchunk), kMaxC * kMaxC, 0, s>>>(n->dz, Cout, n->a[l], Cin, nz, nx, chunk,
                                                          n->part);
      k_wgrad_sum<<<10, kMaxC * kMaxC, 0, s>>>(n->part, nchunk, Cout, Cin, n->g + n->woff[l]);
      if (l == 0) break;
      // Input gradient: mirrored taps, transposed weights, then ReLU'.
      if ((e = launch_conv(kpad(9 * Cout), n->dzb, Cout, nz, nx, n->wb[l], nullptr, Cin, 1, n->da,
                           n->err, s)) != cudaSuccess)
        return cnn_fail(n, e, "cnn dgrad");
      k_relu_back<<<nblk((long long)npix * Cin), 256, 0, s>>>(n->da, n->z[l - 1],
                                                             (long long)npix * Cin, n->dz, n->dzb);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return cnn_fail(n, e, "cnn backward");
    if ((e = cudaMemcpyAsync(hp.data(), n->lpart, lblocks * sizeof(double),
                             cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return cnn_fail(n, e, "cnn loss");
    double ls = 0.0;
    for (int b = 0; b < lblocks; ++b) ls += hp[b];
    lsum += ls / (2.0 * (double)npix);
  }
  // Adam (b1 0.9, b2 0.999, eps 1e-8) on the batch-mean gradient.
  n->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
  k_adam<<<(int)((n->nw + 255) / 256), 256, 0, s>>>(n->w, n->g, n->m, n->v, (int)n->nw, lr, b1, b2,
                                                    1e-8f, c1, c2, 1.f / (float)nbatch);
  if ((st = refresh_bf16(n))) return st;
  if (loss) *loss = lsum / nbatch;
  return check_err(n);
}

}  // extern "C"
